// Tensor-core (tcgen05 + TMA + TMEM) GEMM engine for the mixed-precision
// forms of the contractions, and the mixed-precision H_eff*x built on it.
//
//   C[m, n] = sum_k A[m, k] B[n, k]      (A, B "K-major": k contiguous)
//
// gemm_kernel: one CTA owns a 128 x BN output tile.  Warp 0 streams A/B
// K-slices into a STAGES-deep shared-memory ring with cp.async.bulk.tensor
// (128-byte swizzle, no multicast), warp 1 allocates the TMEM accumulator and
// issues tcgen05.mma from one thread (kind::tf32 or kind::f16 with BF16
// operands, FP32 accumulation), warps 2-5 drain TMEM with tcgen05.ld and store.
// gemm_pair_kernel: the same roles on a cluster of two CTAs sharing a 256 x 256
// tile through tcgen05.mma.cta_group::2 (BF16 GEMMs of more than 128 rows).
// 3xTF32 issues three MMAs per K-step (hi*hi + hi*lo + lo*hi) into the same
// accumulator from operands pre-split into TF32 hi/lo planes.
//
// Every mbarrier wait is bounded (wall clock, ~2 s): on expiry the kernel
// raises a flag that the host turns into FMPT_ERR_TIMEOUT, drains its own
// MMAs and TMA loads with bounded waits, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "tc_ptx.cuh"

namespace fmpt {
namespace tc {

template <int OUT>
__device__ __forceinline__ void store_cols(void* base, int64_t ldc, int n_base, int n_lim,
                                           const uint32_t (&r)[32]) {
  // base points at C[row, n_base]; columns n_base + j for j < 32, those >= n_lim skipped
  if (n_base + 32 <= n_lim) {
#pragma unroll
    for (int j = 0; j < 32; j++) {
      const float v = __uint_as_float(r[j]);
      if (OUT == 1)
        static_cast<double*>(base)[ldc * j] = (double)v;
      else if (OUT == 2)
        static_cast<__nv_bfloat16*>(base)[ldc * j] = __float2bfloat16_rn(v);
      else
        static_cast<float*>(base)[ldc * j] = v;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; j++) {
      if (n_base + j < n_lim) {
        const float v = __uint_as_float(r[j]);
        if (OUT == 1)
          static_cast<double*>(base)[ldc * j] = (double)v;
        else if (OUT == 2)
          static_cast<__nv_bfloat16*>(base)[ldc * j] = __float2bfloat16_rn(v);
        else
          static_cast<float*>(base)[ldc * j] = v;
      }
    }
  }
}

// One thread's accumulator row (TMEM lane) of a 128 x BN tile -> C[row, n0 .. n0+BN).
// 32-column TMEM loads, the next one in flight while the previous one is stored.
template <int BN, int OUT>
__device__ __forceinline__ void store_acc(uint32_t tbase, int row, int n0, int z,
                                          const EpiArgs& ep) {
  constexpr int es = OUT == 1 ? 8 : OUT == 2 ? 2 : 4;
  char* base = static_cast<char*>(ep.C) + es * ((int64_t)row + ep.strideC * z + ep.ldc * n0);
  const bool live = row < ep.M;
  static_assert(BN % 64 == 0, "epilogue chunk pairs");
  uint32_t ra[32], rb[32];
  tmem_ld32_async(tbase, ra);
  tmem_wait_ld(ra);
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 64) {
    tmem_ld32_async(tbase + c0 + 32, rb);
    if (live) store_cols<OUT>(base + es * ep.ldc * c0, ep.ldc, n0 + c0, ep.N, ra);
    tmem_wait_ld(rb);
    if (c0 + 64 < BN) tmem_ld32_async(tbase + c0 + 64, ra);
    if (live) store_cols<OUT>(base + es * ep.ldc * (c0 + 32), ep.ldc, n0 + c0 + 32, ep.N, rb);
    tmem_wait_ld(ra);
  }
}

template <int MODE, int BN, int STAGES, int OUT>
struct Cfg {
  static constexpr int KBYTES = 128;                            // bytes of K per stage row
  static constexpr int KELEMS = MODE == BF16 ? 64 : 32;
  static constexpr int A_BYTES = BM * KBYTES;
  static constexpr int B_BYTES = BN * KBYTES;
  static constexpr int SPLIT = MODE == TF32X3 ? 2 : 1;
  static constexpr int STAGE_BYTES = (A_BYTES + B_BYTES) * SPLIT;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 256;
  static constexpr int TMEM_COLS = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "N tile");
  static_assert(SMEM <= 227 * 1024, "shared memory");
  static_assert(2 * TMEM_COLS <= 512, "two accumulator buffers must fit in TMEM");
  static_assert((2 * STAGES + 5) * 8 + 8 <= 256, "barrier area");
};

template <int MODE, int BN, int STAGES, int OUT>
__global__ void __launch_bounds__(NTHREADS, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                const __grid_constant__ CUtensorMap mapA2, const __grid_constant__ CUtensorMap mapB2,
                int K, int tiles_m, int tiles_n, int batch, EpiArgs ep) {
  // Persistent: CTA b processes tiles b, b + gridDim.x, ...  (M-tile index fastest, so
  // CTAs running at the same time share B tiles in L2).  The accumulator is double
  // buffered in TMEM: the epilogue of one tile drains buffer t&1 while the MMA warp
  // fills the other one with the next tile.
  using C_ = Cfg<MODE, BN, STAGES, OUT>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * C_::STAGE_BYTES);
  // bars: [0,S) full  [S,2S) empty  [2S,2S+2) accumulator full  [2S+2,2S+4) accumulator
  // empty  [2S+4] drain
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = bars + 2 * STAGES + 2;
  uint64_t* drain = bars + 2 * STAGES + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int nk = (K + C_::KELEMS - 1) / C_::KELEMS;
  const int num_tiles = tiles_m * tiles_n * batch;

  auto stageA = [&](int s, int part) { return smem + s * C_::STAGE_BYTES + part * (C_::A_BYTES + C_::B_BYTES); };
  auto stageB = [&](int s, int part) { return stageA(s, part) + C_::A_BYTES; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[STAGES + s]), 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), 4);          // one arrival per epilogue warp
    }
    mbar_init(smem_u32(drain), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * C_::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int it = 0, last = -1;
      for (int tile = blockIdx.x; tile < num_tiles && !*abort_flag; tile += gridDim.x) {
        int mt, nt, z;
        tile_coords(tile, tiles_m, tiles_n, ep.nfast, mt, nt, z);
        const int m0 = mt * BM, n0 = nt * BN;
        for (int kb = 0; kb < nk; kb++, it++) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!mbar_wait(smem_u32(&bars[STAGES + s]), ph ^ 1, abort_flag, ep.err)) break;
          const uint32_t full = smem_u32(&bars[s]);
          mbar_expect_tx(full, C_::STAGE_BYTES);
          const int kc = kb * C_::KELEMS;
          tma_load_3d(smem_u32(stageA(s, 0)), &mapA, full, kc, m0, z);
          tma_load_3d(smem_u32(stageB(s, 0)), &mapB, full, kc, n0, z);
          if (MODE == TF32X3) {
            tma_load_3d(smem_u32(stageA(s, 1)), &mapA2, full, kc, m0, z);
            tma_load_3d(smem_u32(stageB(s, 1)), &mapB2, full, kc, n0, z);
          }
          last = it;
        }
      }
      if (*abort_flag) {
        // drain: every load this thread issued must land before the CTA exits
        for (int j = max(0, last - STAGES + 1); j <= last; j++) {
          const uint32_t bar = smem_u32(&bars[j % STAGES]);
          const unsigned long long t0 = globaltimer();
          while (!mbar_try(bar, (j / STAGES) & 1) && globaltimer() - t0 < WAIT_NS) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc(MODE, BM, BN);
      int it = 0, local = 0;
      for (int tile = blockIdx.x; tile < num_tiles && !*abort_flag; tile += gridDim.x, local++) {
        const int buf = local & 1;
        const uint32_t use = (uint32_t)(local >> 1);
        if (!mbar_wait(smem_u32(&acc_empty[buf]), (use & 1) ^ 1, abort_flag, ep.err)) break;
        tc_fence_after();
        const uint32_t tacc = tmem + buf * C_::TMEM_COLS;
        for (int kb = 0; kb < nk; kb++, it++) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!mbar_wait(smem_u32(&bars[s]), ph, abort_flag, ep.err)) break;
          tc_fence_after();
          const uint32_t a0 = smem_u32(stageA(s, 0)), b0 = smem_u32(stageB(s, 0));
#pragma unroll
          for (int ks = 0; ks < 4; ks++) {                     // 4 x 32 bytes of K per stage
            const uint32_t acc = (kb > 0 || ks > 0) ? 1u : 0u;
            const uint64_t ad = smem_desc(a0 + ks * 32), bd = smem_desc(b0 + ks * 32);
            mma<MODE>(tacc, ad, bd, idesc, acc);
            if (MODE == TF32X3) {
              const uint32_t a1 = smem_u32(stageA(s, 1)), b1 = smem_u32(stageB(s, 1));
              mma<MODE>(tacc, ad, smem_desc(b1 + ks * 32), idesc, 1u);
              mma<MODE>(tacc, smem_desc(a1 + ks * 32), bd, idesc, 1u);
            }
          }
          mma_commit(smem_u32(&bars[STAGES + s]));             // frees the stage when done
        }
        mma_commit(smem_u32(&acc_full[buf]));                  // this tile's accumulator is ready
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lane quarter = warp % 4
    const int q = warp & 3;
    int local = 0;
    for (int tile = blockIdx.x; tile < num_tiles; tile += gridDim.x, local++) {
      const int buf = local & 1;
      const uint32_t use = (uint32_t)(local >> 1);
      const bool ok = mbar_wait(smem_u32(&acc_full[buf]), use & 1, abort_flag, ep.err);
      if (!ok || *abort_flag) break;
      tc_fence_after();
      int mt, nt, z;
      tile_coords(tile, tiles_m, tiles_n, ep.nfast, mt, nt, z);
      const int row = mt * BM + 32 * q + lane;
      store_acc<BN, OUT>(tmem + buf * C_::TMEM_COLS + ((uint32_t)(32 * q) << 16), row, nt * BN,
                         z, ep);
      // the accumulator buffer may be refilled once all four warps have read it
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[buf]))
                     : "memory");
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    if (lane == 0) {
      // all MMAs issued by this CTA have retired before TMEM is released
      mma_commit(smem_u32(drain));
      const unsigned long long t0 = globaltimer();
      while (!mbar_try(smem_u32(drain), 0) && globaltimer() - t0 < WAIT_NS) {
      }
    }
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * C_::TMEM_COLS)
                 : "memory");
  }
}

// ------------------------------------------------- CTA-pair kernel (cta_group::2)
// A cluster of two CTAs owns a 256 x 256 output tile.  CTA r (cluster rank r) holds A rows
// m0 + 128 r and B rows n0 + 128 r of each K-slice in its own shared memory; the even CTA
// issues tcgen05.mma.cta_group::2 (M = 256, N = 256), which reads both CTAs' operands and
// writes CTA r's 128 output rows into CTA r's TMEM.  Per SM and K-slice of 64 BF16 the
// TMA brings 32 KB (48 KB for a one-CTA 128 x 256 tile) and per K=16 step the MMA reads
// 8 KB of shared memory (12 KB): the one-CTA tile asks the shared memory for about 1.5x
// the bandwidth the tensor core's rate leaves it, the pair stays within it, and the
// 32 KB stage leaves room for 6 stages.  TF32 slices are 32 elements of the same 128
// bytes; 3xTF32 stages hold hi and lo planes (64 KB, 3 stages) and take three MMAs per
// K step.
//
// Barriers: full[s] lives in the even CTA; its producer arms it with both CTAs' bytes and
// both CTAs' loads (.cta_group::2) complete on it.  empty[s] and acc_full[b] live in both
// CTAs and take the even CTA's multicast commits.  acc_empty[b] lives in the even CTA and
// counts the pair's 8 epilogue warps.
template <int MODE, int STAGES>
struct PairCfg {
  static constexpr int BN = 256;
  static constexpr int KELEMS = MODE == BF16 ? 64 : 32;
  static constexpr int A_BYTES = BM * 128;          // this CTA's 128 A rows x 128 B of K
  static constexpr int B_BYTES = 128 * 128;         // this CTA's 128 B rows
  static constexpr int SPLIT = MODE == TF32X3 ? 2 : 1;   // hi (and lo) operand planes
  static constexpr int STAGE_BYTES = (A_BYTES + B_BYTES) * SPLIT;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 + 256;
  static constexpr int TMEM_COLS = 256;             // per accumulator buffer
  static_assert(SMEM <= 227 * 1024, "shared memory");
  static_assert((2 * STAGES + 5) * 8 + 8 <= 256, "barrier area");
};

// Work items of the pair kernel.  Items [0, full) are whole tiles (units).  When the last
// round of tiles would leave clusters idle, the `tail` units after them are each cut into
// S pieces along K (items [full, full + tail S)): piece p sums K-slices
// [p nk / S, (p+1) nk / S) and writes its FP32 partial tile to ws; the last piece of a
// tile to finish (per CTA half and epilogue warp, counted in cnt) adds the S partials in
// piece order and stores the tile, so the result does not depend on which piece ends last.
struct PairSched {
  int full, tail, S;
  float* ws;          // [tail * S][256 columns][256 rows]
  int* cnt;           // [tail][2 CTAs][4 warps], zero at launch, reset by the last piece
};

__device__ __forceinline__ void pair_item(const PairSched& sp, int item, int nk, int& u,
                                          int& kb0, int& kb1, int& t) {
  if (item < sp.full) {
    u = item;
    kb0 = 0;
    kb1 = nk;
    t = -1;
  } else {
    t = item - sp.full;
    const int p = t % sp.S;
    u = sp.full + t / sp.S;
    kb0 = (int)((int64_t)p * nk / sp.S);
    kb1 = (int)((int64_t)(p + 1) * nk / sp.S);
  }
}

// One row of a K-split tile: the S partial rows at w0 (pieces 65536 floats apart, columns
// 256 apart) summed in piece order into C.  All 32 S loads of a 32-column chunk are issued
// before the first add.
template <int S, int OUT>
__device__ __forceinline__ void sum_pieces(const float* w0, char* base, int64_t ldc, int n0,
                                           int N) {
  constexpr int es = OUT == 1 ? 8 : OUT == 2 ? 2 : 4;
#pragma unroll 1
  for (int c0 = 0; c0 < 256; c0 += 32) {
    float v[S][32];
#pragma unroll
    for (int pc = 0; pc < S; pc++)
#pragma unroll
      for (int j = 0; j < 32; j++)
        v[pc][j] = __ldcg(w0 + (int64_t)pc * 65536 + (int64_t)(c0 + j) * 256);
    uint32_t r[32];
#pragma unroll
    for (int j = 0; j < 32; j++) {
      float a = v[0][j];
#pragma unroll
      for (int pc = 1; pc < S; pc++) a += v[pc][j];
      r[j] = __float_as_uint(a);
    }
    store_cols<OUT>(base + es * ldc * c0, ldc, n0 + c0, N, r);
  }
}

template <int MODE, int STAGES, int OUT>
__global__ void __launch_bounds__(NTHREADS, 1)
    gemm_pair_kernel(const __grid_constant__ CUtensorMap mapA,
                     const __grid_constant__ CUtensorMap mapB,
                     const __grid_constant__ CUtensorMap mapA2,
                     const __grid_constant__ CUtensorMap mapB2, int K, int tiles_m2, int tiles_n,
                     int batch, EpiArgs ep, PairSched sp) {
  // Persistent over work items: cluster c (CTAs 2c, 2c+1) takes items c, c + clusters, ...
  // Warp roles as in gemm_kernel; only the even CTA's warp 1 issues MMAs.
  using C_ = PairCfg<MODE, STAGES>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * C_::STAGE_BYTES);
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = bars + 2 * STAGES + 2;
  uint64_t* drain = bars + 2 * STAGES + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t rank = cluster_rank();
  const bool lead = rank == 0;
  const int cl = blockIdx.x >> 1, ncl = gridDim.x >> 1;
  const int nk = (K + C_::KELEMS - 1) / C_::KELEMS;
  const int num_items = sp.full + sp.tail * sp.S;
  (void)batch;
  // stage s: [A hi][B hi] and, for 3xTF32, [A lo][B lo]
  auto stageA = [&](int s, int part) {
    return smem + s * C_::STAGE_BYTES + part * (C_::A_BYTES + C_::B_BYTES);
  };
  auto stageB = [&](int s, int part) { return stageA(s, part) + C_::A_BYTES; };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[STAGES + s]), 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), 8);          // 4 epilogue warps in each CTA
    }
    mbar_init(smem_u32(drain), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
    if (MODE == TF32X3) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA2)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB2)) : "memory");
    }
  }
  if (warp == 1) {
    // one warp of each CTA allocates the pair's accumulator columns together
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * C_::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync();                 // both CTAs' barriers exist before either signals the other
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int it = 0, last = -1;
      for (int item = cl; item < num_items && !*abort_flag; item += ncl) {
        int u, kb0, kb1, t, mt2, nt, z;
        pair_item(sp, item, nk, u, kb0, kb1, t);
        tile_coords(u, tiles_m2, tiles_n, ep.nfast, mt2, nt, z);
        // a half tile wholly past the last row or column is loaded from the last one: the
        // MMA then fills only accumulator rows / columns the epilogue does not store
        const int m0 = min(mt2 * 2 * BM + (int)rank * BM, ep.M - 1);
        const int n0 = min(nt * C_::BN + (int)rank * 128, ep.N - 1);
        for (int kb = kb0; kb < kb1; kb++, it++) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!mbar_wait(smem_u32(&bars[STAGES + s]), ph ^ 1, abort_flag, ep.err)) break;
          const uint32_t full = smem_u32(&bars[s]);
          if (lead) mbar_expect_tx(full, 2 * C_::STAGE_BYTES);
          const uint32_t full_lead = cluster_addr(full, 0);
          const int kc = kb * C_::KELEMS;
          tma_load_3d_pair(smem_u32(stageA(s, 0)), &mapA, full_lead, kc, m0, z);
          tma_load_3d_pair(smem_u32(stageB(s, 0)), &mapB, full_lead, kc, n0, z);
          if (MODE == TF32X3) {
            tma_load_3d_pair(smem_u32(stageA(s, 1)), &mapA2, full_lead, kc, m0, z);
            tma_load_3d_pair(smem_u32(stageB(s, 1)), &mapB2, full_lead, kc, n0, z);
          }
          last = it;
        }
      }
      if (*abort_flag && last >= 0) {
        // every load this thread issued must land before the CTA exits: the even CTA
        // watches the full barriers; the odd CTA's loads complete on the even CTA's
        // barriers, so it allows them a fixed, ample time
        const unsigned long long t0 = globaltimer();
        if (lead) {
          for (int j = max(0, last - STAGES + 1); j <= last; j++) {
            const uint32_t bar = smem_u32(&bars[j % STAGES]);
            while (!mbar_try(bar, (j / STAGES) & 1) && globaltimer() - t0 < WAIT_NS) {
            }
          }
        } else {
          while (globaltimer() - t0 < 1000000ull) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      constexpr uint32_t idesc = make_idesc(MODE, 2 * BM, C_::BN);
      int it = 0, local = 0;
      for (int item = cl; item < num_items && !*abort_flag; item += ncl, local++) {
        int u, kb0, kb1, t;
        pair_item(sp, item, nk, u, kb0, kb1, t);
        const int buf = local & 1;
        const uint32_t use = (uint32_t)(local >> 1);
        if (!mbar_wait(smem_u32(&acc_empty[buf]), (use & 1) ^ 1, abort_flag, ep.err)) break;
        tc_fence_after();
        const uint32_t tacc = tmem + buf * C_::TMEM_COLS;
        for (int kb = kb0; kb < kb1; kb++, it++) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1;
          if (!mbar_wait(smem_u32(&bars[s]), ph, abort_flag, ep.err)) break;
          tc_fence_after();
          const uint32_t a0 = smem_u32(stageA(s, 0)), b0 = smem_u32(stageB(s, 0));
#pragma unroll
          for (int ks = 0; ks < 4; ks++) {
            const uint32_t acc = (kb > kb0 || ks > 0) ? 1u : 0u;
            const uint64_t ad = smem_desc(a0 + ks * 32), bd = smem_desc(b0 + ks * 32);
            mma_pair<MODE>(tacc, ad, bd, idesc, acc);
            if (MODE == TF32X3) {                  // hi*hi + hi*lo + lo*hi
              const uint32_t a1 = smem_u32(stageA(s, 1)), b1 = smem_u32(stageB(s, 1));
              mma_pair<MODE>(tacc, ad, smem_desc(b1 + ks * 32), idesc, 1u);
              mma_pair<MODE>(tacc, smem_desc(a1 + ks * 32), bd, idesc, 1u);
            }
          }
          mma_commit_pair(smem_u32(&bars[STAGES + s]), 3);     // frees the stage in both CTAs
        }
        mma_commit_pair(smem_u32(&acc_full[buf]), 3);          // both halves of the tile ready
      }
    }
  } else {
    const int q = warp & 3;
    int local = 0;
    for (int item = cl; item < num_items; item += ncl, local++) {
      int u, kb0, kb1, t, mt2, nt, z;
      pair_item(sp, item, nk, u, kb0, kb1, t);
      const int buf = local & 1;
      const uint32_t use = (uint32_t)(local >> 1);
      const bool ok = mbar_wait(smem_u32(&acc_full[buf]), use & 1, abort_flag, ep.err);
      if (!ok || *abort_flag) break;
      tc_fence_after();
      tile_coords(u, tiles_m2, tiles_n, ep.nfast, mt2, nt, z);
      const int rloc = (int)rank * BM + 32 * q + lane;          // row within the 256-row tile
      const int row = mt2 * 2 * BM + rloc;
      const uint32_t tbase = tmem + buf * C_::TMEM_COLS + ((uint32_t)(32 * q) << 16);
      if (t < 0) {
        store_acc<C_::BN, OUT>(tbase, row, nt * C_::BN, z, ep);
      } else {
        EpiArgs pe{sp.ws + (int64_t)t * 65536, 256, 0, 256, 256, ep.err, 0};
        store_acc<C_::BN, 0>(tbase, rloc, 0, 0, pe);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive_cluster(cluster_addr(smem_u32(&acc_empty[buf]), 0));
      if (t >= 0) {
        // publish this piece, then the last of the S pieces sums them in piece order
        __threadfence();
        __syncwarp();
        const int ut = u - sp.full;
        int* c = sp.cnt + (ut * 2 + (int)rank) * 4 + q;
        int prev = 0;
        if (lane == 0) prev = atomicAdd(c, 1);
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev == sp.S - 1) {
          __threadfence();
          const float* w0 = sp.ws + (int64_t)ut * sp.S * 65536 + rloc;
          if (row < ep.M) {
            const int n0 = nt * C_::BN;
            char* base = static_cast<char*>(ep.C) +
                         (OUT == 1 ? 8 : OUT == 2 ? 2 : 4) *
                             ((int64_t)row + ep.strideC * z + ep.ldc * n0);
            if (sp.S == 2)
              sum_pieces<2, OUT>(w0, base, ep.ldc, n0, ep.N);
            else if (sp.S == 3)
              sum_pieces<3, OUT>(w0, base, ep.ldc, n0, ep.N);
            else
              sum_pieces<4, OUT>(w0, base, ep.ldc, n0, ep.N);
          }
          __syncwarp();
          if (lane == 0) *c = 0;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1 && lead) {
    tc_fence_after();
    if (lane == 0) {
      // every MMA of the pair has retired before either CTA releases TMEM or exits
      mma_commit_pair(smem_u32(drain), 1);
      const unsigned long long t0 = globaltimer();
      while (!mbar_try(smem_u32(drain), 0) && globaltimer() - t0 < WAIT_NS) {
      }
    }
    __syncwarp();
  }
  cluster_sync();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * C_::TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------- tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn(fmpt_handle* h) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  (void)h;
  return fn;
}

int make_map(fmpt_handle* h, CUtensorMap* map, const void* base, int mode, int64_t K,
             int64_t rows, int64_t ld, int64_t batch, int64_t bstride, int box_rows) {
  EncodeTiledFn fn = encode_fn(h);
  if (!fn) return set_error(h, FMPT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const int es = mode == BF16 ? 2 : 4;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * es) % 16 || (bstride * es) % 16)
    return set_error(h, FMPT_ERR_SHAPE, "tensor map: operand not 16-byte aligned");
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)std::max<int64_t>(batch, 1)};
  cuuint64_t strides[2] = {(cuuint64_t)(ld * es), (cuuint64_t)(std::max<int64_t>(bstride, ld * rows) * es)};
  cuuint32_t box[3] = {(cuuint32_t)(128 / es), (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, mode == BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                  3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(h, FMPT_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return FMPT_OK;
}

}  // namespace tc

// ----------------------------------------------------- CTA-pair launch
// FMPT_ERR_UNSUPPORTED (nothing launched) when no cluster of two fits on the device.
template <int MODE, int ST>
static int tc_gemm_pair_st(fmpt_handle* h, int M, int N, int K, int batch, const TcOperand& A,
                           const TcOperand& B, const tc::EpiArgs& ep, int out_f64) {
  using namespace tc;
  using C_ = PairCfg<MODE, ST>;
  CUtensorMap ma, mb, ma2, mb2;
  FMPT_TRY(make_map(h, &ma, A.hi, MODE, K, M, A.ld, batch, A.bstride, BM));
  FMPT_TRY(make_map(h, &mb, B.hi, MODE, K, N, B.ld, batch, B.bstride, 128));
  if (MODE == TF32X3) {
    if (!A.lo || !B.lo) return set_error(h, FMPT_ERR_ARG, "3xTF32 needs lo planes");
    FMPT_TRY(make_map(h, &ma2, A.lo, MODE, K, M, A.ld, batch, A.bstride, BM));
    FMPT_TRY(make_map(h, &mb2, B.lo, MODE, K, N, B.ld, batch, B.bstride, 128));
  } else {
    ma2 = ma;
    mb2 = mb;
  }
  const int tiles_m2 = (M + 2 * BM - 1) / (2 * BM), tiles_n = (N + C_::BN - 1) / C_::BN;
  const int64_t units = (int64_t)tiles_m2 * tiles_n * batch;
  if (units > INT32_MAX) return set_error(h, FMPT_ERR_SHAPE, "tc_gemm: too many tiles");
  void (*kfn)(CUtensorMap, CUtensorMap, CUtensorMap, CUtensorMap, int, int, int, int, EpiArgs,
              PairSched) =
      out_f64 == 1   ? gemm_pair_kernel<MODE, ST, 1>
      : out_f64 == 2 ? gemm_pair_kernel<MODE, ST, MODE == BF16 ? 2 : 0>
                     : gemm_pair_kernel<MODE, ST, 0>;
  const int vi = out_f64 == 1 ? 1 : out_f64 == 2 ? 2 : 0;
  static int clusters[3] = {-1, -1, -1};           // resident 2-CTA clusters, per variant
  cudaLaunchConfig_t cfg{};
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = C_::SMEM;
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (clusters[vi] < 0) {
    FMPT_CUDA(h, cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, C_::SMEM));
    cfg.gridDim = dim3(2 * std::max(1, h->sm_count / 2));
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kfn, &cfg) != cudaSuccess) {
      (void)cudaGetLastError();
      n = 0;
    }
    clusters[vi] = n;
  }
  if (clusters[vi] <= 0) return FMPT_ERR_UNSUPPORTED;
  // Whole tiles fill rounds of `cl` clusters; when the last round holds R < cl / 2 tiles,
  // those are cut along K into S = min(4, cl / R) pieces (at least 4 K-slices each), so
  // the round ends after about 1/S of a tile instead of a whole one.
  const int cl = clusters[vi];
  const int nk = (K + C_::KELEMS - 1) / C_::KELEMS;
  PairSched sp{(int)units, 0, 1, nullptr, nullptr};
  const int rem = (int)(units % cl);
  const int S = rem > 0 ? std::min(std::min(4, cl / rem), nk / 4) : 1;
  if (S >= 2) {
    const size_t part = (size_t)rem * S * 65536 * sizeof(float);
    const size_t need = part + (size_t)rem * 8 * sizeof(int);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(h->stream, &cs) != cudaSuccess) {
      (void)cudaGetLastError();
      cs = cudaStreamCaptureStatusActive;
    }
    // the workspace is grown outside stream capture only; inside, an undersized one
    // leaves the last round whole
    if (h->tc_ws_bytes < need && cs == cudaStreamCaptureStatusNone)
      FMPT_TRY(grow_buffer(h, &h->tc_ws, &h->tc_ws_bytes, need));
    if (h->tc_ws_bytes >= need) {
      sp.full = (int)(units - rem);
      sp.tail = rem;
      sp.S = S;
      sp.ws = static_cast<float*>(h->tc_ws);
      sp.cnt = reinterpret_cast<int*>(static_cast<char*>(h->tc_ws) + part);
      FMPT_CUDA(h, cudaMemsetAsync(sp.cnt, 0, (size_t)rem * 8 * sizeof(int), h->stream));
    }
  }
  const int64_t items = (int64_t)sp.full + (int64_t)sp.tail * sp.S;
  cfg.gridDim = dim3((unsigned)(2 * std::min<int64_t>(items, cl)));
  ProfScope prof(h, FMPT_K_TC_GEMM);
  FMPT_CUDA(h, cudaLaunchKernelEx(&cfg, kfn, ma, mb, ma2, mb2, K, tiles_m2, tiles_n, batch, ep, sp));
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

// 6 stages: on the D=2048 step 5 stages measured 2% slower and 7 no faster
static int tc_gemm_pair(fmpt_handle* h, int mode, int M, int N, int K, int batch,
                        const TcOperand& A, const TcOperand& B, const tc::EpiArgs& ep,
                        int out_f64) {
  if (mode == tc::TF32) return tc_gemm_pair_st<tc::TF32, 6>(h, M, N, K, batch, A, B, ep, out_f64);
  if (mode == tc::TF32X3)
    return tc_gemm_pair_st<tc::TF32X3, 3>(h, M, N, K, batch, A, B, ep, out_f64);
  return tc_gemm_pair_st<tc::BF16, 6>(h, M, N, K, batch, A, B, ep, out_f64);
}

// ----------------------------------------------------- public engine call
int tc_gemm(fmpt_handle* h, int mode, int M, int N, int K, int batch, const TcOperand& A,
            const TcOperand& B, void* C, int out_f64, int64_t ldc, int64_t strideC, int* err_dev) {
  using namespace tc;
  if (M <= 0 || N <= 0 || K <= 0 || batch <= 0) return FMPT_OK;
  EpiArgs ep{C, ldc, strideC, M, N, err_dev, M > N ? 1 : 0};   // A and B share K
  // GEMMs of more than one 128-row tile run on the CTA-pair kernel (256 x 256 tiles; 6
  // stages of 32 KB, or 3 of 64 KB for the hi/lo planes of 3xTF32) unless the handle asks
  // for the one-CTA tile.  Average per
  // BF16 GEMM of the D=2048 step: one CTA 0.2363 ms; pair 0.2200 ms; pair with the
  // overlapped 32-column TMEM epilogue 0.1964 ms (the 16-column load-wait-store epilogue
  // had not kept up with the K = 2048 main loop of GEMM 1); K-split last round 0.1904 ms.
  if (M > BM && h->tc_tile == 0) {
    int st = tc_gemm_pair(h, mode, M, N, K, batch, A, B, ep, out_f64);
    if (st != FMPT_ERR_UNSUPPORTED) return st;
  }
  CUtensorMap ma, mb, ma2, mb2;
  // One-CTA kernel: 256-wide N tiles with 4 stages for TF32/BF16.  Measured on the D=2048
  // step (average per GEMM, 16-column epilogue): 256 x 4 stages 0.2455 ms; 256 x 3 stages 0.2743 ms; 192 x 5 stages 0.2576 ms;
  // 128 x 6 stages 0.2745 ms.  Pipeline depth matters, but not at the cost of the
  // 256-wide MMA's operand reuse.
  const int BN = mode == TF32X3 ? 128 : 256;
  FMPT_TRY(make_map(h, &ma, A.hi, mode, K, M, A.ld, batch, A.bstride, BM));
  FMPT_TRY(make_map(h, &mb, B.hi, mode, K, N, B.ld, batch, B.bstride, BN));
  if (mode == TF32X3) {
    if (!A.lo || !B.lo) return set_error(h, FMPT_ERR_ARG, "3xTF32 needs lo planes");
    FMPT_TRY(make_map(h, &ma2, A.lo, mode, K, M, A.ld, batch, A.bstride, BM));
    FMPT_TRY(make_map(h, &mb2, B.lo, mode, K, N, B.ld, batch, B.bstride, BN));
  } else {
    ma2 = ma;
    mb2 = mb;
  }
  const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const int64_t tiles = (int64_t)tiles_m * tiles_n * batch;
  if (tiles > INT32_MAX) return set_error(h, FMPT_ERR_SHAPE, "tc_gemm: too many tiles");
  const int sms = h->sm_count > 0 ? h->sm_count : 1;
  dim3 grid((unsigned)std::min<int64_t>(tiles, sms), 1, 1);
  ProfScope prof(h, FMPT_K_TC_GEMM);
#define LAUNCH(MODE_, BN_, ST_, OUT_)                                                         \
  do {                                                                                        \
    auto kfn = gemm_kernel<MODE_, BN_, ST_, OUT_>;                                            \
    constexpr int SM_ = Cfg<MODE_, BN_, ST_, OUT_>::SMEM;                                      \
    static bool attr_done = false;                                                            \
    if (!attr_done) {                                                                         \
      FMPT_CUDA(h, cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_)); \
      attr_done = true;                                                                       \
    }                                                                                         \
    kfn<<<grid, NTHREADS, SM_, h->stream>>>(ma, mb, ma2, mb2, K, tiles_m, tiles_n, batch, ep); \
  } while (0)
  if (mode == TF32) {
    if (out_f64) LAUNCH(TF32, 256, 4, 1); else LAUNCH(TF32, 256, 4, 0);
  } else if (mode == TF32X3) {
    if (out_f64) LAUNCH(TF32X3, 128, 3, 1); else LAUNCH(TF32X3, 128, 3, 0);
  } else {
    if (out_f64 == 1) LAUNCH(BF16, 256, 4, 1);
    else if (out_f64 == 2) LAUNCH(BF16, 256, 4, 2);
    else LAUNCH(BF16, 256, 4, 0);
  }
#undef LAUNCH
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

}  // namespace fmpt
