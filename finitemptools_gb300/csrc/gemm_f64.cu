// Plain FP64 (and split-plane complex FP64) GEMM on the CUDA cores.
//
// GB300's FP64 rate is small (about 2 DFMA per clock per SM), so this kernel
// is FP64-pipe bound for every shape that matters, and what decides its speed
// is how evenly it spreads the multiply-adds over the SMs.  Large problems use a
// 64x64 tile with a 4x4 register block per thread.  Small ones (the D <= 128
// contractions of TDVP and of the first DMRG bonds) use 32x32 or 16x16 tiles
// and may split K over the grid; a cost model picks the tile and the split that
// put the fewest multiply-adds on the busiest SM.  Every split writes its
// partial product to a workspace; the last split of a tile to finish (an atomic
// count per tile) sums the tile's partials in split order, so the result does
// not depend on scheduling, applies alpha/beta and resets the count.  Where no
// count is available (a stream capture before the counts exist) a second kernel
// does the same sum.
#include "internal.h"

namespace fmpt {
namespace {

constexpr int BK = 8, NT = 256;

// op(X)(r, c) with trans code: 0 N, 1 T, 2 C, 3 R(conj, no transpose)
__device__ __forceinline__ int64_t a_index(int t, int r, int c, int64_t ld) {
  return (t == 0 || t == 3) ? (int64_t)r + (int64_t)c * ld : (int64_t)c + (int64_t)r * ld;
}

// C (or the split workspace) = op(A) op(B) over k in [k_lo, k_hi).
// gridDim.z = batch * splits; with splits > 1 (batch == 1) the raw partial
// product goes to ws + split * plane_ws (re, then im plane at + m*n).
template <bool CPLX, int BMN>
__global__ void __launch_bounds__(NT) gemm_kernel(GemmArgs g, int splits, int kchunk,
                                                  double* __restrict__ ws,
                                                  int* __restrict__ tile_cnt) {
  constexpr int TPR = BMN / 16;                // outputs per thread along each dimension
  __shared__ double As[2][BK][BMN + 1];
  __shared__ double Bs[2][BK][BMN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.x * BMN, n0 = blockIdx.y * BMN;
  const int zb = blockIdx.z / splits, sp = blockIdx.z % splits;
  const int k_lo = sp * kchunk;
  const int k_hi = min(g.k, k_lo + kchunk);
  const double* A = g.A + zb * g.strideA;
  const double* B = g.B + zb * g.strideB;
  const bool conjA = (g.ta == 2 || g.ta == 3);
  const bool conjB = (g.tb == 2 || g.tb == 3);
  const bool a_mfast = (g.ta == 0 || g.ta == 3);   // op(A) rows contiguous
  const bool b_kfast = (g.tb == 0 || g.tb == 3);   // op(B) rows (k) contiguous

  double acc[TPR][TPR], acci[TPR][TPR];
#pragma unroll
  for (int i = 0; i < TPR; i++)
#pragma unroll
    for (int j = 0; j < TPR; j++) { acc[i][j] = 0.0; acci[i][j] = 0.0; }

  // The K slab k0 .. k0 + BK of A and B goes global -> registers -> shared memory; the
  // next slab's loads are issued before the current one is multiplied, so that their
  // latency overlaps the FMAs (a small GEMM runs one block per SM and has nothing else to
  // hide it behind).  The products are summed in the same order as without it.
  constexpr int NE = (BMN * BK + NT - 1) / NT;       // slab elements per thread and operand
  double ra[NE][2], rb[NE][2];
  auto load_slab = [&](int k0) {
#pragma unroll
    for (int q = 0; q < NE; q++) {
      const int e = tid + q * NT;
      ra[q][0] = ra[q][1] = rb[q][0] = rb[q][1] = 0.0;
      if (e >= BMN * BK) continue;
      int mm, kk;
      if (a_mfast) { mm = e % BMN; kk = e / BMN; } else { kk = e % BK; mm = e / BK; }
      int gm = m0 + mm, gk = k0 + kk;
      if (gm < g.m && gk < k_hi) {
        const int64_t idx = a_index(g.ta, gm, gk, g.lda);
        ra[q][0] = __ldg(A + idx);
        if (CPLX) { ra[q][1] = __ldg(A + g.planeA + idx); if (conjA) ra[q][1] = -ra[q][1]; }
      }
      int nn;
      if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BMN; kk = e / BMN; }
      const int gn = n0 + nn;
      gk = k0 + kk;
      if (gn < g.n && gk < k_hi) {
        const int64_t idx = a_index(g.tb, gk, gn, g.ldb);
        rb[q][0] = __ldg(B + idx);
        if (CPLX) { rb[q][1] = __ldg(B + g.planeB + idx); if (conjB) rb[q][1] = -rb[q][1]; }
      }
    }
  };
  auto store_slab = [&]() {
#pragma unroll
    for (int q = 0; q < NE; q++) {
      const int e = tid + q * NT;
      if (e >= BMN * BK) continue;
      int mm, kk;
      if (a_mfast) { mm = e % BMN; kk = e / BMN; } else { kk = e % BK; mm = e / BK; }
      As[0][kk][mm] = ra[q][0];
      if (CPLX) As[1][kk][mm] = ra[q][1];
      int nn;
      if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BMN; kk = e / BMN; }
      Bs[0][kk][nn] = rb[q][0];
      if (CPLX) Bs[1][kk][nn] = rb[q][1];
    }
  };
  if (k_lo < k_hi) load_slab(k_lo);
  for (int k0 = k_lo; k0 < k_hi; k0 += BK) {
    store_slab();
    __syncthreads();
    if (k0 + BK < k_hi) load_slab(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double a[TPR], b[TPR], ai[TPR], bi[TPR];
#pragma unroll
      for (int i = 0; i < TPR; i++) {
        a[i] = As[0][kk][tx + 16 * i];
        b[i] = Bs[0][kk][ty + 16 * i];
        if (CPLX) { ai[i] = As[1][kk][tx + 16 * i]; bi[i] = Bs[1][kk][ty + 16 * i]; }
      }
#pragma unroll
      for (int i = 0; i < TPR; i++)
#pragma unroll
        for (int j = 0; j < TPR; j++) {
          if (CPLX) {
            acc[i][j] = fma(a[i], b[j], acc[i][j]);
            acc[i][j] = fma(-ai[i], bi[j], acc[i][j]);
            acci[i][j] = fma(a[i], bi[j], acci[i][j]);
            acci[i][j] = fma(ai[i], b[j], acci[i][j]);
          } else {
            acc[i][j] = fma(a[i], b[j], acc[i][j]);
          }
        }
    }
    __syncthreads();
  }
  // ---- epilogue
  if (splits > 1) {
    const int64_t mn = (int64_t)g.m * g.n;
    double* W = ws + (int64_t)sp * mn * (CPLX ? 2 : 1);
#pragma unroll
    for (int i = 0; i < TPR; i++) {
      const int gm = m0 + tx + 16 * i;
      if (gm >= g.m) continue;
#pragma unroll
      for (int j = 0; j < TPR; j++) {
        const int gn = n0 + ty + 16 * j;
        if (gn >= g.n) continue;
        const int64_t idx = (int64_t)gm + (int64_t)gn * g.m;
        W[idx] = acc[i][j];
        if (CPLX) W[mn + idx] = acci[i][j];
      }
    }
    if (!tile_cnt) return;                 // the reduction kernel sums the splits
    // the last split of this tile to arrive sums the partials in split order
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    const int tile = (blockIdx.y * gridDim.x + blockIdx.x) + (int)(gridDim.x * gridDim.y) * zb;
    if (tid == 0) {
      const int prev = atomicAdd(tile_cnt + tile, 1);
      s_last = prev == splits - 1;
      if (s_last) tile_cnt[tile] = 0;      // ready for the next launch (stream order)
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const bool has_beta = (g.beta[0] != 0.0 || g.beta[1] != 0.0);
    double* C = g.C + zb * g.strideC;
#pragma unroll
    for (int i = 0; i < TPR; i++) {
      const int gm = m0 + tx + 16 * i;
      if (gm >= g.m) continue;
#pragma unroll
      for (int j = 0; j < TPR; j++) {
        const int gn = n0 + ty + 16 * j;
        if (gn >= g.n) continue;
        const int64_t t = (int64_t)gm + (int64_t)gn * g.m;
        double sr = 0.0, si = 0.0;
        for (int q = 0; q < splits; q++) {
          const double* Wq = ws + (int64_t)q * mn * (CPLX ? 2 : 1);
          sr += __ldcg(Wq + t);
          if (CPLX) si += __ldcg(Wq + mn + t);
        }
        const int64_t idx = (int64_t)gm + (int64_t)gn * g.ldc;
        if (CPLX) {
          double r = g.alpha[0] * sr - g.alpha[1] * si;
          double im = g.alpha[0] * si + g.alpha[1] * sr;
          if (has_beta) {
            const double cr = C[idx], ci = C[g.planeC + idx];
            r += g.beta[0] * cr - g.beta[1] * ci;
            im += g.beta[0] * ci + g.beta[1] * cr;
          }
          C[idx] = r;
          C[g.planeC + idx] = im;
        } else {
          double r = g.alpha[0] * sr;
          if (has_beta) r += g.beta[0] * C[idx];
          C[idx] = r;
        }
      }
    }
    return;
  }
  double* C = g.C + zb * g.strideC;
  const bool has_beta = (g.beta[0] != 0.0 || g.beta[1] != 0.0);
#pragma unroll
  for (int i = 0; i < TPR; i++) {
    const int gm = m0 + tx + 16 * i;
    if (gm >= g.m) continue;
#pragma unroll
    for (int j = 0; j < TPR; j++) {
      const int gn = n0 + ty + 16 * j;
      if (gn >= g.n) continue;
      const int64_t idx = (int64_t)gm + (int64_t)gn * g.ldc;
      if (CPLX) {
        double r = g.alpha[0] * acc[i][j] - g.alpha[1] * acci[i][j];
        double im = g.alpha[0] * acci[i][j] + g.alpha[1] * acc[i][j];
        if (has_beta) {
          const double cr = C[idx], ci = C[g.planeC + idx];
          r += g.beta[0] * cr - g.beta[1] * ci;
          im += g.beta[0] * ci + g.beta[1] * cr;
        }
        C[idx] = r;
        C[g.planeC + idx] = im;
      } else {
        double r = g.alpha[0] * acc[i][j];
        if (has_beta) r += g.beta[0] * C[idx];
        C[idx] = r;
      }
    }
  }
}

// C = alpha * sum_{s < splits} W_s + beta * C, summed in split order
template <bool CPLX>
__global__ void split_reduce(GemmArgs g, int splits, const double* __restrict__ ws) {
  const int64_t mn = (int64_t)g.m * g.n;
  const bool has_beta = (g.beta[0] != 0.0 || g.beta[1] != 0.0);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < mn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int gm = (int)(t % g.m), gn = (int)(t / g.m);
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < splits; s++) {
      const double* W = ws + (int64_t)s * mn * (CPLX ? 2 : 1);
      sr += W[t];
      if (CPLX) si += W[mn + t];
    }
    const int64_t idx = (int64_t)gm + (int64_t)gn * g.ldc;
    if (CPLX) {
      double r = g.alpha[0] * sr - g.alpha[1] * si;
      double im = g.alpha[0] * si + g.alpha[1] * sr;
      if (has_beta) {
        const double cr = g.C[idx], ci = g.C[g.planeC + idx];
        r += g.beta[0] * cr - g.beta[1] * ci;
        im += g.beta[0] * ci + g.beta[1] * cr;
      }
      g.C[idx] = r;
      g.C[g.planeC + idx] = im;
    } else {
      double r = g.alpha[0] * sr;
      if (has_beta) r += g.beta[0] * g.C[idx];
      g.C[idx] = r;
    }
  }
}

// Per-tile split counters (zeroed once, left zero by every launch): enough for any grid
// the cost model below may choose with a split.
constexpr int kMaxSplitTiles = 1 << 14;

template <bool CPLX>
int launch(fmpt_handle* h, const GemmArgs& g) {
  const int sms = h->sm_count > 0 ? h->sm_count : 1;
  // (tile edge, splits) with the fewest multiply-adds on the busiest SM; a split adds the
  // partials' round trip, priced as that many multiply-adds
  const double cm = CPLX ? 4.0 : 1.0;
  int bmn = 64, splits = 1;
  double best = 1e300;
  for (int e : {64, 32, 16}) {
    const int64_t t = (int64_t)((g.m + e - 1) / e) * ((g.n + e - 1) / e) * g.batch;
    for (int s = 1; s <= 64; s *= 2) {
      if (s > 1 && (g.batch != 1 || g.nosplit || g.k < 4 * BK || g.k / s < 2 * BK)) break;
      const int kc = s > 1 ? ((g.k + s - 1) / s + BK - 1) / BK * BK : g.k;
      const int64_t blocks = t * ((g.k + kc - 1) / kc);
      const int64_t per_sm = (blocks + sms - 1) / sms;
      double cost = (double)per_sm * e * e * kc * cm;
      if (s > 1) cost += 2.0e4 * cm + (double)s * e * e * cm * 4.0;
      if (e == 16) cost *= 1.15;               // one output per thread: more loads per FMA
      if (cost < best * 0.98) {
        best = cost;
        bmn = e;
        splits = s;
      }
    }
  }
  const int kchunk = splits > 1 ? ((g.k + splits - 1) / splits + BK - 1) / BK * BK : g.k;
  if (splits > 1) splits = (g.k + kchunk - 1) / kchunk;
  dim3 grid((g.m + bmn - 1) / bmn, (g.n + bmn - 1) / bmn, g.batch * splits);
  if (grid.y > 65535 || grid.z > 65535)
    return set_error(h, FMPT_ERR_SHAPE, "gemm: grid too large (%d x %d x %d)", grid.x, grid.y,
                     grid.z);
  // the split partials live in the handle's workspace (reused in stream order)
  double* ws = nullptr;
  int* cnt = nullptr;
  if (splits > 1) {
    FMPT_TRY(grow_buffer(h, &h->gemm_ws, &h->gemm_ws_bytes,
                         (size_t)splits * g.m * g.n * sizeof(double) * (CPLX ? 2 : 1)));
    ws = static_cast<double*>(h->gemm_ws);
    if ((int64_t)grid.x * grid.y * g.batch <= kMaxSplitTiles) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (!h->gemm_cnt && cudaStreamIsCapturing(h->stream, &cs) == cudaSuccess &&
          cs == cudaStreamCaptureStatusNone) {
        // created outside a stream capture only; inside one the reduction kernel runs
        FMPT_TRY(grow_buffer(h, &h->gemm_cnt, &h->gemm_cnt_bytes, kMaxSplitTiles * sizeof(int)));
        FMPT_CUDA(h, cudaMemsetAsync(h->gemm_cnt, 0, kMaxSplitTiles * sizeof(int), h->stream));
      }
      cudaGetLastError();
      cnt = static_cast<int*>(h->gemm_cnt);
    }
  }
  ProfScope prof(h, FMPT_K_F64_GEMM);
  if (bmn == 64)
    gemm_kernel<CPLX, 64><<<grid, NT, 0, h->stream>>>(g, splits, kchunk, ws, cnt);
  else if (bmn == 32)
    gemm_kernel<CPLX, 32><<<grid, NT, 0, h->stream>>>(g, splits, kchunk, ws, cnt);
  else
    gemm_kernel<CPLX, 16><<<grid, NT, 0, h->stream>>>(g, splits, kchunk, ws, cnt);
  FMPT_LAUNCHED(h);
  if (splits > 1 && !cnt) {
    const int64_t mn = (int64_t)g.m * g.n;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((mn + 255) / 256, 4LL * sms));
    split_reduce<CPLX><<<blocks, 256, 0, h->stream>>>(g, splits, ws);
    FMPT_LAUNCHED(h);
  }
  return FMPT_OK;
}

}  // namespace

int gemm_f64(fmpt_handle* h, const GemmArgs& g) {
  if (g.m < 0 || g.n < 0 || g.k < 0 || g.batch < 1)
    return set_error(h, FMPT_ERR_SHAPE, "gemm: negative extent");
  if (g.m == 0 || g.n == 0) return FMPT_OK;
  if (g.k == 0 && g.beta[0] == 1.0 && g.beta[1] == 0.0) return FMPT_OK;
  if (g.k > 0 && !g.nosplit && gemm_f64_ozaki_possible(h, g)) {
    const int st = gemm_f64_ozaki(h, g);
    // FMPT_ERR_UNSUPPORTED: nothing launched (no cluster fits, or its workspace would have
    // to grow inside a stream capture); the CUDA-core kernel runs instead
    if (st != FMPT_ERR_UNSUPPORTED) return st;
  }
  return g.cplx ? launch<true>(h, g) : launch<false>(h, g);
}

}  // namespace fmpt
