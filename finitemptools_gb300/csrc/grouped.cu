// Grouped persistent FP64 engine for block-sparse (U(1) charge-sector)
// contractions.
//
// A GroupedProgram is a short sequence of phases; each phase is a list of
// uneven block problems:
//   GEMM phase:  C_p = sum_{j in segs(p)} coef_j * op(A_j) op(B_j)     (overwrite)
//   SUM  phase:  C_p = sum_{j in segs(p)} coef_j * op(A_j)             (overwrite)
// where every operand is a strided sub-matrix (offset + leading dimension) of
// one of a few operand slots (device base pointers given at run time).  The
// whole program runs as ONE cooperative launch: CTAs pull 32x32 output tiles
// of the current phase from a device work counter (atomicAdd, largest blocks
// first) and meet at a grid barrier between phases.  The barrier spin is
// bounded (2 s on %globaltimer); on timeout a CTA sets the launch's abort
// flag and the handle's status word, and every CTA returns.
//
// Each output tile sums its segments in the order they were added, so the
// result does not depend on scheduling.  FP64 is FMA-pipe bound on GB300
// (about 2 DFMA per clock per SM), so the kernel's job is to keep every SM's
// FP64 pipe fed across thousands of 1..400-wide blocks.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <numeric>
#include <vector>

#include "internal.h"

namespace fmpt {
namespace {

constexpr int GK = 8, GNT = 256;
constexpr int kTile[2] = {32, 64};   // tile edge of kernel v & 1
// Schedules (v >> 1), the order in which the CTAs pull a phase's tiles:
//   0: blocks by descending work (sum of their segments' k), each block's tiles together;
//   1: tiles by descending work of their own (block work x the tile's 16-wide groups), so
//      that the narrow edge tiles of large blocks fall to the end of the phase.
// The schedule decides only which CTA runs a tile and when; every output tile sums its
// segments and k in the same order, so no variant changes a result.
constexpr uint64_t kBarrierTimeoutNs = 2000000000ull;

struct GKArgs {
  GPhaseDesc ph[GP_MAX_PHASES];
  int nphase;
  double* slot[GP_SLOTS];
  const GProblem* probs;
  const GSegment* segs;
  const int* tile_prob;
  const int* tile_mn;
  int* ctl;        // [0, GP_MAX_PHASES) tile counters, then barrier count, then abort flag
  int* status;     // handle status word (1 = a bounded wait gave up)
  const int* gate; // nonzero at launch: return at once (nullptr: always run)
  uint64_t wait_ns;   // bound of every barrier wait
  int hold;           // arrivals the barriers wait for beyond the grid (0; > 0 only to test
                      // the bounded wait: the barrier then gives up after wait_ns)
};

__device__ __forceinline__ int64_t op_index(int t, int r, int c, int64_t ld) {
  return (t == FMPT_N || t == FMPT_R) ? (int64_t)r + (int64_t)c * ld
                                      : (int64_t)c + (int64_t)r * ld;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid barrier for a cooperative launch; false when the launch aborts.
__device__ bool grid_barrier(const GKArgs& a, int target, int* s_flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int* bar = a.ctl + GP_MAX_PHASES;
    int* abort_flag = bar + 1;
    __threadfence();
    atomicAdd(bar, 1);
    int ok = 1;
    const uint64_t t0 = global_ns();
    // the count alone is polled; every 32nd poll also looks at the abort flag and the clock
    for (unsigned polls = 1; ld_acquire(bar) < target + a.hold; polls++) {
      if ((polls & 31u) != 0) continue;
      if (ld_acquire(abort_flag)) { ok = 0; break; }
      if (global_ns() - t0 > a.wait_ns) {
        atomicExch(abort_flag, 1);
        atomicExch(a.status, 1);
        ok = 0;
        break;
      }
    }
    __threadfence();
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

// Tile word: origin in 16-row / 16-column units and extent in 16-wide groups,
//   bits 0-11 m0 / 16, bits 12-23 n0 / 16, bits 24-27 MI - 1, bits 28-31 NJ - 1.
// A tile covers (16 MI) x (16 NJ) outputs; the last tile of a block along either
// dimension is only as many 16-wide groups as the block needs, so a 40-row block
// takes a 32-row and a 16-row tile instead of two 32-row tiles.
__host__ __device__ __forceinline__ uint32_t tile_word(int m16, int n16, int mi, int nj) {
  return (uint32_t)m16 | ((uint32_t)n16 << 12) | ((uint32_t)(mi - 1) << 24) |
         ((uint32_t)(nj - 1) << 28);
}
constexpr int kMaxTile16 = 0xfff;   // largest origin in 16-wide units

// One (16 MI)x(16 NJ) output tile of a GEMM problem: 256 threads on a 16x16 grid,
// each owning MI x NJ outputs at rows tx + 16 i, columns ty + 16 j.  Every output
// sums its segments and k in the same order for any tile shape, so the tiling
// never changes the result.  MI and NJ are compile-time, so a narrow edge tile
// issues no FP64 work for the rows or columns it does not hold.
template <int GT, int MI, int NJ>
__device__ __forceinline__ void gemm_tile(const GKArgs& a, const GPhaseDesc& ph, int t,
                                          double (*As)[GT + 1], double (*Bs)[GT + 1]) {
  constexpr int TM = 16 * MI, TN = 16 * NJ;
  const GProblem P = a.probs[a.tile_prob[t]];
  const uint32_t mn = (uint32_t)a.tile_mn[t];
  const int m0 = (int)(mn & 0xfffu) * 16, n0 = (int)((mn >> 12) & 0xfffu) * 16;
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const bool a_mfast = (ph.ta == FMPT_N || ph.ta == FMPT_R);
  const bool b_kfast = (ph.tb == FMPT_N || ph.tb == FMPT_R);
  const double* Ab = a.slot[ph.a_slot];
  const double* Bb = a.slot[ph.b_slot];
  double acc[MI][NJ];
#pragma unroll
  for (int i = 0; i < MI; i++)
#pragma unroll
    for (int j = 0; j < NJ; j++) acc[i][j] = 0.0;
  for (int sg = P.seg0; sg < P.seg1; sg++) {
    const GSegment S = a.segs[sg];
    const double* A = Ab + S.a_off;
    const double* B = Bb + S.b_off;
    for (int k0 = 0; k0 < S.k; k0 += GK) {
#pragma unroll
      for (int e = tid; e < TM * GK; e += GNT) {
        int mm, kk;
        if (a_mfast) { mm = e % TM; kk = e / TM; } else { kk = e % GK; mm = e / GK; }
        const int gm = m0 + mm, gk = k0 + kk;
        double v = 0.0;
        if (gm < P.m && gk < S.k) v = S.coef * __ldg(A + op_index(ph.ta, gm, gk, S.lda));
        As[kk][mm] = v;
      }
#pragma unroll
      for (int e = tid; e < TN * GK; e += GNT) {
        int nn, kk;
        if (b_kfast) { kk = e % GK; nn = e / GK; } else { nn = e % TN; kk = e / TN; }
        const int gn = n0 + nn, gk = k0 + kk;
        double v = 0.0;
        if (gn < P.n && gk < S.k) v = __ldg(B + op_index(ph.tb, gk, gn, S.ldb));
        Bs[kk][nn] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < GK; kk++) {
        double av[MI], bv[NJ];
#pragma unroll
        for (int i = 0; i < MI; i++) av[i] = As[kk][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < NJ; j++) bv[j] = Bs[kk][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < MI; i++)
#pragma unroll
          for (int j = 0; j < NJ; j++) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
      }
      __syncthreads();
    }
  }
  double* C = a.slot[ph.c_slot] + P.c_off;
#pragma unroll
  for (int i = 0; i < MI; i++) {
    const int r = m0 + tx + 16 * i;
    if (r >= P.m) continue;
#pragma unroll
    for (int j = 0; j < NJ; j++) {
      const int c = n0 + ty + 16 * j;
      if (c < P.n) C[r + (int64_t)c * P.ldc] = acc[i][j];
    }
  }
}

// the tile's extent (MI, NJ) picks the instantiation; uniform over the block
template <int GT, int MI = 1, int NJ = 1>
__device__ __forceinline__ void gemm_tile_any(const GKArgs& a, const GPhaseDesc& ph, int t,
                                              int mi, int nj, double (*As)[GT + 1],
                                              double (*Bs)[GT + 1]) {
  constexpr int TPR = GT / 16;
  if (mi == MI && nj == NJ) {
    gemm_tile<GT, MI, NJ>(a, ph, t, As, Bs);
  } else if constexpr (NJ < TPR) {
    gemm_tile_any<GT, MI, NJ + 1>(a, ph, t, mi, nj, As, Bs);
  } else if constexpr (MI < TPR) {
    gemm_tile_any<GT, MI + 1, 1>(a, ph, t, mi, nj, As, Bs);
  }
}

template <int GT>
__device__ __forceinline__ void sum_tile(const GKArgs& a, const GPhaseDesc& ph, int t) {
  const GProblem P = a.probs[a.tile_prob[t]];
  const uint32_t mn = (uint32_t)a.tile_mn[t];
  const int m0 = (int)(mn & 0xfffu) * 16, n0 = (int)((mn >> 12) & 0xfffu) * 16;
  const int r = m0 + (threadIdx.x % GT);
  if (r >= P.m) return;
  const double* Ab = a.slot[ph.a_slot];
  double* C = a.slot[ph.c_slot] + P.c_off;
  constexpr int CSTEP = GNT / GT;
#pragma unroll 4
  for (int j = 0; j < GT / CSTEP; j++) {
    const int c = n0 + threadIdx.x / GT + j * CSTEP;
    if (c >= P.n) break;
    double s = 0.0;
    for (int sg = P.seg0; sg < P.seg1; sg++) {
      const GSegment S = a.segs[sg];
      s = fma(S.coef, __ldg(Ab + S.a_off + op_index(ph.ta, r, c, S.lda)), s);
    }
    C[r + (int64_t)c * P.ldc] = s;
  }
}

template <int GT>
__global__ void __launch_bounds__(GNT) grouped_kernel(const GKArgs a) {
  __shared__ double As[GK][GT + 1];
  __shared__ double Bs[GK][GT + 1];
  __shared__ int s_tile, s_flag;
  if (a.gate && *a.gate) return;   // uniform for the whole grid: set before the launch
  for (int p = 0; p < a.nphase; p++) {
    if (p > 0 && !grid_barrier(a, p * (int)gridDim.x, &s_flag)) return;
    const GPhaseDesc ph = a.ph[p];
    const int ntiles = ph.tile1 - ph.tile0;
    while (true) {
      __syncthreads();
      if (threadIdx.x == 0) s_tile = atomicAdd(a.ctl + p, 1);
      __syncthreads();
      const int t = s_tile;
      if (t >= ntiles) break;
      if (ph.type == GP_GEMM) {
        const uint32_t mn = (uint32_t)a.tile_mn[ph.tile0 + t];
        gemm_tile_any<GT>(a, ph, ph.tile0 + t, (int)((mn >> 24) & 0xfu) + 1,
                          (int)(mn >> 28) + 1, As, Bs);
      } else
        sum_tile<GT>(a, ph, ph.tile0 + t);
    }
  }
}

int g_occupancy[2] = {0, 0};
std::mutex g_occ_mu;

int kernel_occupancy(fmpt_handle* h, int variant) {
  const int v = variant & 1;
  std::lock_guard<std::mutex> lock(g_occ_mu);
  if (g_occupancy[v] == 0) {
    int occ = 0;
    if (v == 0)
      FMPT_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, grouped_kernel<32>, GNT, 0));
    else
      FMPT_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, grouped_kernel<64>, GNT, 0));
    g_occupancy[v] = std::max(1, std::min(occ, 8));
  }
  return g_occupancy[v];
}

}  // namespace

void gp_phase(GroupedProgram& g, int type, int ta, int tb, int a_slot, int b_slot, int c_slot) {
  GPhaseDesc d{};
  d.type = type; d.ta = ta; d.tb = tb;
  d.a_slot = a_slot; d.b_slot = b_slot; d.c_slot = c_slot;
  g.phases.push_back(d);
  g.phase_prob0.push_back((int)g.probs.size());
}

int gp_problem(GroupedProgram& g, int64_t c_off, int64_t ldc, int m, int n) {
  GProblem p{};
  p.c_off = c_off; p.ldc = ldc; p.m = m; p.n = n;
  p.seg0 = p.seg1 = (int)g.segs.size();
  g.probs.push_back(p);
  return (int)g.probs.size() - 1;
}

void gp_segment(GroupedProgram& g, int64_t a_off, int64_t lda, int64_t b_off, int64_t ldb, int k,
                double coef) {
  GSegment s{};
  s.a_off = a_off; s.lda = lda; s.b_off = b_off; s.ldb = ldb; s.coef = coef; s.k = k;
  g.segs.push_back(s);
  GProblem& p = g.probs.back();
  p.seg1 = (int)g.segs.size();
  if (g.phases.back().type == GP_GEMM)
    g.flops += 2.0 * p.m * (double)p.n * k;
  else
    g.sum_elems += (double)p.m * p.n;
}

void gp_slot(GroupedProgram& g, int slot, int64_t elems) {
  if (slot >= 0 && slot < GP_SLOTS) g.slot_elems[slot] = elems;
}

namespace {

// Largest element index of op(X) (rows x cols, leading dimension ld) at offset off.
int64_t footprint(int t, int64_t off, int rows, int cols, int64_t ld) {
  const bool n = (t == FMPT_N || t == FMPT_R);
  return n ? off + (rows - 1) + (int64_t)(cols - 1) * ld : off + (cols - 1) + (int64_t)(rows - 1) * ld;
}

int check_span(fmpt_handle* h, const GroupedProgram& g, int slot, int t, int64_t off, int rows,
               int cols, int64_t ld, const char* what, int prob) {
  if (rows <= 0 || cols <= 0) return FMPT_OK;
  if (slot < 0 || slot >= GP_SLOTS || g.slot_elems[slot] < 0)
    return set_error(h, FMPT_ERR_ARG, "grouped: slot %d of %s has no declared extent", slot, what);
  const int64_t lead = (t == FMPT_N || t == FMPT_R) ? rows : cols;
  if (off < 0 || ld < lead || footprint(t, off, rows, cols, ld) >= g.slot_elems[slot])
    return set_error(h, FMPT_ERR_SHAPE,
                     "grouped: %s of block %d (offset %lld, %d x %d, ld %lld) outside its operand "
                     "(%lld elements)", what, prob, (long long)off, rows, cols, (long long)ld,
                     (long long)g.slot_elems[slot]);
  return FMPT_OK;
}

int validate(fmpt_handle* h, const GroupedProgram& g) {
  for (size_t ph = 0; ph < g.phases.size(); ph++) {
    const GPhaseDesc& d = g.phases[ph];
    for (int i = g.phase_prob0[ph]; i < g.phase_prob0[ph + 1]; i++) {
      const GProblem& p = g.probs[i];
      if (p.m < 0 || p.n < 0 || p.seg0 < 0 || p.seg1 > (int)g.segs.size() || p.seg0 > p.seg1)
        return set_error(h, FMPT_ERR_SHAPE, "grouped: malformed block %d", i);
      FMPT_TRY(check_span(h, g, d.c_slot, FMPT_N, p.c_off, p.m, p.n, p.ldc, "output", i));
      for (int s = p.seg0; s < p.seg1; s++) {
        const GSegment& sg = g.segs[s];
        if (d.type == GP_GEMM) {
          if (sg.k < 0) return set_error(h, FMPT_ERR_SHAPE, "grouped: negative k in block %d", i);
          if (sg.k == 0) continue;
          FMPT_TRY(check_span(h, g, d.a_slot, d.ta, sg.a_off, p.m, sg.k, sg.lda, "A operand", i));
          FMPT_TRY(check_span(h, g, d.b_slot, d.tb, sg.b_off, sg.k, p.n, sg.ldb, "B operand", i));
        } else {
          FMPT_TRY(check_span(h, g, d.a_slot, d.ta, sg.a_off, p.m, p.n, sg.lda, "summand", i));
        }
      }
    }
  }
  return FMPT_OK;
}

}  // namespace

int gp_finalize(fmpt_handle* h, GroupedProgram& g) {
  if ((int)g.phases.size() > GP_MAX_PHASES)
    return set_error(h, FMPT_ERR_UNSUPPORTED, "grouped: more than %d phases", GP_MAX_PHASES);
  g.phase_prob0.push_back((int)g.probs.size());
  FMPT_TRY(validate(h, g));
  g.tile_prob.clear();
  g.tile_mn.clear();
  int max_tiles[GP_VARIANTS] = {0, 0, 0, 0};
  for (int v = 0; v < GP_VARIANTS; v++) {
    const int GT = kTile[v & 1], sched = v >> 1;
    g.vtile0[v].assign(g.phases.size(), 0);
    g.vtile1[v].assign(g.phases.size(), 0);
    for (size_t ph = 0; ph < g.phases.size(); ph++) {
      const int p0 = g.phase_prob0[ph], p1 = g.phase_prob0[ph + 1];
      // largest work per tile first, so the long tiles do not straggle at the end
      std::vector<int64_t> cost(p1 - p0, 0);
      for (int i = p0; i < p1; i++) {
        const GProblem& p = g.probs[i];
        for (int s = p.seg0; s < p.seg1; s++)
          cost[i - p0] += g.phases[ph].type == GP_GEMM ? g.segs[s].k : 1;
      }
      std::vector<int> order(p1 - p0);
      std::iota(order.begin(), order.end(), p0);
      std::stable_sort(order.begin(), order.end(),
                       [&](int x, int y) { return cost[x - p0] > cost[y - p0]; });
      g.vtile0[v][ph] = (int)g.tile_prob.size();
      const size_t first = g.tile_prob.size();
      std::vector<int64_t> tcost;            // schedule 1: work of each emitted tile
      for (int i : order) {
        const GProblem& p = g.probs[i];
        if (p.m <= 0 || p.n <= 0) continue;
        if ((p.m - 1) / 16 > kMaxTile16 || (p.n - 1) / 16 > kMaxTile16)
          return set_error(h, FMPT_ERR_SHAPE, "grouped: block %d x %d too large", p.m, p.n);
        // GEMM tiles: GT wide, the last one along each dimension cut to the 16-wide
        // groups the block needs; SUM tiles (memory-bound) stay GT x GT
        const bool gemm = g.phases[ph].type == GP_GEMM;
        const int g16m = (p.m + 15) / 16, g16n = (p.n + 15) / 16, TPR = GT / 16;
        for (int b = 0; b < g16n; b += TPR)
          for (int a = 0; a < g16m; a += TPR) {
            const int mi = gemm ? std::min(TPR, g16m - a) : TPR;
            const int nj = gemm ? std::min(TPR, g16n - b) : TPR;
            g.tile_prob.push_back(i);
            g.tile_mn.push_back((int)tile_word(a, b, mi, nj));
            tcost.push_back(cost[i - p0] * mi * nj);
          }
      }
      if (sched == 1) {
        const size_t nt = g.tile_prob.size() - first;
        std::vector<size_t> idx(nt);
        std::iota(idx.begin(), idx.end(), (size_t)0);
        std::stable_sort(idx.begin(), idx.end(),
                         [&](size_t x, size_t y) { return tcost[x] > tcost[y]; });
        std::vector<int> tp(nt), tm(nt);
        for (size_t q = 0; q < nt; q++) {
          tp[q] = g.tile_prob[first + idx[q]];
          tm[q] = g.tile_mn[first + idx[q]];
        }
        std::copy(tp.begin(), tp.end(), g.tile_prob.begin() + first);
        std::copy(tm.begin(), tm.end(), g.tile_mn.begin() + first);
      }
      g.vtile1[v][ph] = (int)g.tile_prob.size();
      max_tiles[v] = std::max(max_tiles[v], g.vtile1[v][ph] - g.vtile0[v][ph]);
    }
  }
  for (size_t ph = 0; ph < g.phases.size(); ph++) {
    g.phases[ph].tile0 = g.vtile0[0][ph];
    g.phases[ph].tile1 = g.vtile1[0][ph];
  }
  // one device allocation: problems | segments | tile_prob | tile_mn | control words
  auto up256 = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t bp = up256(g.probs.size() * sizeof(GProblem));
  const size_t bs = up256(g.segs.size() * sizeof(GSegment));
  const size_t bt = up256(g.tile_prob.size() * sizeof(int));
  const size_t ctl_bytes = 256;
  FMPT_TRY(g.dev.alloc(h, bp + bs + 2 * bt + ctl_bytes));
  char* base = static_cast<char*>(g.dev.p);
  g.d_probs = reinterpret_cast<GProblem*>(base);
  g.d_segs = reinterpret_cast<GSegment*>(base + bp);
  g.d_tile_prob = reinterpret_cast<int*>(base + bp + bs);
  g.d_tile_mn = reinterpret_cast<int*>(base + bp + bs + bt);
  g.d_ctl = reinterpret_cast<int*>(base + bp + bs + 2 * bt);
  // pageable-source copies return once the source is staged
  if (!g.probs.empty())
    FMPT_CUDA(h, cudaMemcpyAsync(g.d_probs, g.probs.data(), g.probs.size() * sizeof(GProblem),
                                 cudaMemcpyHostToDevice, h->stream));
  if (!g.segs.empty())
    FMPT_CUDA(h, cudaMemcpyAsync(g.d_segs, g.segs.data(), g.segs.size() * sizeof(GSegment),
                                 cudaMemcpyHostToDevice, h->stream));
  if (!g.tile_prob.empty()) {
    FMPT_CUDA(h, cudaMemcpyAsync(g.d_tile_prob, g.tile_prob.data(),
                                 g.tile_prob.size() * sizeof(int), cudaMemcpyHostToDevice,
                                 h->stream));
    FMPT_CUDA(h, cudaMemcpyAsync(g.d_tile_mn, g.tile_mn.data(), g.tile_mn.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, h->stream));
  }
  const int sms = h->sm_count > 0 ? h->sm_count : 1;
  for (int v = 0; v < GP_VARIANTS; v++) {
    const int occ = kernel_occupancy(h, v);
    if (occ <= 0) return set_error(h, FMPT_ERR_CUDA, "grouped: occupancy query failed");
    g.vgrid[v] = std::max(1, std::min(max_tiles[v], occ * sms));
  }
  g.ready = true;
  return FMPT_OK;
}

int gp_autotune(fmpt_handle* h, GroupedProgram& g, double* const* slots, int nslots, int kind) {
  if (h->tune_mode >= 1 && h->tune_mode <= GP_VARIANTS) {
    g.variant = h->tune_mode - 1;
    return FMPT_OK;
  }
  g.variant = 0;
  // small programs: the 32x32 tile balances better and timing costs more than it saves
  if (g.flops < 2.0e7 || g.tile_prob.empty()) return FMPT_OK;
  const int key = kind * 1000 + (int)std::floor(std::log2(g.flops) * 2.0);
  auto it = h->tune_cache.find(key);
  if (it != h->tune_cache.end()) {
    g.variant = it->second;
    return FMPT_OK;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return FMPT_OK;   // no timing inside a capture: keep the default
  }
  cudaEvent_t e0, e1;
  FMPT_CUDA(h, cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return set_error(h, FMPT_ERR_CUDA, "autotune: event creation failed");
  }
  int best = 0, st = FMPT_OK;
  float best_ms = 0.f;
  for (int v = 0; v < GP_VARIANTS && st == FMPT_OK; v++) {
    st = gp_run(h, g, slots, nslots, nullptr, v);          // warm-up
    if (st == FMPT_OK && cudaEventRecord(e0, h->stream) != cudaSuccess) st = FMPT_ERR_CUDA;
    for (int r = 0; r < 3 && st == FMPT_OK; r++) st = gp_run(h, g, slots, nslots, nullptr, v);
    if (st == FMPT_OK && cudaEventRecord(e1, h->stream) != cudaSuccess) st = FMPT_ERR_CUDA;
    float ms = 0.f;
    if (st == FMPT_OK &&
        (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      st = FMPT_ERR_CUDA;
    if (st == FMPT_OK && (v == 0 || ms < best_ms)) { best = v; best_ms = ms; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != FMPT_OK) return st == FMPT_ERR_CUDA ? set_error(h, st, "autotune: timing failed") : st;
  h->tune_cache[key] = best;
  h->tune_runs++;
  g.variant = best;
  return FMPT_OK;
}

int gp_status_word(fmpt_handle* h, int** out) {
  if (!h->gstatus) {
    FMPT_CUDA(h, cudaMalloc(&h->gstatus, sizeof(int)));
    FMPT_CUDA(h, cudaMemsetAsync(h->gstatus, 0, sizeof(int), h->stream));
  }
  *out = h->gstatus;
  return FMPT_OK;
}

int gp_check_status(fmpt_handle* h) {
  if (!h->gstatus) return FMPT_OK;
  // a local word (not the shared pinned staging buffer, which callers may
  // still be reading from)
  int v = 0;
  FMPT_CUDA(h, cudaMemcpyAsync(&v, h->gstatus, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  if (v != 0) {
    FMPT_CUDA(h, cudaMemsetAsync(h->gstatus, 0, sizeof(int), h->stream));
    return set_error(h, FMPT_ERR_TIMEOUT,
                     "a bounded device wait timed out (grouped block-sparse launch or FP64 "
                     "tensor-core GEMM; results invalid)");
  }
  return FMPT_OK;
}

int gp_prepare(fmpt_handle* h) {
  int* st = nullptr;
  FMPT_TRY(gp_status_word(h, &st));
  for (int v = 0; v < GP_VARIANTS; v++)
    if (kernel_occupancy(h, v) <= 0) return FMPT_ERR_CUDA;
  return FMPT_OK;
}

int gp_run(fmpt_handle* h, const GroupedProgram& g, double* const* slots, int nslots,
           const int* gate, int variant) {
  if (!g.ready) return set_error(h, FMPT_ERR_ARG, "grouped: program not finalised");
  if (g.tile_prob.empty()) return FMPT_OK;
  const int v = variant < 0 ? g.variant : variant;
  if (v < 0 || v >= GP_VARIANTS) return set_error(h, FMPT_ERR_ARG, "grouped: variant %d", v);
  GKArgs a{};
  a.nphase = (int)g.phases.size();
  for (int p = 0; p < a.nphase; p++) {
    a.ph[p] = g.phases[p];
    a.ph[p].tile0 = g.vtile0[v][p];
    a.ph[p].tile1 = g.vtile1[v][p];
  }
  for (int s = 0; s < GP_SLOTS; s++) a.slot[s] = s < nslots ? slots[s] : nullptr;
  for (int p = 0; p < a.nphase; p++) {
    const GPhaseDesc& d = a.ph[p];
    if (d.tile1 == d.tile0) continue;
    if (!a.slot[d.a_slot] || !a.slot[d.c_slot] || (d.type == GP_GEMM && !a.slot[d.b_slot]))
      return set_error(h, FMPT_ERR_ARG, "grouped: operand slot of phase %d is null", p);
  }
  a.probs = g.d_probs; a.segs = g.d_segs;
  a.tile_prob = g.d_tile_prob; a.tile_mn = g.d_tile_mn;
  a.ctl = g.d_ctl;
  a.gate = gate;
  a.wait_ns = h->wait_test_ns > 0 ? (uint64_t)h->wait_test_ns : kBarrierTimeoutNs;
  a.hold = h->wait_test_hold;
  FMPT_TRY(gp_status_word(h, &a.status));
  FMPT_CUDA(h, cudaMemsetAsync(g.d_ctl, 0, (GP_MAX_PHASES + 2) * sizeof(int), h->stream));
  ProfScope prof(h, FMPT_K_GROUPED);
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(g.vgrid[v]);
  cfg.blockDim = dim3(GNT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if ((v & 1) == 0)
    FMPT_CUDA(h, cudaLaunchKernelEx(&cfg, grouped_kernel<32>, a));
  else
    FMPT_CUDA(h, cudaLaunchKernelEx(&cfg, grouped_kernel<64>, a));
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

}  // namespace fmpt
