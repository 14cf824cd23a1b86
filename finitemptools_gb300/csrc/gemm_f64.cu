// Plain FP64 (and split-plane complex FP64) GEMM on the CUDA cores.
//
// GB300's FP64 rate is small (about 2 DFMA per clock per SM), so this kernel
// is FP64-pipe bound for every shape that matters, and what decides its speed
// is how many SMs it keeps busy.  Large problems use a 64x64 tile with a 4x4
// register block per thread.  Small ones (the D <= 128 contractions of TDVP
// and of the first DMRG bonds) use 32x32 tiles and, when that still leaves
// SMs idle, split K over the grid: every split writes its partial product to
// a workspace and a second kernel sums the splits in a fixed order (so the
// result does not depend on scheduling) and applies alpha/beta.
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
                                                  double* __restrict__ ws) {
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

  for (int k0 = k_lo; k0 < k_hi; k0 += BK) {
    for (int e = tid; e < BMN * BK; e += NT) {
      int mm, kk;
      if (a_mfast) { mm = e % BMN; kk = e / BMN; } else { kk = e % BK; mm = e / BK; }
      const int gm = m0 + mm, gk = k0 + kk;
      double vr = 0.0, vi = 0.0;
      if (gm < g.m && gk < k_hi) {
        const int64_t idx = a_index(g.ta, gm, gk, g.lda);
        vr = __ldg(A + idx);
        if (CPLX) { vi = __ldg(A + g.planeA + idx); if (conjA) vi = -vi; }
      }
      As[0][kk][mm] = vr;
      if (CPLX) As[1][kk][mm] = vi;
    }
    for (int e = tid; e < BMN * BK; e += NT) {
      int nn, kk;
      if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BMN; kk = e / BMN; }
      const int gn = n0 + nn, gk = k0 + kk;
      double vr = 0.0, vi = 0.0;
      if (gn < g.n && gk < k_hi) {
        const int64_t idx = a_index(g.tb, gk, gn, g.ldb);
        vr = __ldg(B + idx);
        if (CPLX) { vi = __ldg(B + g.planeB + idx); if (conjB) vi = -vi; }
      }
      Bs[0][kk][nn] = vr;
      if (CPLX) Bs[1][kk][nn] = vi;
    }
    __syncthreads();
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

template <bool CPLX>
int launch(fmpt_handle* h, const GemmArgs& g) {
  const int sms = h->sm_count > 0 ? h->sm_count : 1;
  const int64_t want = 2LL * sms;                      // blocks that keep every SM busy
  auto tiles = [&](int bmn) {
    return (int64_t)((g.m + bmn - 1) / bmn) * ((g.n + bmn - 1) / bmn) * g.batch;
  };
  int bmn = 64;
  if (tiles(64) < want) bmn = 32;
  int splits = 1;
  const int64_t t = tiles(bmn);
  if (t < want && g.batch == 1 && g.k >= 4 * BK && !g.nosplit) {
    const int64_t by_grid = (want + t - 1) / t;
    const int64_t by_k = g.k / (2 * BK);               // at least 16 k per split
    splits = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(by_grid, by_k), 64));
  }
  const int kchunk = splits > 1 ? ((g.k + splits - 1) / splits + BK - 1) / BK * BK : g.k;
  if (splits > 1) splits = (g.k + kchunk - 1) / kchunk;
  dim3 grid((g.m + bmn - 1) / bmn, (g.n + bmn - 1) / bmn, g.batch * splits);
  if (grid.y > 65535 || grid.z > 65535)
    return set_error(h, FMPT_ERR_SHAPE, "gemm: grid too large (%d x %d x %d)", grid.x, grid.y,
                     grid.z);
  // the split partials live in the handle's workspace (reused in stream order)
  double* ws = nullptr;
  if (splits > 1) {
    FMPT_TRY(grow_buffer(h, &h->gemm_ws, &h->gemm_ws_bytes,
                         (size_t)splits * g.m * g.n * sizeof(double) * (CPLX ? 2 : 1)));
    ws = static_cast<double*>(h->gemm_ws);
  }
  ProfScope prof(h, FMPT_K_F64_GEMM);
  if (bmn == 64)
    gemm_kernel<CPLX, 64><<<grid, NT, 0, h->stream>>>(g, splits, kchunk, ws);
  else
    gemm_kernel<CPLX, 32><<<grid, NT, 0, h->stream>>>(g, splits, kchunk, ws);
  FMPT_LAUNCHED(h);
  if (splits > 1) {
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
