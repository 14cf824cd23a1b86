// Plain FP64 (and split-plane complex FP64) GEMM on the CUDA cores.
//
// GB300's FP64 rate is a small fraction of its tensor-core rates, so this
// kernel is FP64-pipe bound for every shape that matters: a 64x64 tile with a
// 4x4 register block per thread keeps shared-memory traffic far below the
// DFMA issue rate.  It is the arithmetic of the plain (FP64) form of every
// contraction in the library and of the small host-plumbing products
// (two-site tensor, gauge moves).
#include "internal.h"

namespace fmpt {
namespace {

constexpr int BM = 64, BN = 64, BK = 8, NT = 256;

// op(A)(m, k) with trans code: 0 N, 1 T, 2 C, 3 R(conj, no transpose)
__device__ __forceinline__ int64_t a_index(int t, int r, int c, int64_t ld) {
  // r: row of op(X), c: col of op(X)
  return (t == 0 || t == 3) ? (int64_t)r + (int64_t)c * ld : (int64_t)c + (int64_t)r * ld;
}

template <bool CPLX>
__global__ void __launch_bounds__(NT) gemm_kernel(GemmArgs g) {
  __shared__ double As[2][BK][BM + 1];
  __shared__ double Bs[2][BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int z = blockIdx.z;
  const double* A = g.A + z * g.strideA;
  const double* B = g.B + z * g.strideB;
  double* C = g.C + z * g.strideC;
  const bool conjA = (g.ta == 2 || g.ta == 3);
  const bool conjB = (g.tb == 2 || g.tb == 3);
  const bool a_mfast = (g.ta == 0 || g.ta == 3);   // op(A) rows contiguous
  const bool b_kfast = (g.tb == 0 || g.tb == 3);   // op(B) rows (k) contiguous

  double acc[4][4], acci[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) { acc[i][j] = 0.0; acci[i][j] = 0.0; }

  for (int k0 = 0; k0 < g.k; k0 += BK) {
    // ---- load op(A) tile (BM x BK) and op(B) tile (BK x BN)
#pragma unroll
    for (int r = 0; r < (BM * BK) / NT; r++) {
      int e = tid + r * NT;
      int mm, kk;
      if (a_mfast) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      int gm = m0 + mm, gk = k0 + kk;
      double vr = 0.0, vi = 0.0;
      if (gm < g.m && gk < g.k) {
        int64_t idx = a_index(g.ta, gm, gk, g.lda);
        vr = __ldg(A + idx);
        if (CPLX) { vi = __ldg(A + g.planeA + idx); if (conjA) vi = -vi; }
      }
      As[0][kk][mm] = vr;
      if (CPLX) As[1][kk][mm] = vi;
    }
#pragma unroll
    for (int r = 0; r < (BN * BK) / NT; r++) {
      int e = tid + r * NT;
      int nn, kk;
      if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      int gn = n0 + nn, gk = k0 + kk;
      double vr = 0.0, vi = 0.0;
      if (gn < g.n && gk < g.k) {
        int64_t idx = a_index(g.tb, gk, gn, g.ldb);
        vr = __ldg(B + idx);
        if (CPLX) { vi = __ldg(B + g.planeB + idx); if (conjB) vi = -vi; }
      }
      Bs[0][kk][nn] = vr;
      if (CPLX) Bs[1][kk][nn] = vi;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      double a[4], b[4], ai[4], bi[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        a[i] = As[0][kk][tx + 16 * i];
        b[i] = Bs[0][kk][ty + 16 * i];
        if (CPLX) { ai[i] = As[1][kk][tx + 16 * i]; bi[i] = Bs[1][kk][ty + 16 * i]; }
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
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
  const bool has_beta = (g.beta[0] != 0.0 || g.beta[1] != 0.0);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int gm = m0 + tx + 16 * i;
    if (gm >= g.m) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int gn = n0 + ty + 16 * j;
      if (gn >= g.n) continue;
      int64_t idx = (int64_t)gm + (int64_t)gn * g.ldc;
      if (CPLX) {
        double r = g.alpha[0] * acc[i][j] - g.alpha[1] * acci[i][j];
        double im = g.alpha[0] * acci[i][j] + g.alpha[1] * acc[i][j];
        if (has_beta) {
          double cr = C[idx], ci = C[g.planeC + idx];
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

}  // namespace

int gemm_f64(fmpt_handle* h, const GemmArgs& g) {
  if (g.m < 0 || g.n < 0 || g.k < 0 || g.batch < 1)
    return set_error(h, FMPT_ERR_SHAPE, "gemm: negative extent");
  if (g.m == 0 || g.n == 0) return FMPT_OK;
  if (g.k == 0 && g.beta[0] == 1.0 && g.beta[1] == 0.0) return FMPT_OK;
  dim3 grid((g.m + BM - 1) / BM, (g.n + BN - 1) / BN, g.batch);
  if (grid.y > 65535 || grid.z > 65535)
    return set_error(h, FMPT_ERR_SHAPE, "gemm: grid too large (%d x %d x %d)", grid.x, grid.y,
                     grid.z);
  ProfScope prof(h, FMPT_K_F64_GEMM);
  if (g.cplx)
    gemm_kernel<true><<<grid, NT, 0, h->stream>>>(g);
  else
    gemm_kernel<false><<<grid, NT, 0, h->stream>>>(g);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

}  // namespace fmpt
