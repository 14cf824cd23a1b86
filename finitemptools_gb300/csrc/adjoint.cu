// Reverse-mode building blocks for the differentiable one-site TDVP.
//
// The adjoint of every contraction on the TDVP path is again a contraction of
// the same GEMM shapes with L, W, R and x permuted (environment gradients are
// environment updates, site-tensor gradients are H_eff applications); those
// run on the existing kernels.  What is new here:
//   fmpt_wgrad      the MPO-tensor gradient  sum conj(a) L b R  -> [w, s', w2, s]
//   fmpt_swap13     X[i,j,k] -> X[k,j,i] (optionally conjugated): L^dagger, R^T
//   fmpt_qr_adjoint Mbar of the thin QR M = Q R with real diag(R) (LAPACK
//                   convention):  Mbar = (I - Q Q^H) Qbar R^-H + Q Y R^-H + Q Rbar,
//                   K = Qbar^H Q - R Rbar^H, Y lower triangular with
//                   Y_ij = conj(K_ji) - K_ij (i > j), Y_ii = -i Im K_ii.
// Complex data are split planes, as everywhere in libfmpt.
#include <algorithm>

#include "internal.h"

namespace fmpt {
namespace {

constexpr int AT = 256;

__device__ __forceinline__ double block_reduce(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < AT / 32 ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;   // valid in thread 0
}

// out[w, s', w2, s] = conj( sum_{a', b'} conj(a[a', s', b']) Q[a', w, s, b', w2] )
// one block per output entry, a fixed-order sum (deterministic)
__global__ void wgrad_reduce(int cplx, int Dl, int d, int Dr, int wl, int wr,
                             const double* __restrict__ a, int64_t pa,
                             const double* __restrict__ Q, int64_t pq, double* __restrict__ out,
                             int64_t po) {
  __shared__ double red[AT / 32];
  int o = blockIdx.x;
  const int w = o % wl; o /= wl;
  const int sp = o % d; o /= d;
  const int w2 = o % wr; o /= wr;
  const int s = o;
  double gr = 0.0, gi = 0.0;
  const int64_t tot = (int64_t)Dl * Dr;
  for (int64_t t = threadIdx.x; t < tot; t += AT) {
    const int ap = (int)(t % Dl), bp = (int)(t / Dl);
    const int64_t ia = ap + (int64_t)Dl * (sp + (int64_t)d * bp);
    const int64_t iq = ap + (int64_t)Dl * (w + (int64_t)wl * (s + (int64_t)d * (bp + (int64_t)Dr * w2)));
    const double ar = a[ia], qr = Q[iq];
    if (cplx) {
      const double ai = a[pa + ia], qi = Q[pq + iq];
      gr += ar * qr + ai * qi;
      gi += ar * qi - ai * qr;
    } else {
      gr += ar * qr;
    }
  }
  gr = block_reduce(gr, red);
  if (cplx) gi = block_reduce(gi, red);
  if (threadIdx.x == 0) {
    const int64_t io = w + (int64_t)wl * (sp + (int64_t)d * (w2 + (int64_t)wr * s));
    out[io] = gr;
    if (cplx) out[po + io] = -gi;
  }
}

// dst[k, j, i] = src[i, j, k] (conjugated when conj)
__global__ void swap13_kernel(int cplx, int n0, int n1, int n2, const double* __restrict__ src,
                              int64_t plane, int conj, double* __restrict__ dst) {
  const int64_t tot = (int64_t)n0 * n1 * n2;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n0);
    const int j = (int)((t / n0) % n1);
    const int k = (int)(t / ((int64_t)n0 * n1));
    const int64_t di = k + (int64_t)n2 * (j + (int64_t)n1 * i);
    dst[di] = src[t];
    if (cplx) dst[plane + di] = conj ? -src[plane + t] : src[plane + t];
  }
}

// Y (n x n, split planes) from K: lower triangle conj(K_ji) - K_ij, diagonal -i Im K_ii
__global__ void qr_adj_y(int n, const double* __restrict__ K, double* __restrict__ Y) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    double yr = 0.0, yi = 0.0;
    if (i > j) {
      const int64_t ji = j + (int64_t)n * i;
      yr = K[ji] - K[t];
      yi = -K[nn + ji] - K[nn + t];
    } else if (i == j) {
      yi = -K[nn + t];
    }
    Y[t] = yr;
    Y[nn + t] = yi;
  }
}

// X R^H = Z for every row of X (m x n, in place in Z); R upper triangular n x n.
// z_j = sum_{k >= j} x_k conj(R_jk): back substitution from j = n-1, one thread per row.
__global__ void trsm_rh(int m, int n, const double* __restrict__ R, int64_t pr,
                        double* __restrict__ Z, int64_t pz) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  for (int j = n - 1; j >= 0; j--) {
    double zr = Z[row + (int64_t)m * j], zi = Z[pz + row + (int64_t)m * j];
    for (int k = j + 1; k < n; k++) {
      const double xr = Z[row + (int64_t)m * k], xi = Z[pz + row + (int64_t)m * k];
      const double rr = R[j + (int64_t)n * k], ri = -R[pr + j + (int64_t)n * k];   // conj(R_jk)
      zr -= xr * rr - xi * ri;
      zi -= xr * ri + xi * rr;
    }
    const double dr = R[j + (int64_t)n * j], di = -R[pr + j + (int64_t)n * j];      // conj(R_jj)
    const double den = dr * dr + di * di;
    Z[row + (int64_t)m * j] = (zr * dr + zi * di) / den;
    Z[pz + row + (int64_t)m * j] = (zi * dr - zr * di) / den;
  }
}

GemmArgs cgemm(int ta, int tb, int m, int n, int k, double alpha, double beta, const double* A,
               int64_t lda, int64_t pA, const double* B, int64_t ldb, int64_t pB, double* C,
               int64_t ldc, int64_t pC) {
  GemmArgs g{};
  g.cplx = 1; g.ta = ta; g.tb = tb; g.m = m; g.n = n; g.k = k;
  g.alpha[0] = alpha; g.beta[0] = beta; g.batch = 1;
  g.A = A; g.lda = lda; g.planeA = pA;
  g.B = B; g.ldb = ldb; g.planeB = pB;
  g.C = C; g.ldc = ldc; g.planeC = pC;
  return g;
}

// dst(i, j) = src(i, j) for an m x n block; complex: split planes at the given offsets
__global__ void copy2d_kernel(int cplx, int m, int n, const double* __restrict__ src, int64_t lds,
                              int64_t ps, double* __restrict__ dst, int64_t ldd, int64_t pd) {
  const int64_t tot = (int64_t)m * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % m);
    const int64_t j = t / m;
    dst[i + ldd * j] = src[i + lds * j];
    if (cplx) dst[pd + i + ldd * j] = src[ps + i + lds * j];
  }
}

}  // namespace
}  // namespace fmpt

using namespace fmpt;

extern "C" {

int fmpt_wgrad(fmpt_handle* h, int dtype, const double* a, const double* Lenv, const double* b,
               const double* Renv, double* out, int Dl, int d, int Dr, int wl, int wr) {
  if (!h) return FMPT_ERR_ARG;
  if (!a || !Lenv || !b || !Renv || !out) return set_error(h, FMPT_ERR_ARG, "wgrad: null pointer");
  if (Dl < 1 || d < 1 || Dr < 1 || wl < 1 || wr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "wgrad: non-positive dimension");
  const int cp = dtype == FMPT_C128;
  const int64_t nP = (int64_t)Dl * wl * d * Dr, nQ = nP * wr;
  DevBuf P, Q;
  FMPT_TRY(P.alloc(h, nP * sizeof(double) * (cp ? 2 : 1)));
  FMPT_TRY(Q.alloc(h, nQ * sizeof(double) * (cp ? 2 : 1)));
  GemmArgs g{};
  g.cplx = cp; g.alpha[0] = 1.0; g.batch = 1;
  // P[(a' w), (s b)] = L[(a' w), a] b[a, (s b)]
  g.ta = FMPT_N; g.tb = FMPT_N; g.m = Dl * wl; g.n = d * Dr; g.k = Dl;
  g.A = Lenv; g.lda = (int64_t)Dl * wl; g.planeA = (int64_t)Dl * wl * Dl;
  g.B = b; g.ldb = Dl; g.planeB = (int64_t)Dl * d * Dr;
  g.C = P.d(); g.ldc = (int64_t)Dl * wl; g.planeC = nP;
  FMPT_TRY(gemm_f64(h, g));
  // Q[(a' w s), (b' w2)] = P[(a' w s), b] R[(b' w2), b]^T
  g.ta = FMPT_N; g.tb = FMPT_T; g.m = Dl * wl * d; g.n = Dr * wr; g.k = Dr;
  g.A = P.d(); g.lda = (int64_t)Dl * wl * d; g.planeA = nP;
  g.B = Renv; g.ldb = (int64_t)Dr * wr; g.planeB = (int64_t)Dr * wr * Dr;
  g.C = Q.d(); g.ldc = (int64_t)Dl * wl * d; g.planeC = nQ;
  FMPT_TRY(gemm_f64(h, g));
  const int nout = wl * d * wr * d;
  wgrad_reduce<<<nout, AT, 0, h->stream>>>(cp, Dl, d, Dr, wl, wr, a, (int64_t)Dl * d * Dr, Q.d(),
                                           nQ, out, nout);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int fmpt_copy2d(fmpt_handle* h, int dtype, int m, int n, const double* src, int64_t lds,
                int64_t plane_src, double* dst, int64_t ldd, int64_t plane_dst) {
  if (!h) return FMPT_ERR_ARG;
  if (m < 0 || n < 0) return set_error(h, FMPT_ERR_SHAPE, "copy2d: negative extent");
  if ((int64_t)m * n == 0) return FMPT_OK;
  if (!src || !dst) return set_error(h, FMPT_ERR_ARG, "copy2d: null pointer");
  if (lds < m || ldd < m) return set_error(h, FMPT_ERR_SHAPE, "copy2d: leading dimension < rows");
  const int64_t tot = (int64_t)m * n;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, 8LL * h->sm_count));
  copy2d_kernel<<<blocks, 256, 0, h->stream>>>(dtype == FMPT_C128, m, n, src, lds, plane_src, dst,
                                               ldd, plane_dst);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int fmpt_swap13(fmpt_handle* h, int dtype, const double* src, double* dst, int n0, int n1, int n2,
                int conj) {
  if (!h) return FMPT_ERR_ARG;
  if (!src || !dst) return set_error(h, FMPT_ERR_ARG, "swap13: null pointer");
  if (n0 < 1 || n1 < 1 || n2 < 1) return set_error(h, FMPT_ERR_SHAPE, "swap13: bad extents");
  if (src == dst) return set_error(h, FMPT_ERR_ARG, "swap13: out of place only");
  const int64_t tot = (int64_t)n0 * n1 * n2;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, 8LL * h->sm_count));
  swap13_kernel<<<blocks, 256, 0, h->stream>>>(dtype == FMPT_C128, n0, n1, n2, src, tot, conj, dst);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int fmpt_qr_adjoint(fmpt_handle* h, int dtype, const double* Q, const double* R, const double* Qbar,
                    const double* Rbar, double* Mbar, int m, int n) {
  if (!h) return FMPT_ERR_ARG;
  if (!Q || !R || !Qbar || !Rbar || !Mbar) return set_error(h, FMPT_ERR_ARG, "qr_adjoint: null");
  if (dtype != FMPT_C128)
    return set_error(h, FMPT_ERR_UNSUPPORTED, "qr_adjoint: complex (C128) data only");
  if (m < n || n < 1) return set_error(h, FMPT_ERR_SHAPE, "qr_adjoint: needs m >= n >= 1");
  const int64_t mn = (int64_t)m * n, nn = (int64_t)n * n;
  DevBuf K, Y, T;
  FMPT_TRY(K.alloc(h, 2 * nn * sizeof(double)));
  FMPT_TRY(Y.alloc(h, 2 * nn * sizeof(double)));
  FMPT_TRY(T.alloc(h, 2 * nn * sizeof(double)));
  // K = Qbar^H Q - R Rbar^H
  FMPT_TRY(gemm_f64(h, cgemm(FMPT_C, FMPT_N, n, n, m, 1.0, 0.0, Qbar, m, mn, Q, m, mn, K.d(), n, nn)));
  FMPT_TRY(gemm_f64(h, cgemm(FMPT_N, FMPT_C, n, n, n, -1.0, 1.0, R, n, nn, Rbar, n, nn, K.d(), n, nn)));
  qr_adj_y<<<(unsigned)std::max<int64_t>(1, (nn + 255) / 256), 256, 0, h->stream>>>(n, K.d(), Y.d());
  FMPT_LAUNCHED(h);
  // Z = Qbar - Q (Q^H Qbar) + Q Y   (in Mbar)
  FMPT_CUDA(h, cudaMemcpyAsync(Mbar, Qbar, 2 * mn * sizeof(double), cudaMemcpyDeviceToDevice,
                               h->stream));
  FMPT_TRY(gemm_f64(h, cgemm(FMPT_C, FMPT_N, n, n, m, 1.0, 0.0, Q, m, mn, Qbar, m, mn, T.d(), n, nn)));
  FMPT_TRY(gemm_f64(h, cgemm(FMPT_N, FMPT_N, m, n, n, -1.0, 1.0, Q, m, mn, T.d(), n, nn, Mbar, m, mn)));
  FMPT_TRY(gemm_f64(h, cgemm(FMPT_N, FMPT_N, m, n, n, 1.0, 1.0, Q, m, mn, Y.d(), n, nn, Mbar, m, mn)));
  // Mbar = Z R^-H + Q Rbar
  trsm_rh<<<(m + 127) / 128, 128, 0, h->stream>>>(m, n, R, nn, Mbar, mn);
  FMPT_LAUNCHED(h);
  FMPT_TRY(gemm_f64(h, cgemm(FMPT_N, FMPT_N, m, n, n, 1.0, 1.0, Q, m, mn, Rbar, n, nn, Mbar, m, mn)));
  return FMPT_OK;
}

}  // extern "C"
