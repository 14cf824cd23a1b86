// Dense FP64 factorisations on the device through cuSOLVER: the truncated
// two-site SVD (auxiliary/stable_svd.jl + truncation.jl) and the QR/LQ gauge
// moves (leftorth!/rightorth with QR()/LQ()).  cuSOLVER is a library call;
// the truncation rule, the layout plumbing and the gesvd -> gesvdj fallback
// (the reference retries gesdd with gesvd) are here.
#include <cuComplex.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

namespace fmpt {
namespace {

// dst(i, j) = op(src)(i, j) for a rows x cols destination.
//   src/dst plane < 0: interleaved complex (re, im pairs); >= 0: split planes
//   trans: read src(j, i); conj: negate the imaginary part
__global__ void mat_copy(int cplx, int rows, int cols, const double* __restrict__ src,
                         int64_t s_ld, int64_t s_plane, int trans, int conj,
                         double* __restrict__ dst, int64_t d_ld, int64_t d_plane) {
  int64_t tot = (int64_t)rows * cols;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % rows), j = (int)(t / rows);
    int64_t si = trans ? (int64_t)j + (int64_t)i * s_ld : (int64_t)i + (int64_t)j * s_ld;
    int64_t di = (int64_t)i + (int64_t)j * d_ld;
    double re, im = 0.0;
    if (!cplx) {
      re = src[si];
    } else if (s_plane < 0) {
      re = src[2 * si]; im = src[2 * si + 1];
    } else {
      re = src[si]; im = src[s_plane + si];
    }
    if (conj) im = -im;
    if (!cplx) {
      dst[di] = re;
    } else if (d_plane < 0) {
      dst[2 * di] = re; dst[2 * di + 1] = im;
    } else {
      dst[di] = re; dst[d_plane + di] = im;
    }
  }
}

// zero the strictly lower triangle of a rows x cols (ld) matrix (split planes)
__global__ void zero_lower(int cplx, int rows, int cols, double* M, int64_t ld, int64_t plane) {
  int64_t tot = (int64_t)rows * cols;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % rows), j = (int)(t / rows);
    if (i > j) {
      M[i + j * ld] = 0.0;
      if (cplx) M[plane + i + j * ld] = 0.0;
    }
  }
}

}  // namespace

int copy_mat(fmpt_handle* h, int cplx, int rows, int cols, const double* src, int64_t s_ld,
             int64_t s_plane, int trans, int conj, double* dst, int64_t d_ld, int64_t d_plane) {
  int64_t tot = (int64_t)rows * cols;
  if (tot == 0) return FMPT_OK;
  int64_t g = std::min<int64_t>((tot + 255) / 256, (int64_t)h->sm_count * 8);
  mat_copy<<<(unsigned)std::max<int64_t>(g, 1), 256, 0, h->stream>>>(
      cplx, rows, cols, src, s_ld, s_plane, trans, conj, dst, d_ld, d_plane);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

#define FMPT_SOLVER(h, expr)                                                         \
  do {                                                                               \
    cusolverStatus_t _s = (expr);                                                    \
    if (_s != CUSOLVER_STATUS_SUCCESS)                                               \
      return set_error((h), FMPT_ERR_CUSOLVER, "%s:%d %s -> cusolver status %d",     \
                       __FILE__, __LINE__, #expr, (int)_s);                          \
  } while (0)

static int read_info(fmpt_handle* h, const int* dinfo, int* out) {
  FMPT_TRY(ensure_pinned(h, 1));
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, dinfo, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  *out = *reinterpret_cast<int*>(h->pinned);
  return FMPT_OK;
}

static int svd_tall_jacobi(fmpt_handle* h, int cplx, int m, int n, double* Awork, double* S,
                           double* U, double* VT);

// Thin SVD through the polar decomposition A = U_p H (cuSOLVER Xgesvdp, the
// QDWH iteration followed by an eigendecomposition of H): mostly level-3 work,
// where gesvd's bidiagonalisation is level-2 bound.  Returns FMPT_OK and
// *ok = false when the routine reports failure, so that the caller can fall
// back.  A is overwritten.
static int svd_tall_polar(fmpt_handle* h, int cplx, int m, int n, double* Awork, double* S,
                          double* U, double* VT, bool* ok) {
  *ok = false;
  cusolverDnParams_t params = nullptr;
  FMPT_SOLVER(h, cusolverDnCreateParams(&params));
  const cudaDataType dt = cplx ? CUDA_C_64F : CUDA_R_64F;
  DevBuf V, dinfo, wd;
  int st = V.alloc(h, (size_t)n * n * sizeof(double) * (cplx ? 2 : 1));
  if (st == FMPT_OK) st = dinfo.alloc(h, sizeof(int));
  size_t wdev = 0, whost = 0;
  cusolverStatus_t cs = CUSOLVER_STATUS_SUCCESS;
  if (st == FMPT_OK)
    cs = cusolverDnXgesvdp_bufferSize(h->solver, params, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, dt,
                                      Awork, m, CUDA_R_64F, S, dt, U, m, dt, V.p, n, dt, &wdev,
                                      &whost);
  std::vector<char> wh;
  if (st == FMPT_OK && cs == CUSOLVER_STATUS_SUCCESS) {
    st = wd.alloc(h, std::max<size_t>(wdev, 16));
    wh.resize(std::max<size_t>(whost, 16));
  }
  double err_sigma = 0.0;
  if (st == FMPT_OK && cs == CUSOLVER_STATUS_SUCCESS)
    cs = cusolverDnXgesvdp(h->solver, params, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, dt, Awork, m,
                           CUDA_R_64F, S, dt, U, m, dt, V.p, n, dt, wd.p, wdev, wh.data(), whost,
                           (int*)dinfo.p, &err_sigma);
  cusolverDnDestroyParams(params);
  FMPT_TRY(st);
  if (cs != CUSOLVER_STATUS_SUCCESS) return FMPT_OK;
  int info = 0;
  FMPT_TRY(read_info(h, (const int*)dinfo.p, &info));
  if (info != 0 || !std::isfinite(err_sigma)) return FMPT_OK;
  *ok = true;
  // VT = V^H (interleaved layout, n x n)
  return copy_mat(h, cplx, n, n, V.d(), n, cplx ? -1 : 0, 1, cplx, VT, n, cplx ? -1 : 0);
}

// Full thin SVD of a tall (m >= n) matrix given in solver layout (real, or
// interleaved complex) in Awork (overwritten).  U: m x n, S: n, VT: n x n.
// The handle's svd_method selects gesvd (default), the polar-decomposition SVD
// or the one-sided Jacobi SVD; a failure of the first two falls back to Jacobi.
int svd_tall(fmpt_handle* h, int cplx, int m, int n, double* Awork, double* S, double* U,
             double* VT) {
  if (h->svd_method == 2) return svd_tall_jacobi(h, cplx, m, n, Awork, S, U, VT);
  if (h->svd_method == 1) {
    DevBuf Acopy;
    const size_t abytes = (size_t)m * n * sizeof(double) * (cplx ? 2 : 1);
    FMPT_TRY(Acopy.alloc(h, abytes));
    FMPT_CUDA(h, cudaMemcpyAsync(Acopy.p, Awork, abytes, cudaMemcpyDeviceToDevice, h->stream));
    bool ok = false;
    FMPT_TRY(svd_tall_polar(h, cplx, m, n, Acopy.d(), S, U, VT, &ok));
    if (ok) return FMPT_OK;
  }
  DevBuf work, rwork, dinfo;
  FMPT_TRY(dinfo.alloc(h, sizeof(int)));
  int lwork = 0;
  if (cplx)
    FMPT_SOLVER(h, cusolverDnZgesvd_bufferSize(h->solver, m, n, &lwork));
  else
    FMPT_SOLVER(h, cusolverDnDgesvd_bufferSize(h->solver, m, n, &lwork));
  // gesvd destroys A: keep a copy for the Jacobi fallback
  DevBuf Acopy;
  const size_t abytes = (size_t)m * n * sizeof(double) * (cplx ? 2 : 1);
  FMPT_TRY(Acopy.alloc(h, abytes));
  FMPT_CUDA(h, cudaMemcpyAsync(Acopy.p, Awork, abytes, cudaMemcpyDeviceToDevice, h->stream));
  FMPT_TRY(work.alloc(h, (size_t)std::max(lwork, 1) * sizeof(double) * (cplx ? 2 : 1)));
  FMPT_TRY(rwork.alloc(h, (size_t)std::max(n, 1) * 5 * sizeof(double)));
  if (cplx)
    FMPT_SOLVER(h, cusolverDnZgesvd(h->solver, 'S', 'S', m, n, (cuDoubleComplex*)Awork, m, S,
                                    (cuDoubleComplex*)U, m, (cuDoubleComplex*)VT, n,
                                    (cuDoubleComplex*)work.p, lwork, rwork.d(), (int*)dinfo.p));
  else
    FMPT_SOLVER(h, cusolverDnDgesvd(h->solver, 'S', 'S', m, n, Awork, m, S, U, m, VT, n,
                                    work.d(), lwork, rwork.d(), (int*)dinfo.p));
  int info = 0;
  FMPT_TRY(read_info(h, (const int*)dinfo.p, &info));
  if (info == 0) return FMPT_OK;
  if (info < 0) return set_error(h, FMPT_ERR_CUSOLVER, "gesvd: illegal argument %d", -info);
  // not converged: retry with the one-sided Jacobi SVD (stable_svd.jl:12-18 pattern)
  return svd_tall_jacobi(h, cplx, m, n, Acopy.d(), S, U, VT);
}

// One-sided Jacobi SVD (cuSOLVER gesvdj, default tolerance and sweep limit) of a
// tall matrix in solver layout; A is overwritten.
static int svd_tall_jacobi(fmpt_handle* h, int cplx, int m, int n, double* Awork, double* S,
                           double* U, double* VT) {
  DevBuf dinfo;
  FMPT_TRY(dinfo.alloc(h, sizeof(int)));
  double* Aj = Awork;
  int info = 0;
  gesvdjInfo_t params;
  FMPT_SOLVER(h, cusolverDnCreateGesvdjInfo(&params));
  DevBuf V;
  FMPT_TRY(V.alloc(h, (size_t)n * n * sizeof(double) * (cplx ? 2 : 1)));
  int lw2 = 0;
  cusolverStatus_t st;
  if (cplx)
    st = cusolverDnZgesvdj_bufferSize(h->solver, CUSOLVER_EIG_MODE_VECTOR, 1, m, n,
                                      (cuDoubleComplex*)Aj, m, S, (cuDoubleComplex*)U, m,
                                      (cuDoubleComplex*)V.p, n, &lw2, params);
  else
    st = cusolverDnDgesvdj_bufferSize(h->solver, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, Aj, m,
                                      S, U, m, V.d(), n, &lw2, params);
  DevBuf w2;
  if (st == CUSOLVER_STATUS_SUCCESS) {
    int s2 = w2.alloc(h, (size_t)std::max(lw2, 1) * sizeof(double) * (cplx ? 2 : 1));
    if (s2 != FMPT_OK) { cusolverDnDestroyGesvdjInfo(params); return s2; }
    if (cplx)
      st = cusolverDnZgesvdj(h->solver, CUSOLVER_EIG_MODE_VECTOR, 1, m, n,
                             (cuDoubleComplex*)Aj, m, S, (cuDoubleComplex*)U, m,
                             (cuDoubleComplex*)V.p, n, (cuDoubleComplex*)w2.p, lw2,
                             (int*)dinfo.p, params);
    else
      st = cusolverDnDgesvdj(h->solver, CUSOLVER_EIG_MODE_VECTOR, 1, m, n, Aj, m, S, U, m,
                             V.d(), n, w2.d(), lw2, (int*)dinfo.p, params);
  }
  cusolverDnDestroyGesvdjInfo(params);
  if (st != CUSOLVER_STATUS_SUCCESS)
    return set_error(h, FMPT_ERR_CUSOLVER, "gesvdj failed (status %d)", (int)st);
  FMPT_TRY(read_info(h, (const int*)dinfo.p, &info));
  if (info != 0) return set_error(h, FMPT_ERR_CUSOLVER, "gesvdj did not converge (info %d)", info);
  // VT = V^H (interleaved layout, n x n)
  return copy_mat(h, cplx, n, n, V.d(), n, cplx ? -1 : 0, 1, cplx, VT, n, cplx ? -1 : 0);
}

}  // namespace fmpt

using namespace fmpt;

extern "C" {

int fmpt_svd_trunc(fmpt_handle* h, int dtype, const double* M, int m, int n, int maxD,
                   double eps, double* U, double* S, double* Vt, int* kout, double* errout) {
  if (!h || !M || !U || !S || !Vt || !kout) return FMPT_ERR_ARG;
  if (m < 1 || n < 1 || maxD < 1) return set_error(h, FMPT_ERR_SHAPE, "svd: bad extents");
  const int cp = dtype == FMPT_C128;
  const int r = std::min(m, n);
  const bool tall = m >= n;
  const int mm = tall ? m : n, nn = tall ? n : m;   // solver problem is mm x nn, mm >= nn
  const int64_t planeM = (int64_t)m * n;
  DevBuf A, Uw, VTw, Sw;
  const size_t es = sizeof(double) * (cp ? 2 : 1);
  FMPT_TRY(A.alloc(h, (size_t)mm * nn * es));
  FMPT_TRY(Uw.alloc(h, (size_t)mm * nn * es));
  FMPT_TRY(VTw.alloc(h, (size_t)nn * nn * es));
  FMPT_TRY(Sw.alloc(h, (size_t)nn * sizeof(double)));
  // solver input: M (tall) or M^H (wide), interleaved for complex
  FMPT_TRY(copy_mat(h, cp, mm, nn, M, m, planeM, tall ? 0 : 1, tall ? 0 : cp, A.d(), mm,
                    cp ? -1 : 0));
  FMPT_TRY(svd_tall(h, cp, mm, nn, A.d(), Sw.d(), Uw.d(), VTw.d()));
  // singular values to the host, MPSTruncation rule
  std::vector<double> s(r);
  FMPT_CUDA(h, cudaMemcpyAsync(s.data(), Sw.d(), r * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  double nrm = 0.0;
  for (double v : s) nrm += v * v;
  nrm = std::sqrt(nrm);
  int keep = 0;
  for (double v : s) keep += (v >= eps * nrm) ? 1 : 0;   // s is sorted descending
  double e1 = 0.0, e2 = 0.0;
  for (int i = keep; i < r; i++) e1 += s[i] * s[i];
  int k = keep;
  if (keep > maxD) {
    for (int i = maxD; i < keep; i++) e2 += s[i] * s[i];
    k = maxD;
  }
  if (errout) *errout = std::sqrt(e1 + e2);
  *kout = k;
  FMPT_CUDA(h, cudaMemcpyAsync(S, Sw.d(), k * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  if (tall) {
    // U = Uw[:, :k] (m x k), Vt = VTw[:k, :] (k x n)
    FMPT_TRY(copy_mat(h, cp, m, k, Uw.d(), mm, cp ? -1 : 0, 0, 0, U, m, (int64_t)m * k));
    FMPT_TRY(copy_mat(h, cp, k, n, VTw.d(), nn, cp ? -1 : 0, 0, 0, Vt, k, (int64_t)k * n));
  } else {
    // M^H = Uw S VTw  ->  M = VTw^H S Uw^H : U = (VTw[:k, :])^H, Vt = (Uw[:, :k])^H
    FMPT_TRY(copy_mat(h, cp, m, k, VTw.d(), nn, cp ? -1 : 0, 1, cp, U, m, (int64_t)m * k));
    FMPT_TRY(copy_mat(h, cp, k, n, Uw.d(), mm, cp ? -1 : 0, 1, cp, Vt, k, (int64_t)k * n));
  }
  return FMPT_OK;
}

namespace fmpt {
namespace {

// Hermitian eigendecomposition of an r x r split-plane matrix H (lower triangle used):
// eigenvalues ascending into W (device), eigenvectors (columns, split planes) into V.
int eigh_split(fmpt_handle* h, int cp, int r, const double* H, double* W, double* V) {
  DevBuf inter, work, dinfo;
  double* A = V;
  if (cp) {
    FMPT_TRY(inter.alloc(h, (size_t)r * r * 2 * sizeof(double)));
    FMPT_TRY(copy_mat(h, 1, r, r, H, r, (int64_t)r * r, 0, 0, inter.d(), r, -1));
    A = inter.d();
  } else if (H != V) {
    FMPT_CUDA(h, cudaMemcpyAsync(V, H, (size_t)r * r * sizeof(double), cudaMemcpyDeviceToDevice,
                                 h->stream));
  }
  FMPT_TRY(dinfo.alloc(h, sizeof(int)));
  int lwork = 0;
  if (cp)
    FMPT_SOLVER(h, cusolverDnZheevd_bufferSize(h->solver, CUSOLVER_EIG_MODE_VECTOR,
                                               CUBLAS_FILL_MODE_LOWER, r, (cuDoubleComplex*)A, r,
                                               W, &lwork));
  else
    FMPT_SOLVER(h, cusolverDnDsyevd_bufferSize(h->solver, CUSOLVER_EIG_MODE_VECTOR,
                                               CUBLAS_FILL_MODE_LOWER, r, A, r, W, &lwork));
  FMPT_TRY(work.alloc(h, (size_t)std::max(lwork, 1) * sizeof(double) * (cp ? 2 : 1)));
  if (cp)
    FMPT_SOLVER(h, cusolverDnZheevd(h->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, r,
                                    (cuDoubleComplex*)A, r, W, (cuDoubleComplex*)work.p, lwork,
                                    (int*)dinfo.p));
  else
    FMPT_SOLVER(h, cusolverDnDsyevd(h->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, r,
                                    A, r, W, work.d(), lwork, (int*)dinfo.p));
  int info = 0;
  FMPT_TRY(read_info(h, (const int*)dinfo.p, &info));
  if (info != 0) return set_error(h, FMPT_ERR_CUSOLVER, "syevd/heevd info %d", info);
  if (cp) FMPT_TRY(copy_mat(h, 1, r, r, A, r, -1, 0, 0, V, r, (int64_t)r * r));
  return FMPT_OK;
}

// dst column j = src column idx[j] (r rows, split planes with the given plane strides)
__global__ void gather_cols(int cp, int r, int k, const double* __restrict__ src, int64_t splane,
                            const int* __restrict__ idx, double* __restrict__ dst,
                            int64_t dplane) {
  const int64_t tot = (int64_t)r * k;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % r), j = (int)(t / r);
    const int64_t s = (int64_t)idx[j] * r + i;
    dst[t] = src[s];
    if (cp) dst[dplane + t] = src[splane + s];
  }
}

GemmArgs gemm_plain(int cp, int ta, int tb, int m, int n, int k, const double* A, int64_t lda,
                    int64_t pA, const double* B, int64_t ldb, int64_t pB, double* C, int64_t ldc,
                    int64_t pC) {
  GemmArgs g{};
  g.cplx = cp; g.ta = ta; g.tb = tb; g.m = m; g.n = n; g.k = k;
  g.alpha[0] = 1.0; g.batch = 1;
  g.A = A; g.lda = lda; g.planeA = pA;
  g.B = B; g.ldb = ldb; g.planeB = pB;
  g.C = C; g.ldc = ldc; g.planeC = pC;
  return g;
}

}  // namespace
}  // namespace fmpt

int fmpt_dm_split(fmpt_handle* h, int dtype, const double* M, int m, int n, int maxD,
                  double eps, int side, double* Aout, double* S, double* Bout, int* kout,
                  double* errout) {
  if (!h || !M || !Aout || !S || !Bout || !kout) return FMPT_ERR_ARG;
  if (m < 1 || n < 1 || maxD < 1) return set_error(h, FMPT_ERR_SHAPE, "dm_split: bad extents");
  if (side != 0 && side != 1) return set_error(h, FMPT_ERR_ARG, "dm_split: side must be 0 or 1");
  const int cp = dtype == FMPT_C128;
  const bool left = side == 0;
  // The split's GEMMs (Gram matrix, refinement projections, the factors) go to the
  // FP64-accurate tensor-core engine wherever its cost model is faster than the CUDA
  // cores: FP64-class results at a fraction of the FP64 pipe's time
  auto split_gemm = [](fmpt_handle* hh, GemmArgs g) {
    g.engine = 1;
    return gemm_f64(hh, g);
  };
  // X = op(M): M (left, r = m rows of length c = n) or M^H (right, r = n, c = m)
  const int r = left ? m : n, c = left ? n : m;
  const int xop = left ? FMPT_N : FMPT_C;
  const int64_t planeM = (int64_t)m * n, pr = (int64_t)r * r;
  // pass 1: rho = X X^H, U diag(lam) U^H (FP64 GEMM + cuSOLVER syevd/heevd)
  DevBuf rho, U, W;
  FMPT_TRY(rho.alloc(h, (size_t)pr * sizeof(double) * (cp ? 2 : 1)));
  FMPT_TRY(U.alloc(h, (size_t)pr * sizeof(double) * (cp ? 2 : 1)));
  FMPT_TRY(W.alloc(h, (size_t)r * sizeof(double)));
  FMPT_TRY(split_gemm(h, gemm_plain(cp, xop, left ? FMPT_C : FMPT_N, r, r, c, M, m, planeM, M, m,
                                  planeM, rho.d(), r, pr)));
  FMPT_TRY(eigh_split(h, cp, r, rho.d(), W.d(), U.d()));
  std::vector<double> lam(r);
  FMPT_CUDA(h, cudaMemcpyAsync(lam.data(), W.d(), r * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  const int rank_max = std::min(m, n);
  const double epsm = 2.220446049250313e-16;
  // Squaring the matrix leaves an eigenvalue lam resolved only to ~ r eps lam_max, i.e. a
  // singular value to ~ sqrt(r eps) sigma_max.  Refinement passes resolve the tail: the
  // columns [0, t) of U (ascending lam) whose lam is below TAU times the largest of the
  // pass are rotated again, by the eigenvectors of the Gram matrix of their rows of
  // U^H X -- rows from which the components along the resolved rows have been projected
  // out -- so that the next pass resolves lam relative to the tail's own largest value.
  const double TAU = 1e-8;
  const int MAXPASS = 4;
  int t = r;                                          // unresolved prefix of U's columns
  double floor_ = 4.0 * r * epsm * std::max(lam[r - 1], 0.0);
  for (int pass = 1; pass < MAXPASS && t > 0; pass++) {
    const double top = std::max(lam[t - 1], 0.0);
    const double thr = TAU * top;
    int tn = 0;
    while (tn < t && lam[tn] < thr) tn++;
    if (tn == 0) break;
    const int nres = r - tn;
    // nothing below the resolved set can be kept: the bond is full, or the tail lies
    // below the cutoff eps ||sigma||_2
    double nrm2 = 0.0;
    for (int i = tn; i < r; i++) nrm2 += std::max(lam[i], 0.0);
    if (std::min(nres, rank_max) >= maxD) break;
    if (std::sqrt(thr) < 0.25 * eps * std::sqrt(nrm2)) break;
    if (top <= 0.0) break;
    // rows of the resolved directions, normalised: Qr = diag(lam)^-1/2 U_res^H X
    DevBuf Qr, Bt, G, inv, Gt, Wt, Vt, Ut;
    const int64_t pq = (int64_t)nres * c, pb = (int64_t)tn * c;
    FMPT_TRY(Qr.alloc(h, (size_t)pq * sizeof(double) * (cp ? 2 : 1)));
    FMPT_TRY(Bt.alloc(h, (size_t)pb * sizeof(double) * (cp ? 2 : 1)));
    const double* Ures = U.d() + (int64_t)tn * r;
    FMPT_TRY(split_gemm(h, gemm_plain(cp, FMPT_C, xop, nres, c, r, Ures, r, pr, M, m, planeM,
                                    Qr.d(), nres, pq)));
    std::vector<double> sc(nres);
    for (int i = 0; i < nres; i++) sc[i] = lam[tn + i] > 0.0 ? 1.0 / std::sqrt(lam[tn + i]) : 0.0;
    FMPT_TRY(inv.alloc(h, (size_t)nres * sizeof(double)));
    FMPT_CUDA(h, cudaMemcpyAsync(inv.d(), sc.data(), nres * sizeof(double), cudaMemcpyHostToDevice,
                                 h->stream));
    FMPT_TRY(fmpt_scale_dim(h, dtype, 0, nres, c, inv.d(), Qr.d()));
    // tail rows Bt = U_tail^H X, minus their components along the resolved rows (twice)
    FMPT_TRY(split_gemm(h, gemm_plain(cp, FMPT_C, xop, tn, c, r, U.d(), r, pr, M, m, planeM,
                                    Bt.d(), tn, pb)));
    FMPT_TRY(G.alloc(h, (size_t)tn * nres * sizeof(double) * (cp ? 2 : 1)));
    for (int rep = 0; rep < 2; rep++) {
      FMPT_TRY(split_gemm(h, gemm_plain(cp, FMPT_N, FMPT_C, tn, nres, c, Bt.d(), tn, pb, Qr.d(),
                                      nres, pq, G.d(), tn, (int64_t)tn * nres)));
      GemmArgs g = gemm_plain(cp, FMPT_N, FMPT_N, tn, c, nres, G.d(), tn, (int64_t)tn * nres,
                              Qr.d(), nres, pq, Bt.d(), tn, pb);
      g.alpha[0] = -1.0;
      g.beta[0] = 1.0;
      FMPT_TRY(split_gemm(h, g));
    }
    // Gram of the tail rows, its eigenvectors rotate the tail columns of U
    const int64_t pt = (int64_t)tn * tn;
    FMPT_TRY(Gt.alloc(h, (size_t)pt * sizeof(double) * (cp ? 2 : 1)));
    FMPT_TRY(Wt.alloc(h, (size_t)tn * sizeof(double)));
    FMPT_TRY(Vt.alloc(h, (size_t)pt * sizeof(double) * (cp ? 2 : 1)));
    FMPT_TRY(split_gemm(h, gemm_plain(cp, FMPT_N, FMPT_C, tn, tn, c, Bt.d(), tn, pb, Bt.d(), tn, pb,
                                    Gt.d(), tn, pt)));
    FMPT_TRY(eigh_split(h, cp, tn, Gt.d(), Wt.d(), Vt.d()));
    FMPT_TRY(Ut.alloc(h, (size_t)r * tn * sizeof(double) * (cp ? 2 : 1)));
    FMPT_TRY(split_gemm(h, gemm_plain(cp, FMPT_N, FMPT_N, r, tn, tn, U.d(), r, pr, Vt.d(), tn, pt,
                                    Ut.d(), r, (int64_t)r * tn)));
    FMPT_TRY(copy_mat(h, cp, r, tn, Ut.d(), r, (int64_t)r * tn, 0, 0, U.d(), r, pr));
    FMPT_CUDA(h, cudaMemcpyAsync(lam.data(), Wt.d(), tn * sizeof(double), cudaMemcpyDeviceToHost,
                                 h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
    floor_ = 4.0 * tn * epsm * std::max(lam[tn - 1], 0.0);
    t = tn;
  }
  // sigma descending: the resolved columns [t, r) and the prefix [0, t) above its pass's
  // noise floor (below it an eigenvalue is rounding noise and counts as an exact zero)
  std::vector<int> order(r);
  for (int i = 0; i < r; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return lam[a] > lam[b]; });
  std::vector<double> s(r);
  for (int i = 0; i < r; i++) {
    const int j = order[i];
    const double l = lam[j];
    const bool ok = j >= t ? l > 0.0 : l > floor_;
    s[i] = (i < rank_max && ok) ? std::sqrt(l) : 0.0;
  }
  double nrm = 0.0;
  for (double v : s) nrm += v * v;
  nrm = std::sqrt(nrm);
  int keep = 0;
  for (double v : s) keep += (v >= eps * nrm && v > 0.0) ? 1 : 0;
  double e1 = 0.0, e2 = 0.0;
  for (int i = keep; i < r; i++) e1 += s[i] * s[i];
  int k = keep;
  if (keep > maxD) {
    for (int i = maxD; i < keep; i++) e2 += s[i] * s[i];
    k = maxD;
  }
  if (k < 1) return set_error(h, FMPT_ERR_NONFINITE, "dm_split: zero matrix");
  *kout = k;
  if (errout) *errout = std::sqrt(e1 + e2);
  FMPT_CUDA(h, cudaMemcpyAsync(S, s.data(), k * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  // Q (r x k, split planes): the columns of the k largest, descending
  DevBuf Q, didx;
  FMPT_TRY(Q.alloc(h, (size_t)r * k * sizeof(double) * (cp ? 2 : 1)));
  FMPT_TRY(didx.alloc(h, (size_t)k * sizeof(int)));
  FMPT_CUDA(h, cudaMemcpyAsync(didx.p, order.data(), k * sizeof(int), cudaMemcpyHostToDevice,
                               h->stream));
  {
    const int64_t tot = (int64_t)r * k;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, 8LL * h->sm_count));
    gather_cols<<<blocks, 256, 0, h->stream>>>(cp, r, k, U.d(), pr, (const int*)didx.p, Q.d(),
                                               (int64_t)r * k);
    FMPT_LAUNCHED(h);
  }
  GemmArgs g{};
  g.cplx = cp; g.alpha[0] = 1.0; g.batch = 1;
  if (left) {
    // A = Q (m x k);  B = Q^H M (k x n)
    FMPT_CUDA(h, cudaMemcpyAsync(Aout, Q.d(), (size_t)m * k * sizeof(double) * (cp ? 2 : 1),
                                 cudaMemcpyDeviceToDevice, h->stream));
    g.ta = FMPT_C; g.tb = FMPT_N; g.m = k; g.n = n; g.k = m;
    g.A = Q.d(); g.lda = m; g.planeA = (int64_t)m * k;
    g.B = M; g.ldb = m; g.planeB = planeM;
    g.C = Bout; g.ldc = k; g.planeC = (int64_t)k * n;
    FMPT_TRY(split_gemm(h, g));
  } else {
    // B = Q^H (k x n);  A = M Q (m x k)
    FMPT_TRY(copy_mat(h, cp, k, n, Q.d(), n, (int64_t)n * k, 1, cp, Bout, k, (int64_t)k * n));
    g.ta = FMPT_N; g.tb = FMPT_N; g.m = m; g.n = k; g.k = n;
    g.A = M; g.lda = m; g.planeA = planeM;
    g.B = Q.d(); g.ldb = n; g.planeB = (int64_t)n * k;
    g.C = Aout; g.ldc = m; g.planeC = (int64_t)m * k;
    FMPT_TRY(split_gemm(h, g));
  }
  // the host vectors must stay alive until their async copies finish
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  return FMPT_OK;
}

int fmpt_qr(fmpt_handle* h, int dtype, const double* M, int m, int n, double* Q, double* R) {
  if (!h || !M || !Q || !R) return FMPT_ERR_ARG;
  if (m < 1 || n < 1) return set_error(h, FMPT_ERR_SHAPE, "qr: bad extents");
  const int cp = dtype == FMPT_C128;
  const int r = std::min(m, n);
  const size_t es = sizeof(double) * (cp ? 2 : 1);
  // small tall panels: one thread-block cluster, LAPACK's conventions (qr_cluster.cu)
  {
    const int st = qr_small_cluster(h, cp, m, n, M, Q, R);
    if (st != FMPT_ERR_UNSUPPORTED) return st;
  }
  DevBuf A, tau, work, dinfo;
  FMPT_TRY(A.alloc(h, (size_t)m * std::max(n, r) * es));
  FMPT_TRY(tau.alloc(h, (size_t)r * es));
  FMPT_TRY(dinfo.alloc(h, sizeof(int)));
  FMPT_TRY(copy_mat(h, cp, m, n, M, m, (int64_t)m * n, 0, 0, A.d(), m, cp ? -1 : 0));
  int lw1 = 0, lw2 = 0;
  if (cp) {
    FMPT_SOLVER(h, cusolverDnZgeqrf_bufferSize(h->solver, m, n, (cuDoubleComplex*)A.p, m, &lw1));
    FMPT_SOLVER(h, cusolverDnZungqr_bufferSize(h->solver, m, r, r, (cuDoubleComplex*)A.p, m,
                                               (cuDoubleComplex*)tau.p, &lw2));
  } else {
    FMPT_SOLVER(h, cusolverDnDgeqrf_bufferSize(h->solver, m, n, A.d(), m, &lw1));
    FMPT_SOLVER(h, cusolverDnDorgqr_bufferSize(h->solver, m, r, r, A.d(), m, tau.d(), &lw2));
  }
  int lw = std::max(std::max(lw1, lw2), 1);
  FMPT_TRY(work.alloc(h, (size_t)lw * es));
  if (cp)
    FMPT_SOLVER(h, cusolverDnZgeqrf(h->solver, m, n, (cuDoubleComplex*)A.p, m,
                                    (cuDoubleComplex*)tau.p, (cuDoubleComplex*)work.p, lw,
                                    (int*)dinfo.p));
  else
    FMPT_SOLVER(h, cusolverDnDgeqrf(h->solver, m, n, A.d(), m, tau.d(), work.d(), lw,
                                    (int*)dinfo.p));
  // R = upper triangle of A[0:r, 0:n]
  FMPT_TRY(copy_mat(h, cp, r, n, A.d(), m, cp ? -1 : 0, 0, 0, R, r, (int64_t)r * n));
  {
    int64_t tot = (int64_t)r * n;
    zero_lower<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, 4096)), 256, 0,
                 h->stream>>>(cp, r, n, R, r, (int64_t)r * n);
    FMPT_LAUNCHED(h);
  }
  if (cp)
    FMPT_SOLVER(h, cusolverDnZungqr(h->solver, m, r, r, (cuDoubleComplex*)A.p, m,
                                    (cuDoubleComplex*)tau.p, (cuDoubleComplex*)work.p, lw,
                                    (int*)dinfo.p));
  else
    FMPT_SOLVER(h, cusolverDnDorgqr(h->solver, m, r, r, A.d(), m, tau.d(), work.d(), lw,
                                    (int*)dinfo.p));
  int info = 0;
  FMPT_TRY(read_info(h, (const int*)dinfo.p, &info));
  if (info != 0) return set_error(h, FMPT_ERR_CUSOLVER, "qr: info %d", info);
  return copy_mat(h, cp, m, r, A.d(), m, cp ? -1 : 0, 0, 0, Q, m, (int64_t)m * r);
}

int fmpt_lq(fmpt_handle* h, int dtype, const double* M, int m, int n, double* Lout, double* Q) {
  if (!h || !M || !Lout || !Q) return FMPT_ERR_ARG;
  if (m < 1 || n < 1) return set_error(h, FMPT_ERR_SHAPE, "lq: bad extents");
  const int cp = dtype == FMPT_C128;
  const int r = std::min(m, n);
  const size_t es = sizeof(double) * (cp ? 2 : 1);
  // M^H (n x m) = Q' R'  ->  M = R'^H Q'^H
  DevBuf MH, Qp, Rp;
  FMPT_TRY(MH.alloc(h, (size_t)n * m * es));
  FMPT_TRY(Qp.alloc(h, (size_t)n * r * es));
  FMPT_TRY(Rp.alloc(h, (size_t)r * m * es));
  FMPT_TRY(copy_mat(h, cp, n, m, M, m, (int64_t)m * n, 1, cp, MH.d(), n, (int64_t)n * m));
  FMPT_TRY(fmpt_qr(h, dtype, MH.d(), n, m, Qp.d(), Rp.d()));
  FMPT_TRY(copy_mat(h, cp, m, r, Rp.d(), r, (int64_t)r * m, 1, cp, Lout, m, (int64_t)m * r));
  FMPT_TRY(copy_mat(h, cp, r, n, Qp.d(), n, (int64_t)n * r, 1, cp, Q, r, (int64_t)r * n));
  return FMPT_OK;
}

}  // extern "C"
