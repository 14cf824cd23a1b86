// One whole DMRG2 sweep behind one C-ABI call (sweep! of algorithms/dmrgexcited.jl:219-223
// for DMRG2: leftsweep! then rightsweep!, algorithms/dmrg.jl:89-144).
//
// The chain lives in caller-owned device buffers sized for the largest bond dimension the
// sweep can reach: site tensors A_i[D_i, d_i, D_{i+1}] and environments h_i[D_i, w_i, D_i],
// all column-major (complex as split planes).  The bond dimensions are a host array that
// the sweep updates.  Each bond runs the same library calls, with the same arguments and
// in the same order, as the Python-driven bond of algorithms.py: two-site product,
// prepared ac2 operator, device Lanczos, truncated split (gesvd or density matrix), s
// normalisation, fidelity delta, and the environment update -- so the Ritz values and the
// tensors are bit-identical to that driver's.  Nothing returns to the host per bond except
// the scalars the algorithm itself needs there (the Ritz value, the kept rank k, the two
// norms and the overlap of the fidelity).
#include <algorithm>
#include <cmath>

#include "internal.h"

namespace fmpt {
namespace {

struct Chain {
  fmpt_handle* h;
  int dtype, precision, env_precision, L;
  const int* phys;
  int* bond;
  double* const* sites;
  const int64_t* site_cap;
  double* const* envs;
  const int64_t* env_cap;
  const double* const* W;
  const int* wb;
  double* const* svals;
  int maxD;
  double eps;
  int eig_maxiter;
  double eig_tol;
  int reorth, split;
  size_t es() const { return sizeof(double) * (dtype == FMPT_C128 ? 2 : 1); }
};

const double kOne[2] = {1.0, 0.0};
const double kZero[2] = {0.0, 0.0};

// |1 - |<usv, x2>|| (dmrg.jl:109-110, :139-140)
int fidelity_delta(const Chain& c, const double* U, const double* SV, const double* x2, int m,
                   int n, int k, double* delta) {
  fmpt_handle* h = c.h;
  DevBuf usv;
  FMPT_TRY(usv.alloc(h, (size_t)m * n * c.es()));
  FMPT_TRY(fmpt_gemm(h, c.dtype, 0, 0, m, n, k, kOne, U, m, SV, k, kZero, usv.d(), m));
  double ov[2] = {0.0, 0.0};
  FMPT_TRY(fmpt_dot(h, c.dtype, (int64_t)m * n, usv.d(), x2, ov));
  const double a = c.dtype == FMPT_C128 ? std::hypot(ov[0], ov[1]) : std::fabs(ov[0]);
  *delta = std::fabs(1.0 - a);
  return FMPT_OK;
}

// x2 = A_i A_{i+1} and its lowest Ritz pair under ac2_prime (dmrg.jl:98-104)
int bond_eig(const Chain& c, int i, DevBuf& x2, DevBuf& vec, double* E) {
  fmpt_handle* h = c.h;
  const int Dl = c.bond[i], d1 = c.phys[i], Dm = c.bond[i + 1], d2 = c.phys[i + 1],
            Dr = c.bond[i + 2];
  const int m = Dl * d1, n = d2 * Dr;
  FMPT_TRY(x2.alloc(h, (size_t)m * n * c.es()));
  FMPT_TRY(fmpt_gemm(h, c.dtype, 0, 0, m, n, Dm, kOne, c.sites[i], m, c.sites[i + 1], Dm, kZero,
                     x2.d(), m));
  fmpt_op* op = nullptr;
  FMPT_TRY(fmpt_op_ac2(h, c.dtype, c.precision, c.W[i], c.W[i + 1], c.envs[i], c.envs[i + 2],
                       Dl, d1, d2, Dr, c.wb[i], c.wb[i + 1], c.wb[i + 2], &op));
  int st = vec.alloc(h, (size_t)m * n * c.es());
  int info = 0, iters = 0;
  if (st == FMPT_OK)
    st = fmpt_lanczos_ground(op, x2.d(), c.eig_maxiter, c.eig_tol, c.reorth, E, vec.d(), &info,
                             &iters);
  fmpt_op_destroy(op);
  return st;
}

int check_caps(const Chain& c, int i, int m, int n, int k) {
  if ((int64_t)m * k > c.site_cap[i] || (int64_t)k * n > c.site_cap[i + 1])
    return set_error(c.h, FMPT_ERR_SHAPE,
                     "dmrg2_sweep: bond %d keeps %d states; site buffers hold %lld and %lld "
                     "elements, need %lld and %lld", i + 1, k, (long long)c.site_cap[i],
                     (long long)c.site_cap[i + 1], (long long)m * k, (long long)k * n);
  return FMPT_OK;
}

int check_env(const Chain& c, int b, int D) {
  if ((int64_t)D * c.wb[b] * D > c.env_cap[b])
    return set_error(c.h, FMPT_ERR_SHAPE,
                     "dmrg2_sweep: environment %d needs %lld elements, its buffer holds %lld", b,
                     (long long)D * c.wb[b] * D, (long long)c.env_cap[b]);
  return FMPT_OK;
}

// leftsweep! bond body (dmrg.jl:95-113): A_i = u, A_{i+1} = s*v, then updateleft!
int left_bond(Chain& c, int i, double* E, double* delta) {
  fmpt_handle* h = c.h;
  const int Dl = c.bond[i], d1 = c.phys[i], d2 = c.phys[i + 1], Dr = c.bond[i + 2];
  const int m = Dl * d1, n = d2 * Dr, r = std::min(m, n);
  const size_t es = c.es();
  DevBuf x2, vec, U, S, V;
  FMPT_TRY(bond_eig(c, i, x2, vec, E));
  FMPT_TRY(U.alloc(h, (size_t)m * r * es));
  FMPT_TRY(S.alloc(h, (size_t)r * sizeof(double)));
  FMPT_TRY(V.alloc(h, (size_t)r * n * es));
  int k = 0;
  double err = 0.0, nrm = 0.0;
  if (c.split == 1) {
    // U orthonormal from M M^H; s*v = U^H M, normalised with s
    FMPT_TRY(fmpt_dm_split(h, c.dtype, vec.d(), m, n, c.maxD, c.eps, 0, U.d(), S.d(), V.d(), &k,
                           &err));
    FMPT_TRY(fmpt_nrm2(h, FMPT_F64, k, S.d(), &nrm));
    const double a[2] = {1.0 / nrm, 0.0};
    FMPT_TRY(fmpt_scal(h, FMPT_F64, k, a, S.d()));
    FMPT_TRY(fmpt_scal(h, c.dtype, (int64_t)k * n, a, V.d()));
  } else {
    FMPT_TRY(fmpt_svd_trunc(h, c.dtype, vec.d(), m, n, c.maxD, c.eps, U.d(), S.d(), V.d(), &k,
                            &err));
    FMPT_TRY(fmpt_nrm2(h, FMPT_F64, k, S.d(), &nrm));
    const double a[2] = {1.0 / nrm, 0.0};
    FMPT_TRY(fmpt_scal(h, FMPT_F64, k, a, S.d()));              // normalize!(s)
    FMPT_TRY(fmpt_scale_dim(h, c.dtype, 0, k, n, S.d(), V.d()));  // s * v
  }
  FMPT_TRY(fidelity_delta(c, U.d(), V.d(), x2.d(), m, n, k, delta));
  FMPT_TRY(check_caps(c, i, m, n, k));
  FMPT_TRY(check_env(c, i + 1, k));
  FMPT_CUDA(h, cudaMemcpyAsync(c.sites[i], U.p, (size_t)m * k * es, cudaMemcpyDeviceToDevice,
                               h->stream));
  FMPT_CUDA(h, cudaMemcpyAsync(c.sites[i + 1], V.p, (size_t)k * n * es,
                               cudaMemcpyDeviceToDevice, h->stream));
  c.bond[i + 1] = k;
  // updateleft!(m, site): h_{i+1} from h_i and the new A_i
  return fmpt_updateleft(h, c.dtype, c.env_precision, c.envs[i], c.sites[i], c.W[i], c.sites[i],
                         c.envs[i + 1], Dl, d1, k, c.wb[i], c.wb[i + 1]);
}

// rightsweep! bond body (dmrg.jl:123-142): A_i = u*s, A_{i+1} = v, s stored, updateright!
int right_bond(Chain& c, int i, double* E, double* delta) {
  fmpt_handle* h = c.h;
  const int Dl = c.bond[i], d1 = c.phys[i], d2 = c.phys[i + 1], Dr = c.bond[i + 2];
  const int m = Dl * d1, n = d2 * Dr, r = std::min(m, n);
  const size_t es = c.es();
  DevBuf x2, vec, U, S, V;
  FMPT_TRY(bond_eig(c, i, x2, vec, E));
  FMPT_TRY(U.alloc(h, (size_t)m * r * es));
  FMPT_TRY(S.alloc(h, (size_t)r * sizeof(double)));
  FMPT_TRY(V.alloc(h, (size_t)r * n * es));
  int k = 0;
  double err = 0.0, nrm = 0.0;
  if (c.split == 1) {
    // v^H orthonormal from M^H M; u*s = M V, normalised with s
    FMPT_TRY(fmpt_dm_split(h, c.dtype, vec.d(), m, n, c.maxD, c.eps, 1, U.d(), S.d(), V.d(), &k,
                           &err));
    FMPT_TRY(fmpt_nrm2(h, FMPT_F64, k, S.d(), &nrm));
    const double a[2] = {1.0 / nrm, 0.0};
    FMPT_TRY(fmpt_scal(h, FMPT_F64, k, a, S.d()));
    FMPT_TRY(fmpt_scal(h, c.dtype, (int64_t)m * k, a, U.d()));
    FMPT_TRY(fidelity_delta(c, U.d(), V.d(), x2.d(), m, n, k, delta));
  } else {
    FMPT_TRY(fmpt_svd_trunc(h, c.dtype, vec.d(), m, n, c.maxD, c.eps, U.d(), S.d(), V.d(), &k,
                            &err));
    FMPT_TRY(fmpt_nrm2(h, FMPT_F64, k, S.d(), &nrm));
    const double a[2] = {1.0 / nrm, 0.0};
    FMPT_TRY(fmpt_scal(h, FMPT_F64, k, a, S.d()));
    // the fidelity needs u, s and v before s is absorbed into u
    DevBuf SV;
    FMPT_TRY(SV.alloc(h, (size_t)k * n * es));
    FMPT_CUDA(h, cudaMemcpyAsync(SV.p, V.p, (size_t)k * n * es, cudaMemcpyDeviceToDevice,
                                 h->stream));
    FMPT_TRY(fmpt_scale_dim(h, c.dtype, 0, k, n, S.d(), SV.d()));
    FMPT_TRY(fidelity_delta(c, U.d(), SV.d(), x2.d(), m, n, k, delta));
    FMPT_TRY(fmpt_scale_dim(h, c.dtype, 1, m, k, S.d(), U.d()));   // u * s
  }
  FMPT_TRY(check_caps(c, i, m, n, k));
  FMPT_TRY(check_env(c, i + 1, k));
  FMPT_CUDA(h, cudaMemcpyAsync(c.sites[i], U.p, (size_t)m * k * es, cudaMemcpyDeviceToDevice,
                               h->stream));
  FMPT_CUDA(h, cudaMemcpyAsync(c.sites[i + 1], V.p, (size_t)k * n * es,
                               cudaMemcpyDeviceToDevice, h->stream));
  if (c.svals && c.svals[i + 1])
    FMPT_CUDA(h, cudaMemcpyAsync(c.svals[i + 1], S.p, (size_t)k * sizeof(double),
                                 cudaMemcpyDeviceToDevice, h->stream));
  c.bond[i + 1] = k;
  // updateright!(m, site+1): h_{i+1} from h_{i+2} and the new A_{i+1}
  return fmpt_updateright(h, c.dtype, c.env_precision, c.envs[i + 2], c.sites[i + 1], c.W[i + 1],
                          c.sites[i + 1], c.envs[i + 1], k, d2, Dr, c.wb[i + 1], c.wb[i + 2]);
}

}  // namespace
}  // namespace fmpt

using namespace fmpt;

extern "C" int fmpt_dmrg2_sweep(fmpt_handle* h, int dtype, int precision, int env_precision,
                                int L, const int* phys, int* bond, double* const* sites,
                                const int64_t* site_cap, double* const* envs,
                                const int64_t* env_cap, const double* const* W_host,
                                const int* wbond, double* const* svals, int maxD, double eps,
                                int eig_maxiter, double eig_tol, int reorth, int split,
                                double* energies, double* delta) {
  if (!h) return FMPT_ERR_ARG;
  if (dtype != FMPT_F64 && dtype != FMPT_C128)
    return set_error(h, FMPT_ERR_ARG, "dmrg2_sweep: unknown dtype %d", dtype);
  if (L < 2) return set_error(h, FMPT_ERR_SHAPE, "dmrg2_sweep: the chain needs 2 sites");
  if (!phys || !bond || !sites || !site_cap || !envs || !env_cap || !W_host || !wbond ||
      !energies || !delta)
    return set_error(h, FMPT_ERR_ARG, "dmrg2_sweep: null pointer");
  if (split != 0 && split != 1)
    return set_error(h, FMPT_ERR_ARG, "dmrg2_sweep: split must be 0 (gesvd) or 1 (dm)");
  if (maxD < 1) return set_error(h, FMPT_ERR_ARG, "dmrg2_sweep: maxD must be positive");
  for (int i = 0; i < L; i++) {
    if (!sites[i] || !W_host[i] || phys[i] < 1 || bond[i] < 1 || bond[i + 1] < 1)
      return set_error(h, FMPT_ERR_ARG, "dmrg2_sweep: site %d: null buffer or bad dims", i + 1);
    if ((int64_t)bond[i] * phys[i] * bond[i + 1] > site_cap[i])
      return set_error(h, FMPT_ERR_SHAPE, "dmrg2_sweep: site %d does not fit its buffer", i + 1);
  }
  Chain c{h, dtype, precision, env_precision, L, phys, bond, sites, site_cap, envs, env_cap,
          W_host, wbond, svals, maxD, eps, eig_maxiter, eig_tol, reorth, split};
  for (int b = 0; b <= L; b++) {
    if (!envs[b] || wbond[b] < 1)
      return set_error(h, FMPT_ERR_ARG, "dmrg2_sweep: environment %d: null or bad width", b);
    FMPT_TRY(check_env(c, b, bond[b]));
  }
  double dmax = 0.0;
  int e = 0;
  for (int i = 0; i + 2 < L; i++) {              // leftsweep!: sites 1 .. L-2
    double E = 0.0, dl = 0.0;
    FMPT_TRY(left_bond(c, i, &E, &dl));
    energies[e++] = E;
    dmax = std::max(dmax, dl);
  }
  for (int i = L - 2; i >= 0; i--) {             // rightsweep!: sites L-1 .. 1
    double E = 0.0, dl = 0.0;
    FMPT_TRY(right_bond(c, i, &E, &dl));
    energies[e++] = E;
    dmax = std::max(dmax, dl);
  }
  *delta = dmax;
  return FMPT_OK;
}
