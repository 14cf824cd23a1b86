// U(1) charge-sector bookkeeping for the block-sparse DMRG path.
//
// TensorKit does this for the reference when the legs are U1Space: every
// contraction of ac2_prime (derivatives.jl:20-22) and of the environment
// updates (mpo/transfer.jl:26-34) runs block by block over the charge
// sectors, and tsvd! factorises each sector of the two-site matrix.  Here the
// block lists are built on the host from the sector tables and run on the
// grouped persistent engine (grouped.cu): one launch per contraction, three
// phases (GEMM, MPO step, GEMM) separated by bounded grid barriers.
//
// Conventions (see include/fmpt.h): legs are charge-sorted; A[a, s, b] is
// nonzero iff q(a) + qp(s) == q(b); L[a', w, a] iff q(a') == q(a) + qw(w);
// W[wl, s', wr, s] conserves qw(wl) + qp(s') == qw(wr) + qp(s).
#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "internal.h"

namespace fmpt {
namespace {

struct Leg {
  std::vector<int> q, dim;
  std::vector<int64_t> off;
  int64_t total = 0;
  int n() const { return (int)q.size(); }
  int find(int c) const {
    auto it = std::lower_bound(q.begin(), q.end(), c);
    return (it != q.end() && *it == c) ? (int)(it - q.begin()) : -1;
  }
};

int read_leg(fmpt_handle* h, const fmpt_u1_space* s, Leg& L, const char* what) {
  if (!s || s->nsect < 1 || !s->charge || !s->dim)
    return set_error(h, FMPT_ERR_ARG, "u1: %s: empty or null sector table", what);
  L.q.assign(s->charge, s->charge + s->nsect);
  L.dim.assign(s->dim, s->dim + s->nsect);
  L.off.assign(s->nsect, 0);
  L.total = 0;
  for (int i = 0; i < s->nsect; i++) {
    if (L.dim[i] < 1)
      return set_error(h, FMPT_ERR_SHAPE, "u1: %s: sector %d has dimension %d", what, i,
                       L.dim[i]);
    if (i && L.q[i] <= L.q[i - 1])
      return set_error(h, FMPT_ERR_ARG, "u1: %s: charges must be strictly increasing", what);
    L.off[i] = L.total;
    L.total += L.dim[i];
  }
  if (L.total > (1 << 24)) return set_error(h, FMPT_ERR_SHAPE, "u1: %s: leg too large", what);
  return FMPT_OK;
}

int check_real(fmpt_handle* h, int dtype) {
  if (!h) return FMPT_ERR_ARG;
  if (dtype == FMPT_C128)
    return set_error(h, FMPT_ERR_UNSUPPORTED, "u1: complex tensors are not implemented");
  if (dtype != FMPT_F64) return set_error(h, FMPT_ERR_ARG, "u1: unknown dtype %d", dtype);
  return FMPT_OK;
}

int check_phys(fmpt_handle* h, int d, const int* qp, const char* what) {
  if (d < 1 || !qp) return set_error(h, FMPT_ERR_ARG, "u1: %s: bad physical leg", what);
  return FMPT_OK;
}

// W[wl, s', wr, s] must conserve qw(wl) + qp(s') == qw(wr) + qp(s).
int check_mpo(fmpt_handle* h, const double* W, int d, const int* qp, int wl, const int* qwl,
              int wr, const int* qwr, const char* what) {
  if (!W || !qwl || !qwr || wl < 1 || wr < 1)
    return set_error(h, FMPT_ERR_ARG, "u1: %s: null MPO tensor or channel charges", what);
  for (int w = 0; w < wl; w++)
    for (int so = 0; so < d; so++)
      for (int w2 = 0; w2 < wr; w2++)
        for (int si = 0; si < d; si++) {
          const double v = W[w + (int64_t)wl * (so + d * (w2 + (int64_t)wr * si))];
          if (v != 0.0 && qwl[w] + qp[so] != qwr[w2] + qp[si])
            return set_error(h, FMPT_ERR_ARG,
                             "u1: %s: MPO entry (%d,%d,%d,%d) does not conserve the charge", what,
                             w, so, w2, si);
        }
  return FMPT_OK;
}

// Packed two-site layout: offsets of the allowed blocks (ia, s, ib), -1 elsewhere.
struct Pack2 {
  int nl = 0, nr = 0, P = 0;
  std::vector<int> qs;          // charge of the fused physical index s = s1 + d1*s2
  std::vector<int64_t> off;     // [ia + nl*(s + P*ib)]
  int64_t n = 0;
  int64_t at(int ia, int s, int ib) const { return off[ia + (int64_t)nl * (s + (int64_t)P * ib)]; }
};

void build_pack2(const Leg& Vl, const Leg& Vr, int d1, const int* qp1, int d2, const int* qp2,
                 Pack2& pk) {
  pk.nl = Vl.n(); pk.nr = Vr.n(); pk.P = d1 * d2;
  pk.qs.resize(pk.P);
  for (int s = 0; s < pk.P; s++) pk.qs[s] = qp1[s % d1] + qp2[s / d1];
  pk.off.assign((size_t)pk.nl * pk.P * pk.nr, -1);
  pk.n = 0;
  for (int ib = 0; ib < pk.nr; ib++)
    for (int s = 0; s < pk.P; s++)
      for (int ia = 0; ia < pk.nl; ia++)
        if (Vl.q[ia] + pk.qs[s] == Vr.q[ib]) {
          pk.off[ia + (int64_t)pk.nl * (s + (int64_t)pk.P * ib)] = pk.n;
          pk.n += (int64_t)Vl.dim[ia] * Vr.dim[ib];
        }
}

// One block of the MPO step: out = sum_t coef_t * in_t (in_t are keys of phase-1 blocks).
struct MidBlock {
  int64_t key_out;     // key of the phase-3 operand block
  int m, n;
  std::vector<std::pair<double, int64_t>> terms;
};

// Emits phase 1 (only the blocks the MPO step reads) and the MPO step.
// p1: candidate phase-1 problems by key: (m, n, a_off, lda, b_off, ldb, k)
struct P1 {
  int m = 0, n = 0, k = 0;
  int64_t a_off = 0, lda = 0, b_off = 0, ldb = 0;
  bool valid = false, used = false;
  int64_t out = -1;    // packed offset in the T1 scratch
};

int64_t emit_phase1_and_mid(GroupedProgram& g, int ta1, int tb1, int a1, int b1, std::vector<P1>& p1,
                            std::vector<MidBlock>& mids, std::vector<int64_t>& t3off,
                            int64_t* t3_total) {
  for (auto& mb : mids)
    for (auto& t : mb.terms) p1[t.second].used = true;
  gp_phase(g, GP_GEMM, ta1, tb1, a1, b1, /*c*/ 4);
  int64_t t1n = 0;
  for (auto& p : p1) {
    if (!p.valid || !p.used) continue;
    p.out = t1n;
    t1n += (int64_t)p.m * p.n;
    gp_problem(g, p.out, p.m, p.m, p.n);
    gp_segment(g, p.a_off, p.lda, p.b_off, p.ldb, p.k, 1.0);
  }
  gp_phase(g, GP_SUM, FMPT_N, FMPT_N, 4, 4, 5);
  int64_t t3n = 0;
  for (auto& mb : mids) {
    t3off[mb.key_out] = t3n;
    gp_problem(g, t3n, mb.m, mb.m, mb.n);
    for (auto& t : mb.terms) gp_segment(g, p1[t.second].out, mb.m, 0, 0, 0, t.first);
    t3n += (int64_t)mb.m * mb.n;
  }
  *t3_total = t3n;
  return t1n;
}

// Two-site MPO O[w][w2][s'][s] (real), s = s1 + d1*s2 (derivatives.jl:21 wiring).
std::vector<double> two_site_mpo(const double* W1, const double* W2, int d1, int d2, int wl,
                                 int wm, int wr) {
  const int P = d1 * d2;
  std::vector<double> O((size_t)wl * wr * P * P, 0.0);
  for (int w = 0; w < wl; w++)
    for (int m = 0; m < wm; m++)
      for (int a1 = 0; a1 < d1; a1++)
        for (int b1 = 0; b1 < d1; b1++) {
          const double x = W1[w + (int64_t)wl * (a1 + d1 * (m + (int64_t)wm * b1))];
          if (x == 0.0) continue;
          for (int w2 = 0; w2 < wr; w2++)
            for (int a2 = 0; a2 < d2; a2++)
              for (int b2 = 0; b2 < d2; b2++) {
                const double y = W2[m + (int64_t)wm * (a2 + d2 * (w2 + (int64_t)wr * b2))];
                if (y == 0.0) continue;
                O[(((size_t)w * wr + w2) * P + a1 + d1 * a2) * P + b1 + d1 * b2] += x * y;
              }
        }
  return O;
}

struct U1OpState {
  GroupedProgram prog;
  DevBuf T1, T3;
  int64_t n = 0;
};

struct ScratchPair {
  DevBuf T1, T3;
};

int alloc_scratch(fmpt_handle* h, DevBuf& b, int64_t n) {
  return b.alloc(h, (size_t)std::max<int64_t>(n, 1) * sizeof(double));
}


// One charge sector of the new bond in a two-site split.
struct SplitSeg {
  int s, i;
  int64_t off;
};
struct SplitSector {
  int q = 0;
  std::vector<SplitSeg> rows, cols;   // (s1, ia) row blocks, (s2, ib) column blocks
  int r = 0, c = 0, kq = 0, keep = 0;
  int64_t moff = 0, uoff = 0, voff = 0, soff = 0;
  // density-matrix form: Gram extent n, padded extent npad, offset of the
  // (padded) Gram / eigenvector matrix
  int n = 0, npad = 0;
  int64_t goff = 0;
};

// Pads every Gram matrix of a batch to its class size: the padded diagonal
// gets -trace (so the padded eigenvalues sort below the nonnegative spectrum
// and their eigenvectors stay on the padded coordinates).  One CTA per matrix.
__global__ void pad_gram_kernel(const int64_t* __restrict__ goff, const int* __restrict__ nn,
                                const int* __restrict__ np, double* __restrict__ G) {
  __shared__ double red[256];
  double* g = G + goff[blockIdx.x];
  const int n = nn[blockIdx.x], npad = np[blockIdx.x];
  double t = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) t += g[i + (int64_t)i * npad];
  red[threadIdx.x] = t;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double pad = red[0] > 0.0 ? -red[0] : -1.0;
  for (int i = n + threadIdx.x; i < npad; i += blockDim.x) g[i + (int64_t)i * npad] = pad;
}

#define FMPT_SOLVER_U1(h, expr)                                                      \
  do {                                                                               \
    cusolverStatus_t _s = (expr);                                                    \
    if (_s != CUSOLVER_STATUS_SUCCESS)                                               \
      return set_error((h), FMPT_ERR_CUSOLVER, "%s:%d %s -> cusolver status %d",     \
                       __FILE__, __LINE__, #expr, (int)_s);                          \
  } while (0)

// Density-matrix form of the sector factorisation: Gram matrix of every
// sector (side 0: M M^T, side 1: M^T M) in one grouped launch, padded to
// multiples of 32, then one batched symmetric eigensolve (cuSOLVER
// Xsyev, FP64) per padded size.  On return Gw holds the eigenvectors
// (ascending eigenvalues), sv the singular values sqrt(max(lambda, 0)),
// largest first, min(r, c) per sector.
int density_eigen(fmpt_handle* h, int side, std::vector<SplitSector>& sec, const double* Mw,
                  int64_t mtot, DevBuf& Gw, std::vector<double>& sv) {
  std::map<int, std::vector<int>> classes;   // padded size -> sectors
  for (size_t si = 0; si < sec.size(); si++) {
    SplitSector& S_ = sec[si];
    S_.n = side == 0 ? S_.r : S_.c;
    S_.npad = std::max(32, (S_.n + 31) / 32 * 32);
    classes[S_.npad].push_back((int)si);
  }
  int64_t gtot = 0, wtot = 0;
  std::vector<int64_t> woff(sec.size(), 0);
  for (auto& kv : classes)
    for (int si : kv.second) {
      sec[si].goff = gtot;
      gtot += (int64_t)kv.first * kv.first;
      woff[si] = wtot;
      wtot += kv.first;
    }
  DevBuf Ww, info, tab;
  FMPT_TRY(alloc_scratch(h, Gw, gtot));
  FMPT_TRY(alloc_scratch(h, Ww, wtot));
  FMPT_TRY(info.alloc(h, sizeof(int) * sec.size()));
  FMPT_CUDA(h, cudaMemsetAsync(Gw.p, 0, (size_t)gtot * sizeof(double), h->stream));
  {  // all Gram matrices in one grouped launch
    GroupedProgram g;
    if (side == 0)
      gp_phase(g, GP_GEMM, FMPT_N, FMPT_T, 0, 0, 1);
    else
      gp_phase(g, GP_GEMM, FMPT_T, FMPT_N, 0, 0, 1);
    for (const SplitSector& S_ : sec) {
      gp_problem(g, S_.goff, S_.npad, S_.n, S_.n);
      gp_segment(g, S_.moff, S_.r, S_.moff, S_.r, side == 0 ? S_.c : S_.r, 1.0);
    }
    gp_slot(g, 0, mtot);
    gp_slot(g, 1, gtot);
    FMPT_TRY(gp_finalize(h, g));
    double* slots[2] = {const_cast<double*>(Mw), Gw.d()};
    FMPT_TRY(gp_run(h, g, slots, 2));
  }
  {  // padding
    const size_t ns = sec.size();
    std::vector<int64_t> go(ns);
    std::vector<int> nn(ns), np(ns);
    for (size_t i = 0; i < ns; i++) { go[i] = sec[i].goff; nn[i] = sec[i].n; np[i] = sec[i].npad; }
    FMPT_TRY(tab.alloc(h, ns * (sizeof(int64_t) + 2 * sizeof(int)) + 64));
    char* t = static_cast<char*>(tab.p);
    FMPT_CUDA(h, cudaMemcpyAsync(t, go.data(), ns * sizeof(int64_t), cudaMemcpyHostToDevice,
                                 h->stream));
    FMPT_CUDA(h, cudaMemcpyAsync(t + ns * sizeof(int64_t), nn.data(), ns * sizeof(int),
                                 cudaMemcpyHostToDevice, h->stream));
    FMPT_CUDA(h, cudaMemcpyAsync(t + ns * (sizeof(int64_t) + sizeof(int)), np.data(),
                                 ns * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    pad_gram_kernel<<<(unsigned)ns, 256, 0, h->stream>>>(
        reinterpret_cast<const int64_t*>(t), reinterpret_cast<const int*>(t + ns * sizeof(int64_t)),
        reinterpret_cast<const int*>(t + ns * (sizeof(int64_t) + sizeof(int))), Gw.d());
    FMPT_LAUNCHED(h);
  }
  // one batched eigensolve per padded size, the sizes concurrently on
  // auxiliary streams (each call is latency bound for n <= a few hundred)
  const int nclass = (int)classes.size();
  const int nstream = std::min(nclass, 6);
  std::vector<size_t> dbytes(nclass, 0), hbytes(nclass, 0), doff(nclass, 0);
  cusolverDnParams_t params;
  FMPT_SOLVER_U1(h, cusolverDnCreateParams(&params));
  int st = ensure_aux(h, nstream);
  size_t dtot = 0;
  int ci = 0;
  for (auto& kv : classes) {
    if (st != FMPT_OK) break;
    const int64_t npad = kv.first, batch = (int64_t)kv.second.size();
    cusolverStatus_t cs = cusolverDnXsyevBatched_bufferSize(
        h->aux_solver[ci % nstream], params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
        npad, CUDA_R_64F, Gw.d() + sec[kv.second[0]].goff, npad, CUDA_R_64F,
        Ww.d() + woff[kv.second[0]], CUDA_R_64F, &dbytes[ci], &hbytes[ci], batch);
    if (cs != CUSOLVER_STATUS_SUCCESS)
      st = set_error(h, FMPT_ERR_CUSOLVER, "syevBatched buffer size: status %d", (int)cs);
    doff[ci] = dtot;
    dtot += (dbytes[ci] + 255) / 256 * 256;
    ci++;
  }
  DevBuf dwork;
  if (st == FMPT_OK) st = dwork.alloc(h, std::max<size_t>(dtot, 256));
  std::vector<std::vector<char>> hwork(nclass);
  if (st == FMPT_OK) st = aux_fork(h, nstream);
  ci = 0;
  int idx0 = 0;
  for (auto& kv : classes) {
    if (st != FMPT_OK) break;
    const int64_t npad = kv.first, batch = (int64_t)kv.second.size();
    hwork[ci].resize(std::max<size_t>(hbytes[ci], 1));
    cusolverStatus_t cs = cusolverDnXsyevBatched(
        h->aux_solver[ci % nstream], params, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
        npad, CUDA_R_64F, Gw.d() + sec[kv.second[0]].goff, npad, CUDA_R_64F,
        Ww.d() + woff[kv.second[0]], CUDA_R_64F, static_cast<char*>(dwork.p) + doff[ci],
        dbytes[ci], hwork[ci].data(), hbytes[ci], static_cast<int*>(info.p) + idx0, batch);
    if (cs != CUSOLVER_STATUS_SUCCESS)
      st = set_error(h, FMPT_ERR_CUSOLVER, "syevBatched: status %d", (int)cs);
    idx0 += (int)batch;
    ci++;
  }
  // join even after a failed call, so no auxiliary work outlives the scratch
  const int jst = ensure_aux(h, nstream) == FMPT_OK ? aux_join(h, nstream) : FMPT_ERR_CUDA;
  cusolverDnDestroyParams(params);
  FMPT_TRY(st);
  FMPT_TRY(jst);
  std::vector<double> lam(wtot);
  std::vector<int> inf(sec.size());
  FMPT_CUDA(h, cudaMemcpyAsync(lam.data(), Ww.p, wtot * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaMemcpyAsync(inf.data(), info.p, sec.size() * sizeof(int),
                               cudaMemcpyDeviceToHost, h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int v : inf)
    if (v != 0) return set_error(h, FMPT_ERR_CUSOLVER, "syevBatched: info %d", v);
  // eigenvalues below the eigensolver's noise floor (~ n eps lambda_max) are
  // exact zeros: their square roots (~1e-8 sigma_max) would be junk directions
  for (size_t si = 0; si < sec.size(); si++) {
    const SplitSector& S_ = sec[si];
    const double lmax = std::max(lam[woff[si] + S_.npad - 1], 0.0);
    const double floor_ = 4.0 * S_.n * 2.220446049250313e-16 * lmax;
    for (int i = 0; i < S_.kq; i++) {
      const double l = lam[woff[si] + S_.npad - 1 - i];
      sv[S_.soff + i] = l > floor_ ? std::sqrt(l) : 0.0;
    }
  }
  return FMPT_OK;
}

}  // namespace

int op_u1_apply(fmpt_op* op, const double* x, double* y, const int* gate) {
  U1OpState* st = static_cast<U1OpState*>(op->u1);
  double* slots[6] = {const_cast<double*>(op->hleft), const_cast<double*>(op->hright),
                      const_cast<double*>(x), y, st->T1.d(), st->T3.d()};
  return gp_run(op->h, st->prog, slots, 6, gate);
}

void op_u1_free(fmpt_op* op) {
  delete static_cast<U1OpState*>(op->u1);
  op->u1 = nullptr;
}

}  // namespace fmpt

using namespace fmpt;

extern "C" {

int fmpt_u1_twosite_size(fmpt_handle* h, const fmpt_u1_space* Vl, const fmpt_u1_space* Vr,
                         int d1, const int* qp1, int d2, const int* qp2, int64_t* n) {
  if (!n) return set_error(h, FMPT_ERR_ARG, "u1: null output");
  Leg L, R;
  FMPT_TRY(read_leg(h, Vl, L, "left leg"));
  FMPT_TRY(read_leg(h, Vr, R, "right leg"));
  FMPT_TRY(check_phys(h, d1, qp1, "site 1"));
  FMPT_TRY(check_phys(h, d2, qp2, "site 2"));
  Pack2 pk;
  build_pack2(L, R, d1, qp1, d2, qp2, pk);
  *n = pk.n;
  return FMPT_OK;
}

int fmpt_u1_pack2(fmpt_handle* h, int dtype, const double* src, double* dst,
                  const fmpt_u1_space* Vl, const fmpt_u1_space* Vr, int d1, const int* qp1,
                  int d2, const int* qp2, int direction) {
  FMPT_TRY(check_real(h, dtype));
  if (!src || !dst) return set_error(h, FMPT_ERR_ARG, "u1_pack2: null pointer");
  if (direction != 0 && direction != 1)
    return set_error(h, FMPT_ERR_ARG, "u1_pack2: direction must be 0 or 1");
  Leg L, R;
  FMPT_TRY(read_leg(h, Vl, L, "left leg"));
  FMPT_TRY(read_leg(h, Vr, R, "right leg"));
  FMPT_TRY(check_phys(h, d1, qp1, "site 1"));
  FMPT_TRY(check_phys(h, d2, qp2, "site 2"));
  Pack2 pk;
  build_pack2(L, R, d1, qp1, d2, qp2, pk);
  const int64_t Dl = L.total, P = pk.P;
  GroupedProgram g;
  gp_phase(g, GP_SUM, FMPT_N, FMPT_N, 0, 0, 1);
  for (int ib = 0; ib < pk.nr; ib++)
    for (int s = 0; s < pk.P; s++)
      for (int ia = 0; ia < pk.nl; ia++) {
        const int64_t po = pk.at(ia, s, ib);
        if (po < 0) continue;
        const int64_t dn = L.off[ia] + Dl * s + Dl * P * R.off[ib];
        if (direction == 0) {
          gp_problem(g, po, L.dim[ia], L.dim[ia], R.dim[ib]);
          gp_segment(g, dn, Dl * P, 0, 0, 0, 1.0);
        } else {
          gp_problem(g, dn, Dl * P, L.dim[ia], R.dim[ib]);
          gp_segment(g, po, L.dim[ia], 0, 0, 0, 1.0);
        }
      }
  const int64_t dense_n = Dl * P * R.total;
  gp_slot(g, 0, direction == 0 ? dense_n : pk.n);
  gp_slot(g, 1, direction == 0 ? pk.n : dense_n);
  FMPT_TRY(gp_finalize(h, g));
  if (direction == 1)
    FMPT_CUDA(h, cudaMemsetAsync(dst, 0, (size_t)Dl * P * R.total * sizeof(double), h->stream));
  double* slots[2] = {const_cast<double*>(src), dst};
  return gp_run(h, g, slots, 2);
}

int fmpt_u1_op_ac2(fmpt_handle* h, int dtype, const double* W1, const double* W2,
                   const double* hleft, const double* hright, const fmpt_u1_space* Vl,
                   const fmpt_u1_space* Vr, int d1, const int* qp1, int d2, const int* qp2,
                   int wl, const int* qwl, int wm, const int* qwm, int wr, const int* qwr,
                   fmpt_op** out) {
  FMPT_TRY(check_real(h, dtype));
  if (!out || !hleft || !hright) return set_error(h, FMPT_ERR_ARG, "u1_op_ac2: null pointer");
  Leg L, R;
  FMPT_TRY(read_leg(h, Vl, L, "left leg"));
  FMPT_TRY(read_leg(h, Vr, R, "right leg"));
  FMPT_TRY(check_phys(h, d1, qp1, "site 1"));
  FMPT_TRY(check_phys(h, d2, qp2, "site 2"));
  FMPT_TRY(check_mpo(h, W1, d1, qp1, wl, qwl, wm, qwm, "W1"));
  FMPT_TRY(check_mpo(h, W2, d2, qp2, wm, qwm, wr, qwr, "W2"));
  Pack2 pk;
  build_pack2(L, R, d1, qp1, d2, qp2, pk);
  const int nl = L.n(), nr = R.n(), P = pk.P;
  const int64_t Dl = L.total, Dr = R.total;
  const std::vector<double> O = two_site_mpo(W1, W2, d1, d2, wl, wm, wr);
  auto Oat = [&](int w, int w2, int so, int si) {
    return O[(((size_t)w * wr + w2) * P + so) * P + si];
  };
  // phase 1 candidates: T1(ia', w, s, ib) = L(ia', w, ia) x(ia, s, ib)
  auto key1 = [&](int iap, int w, int s, int ib) {
    return (((int64_t)iap * wl + w) * P + s) * nr + ib;
  };
  std::vector<P1> p1((size_t)nl * wl * P * nr);
  for (int ib = 0; ib < nr; ib++)
    for (int s = 0; s < P; s++)
      for (int ia = 0; ia < nl; ia++) {
        const int64_t xo = pk.at(ia, s, ib);
        if (xo < 0) continue;
        for (int w = 0; w < wl; w++) {
          const int iap = L.find(L.q[ia] + qwl[w]);
          if (iap < 0) continue;
          P1& p = p1[key1(iap, w, s, ib)];
          p.valid = true;
          p.m = L.dim[iap]; p.n = R.dim[ib]; p.k = L.dim[ia];
          p.a_off = L.off[iap] + Dl * w + Dl * wl * L.off[ia]; p.lda = Dl * wl;
          p.b_off = xo; p.ldb = L.dim[ia];
        }
      }
  // MPO step: T3(ia', s', w2, ib) = sum_{w, s} O[w, w2][s', s] T1(ia', w, s, ib)
  auto key3 = [&](int iap, int so, int w2, int ib) {
    return (((int64_t)iap * P + so) * wr + w2) * nr + ib;
  };
  std::vector<MidBlock> mids;
  for (int ib = 0; ib < nr; ib++)
    for (int w2 = 0; w2 < wr; w2++) {
      const int ibp = R.find(R.q[ib] + qwr[w2]);
      if (ibp < 0) continue;
      for (int so = 0; so < P; so++) {
        const int iap = L.find(R.q[ibp] - pk.qs[so]);
        if (iap < 0) continue;
        MidBlock mb;
        mb.key_out = key3(iap, so, w2, ib);
        mb.m = L.dim[iap]; mb.n = R.dim[ib];
        for (int w = 0; w < wl; w++)
          for (int si = 0; si < P; si++) {
            const double c = Oat(w, w2, so, si);
            if (c == 0.0) continue;
            const int64_t k1 = key1(iap, w, si, ib);
            if (!p1[k1].valid) continue;
            mb.terms.emplace_back(c, k1);
          }
        if (!mb.terms.empty()) mids.push_back(std::move(mb));
      }
    }
  U1OpState* st = new U1OpState();
  GroupedProgram& g = st->prog;
  std::vector<int64_t> t3off((size_t)nl * P * wr * nr, -1);
  int64_t t3n = 0;
  const int64_t t1n = emit_phase1_and_mid(g, FMPT_N, FMPT_N, 0, 2, p1, mids, t3off, &t3n);
  // phase 3: y(ia', s', ib') = sum_{w2} T3(ia', s', w2, ib) R(ib', w2, ib)^T
  gp_phase(g, GP_GEMM, FMPT_N, FMPT_T, 5, 1, 3);
  for (int ibp = 0; ibp < nr; ibp++)
    for (int so = 0; so < P; so++)
      for (int iap = 0; iap < nl; iap++) {
        const int64_t yo = pk.at(iap, so, ibp);
        if (yo < 0) continue;
        gp_problem(g, yo, L.dim[iap], L.dim[iap], R.dim[ibp]);
        for (int w2 = 0; w2 < wr; w2++) {
          const int ib = R.find(R.q[ibp] - qwr[w2]);
          if (ib < 0) continue;
          const int64_t t3 = t3off[key3(iap, so, w2, ib)];
          if (t3 < 0) continue;
          gp_segment(g, t3, L.dim[iap], R.off[ibp] + Dr * w2 + Dr * wr * R.off[ib], Dr * wr,
                     R.dim[ib], 1.0);
        }
      }
  fmpt_op* op = new fmpt_op();
  op->h = h; op->kind = 0; op->dtype = dtype; op->precision = FMPT_PREC_FP64;
  op->Dl = (int)Dl; op->Dr = (int)Dr; op->d1 = d1; op->d2 = d2;
  op->wl = wl; op->wm = wm; op->wr = wr;
  op->hleft = hleft; op->hright = hright;
  op->n = pk.n;
  op->u1 = st;
  st->n = pk.n;
  gp_slot(g, 0, Dl * wl * Dl);
  gp_slot(g, 1, Dr * wr * Dr);
  gp_slot(g, 2, pk.n);
  gp_slot(g, 3, pk.n);
  gp_slot(g, 4, t1n);
  gp_slot(g, 5, t3n);
  int s = gp_finalize(h, g);
  if (s == FMPT_OK) s = alloc_scratch(h, st->T1, t1n);
  if (s == FMPT_OK) s = alloc_scratch(h, st->T3, t3n);
  if (s == FMPT_OK) {
    // tile variant: timed on scratch vectors the first time this work size is seen
    DevBuf xs, ys;
    const bool tune = h->tune_mode == 0 && g.flops >= 2.0e7;
    if (tune) s = alloc_scratch(h, xs, pk.n);
    if (s == FMPT_OK && tune) s = alloc_scratch(h, ys, pk.n);
    if (s == FMPT_OK && tune)
      s = cudaMemsetAsync(xs.p, 0, (size_t)pk.n * sizeof(double), h->stream) == cudaSuccess
              ? FMPT_OK : set_error(h, FMPT_ERR_CUDA, "u1_op_ac2: memset failed");
    if (s == FMPT_OK) {
      double* slots[6] = {const_cast<double*>(hleft), const_cast<double*>(hright), xs.d(), ys.d(),
                          st->T1.d(), st->T3.d()};
      s = gp_autotune(h, g, slots, 6, GP_KIND_HEFF);
    }
  }
  if (s != FMPT_OK) {
    fmpt_op_destroy(op);
    return s;
  }
  *out = op;
  return FMPT_OK;
}

int fmpt_op_tile(fmpt_op* op) {
  if (!op || !op->u1) return 0;
  return (static_cast<U1OpState*>(op->u1)->prog.variant & 1) == 0 ? 32 : 64;
}

int fmpt_op_flops(fmpt_op* op, double* flops) {
  if (!op || !flops) return FMPT_ERR_ARG;
  if (op->u1) {
    const GroupedProgram& g = static_cast<U1OpState*>(op->u1)->prog;
    *flops = g.flops + 2.0 * g.sum_elems;
    return FMPT_OK;
  }
  const double Dl = op->Dl, Dr = op->Dr, D3 = Dl * Dl * Dr;
  const double cf = op->dtype == FMPT_C128 ? 4.0 : 1.0;
  double f = 0.0;
  if (op->kind == 0) {
    const double w = op->wl, P = (double)op->d1 * op->d2;
    f = 4.0 * w * P * D3 + 4.0 * w * w * P * op->d1 * Dl * Dr;
  } else if (op->kind == 1) {
    const double w = op->wl, d = op->d1;
    f = 4.0 * w * d * D3 + 2.0 * w * w * d * d * Dl * Dr;
  } else {
    f = 4.0 * op->wl * D3;
  }
  *flops = cf * f;
  return FMPT_OK;
}

int fmpt_u1_twosite(fmpt_handle* h, int dtype, const double* A, const double* B, double* x,
                    const fmpt_u1_space* Vl, const fmpt_u1_space* Vm, const fmpt_u1_space* Vr,
                    int d1, const int* qp1, int d2, const int* qp2) {
  FMPT_TRY(check_real(h, dtype));
  if (!A || !B || !x) return set_error(h, FMPT_ERR_ARG, "u1_twosite: null pointer");
  Leg L, M, R;
  FMPT_TRY(read_leg(h, Vl, L, "left leg"));
  FMPT_TRY(read_leg(h, Vm, M, "middle leg"));
  FMPT_TRY(read_leg(h, Vr, R, "right leg"));
  FMPT_TRY(check_phys(h, d1, qp1, "site 1"));
  FMPT_TRY(check_phys(h, d2, qp2, "site 2"));
  Pack2 pk;
  build_pack2(L, R, d1, qp1, d2, qp2, pk);
  const int64_t Dl = L.total, Dm = M.total;
  GroupedProgram g;
  gp_phase(g, GP_GEMM, FMPT_N, FMPT_N, 0, 1, 2);
  for (int ib = 0; ib < pk.nr; ib++)
    for (int s = 0; s < pk.P; s++)
      for (int ia = 0; ia < pk.nl; ia++) {
        const int64_t xo = pk.at(ia, s, ib);
        if (xo < 0) continue;
        const int s1 = s % d1, s2 = s / d1;
        gp_problem(g, xo, L.dim[ia], L.dim[ia], R.dim[ib]);
        const int im = M.find(L.q[ia] + qp1[s1]);
        if (im < 0) continue;   // no such middle sector: the block is zero
        gp_segment(g, L.off[ia] + Dl * s1 + Dl * d1 * M.off[im], Dl * d1,
                   M.off[im] + Dm * s2 + Dm * d2 * R.off[ib], Dm * d2, M.dim[im], 1.0);
      }
  gp_slot(g, 0, Dl * d1 * Dm);
  gp_slot(g, 1, Dm * d2 * R.total);
  gp_slot(g, 2, pk.n);
  FMPT_TRY(gp_finalize(h, g));
  double* slots[3] = {const_cast<double*>(A), const_cast<double*>(B), x};
  return gp_run(h, g, slots, 3);
}

static int u1_env(fmpt_handle* h, bool right, int dtype, const double* hold, const double* A,
                  const double* W, const double* B, double* hnew, const fmpt_u1_space* Vl,
                  const fmpt_u1_space* Vr, int d, const int* qp, int wl, const int* qwl, int wr,
                  const int* qwr) {
  FMPT_TRY(check_real(h, dtype));
  if (!hold || !A || !B || !hnew) return set_error(h, FMPT_ERR_ARG, "u1 env: null pointer");
  Leg L, R;
  FMPT_TRY(read_leg(h, Vl, L, "left leg"));
  FMPT_TRY(read_leg(h, Vr, R, "right leg"));
  FMPT_TRY(check_phys(h, d, qp, "site"));
  FMPT_TRY(check_mpo(h, W, d, qp, wl, qwl, wr, qwr, "W"));
  const int nl = L.n(), nr = R.n();
  const int64_t Dl = L.total, Dr = R.total;
  auto Wat = [&](int w, int so, int w2, int si) {
    return W[w + (int64_t)wl * (so + d * (w2 + (int64_t)wr * si))];
  };
  GroupedProgram g;
  std::vector<P1> p1;
  std::vector<MidBlock> mids;
  std::vector<int64_t> t3off;
  int64_t t1n = 0, t3n = 0;
  int64_t out_elems = 0;
  if (!right) {
    // T1(ia', w, s, ib) = hold(ia', w, ia) B(ia, s, ib)
    auto key1 = [&](int iap, int w, int s, int ib) {
      return (((int64_t)iap * wl + w) * d + s) * nr + ib;
    };
    p1.resize((size_t)nl * wl * d * nr);
    for (int ib = 0; ib < nr; ib++)
      for (int s = 0; s < d; s++) {
        const int ia = L.find(R.q[ib] - qp[s]);
        if (ia < 0) continue;
        for (int w = 0; w < wl; w++) {
          const int iap = L.find(L.q[ia] + qwl[w]);
          if (iap < 0) continue;
          P1& p = p1[key1(iap, w, s, ib)];
          p.valid = true;
          p.m = L.dim[iap]; p.n = R.dim[ib]; p.k = L.dim[ia];
          p.a_off = L.off[iap] + Dl * w + Dl * wl * L.off[ia]; p.lda = Dl * wl;
          p.b_off = L.off[ia] + Dl * s + Dl * d * R.off[ib]; p.ldb = Dl * d;
        }
      }
    // T3(ia', s', w2, ib) = sum_{w, s} W[w, s', w2, s] T1(ia', w, s, ib)
    auto key3 = [&](int iap, int so, int w2, int ib) {
      return (((int64_t)iap * d + so) * wr + w2) * nr + ib;
    };
    for (int ib = 0; ib < nr; ib++)
      for (int w2 = 0; w2 < wr; w2++) {
        const int ibp = R.find(R.q[ib] + qwr[w2]);
        if (ibp < 0) continue;
        for (int so = 0; so < d; so++) {
          const int iap = L.find(R.q[ibp] - qp[so]);
          if (iap < 0) continue;
          MidBlock mb;
          mb.key_out = key3(iap, so, w2, ib);
          mb.m = L.dim[iap]; mb.n = R.dim[ib];
          for (int w = 0; w < wl; w++)
            for (int si = 0; si < d; si++) {
              const double c = Wat(w, so, w2, si);
              if (c == 0.0) continue;
              const int64_t k1 = key1(iap, w, si, ib);
              if (p1[k1].valid) mb.terms.emplace_back(c, k1);
            }
          if (!mb.terms.empty()) mids.push_back(std::move(mb));
        }
      }
    t3off.assign((size_t)nl * d * wr * nr, -1);
    t1n = emit_phase1_and_mid(g, FMPT_N, FMPT_N, 0, 2, p1, mids, t3off, &t3n);
    // hnew(ib', w2, ib) = sum_{s'} A(ia', s', ib')^T T3(ia', s', w2, ib)
    gp_phase(g, GP_GEMM, FMPT_T, FMPT_N, 1, 5, 3);
    for (int ib = 0; ib < nr; ib++)
      for (int w2 = 0; w2 < wr; w2++) {
        const int ibp = R.find(R.q[ib] + qwr[w2]);
        if (ibp < 0) continue;
        gp_problem(g, R.off[ibp] + Dr * w2 + Dr * wr * R.off[ib], Dr * wr, R.dim[ibp], R.dim[ib]);
        for (int so = 0; so < d; so++) {
          const int iap = L.find(R.q[ibp] - qp[so]);
          if (iap < 0) continue;
          const int64_t t3 = t3off[key3(iap, so, w2, ib)];
          if (t3 < 0) continue;
          gp_segment(g, L.off[iap] + Dl * so + Dl * d * R.off[ibp], Dl * d, t3, L.dim[iap],
                     L.dim[iap], 1.0);
        }
      }
    out_elems = Dr * wr * Dr;
  } else {
    // T1(ia, s, w2, ib') = B(ia, s, ib) hold(ib', w2, ib)^T
    auto key1 = [&](int ia, int s, int w2, int ibp) {
      return (((int64_t)ia * d + s) * wr + w2) * nr + ibp;
    };
    p1.resize((size_t)nl * d * wr * nr);
    for (int ia = 0; ia < nl; ia++)
      for (int s = 0; s < d; s++) {
        const int ib = R.find(L.q[ia] + qp[s]);
        if (ib < 0) continue;
        for (int w2 = 0; w2 < wr; w2++) {
          const int ibp = R.find(R.q[ib] + qwr[w2]);
          if (ibp < 0) continue;
          P1& p = p1[key1(ia, s, w2, ibp)];
          p.valid = true;
          p.m = L.dim[ia]; p.n = R.dim[ibp]; p.k = R.dim[ib];
          p.a_off = L.off[ia] + Dl * s + Dl * d * R.off[ib]; p.lda = Dl * d;
          p.b_off = R.off[ibp] + Dr * w2 + Dr * wr * R.off[ib]; p.ldb = Dr * wr;
        }
      }
    // T3(ia, s', w, ib') = sum_{w2, s} W[w, s', w2, s] T1(ia, s, w2, ib')
    auto key3 = [&](int ia, int so, int w, int ibp) {
      return (((int64_t)ia * d + so) * wl + w) * nr + ibp;
    };
    for (int ia = 0; ia < nl; ia++)
      for (int w = 0; w < wl; w++) {
        const int iap = L.find(L.q[ia] + qwl[w]);
        if (iap < 0) continue;
        for (int so = 0; so < d; so++) {
          const int ibp = R.find(L.q[iap] + qp[so]);
          if (ibp < 0) continue;
          MidBlock mb;
          mb.key_out = key3(ia, so, w, ibp);
          mb.m = L.dim[ia]; mb.n = R.dim[ibp];
          for (int w2 = 0; w2 < wr; w2++)
            for (int si = 0; si < d; si++) {
              const double c = Wat(w, so, w2, si);
              if (c == 0.0) continue;
              const int64_t k1 = key1(ia, si, w2, ibp);
              if (p1[k1].valid) mb.terms.emplace_back(c, k1);
            }
          if (!mb.terms.empty()) mids.push_back(std::move(mb));
        }
      }
    t3off.assign((size_t)nl * d * wl * nr, -1);
    t1n = emit_phase1_and_mid(g, FMPT_N, FMPT_T, 2, 0, p1, mids, t3off, &t3n);
    // hnew(ia', w, ia) = sum_{s'} A(ia', s', ib') T3(ia, s', w, ib')^T
    gp_phase(g, GP_GEMM, FMPT_N, FMPT_T, 1, 5, 3);
    for (int ia = 0; ia < nl; ia++)
      for (int w = 0; w < wl; w++) {
        const int iap = L.find(L.q[ia] + qwl[w]);
        if (iap < 0) continue;
        gp_problem(g, L.off[iap] + Dl * w + Dl * wl * L.off[ia], Dl * wl, L.dim[iap], L.dim[ia]);
        for (int so = 0; so < d; so++) {
          const int ibp = R.find(L.q[iap] + qp[so]);
          if (ibp < 0) continue;
          const int64_t t3 = t3off[key3(ia, so, w, ibp)];
          if (t3 < 0) continue;
          gp_segment(g, L.off[iap] + Dl * so + Dl * d * R.off[ibp], Dl * d, t3, L.dim[ia],
                     R.dim[ibp], 1.0);
        }
      }
    out_elems = Dl * wl * Dl;
  }
  gp_slot(g, 0, right ? Dr * wr * Dr : Dl * wl * Dl);
  gp_slot(g, 1, Dl * d * Dr);
  gp_slot(g, 2, Dl * d * Dr);
  gp_slot(g, 3, out_elems);
  gp_slot(g, 4, t1n);
  gp_slot(g, 5, t3n);
  FMPT_TRY(gp_finalize(h, g));
  ScratchPair sc;
  FMPT_TRY(alloc_scratch(h, sc.T1, t1n));
  FMPT_TRY(alloc_scratch(h, sc.T3, t3n));
  FMPT_CUDA(h, cudaMemsetAsync(hnew, 0, (size_t)out_elems * sizeof(double), h->stream));
  double* slots[6] = {const_cast<double*>(hold), const_cast<double*>(A), const_cast<double*>(B),
                      hnew, sc.T1.d(), sc.T3.d()};
  FMPT_TRY(gp_autotune(h, g, slots, 6, GP_KIND_ENV));   // reruns write the same values
  return gp_run(h, g, slots, 6);
}

int fmpt_u1_updateleft(fmpt_handle* h, int dtype, const double* hold, const double* A,
                       const double* W, const double* B, double* hnew, const fmpt_u1_space* Vl,
                       const fmpt_u1_space* Vr, int d, const int* qp, int wl, const int* qwl,
                       int wr, const int* qwr) {
  return u1_env(h, false, dtype, hold, A, W, B, hnew, Vl, Vr, d, qp, wl, qwl, wr, qwr);
}

int fmpt_u1_updateright(fmpt_handle* h, int dtype, const double* hold, const double* A,
                        const double* W, const double* B, double* hnew, const fmpt_u1_space* Vl,
                        const fmpt_u1_space* Vr, int d, const int* qp, int wl, const int* qwl,
                        int wr, const int* qwr) {
  return u1_env(h, true, dtype, hold, A, W, B, hnew, Vl, Vr, d, qp, wl, qwl, wr, qwr);
}

int fmpt_u1_split(fmpt_handle* h, int dtype, const double* x, const fmpt_u1_space* Vl,
                  const fmpt_u1_space* Vr, int d1, const int* qp1, int d2, const int* qp2,
                  int maxD, double eps, int side, int method, double* A, double* S, double* B,
                  int cap, int* nsect_out, int* charge_out, int* dim_out, double* err) {
  FMPT_TRY(check_real(h, dtype));
  if (!x || !A || !S || !B || !nsect_out || !charge_out || !dim_out)
    return set_error(h, FMPT_ERR_ARG, "u1_split: null pointer");
  if (maxD < 1) return set_error(h, FMPT_ERR_SHAPE, "u1_split: maxD must be >= 1");
  if (side != 0 && side != 1) return set_error(h, FMPT_ERR_ARG, "u1_split: side must be 0 or 1");
  if (method != 0 && method != 1)
    return set_error(h, FMPT_ERR_ARG, "u1_split: method must be 0 (SVD) or 1 (density matrix)");
  Leg L, R;
  FMPT_TRY(read_leg(h, Vl, L, "left leg"));
  FMPT_TRY(read_leg(h, Vr, R, "right leg"));
  FMPT_TRY(check_phys(h, d1, qp1, "site 1"));
  FMPT_TRY(check_phys(h, d2, qp2, "site 2"));
  Pack2 pk;
  build_pack2(L, R, d1, qp1, d2, qp2, pk);
  const int nl = L.n(), nr = R.n();
  const int64_t Dl = L.total, Dr = R.total;
  // sectors of the new bond: rows (s1, ia) and columns (s2, ib) of each charge
  std::vector<int> cand;
  for (int s1 = 0; s1 < d1; s1++)
    for (int ia = 0; ia < nl; ia++) cand.push_back(L.q[ia] + qp1[s1]);
  std::sort(cand.begin(), cand.end());
  cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
  std::vector<SplitSector> sec;
  int64_t mtot = 0, utot = 0, vtot = 0, stot = 0, wmax = 0;
  for (int qc : cand) {
    SplitSector S_;
    S_.q = qc;
    for (int s1 = 0; s1 < d1; s1++)
      for (int ia = 0; ia < nl; ia++)
        if (L.q[ia] + qp1[s1] == qc) { S_.rows.push_back({s1, ia, S_.r}); S_.r += L.dim[ia]; }
    for (int s2 = 0; s2 < d2; s2++)
      for (int ib = 0; ib < nr; ib++)
        if (R.q[ib] - qp2[s2] == qc) { S_.cols.push_back({s2, ib, S_.c}); S_.c += R.dim[ib]; }
    if (S_.r == 0 || S_.c == 0) continue;
    S_.kq = std::min(S_.r, S_.c);
    S_.moff = mtot; mtot += (int64_t)S_.r * S_.c;
    S_.soff = stot; stot += S_.kq;
    if (method == 0) {
      S_.uoff = utot; utot += (int64_t)S_.r * S_.kq;
      S_.voff = vtot; vtot += (int64_t)S_.kq * S_.c;
      if (S_.r < S_.c) wmax = std::max(wmax, (int64_t)S_.r * S_.c);
    }
    sec.push_back(std::move(S_));
  }
  if (sec.empty()) return set_error(h, FMPT_ERR_SHAPE, "u1_split: no allowed charge sector");
  DevBuf Mw, Uw, Vw, Sw, Tw;
  FMPT_TRY(alloc_scratch(h, Mw, mtot));
  {  // gather every sector matrix in one launch
    GroupedProgram g;
    gp_phase(g, GP_SUM, FMPT_N, FMPT_N, 0, 0, 1);
    for (const SplitSector& S_ : sec)
      for (const SplitSeg& rs : S_.rows)
        for (const SplitSeg& cs : S_.cols) {
          const int64_t xo = pk.at(rs.i, rs.s + d1 * cs.s, cs.i);
          if (xo < 0) return set_error(h, FMPT_ERR_ARG, "u1_split: inconsistent sector table");
          gp_problem(g, S_.moff + rs.off + cs.off * S_.r, S_.r, L.dim[rs.i], R.dim[cs.i]);
          gp_segment(g, xo, L.dim[rs.i], 0, 0, 0, 1.0);
        }
    gp_slot(g, 0, pk.n);
    gp_slot(g, 1, mtot);
    FMPT_TRY(gp_finalize(h, g));
    double* slots[2] = {const_cast<double*>(x), Mw.d()};
    FMPT_TRY(gp_run(h, g, slots, 2));
  }
  std::vector<double> sv(stot, 0.0);
  DevBuf Gw;   // density-matrix form: Gram matrices, then their eigenvectors
  if (method == 0) {
    // per-sector FP64 SVD on the device
    FMPT_TRY(alloc_scratch(h, Uw, utot));
    FMPT_TRY(alloc_scratch(h, Vw, vtot));
    FMPT_TRY(alloc_scratch(h, Sw, stot));
    FMPT_TRY(alloc_scratch(h, Tw, wmax));
    for (const SplitSector& S_ : sec) {
      double* Mq = Mw.d() + S_.moff;
      double* Uq = Uw.d() + S_.uoff;
      double* Vq = Vw.d() + S_.voff;
      double* Sq = Sw.d() + S_.soff;
      if (S_.r >= S_.c) {
        FMPT_TRY(svd_tall(h, 0, S_.r, S_.c, Mq, Sq, Uq, Vq));
      } else {
        // M^T (c x r) = U' S VT'  ->  M = VT'^T S U'^T
        DevBuf U2, V2;
        FMPT_TRY(alloc_scratch(h, U2, (int64_t)S_.c * S_.r));
        FMPT_TRY(alloc_scratch(h, V2, (int64_t)S_.r * S_.r));
        FMPT_TRY(copy_mat(h, 0, S_.c, S_.r, Mq, S_.r, 0, 1, 0, Tw.d(), S_.c, 0));
        FMPT_TRY(svd_tall(h, 0, S_.c, S_.r, Tw.d(), Sq, U2.d(), V2.d()));
        FMPT_TRY(copy_mat(h, 0, S_.r, S_.r, V2.d(), S_.r, 0, 1, 0, Uq, S_.r, 0));
        FMPT_TRY(copy_mat(h, 0, S_.r, S_.c, U2.d(), S_.c, 0, 1, 0, Vq, S_.kq, 0));
      }
    }
    FMPT_CUDA(h, cudaMemcpyAsync(sv.data(), Sw.d(), stot * sizeof(double),
                                 cudaMemcpyDeviceToHost, h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  } else {
    FMPT_TRY(density_eigen(h, side, sec, Mw.d(), mtot, Gw, sv));
  }
  FMPT_TRY(gp_check_status(h));
  // truncation across sectors (MPSTruncation: cutoff relative to the norm, then dimension)
  double nrm2 = 0.0;
  for (double v : sv) nrm2 += v * v;
  const double nrm = std::sqrt(nrm2);
  struct Val { double v; int sec, idx; };
  std::vector<Val> kept;
  for (int si = 0; si < (int)sec.size(); si++)
    for (int i = 0; i < sec[si].kq; i++) {
      const double v = sv[sec[si].soff + i];
      if (v >= eps * nrm && (method == 0 || v > 0.0)) kept.push_back({v, si, i});
    }
  std::stable_sort(kept.begin(), kept.end(), [](const Val& a, const Val& b) {
    if (a.v != b.v) return a.v > b.v;
    if (a.sec != b.sec) return a.sec < b.sec;
    return a.idx < b.idx;
  });
  if ((int)kept.size() > maxD) kept.resize(maxD);
  for (const Val& v : kept) sec[v.sec].keep = std::max(sec[v.sec].keep, v.idx + 1);
  double kept2 = 0.0, drop2 = 0.0;
  for (const SplitSector& S_ : sec)
    for (int i = 0; i < S_.kq; i++) {
      const double v2 = sv[S_.soff + i] * sv[S_.soff + i];
      if (i < S_.keep) kept2 += v2; else drop2 += v2;
    }
  if (!(kept2 > 0.0)) return set_error(h, FMPT_ERR_NONFINITE, "u1_split: zero two-site tensor");
  if (err) *err = std::sqrt(drop2);
  const double knorm = std::sqrt(kept2);
  // the new leg
  int ns = 0;
  int64_t Dm = 0;
  std::vector<int64_t> moff2(sec.size(), -1);
  for (size_t si = 0; si < sec.size(); si++) {
    if (sec[si].keep == 0) continue;
    if (ns >= cap) return set_error(h, FMPT_ERR_SHAPE, "u1_split: sector capacity %d too small", cap);
    charge_out[ns] = sec[si].q;
    dim_out[ns] = sec[si].keep;
    moff2[si] = Dm;
    Dm += sec[si].keep;
    ns++;
  }
  *nsect_out = ns;
  std::vector<double> sn(stot, 0.0), skept;
  for (const SplitSector& S_ : sec)
    for (int i = 0; i < S_.keep; i++) {
      sn[S_.soff + i] = sv[S_.soff + i] / knorm;
      skept.push_back(sn[S_.soff + i]);
    }
  FMPT_CUDA(h, cudaMemcpyAsync(S, skept.data(), skept.size() * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
  FMPT_CUDA(h, cudaMemsetAsync(A, 0, (size_t)Dl * d1 * Dm * sizeof(double), h->stream));
  FMPT_CUDA(h, cudaMemsetAsync(B, 0, (size_t)Dm * d2 * Dr * sizeof(double), h->stream));
  GroupedProgram g;
  if (method == 0) {
    // normalised sigma (zero past the kept prefix) into the factor that carries s
    FMPT_CUDA(h, cudaMemcpyAsync(Sw.d(), sn.data(), stot * sizeof(double),
                                 cudaMemcpyHostToDevice, h->stream));
    for (const SplitSector& S_ : sec) {
      if (S_.keep == 0) continue;
      if (side == 0)
        FMPT_TRY(fmpt_scale_dim(h, FMPT_F64, 0, S_.kq, S_.c, Sw.d() + S_.soff, Vw.d() + S_.voff));
      else
        FMPT_TRY(fmpt_scale_dim(h, FMPT_F64, 1, S_.r, S_.kq, Sw.d() + S_.soff, Uw.d() + S_.uoff));
    }
    // scatter the kept columns of U into A[a, s1, m] and rows of V into B[m, s2, b]
    gp_phase(g, GP_SUM, FMPT_N, FMPT_N, 0, 0, 2);
    for (size_t si = 0; si < sec.size(); si++) {
      const SplitSector& S_ = sec[si];
      if (S_.keep == 0) continue;
      for (const SplitSeg& rs : S_.rows) {
        gp_problem(g, L.off[rs.i] + Dl * rs.s + Dl * d1 * moff2[si], Dl * d1, L.dim[rs.i], S_.keep);
        gp_segment(g, S_.uoff + rs.off, S_.r, 0, 0, 0, 1.0);
      }
    }
    gp_phase(g, GP_SUM, FMPT_N, FMPT_N, 1, 1, 3);
    for (size_t si = 0; si < sec.size(); si++) {
      const SplitSector& S_ = sec[si];
      if (S_.keep == 0) continue;
      for (const SplitSeg& cs : S_.cols) {
        gp_problem(g, moff2[si] + Dm * cs.s + Dm * d2 * R.off[cs.i], Dm * d2, S_.keep, R.dim[cs.i]);
        gp_segment(g, S_.voff + cs.off * S_.kq, S_.kq, 0, 0, 0, 1.0);
      }
    }
    gp_slot(g, 0, utot);
    gp_slot(g, 1, vtot);
  } else {
    // Q: the kept eigenvectors (largest first), n x keep per sector, contiguous
    int64_t qtot = 0;
    std::vector<int64_t> qoff(sec.size(), 0);
    for (size_t si = 0; si < sec.size(); si++) {
      qoff[si] = qtot;
      qtot += (int64_t)sec[si].n * sec[si].keep;
    }
    FMPT_TRY(alloc_scratch(h, Uw, qtot));
    for (size_t si = 0; si < sec.size(); si++) {
      const SplitSector& S_ = sec[si];
      if (S_.keep == 0) continue;
      FMPT_TRY(copy_mat(h, 0, S_.n, S_.keep, Gw.d() + S_.goff + (int64_t)(S_.npad - 1) * S_.npad,
                        -(int64_t)S_.npad, 0, 0, 0, Uw.d() + qoff[si], S_.n, 0));
    }
    const double inv = 1.0 / knorm;
    if (side == 0) {
      // A = U (isometric); B = U^T M / ||s_kept|| (= normalised s * v)
      gp_phase(g, GP_SUM, FMPT_N, FMPT_N, 0, 0, 2);
      for (size_t si = 0; si < sec.size(); si++) {
        const SplitSector& S_ = sec[si];
        if (S_.keep == 0) continue;
        for (const SplitSeg& rs : S_.rows) {
          gp_problem(g, L.off[rs.i] + Dl * rs.s + Dl * d1 * moff2[si], Dl * d1, L.dim[rs.i],
                     S_.keep);
          gp_segment(g, qoff[si] + rs.off, S_.r, 0, 0, 0, 1.0);
        }
      }
      gp_phase(g, GP_GEMM, FMPT_T, FMPT_N, 0, 1, 3);
      for (size_t si = 0; si < sec.size(); si++) {
        const SplitSector& S_ = sec[si];
        if (S_.keep == 0) continue;
        for (const SplitSeg& cs : S_.cols) {
          gp_problem(g, moff2[si] + Dm * cs.s + Dm * d2 * R.off[cs.i], Dm * d2, S_.keep,
                     R.dim[cs.i]);
          gp_segment(g, qoff[si], S_.r, S_.moff + cs.off * S_.r, S_.r, S_.r, inv);
        }
      }
    } else {
      // B = V^T (isometric rows); A = M V / ||s_kept|| (= u * normalised s)
      gp_phase(g, GP_SUM, FMPT_T, FMPT_N, 0, 0, 3);
      for (size_t si = 0; si < sec.size(); si++) {
        const SplitSector& S_ = sec[si];
        if (S_.keep == 0) continue;
        for (const SplitSeg& cs : S_.cols) {
          gp_problem(g, moff2[si] + Dm * cs.s + Dm * d2 * R.off[cs.i], Dm * d2, S_.keep,
                     R.dim[cs.i]);
          gp_segment(g, qoff[si] + cs.off, S_.c, 0, 0, 0, 1.0);
        }
      }
      gp_phase(g, GP_GEMM, FMPT_N, FMPT_N, 1, 0, 2);
      for (size_t si = 0; si < sec.size(); si++) {
        const SplitSector& S_ = sec[si];
        if (S_.keep == 0) continue;
        for (const SplitSeg& rs : S_.rows) {
          gp_problem(g, L.off[rs.i] + Dl * rs.s + Dl * d1 * moff2[si], Dl * d1, L.dim[rs.i],
                     S_.keep);
          gp_segment(g, S_.moff + rs.off, S_.r, qoff[si], S_.c, S_.c, inv);
        }
      }
    }
    gp_slot(g, 0, qtot);
    gp_slot(g, 1, mtot);
  }
  gp_slot(g, 2, Dl * d1 * Dm);
  gp_slot(g, 3, Dm * d2 * Dr);
  FMPT_TRY(gp_finalize(h, g));
  double* slots[4] = {Uw.d(), method == 0 ? Vw.d() : Mw.d(), A, B};
  FMPT_TRY(gp_run(h, g, slots, 4));
  // host vectors above were staged by the (pageable) copies; the scratch
  // buffers are stream-ordered, so nothing else needs to wait here
  return FMPT_OK;
}

}  // extern "C"
