// Effective-Hamiltonian actions and environment updates, plain FP64 form.
//
// Every contraction is GEMM -> block-sparse MPO step -> GEMM, in the
// reference's pairwise order (derivatives.jl:21, mpo/transfer.jl:27,32):
//   1. L . x            one GEMM over the ket index          (2 w P D^3 flop)
//   2. MPO step         sum over the NONZERO (w, w') blocks    (D^2 cost)
//   3. . R / . conj(A)  one GEMM over (w', ket)              (2 w P D^3 flop)
// The MPO step replaces the reference's per-chain recontraction of the
// Schur form (derivatives.jl:24-49): the nonzero (w, w') blocks of the
// (two-site) MPO are found once on the host and applied at O(D^2) cost.
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "internal.h"

namespace fmpt {
namespace {

template <int MAXP, bool CPLX>
__global__ void mid_kernel(const double* __restrict__ in, int64_t plane_in, MidStrides si,
                           double* __restrict__ out, int64_t plane_out, MidStrides so, int n1,
                           int n2, int nw_out, int p_in, int p_out, const int* __restrict__ win,
                           const int* __restrict__ wstart, const double* __restrict__ coef) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n1 * n2) return;
  const int o1 = (int)(t % n1), o2 = (int)(t / n1);
  const double* ib = in + o1 * si.o1 + o2 * si.o2;
  double* ob = out + o1 * so.o1 + o2 * so.o2;
  const int csz = p_out * p_in;
  for (int wo = 0; wo < nw_out; wo++) {
    double acc[MAXP], acci[MAXP];
#pragma unroll
    for (int q = 0; q < MAXP; q++) { acc[q] = 0.0; acci[q] = 0.0; }
    const int b1 = __ldg(wstart + wo + 1);
    for (int b = __ldg(wstart + wo); b < b1; b++) {
      const int wi = __ldg(win + b);
      const double* c = coef + (int64_t)b * csz * (CPLX ? 2 : 1);
      double v[MAXP], vi[MAXP];
#pragma unroll
      for (int s = 0; s < MAXP; s++) {
        v[s] = 0.0; vi[s] = 0.0;
        if (s < p_in) {
          v[s] = ib[wi * si.w + s * si.s];
          if (CPLX) vi[s] = ib[plane_in + wi * si.w + s * si.s];
        }
      }
#pragma unroll
      for (int q = 0; q < MAXP; q++) {
        if (q >= p_out) break;
#pragma unroll
        for (int s = 0; s < MAXP; s++) {
          if (s >= p_in) break;
          const double cr = __ldg(c + q * p_in + s);
          if (CPLX) {
            const double ci = __ldg(c + csz + q * p_in + s);
            acc[q] = fma(cr, v[s], acc[q]);
            acc[q] = fma(-ci, vi[s], acc[q]);
            acci[q] = fma(cr, vi[s], acci[q]);
            acci[q] = fma(ci, v[s], acci[q]);
          } else {
            acc[q] = fma(cr, v[s], acc[q]);
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < MAXP; q++) {
      if (q >= p_out) break;
      ob[wo * so.w + q * so.s] = acc[q];
      if (CPLX) ob[plane_out + wo * so.w + q * so.s] = acci[q];
    }
  }
}

// Sparse form of the block step: for each output (wo, q) the list of its nonzero terms
// (wi, s, coefficient), in block order then s -- the order in which mid_kernel adds them,
// so that both give the same sums.  It does only the nonzero multiply-adds (the two-site
// blocks are Kronecker products of single-site operators, mostly zeros), which is what
// bounds the step on GB300's FP64 pipe.  Passed by value.
struct MidSparse {
  int n_out;                          // nw_out * p_out
  short start[MS_MAX_OUT + 1];
  short idx[MS_MAX_T];                // wi * 16 + s
  double c[MS_MAX_T];                 // real coefficients; complex: re, im pairs
};

template <bool CPLX>
__global__ void mid_sparse_kernel(const double* __restrict__ in, int64_t plane_in, MidStrides si,
                                  double* __restrict__ out, int64_t plane_out, MidStrides so,
                                  int n1, int n2, int p_out, const __grid_constant__ MidSparse ms) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n1 * n2) return;
  const int o1 = (int)(t % n1), o2 = (int)(t / n1);
  const double* ib = in + o1 * si.o1 + o2 * si.o2;
  double* ob = out + o1 * so.o1 + o2 * so.o2;
  for (int o = 0; o < ms.n_out; o++) {
    const int wo = o / p_out, q = o - wo * p_out;
    double ar = 0.0, ai = 0.0;
    for (int e = ms.start[o]; e < ms.start[o + 1]; e++) {
      const int ix = ms.idx[e];
      const int64_t off = (ix >> 4) * si.w + (ix & 15) * si.s;
      const double vr = ib[off];
      if (CPLX) {
        const double vi = ib[plane_in + off];
        const double cr = ms.c[2 * e], ci = ms.c[2 * e + 1];
        ar = fma(cr, vr, ar);
        ar = fma(-ci, vi, ar);
        ai = fma(cr, vi, ai);
        ai = fma(ci, vr, ai);
      } else {
        ar = fma(ms.c[e], vr, ar);
      }
    }
    ob[wo * so.w + q * so.s] = ar;
    if (CPLX) ob[plane_out + wo * so.w + q * so.s] = ai;
  }
}

// host-side complex helpers for schedule construction
struct C2 { double r, i; };
inline C2 cmul(C2 a, C2 b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }

inline C2 wget(const double* W, int cplx, int64_t nW, int64_t idx) {
  return {W[idx], cplx ? W[nW + idx] : 0.0};
}

// Builds the block list from a dense tensor O[wi][wo][so][si] (host).
void build_schedule(int cplx, int nw_in, int nw_out, int p_in, int p_out,
                    const std::vector<C2>& O, MidSchedule& s) {
  s.nw_in = nw_in; s.nw_out = nw_out; s.p_in = p_in; s.p_out = p_out; s.cplx = cplx;
  s.blk_win.clear(); s.wout_start.assign(nw_out + 1, 0); s.coef.clear();
  const int csz = p_in * p_out;
  for (int wo = 0; wo < nw_out; wo++) {
    s.wout_start[wo] = (int)s.blk_win.size();
    for (int wi = 0; wi < nw_in; wi++) {
      const C2* blk = &O[((size_t)wi * nw_out + wo) * csz];
      bool nz = false;
      for (int q = 0; q < csz; q++) nz |= (blk[q].r != 0.0 || blk[q].i != 0.0);
      if (!nz) continue;
      s.blk_win.push_back(wi);
      for (int q = 0; q < csz; q++) s.coef.push_back(blk[q].r);
      if (cplx)
        for (int q = 0; q < csz; q++) s.coef.push_back(blk[q].i);
    }
  }
  s.wout_start[nw_out] = (int)s.blk_win.size();
  // the sparse term lists (left empty when they do not fit MidSparse)
  s.sp_start.clear();
  s.sp_idx.clear();
  s.sp_coef.clear();
  const int cap = cplx ? MS_MAX_T / 2 : MS_MAX_T;
  bool fits = nw_out * p_out <= MS_MAX_OUT && p_in <= 16;
  std::vector<int> st, ix;
  std::vector<double> cf;
  for (int wo = 0; wo < nw_out && fits; wo++)
    for (int q = 0; q < p_out && fits; q++) {
      st.push_back((int)ix.size());
      for (int b = s.wout_start[wo]; b < s.wout_start[wo + 1]; b++) {
        const double* cb = &s.coef[(size_t)b * csz * (cplx ? 2 : 1)];
        for (int si = 0; si < p_in; si++) {
          const double cr = cb[q * p_in + si], ci = cplx ? cb[csz + q * p_in + si] : 0.0;
          if (cr == 0.0 && ci == 0.0) continue;
          ix.push_back(s.blk_win[b] * 16 + si);
          cf.push_back(cr);
          if (cplx) cf.push_back(ci);
        }
      }
      if ((int)ix.size() > cap) fits = false;
    }
  if (fits) {
    st.push_back((int)ix.size());
    s.sp_start = st;
    s.sp_idx = ix;
    s.sp_coef = cf;
  }
}

}  // namespace

int set_error(fmpt_handle* h, int status, const char* fmt, ...) {
  if (h) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->err = buf;
  }
  return status;
}

int schedule_ac2(fmpt_handle* h, int cplx, const double* W1, const double* W2, int d1, int d2,
                 int wl, int wm, int wr, MidSchedule& s) {
  if (!W1 || !W2) return set_error(h, FMPT_ERR_ARG, "ac2: null MPO tensor");
  schedule_ac2_host(cplx, W1, W2, d1, d2, wl, wm, wr, s);
  return mid_upload(h, s);
}

void schedule_ac2_host(int cplx, const double* W1, const double* W2, int d1, int d2, int wl,
                       int wm, int wr, MidSchedule& s) {
  const int P = d1 * d2;
  const int64_t n1 = (int64_t)wl * d1 * wm * d1, n2 = (int64_t)wm * d2 * wr * d2;
  std::vector<C2> O((size_t)wl * wr * P * P, C2{0, 0});
  for (int w = 0; w < wl; w++)
    for (int w2 = 0; w2 < wr; w2++)
      for (int m = 0; m < wm; m++)
        for (int a1 = 0; a1 < d1; a1++)        // s1'
          for (int b1 = 0; b1 < d1; b1++) {    // s1
            C2 x = wget(W1, cplx, n1, w + (int64_t)wl * (a1 + d1 * (m + (int64_t)wm * b1)));
            if (x.r == 0.0 && x.i == 0.0) continue;
            for (int a2 = 0; a2 < d2; a2++)    // s2'
              for (int b2 = 0; b2 < d2; b2++) {
                C2 y = wget(W2, cplx, n2, m + (int64_t)wm * (a2 + d2 * (w2 + (int64_t)wr * b2)));
                if (y.r == 0.0 && y.i == 0.0) continue;
                C2 p = cmul(x, y);
                int so = a1 + d1 * a2, si = b1 + d1 * b2;
                C2& o = O[(((size_t)w * wr + w2) * P + so) * P + si];
                o.r += p.r; o.i += p.i;
              }
          }
  build_schedule(cplx, wl, wr, P, P, O, s);
}

int schedule_ac(fmpt_handle* h, int cplx, const double* W, int d, int wl, int wr,
                MidSchedule& s) {
  return schedule_env(h, cplx, W, d, wl, wr, false, s);
}

int schedule_env(fmpt_handle* h, int cplx, const double* W, int d, int wl, int wr, bool right,
                 MidSchedule& s) {
  std::vector<C2> O((size_t)wl * wr * d * d, C2{0, 0});
  const int64_t nW = (int64_t)wl * d * wr * d;
  const int nw_in = right ? wr : wl, nw_out = right ? wl : wr;
  for (int w = 0; w < wl; w++)
    for (int w2 = 0; w2 < wr; w2++)
      for (int so = 0; so < d; so++)
        for (int si = 0; si < d; si++) {
          C2 v;
          if (W)
            v = wget(W, cplx, nW, w + (int64_t)wl * (so + d * (w2 + (int64_t)wr * si)));
          else
            v = C2{(w == w2 && so == si) ? 1.0 : 0.0, 0.0};
          int wi = right ? w2 : w, wo = right ? w : w2;
          O[(((size_t)wi * nw_out + wo) * d + so) * d + si] = v;
        }
  build_schedule(cplx, nw_in, nw_out, d, d, O, s);
  return mid_upload(h, s);
}

int mid_upload(fmpt_handle* h, MidSchedule& s) {
  mid_free(h, s);
  size_t nb = s.blk_win.size();
  size_t bytes_w = std::max<size_t>(nb, 1) * sizeof(int);
  size_t bytes_s = s.wout_start.size() * sizeof(int);
  size_t bytes_c = std::max<size_t>(s.coef.size(), 1) * sizeof(double);
  FMPT_CUDA(h, cudaMallocAsync((void**)&s.d_win, bytes_w, h->stream));
  FMPT_CUDA(h, cudaMallocAsync((void**)&s.d_wstart, bytes_s, h->stream));
  FMPT_CUDA(h, cudaMallocAsync((void**)&s.d_coef, bytes_c, h->stream));
  if (nb) FMPT_CUDA(h, cudaMemcpyAsync(s.d_win, s.blk_win.data(), nb * sizeof(int),
                                       cudaMemcpyHostToDevice, h->stream));
  FMPT_CUDA(h, cudaMemcpyAsync(s.d_wstart, s.wout_start.data(), bytes_s,
                               cudaMemcpyHostToDevice, h->stream));
  if (!s.coef.empty())
    FMPT_CUDA(h, cudaMemcpyAsync(s.d_coef, s.coef.data(), s.coef.size() * sizeof(double),
                                 cudaMemcpyHostToDevice, h->stream));
  // the host vectors must outlive the async copies: make the copies complete
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  return FMPT_OK;
}

void mid_free(fmpt_handle* h, MidSchedule& s) {
  if (s.d_win) cudaFreeAsync(s.d_win, h->stream);
  if (s.d_wstart) cudaFreeAsync(s.d_wstart, h->stream);
  if (s.d_coef) cudaFreeAsync(s.d_coef, h->stream);
  s.d_win = nullptr; s.d_wstart = nullptr; s.d_coef = nullptr;
}

int mid_apply(fmpt_handle* h, const MidSchedule& s, const double* in, int64_t plane_in,
              MidStrides si, double* out, int64_t plane_out, MidStrides so, int n1, int n2) {
  int64_t nt = (int64_t)n1 * n2;
  if (nt == 0) return FMPT_OK;
  const int threads = 256;
  int64_t blocks = (nt + threads - 1) / threads;
  if (blocks > 2147483647LL) return set_error(h, FMPT_ERR_SHAPE, "mid: too many threads");
  int P = std::max(s.p_in, s.p_out);
  if (P > 16) return set_error(h, FMPT_ERR_UNSUPPORTED, "physical dimension product %d > 16", P);
  ProfScope prof(h, FMPT_K_MPO_STEP);
  if (!s.sp_start.empty()) {
    MidSparse ms;
    ms.n_out = (int)s.sp_start.size() - 1;
    for (size_t i = 0; i < s.sp_start.size(); i++) ms.start[i] = (short)s.sp_start[i];
    for (size_t i = 0; i < s.sp_idx.size(); i++) ms.idx[i] = (short)s.sp_idx[i];
    for (size_t i = 0; i < s.sp_coef.size(); i++) ms.c[i] = s.sp_coef[i];
    if (s.cplx)
      mid_sparse_kernel<true><<<(unsigned)blocks, threads, 0, h->stream>>>(
          in, plane_in, si, out, plane_out, so, n1, n2, s.p_out, ms);
    else
      mid_sparse_kernel<false><<<(unsigned)blocks, threads, 0, h->stream>>>(
          in, plane_in, si, out, plane_out, so, n1, n2, s.p_out, ms);
    FMPT_LAUNCHED(h);
    return FMPT_OK;
  }
#define MIDL(MP, CP)                                                                          \
  mid_kernel<MP, CP><<<(unsigned)blocks, threads, 0, h->stream>>>(                            \
      in, plane_in, si, out, plane_out, so, n1, n2, s.nw_out, s.p_in, s.p_out, s.d_win,       \
      s.d_wstart, s.d_coef)
  if (P <= 2) { if (s.cplx) MIDL(2, true); else MIDL(2, false); }
  else if (P <= 4) { if (s.cplx) MIDL(4, true); else MIDL(4, false); }
  else { if (s.cplx) MIDL(16, true); else MIDL(16, false); }
#undef MIDL
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

// ---------------------------------------------------------------- ops
static GemmArgs gemm_args(int cplx, int ta, int tb, int m, int n, int k, const double* A,
                          int64_t lda, int64_t planeA, const double* B, int64_t ldb,
                          int64_t planeB, double* C, int64_t ldc, int64_t planeC) {
  GemmArgs g{};
  g.cplx = cplx; g.ta = ta; g.tb = tb; g.m = m; g.n = n; g.k = k;
  g.alpha[0] = 1.0; g.alpha[1] = 0.0; g.beta[0] = 0.0; g.beta[1] = 0.0;
  g.A = A; g.lda = lda; g.planeA = planeA;
  g.B = B; g.ldb = ldb; g.planeB = planeB;
  g.C = C; g.ldc = ldc; g.planeC = planeC;
  g.batch = 1; g.strideA = g.strideB = g.strideC = 0;
  return g;
}

int op_apply_fp64(fmpt_op* op, const double* x, double* y) {
  fmpt_handle* h = op->h;
  // FP64_TC: the GEMMs go to the tensor-core FP64 engine wherever it is faster; the digit
  // planes of the environments (A of the first GEMM, B of the second) are kept in the
  // operator, since they do not change while it lives
  const int eng = op->precision == FMPT_PREC_FP64_TC ? 1 : 0;
  auto gemm_f64 = [&](fmpt_handle* hh, GemmArgs g) {
    g.engine = eng;
    if (eng && g.A == op->hleft) g.cacheA = &op->oz_left;
    if (eng && g.B == op->hright) g.cacheB = &op->oz_right;
    return fmpt::gemm_f64(hh, g);
  };
  const int cp = op->dtype == FMPT_C128;
  const int Dl = op->Dl, Dr = op->Dr;
  const size_t es = sizeof(double) * (cp ? 2 : 1);
  if (op->kind == 2) {  // c_prime: y = sum_w L_w C R_w^T
    const int w = op->wl;
    int64_t nT = (int64_t)Dl * w * Dr;
    FMPT_TRY(grow_buffer(h, reinterpret_cast<void**>(&op->scratch), &op->scratch_bytes,
                         (size_t)nT * es));
    double* Td = op->scratch;
    FMPT_TRY(gemm_f64(h, gemm_args(cp, FMPT_N, FMPT_N, Dl * w, Dr, Dl, op->hleft, (int64_t)Dl * w,
                                   (int64_t)Dl * w * Dl, x, Dl, (int64_t)Dl * Dr, Td,
                                   (int64_t)Dl * w, nT)));
    FMPT_TRY(gemm_f64(h, gemm_args(cp, FMPT_N, FMPT_T, Dl, Dr, w * Dr, Td, Dl, nT,
                                   op->hright, Dr, (int64_t)Dr * w * Dr, y, Dl,
                                   (int64_t)Dl * Dr)));
    return FMPT_OK;
  }
  FMPT_TRY(op_fp64_head(op, x));
  return op_fp64_tail(op, y);
}

// One- and two-site FP64 application in two halves, so that a caller can overlap the
// upload of the right environment with the first half: head = GEMM 1 and the MPO step
// (reads x and the left environment, writes T1 and T3 in the operator's scratch), tail =
// GEMM 2 (reads T3 and the right environment, writes y).
int op_fp64_head(fmpt_op* op, const double* x) {
  fmpt_handle* h = op->h;
  const int eng = op->precision == FMPT_PREC_FP64_TC ? 1 : 0;
  const int cp = op->dtype == FMPT_C128;
  const int Dl = op->Dl, Dr = op->Dr;
  const size_t es = sizeof(double) * (cp ? 2 : 1);
  const int P = op->kind == 0 ? op->d1 * op->d2 : op->d1;
  const int wl = op->wl, wr = op->wr;
  const int64_t nx = (int64_t)Dl * P * Dr;
  const int64_t n1 = (int64_t)Dl * wl * P * Dr, n3 = (int64_t)Dl * P * wr * Dr;
  // T1 and T3 in the operator's scratch (one buffer, T3 after T1)
  FMPT_TRY(grow_buffer(h, reinterpret_cast<void**>(&op->scratch), &op->scratch_bytes,
                       (size_t)(n1 + n3) * es));
  double* T1 = op->scratch;
  double* T3 = op->scratch + n1 * (cp ? 2 : 1);
  // 1. T1[(a' w), (s b)] = L[(a' w), a] x[a, (s b)]
  GemmArgs g1 = gemm_args(cp, FMPT_N, FMPT_N, Dl * wl, P * Dr, Dl, op->hleft, (int64_t)Dl * wl,
                          (int64_t)Dl * wl * Dl, x, Dl, nx, T1, (int64_t)Dl * wl, n1);
  g1.engine = eng;
  if (eng) g1.cacheA = &op->oz_left;
  FMPT_TRY(gemm_f64(h, g1));
  // 2. T3[a', s', w2, b] = sum_blocks O[s', s] T1[a', w, s, b]
  MidStrides si{1, (int64_t)Dl * wl * P, Dl, (int64_t)Dl * wl};
  MidStrides so{1, (int64_t)Dl * P * wr, (int64_t)Dl * P, Dl};
  return mid_apply(h, op->sched, T1, n1, si, T3, n3, so, Dl, Dr);
}

int op_fp64_tail(fmpt_op* op, double* y) {
  fmpt_handle* h = op->h;
  const int eng = op->precision == FMPT_PREC_FP64_TC ? 1 : 0;
  const int cp = op->dtype == FMPT_C128;
  const int Dl = op->Dl, Dr = op->Dr;
  const int P = op->kind == 0 ? op->d1 * op->d2 : op->d1;
  const int wl = op->wl, wr = op->wr;
  const int64_t nx = (int64_t)Dl * P * Dr;
  const int64_t n1 = (int64_t)Dl * wl * P * Dr, n3 = (int64_t)Dl * P * wr * Dr;
  const double* T3 = op->scratch + n1 * (cp ? 2 : 1);
  // 3. y[(a' s'), b'] = T3[(a' s'), (w2 b)] R[b', (w2 b)]^T
  GemmArgs g2 = gemm_args(cp, FMPT_N, FMPT_T, Dl * P, Dr, wr * Dr, T3, (int64_t)Dl * P, n3,
                          op->hright, Dr, (int64_t)Dr * wr * Dr, y, (int64_t)Dl * P, nx);
  g2.engine = eng;
  if (eng) g2.cacheB = &op->oz_right;
  return gemm_f64(h, g2);
}

}  // namespace fmpt

using namespace fmpt;

static int check_dtype_prec(fmpt_handle* h, int dtype, int precision) {
  if (!h) return FMPT_ERR_ARG;
  if (dtype != FMPT_F64 && dtype != FMPT_C128)
    return set_error(h, FMPT_ERR_ARG, "unknown dtype %d", dtype);
  if (precision < FMPT_PREC_FP64 || precision > FMPT_PREC_FP64_TC)
    return set_error(h, FMPT_ERR_ARG, "unknown precision %d", precision);
  return FMPT_OK;
}

static int make_op(fmpt_handle* h, int kind, int dtype, int precision, const double* W1,
                   const double* W2, const double* hleft, const double* hright, int Dl, int d1,
                   int d2, int Dr, int wl, int wm, int wr, fmpt_op** out,
                   bool defer_right = false) {
  FMPT_TRY(check_dtype_prec(h, dtype, precision));
  if (!out || !hleft || !hright) return set_error(h, FMPT_ERR_ARG, "null pointer");
  if (Dl < 1 || Dr < 1 || d1 < 1 || d2 < 1 || wl < 1 || wm < 1 || wr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "non-positive dimension");
  fmpt_op* op = new fmpt_op();
  op->h = h; op->kind = kind; op->dtype = dtype; op->precision = precision;
  op->Dl = Dl; op->Dr = Dr; op->d1 = d1; op->d2 = d2; op->wl = wl; op->wm = wm; op->wr = wr;
  op->hleft = hleft; op->hright = hright;
  op->defer_right = defer_right && !prec_is_f64(precision) && dtype == FMPT_F64 && kind == 0;
  const int cp = dtype == FMPT_C128;
  int st = FMPT_OK;
  if (kind == 0) {
    op->n = (int64_t)Dl * d1 * d2 * Dr;
    st = schedule_ac2(h, cp, W1, W2, d1, d2, wl, wm, wr, op->sched);
  } else if (kind == 1) {
    op->n = (int64_t)Dl * d1 * Dr;
    st = W1 ? schedule_ac(h, cp, W1, d1, wl, wr, op->sched)
            : set_error(h, FMPT_ERR_ARG, "ac: null MPO tensor");
  } else {
    op->n = (int64_t)Dl * Dr;
  }
  if (st == FMPT_OK && !prec_is_f64(precision)) st = op_tc_prepare(op);
  if (st != FMPT_OK) {
    fmpt_op_destroy(op);
    return st;
  }
  *out = op;
  return FMPT_OK;
}

extern "C" {

int fmpt_op_ac2(fmpt_handle* h, int dtype, int precision, const double* W1, const double* W2,
                const double* hleft, const double* hright, int Dl, int d1, int d2, int Dr,
                int wl, int wm, int wr, fmpt_op** out) {
  return make_op(h, 0, dtype, precision, W1, W2, hleft, hright, Dl, d1, d2, Dr, wl, wm, wr, out);
}

int fmpt_op_ac(fmpt_handle* h, int dtype, int precision, const double* W, const double* hleft,
               const double* hright, int Dl, int d, int Dr, int wl, int wr, fmpt_op** out) {
  return make_op(h, 1, dtype, precision, W, nullptr, hleft, hright, Dl, d, 1, Dr, wl, 1, wr, out);
}

int fmpt_op_c(fmpt_handle* h, int dtype, int precision, const double* hleft,
              const double* hright, int Dl, int Dr, int w, fmpt_op** out) {
  return make_op(h, 2, dtype, precision, nullptr, nullptr, hleft, hright, Dl, 1, 1, Dr, w, 1, w,
                 out);
}

int fmpt_op_apply(fmpt_op* op, const double* x, double* y) {
  if (!op) return FMPT_ERR_ARG;
  if (!x || !y) return set_error(op->h, FMPT_ERR_ARG, "op_apply: null vector");
  if (op->u1) {
    FMPT_TRY(op_u1_apply(op, x, y));
  } else if (!prec_is_f64(op->precision)) {
    FMPT_TRY(op_tc_apply(op, x, y));
  } else {
    FMPT_TRY(op_apply_fp64(op, x, y));
  }
  return op_project(op, y);
}

int64_t fmpt_op_size(fmpt_op* op) { return op ? op->n : -1; }

int fmpt_op_destroy(fmpt_op* op) {
  if (!op) return FMPT_OK;
  mid_free(op->h, op->sched);
  oz_cache_free(op->h, op->oz_left);
  oz_cache_free(op->h, op->oz_right);
  op_tc_free(op);
  op_u1_free(op);
  if (op->proj_part) cudaFreeAsync(op->proj_part, op->h->stream);
  if (op->scratch) cudaFreeAsync(op->scratch, op->h->stream);
  delete op;
  return FMPT_OK;
}

int fmpt_ac2_prime(fmpt_handle* h, int dtype, int precision, const double* x, const double* W1,
                   const double* W2, const double* hleft, const double* hright, double* y,
                   int Dl, int d1, int d2, int Dr, int wl, int wm, int wr) {
  fmpt_op* op = nullptr;
  FMPT_TRY(fmpt_op_ac2(h, dtype, precision, W1, W2, hleft, hright, Dl, d1, d2, Dr, wl, wm, wr,
                       &op));
  int st = fmpt_op_apply(op, x, y);
  fmpt_op_destroy(op);
  return st;
}

int fmpt_ac2_prime_host(fmpt_handle* h, int dtype, int precision, const double* x,
                        const double* W1, const double* W2, const double* hleft,
                        const double* hright, double* y, int Dl, int d1, int d2, int Dr, int wl,
                        int wm, int wr) {
  FMPT_TRY(check_dtype_prec(h, dtype, precision));
  if (!x || !W1 || !W2 || !hleft || !hright || !y)
    return set_error(h, FMPT_ERR_ARG, "ac2_prime_host: null pointer");
  if (Dl < 1 || Dr < 1 || d1 < 1 || d2 < 1 || wl < 1 || wm < 1 || wr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "non-positive dimension");
  const size_t es = sizeof(double) * (dtype == FMPT_C128 ? 2 : 1);
  const size_t bx = (size_t)Dl * d1 * d2 * Dr * es, bL = (size_t)Dl * wl * Dl * es,
               bR = (size_t)Dr * wr * Dr * es;
  DevBuf dx, dL, dR, dy;
  FMPT_TRY(dx.alloc(h, bx));
  FMPT_TRY(dL.alloc(h, bL));
  FMPT_TRY(dR.alloc(h, bR));
  FMPT_TRY(dy.alloc(h, bx));
  cudaStream_t ms = h->stream;
  if (prec_is_f64(precision)) {
    // FP64 forms: the uploads run on a copy stream in the order L, x, R; the main stream
    // starts GEMM 1 and the MPO step once L and x have arrived, so R's upload overlaps them,
    // and GEMM 2 once R has
    FMPT_TRY(aux_fork(h, 1));       // the copies follow the allocations above
    cudaStream_t as = h->aux_stream[0];
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    int st = FMPT_OK;
    auto ok = [&](cudaError_t e) {
      if (e != cudaSuccess && st == FMPT_OK)
        st = set_error(h, FMPT_ERR_CUDA, "ac2_prime_host: %s", cudaGetErrorString(e));
      return st == FMPT_OK;
    };
    for (int i = 0; i < 3 && st == FMPT_OK; i++)
      ok(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    if (st == FMPT_OK) {
      ok(cudaMemcpyAsync(dL.p, hleft, bL, cudaMemcpyHostToDevice, as)) && ok(cudaEventRecord(ev[0], as));
      ok(cudaMemcpyAsync(dx.p, x, bx, cudaMemcpyHostToDevice, as)) && ok(cudaEventRecord(ev[1], as));
      ok(cudaMemcpyAsync(dR.p, hright, bR, cudaMemcpyHostToDevice, as)) && ok(cudaEventRecord(ev[2], as));
    }
    fmpt_op* op = nullptr;
    if (st == FMPT_OK)
      st = make_op(h, 0, dtype, precision, W1, W2, dL.d(), dR.d(), Dl, d1, d2, Dr, wl, wm, wr,
                   &op);
    if (st == FMPT_OK && ok(cudaStreamWaitEvent(ms, ev[0], 0)) &&
        ok(cudaStreamWaitEvent(ms, ev[1], 0)))
      st = op_fp64_head(op, dx.d());
    if (st == FMPT_OK && ok(cudaStreamWaitEvent(ms, ev[2], 0))) st = op_fp64_tail(op, dy.d());
    if (st == FMPT_OK) ok(cudaMemcpyAsync(y, dy.p, bx, cudaMemcpyDeviceToHost, ms));
    // every queued copy and kernel ends before the buffers are released
    ok(cudaStreamSynchronize(as));
    ok(cudaStreamSynchronize(ms));
    if (op) fmpt_op_destroy(op);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    return st;
  }
  const bool pipeline = dtype == FMPT_F64;
  if (!pipeline) {
    FMPT_CUDA(h, cudaMemcpyAsync(dx.p, x, bx, cudaMemcpyHostToDevice, ms));
    FMPT_CUDA(h, cudaMemcpyAsync(dL.p, hleft, bL, cudaMemcpyHostToDevice, ms));
    FMPT_CUDA(h, cudaMemcpyAsync(dR.p, hright, bR, cudaMemcpyHostToDevice, ms));
    FMPT_TRY(fmpt_ac2_prime(h, dtype, precision, dx.d(), W1, W2, dL.d(), dR.d(), dy.d(), Dl, d1,
                            d2, Dr, wl, wm, wr));
    FMPT_CUDA(h, cudaMemcpyAsync(y, dy.p, bx, cudaMemcpyDeviceToHost, ms));
    FMPT_CUDA(h, cudaStreamSynchronize(ms));
    return FMPT_OK;
  }
  // Uploads on one copy stream in the order L, x, R (R in column blocks of b'), downloads
  // of y on a second one.  The main stream starts on each operand as soon as it has
  // arrived: the L conversion overlaps the x copy; the x conversion, GEMM 1 and the MPO
  // step overlap the R copy; block c of R is converted and multiplied (GEMM 2 for the
  // columns b' of block c) while block c+1 is uploaded, and y's block c is downloaded
  // meanwhile.  A block of R[b', w2, b] (b' fastest) is a pitched 2-D copy.
  // more blocks shorten the tail after the last upload (one block's GEMM 2 and y download)
  const int nblk = Dr >= 2048 ? 8 : Dr >= 1024 ? 4 : (Dr >= 256 ? 2 : 1);
  FMPT_TRY(aux_fork(h, 2));        // the copies follow the allocations above
  cudaStream_t as = h->aux_stream[0], ds = h->aux_stream[1];
  std::vector<cudaEvent_t> ev(2 + 2 * nblk, nullptr);   // L, x, R blocks, y blocks
  int st = FMPT_OK;
  for (size_t i = 0; i < ev.size() && st == FMPT_OK; i++)
    if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess)
      st = set_error(h, FMPT_ERR_CUDA, "ac2_prime_host: event creation failed");
  auto rows = [&](int c) { return std::make_pair((int)((int64_t)Dr * c / nblk),
                                                 (int)((int64_t)Dr * (c + 1) / nblk)); };
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && st == FMPT_OK)
      st = set_error(h, FMPT_ERR_CUDA, "ac2_prime_host: %s", cudaGetErrorString(e));
    return st == FMPT_OK;
  };
  if (st == FMPT_OK) {
    ok(cudaMemcpyAsync(dL.p, hleft, bL, cudaMemcpyHostToDevice, as)) && ok(cudaEventRecord(ev[0], as));
    ok(cudaMemcpyAsync(dx.p, x, bx, cudaMemcpyHostToDevice, as)) && ok(cudaEventRecord(ev[1], as));
    for (int c = 0; c < nblk && st == FMPT_OK; c++) {
      const auto r = rows(c);
      ok(cudaMemcpy2DAsync(dR.d() + r.first, (size_t)Dr * sizeof(double), hright + r.first,
                           (size_t)Dr * sizeof(double), (size_t)(r.second - r.first) * sizeof(double),
                           (size_t)wr * Dr, cudaMemcpyHostToDevice, as)) &&
          ok(cudaEventRecord(ev[2 + c], as));
    }
  }
  fmpt_op* op = nullptr;
  if (st == FMPT_OK && ok(cudaStreamWaitEvent(ms, ev[0], 0)))
    st = make_op(h, 0, dtype, precision, W1, W2, dL.d(), dR.d(), Dl, d1, d2, Dr, wl, wm, wr, &op,
                 true);
  if (st == FMPT_OK && !op->defer_right)
    st = set_error(h, FMPT_ERR_ARG, "ac2_prime_host: operator without a deferred right side");
  if (st == FMPT_OK && ok(cudaStreamWaitEvent(ms, ev[1], 0))) st = op_tc_apply_head(op, dx.d());
  const size_t col = (size_t)Dl * d1 * d2 * sizeof(double);    // bytes of one column b' of y
  for (int c = 0; c < nblk && st == FMPT_OK; c++) {
    const auto r = rows(c);
    if (!ok(cudaStreamWaitEvent(ms, ev[2 + c], 0))) break;
    st = op_tc_prepare_right_rows(op, r.first, r.second);
    if (st == FMPT_OK) st = op_tc_apply_tail_rows(op, dy.d(), r.first, r.second);
    if (st == FMPT_OK && ok(cudaEventRecord(ev[2 + nblk + c], ms)) &&
        ok(cudaStreamWaitEvent(ds, ev[2 + nblk + c], 0)))
      ok(cudaMemcpyAsync(reinterpret_cast<char*>(y) + col * r.first,
                         reinterpret_cast<char*>(dy.p) + col * r.first,
                         col * (r.second - r.first), cudaMemcpyDeviceToHost, ds));
  }
  // every queued copy and kernel ends before the buffers are released
  ok(cudaStreamSynchronize(as));
  ok(cudaStreamSynchronize(ms));
  ok(cudaStreamSynchronize(ds));
  if (op) {
    if (st == FMPT_OK) st = op_tc_check(op);
    fmpt_op_destroy(op);
  }
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  return st;
}

int fmpt_ac_prime(fmpt_handle* h, int dtype, int precision, const double* x, const double* W,
                  const double* hleft, const double* hright, double* y, int Dl, int d, int Dr,
                  int wl, int wr) {
  fmpt_op* op = nullptr;
  FMPT_TRY(fmpt_op_ac(h, dtype, precision, W, hleft, hright, Dl, d, Dr, wl, wr, &op));
  int st = fmpt_op_apply(op, x, y);
  fmpt_op_destroy(op);
  return st;
}

int fmpt_c_prime(fmpt_handle* h, int dtype, int precision, const double* C, const double* hleft,
                 const double* hright, double* y, int Dl, int Dr, int w) {
  fmpt_op* op = nullptr;
  FMPT_TRY(fmpt_op_c(h, dtype, precision, hleft, hright, Dl, Dr, w, &op));
  int st = fmpt_op_apply(op, C, y);
  fmpt_op_destroy(op);
  return st;
}

int fmpt_updateleft(fmpt_handle* h, int dtype, int precision, const double* hold,
                    const double* A, const double* W, const double* B, double* hnew, int Dl,
                    int d, int Dr, int wl, int wr) {
  FMPT_TRY(check_dtype_prec(h, dtype, precision));
  if (!hold || !A || !B || !hnew) return set_error(h, FMPT_ERR_ARG, "updateleft: null pointer");
  if (Dl < 1 || d < 1 || Dr < 1 || wl < 1 || wr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "updateleft: non-positive dimension");
  if (!W && wl != wr) return set_error(h, FMPT_ERR_SHAPE, "overlap update needs wl == wr");
  const int cp = dtype == FMPT_C128;
  if (!prec_is_f64(precision)) {
    if (cp) return set_error(h, FMPT_ERR_UNSUPPORTED, "mixed precision: complex environments");
    return env_update_tc(h, false, precision, hold, A, W, B, hnew, Dl, d, Dr, wl, wr);
  }
  const int eng = precision == FMPT_PREC_FP64_TC ? 1 : 0;
  auto gemm_f64 = [&](fmpt_handle* hh, GemmArgs g) {
    g.engine = eng;
    return fmpt::gemm_f64(hh, g);
  };
  MidSchedule s;
  FMPT_TRY(schedule_env(h, cp, W, d, wl, wr, false, s));
  const int64_t nT = (int64_t)Dl * wl * d * Dr, nU = (int64_t)Dl * d * wr * Dr;
  DevBuf T, U;
  int st = T.alloc(h, nT * sizeof(double) * (cp ? 2 : 1));
  if (st == FMPT_OK) st = U.alloc(h, nU * sizeof(double) * (cp ? 2 : 1));
  if (st == FMPT_OK)  // T[(a' w), (s b)] = hold[(a' w), a] B[a, (s b)]
    st = gemm_f64(h, gemm_args(cp, FMPT_N, FMPT_N, Dl * wl, d * Dr, Dl, hold, (int64_t)Dl * wl,
                               (int64_t)Dl * wl * Dl, B, Dl, (int64_t)Dl * d * Dr, T.d(),
                               (int64_t)Dl * wl, nT));
  if (st == FMPT_OK) {
    MidStrides si{1, (int64_t)Dl * wl * d, Dl, (int64_t)Dl * wl};
    MidStrides so{1, (int64_t)Dl * d * wr, (int64_t)Dl * d, Dl};
    st = mid_apply(h, s, T.d(), nT, si, U.d(), nU, so, Dl, Dr);
  }
  if (st == FMPT_OK)  // hnew[b', (w2 b)] = A[(a' s'), b']^H U[(a' s'), (w2 b)]
    st = gemm_f64(h, gemm_args(cp, FMPT_C, FMPT_N, Dr, wr * Dr, Dl * d, A, (int64_t)Dl * d,
                               (int64_t)Dl * d * Dr, U.d(), (int64_t)Dl * d, nU, hnew, Dr,
                               (int64_t)Dr * wr * Dr));
  mid_free(h, s);
  return st;
}

int fmpt_updateright(fmpt_handle* h, int dtype, int precision, const double* hold,
                     const double* A, const double* W, const double* B, double* hnew, int Dl,
                     int d, int Dr, int wl, int wr) {
  FMPT_TRY(check_dtype_prec(h, dtype, precision));
  if (!hold || !A || !B || !hnew) return set_error(h, FMPT_ERR_ARG, "updateright: null pointer");
  if (Dl < 1 || d < 1 || Dr < 1 || wl < 1 || wr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "updateright: non-positive dimension");
  if (!W && wl != wr) return set_error(h, FMPT_ERR_SHAPE, "overlap update needs wl == wr");
  const int cp = dtype == FMPT_C128;
  if (!prec_is_f64(precision)) {
    if (cp) return set_error(h, FMPT_ERR_UNSUPPORTED, "mixed precision: complex environments");
    return env_update_tc(h, true, precision, hold, A, W, B, hnew, Dl, d, Dr, wl, wr);
  }
  const int eng = precision == FMPT_PREC_FP64_TC ? 1 : 0;
  auto gemm_f64 = [&](fmpt_handle* hh, GemmArgs g) {
    g.engine = eng;
    return fmpt::gemm_f64(hh, g);
  };
  MidSchedule s;
  FMPT_TRY(schedule_env(h, cp, W, d, wl, wr, true, s));
  const int64_t nT = (int64_t)Dl * d * Dr * wr, nU = (int64_t)wl * Dl * d * Dr;
  DevBuf T, U;
  int st = T.alloc(h, nT * sizeof(double) * (cp ? 2 : 1));
  if (st == FMPT_OK) st = U.alloc(h, nU * sizeof(double) * (cp ? 2 : 1));
  if (st == FMPT_OK)  // T[(a s), (b' w2)] = B[(a s), b] hold[(b' w2), b]^T
    st = gemm_f64(h, gemm_args(cp, FMPT_N, FMPT_T, Dl * d, Dr * wr, Dr, B, (int64_t)Dl * d,
                               (int64_t)Dl * d * Dr, hold, (int64_t)Dr * wr,
                               (int64_t)Dr * wr * Dr, T.d(), (int64_t)Dl * d, nT));
  if (st == FMPT_OK) {
    MidStrides si{1, (int64_t)Dl * d, (int64_t)Dl * d * Dr, Dl};
    MidStrides so{wl, (int64_t)wl * Dl * d, 1, (int64_t)wl * Dl};
    st = mid_apply(h, s, T.d(), nT, si, U.d(), nU, so, Dl, Dr);
  }
  if (st == FMPT_OK)  // hnew[a', (w a)] = conj(A)[a', (s' b')] U2[(w a), (s' b')]^T
    st = gemm_f64(h, gemm_args(cp, FMPT_R, FMPT_T, Dl, wl * Dl, d * Dr, A, Dl,
                               (int64_t)Dl * d * Dr, U.d(), (int64_t)wl * Dl, nU, hnew, Dl,
                               (int64_t)Dl * wl * Dl));
  mid_free(h, s);
  return st;
}

}  // extern "C"
