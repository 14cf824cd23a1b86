// Mixed-precision H_eff*x (two-site, one-site, zero-site) on the tcgen05
// GEMM engine.
//
// Device layouts (K contiguous for both tensor-core operands, K padded to a
// multiple of 8 so every TMA row starts on a 16-byte boundary):
//   xg [a][(s, b)]            the state itself (x[a, s, b] is already K-major)
//   Lg [a][(a', w)]           Lg[a + Kp*(a' + Dl*w)]      = L[a', w, a]
//   Rg [(b, w2)][b']          Rg[(b + Drp*w2) + K2*b']    = R[b', w2, b]
//   T1 [(s, b)][(a', w)]      FP32 accumulator output of GEMM 1
//   T3 [(b, w2)][(a', s')]    MPO step output, operand of GEMM 2
//   y  [(a', s')][b']         FP64, the reference layout of y[a', s', b']
// GEMM 1:  T1 = xg^T . Lg          M = P*Dr, N = wl*Dl, K = Kp
// MPO step: T3[a', s', w2, b] = sum_blocks O[s', s] T1[a', w, s, b]
// GEMM 2:  y  = T3 . Rg^T          M = P*Dl, N = Dr,    K = K2 = wr*Drp
// Environments are converted once per operator (they are fixed during a
// Krylov solve); x is converted on every application.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "internal.h"

namespace fmpt {

namespace {

enum { M_TF32 = 0, M_TF32X3 = 1, M_BF16 = 2 };

int tc_mode_of(int precision) {
  return precision == FMPT_PREC_TF32 ? M_TF32 : precision == FMPT_PREC_TF32X3 ? M_TF32X3 : M_BF16;
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// write one converted value: TF32 (hi, optional lo) or BF16
template <int MODE>
__device__ __forceinline__ void put(void* hi, void* lo, int64_t i, double v) {
  if (MODE == M_BF16) {
    static_cast<__nv_bfloat16*>(hi)[i] = __float2bfloat16_rn((float)v);
  } else {
    const float h = tf32_rna((float)v);
    static_cast<float*>(hi)[i] = h;
    if (MODE == M_TF32X3) static_cast<float*>(lo)[i] = tf32_rna((float)(v - (double)h));
  }
}

// xg[a + dld*m] = x[a + Dl*m] for a < Kp (zero for a >= Dl); dld >= Kp is the row
// stride (2*Kp for the real embedding of complex data: real part, then imaginary part)
template <int MODE>
__global__ void conv_state(const double* __restrict__ x, int Dl, int Kp, int64_t M, void* hi,
                           void* lo, int64_t dld) {
  const int64_t tot = (int64_t)Kp * M;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(t % Kp);
    const int64_t m = t / Kp;
    put<MODE>(hi, lo, a + dld * m, a < Dl ? x[a + (int64_t)Dl * m] : 0.0);
  }
}

// conv_state for the identity layout (Dl == Kp == dld): four consecutive elements per
// thread, 32-byte loads and 8-byte (BF16) / 16-byte (TF32) stores; x 16-byte aligned and
// n4 = Kp*M/4 (Kp is a multiple of 8).  Same rounding per element as put().
template <int MODE>
__global__ void conv_state_vec(const double* __restrict__ x, int64_t n4, void* hi, void* lo) {
  const double2* x2 = reinterpret_cast<const double2*>(x);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double2 p = x2[2 * t], q = x2[2 * t + 1];
    if (MODE == M_BF16) {
      const __nv_bfloat162 u = __floats2bfloat162_rn((float)p.x, (float)p.y);
      const __nv_bfloat162 w = __floats2bfloat162_rn((float)q.x, (float)q.y);
      uint2 o;
      o.x = *reinterpret_cast<const uint32_t*>(&u);
      o.y = *reinterpret_cast<const uint32_t*>(&w);
      reinterpret_cast<uint2*>(hi)[t] = o;
    } else {
      const float4 hv = make_float4(tf32_rna((float)p.x), tf32_rna((float)p.y),
                                    tf32_rna((float)q.x), tf32_rna((float)q.y));
      reinterpret_cast<float4*>(hi)[t] = hv;
      if (MODE == M_TF32X3)
        reinterpret_cast<float4*>(lo)[t] =
            make_float4(tf32_rna((float)(p.x - (double)hv.x)), tf32_rna((float)(p.y - (double)hv.y)),
                        tf32_rna((float)(q.x - (double)hv.z)), tf32_rna((float)(q.y - (double)hv.w)));
    }
  }
}

// batched transpose with conversion:
//   dst[c + dld*r + dz*z] = scale * src[r + sld*c + sz*z]   for r < R, c < Cp (zero for c >= C)
template <int MODE>
__global__ void conv_transpose(const double* __restrict__ src, int64_t sld, int64_t sz, int R,
                               int C, int Cp, void* hi, void* lo, int64_t dld, int64_t dz,
                               double scale) {
  __shared__ double tile[32][33];
  const int z = blockIdx.z;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;      // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    const int r = r0 + tx, c = c0 + j;
    tile[j][tx] = (r < R && c < C) ? src[r + sld * c + sz * z] : 0.0;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int c = c0 + tx, r = r0 + j;
    if (r < R && c < Cp) put<MODE>(hi, lo, (int64_t)c + dld * r + dz * z, scale * tile[tx][j]);
  }
}

// MPO step on the FP32 GEMM-1 output, converted for GEMM 2.
//   in : T1[(s + P*b) + P*Dr*(a' + Dl*w)]
//   out: T3[(b + Drp*w2) + K2*(a' + Dl*s')]
template <int MODE, int MAXP>
__global__ void mid_tc(const float* __restrict__ T1, int P, int Dl, int Dr, int Drp, int64_t K2,
                       int nw_out, const int* __restrict__ win, const int* __restrict__ wstart,
                       const double* __restrict__ coef, void* hi, void* lo) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)Dl * Dr) return;
  const int b = (int)(t % Dr), ap = (int)(t / Dr);
  const int64_t in_w = (int64_t)P * Dr * Dl;
  const float* ib = T1 + (int64_t)P * b + (int64_t)P * Dr * ap;
  for (int wo = 0; wo < nw_out; wo++) {
    float acc[MAXP];
#pragma unroll
    for (int q = 0; q < MAXP; q++) acc[q] = 0.f;
    const int e1 = __ldg(wstart + wo + 1);
    for (int e = __ldg(wstart + wo); e < e1; e++) {
      const int wi = __ldg(win + e);
      const double* c = coef + (int64_t)e * P * P;
      float v[MAXP];
#pragma unroll
      for (int s = 0; s < MAXP; s++) v[s] = s < P ? ib[in_w * wi + s] : 0.f;
#pragma unroll
      for (int q = 0; q < MAXP; q++) {
        if (q >= P) break;
#pragma unroll
        for (int s = 0; s < MAXP; s++) {
          if (s >= P) break;
          acc[q] = fmaf((float)__ldg(c + q * P + s), v[s], acc[q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < MAXP; q++) {
      if (q >= P) break;
      put<MODE>(hi, lo, (int64_t)b + (int64_t)Drp * wo + K2 * (ap + (int64_t)Dl * q), (double)acc[q]);
    }
  }
}

// Fast path of the MPO step for two spin-1/2 sites (P = 4) and MPO bonds
// w <= 8: the nonzero (w, w') block pattern is a bitmask, every loop is
// unrolled with static indices (registers only), T1 is read once as float4
// and the block coefficients sit in shared memory.
__device__ __forceinline__ float4 load4(const float4* p) { return *p; }
__device__ __forceinline__ float4 load4(const uint2* p) {
  const uint2 u = *p;   // four BF16 values
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u),
                     __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xffff0000u));
}

// The block coefficients travel as a by-value kernel parameter (constant bank): every
// index below is a compile-time constant after unrolling, so each FFMA reads its
// coefficient as a constant-bank operand instead of issuing a shared-memory load (with
// ~13 nonzero blocks of 16 coefficients the loads, not DRAM, bounded the kernel).
struct MidCoef {
  float c[64][16];                                // [wi*8 + wo][q*4 + s]
};

template <int MODE, typename V4, int NW>
__global__ void __launch_bounds__(256) mid_tc_p4(const V4* __restrict__ T1, int Dl, int Dr,
                                                 int Drp, int64_t K2, int nw_in, int nw_out,
                                                 uint64_t mask, const __grid_constant__ MidCoef cp,
                                                 void* hi, void* lo) {
  const auto& c = cp.c;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)Dl * Dr) return;
  const int b = (int)(t % Dr), ap = (int)(t / Dr);
  const int64_t in_w = (int64_t)Dr * Dl;          // float4 stride between w planes
  const V4* ib = T1 + b + (int64_t)Dr * ap;
  // NW (4, 6 or 8) bounds both MPO bonds at compile time: only NW input planes are held
  // in registers (fewer registers per thread, more threads and loads in flight per SM)
  float4 v[NW];
#pragma unroll
  for (int wi = 0; wi < NW; wi++)
    v[wi] = wi < nw_in ? load4(ib + in_w * wi) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int wo = 0; wo < NW; wo++) {
    if (wo >= nw_out) break;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int wi = 0; wi < NW; wi++) {
      if (!((mask >> (wi * 8 + wo)) & 1ull)) continue;
      const float* cc = c[wi * 8 + wo];
      a0 = fmaf(cc[0], v[wi].x, fmaf(cc[1], v[wi].y, fmaf(cc[2], v[wi].z, fmaf(cc[3], v[wi].w, a0))));
      a1 = fmaf(cc[4], v[wi].x, fmaf(cc[5], v[wi].y, fmaf(cc[6], v[wi].z, fmaf(cc[7], v[wi].w, a1))));
      a2 = fmaf(cc[8], v[wi].x, fmaf(cc[9], v[wi].y, fmaf(cc[10], v[wi].z, fmaf(cc[11], v[wi].w, a2))));
      a3 = fmaf(cc[12], v[wi].x, fmaf(cc[13], v[wi].y, fmaf(cc[14], v[wi].z, fmaf(cc[15], v[wi].w, a3))));
    }
    const int64_t o = (int64_t)b + (int64_t)Drp * wo + K2 * ap;
    const int64_t qs = K2 * Dl;
    put<MODE>(hi, lo, o, (double)a0);
    put<MODE>(hi, lo, o + qs, (double)a1);
    put<MODE>(hi, lo, o + 2 * qs, (double)a2);
    put<MODE>(hi, lo, o + 3 * qs, (double)a3);
  }
}

// mid_tc_p4 for BF16 with two consecutive b per thread (Dr even): one 16-byte load per
// input plane and 4-byte bf16x2 stores, half the memory instructions of the one-b form.
// Each output element is rounded exactly as there.
__device__ __forceinline__ float4 bf16x4_lo(uint32_t x, uint32_t y) {
  return make_float4(__uint_as_float(x << 16), __uint_as_float(x & 0xffff0000u),
                     __uint_as_float(y << 16), __uint_as_float(y & 0xffff0000u));
}

template <int NW>
__global__ void __launch_bounds__(256) mid_bf16_x2(const uint4* __restrict__ T1, int Dl, int Dr,
                                                   int Drp, int64_t K2, int nw_in, int nw_out,
                                                   uint64_t mask,
                                                   const __grid_constant__ MidCoef cp,
                                                   __nv_bfloat16* __restrict__ out) {
  const auto& c = cp.c;
  const int hr = Dr >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)Dl * hr) return;
  const int bh = (int)(t % hr), ap = (int)(t / hr);
  const int b = 2 * bh;
  const int64_t in_w = (int64_t)hr * Dl;          // uint4 stride between w planes
  const uint4* ib = T1 + bh + (int64_t)hr * ap;
  float4 u[NW], v[NW];                             // planes of b and of b + 1
#pragma unroll
  for (int wi = 0; wi < NW; wi++) {
    if (wi < nw_in) {
      const uint4 q = ib[in_w * wi];
      u[wi] = bf16x4_lo(q.x, q.y);
      v[wi] = bf16x4_lo(q.z, q.w);
    } else {
      u[wi] = make_float4(0.f, 0.f, 0.f, 0.f);
      v[wi] = u[wi];
    }
  }
  const int64_t qs = K2 * Dl;
#pragma unroll
  for (int wo = 0; wo < NW; wo++) {
    if (wo >= nw_out) break;
    float a[4] = {0.f, 0.f, 0.f, 0.f}, e[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int wi = 0; wi < NW; wi++) {
      if (!((mask >> (wi * 8 + wo)) & 1ull)) continue;
      const float* cc = c[wi * 8 + wo];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        a[q] = fmaf(cc[4 * q], u[wi].x, fmaf(cc[4 * q + 1], u[wi].y,
               fmaf(cc[4 * q + 2], u[wi].z, fmaf(cc[4 * q + 3], u[wi].w, a[q]))));
        e[q] = fmaf(cc[4 * q], v[wi].x, fmaf(cc[4 * q + 1], v[wi].y,
               fmaf(cc[4 * q + 2], v[wi].z, fmaf(cc[4 * q + 3], v[wi].w, e[q]))));
      }
    }
    const int64_t o = (int64_t)b + (int64_t)Drp * wo + K2 * ap;   // even: b, Drp, K2 are
#pragma unroll
    for (int q = 0; q < 4; q++)
      *reinterpret_cast<__nv_bfloat162*>(out + o + q * qs) = __floats2bfloat162_rn(a[q], e[q]);
  }
}

// Strided MPO step for the environment updates (any layout, P = d <= 4,
// MPO bonds <= 8): out[o1,o2,wo,q] = sum_{(wi,wo) in mask} sum_s c[wi,wo][q,s] in[o1,o2,wi,s]
template <int MODE, int P>
__global__ void __launch_bounds__(256) mid_tc_mask(const float* __restrict__ T, int64_t i1,
                                                   int64_t i2, int64_t iw, int64_t is, int n1,
                                                   int n2, int nw_in, int nw_out, uint64_t mask,
                                                   const __grid_constant__ MidCoef cp, void* hi,
                                                   void* lo, int64_t o1s, int64_t o2s,
                                                   int64_t ows, int64_t oqs) {
  const auto& c = cp.c;                           // [wi*8 + wo][q*P + s], constant bank
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n1 * n2) return;
  const int o1 = (int)(t % n1), o2 = (int)(t / n1);
  const float* ib = T + o1 * i1 + o2 * i2;
  float v[8][P];
#pragma unroll
  for (int wi = 0; wi < 8; wi++)
#pragma unroll
    for (int q = 0; q < P; q++) v[wi][q] = wi < nw_in ? ib[wi * iw + q * is] : 0.f;
  const int64_t ob = o1 * o1s + o2 * o2s;
#pragma unroll
  for (int wo = 0; wo < 8; wo++) {
    if (wo >= nw_out) break;
    float acc[P];
#pragma unroll
    for (int q = 0; q < P; q++) acc[q] = 0.f;
#pragma unroll
    for (int wi = 0; wi < 8; wi++) {
      if (!((mask >> (wi * 8 + wo)) & 1ull)) continue;
#pragma unroll
      for (int q = 0; q < P; q++)
#pragma unroll
        for (int s2 = 0; s2 < P; s2++) acc[q] = fmaf(c[wi * 8 + wo][q * P + s2], v[wi][s2], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < P; q++) put<MODE>(hi, lo, ob + wo * ows + q * oqs, (double)acc[q]);
  }
}

struct TcState {
  int mode = 0, P = 1, es = 4;
  bool cplx = false;        // complex data: real embedding, every GEMM's K and N doubled
  MidSchedule rsched;       // real coefficients of a complex operator's MPO step
  int Kp = 0, Drp = 0;
  int64_t K2 = 0;
  DevBuf Lg[2], Rg[2], xg[2], T1, T3[2];
  int* err = nullptr;
  // fast MPO step (P = 4, w <= 8): block bitmask and dense float coefficients
  bool fast_mid = false;
  uint64_t mask = 0;
  MidCoef cpar;             // block coefficients, passed to mid_tc_p4 by value
};

inline int round_up8(int v) { return (v + 7) / 8 * 8; }

int grid1(fmpt_handle* h, int64_t n) {
  int64_t g = (n + 255) / 256, cap = (int64_t)h->sm_count * 16;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

template <int MODE>
int launch_transpose(fmpt_handle* h, const double* src, int64_t sld, int64_t sz, int R, int C,
                     int Cp, int Z, void* hi, void* lo, int64_t dld, int64_t dz, double scale) {
  dim3 grid((R + 31) / 32, (Cp + 31) / 32, Z);
  ProfScope prof(h, FMPT_K_CONVERT);
  conv_transpose<MODE><<<grid, dim3(32, 8), 0, h->stream>>>(src, sld, sz, R, C, Cp, hi, lo, dld, dz,
                                                           scale);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int transpose_any(fmpt_handle* h, int mode, const double* src, int64_t sld, int64_t sz, int R,
                  int C, int Cp, int Z, void* hi, void* lo, int64_t dld, int64_t dz,
                  double scale = 1.0) {
  if (mode == M_TF32)
    return launch_transpose<M_TF32>(h, src, sld, sz, R, C, Cp, Z, hi, lo, dld, dz, scale);
  if (mode == M_TF32X3)
    return launch_transpose<M_TF32X3>(h, src, sld, sz, R, C, Cp, Z, hi, lo, dld, dz, scale);
  return launch_transpose<M_BF16>(h, src, sld, sz, R, C, Cp, Z, hi, lo, dld, dz, scale);
}

inline void* offset(void* p, int64_t elems, int es) {
  return p ? static_cast<char*>(p) + elems * es : nullptr;
}

// Complex operand in the real embedding, K-major with row length 2*Kc:
//   rows [0, N):   [ Re | -Im ]      rows [N, 2N):  [ Im | Re ]
// from a split-plane complex source read by the same batched transpose as the real case
// (src plane offset `plane`); N rows; dz is the destination offset of batch z.
int embed_complex(fmpt_handle* h, int mode, const double* src, int64_t plane, int64_t sld,
                  int64_t sz, int R, int C, int Cp, int Z, int64_t dz, int64_t N, int Kc,
                  void* hi, void* lo, int es) {
  const int64_t dld = 2LL * Kc;
  const double* re = src;
  const double* im = src + plane;
  FMPT_TRY(transpose_any(h, mode, re, sld, sz, R, C, Cp, Z, hi, lo, dld, dz, 1.0));
  FMPT_TRY(transpose_any(h, mode, im, sld, sz, R, C, Cp, Z, offset(hi, Kc, es), offset(lo, Kc, es),
                         dld, dz, -1.0));
  FMPT_TRY(transpose_any(h, mode, im, sld, sz, R, C, Cp, Z, offset(hi, N * dld, es),
                         offset(lo, N * dld, es), dld, dz, 1.0));
  return transpose_any(h, mode, re, sld, sz, R, C, Cp, Z, offset(hi, N * dld + Kc, es),
                       offset(lo, N * dld + Kc, es), dld, dz, 1.0);
}

}  // namespace

int op_tc_prepare(fmpt_op* op) {
  fmpt_handle* h = op->h;
  TcState* st = new TcState();
  op->tc = st;
  st->mode = tc_mode_of(op->precision);
  st->es = st->mode == M_BF16 ? 2 : 4;
  st->cplx = op->dtype == FMPT_C128;
  if (st->cplx && op->kind != 2) {
    // the MPO step of the embedding acts on the real and imaginary planes alike: it needs
    // real coefficients (true for the spin and fermion MPOs of the utilities module)
    const MidSchedule& cs = op->sched;
    MidSchedule& rs = st->rsched;
    rs.nw_in = cs.nw_in; rs.nw_out = cs.nw_out; rs.p_in = cs.p_in; rs.p_out = cs.p_out;
    rs.cplx = 0;
    rs.blk_win = cs.blk_win;
    rs.wout_start = cs.wout_start;
    const size_t pp = (size_t)cs.p_in * cs.p_out;
    for (size_t e = 0; e < cs.blk_win.size(); e++) {
      for (size_t q = 0; q < pp; q++) {
        if (cs.coef[e * 2 * pp + pp + q] != 0.0)
          return set_error(h, FMPT_ERR_UNSUPPORTED,
                           "mixed precision, complex data: the MPO must be real");
        rs.coef.push_back(cs.coef[e * 2 * pp + q]);
      }
    }
    FMPT_TRY(mid_upload(h, rs));
  }
  const int Dl = op->Dl, Dr = op->Dr, wl = op->wl, wr = op->wr;
  if (op->kind == 2) {
    // c_prime: identity MPO step over w (wl == wr), one "physical" index
    st->P = 1;
    MidSchedule& s = op->sched;
    s.nw_in = wl; s.nw_out = wl; s.p_in = 1; s.p_out = 1; s.cplx = 0;
    s.blk_win.resize(wl); s.wout_start.resize(wl + 1); s.coef.assign(wl, 1.0);
    for (int w = 0; w < wl; w++) { s.blk_win[w] = w; s.wout_start[w] = w; }
    s.wout_start[wl] = wl;
    FMPT_TRY(mid_upload(h, s));
  } else {
    st->P = op->kind == 0 ? op->d1 * op->d2 : op->d1;
  }
  if (st->P > 16) return set_error(h, FMPT_ERR_UNSUPPORTED, "physical dimension product > 16");
  const int P = st->P;
  st->Kp = round_up8(Dl);
  st->Drp = round_up8(Dr);
  st->K2 = (int64_t)wr * st->Drp;
  const int split = st->mode == M_TF32X3 ? 2 : 1;
  const size_t es = st->es;
  const int cf = st->cplx ? 2 : 1;   // the real embedding doubles K and N of both GEMMs
  for (int p = 0; p < split; p++) {
    FMPT_TRY(st->Lg[p].alloc(h, (size_t)cf * st->Kp * Dl * wl * cf * es));
    FMPT_TRY(st->Rg[p].alloc(h, (size_t)cf * st->K2 * Dr * cf * es));
    FMPT_TRY(st->xg[p].alloc(h, (size_t)cf * st->Kp * P * Dr * es));
    FMPT_TRY(st->T3[p].alloc(h, (size_t)cf * st->K2 * P * Dl * es));
    FMPT_CUDA(h, cudaMemsetAsync(st->T3[p].p, 0, st->T3[p].bytes, h->stream));  // K padding
  }
  {
    const MidSchedule& ms = st->cplx && op->kind != 2 ? st->rsched : op->sched;
    if (P == 4 && ms.nw_in <= 8 && ms.nw_out <= 8) {
      std::vector<float> cf(64 * 16, 0.f);
      uint64_t mask = 0;
      for (int wo = 0; wo < ms.nw_out; wo++)
        for (int e = ms.wout_start[wo]; e < ms.wout_start[wo + 1]; e++) {
          const int wi = ms.blk_win[e];
          mask |= 1ull << (wi * 8 + wo);
          for (int q = 0; q < 16; q++) cf[(wi * 8 + wo) * 16 + q] += (float)ms.coef[(size_t)e * 16 + q];
        }
      std::memcpy(st->cpar.c, cf.data(), sizeof(st->cpar.c));
      st->mask = mask;
      st->fast_mid = true;
    }
  }
  // T1 is BF16 when the BF16 fast MPO step reads it (its values are rounded to BF16 for
  // GEMM 2 anyway), FP32 otherwise; the GEMM-1 output type in op_tc_apply matches this.
  const bool t1_bf16 = st->mode == M_BF16 && st->fast_mid && !st->cplx;
  FMPT_TRY(st->T1.alloc(h, (size_t)cf * P * Dr * wl * Dl * (t1_bf16 ? 2 : sizeof(float))));
  FMPT_CUDA(h, cudaMallocAsync((void**)&st->err, sizeof(int), h->stream));
  FMPT_CUDA(h, cudaMemsetAsync(st->err, 0, sizeof(int), h->stream));
  void* lo_L = split > 1 ? st->Lg[1].p : nullptr;
  void* lo_R = split > 1 ? st->Rg[1].p : nullptr;
  if (st->cplx) {
    // rows (a' + Dl*w) of [Re L | -Im L] then [Im L | Re L], K = a (twice)
    FMPT_TRY(embed_complex(h, st->mode, op->hleft, (int64_t)Dl * wl * Dl, (int64_t)Dl * wl, Dl,
                           Dl, Dl, st->Kp, wl, 2LL * st->Kp * Dl, (int64_t)Dl * wl, st->Kp,
                           st->Lg[0].p, lo_L, (int)es));
    // rows b' of [Re R | -Im R] then [Im R | Re R], K = (b + Drp*w2) (twice)
    FMPT_TRY(embed_complex(h, st->mode, op->hright, (int64_t)Dr * wr * Dr, (int64_t)Dr * wr, Dr,
                           Dr, Dr, st->Drp, wr, st->Drp, Dr, (int)st->K2, st->Rg[0].p, lo_R,
                           (int)es));
    return FMPT_OK;
  }
  // Lg[a + Kp*(a' + Dl*w)] = L[a' + Dl*w + Dl*wl*a]: per w, (r=a', c=a)
  FMPT_TRY(transpose_any(h, st->mode, op->hleft, (int64_t)Dl * wl, Dl, Dl, Dl, st->Kp, wl,
                         st->Lg[0].p, lo_L, st->Kp, (int64_t)st->Kp * Dl));
  if (op->defer_right) return FMPT_OK;
  return op_tc_prepare_right(op);
}

// Rg[b + Drp*w2 + K2*b'] = R[b' + Dr*w2 + Dr*wr*b]: per w2, (r=b', c=b).  Part of
// op_tc_prepare, run later for an operator created with defer_right (real data), once
// the right environment has arrived.
int op_tc_prepare_right(fmpt_op* op) { return op_tc_prepare_right_rows(op, 0, op->Dr); }

// Rows b' in [r0, r1) of the converted right environment (they need R[b', :, :] only).
int op_tc_prepare_right_rows(fmpt_op* op, int r0, int r1) {
  fmpt_handle* h = op->h;
  TcState* st = static_cast<TcState*>(op->tc);
  if (!st || st->cplx) return set_error(h, FMPT_ERR_ARG, "prepare_right: real tensor-core operator only");
  const int Dr = op->Dr, wr = op->wr;
  if (r0 < 0 || r1 > Dr || r0 >= r1) return set_error(h, FMPT_ERR_ARG, "prepare_right: bad row range");
  void* lo_R = st->mode == M_TF32X3 ? st->Rg[1].p : nullptr;
  const int64_t off = st->K2 * r0;
  return transpose_any(h, st->mode, op->hright + r0, (int64_t)Dr * wr, Dr, r1 - r0, Dr, st->Drp,
                       wr, offset(st->Rg[0].p, off, st->es), offset(lo_R, off, st->es), st->K2,
                       st->Drp);
}

int op_tc_apply_complex(fmpt_op* op, TcState* st, const double* x, double* y);

int op_tc_apply(fmpt_op* op, const double* x, double* y) {
  fmpt_handle* h = op->h;
  TcState* st = static_cast<TcState*>(op->tc);
  if (!st) return set_error(h, FMPT_ERR_ARG, "operator has no tensor-core state");
  if (st->cplx) return op_tc_apply_complex(op, st, x, y);
  FMPT_TRY(op_tc_apply_head(op, x));
  return op_tc_apply_tail(op, y);
}

// The part of a real two-site application that needs x and the left environment
// only: x conversion, GEMM 1 and the MPO step (T3 is left in the operator).
int op_tc_apply_head(fmpt_op* op, const double* x) {
  fmpt_handle* h = op->h;
  TcState* st = static_cast<TcState*>(op->tc);
  if (!st || st->cplx) return set_error(h, FMPT_ERR_ARG, "apply_head: real tensor-core operator only");
  const int Dl = op->Dl, Dr = op->Dr, wl = op->wl, P = st->P;
  const int split = st->mode == M_TF32X3 ? 2 : 1;
  void* xlo = split > 1 ? st->xg[1].p : nullptr;
  void* tlo = split > 1 ? st->T3[1].p : nullptr;
  const int64_t nx = (int64_t)st->Kp * P * Dr;
  {
  ProfScope prof(h, FMPT_K_CONVERT);
  const bool ident = st->Kp == Dl && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
  if (ident) {
    const int64_t n4 = nx / 4;
    if (st->mode == M_TF32)
      conv_state_vec<M_TF32><<<grid1(h, n4), 256, 0, h->stream>>>(x, n4, st->xg[0].p, xlo);
    else if (st->mode == M_TF32X3)
      conv_state_vec<M_TF32X3><<<grid1(h, n4), 256, 0, h->stream>>>(x, n4, st->xg[0].p, xlo);
    else
      conv_state_vec<M_BF16><<<grid1(h, n4), 256, 0, h->stream>>>(x, n4, st->xg[0].p, xlo);
  } else if (st->mode == M_TF32)
    conv_state<M_TF32><<<grid1(h, nx), 256, 0, h->stream>>>(x, Dl, st->Kp, (int64_t)P * Dr, st->xg[0].p, xlo, st->Kp);
  else if (st->mode == M_TF32X3)
    conv_state<M_TF32X3><<<grid1(h, nx), 256, 0, h->stream>>>(x, Dl, st->Kp, (int64_t)P * Dr, st->xg[0].p, xlo, st->Kp);
  else
    conv_state<M_BF16><<<grid1(h, nx), 256, 0, h->stream>>>(x, Dl, st->Kp, (int64_t)P * Dr, st->xg[0].p, xlo, st->Kp);
  FMPT_LAUNCHED(h);
  }
  // GEMM 1: T1[(s b), (a' w)] = sum_a xg[a, (s b)] Lg[a, (a' w)]
  TcOperand A1{st->xg[0].p, xlo, st->Kp, 0};
  TcOperand B1{st->Lg[0].p, split > 1 ? st->Lg[1].p : nullptr, st->Kp, 0};
  const bool t1_bf16 = st->mode == M_BF16 && st->fast_mid;
  FMPT_TRY(tc_gemm(h, st->mode, P * Dr, wl * Dl, st->Kp, 1, A1, B1, st->T1.p, t1_bf16 ? 2 : 0,
                   (int64_t)P * Dr, 0, st->err));
  // MPO step
  {
    const int64_t nt = (int64_t)Dl * Dr;
    const unsigned blocks = (unsigned)((nt + 255) / 256);
    const MidSchedule& s = op->sched;
    ProfScope prof(h, FMPT_K_MPO_STEP);
    if (st->fast_mid) {
      const float4* t1 = (const float4*)st->T1.p;
      const int nw = std::max(s.nw_in, s.nw_out);
#define MIDP4(NW_)                                                                                \
  do {                                                                                            \
    if (st->mode == M_TF32)                                                                       \
      mid_tc_p4<M_TF32, float4, NW_><<<blocks, 256, 0, h->stream>>>(                              \
          t1, Dl, Dr, st->Drp, st->K2, s.nw_in, s.nw_out, st->mask, st->cpar, st->T3[0].p, tlo); \
    else if (st->mode == M_TF32X3)                                                                \
      mid_tc_p4<M_TF32X3, float4, NW_><<<blocks, 256, 0, h->stream>>>(                            \
          t1, Dl, Dr, st->Drp, st->K2, s.nw_in, s.nw_out, st->mask, st->cpar, st->T3[0].p, tlo); \
    else if (Dr % 2 == 0)                                                                         \
      mid_bf16_x2<NW_><<<(unsigned)((nt / 2 + 255) / 256), 256, 0, h->stream>>>(                  \
          (const uint4*)st->T1.p, Dl, Dr, st->Drp, st->K2, s.nw_in, s.nw_out, st->mask, st->cpar, \
          (__nv_bfloat16*)st->T3[0].p);                                                           \
    else                                                                                          \
      mid_tc_p4<M_BF16, uint2, NW_><<<blocks, 256, 0, h->stream>>>(                               \
          (const uint2*)st->T1.p, Dl, Dr, st->Drp, st->K2, s.nw_in, s.nw_out, st->mask, st->cpar, \
          st->T3[0].p, tlo);                                                                      \
  } while (0)
      if (nw <= 4) MIDP4(4); else if (nw <= 6) MIDP4(6); else MIDP4(8);
#undef MIDP4
    } else
#define MIDTC(MODE_, MP_)                                                                    \
  mid_tc<MODE_, MP_><<<blocks, 256, 0, h->stream>>>((const float*)st->T1.p,                \
                                                    P, Dl, Dr, st->Drp, st->K2, s.nw_out,      \
                                                    s.d_win, s.d_wstart, s.d_coef, st->T3[0].p, tlo)
    if (P <= 4) {
      if (st->mode == M_TF32) MIDTC(M_TF32, 4); else if (st->mode == M_TF32X3) MIDTC(M_TF32X3, 4); else MIDTC(M_BF16, 4);
    } else {
      if (st->mode == M_TF32) MIDTC(M_TF32, 16); else if (st->mode == M_TF32X3) MIDTC(M_TF32X3, 16); else MIDTC(M_BF16, 16);
    }
#undef MIDTC
    FMPT_LAUNCHED(h);
  }
  return FMPT_OK;
}

// GEMM 2 of a real application, after op_tc_apply_head:
// y[(a' s'), b'] = sum_(b w2) T3[(b w2), (a' s')] Rg[(b w2), b']
int op_tc_apply_tail(fmpt_op* op, double* y) { return op_tc_apply_tail_rows(op, y, 0, op->Dr); }

// GEMM 2 for the output columns b' in [r0, r1): y[:, b'] needs rows b' of Rg only.  The
// B operand starts K2*r0 elements in (16-byte aligned: K2 is a multiple of 8 elements of
// at least 2 bytes) and the output P*Dl*r0 doubles in.
int op_tc_apply_tail_rows(fmpt_op* op, double* y, int r0, int r1) {
  fmpt_handle* h = op->h;
  TcState* st = static_cast<TcState*>(op->tc);
  if (!st || st->cplx) return set_error(h, FMPT_ERR_ARG, "apply_tail: real tensor-core operator only");
  const int Dl = op->Dl, P = st->P;
  if (r0 < 0 || r1 > op->Dr || r0 >= r1) return set_error(h, FMPT_ERR_ARG, "apply_tail: bad row range");
  const int Dr = r1 - r0;
  const int split = st->mode == M_TF32X3 ? 2 : 1;
  void* tlo = split > 1 ? st->T3[1].p : nullptr;
  y += (int64_t)P * Dl * r0;
  TcOperand A2{st->T3[0].p, tlo, st->K2, 0};
  TcOperand B2{offset(st->Rg[0].p, st->K2 * r0, st->es),
               split > 1 ? offset(st->Rg[1].p, st->K2 * r0, st->es) : nullptr, st->K2, 0};
  FMPT_TRY(tc_gemm(h, st->mode, P * Dl, Dr, (int)st->K2, 1, A2, B2, y, 1, (int64_t)P * Dl, 0,
                   st->err));
  return FMPT_OK;
}

// Complex data in the real embedding (split planes in, split planes out):
//   GEMM 1  T1[(s b), (a' w)] (+ imaginary plane) = xg'[(s b), 2K] . Lg'[(a' w) x 2, 2K]
//           with xg' rows [Re x | Im x] and Lg' rows [Re L | -Im L], [Im L | Re L]; the
//           doubled N makes the second half of the output exactly the imaginary plane
//   MPO     the real step on each plane, written as T3' rows [Re T3 | Im T3]
//   GEMM 2  y (both planes) = T3'[(a' s'), 2 K2] . Rg'[b' x 2, 2 K2]
int op_tc_apply_complex(fmpt_op* op, TcState* st, const double* x, double* y) {
  fmpt_handle* h = op->h;
  const int Dl = op->Dl, Dr = op->Dr, wl = op->wl, P = st->P;
  const int split = st->mode == M_TF32X3 ? 2 : 1;
  const int es = st->es;
  void* xlo = split > 1 ? st->xg[1].p : nullptr;
  void* tlo = split > 1 ? st->T3[1].p : nullptr;
  const int64_t nplane = (int64_t)Dl * P * Dr;
  const int64_t nx = (int64_t)st->Kp * P * Dr;
  {
    ProfScope prof(h, FMPT_K_CONVERT);
    for (int part = 0; part < 2; part++) {
      const double* src = x + part * nplane;
      void* hi = offset(st->xg[0].p, part * st->Kp, es);
      void* lo = offset(xlo, part * st->Kp, es);
      if (st->mode == M_TF32)
        conv_state<M_TF32><<<grid1(h, nx), 256, 0, h->stream>>>(src, Dl, st->Kp, (int64_t)P * Dr, hi, lo, 2LL * st->Kp);
      else if (st->mode == M_TF32X3)
        conv_state<M_TF32X3><<<grid1(h, nx), 256, 0, h->stream>>>(src, Dl, st->Kp, (int64_t)P * Dr, hi, lo, 2LL * st->Kp);
      else
        conv_state<M_BF16><<<grid1(h, nx), 256, 0, h->stream>>>(src, Dl, st->Kp, (int64_t)P * Dr, hi, lo, 2LL * st->Kp);
      FMPT_LAUNCHED(h);
    }
  }
  TcOperand A1{st->xg[0].p, xlo, 2LL * st->Kp, 0};
  TcOperand B1{st->Lg[0].p, split > 1 ? st->Lg[1].p : nullptr, 2LL * st->Kp, 0};
  FMPT_TRY(tc_gemm(h, st->mode, P * Dr, 2 * wl * Dl, 2 * st->Kp, 1, A1, B1, st->T1.p, 0,
                   (int64_t)P * Dr, 0, st->err));
  {
    const int64_t nt = (int64_t)Dl * Dr;
    const unsigned blocks = (unsigned)((nt + 255) / 256);
    const MidSchedule& s = op->kind == 2 ? op->sched : st->rsched;
    const int64_t t1plane = (int64_t)P * Dr * wl * Dl;
    const int64_t K2c = 2 * st->K2;     // row stride of T3'
    ProfScope prof(h, FMPT_K_MPO_STEP);
    for (int part = 0; part < 2; part++) {
      const float* t1 = static_cast<const float*>(st->T1.p) + part * t1plane;
      void* hi = offset(st->T3[0].p, part * st->K2, es);
      void* lo = offset(tlo, part * st->K2, es);
      if (st->fast_mid) {
          if (st->mode == M_TF32)
          mid_tc_p4<M_TF32, float4, 8><<<blocks, 256, 0, h->stream>>>((const float4*)t1, Dl, Dr, st->Drp, K2c, s.nw_in, s.nw_out, st->mask, st->cpar, hi, lo);
        else if (st->mode == M_TF32X3)
          mid_tc_p4<M_TF32X3, float4, 8><<<blocks, 256, 0, h->stream>>>((const float4*)t1, Dl, Dr, st->Drp, K2c, s.nw_in, s.nw_out, st->mask, st->cpar, hi, lo);
        else
          mid_tc_p4<M_BF16, float4, 8><<<blocks, 256, 0, h->stream>>>((const float4*)t1, Dl, Dr, st->Drp, K2c, s.nw_in, s.nw_out, st->mask, st->cpar, hi, lo);
      } else {
#define MIDTCC(MODE_, MP_)                                                                   \
  mid_tc<MODE_, MP_><<<blocks, 256, 0, h->stream>>>(t1, P, Dl, Dr, st->Drp, K2c, s.nw_out,    \
                                                    s.d_win, s.d_wstart, s.d_coef, hi, lo)
        if (P <= 4) {
          if (st->mode == M_TF32) MIDTCC(M_TF32, 4); else if (st->mode == M_TF32X3) MIDTCC(M_TF32X3, 4); else MIDTCC(M_BF16, 4);
        } else {
          if (st->mode == M_TF32) MIDTCC(M_TF32, 16); else if (st->mode == M_TF32X3) MIDTCC(M_TF32X3, 16); else MIDTCC(M_BF16, 16);
        }
#undef MIDTCC
      }
      FMPT_LAUNCHED(h);
    }
  }
  TcOperand A2{st->T3[0].p, tlo, 2 * st->K2, 0};
  TcOperand B2{st->Rg[0].p, split > 1 ? st->Rg[1].p : nullptr, 2 * st->K2, 0};
  return tc_gemm(h, st->mode, P * Dl, 2 * Dr, (int)(2 * st->K2), 1, A2, B2, y, 1, (int64_t)P * Dl,
                 0, st->err);
}

// ---------------------------------------------------------------------------
// Mixed-precision environment updates (mpo/transfer.jl:26-34), real data.
//   updateleft : T1[(s,b),(a',w)] = sum_a Bg[a,(s,b)] Lg[a,(a',w)]          (GEMM 1)
//                U [(a',s'),(w2,b)] = MPO step over (w, s)                    (bitmask)
//                hnew[b',(w2,b)]  = sum_(a',s') Ag[(a',s'),b'] U[...]        (GEMM 2, FP64 out)
//   updateright: T1[(a,s),(b',w2)] = sum_b Bt[b,(a,s)] Rt[b,(b',w2)]          (GEMM 1)
//                U [(s',b'),(w,a)] = MPO step over (w2, s)
//                hnew[a',(w,a)]   = sum_(s',b') At[(s',b'),a'] U[...]        (GEMM 2, FP64 out)
namespace {

int mask_and_coef(fmpt_handle* h, const MidSchedule& ms, int P, uint64_t* mask, MidCoef& cp) {
  if (ms.nw_in > 8 || ms.nw_out > 8 || (P != 2 && P != 4))
    return set_error(h, FMPT_ERR_UNSUPPORTED,
                     "mixed-precision environment update needs MPO bonds <= 8 and d = 2 or 4");
  std::vector<float> cf((size_t)64 * P * P, 0.f);
  uint64_t m = 0;
  for (int wo = 0; wo < ms.nw_out; wo++)
    for (int e = ms.wout_start[wo]; e < ms.wout_start[wo + 1]; e++) {
      const int wi = ms.blk_win[e];
      m |= 1ull << (wi * 8 + wo);
      for (int q = 0; q < P * P; q++)
        cf[(size_t)(wi * 8 + wo) * P * P + q] += (float)ms.coef[(size_t)e * P * P + q];
    }
  std::memset(&cp, 0, sizeof(cp));
  for (int blk = 0; blk < 64; blk++)
    for (int q = 0; q < P * P; q++) cp.c[blk][q] = cf[(size_t)blk * P * P + q];
  *mask = m;
  return FMPT_OK;
}

template <int MODE>
int launch_mask(fmpt_handle* h, int P, const float* T, int64_t i1, int64_t i2, int64_t iw,
                int64_t is, int n1, int n2, int nw_in, int nw_out, uint64_t mask, const MidCoef& c,
                void* hi, void* lo, int64_t o1, int64_t o2, int64_t ow, int64_t oq) {
  const int64_t nt = (int64_t)n1 * n2;
  const unsigned blocks = (unsigned)((nt + 255) / 256);
  ProfScope prof(h, FMPT_K_MPO_STEP);
  if (P <= 2)
    mid_tc_mask<MODE, 2><<<blocks, 256, 0, h->stream>>>(T, i1, i2, iw, is, n1, n2, nw_in, nw_out,
                                                         mask, c, hi, lo, o1, o2, ow, oq);
  else
    mid_tc_mask<MODE, 4><<<blocks, 256, 0, h->stream>>>(T, i1, i2, iw, is, n1, n2, nw_in, nw_out,
                                                         mask, c, hi, lo, o1, o2, ow, oq);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int conv_state_any(fmpt_handle* h, int mode, const double* x, int K, int Kp, int64_t M, void* hi,
                   void* lo) {
  const int64_t n = (int64_t)Kp * M;
  ProfScope prof(h, FMPT_K_CONVERT);
  if (mode == M_TF32)
    conv_state<M_TF32><<<grid1(h, n), 256, 0, h->stream>>>(x, K, Kp, M, hi, lo, Kp);
  else if (mode == M_TF32X3)
    conv_state<M_TF32X3><<<grid1(h, n), 256, 0, h->stream>>>(x, K, Kp, M, hi, lo, Kp);
  else
    conv_state<M_BF16><<<grid1(h, n), 256, 0, h->stream>>>(x, K, Kp, M, hi, lo, Kp);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

struct Planes {
  DevBuf p[2];
  void* hi() const { return p[0].p; }
  void* lo() const { return p[1].p; }
  int alloc(fmpt_handle* h, int mode, size_t n) {
    const size_t es = mode == M_BF16 ? 2 : 4;
    FMPT_TRY(p[0].alloc(h, n * es));
    if (mode == M_TF32X3) FMPT_TRY(p[1].alloc(h, n * es));
    return FMPT_OK;
  }
  int zero(fmpt_handle* h) {
    for (auto& b : p)
      if (b.p) FMPT_CUDA(h, cudaMemsetAsync(b.p, 0, b.bytes, h->stream));
    return FMPT_OK;
  }
};

int env_left_tc(fmpt_handle* h, int precision, const double* hold, const double* A,
                const double* W, const double* B, double* hnew, int Dl, int d, int Dr, int wl,
                int wr) {
  const int mode = tc_mode_of(precision);
  MidSchedule ms;
  FMPT_TRY(schedule_env(h, 0, W, d, wl, wr, false, ms));
  uint64_t mask = 0;
  MidCoef cpar;
  int st = mask_and_coef(h, ms, d, &mask, cpar);
  mid_free(h, ms);
  FMPT_TRY(st);
  const int Kp = round_up8(Dl), K2 = round_up8(Dl * d);
  Planes Bg, Lg, Ag, U;
  DevBuf T1;
  FMPT_TRY(Bg.alloc(h, mode, (size_t)Kp * d * Dr));
  FMPT_TRY(Lg.alloc(h, mode, (size_t)Kp * Dl * wl));
  FMPT_TRY(Ag.alloc(h, mode, (size_t)K2 * Dr));
  FMPT_TRY(U.alloc(h, mode, (size_t)K2 * wr * Dr));
  FMPT_TRY(U.zero(h));                                         // K padding
  FMPT_TRY(T1.alloc(h, (size_t)d * Dr * wl * Dl * sizeof(float)));
  FMPT_TRY(conv_state_any(h, mode, B, Dl, Kp, (int64_t)d * Dr, Bg.hi(), Bg.lo()));
  FMPT_TRY(transpose_any(h, mode, hold, (int64_t)Dl * wl, Dl, Dl, Dl, Kp, wl, Lg.hi(), Lg.lo(), Kp,
                         (int64_t)Kp * Dl));
  FMPT_TRY(conv_state_any(h, mode, A, Dl * d, K2, Dr, Ag.hi(), Ag.lo()));
  int* err = nullptr;
  FMPT_CUDA(h, cudaMallocAsync((void**)&err, sizeof(int), h->stream));
  FMPT_CUDA(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
  TcOperand A1{Bg.hi(), Bg.lo(), Kp, 0}, B1{Lg.hi(), Lg.lo(), Kp, 0};
  st = tc_gemm(h, mode, d * Dr, wl * Dl, Kp, 1, A1, B1, T1.p, 0, (int64_t)d * Dr, 0, err);
  // in : T1[(s + d b) + d Dr (a' + Dl w)]  (o1 = b, o2 = a')
  // out: U[(a' + Dl s') + K2 (w2 + wr b)]
  if (st == FMPT_OK) {
    const float* t1 = (const float*)T1.p;
    const MidCoef& c = cpar;
    const int64_t i1 = d, i2 = (int64_t)d * Dr, iw = (int64_t)d * Dr * Dl, is = 1;
    const int64_t o1 = (int64_t)K2 * wr, o2 = 1, ow = K2, oq = Dl;
    if (mode == M_TF32)
      st = launch_mask<M_TF32>(h, d, t1, i1, i2, iw, is, Dr, Dl, wl, wr, mask, c, U.hi(), U.lo(), o1, o2, ow, oq);
    else if (mode == M_TF32X3)
      st = launch_mask<M_TF32X3>(h, d, t1, i1, i2, iw, is, Dr, Dl, wl, wr, mask, c, U.hi(), U.lo(), o1, o2, ow, oq);
    else
      st = launch_mask<M_BF16>(h, d, t1, i1, i2, iw, is, Dr, Dl, wl, wr, mask, c, U.hi(), U.lo(), o1, o2, ow, oq);
  }
  if (st == FMPT_OK) {
    TcOperand A2{Ag.hi(), Ag.lo(), K2, 0}, B2{U.hi(), U.lo(), K2, 0};
    st = tc_gemm(h, mode, Dr, wr * Dr, K2, 1, A2, B2, hnew, 1, Dr, 0, err);
  }
  int e = 0;
  if (st == FMPT_OK) {
    FMPT_CUDA(h, cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  cudaFreeAsync(err, h->stream);
  FMPT_TRY(st);
  if (e) return set_error(h, FMPT_ERR_TIMEOUT, "tensor-core GEMM wait timed out");
  return FMPT_OK;
}

int env_right_tc(fmpt_handle* h, int precision, const double* hold, const double* A,
                 const double* W, const double* B, double* hnew, int Dl, int d, int Dr, int wl,
                 int wr) {
  const int mode = tc_mode_of(precision);
  MidSchedule ms;
  FMPT_TRY(schedule_env(h, 0, W, d, wl, wr, true, ms));
  uint64_t mask = 0;
  MidCoef cpar;
  int st = mask_and_coef(h, ms, d, &mask, cpar);
  mid_free(h, ms);
  FMPT_TRY(st);
  const int Kb = round_up8(Dr), Kq = round_up8(d * Dr);
  Planes Bt, Rt, At, U;
  DevBuf T1;
  FMPT_TRY(Bt.alloc(h, mode, (size_t)Kb * Dl * d));
  FMPT_TRY(Rt.alloc(h, mode, (size_t)Kb * Dr * wr));
  FMPT_TRY(At.alloc(h, mode, (size_t)Kq * Dl));
  FMPT_TRY(U.alloc(h, mode, (size_t)Kq * wl * Dl));
  FMPT_TRY(U.zero(h));
  FMPT_TRY(T1.alloc(h, (size_t)Dl * d * Dr * wr * sizeof(float)));
  // Bt[b + Kb (a + Dl s)] = B[(a + Dl s) + Dl d b]
  FMPT_TRY(transpose_any(h, mode, B, (int64_t)Dl * d, 0, Dl * d, Dr, Kb, 1, Bt.hi(), Bt.lo(), Kb, 0));
  // Rt[b + Kb (b' + Dr w2)] = hold[b' + Dr w2 + Dr wr b]
  FMPT_TRY(transpose_any(h, mode, hold, (int64_t)Dr * wr, Dr, Dr, Dr, Kb, wr, Rt.hi(), Rt.lo(), Kb,
                         (int64_t)Kb * Dr));
  // At[(s' + d b') + Kq a'] = A[a' + Dl (s' + d b')]   (rows a', columns (s', b'))
  FMPT_TRY(transpose_any(h, mode, A, Dl, 0, Dl, d * Dr, Kq, 1, At.hi(), At.lo(), Kq, 0));
  int* err = nullptr;
  FMPT_CUDA(h, cudaMallocAsync((void**)&err, sizeof(int), h->stream));
  FMPT_CUDA(h, cudaMemsetAsync(err, 0, sizeof(int), h->stream));
  TcOperand A1{Bt.hi(), Bt.lo(), Kb, 0}, B1{Rt.hi(), Rt.lo(), Kb, 0};
  st = tc_gemm(h, mode, Dl * d, Dr * wr, Kb, 1, A1, B1, T1.p, 0, (int64_t)Dl * d, 0, err);
  // in : T1[(a + Dl s) + Dl d (b' + Dr w2)]   (o1 = a, o2 = b', w = w2)
  // out: U[(s' + d b') + Kq (w + wl a)]
  if (st == FMPT_OK) {
    const float* t1 = (const float*)T1.p;
    const MidCoef& c = cpar;
    const int64_t i1 = 1, i2 = (int64_t)Dl * d, iw = (int64_t)Dl * d * Dr, is = Dl;
    const int64_t o1 = (int64_t)Kq * wl, o2 = d, ow = Kq, oq = 1;
    if (mode == M_TF32)
      st = launch_mask<M_TF32>(h, d, t1, i1, i2, iw, is, Dl, Dr, wr, wl, mask, c, U.hi(), U.lo(), o1, o2, ow, oq);
    else if (mode == M_TF32X3)
      st = launch_mask<M_TF32X3>(h, d, t1, i1, i2, iw, is, Dl, Dr, wr, wl, mask, c, U.hi(), U.lo(), o1, o2, ow, oq);
    else
      st = launch_mask<M_BF16>(h, d, t1, i1, i2, iw, is, Dl, Dr, wr, wl, mask, c, U.hi(), U.lo(), o1, o2, ow, oq);
  }
  if (st == FMPT_OK) {
    TcOperand A2{At.hi(), At.lo(), Kq, 0}, B2{U.hi(), U.lo(), Kq, 0};
    st = tc_gemm(h, mode, Dl, wl * Dl, Kq, 1, A2, B2, hnew, 1, Dl, 0, err);
  }
  int e = 0;
  if (st == FMPT_OK) {
    FMPT_CUDA(h, cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  cudaFreeAsync(err, h->stream);
  FMPT_TRY(st);
  if (e) return set_error(h, FMPT_ERR_TIMEOUT, "tensor-core GEMM wait timed out");
  return FMPT_OK;
}

}  // namespace

int env_update_tc(fmpt_handle* h, bool right, int precision, const double* hold,
                  const double* A, const double* W, const double* B, double* hnew, int Dl, int d,
                  int Dr, int wl, int wr) {
  return right ? env_right_tc(h, precision, hold, A, W, B, hnew, Dl, d, Dr, wl, wr)
               : env_left_tc(h, precision, hold, A, W, B, hnew, Dl, d, Dr, wl, wr);
}

int op_tc_check(fmpt_op* op) {
  TcState* st = static_cast<TcState*>(op->tc);
  if (!st || !st->err) return FMPT_OK;
  int e = 0;
  FMPT_CUDA(op->h, cudaMemcpyAsync(&e, st->err, sizeof(int), cudaMemcpyDeviceToHost, op->h->stream));
  FMPT_CUDA(op->h, cudaStreamSynchronize(op->h->stream));
  if (e) return set_error(op->h, FMPT_ERR_TIMEOUT, "tensor-core GEMM wait timed out");
  return FMPT_OK;
}

void op_tc_free(fmpt_op* op) {
  TcState* st = static_cast<TcState*>(op->tc);
  if (!st) return;
  if (st->err) cudaFreeAsync(st->err, op->h->stream);
  delete st;
  op->tc = nullptr;
}

}  // namespace fmpt
