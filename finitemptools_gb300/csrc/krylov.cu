// Krylov solvers on device-resident vectors: the reference's plain Lanczos
// for the lowest eigenpair and a Krylov exponential for TDVP.
//
// Vectors stay in HBM for the whole solve; only the small matrices and scalars
// that steer the host loop come back to the host (beta for the Lanczos stopping
// test; the Krylov exponential's Hessenberg matrix, whose small exponential and
// step-size control run on the host).  All reductions are deterministic
// two-level sums (warp shuffles inside a block, a fixed-order sum over the block
// partials, recomputed by every consumer block so that no separate
// finalisation launch is needed).
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "internal.h"

namespace fmpt {
namespace {

constexpr int KT = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Warp sums of K values at once (K a power of two <= 32).  GB300 issues an FP64 warp
// instruction at about 2 lanes per clock per SM, so the adds of a reduction cost more than
// the shuffles: plain xor-sums take 5 K adds per lane, this takes K - 1 + (5 - log2 K).
// Recursive halving: at each butterfly step (lane offsets 16, 8, ...) a lane keeps one half
// of its values, the partner lane the other half, and each adds the partner's copy of the
// half it keeps; then a plain xor-sum over the remaining lane bits.  a[0] ends up holding
// the warp sum of value (lane >> (5 - log2 K)); the order of the adds is fixed.
template <int K>
__device__ __forceinline__ void warp_sum_many(double (&a)[K]) {
  const int lane = threadIdx.x & 31;
  int o = 16;
#pragma unroll
  for (int cnt = K; cnt > 1; cnt >>= 1, o >>= 1) {
    const int half = cnt >> 1;
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < half; i++) {
      const double send = upper ? a[i] : a[i + half];
      const double keep = upper ? a[i + half] : a[i];
      a[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
#pragma unroll
  for (; o > 0; o >>= 1) a[0] += __shfl_xor_sync(0xffffffffu, a[0], o);
}

// Warps at or above nw hold exact zeros (the threads of a block past its elements) and skip
// their shuffle sums: the result is the same, and their FP64 adds no longer queue on the
// SM's FP64 pipe in front of the warps with data.
__device__ double block_sum(double v, int nw = KT / 32) {
  __shared__ double red[KT / 32];
  __shared__ double total;
  if ((threadIdx.x >> 5) < nw) v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (threadIdx.x >> 5) < nw ? v : 0.0;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < KT / 32 ? red[threadIdx.x] : 0.0;
    w = warp_sum(w);
    if (threadIdx.x == 0) total = w;
  }
  __syncthreads();
  double r = total;
  __syncthreads();
  return r;
}

// fixed-order sum of G partials (every block computes the same value)
__device__ double sum_parts(const double* part, int G) {
  double s = 0.0;
  for (int i = threadIdx.x; i < G; i += KT) s += part[i];
  return block_sum(s, G >= KT ? KT / 32 : (G + 31) / 32);
}

// part[b] = sum x*y over a grid-stride slice (real view of length n)
__global__ void rdot_partial(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                             double* __restrict__ part, const int* gate = nullptr) {
  if (gate && *gate) return;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
    s = fma(x[i], y[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// x = v / ||v|| with ||v||^2 = sum(part); stores the norm in *nrm
__global__ void normalize_from_parts(int64_t n, const double* __restrict__ v, double* __restrict__ x,
                                     const double* __restrict__ part, int G, double* nrm) {
  double s = sqrt(sum_parts(part, G));
  if (blockIdx.x == 0 && threadIdx.x == 0) *nrm = s;
  double inv = s > 0.0 ? 1.0 / s : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
    x[i] = v[i] * inv;
}

// a = sum(part_a); alpha_out = a; y -= (q*a + qm1*b_old); part_b = partial |y|^2
__global__ void lanczos_axpy(int64_t n, double* __restrict__ y, const double* __restrict__ q,
                             const double* __restrict__ qm1, const double* __restrict__ part_a,
                             int G, const double* b_old, double* alpha_out,
                             double* __restrict__ part_b, const int* gate = nullptr) {
  if (gate && *gate) return;
  const double a = sum_parts(part_a, G);
  const double b = (qm1 != nullptr) ? *b_old : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) *alpha_out = a;
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT) {
    double t = q[i] * a;
    if (qm1) t += qm1[i] * b;
    double v = y[i] - t;
    y[i] = v;
    s = fma(v, v, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part_b[blockIdx.x] = s;
}

// b = sqrt(sum(part_b)); beta_out = b; if b != 0: y /= b
__global__ void lanczos_scale(int64_t n, double* __restrict__ y, const double* __restrict__ part_b,
                              int G, double* beta_out) {
  const double b = sqrt(sum_parts(part_b, G));
  if (blockIdx.x == 0 && threadIdx.x == 0) *beta_out = b;
  if (b == 0.0) return;
  // Julia's qi /= b divides element-wise; so does this (no reciprocal)
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
    y[i] = y[i] / b;
}

// ---- multi-vector kernels over the Krylov basis V (j vectors of length n,
// complex split planes when cplx: V_i re at V + i*2n, im at V + i*2n + n)
// partial dots h_i = <V_i, z> ; part layout [G][j][2].  Chunks of MD_CH vectors per pass
// over z: every thread keeps MD_CH running sums (re, im), reduced by warp shuffles and one
// shared-memory pass per chunk -- instead of one full block reduction per vector.  Fixed
// summation order throughout (deterministic).
constexpr int MD_CH = 8;
template <int CH = MD_CH>
__device__ __forceinline__ void multidot_body(int cplx, int64_t n, int j,
                                              const double* __restrict__ V, int64_t vstride,
                                              const double* __restrict__ z,
                                              double* __restrict__ part, int epb = KT) {
  constexpr int MD_CH = CH;       // vectors per pass over z (the sums do not depend on it)
  __shared__ double red[KT / 32][2 * MD_CH];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i0 = 0; i0 < j; i0 += MD_CH) {
    double sr[MD_CH], si[MD_CH];
#pragma unroll
    for (int c = 0; c < MD_CH; c++) {
      sr[c] = 0.0;
      si[c] = 0.0;
    }
    for (int64_t e = (int64_t)blockIdx.x * epb + threadIdx.x; threadIdx.x < epb && e < n;
         e += (int64_t)gridDim.x * epb) {
      const double zr = z[e], zi = cplx ? z[n + e] : 0.0;
#pragma unroll
      for (int c = 0; c < MD_CH; c++) {
        if (i0 + c < j) {
          const double* v = V + (int64_t)(i0 + c) * vstride;
          const double vr = v[e];
          sr[c] = fma(vr, zr, sr[c]);
          if (cplx) {
            const double vi = v[n + e];
            sr[c] = fma(vi, zi, sr[c]);
            si[c] = fma(vr, zi, si[c]);
            si[c] = fma(-vi, zr, si[c]);
          }
        }
      }
    }
    double v[2 * MD_CH];
#pragma unroll
    for (int c = 0; c < MD_CH; c++) {
      v[2 * c] = sr[c];
      v[2 * c + 1] = si[c];
    }
    // warps past the block's elements hold zeros: they store them without the shuffle sums
    const bool holds = wid * 32 < epb;
    if (holds) warp_sum_many<2 * MD_CH>(v);
    {
      constexpr int sh = MD_CH == 16 ? 0 : (MD_CH == 8 ? 1 : (MD_CH == 4 ? 2 : 3));
      if ((lane & ((1 << sh) - 1)) == 0) red[wid][lane >> sh] = holds ? v[0] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 2 * MD_CH) {
      const int c = threadIdx.x >> 1;
      double t = 0.0;
      for (int w = 0; w < KT / 32; w++) t += red[w][threadIdx.x];
      if (i0 + c < j) part[((int64_t)blockIdx.x * j + i0 + c) * 2 + (threadIdx.x & 1)] = t;
    }
    __syncthreads();
  }
}

__global__ void multidot_partial(int cplx, int64_t n, int j, const double* __restrict__ V,
                                 int64_t vstride, const double* __restrict__ z,
                                 double* __restrict__ part, const int* gate = nullptr,
                                 int epb = KT) {
  if (gate && *gate) return;
  multidot_body<>(cplx, n, j, V, vstride, z, part, epb);
}

// coef[i] (re, im) = sum over the G partials, one warp per value (lanes stride over the
// partials in a fixed order, then a shuffle sum); launched with one block of KT threads
// Coefficients t0 .. t0 + 63 (t = 2 i + re/im) of the sums over the G partials [G][j][2]:
// warp w takes t = t0 + w + 8 u (u < 8); a lane adds its partials g = lane, lane + 32, ...
// in g order, then the warp sums its 8 values with warp_sum_many.  out[t] = the sum
// (accum[t] += it when given).  QMAX > 0: at most QMAX partials per lane, loads unrolled.
template <int QMAX>
__device__ __forceinline__ void coef_group(int j, int G, const double* __restrict__ part, int t0,
                                           double* out, double* accum) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double acc[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    const int t = t0 + wid + 8 * u;
    double sum = 0.0;
    if (t < 2 * j) {
      const int i = t >> 1, comp = t & 1;
      if (QMAX > 0) {
#pragma unroll
        for (int q = 0; q < QMAX; q++) {
          const int g = lane + 32 * q;
          if (g < G) sum += part[((int64_t)g * j + i) * 2 + comp];
        }
      } else {
        for (int g = lane; g < G; g += 32) sum += part[((int64_t)g * j + i) * 2 + comp];
      }
    }
    acc[u] = sum;
  }
  warp_sum_many<8>(acc);
  const int t = t0 + wid + 8 * (lane >> 2);
  if ((lane & 3) == 0 && t < 2 * j) {
    out[t] = acc[0];
    if (accum) accum[t] += acc[0];
  }
}

// coef[t] = the sums (accum[t] += them when given); launched with one block of KT threads
__global__ void multidot_finalize(int j, int G, const double* __restrict__ part,
                                  double* __restrict__ coef, double* __restrict__ accum,
                                  const int* gate = nullptr) {
  if (gate && *gate) return;
  for (int t0 = 0; t0 < 2 * j; t0 += 64) coef_group<0>(j, G, part, t0, coef, accum);
}

__device__ __forceinline__ void multi_axpy_body(int cplx, int64_t n, int j,
                                                const double* __restrict__ V, int64_t vstride,
                                                const double* __restrict__ coef,
                                                double* __restrict__ z, double* __restrict__ part,
                                                int epb = KT) {
  double s = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * epb + threadIdx.x; threadIdx.x < epb && e < n;
       e += (int64_t)gridDim.x * epb) {
    double zr = z[e], zi = cplx ? z[n + e] : 0.0;
    // MD_CH vectors' elements are loaded together (their L2 latencies overlap), then
    // subtracted in vector order
    for (int i0 = 0; i0 < j; i0 += MD_CH) {
      double vr[MD_CH], vi[MD_CH];
#pragma unroll
      for (int c = 0; c < MD_CH; c++) {
        vr[c] = 0.0;
        vi[c] = 0.0;
        if (i0 + c < j) {
          const double* v = V + (int64_t)(i0 + c) * vstride;
          vr[c] = v[e];
          if (cplx) vi[c] = v[n + e];
        }
      }
#pragma unroll
      for (int c = 0; c < MD_CH; c++) {
        if (i0 + c < j) {
          const double cr = coef[2 * (i0 + c)], ci = coef[2 * (i0 + c) + 1];
          if (cplx) {
            zr -= cr * vr[c] - ci * vi[c];
            zi -= cr * vi[c] + ci * vr[c];
          } else {
            zr -= cr * vr[c];
          }
        }
      }
    }
    z[e] = zr;
    if (cplx) z[n + e] = zi;
    s = fma(zr, zr, s);
    if (cplx) s = fma(zi, zi, s);
  }
  s = block_sum(s, (epb + 31) / 32);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void multi_axpy_sub(int cplx, int64_t n, int j, const double* __restrict__ V,
                               int64_t vstride, const double* __restrict__ coef,
                               double* __restrict__ z, double* __restrict__ part,
                               const int* gate = nullptr, int epb = KT) {
  if (gate && *gate) return;
  multi_axpy_body(cplx, n, j, V, vstride, coef, z, part, epb);
}

// out = sum_i c_i V_i (c complex when cplx, real otherwise); scale multiplies
__global__ void combine_basis(int cplx, int64_t n, int j, const double* __restrict__ V,
                              int64_t vstride, const double* __restrict__ c, int cstride,
                              double scale, int last_first, double* __restrict__ out,
                              const int* j_dev = nullptr) {
  if (j_dev) j = *j_dev;
  for (int64_t e = (int64_t)blockIdx.x * KT + threadIdx.x; e < n; e += (int64_t)gridDim.x * KT) {
    double r = 0.0, im = 0.0;
    // lanczos_linear_transformation_single (simple_lanczos.jl:70-78) adds the
    // last basis vector first
    for (int t = 0; t < j; t++) {
      int i = last_first ? (t == 0 ? j - 1 : t - 1) : t;
      const double* v = V + (int64_t)i * vstride;
      double cr = c[i * cstride], ci = cplx ? c[i * cstride + 1] : 0.0;
      double vr = v[e];
      if (cplx) {
        double vi = v[n + e];
        r += cr * vr - ci * vi;
        im += cr * vi + ci * vr;
      } else {
        r += cr * vr;
      }
    }
    out[e] = r * scale;
    if (cplx) out[n + e] = im * scale;
  }
}

// Arnoldi step closure on the device: s = ||z|| after orthogonalisation; the
// norm before it is sqrt(s^2 + sum_i |H[i][j]|^2).  If s is below 1e-12 of
// that (the Krylov space is exhausted: happy breakdown) the next basis vector
// and H[j+1][j] are zero, otherwise V_{j+1} = z / s and H[j+1][j] = s.
__device__ __forceinline__ void arnoldi_normalize_body(int64_t n_real,
                                                       const double* __restrict__ z,
                                                       const double* __restrict__ part, int G,
                                                       const double* hc, double* __restrict__ Hcol,
                                                       int j, double* __restrict__ vnext,
                                                       int epb = KT) {
  const double s = sqrt(sum_parts(part, G));
  double ref = s * s;
  for (int i = 0; i <= j; i++) ref += hc[2 * i] * hc[2 * i] + hc[2 * i + 1] * hc[2 * i + 1];
  const bool breakdown = !(s > 1e-12 * sqrt(ref));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Hcol[2 * (j + 1)] = breakdown ? 0.0 : s;
    Hcol[2 * (j + 1) + 1] = 0.0;
  }
  const double inv = breakdown ? 0.0 : 1.0 / s;
  for (int64_t e = (int64_t)blockIdx.x * epb + threadIdx.x; threadIdx.x < epb && e < n_real;
       e += (int64_t)gridDim.x * epb)
    vnext[e] = z[e] * inv;
}

__global__ void arnoldi_normalize(int64_t n_real, const double* __restrict__ z,
                                  const double* __restrict__ part, int G,
                                  double* __restrict__ Hcol, int j, double* __restrict__ vnext,
                                  int epb = KT) {
  arnoldi_normalize_body(n_real, z, part, G, Hcol, Hcol, j, vnext, epb);
}

// ---- the whole orthogonalisation step of one Arnoldi vector as ONE cooperative launch:
// pass 1 (partial dots, barrier, coefficients, z -= V c), pass 2 (the same), barrier,
// normalisation.  Every block computes the coefficients itself in the summation order of
// multidot_finalize (coef_group), so the results are bit-identical to the seven separate
// launches.  The
// grid barriers are bounded (2 s on %globaltimer): a timeout sets the abort flag and the
// handle's status word and every block returns.
struct CoopBar {
  int* count;        // arrivals (zeroed before each launch, in stream order)
  int* abort_flag;
  int* status;       // handle status word
  uint64_t wait_ns;
  int hold;          // arrivals waited for beyond the grid: 0, or 1 only to test the bound
};

__device__ __forceinline__ int ld_acquire_i(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ bool coop_barrier(const CoopBar& b, int target) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(b.count, 1);
    int ok = 1;
    const uint64_t t0 = now_ns();
    // the count alone is polled; every 32nd poll also looks at the abort flag, the status
    // word (this launch gave up, or an earlier one of the same solve did: the word stays
    // set until the host reads it) and the clock
    for (unsigned polls = 1; ld_acquire_i(b.count) < target + b.hold; polls++) {
      if ((polls & 31u) != 0) continue;
      if (ld_acquire_i(b.abort_flag) || ld_acquire_i(b.status)) { ok = 0; break; }
      if (now_ns() - t0 > b.wait_ns) {
        atomicExch(b.abort_flag, 1);
        atomicExch(b.status, 1);
        ok = 0;
        break;
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

template <int QMAX>
__global__ void __launch_bounds__(KT) arnoldi_gs_fused(int cplx, int64_t n, int j,
                                                       const double* __restrict__ V,
                                                       int64_t vstride, double* __restrict__ z,
                                                       double* __restrict__ partA,
                                                       double* __restrict__ partB,
                                                       double* __restrict__ partN,
                                                       double* __restrict__ Hcol,
                                                       double* __restrict__ vnext, CoopBar bar,
                                                       int epb) {
  __shared__ double c1[64], c2[64], hc[64];
  const int G = gridDim.x, jj = j + 1;
  // pass 1
  multidot_body<16>(cplx, n, jj, V, vstride, z, partA, epb);
  if (!coop_barrier(bar, G)) return;
  coef_group<QMAX>(jj, G, partA, 0, c1, nullptr);     // 2 jj <= 62 values: one group
  __syncthreads();
  multi_axpy_body(cplx, n, jj, V, vstride, c1, z, partN, epb);
  // pass 2 (each thread reads back only the elements it has just written)
  multidot_body<16>(cplx, n, jj, V, vstride, z, partB, epb);
  if (!coop_barrier(bar, 2 * G)) return;
  coef_group<QMAX>(jj, G, partB, 0, c2, nullptr);
  __syncthreads();
  for (int t = threadIdx.x; t < 2 * jj; t += KT) {
    hc[t] = (0.0 + c1[t]) + c2[t];    // the accumulation order of Hcol in the separate form
    if (blockIdx.x == 0) Hcol[t] = hc[t];
  }
  __syncthreads();
  multi_axpy_body(cplx, n, jj, V, vstride, c2, z, partN, epb);
  if (!coop_barrier(bar, 3 * G)) return;
  arnoldi_normalize_body(n * (cplx ? 2 : 1), z, partN, G, hc, Hcol, j, vnext, epb);
}

// the kernel instance for a grid of G blocks (partials per lane: G / 32 rounded up)
using GsKernel = void (*)(int, int64_t, int, const double*, int64_t, double*, double*, double*,
                          double*, double*, double*, CoopBar, int);
GsKernel gs_kernel_for(int G) {
  if (G <= 64) return arnoldi_gs_fused<2>;
  if (G <= 160) return arnoldi_gs_fused<5>;
  if (G <= 320) return arnoldi_gs_fused<10>;
  return arnoldi_gs_fused<19>;                 // G <= 608 = 4 blocks x 152 SMs
}

// acc *= v (device scalars)
__global__ void mul_scalar(double* acc, const double* v) { *acc *= *v; }

// x *= *a (device scalar)
__global__ void scale_by(int64_t n, double* __restrict__ x, const double* a) {
  const double f = *a;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    x[e] *= f;
}

// Lowest eigenpair of the symmetric tridiagonal (alpha[0..k-1], beta[0..k-2])
// by Sturm-sequence bisection and inverse iteration with a partially pivoted
// tridiagonal solve (the LAPACK dgtsv elimination).  One thread: k <= 128.
__device__ void tridiag_lowest_body(int k, const double* __restrict__ alpha,
                                    const double* __restrict__ beta, double* eval_out,
                                    double* __restrict__ evec_out) {
  double lo = alpha[0], hi = alpha[0];
  for (int i = 0; i < k; i++) {
    double r = (i > 0 ? fabs(beta[i - 1]) : 0.0) + (i < k - 1 ? fabs(beta[i]) : 0.0);
    lo = fmin(lo, alpha[i] - r);
    hi = fmax(hi, alpha[i] + r);
  }
  const double tiny = 1e-300;
  for (int it = 0; it < 200; it++) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    int cnt = 0;
    double q = alpha[0] - mid;
    if (q < 0) cnt++;
    for (int i = 1; i < k; i++) {
      if (q == 0.0) q = tiny;
      q = (alpha[i] - mid) - beta[i - 1] * beta[i - 1] / q;
      if (q < 0) cnt++;
    }
    if (cnt >= 1) hi = mid; else lo = mid;
  }
  const double lam = 0.5 * (lo + hi);
  *eval_out = lam;
  if (k == 1) { evec_out[0] = 1.0; return; }
  double dl[128], dd[128], du[128], du2[128], x[128];
  for (int i = 0; i < k; i++) x[i] = 1.0 / sqrt((double)k) * (1.0 + 0.01 * i);
  // a zero pivot is replaced by eps*|T| (the LAPACK dlagts perturbation idea)
  const double pert = 2.2e-16 * (fmax(fabs(lo), fabs(hi)) + 1e-300);
  for (int iter = 0; iter < 3; iter++) {
    for (int i = 0; i < k; i++) {
      dd[i] = alpha[i] - lam;
      if (i < k - 1) { dl[i] = beta[i]; du[i] = beta[i]; }
      du2[i] = 0.0;
    }
    // forward elimination with row interchanges
    for (int i = 0; i < k - 1; i++) {
      if (fabs(dd[i]) >= fabs(dl[i])) {
        if (dd[i] == 0.0) dd[i] = pert;
        double f = dl[i] / dd[i];
        dd[i + 1] -= f * du[i];
        x[i + 1] -= f * x[i];
        dl[i] = 0.0;
      } else {
        double f = dd[i] / dl[i];
        dd[i] = dl[i];
        double t = dd[i + 1];
        dd[i + 1] = du[i] - f * t;
        if (i < k - 2) {
          du2[i] = du[i + 1];
          du[i + 1] = -f * du2[i];
        }
        du[i] = t;
        double xt = x[i];
        x[i] = x[i + 1];
        x[i + 1] = xt - f * x[i + 1];
      }
    }
    if (dd[k - 1] == 0.0) dd[k - 1] = pert;
    // back substitution
    x[k - 1] = x[k - 1] / dd[k - 1];
    x[k - 2] = (x[k - 2] - du[k - 2] * x[k - 1]) / dd[k - 2];
    for (int i = k - 3; i >= 0; i--) x[i] = (x[i] - du[i] * x[i + 1] - du2[i] * x[i + 2]) / dd[i];
    // normalise without overflow: scale by the largest entry first
    double mx = 0.0;
    for (int i = 0; i < k; i++) mx = fmax(mx, fabs(x[i]));
    if (!(mx > 0.0) || !isfinite(mx)) { for (int i = 0; i < k; i++) x[i] = (i == 0); mx = 1.0; }
    double nrm = 0.0;
    for (int i = 0; i < k; i++) { x[i] /= mx; nrm += x[i] * x[i]; }
    nrm = sqrt(nrm);
    for (int i = 0; i < k; i++) x[i] /= nrm;
  }
  for (int i = 0; i < k; i++) evec_out[i] = x[i];
}

__global__ void tridiag_lowest(int k, const double* __restrict__ alpha,
                               const double* __restrict__ beta, double* eval_out,
                               double* __restrict__ evec_out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  tridiag_lowest_body(k, alpha, beta, eval_out, evec_out);
}

// the same with the Krylov dimension read from the device (graph-driven solve)
__global__ void tridiag_lowest_dev(const int* __restrict__ k, const double* __restrict__ alpha,
                                   const double* __restrict__ beta, double* eval_out,
                                   double* __restrict__ evec_out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  tridiag_lowest_body(*k, alpha, beta, eval_out, evec_out);
}

// Graph-driven Lanczos step closure.  ctl: [0] stop (converged or failed),
// [1] Krylov dimension k, [2] beta was not finite, [3] converged (beta < btol).
// Step j has produced alpha_j and the partial norms of the new residual y:
// beta_j = ||y||; k = j + 1; stop when beta_j < btol (or is not finite),
// otherwise V_{j+1} = y / beta_j.
__global__ void lanczos_close(int64_t n, const double* __restrict__ y,
                              const double* __restrict__ part_b, int G, double* beta_out,
                              int* ctl, double btol, int j, double* __restrict__ vnext) {
  if (ctl[0]) return;
  const double b = sqrt(sum_parts(part_b, G));
  const bool bad = !isfinite(b);
  const bool conv = !bad && b < btol;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *beta_out = b;
    ctl[1] = j + 1;
    if (bad) ctl[2] = 1;
    if (conv) ctl[3] = 1;
    if (bad || conv) ctl[0] = 1;
  }
  if (bad || conv) return;
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT)
    vnext[i] = y[i] / b;
}

// exp(A) e_1 for the small complex matrix A = t * H_m of a Krylov exponential (m <= 31,
// column-major (re, im) pairs), on the host: the m x m problem is a few hundred thousand
// flops, which a host core runs in tens of microseconds while one SM's FP64 pipe (about
// 2 DFMA per clock) needs a millisecond -- and the step-size control reads the result on
// the host anyway.  Taylor scaling and squaring (Moler & Van Loan, method 3): s halvings
// bring ||A||_1 to <= 1, where the degree-kDeg Taylor polynomial T is exact to rounding
// (remainder < e / 19! ~ 2e-17); exp(A) e_1 = T(A / 2^s)^(2^s) e_1, applied to the vector
// when 2^s applications of T cost less than s squarings of the matrix, else by squaring.
constexpr int kDeg = 18;
constexpr double kTheta = 1.0;     // ||A / 2^s||_1 <= 1: the Taylor remainder is < 1 / 19!
using cplx = std::complex<double>;

// y = a x for an m x m complex matrix in split planes (ar, ai column-major) whose column c
// is zero below row rows[c] - 1 (an upper Hessenberg matrix has rows[c] = c + 2); plain
// double arithmetic (std::complex products take a slow special-value path without
// fast-math)
void cmatvec(int m, const double* ar, const double* ai, const int* rows, const double* xr,
             const double* xi, double* yr, double* yi) {
  for (int r = 0; r < m; r++) { yr[r] = 0.0; yi[r] = 0.0; }
  for (int c = 0; c < m; c++) {
    const double br = xr[c], bi = xi[c];
    const double* cr = ar + (size_t)m * c;
    const double* ci = ai + (size_t)m * c;
    const int nr = rows[c];
    for (int r = 0; r < nr; r++) {
      yr[r] += cr[r] * br - ci[r] * bi;
      yi[r] += cr[r] * bi + ci[r] * br;
    }
  }
}

void host_expm_col(int m, const double* A, std::vector<cplx>& out) {
  const size_t mm = (size_t)m * m;
  std::vector<double> ar(mm), ai(mm);
  std::vector<int> rows(m, 0), full(m, m);
  double nrm = 0.0;
  for (int c = 0; c < m; c++) {
    double col = 0.0;
    for (int r = 0; r < m; r++) {
      const size_t e = r + (size_t)m * c;
      ar[e] = A[2 * e];
      ai[e] = A[2 * e + 1];
      col += std::hypot(ar[e], ai[e]);
      if (ar[e] != 0.0 || ai[e] != 0.0) rows[c] = r + 1;
    }
    nrm = std::max(nrm, col);
  }
  int sq = 0;
  while (nrm > kTheta && sq < 60) { nrm *= 0.5; sq++; }
  const double sc = std::ldexp(1.0, -sq);
  for (size_t e = 0; e < mm; e++) { ar[e] *= sc; ai[e] *= sc; }
  out.assign(m, cplx(0.0, 0.0));
  const bool by_vector = sq < 20 && (double)(1 << sq) * kDeg < (double)(kDeg + sq) * m;
  if (by_vector) {
    // Horner: T(A) w = w + A (w + A / 2 (w + ... (w + A w / kDeg)))
    std::vector<double> wr(m, 0.0), wi(m, 0.0), ur(m), ui(m), tr(m), ti(m);
    wr[0] = 1.0;
    for (int round = 0; round < (1 << sq); round++) {
      ur = wr;
      ui = wi;
      for (int k = kDeg; k >= 1; k--) {
        cmatvec(m, ar.data(), ai.data(), rows.data(), ur.data(), ui.data(), tr.data(),
                ti.data());
        const double inv = 1.0 / (double)k;
        for (int r = 0; r < m; r++) {
          ur[r] = wr[r] + tr[r] * inv;
          ui[r] = wi[r] + ti[r] * inv;
        }
      }
      wr.swap(ur);
      wi.swap(ui);
    }
    for (int r = 0; r < m; r++) out[r] = cplx(wr[r], wi[r]);
    return;
  }
  // matrix form: E = T(A) by the powers A^k / k!, then s squarings; column 0 out
  std::vector<double> er(mm, 0.0), ei(mm, 0.0), pr(mm, 0.0), pi(mm, 0.0), qr(mm), qi(mm);
  for (int r = 0; r < m; r++) { er[r + (size_t)m * r] = 1.0; pr[r + (size_t)m * r] = 1.0; }
  // Z = X Y, column by column as matrix-vector products
  auto matmul = [&](const std::vector<double>& xr, const std::vector<double>& xi,
                    const std::vector<double>& yr, const std::vector<double>& yi,
                    std::vector<double>& zr, std::vector<double>& zi) {
    for (int c = 0; c < m; c++)
      cmatvec(m, xr.data(), xi.data(), full.data(), yr.data() + (size_t)m * c,
              yi.data() + (size_t)m * c, zr.data() + (size_t)m * c, zi.data() + (size_t)m * c);
  };
  for (int k = 1; k <= kDeg; k++) {
    matmul(pr, pi, ar, ai, qr, qi);
    const double inv = 1.0 / (double)k;
    for (size_t e = 0; e < mm; e++) {
      pr[e] = qr[e] * inv;
      pi[e] = qi[e] * inv;
      er[e] += pr[e];
      ei[e] += pi[e];
    }
  }
  for (int t = 0; t < sq; t++) {
    matmul(er, ei, er, ei, qr, qi);
    er.swap(qr);
    ei.swap(qi);
  }
  for (int r = 0; r < m; r++) out[r] = cplx(er[r], ei[r]);
}


int grid_for(fmpt_handle* h, int64_t n) {
  int64_t g = (n + KT - 1) / KT;
  int64_t cap = (int64_t)h->sm_count * 4;
  if (cap < 1) cap = 1;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

// Lanczos on a block-sparse operator as ONE CUDA graph: every step of the
// reference recurrence (simple_lanczos.jl:27-68) for j = 0..kmax-1 is
// captured; the step closure (lanczos_close) raises a device stop flag when
// beta < btol, and every later node of the graph -- the grouped H_eff launch
// included -- reads it and returns at once.  One host synchronisation per
// solve.  Any capture or instantiation failure sets *fallback and leaves the
// stream as it was, so the caller runs the host-driven loop instead.
int lanczos_graph(fmpt_op* op, const double* x0, int kmax, double btol, int reorth,
                  double* eigval, double* xout, int* info, int* niter, bool* fallback) {
  fmpt_handle* h = op->h;
  *fallback = true;
  cudaStreamCaptureStatus cap0 = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &cap0) != cudaSuccess ||
      cap0 != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return FMPT_OK;   // the caller is capturing already: no nested capture
  }
  const int64_t n = op->n;   // real data
  const int G = grid_for(h, n);
  DevBuf Vb, Yb, scal, partA, partB, partM, coef, ctlb;
  FMPT_TRY(Vb.alloc(h, (size_t)(kmax + 1) * n * sizeof(double)));
  FMPT_TRY(Yb.alloc(h, (size_t)n * sizeof(double)));
  FMPT_TRY(scal.alloc(h, (size_t)(3 * kmax + 8) * sizeof(double)));
  FMPT_TRY(partA.alloc(h, (size_t)G * sizeof(double)));
  FMPT_TRY(partB.alloc(h, (size_t)G * sizeof(double)));
  FMPT_TRY(partM.alloc(h, (size_t)G * (kmax + 1) * 2 * sizeof(double)));
  FMPT_TRY(coef.alloc(h, (size_t)(kmax + 1) * 2 * sizeof(double)));
  FMPT_TRY(ctlb.alloc(h, 4 * sizeof(int)));
  FMPT_TRY(gp_prepare(h));
  FMPT_TRY(ensure_pinned(h, 4));
  double* V = Vb.d();
  double* y = Yb.d();
  double* s_vm = scal.d();
  double* s_alpha = scal.d() + 1;
  double* s_beta = scal.d() + 1 + kmax;
  double* s_eval = scal.d() + 1 + 2 * kmax;
  double* s_evec = scal.d() + 2 + 2 * kmax;
  int* ctl = static_cast<int*>(ctlb.p);
  auto V_ = [&](int i) { return V + (int64_t)i * n; };
  cudaStream_t st = h->stream;
  auto record = [&]() -> int {
    FMPT_CUDA(h, cudaMemsetAsync(ctl, 0, 4 * sizeof(int), st));
    rdot_partial<<<G, KT, 0, st>>>(n, x0, x0, partA.d());
    FMPT_LAUNCHED(h);
    normalize_from_parts<<<G, KT, 0, st>>>(n, x0, V_(0), partA.d(), G, s_vm);
    FMPT_LAUNCHED(h);
    for (int j = 0; j < kmax; j++) {
      FMPT_TRY(op_u1_apply(op, V_(j), y, ctl));
      FMPT_TRY(op_project(op, y, ctl));
      rdot_partial<<<G, KT, 0, st>>>(n, V_(j), y, partA.d(), ctl);
      FMPT_LAUNCHED(h);
      lanczos_axpy<<<G, KT, 0, st>>>(n, y, V_(j), j ? V_(j - 1) : nullptr, partA.d(), G,
                                     j ? s_beta + (j - 1) : nullptr, s_alpha + j, partB.d(), ctl);
      FMPT_LAUNCHED(h);
      if (reorth) {
        multidot_partial<<<G, KT, 0, st>>>(0, n, j + 1, V, n, y, partM.d(), ctl);
        FMPT_LAUNCHED(h);
        multidot_finalize<<<1, KT, 0, st>>>(j + 1, G, partM.d(), coef.d(), nullptr, ctl);
        FMPT_LAUNCHED(h);
        multi_axpy_sub<<<G, KT, 0, st>>>(0, n, j + 1, V, n, coef.d(), y, partB.d(), ctl);
        FMPT_LAUNCHED(h);
      }
      lanczos_close<<<G, KT, 0, st>>>(n, y, partB.d(), G, s_beta + j, ctl, btol, j, V_(j + 1));
      FMPT_LAUNCHED(h);
    }
    tridiag_lowest_dev<<<1, 1, 0, st>>>(ctl + 1, s_alpha, s_beta, s_eval, s_evec);
    FMPT_LAUNCHED(h);
    combine_basis<<<G, KT, 0, st>>>(0, n, 0, V, n, s_evec, 1, 1.0, 1, xout, ctl + 1);
    FMPT_LAUNCHED(h);
    FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, s_eval, sizeof(double), cudaMemcpyDeviceToHost, st));
    FMPT_CUDA(h, cudaMemcpyAsync(h->pinned + 1, ctl, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    return FMPT_OK;
  };
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return FMPT_OK;
  }
  const int rst = record();
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (rst != FMPT_OK || ce != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return FMPT_OK;
  }
  bool ready = false;
  if (h->lanczos_exec) {
    cudaGraphExecUpdateResultInfo ri;
    if (cudaGraphExecUpdate(h->lanczos_exec, graph, &ri) == cudaSuccess) {
      ready = true;
    } else {
      cudaGetLastError();
      cudaGraphExecDestroy(h->lanczos_exec);
      h->lanczos_exec = nullptr;
    }
  }
  if (!ready && cudaGraphInstantiate(&h->lanczos_exec, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    h->lanczos_exec = nullptr;
    cudaGraphDestroy(graph);
    return FMPT_OK;
  }
  cudaGraphDestroy(graph);
  *fallback = false;
  FMPT_CUDA(h, cudaGraphLaunch(h->lanczos_exec, st));
  h->graph_launches++;
  FMPT_CUDA(h, cudaStreamSynchronize(st));
  // read the staged results before anything else reuses the pinned buffer
  const int* c = reinterpret_cast<const int*>(h->pinned + 1);
  const int k = c[1], bad = c[2], conv = c[3];
  const double ev = h->pinned[0];
  FMPT_TRY(gp_check_status(h));
  if (bad) return set_error(h, FMPT_ERR_NONFINITE, "lanczos: beta is not finite");
  *eigval = ev;
  if (info) *info = conv ? 0 : -1;
  if (niter) *niter = k;
  return FMPT_OK;
}

// part[2b], part[2b+1] = Re, Im of a grid-stride slice of dot(y, p) = sum conj(y) p
// (Julia's dot, as in _project!); split planes at offset n when cplx
__global__ void proj_dot_partial(int cplx, int64_t n, const double* __restrict__ y,
                                 const double* __restrict__ p, double* __restrict__ part,
                                 const int* gate) {
  if (gate && *gate) return;
  double sr = 0.0, si = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT) {
    sr = fma(y[i], p[i], sr);
    if (cplx) {
      sr = fma(y[n + i], p[n + i], sr);
      si = fma(y[i], p[n + i], si);
      si = fma(-y[n + i], p[i], si);
    }
  }
  sr = block_sum(sr);
  if (cplx) si = block_sum(si);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sr;
    part[2 * blockIdx.x + 1] = si;
  }
}

// c = sum of the G partials (same fixed order in every block); y -= c p
__global__ void proj_axpy(int cplx, int64_t n, double* __restrict__ y, const double* __restrict__ p,
                          const double* __restrict__ part, int G, const int* gate) {
  if (gate && *gate) return;
  double ar = 0.0, ai = 0.0;
  for (int i = threadIdx.x; i < G; i += KT) {
    ar += part[2 * i];
    ai += part[2 * i + 1];
  }
  const double cr = block_sum(ar);
  const double ci = cplx ? block_sum(ai) : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * KT + threadIdx.x; i < n; i += (int64_t)gridDim.x * KT) {
    if (cplx) {
      const double pr = p[i], pi = p[n + i];
      y[i] -= cr * pr - ci * pi;
      y[n + i] -= cr * pi + ci * pr;
    } else {
      y[i] -= cr * p[i];
    }
  }
}

// ---- several eigenpairs: thick-restart Lanczos (exact diagonalisation)

// Symmetric eigendecomposition of a small dense matrix by cyclic Jacobi
// rotations (the two-sided rotation of Golub & Van Loan, Matrix Computations,
// sec. 8.5): A (column-major m x m) is destroyed, w receives the eigenvalues in
// ascending order and Z the matching orthonormal columns.
void jacobi_eigh(int m, std::vector<double>& A, std::vector<double>& w, std::vector<double>& Z) {
  std::vector<double> R((size_t)m * m, 0.0);
  for (int i = 0; i < m; i++) R[i + (size_t)i * m] = 1.0;
  auto a = [&](int i, int j) -> double& { return A[i + (size_t)j * m]; };
  double fro = 0.0;
  for (double v : A) fro += v * v;
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = 0.0;
    for (int q = 1; q < m; q++)
      for (int p = 0; p < q; p++) off += a(p, q) * a(p, q);
    if (off <= 1e-32 * fro) break;
    for (int p = 0; p < m - 1; p++)
      for (int q = p + 1; q < m; q++) {
        const double apq = a(p, q);
        if (apq == 0.0) continue;
        const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) /
                         (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < m; k++) {          // A J
          const double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - sn * akq;
          a(k, q) = sn * akp + c * akq;
        }
        for (int k = 0; k < m; k++) {          // J^T (A J)
          const double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - sn * aqk;
          a(q, k) = sn * apk + c * aqk;
        }
        for (int k = 0; k < m; k++) {          // Z J
          double* zp = &R[k + (size_t)p * m];
          double* zq = &R[k + (size_t)q * m];
          const double zkp = *zp, zkq = *zq;
          *zp = c * zkp - sn * zkq;
          *zq = sn * zkp + c * zkq;
        }
      }
  }
  std::vector<int> ord(m);
  for (int i = 0; i < m; i++) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  w.resize(m);
  Z.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; i++) {
    w[i] = a(ord[i], ord[i]);
    for (int k = 0; k < m; k++) Z[k + (size_t)i * m] = R[k + (size_t)ord[i] * m];
  }
}

// C (nr x c) = V (nr x mm, real view, ld nr) * Y (mm x c, host) on the stream
int basis_times(fmpt_handle* h, const double* V, int64_t nr, int mm, const std::vector<double>& Y,
                int c, DevBuf& Yd, double* C) {
  FMPT_CUDA(h, cudaMemcpyAsync(Yd.d(), Y.data(), (size_t)mm * c * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
  GemmArgs g{};
  g.cplx = 0; g.ta = FMPT_N; g.tb = FMPT_N;
  g.m = (int)nr; g.n = c; g.k = mm;
  g.alpha[0] = 1.0; g.beta[0] = 0.0;
  g.A = V; g.lda = nr; g.planeA = 0;
  g.B = Yd.d(); g.ldb = mm; g.planeB = 0;
  g.C = C; g.ldc = nr; g.planeC = 0;
  g.batch = 1;
  return gemm_f64(h, g);
}

// Thick-restart Lanczos (Wu & Simon, SIAM J. Matrix Anal. Appl. 22 (2000) 602)
// with full reorthogonalisation (two classical Gram-Schmidt passes) for the
// ``num`` eigenvalues of a Hermitian operator at one end of the spectrum
// (which 0: smallest, 1: largest).  The basis lives on the device; the
// Rayleigh quotient (at most krylovdim x krylovdim, real symmetric: the
// Lanczos coefficients of a Hermitian operator are real) is solved on the host.
// A Ritz pair has converged when its residual norm |beta_m y_m| <= tol.
int eigsolve_impl(fmpt_op* op, const double* x0, int num, int kdim, int maxiter, double tol,
                  int which, double* evals, double* evecs, double* resid, int* nconv,
                  int* napply) {
  fmpt_handle* h = op->h;
  const int cp = op->dtype == FMPT_C128;
  const int64_t n = op->n;
  const int64_t nr = n * (cp ? 2 : 1);
  const int m = (int)std::min<int64_t>(kdim, n);
  if (num > m) return set_error(h, FMPT_ERR_ARG, "eigsolve: num %d exceeds the space", num);
  if (m < n && m < num + 2)
    return set_error(h, FMPT_ERR_ARG, "eigsolve: krylovdim must be at least num + 2");
  const int G = grid_for(h, n);
  DevBuf Vb, zb, partA, partM, coef, acc, Yd, tmp, snrm;
  FMPT_TRY(Vb.alloc(h, (size_t)(m + 1) * nr * sizeof(double)));
  FMPT_TRY(zb.alloc(h, (size_t)nr * sizeof(double)));
  FMPT_TRY(partA.alloc(h, (size_t)G * sizeof(double)));
  FMPT_TRY(partM.alloc(h, (size_t)G * (m + 1) * 2 * sizeof(double)));
  FMPT_TRY(coef.alloc(h, (size_t)(m + 1) * 2 * sizeof(double)));
  FMPT_TRY(acc.alloc(h, (size_t)(m + 1) * 2 * sizeof(double)));
  FMPT_TRY(Yd.alloc(h, (size_t)m * m * sizeof(double)));
  FMPT_TRY(snrm.alloc(h, sizeof(double)));
  FMPT_TRY(ensure_pinned(h, (size_t)2 * (m + 1) + G + 1));
  double* V = Vb.d();
  double* z = zb.d();
  auto V_ = [&](int i) { return V + (int64_t)i * nr; };
  cudaStream_t st = h->stream;
  rdot_partial<<<G, KT, 0, st>>>(nr, x0, x0, partA.d());
  FMPT_LAUNCHED(h);
  normalize_from_parts<<<G, KT, 0, st>>>(nr, x0, V_(0), partA.d(), G, snrm.d());
  FMPT_LAUNCHED(h);
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, snrm.d(), sizeof(double), cudaMemcpyDeviceToHost, st));
  FMPT_CUDA(h, cudaStreamSynchronize(st));
  if (!(h->pinned[0] > 0.0) || !std::isfinite(h->pinned[0]))
    return set_error(h, FMPT_ERR_ARG, "eigsolve: the start vector is zero or not finite");
  std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0);
  auto Hx = [&](int i, int j) -> double& { return H[i + (size_t)j * (m + 1)]; };
  std::vector<double> theta, Y, A;
  int k = 0, applies = 0;
  for (int it = 0;; it++) {
    bool breakdown = false;
    int j = k;
    for (; j < m; j++) {
      FMPT_TRY(fmpt_op_apply(op, V_(j), z));
      applies++;
      FMPT_CUDA(h, cudaMemsetAsync(acc.d(), 0, (size_t)2 * (j + 1) * sizeof(double), st));
      for (int pass = 0; pass < 2; pass++) {
        multidot_partial<<<G, KT, 0, st>>>(cp, n, j + 1, V, nr, z, partM.d());
        FMPT_LAUNCHED(h);
        multidot_finalize<<<1, KT, 0, st>>>(j + 1, G, partM.d(), coef.d(), acc.d());
        FMPT_LAUNCHED(h);
        multi_axpy_sub<<<G, KT, 0, st>>>(cp, n, j + 1, V, nr, coef.d(), z, partA.d());
        FMPT_LAUNCHED(h);
      }
      double* hp = h->pinned;
      FMPT_CUDA(h, cudaMemcpyAsync(hp, acc.d(), (size_t)2 * (j + 1) * sizeof(double),
                                   cudaMemcpyDeviceToHost, st));
      FMPT_CUDA(h, cudaMemcpyAsync(hp + 2 * (j + 1), partA.d(), (size_t)G * sizeof(double),
                                   cudaMemcpyDeviceToHost, st));
      FMPT_CUDA(h, cudaStreamSynchronize(st));
      double b2 = 0.0;
      for (int g = 0; g < G; g++) b2 += hp[2 * (j + 1) + g];
      double ref = b2;
      for (int i = 0; i <= j; i++) {
        Hx(i, j) = Hx(j, i) = hp[2 * i];
        ref += hp[2 * i] * hp[2 * i] + hp[2 * i + 1] * hp[2 * i + 1];
      }
      if (!std::isfinite(b2)) return set_error(h, FMPT_ERR_NONFINITE, "eigsolve: not finite");
      const double beta = std::sqrt(b2);
      if (!(beta > 1e-12 * std::sqrt(ref))) {     // invariant subspace: exact Ritz pairs
        breakdown = true;
        j++;
        break;
      }
      normalize_from_parts<<<G, KT, 0, st>>>(nr, z, V_(j + 1), partA.d(), G, snrm.d());
      FMPT_LAUNCHED(h);
      Hx(j + 1, j) = Hx(j, j + 1) = beta;
    }
    const int mm = j;
    const double beta_last = breakdown ? 0.0 : Hx(mm, mm - 1);
    A.assign((size_t)mm * mm, 0.0);
    for (int c = 0; c < mm; c++)
      for (int r = 0; r < mm; r++) A[r + (size_t)c * mm] = Hx(r, c);
    jacobi_eigh(mm, A, theta, Y);
    std::vector<int> idx(mm);
    for (int i = 0; i < mm; i++) idx[i] = which == 1 ? mm - 1 - i : i;
    std::vector<double> res(mm);
    int conv = 0;
    for (int i = 0; i < mm; i++) res[i] = std::fabs(beta_last * Y[(mm - 1) + (size_t)idx[i] * mm]);
    while (conv < num && res[conv] <= tol) conv++;
    if (conv >= num || breakdown || it + 1 >= maxiter) {
      if (mm < num)
        return set_error(h, FMPT_ERR_ARG,
                         "eigsolve: the start vector lies in an invariant subspace of "
                         "dimension %d < num", mm);
      std::vector<double> Ys((size_t)mm * num);
      for (int i = 0; i < num; i++)
        for (int r = 0; r < mm; r++) Ys[r + (size_t)i * mm] = Y[r + (size_t)idx[i] * mm];
      FMPT_TRY(basis_times(h, V, nr, mm, Ys, num, Yd, evecs));
      for (int i = 0; i < num; i++) {
        evals[i] = theta[idx[i]];
        if (resid) resid[i] = res[i];
      }
      if (nconv) *nconv = breakdown ? num : conv;
      if (napply) *napply = applies;
      FMPT_CUDA(h, cudaStreamSynchronize(st));
      return FMPT_OK;
    }
    // keep the ``keep`` best Ritz vectors and the residual direction
    const int keep = std::min(mm - 1, num + (mm - num) / 2);
    std::vector<double> Ys((size_t)mm * keep);
    for (int i = 0; i < keep; i++)
      for (int r = 0; r < mm; r++) Ys[r + (size_t)i * mm] = Y[r + (size_t)idx[i] * mm];
    if (!tmp.p) {
      FMPT_TRY(tmp.alloc(h, (size_t)m * nr * sizeof(double)));
    }
    FMPT_TRY(basis_times(h, V, nr, mm, Ys, keep, Yd, tmp.d()));
    FMPT_CUDA(h, cudaMemcpyAsync(V, tmp.d(), (size_t)keep * nr * sizeof(double),
                                 cudaMemcpyDeviceToDevice, st));
    FMPT_CUDA(h, cudaMemcpyAsync(V_(keep), V_(mm), (size_t)nr * sizeof(double),
                                 cudaMemcpyDeviceToDevice, st));
    std::fill(H.begin(), H.end(), 0.0);
    for (int i = 0; i < keep; i++) {
      Hx(i, i) = theta[idx[i]];
      Hx(i, keep) = Hx(keep, i) = beta_last * Y[(mm - 1) + (size_t)idx[i] * mm];
    }
    k = keep;
  }
}

}  // namespace

// _project! (algorithms/dmrgexcited.jl:1-6): y = y - dot(y, p) p for every
// projector in turn, on the handle's stream with the scalars kept on the device
int op_project(fmpt_op* op, double* y, const int* gate) {
  if (op->proj.empty()) return FMPT_OK;
  fmpt_handle* h = op->h;
  const int cp = op->dtype == FMPT_C128;
  for (const double* p : op->proj) {
    proj_dot_partial<<<op->proj_G, KT, 0, h->stream>>>(cp, op->n, y, p, op->proj_part, gate);
    FMPT_LAUNCHED(h);
    proj_axpy<<<op->proj_G, KT, 0, h->stream>>>(cp, op->n, y, p, op->proj_part, op->proj_G,
                                                 gate);
    FMPT_LAUNCHED(h);
  }
  return FMPT_OK;
}

// Grid of the Arnoldi orthogonalisation kernels: EPB_A vector elements (complex elements
// for complex data) per block and pass.  A D = 64 vector (8192 elements) runs on 64 blocks
// whose four element-holding warps spread over the SM's four FP64 sub-partitions (one
// exponential of 20 vectors: 1.92 ms, against 1.97 ms with 64 elements per block on 128
// SMs and 2.18 ms with 32); at most two blocks per SM.
constexpr int EPB_A = 128;
int arnoldi_grid(fmpt_handle* h, int64_t n) {
  const int64_t g = (n + EPB_A - 1) / EPB_A;
  const int64_t cap = 2LL * std::max(1, h->sm_count);
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

// Workspace of the fused orthogonalisation step (arnoldi_gs_fused): the pass-2 partials
// (pass 1 uses the caller's partM), the barrier words and the status word.
struct GsWork {
  double* partB;
  int* bar;
  int* status;
  uint64_t wait_ns;
  int hold;
};

// Whether G blocks of arnoldi_gs_fused are co-resident on this device (the cooperative
// launch needs it); measured once per device.
bool gs_fused_fits(fmpt_handle* h, int G) {
  static int occ[64] = {};
  static bool done[64] = {};
  const int dev = h->device;
  if (dev < 0 || dev >= 64) return false;
  if (!done[dev]) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, arnoldi_gs_fused<19>, KT, 0) !=
        cudaSuccess) {
      cudaGetLastError();
      b = 0;
    }
    occ[dev] = b;
    done[dev] = true;
  }
  return (int64_t)occ[dev] * h->sm_count >= G;
}

// Set up the fused step's workspace in `buf` (allocated here) when it applies: enabled on
// the handle (fmpt_set_fused_krylov), a co-resident grid and a Krylov space of at most 31
// vectors.  gs stays null otherwise (the separate launches run).
int gs_setup(fmpt_op* op, int G, int M, DevBuf& buf, GsWork& w, const GsWork** gs) {
  fmpt_handle* h = op->h;
  *gs = nullptr;
  if (!h->fused_gs || M > 31 || !gs_fused_fits(h, G)) return FMPT_OK;
  const size_t nb = (size_t)G * (M + 1) * 2 * sizeof(double);
  FMPT_TRY(buf.alloc(h, nb + 16 * sizeof(int)));
  w.partB = buf.d();
  w.bar = reinterpret_cast<int*>(static_cast<char*>(buf.p) + nb);
  FMPT_TRY(gp_status_word(h, &w.status));
  w.wait_ns = h->wait_test_ns > 0 ? (uint64_t)h->wait_test_ns : 2000000000ull;
  w.hold = h->wait_test_hold;
  *gs = &w;
  return FMPT_OK;
}

// The Arnoldi basis V_1..V_M of fmpt_exponentiate / fmpt_expm_nodes (two-pass classical
// Gram-Schmidt; the columns of H into Hdev), device launches only.  With graphs enabled the
// launches are captured into one CUDA graph per operator structure and replayed: the
// executable graph is updated in place (cudaGraphExecUpdate) for the next operator of the
// same structure, so the host issues one launch per basis instead of about a dozen per
// vector.  Any capture, instantiation, update or launch failure -- the first call on a
// fresh operator among them, whose scratch is sized outside capture -- runs the same
// launches directly.
int arnoldi_basis(fmpt_op* op, int cp, int64_t n, int64_t nr, int G, int M, int ldh, double* V,
                  double* z, double* part, double* partM, double* coef, DevBuf& Hdev,
                  const GsWork* gs) {
  fmpt_handle* h = op->h;
  cudaStream_t st = h->stream;
  auto record = [&]() -> int {
    FMPT_CUDA(h, cudaMemsetAsync(Hdev.p, 0, Hdev.bytes, st));
    for (int j = 0; j < M; j++) {
      double* Hcol = Hdev.d() + (size_t)2 * ldh * j;
      double* vj = V + (int64_t)j * nr;
      FMPT_TRY(fmpt_op_apply(op, vj, z));
      if (gs) {
        FMPT_CUDA(h, cudaMemsetAsync(gs->bar, 0, 2 * sizeof(int), st));
        CoopBar bar{gs->bar, gs->bar + 1, gs->status, gs->wait_ns, gs->hold};
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(G);
        cfg.blockDim = dim3(KT);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        FMPT_CUDA(h, cudaLaunchKernelEx(&cfg, gs_kernel_for(G), cp, n, j, (const double*)V, nr,
                                        z, partM, gs->partB, part, Hcol, vj + nr, bar, EPB_A));
        FMPT_LAUNCHED(h);
        continue;
      }
      for (int pass = 0; pass < 2; pass++) {
        multidot_partial<<<G, KT, 0, st>>>(cp, n, j + 1, V, nr, z, partM, nullptr, EPB_A);
        FMPT_LAUNCHED(h);
        multidot_finalize<<<1, KT, 0, st>>>(j + 1, G, partM, coef, Hcol);
        FMPT_LAUNCHED(h);
        multi_axpy_sub<<<G, KT, 0, st>>>(cp, n, j + 1, V, nr, coef, z, part, nullptr, EPB_A);
        FMPT_LAUNCHED(h);
      }
      arnoldi_normalize<<<G, KT, 0, st>>>(nr, z, part, G, Hcol, j, vj + nr, EPB_A);
      FMPT_LAUNCHED(h);
    }
    return FMPT_OK;
  };
  cudaStreamCaptureStatus cap0 = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap0) != cudaSuccess) {
    cudaGetLastError();
    return record();
  }
  if (!h->graphs || cap0 != cudaStreamCaptureStatusNone) return record();
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return record();
  }
  const int rs = record();
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &graph);
  if (rs != FMPT_OK || ce != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return record();
  }
  char key[96];
  std::snprintf(key, sizeof(key), "k%d p%d c%d u%d q%zu M%d g%d", op->kind, op->precision, cp,
                op->u1 ? 1 : 0, op->proj.size(), M, gs ? 1 : 0);
  cudaGraphExec_t& ex = h->arnoldi_exec[key];
  bool ready = false;
  if (ex) {
    cudaGraphExecUpdateResultInfo ri;
    if (cudaGraphExecUpdate(ex, graph, &ri) == cudaSuccess) {
      ready = true;
    } else {
      cudaGetLastError();
      cudaGraphExecDestroy(ex);
      ex = nullptr;
    }
  }
  if (!ready && cudaGraphInstantiate(&ex, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    ex = nullptr;
  }
  cudaGraphDestroy(graph);
  if (!ex || cudaGraphLaunch(ex, st) != cudaSuccess) {
    cudaGetLastError();
    return record();
  }
  h->graph_launches++;
  return FMPT_OK;
}

}  // namespace fmpt

using namespace fmpt;

extern "C" {

int fmpt_eigsolve(fmpt_op* op, const double* x0, int num, int krylovdim, int maxiter, double tol,
                  int which, double* evals, double* evecs, double* resid, int* nconv,
                  int* napply) {
  if (!op) return FMPT_ERR_ARG;
  fmpt_handle* h = op->h;
  if (!x0 || !evals || !evecs) return set_error(h, FMPT_ERR_ARG, "eigsolve: null pointer");
  if (num < 1 || krylovdim < 2 || krylovdim > 256 || maxiter < 1 || !(tol >= 0.0) ||
      (which != 0 && which != 1))
    return set_error(h, FMPT_ERR_ARG, "eigsolve: bad num/krylovdim/maxiter/tol/which");
  return eigsolve_impl(op, x0, num, krylovdim, maxiter, tol, which, evals, evecs, resid, nconv,
                       napply);
}

int fmpt_op_set_projectors(fmpt_op* op, int nproj, const double* const* p) {
  if (!op) return FMPT_ERR_ARG;
  fmpt_handle* h = op->h;
  if (nproj < 0 || (nproj > 0 && !p))
    return set_error(h, FMPT_ERR_ARG, "set_projectors: bad projector list");
  for (int i = 0; i < nproj; i++)
    if (!p[i]) return set_error(h, FMPT_ERR_ARG, "set_projectors: null projector %d", i);
  if (nproj > 0 && !op->proj_part) {
    const int G = grid_for(h, op->n);
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, 2 * (size_t)G * sizeof(double), h->stream);
    if (e != cudaSuccess)
      return set_error(h, e == cudaErrorMemoryAllocation ? FMPT_ERR_NOMEM : FMPT_ERR_CUDA,
                       "set_projectors: %s", cudaGetErrorString(e));
    op->proj_part = static_cast<double*>(q);
    op->proj_G = G;
  }
  op->proj.assign(p, p + nproj);
  return FMPT_OK;
}

int fmpt_lanczos_ground(fmpt_op* op, const double* x0, int kmax, double btol, int reorth,
                        double* eigval, double* xout, int* info, int* niter) {
  if (!op) return FMPT_ERR_ARG;
  fmpt_handle* h = op->h;
  if (!x0 || !xout || !eigval) return set_error(h, FMPT_ERR_ARG, "lanczos: null pointer");
  if (kmax < 1 || kmax > 128) return set_error(h, FMPT_ERR_ARG, "lanczos: kmax must be 1..128");
  if (op->u1 && h->graphs) {
    bool fallback = false;
    const int st = lanczos_graph(op, x0, kmax, btol, reorth, eigval, xout, info, niter, &fallback);
    if (!fallback) return st;
  }
  const int cp = op->dtype == FMPT_C128;
  const int64_t n = op->n * (cp ? 2 : 1);   // real view of the vector
  const int G = grid_for(h, n);
  DevBuf Vb, Yb, scal, partA, partB, partM, coef;
  FMPT_TRY(Vb.alloc(h, (size_t)(kmax + 1) * n * sizeof(double)));
  FMPT_TRY(Yb.alloc(h, (size_t)n * sizeof(double)));
  // scal: [0] vm, [1..kmax] alpha, [kmax+1 .. 2kmax] beta, [2kmax+1] eval, then evec (kmax)
  FMPT_TRY(scal.alloc(h, (size_t)(3 * kmax + 8) * sizeof(double)));
  FMPT_TRY(partA.alloc(h, (size_t)G * sizeof(double)));
  FMPT_TRY(partB.alloc(h, (size_t)G * sizeof(double)));
  FMPT_TRY(partM.alloc(h, (size_t)G * (kmax + 1) * 2 * sizeof(double)));
  FMPT_TRY(coef.alloc(h, (size_t)(kmax + 1) * 2 * sizeof(double)));
  FMPT_TRY(ensure_pinned(h, 4));
  double* V = Vb.d();
  double* y = Yb.d();
  double* s_vm = scal.d();
  double* s_alpha = scal.d() + 1;
  double* s_beta = scal.d() + 1 + kmax;
  double* s_eval = scal.d() + 1 + 2 * kmax;
  double* s_evec = scal.d() + 2 + 2 * kmax;
  auto V_ = [&](int i) { return V + (int64_t)i * n; };

  // reorthogonalise y against V_0..V_{j-1} (classical Gram-Schmidt, one pass)
  auto reorthogonalise = [&](int j) -> int {
    multidot_partial<<<G, KT, 0, h->stream>>>(0, n, j, V, n, y, partM.d());
    FMPT_LAUNCHED(h);
    multidot_finalize<<<1, KT, 0, h->stream>>>(j, G, partM.d(), coef.d(), nullptr);
    FMPT_LAUNCHED(h);
    multi_axpy_sub<<<G, KT, 0, h->stream>>>(0, n, j, V, n, coef.d(), y, partB.d());
    FMPT_LAUNCHED(h);
    return FMPT_OK;
  };

  // ---- lanczos_make_first_step (simple_lanczos.jl:27-42)
  rdot_partial<<<G, KT, 0, h->stream>>>(n, x0, x0, partA.d());
  FMPT_LAUNCHED(h);
  normalize_from_parts<<<G, KT, 0, h->stream>>>(n, x0, V_(0), partA.d(), G, s_vm);
  FMPT_LAUNCHED(h);
  FMPT_TRY(fmpt_op_apply(op, V_(0), y));
  rdot_partial<<<G, KT, 0, h->stream>>>(n, V_(0), y, partA.d());
  FMPT_LAUNCHED(h);
  lanczos_axpy<<<G, KT, 0, h->stream>>>(n, y, V_(0), nullptr, partA.d(), G, nullptr, s_alpha,
                                        partB.d());
  FMPT_LAUNCHED(h);
  if (reorth) FMPT_TRY(reorthogonalise(1));
  lanczos_scale<<<G, KT, 0, h->stream>>>(n, y, partB.d(), G, s_beta);
  FMPT_LAUNCHED(h);
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, s_beta, sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  double b = h->pinned[0];
  int k = 1;
  int inf = 0;
  if (!std::isfinite(b)) return set_error(h, FMPT_ERR_NONFINITE, "lanczos: beta is not finite");
  if (b < btol) {
    // converged after the first step: Rayleigh quotient and the start vector
    FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, s_alpha, sizeof(double), cudaMemcpyDeviceToHost,
                                 h->stream));
    FMPT_CUDA(h, cudaMemcpyAsync(xout, V_(0), n * sizeof(double), cudaMemcpyDeviceToDevice,
                                 h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
    *eigval = h->pinned[0];
    if (info) *info = 0;
    if (niter) *niter = 1;
    return FMPT_OK;
  }
  // y holds q_1 (normalised); move it into V_1
  FMPT_CUDA(h, cudaMemcpyAsync(V_(1), y, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  bool converged = false;
  while (k < kmax) {
    // lanczos_make_step(A, V[k-1], V[k], beta[k-1])  (simple_lanczos.jl:49-68)
    FMPT_TRY(fmpt_op_apply(op, V_(k), y));
    rdot_partial<<<G, KT, 0, h->stream>>>(n, V_(k), y, partA.d());
    FMPT_LAUNCHED(h);
    lanczos_axpy<<<G, KT, 0, h->stream>>>(n, y, V_(k), V_(k - 1), partA.d(), G, s_beta + (k - 1),
                                          s_alpha + k, partB.d());
    FMPT_LAUNCHED(h);
    if (reorth) FMPT_TRY(reorthogonalise(k + 1));
    lanczos_scale<<<G, KT, 0, h->stream>>>(n, y, partB.d(), G, s_beta + k);
    FMPT_LAUNCHED(h);
    FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, s_beta + k, sizeof(double), cudaMemcpyDeviceToHost,
                                 h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
    b = h->pinned[0];
    k += 1;
    if (!std::isfinite(b)) return set_error(h, FMPT_ERR_NONFINITE, "lanczos: beta is not finite");
    if (b < btol) { converged = true; break; }
    if (k < kmax)
      FMPT_CUDA(h, cudaMemcpyAsync(V_(k), y, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                   h->stream));
  }
  if (!converged) inf = -1;
  // eigen(Symmetric(T[1:k,1:k])) on the device, lowest pair (find_lanczos "SR")
  tridiag_lowest<<<1, 1, 0, h->stream>>>(k, s_alpha, s_beta, s_eval, s_evec);
  FMPT_LAUNCHED(h);
  combine_basis<<<G, KT, 0, h->stream>>>(0, n, k, V, n, s_evec, 1, 1.0, 1, xout);
  FMPT_LAUNCHED(h);
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, s_eval, sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  *eigval = h->pinned[0];
  if (!prec_is_f64(op->precision)) FMPT_TRY(op_tc_check(op));
  if (op->u1) FMPT_TRY(gp_check_status(op->h));
  if (info) *info = inf;
  if (niter) *niter = k;
  return FMPT_OK;
}

int fmpt_exponentiate(fmpt_op* op, double t_re, double t_im, const double* x, double* xout,
                      int krylovdim, double tol, int* info) {
  if (!op) return FMPT_ERR_ARG;
  fmpt_handle* h = op->h;
  if (!x || !xout) return set_error(h, FMPT_ERR_ARG, "exponentiate: null pointer");
  if (krylovdim < 1 || krylovdim > 31)
    return set_error(h, FMPT_ERR_ARG, "exponentiate: krylovdim must be 1..31");
  const int cp = op->dtype == FMPT_C128;
  if (!cp && t_im != 0.0)
    return set_error(h, FMPT_ERR_ARG, "exponentiate: complex time step needs dtype C128");
  const int64_t n = op->n;                     // elements (complex for C128)
  const int64_t nr = n * (cp ? 2 : 1);         // real view
  const int G = grid_for(h, nr);
  const int Ga = arnoldi_grid(h, n);           // grid of the orthogonalisation kernels
  // the Krylov space cannot be larger than the vector space
  const int M = (int)std::min<int64_t>(krylovdim, n);
  const int ldh = M + 1;
  DevBuf Vb, zb, part, partM, coef, Hdev, Ed, nrm, acc;
  FMPT_TRY(Vb.alloc(h, (size_t)(M + 1) * nr * sizeof(double)));
  FMPT_TRY(zb.alloc(h, (size_t)nr * sizeof(double)));
  FMPT_TRY(part.alloc(h, (size_t)std::max(G, Ga) * sizeof(double)));
  FMPT_TRY(partM.alloc(h, (size_t)Ga * (M + 1) * 2 * sizeof(double)));
  FMPT_TRY(coef.alloc(h, (size_t)(M + 1) * 2 * sizeof(double)));
  FMPT_TRY(Hdev.alloc(h, (size_t)ldh * M * 2 * sizeof(double)));
  FMPT_TRY(Ed.alloc(h, (size_t)M * 2 * sizeof(double)));
  std::vector<double> colbuf((size_t)2 * M);
  FMPT_TRY(nrm.alloc(h, 2 * sizeof(double)));
  FMPT_TRY(acc.alloc(h, 2 * sizeof(double)));
  FMPT_TRY(ensure_pinned(h, (size_t)ldh * M * 2 + 8));
  DevBuf gsbuf;
  GsWork gsw{};
  const GsWork* gs = nullptr;
  FMPT_TRY(gs_setup(op, Ga, M, gsbuf, gsw, &gs));
  double* V = Vb.d();
  auto V_ = [&](int i) { return V + (int64_t)i * nr; };
  const double tabs = std::hypot(t_re, t_im);
  if (tabs == 0.0) {
    FMPT_CUDA(h, cudaMemcpyAsync(xout, x, nr * sizeof(double), cudaMemcpyDeviceToDevice,
                                 h->stream));
    if (info) *info = 0;
    return FMPT_OK;
  }
  const double sg_r = t_re / tabs, sg_i = t_im / tabs;
  // w = x / ||x||, acc = ||x|| (the running norm stays on the device)
  rdot_partial<<<G, KT, 0, h->stream>>>(nr, x, x, part.d());
  FMPT_LAUNCHED(h);
  normalize_from_parts<<<G, KT, 0, h->stream>>>(nr, x, V_(0), part.d(), G, acc.d());
  FMPT_LAUNCHED(h);
  double tau_done = 0.0, dtau = tabs;
  int steps = 0;
  std::vector<double> Hh((size_t)ldh * M * 2);
  std::vector<double> Hs;
  while (tau_done < tabs * (1.0 - 1e-15)) {
    if (++steps > 1000) return set_error(h, FMPT_ERR_NOCONV, "exponentiate: too many steps");
    // ---- Arnoldi (two-pass classical Gram-Schmidt) entirely on the device
    FMPT_TRY(arnoldi_basis(op, cp, n, nr, Ga, M, ldh, V, zb.d(), part.d(), partM.d(), coef.d(),
                           Hdev, gs));
    FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, Hdev.p, Hdev.bytes, cudaMemcpyDeviceToHost,
                                 h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
    if (gs) FMPT_TRY(gp_check_status(h));     // a fused step that gave up left H invalid
    std::copy(h->pinned, h->pinned + Hh.size(), Hh.begin());
    for (double v : Hh)
      if (!std::isfinite(v)) return set_error(h, FMPT_ERR_NONFINITE, "exponentiate: NaN");
    // happy breakdown: the first zero subdiagonal closes the Krylov space
    int m = M;
    bool happy = M == n;
    for (int j = 0; j < M; j++)
      if (Hh[2 * (j + 1 + (size_t)ldh * j)] == 0.0) { m = j + 1; happy = true; break; }
    dtau = happy ? (tabs - tau_done) : std::min(dtau, tabs - tau_done);
    Hs.assign((size_t)m * m * 2, 0.0);
    std::vector<cplx> col;
    for (int tries = 0; tries < 200; tries++) {
      const double fr = sg_r * dtau, fi = sg_i * dtau;
      for (int c = 0; c < m; c++)
        for (int r = 0; r < m; r++) {
          const double hr = Hh[2 * (r + (size_t)ldh * c)], hi = Hh[2 * (r + (size_t)ldh * c) + 1];
          Hs[2 * (r + (size_t)m * c)] = fr * hr - fi * hi;
          Hs[2 * (r + (size_t)m * c) + 1] = fr * hi + fi * hr;
        }
      host_expm_col(m, Hs.data(), col);
      if (happy) break;
      // error estimate |h_{m+1,m} dtau [exp(dtau H)]_{m,1}|
      const double hlast = Hh[2 * (m + (size_t)ldh * (m - 1))];
      const double err = std::abs(hlast * dtau) * std::abs(col[m - 1]);
      if (err <= 0.9 * tol * dtau) break;
      dtau *= 0.5;
    }
    // pageable source: the copy has left colbuf when cudaMemcpyAsync returns
    for (int r = 0; r < m; r++) {
      colbuf[2 * r] = col[r].real();
      colbuf[2 * r + 1] = col[r].imag();
    }
    FMPT_CUDA(h, cudaMemcpyAsync(Ed.d(), colbuf.data(), (size_t)2 * m * sizeof(double),
                                 cudaMemcpyHostToDevice, h->stream));
    // w = sum_i E[i, 0] V_i, renormalised into V_0; acc *= ||w||
    combine_basis<<<G, KT, 0, h->stream>>>(cp, n, m, V, nr, Ed.d(), 2, 1.0, 0, zb.d());
    FMPT_LAUNCHED(h);
    rdot_partial<<<G, KT, 0, h->stream>>>(nr, zb.d(), zb.d(), part.d());
    FMPT_LAUNCHED(h);
    normalize_from_parts<<<G, KT, 0, h->stream>>>(nr, zb.d(), V_(0), part.d(), G, nrm.d());
    FMPT_LAUNCHED(h);
    mul_scalar<<<1, 1, 0, h->stream>>>(acc.d(), nrm.d());
    FMPT_LAUNCHED(h);
    tau_done += dtau;
    if (!happy && tau_done < tabs) dtau = std::min(2.0 * dtau, tabs - tau_done);
  }
  // xout = acc * V_0
  FMPT_CUDA(h, cudaMemcpyAsync(xout, V_(0), nr * sizeof(double), cudaMemcpyDeviceToDevice,
                               h->stream));
  scale_by<<<G, KT, 0, h->stream>>>(nr, xout, acc.d());
  FMPT_LAUNCHED(h);
  if (!prec_is_f64(op->precision)) FMPT_TRY(op_tc_check(op));
  if (op->u1 || gs) FMPT_TRY(gp_check_status(op->h));
  if (info) *info = steps;
  return FMPT_OK;
}

// exp(s_j t H) x for several s_j from ONE Krylov space of x (the quadrature
// nodes of the exponential's adjoint).  Arnoldi as in fmpt_exponentiate;
// no step-size control: err_est (host) gets max_j |h_{m+1,m} [exp(s_j t H_m)]_{m,1}|,
// the usual a-posteriori estimate relative to ||x||.
int fmpt_expm_nodes(fmpt_op* op, double t_re, double t_im, const double* x, int krylovdim,
                    int nnodes, const double* nodes, double* out, double* err_est) {
  if (!op) return FMPT_ERR_ARG;
  fmpt_handle* h = op->h;
  if (!x || !out || !nodes || nnodes < 1)
    return set_error(h, FMPT_ERR_ARG, "expm_nodes: null pointer or no nodes");
  if (krylovdim < 1 || krylovdim > 31)
    return set_error(h, FMPT_ERR_ARG, "expm_nodes: krylovdim must be 1..31");
  const int cp = op->dtype == FMPT_C128;
  if (!cp && t_im != 0.0)
    return set_error(h, FMPT_ERR_ARG, "expm_nodes: complex time needs dtype C128");
  const int64_t n = op->n;
  const int64_t nr = n * (cp ? 2 : 1);
  const int G = grid_for(h, nr);
  const int Ga = arnoldi_grid(h, n);           // grid of the orthogonalisation kernels
  const int M = (int)std::min<int64_t>(krylovdim, n);
  const int ldh = M + 1;
  DevBuf Vb, zb, part, partM, coef, Hdev, Ed, acc;
  FMPT_TRY(Vb.alloc(h, (size_t)(M + 1) * nr * sizeof(double)));
  FMPT_TRY(zb.alloc(h, (size_t)nr * sizeof(double)));
  FMPT_TRY(part.alloc(h, (size_t)std::max(G, Ga) * sizeof(double)));
  FMPT_TRY(partM.alloc(h, (size_t)Ga * (M + 1) * 2 * sizeof(double)));
  FMPT_TRY(coef.alloc(h, (size_t)(M + 1) * 2 * sizeof(double)));
  FMPT_TRY(Hdev.alloc(h, (size_t)ldh * M * 2 * sizeof(double)));
  FMPT_TRY(Ed.alloc(h, (size_t)nnodes * M * 2 * sizeof(double)));
  FMPT_TRY(acc.alloc(h, 2 * sizeof(double)));
  FMPT_TRY(ensure_pinned(h, (size_t)ldh * M * 2 + 8));
  DevBuf gsbuf;
  GsWork gsw{};
  const GsWork* gs = nullptr;
  FMPT_TRY(gs_setup(op, Ga, M, gsbuf, gsw, &gs));
  double* V = Vb.d();
  auto V_ = [&](int i) { return V + (int64_t)i * nr; };
  rdot_partial<<<G, KT, 0, h->stream>>>(nr, x, x, part.d());
  FMPT_LAUNCHED(h);
  normalize_from_parts<<<G, KT, 0, h->stream>>>(nr, x, V_(0), part.d(), G, acc.d());
  FMPT_LAUNCHED(h);
  FMPT_TRY(arnoldi_basis(op, cp, n, nr, Ga, M, ldh, V, zb.d(), part.d(), partM.d(), coef.d(),
                         Hdev, gs));
  std::vector<double> Hh((size_t)ldh * M * 2);
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, Hdev.p, Hdev.bytes, cudaMemcpyDeviceToHost, h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  if (gs) FMPT_TRY(gp_check_status(h));       // a fused step that gave up left H invalid
  std::copy(h->pinned, h->pinned + Hh.size(), Hh.begin());
  for (double v : Hh)
    if (!std::isfinite(v)) return set_error(h, FMPT_ERR_NONFINITE, "expm_nodes: NaN");
  int m = M;
  bool happy = M == n;
  for (int j = 0; j < M; j++)
    if (Hh[2 * (j + 1 + (size_t)ldh * j)] == 0.0) { m = j + 1; happy = true; break; }
  // every node's exp(s_q t H_m) e_1 on the host, uploaded in one copy (pageable source:
  // the copy has left it when cudaMemcpyAsync returns)
  std::vector<double> Hs((size_t)m * m * 2), cols((size_t)nnodes * m * 2);
  std::vector<cplx> col;
  double e = 0.0;
  const double hlast = happy ? 0.0 : std::abs(Hh[2 * (m + (size_t)ldh * (m - 1))]);
  for (int q = 0; q < nnodes; q++) {
    const double fr = nodes[q] * t_re, fi = nodes[q] * t_im;
    for (int c = 0; c < m; c++)
      for (int r = 0; r < m; r++) {
        const double hr = Hh[2 * (r + (size_t)ldh * c)], hi = Hh[2 * (r + (size_t)ldh * c) + 1];
        Hs[2 * (r + (size_t)m * c)] = fr * hr - fi * hi;
        Hs[2 * (r + (size_t)m * c) + 1] = fr * hi + fi * hr;
      }
    host_expm_col(m, Hs.data(), col);
    for (int r = 0; r < m; r++) {
      cols[2 * (r + (size_t)m * q)] = col[r].real();
      cols[2 * (r + (size_t)m * q) + 1] = col[r].imag();
    }
    if (!happy) e = std::max(e, hlast * std::abs(col[m - 1]));
  }
  FMPT_CUDA(h, cudaMemcpyAsync(Ed.d(), cols.data(), cols.size() * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
  for (int q = 0; q < nnodes; q++) {
    double* oq = out + (int64_t)q * nr;
    combine_basis<<<G, KT, 0, h->stream>>>(cp, n, m, V, nr, Ed.d() + (size_t)2 * m * q, 2, 1.0,
                                           0, oq);
    FMPT_LAUNCHED(h);
    scale_by<<<G, KT, 0, h->stream>>>(nr, oq, acc.d());
    FMPT_LAUNCHED(h);
  }
  if (err_est) *err_est = e;
  if (!prec_is_f64(op->precision)) FMPT_TRY(op_tc_check(op));
  if (op->u1 || gs) FMPT_TRY(gp_check_status(op->h));
  return FMPT_OK;
}

}  // extern "C"
