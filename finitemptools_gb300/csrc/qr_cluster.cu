// Thin Householder QR of a small panel on one thread-block cluster (the gauge moves of the
// one-site sweeps: leftorth! / rightorth, e.g. 128 x 64 complex at D = 64).
//
// cuSOLVER's geqrf + ungqr take about 2 ms on such a panel: a chain of small launches,
// each bound by one SM's FP64 rate (about 2 DFMA per clock).  Here the n columns are dealt
// round-robin to the CL CTAs of one cluster (column j lives in the shared memory of CTA
// j % CL), so every Householder update runs on CL SMs at once:
//   for k = 0 .. n-1:  the owner of column k forms the reflector (v_k, tau_k) from it
//                      (LAPACK's zlarfg / dlarfg convention: beta = -sign(Re a) |(a, x)|,
//                      tau = (beta - a) / beta, v = x / (a - beta), R(k, k) = beta real);
//                      cluster barrier; every CTA reads v_k and tau_k from the owner's
//                      shared memory (distributed shared memory) and applies
//                      H_k^H = I - conj(tau_k) v_k v_k^H to its own columns j > k;
//   Q = H_0 H_1 .. H_{n-1} [I; 0] as LAPACK's zung2r does it, backwards over k, each CTA
//   on its own columns of Q -- the reflectors no longer change, so this half needs no
//   barrier at all.
// The conventions are LAPACK's, so Q and R match geqrf/ungqr to rounding (real diagonal of
// R; a zero column gives tau = 0, H = I).  Barriers are the cluster's hardware barrier.
#include <cooperative_groups.h>

#include "internal.h"

namespace cg = cooperative_groups;

namespace fmpt {
namespace {

constexpr int QT = 256;                  // threads per CTA
constexpr int QR_MAX_LOCAL = 4096;       // m * (columns per CTA) held per CTA (64 KB a plane pair)

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum over the CTA of v (every thread gets it); red holds QT / 32 doubles
__device__ double cta_sum(double v, double* red) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int w = 0; w < QT / 32; w++) s += red[w];
  return s;
}

// Smem layout (doubles): A re/im [nloc][m] (own columns, column-major), Q re/im [nloc][m],
// v re/im [m] (the current reflector, local copy), tau re/im [n] (written by the owner of
// each column), red [QT / 32], scal [4].
template <int CL>
__global__ void __launch_bounds__(QT) qr_cluster_kernel(int cplx, int m, int n,
                                                        const double* __restrict__ M,
                                                        int64_t planeM, double* __restrict__ Q,
                                                        int64_t planeQ, double* __restrict__ R,
                                                        int64_t planeR, int nloc) {
  extern __shared__ double sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  double* Ar = sm;
  double* Ai = Ar + (size_t)nloc * m;
  double* Qr = Ai + (size_t)nloc * m;
  double* Qi = Qr + (size_t)nloc * m;
  double* vr = Qi + (size_t)nloc * m;
  double* vi = vr + m;
  double* tr = vi + m;
  double* ti = tr + n;
  double* red = ti + n;
  double* scal = red + QT / 32;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int mine = (n - rank + CL - 1) / CL;     // own columns j = rank + CL c, c < mine
  // own columns of M into shared memory
  for (int e = tid; e < mine * m; e += QT) {
    const int c = e / m, i = e - c * m;
    const int64_t g = (int64_t)(rank + CL * c) * m + i;
    Ar[(size_t)c * m + i] = M[g];
    Ai[(size_t)c * m + i] = cplx ? M[planeM + g] : 0.0;
  }
  __syncthreads();
  cluster.sync();
  // ---------------------------------------------------------------- factorisation
  for (int k = 0; k < n; k++) {
    const int owner = k % CL, lc = k / CL;
    if (rank == owner) {
      double* cr = Ar + (size_t)lc * m;
      double* ci = Ai + (size_t)lc * m;
      double s = 0.0;
      for (int i = k + 1 + tid; i < m; i += QT) s += cr[i] * cr[i] + ci[i] * ci[i];
      const double xnorm = sqrt(cta_sum(s, red));
      const double ar = cr[k], ai = ci[k];
      double taur = 0.0, taui = 0.0, beta = ar, sr = 0.0, si = 0.0;
      const bool trivial = xnorm == 0.0 && ai == 0.0;
      if (!trivial) {
        const double nrm = sqrt(ar * ar + ai * ai + xnorm * xnorm);
        beta = ar >= 0.0 ? -nrm : nrm;                 // -sign(|(a, x)|, Re a)
        taur = (beta - ar) / beta;
        taui = -ai / beta;
        // 1 / (a - beta), Smith's division
        const double dr = ar - beta, di = ai;
        if (fabs(dr) >= fabs(di)) {
          const double t = di / dr, den = dr + di * t;
          sr = 1.0 / den;
          si = -t / den;
        } else {
          const double t = dr / di, den = di + dr * t;
          sr = t / den;
          si = -1.0 / den;
        }
      }
      if (!trivial)
        for (int i = k + 1 + tid; i < m; i += QT) {
          const double xr = cr[i], xi = ci[i];
          cr[i] = xr * sr - xi * si;
          ci[i] = xr * si + xi * sr;
        }
      __syncthreads();
      if (tid == 0) {
        cr[k] = beta;
        ci[k] = 0.0;
        tr[k] = taur;
        ti[k] = taui;
      }
    }
    cluster.sync();                                  // v_k and tau_k are published
    // columns of this CTA after k
    int c0 = (k + 1 - rank + CL - 1) / CL;
    if (k + 1 - rank <= 0) c0 = 0;
    if (c0 >= mine) continue;
    const double* rvr = cluster.map_shared_rank(Ar + (size_t)lc * m, owner);
    const double* rvi = cluster.map_shared_rank(Ai + (size_t)lc * m, owner);
    const double* rtr = cluster.map_shared_rank(tr, owner);
    const double* rti = cluster.map_shared_rank(ti, owner);
    for (int i = k + 1 + tid; i < m; i += QT) {
      vr[i] = rvr[i];
      vi[i] = rvi[i];
    }
    if (tid == 0) {
      vr[k] = 1.0;
      vi[k] = 0.0;
      scal[0] = rtr[k];
      scal[1] = rti[k];
    }
    __syncthreads();
    // H^H = I - conj(tau) v v^H on column j: w = v^H a_j, a_j -= conj(tau) w v
    const double ctr = scal[0], cti = -scal[1];
    if (ctr != 0.0 || cti != 0.0) {
      for (int c = c0 + wid; c < mine; c += QT / 32) {
        double* cr = Ar + (size_t)c * m;
        double* ci = Ai + (size_t)c * m;
        double wr = 0.0, wi = 0.0;
        for (int i = k + lane; i < m; i += 32) {
          wr += vr[i] * cr[i] + vi[i] * ci[i];
          wi += vr[i] * ci[i] - vi[i] * cr[i];
        }
        wr = warp_sum_d(wr);
        wi = warp_sum_d(wi);
        const double fr = ctr * wr - cti * wi, fi = ctr * wi + cti * wr;   // conj(tau) w
        for (int i = k + lane; i < m; i += 32) {
          const double pr = vr[i], pi = vi[i];
          cr[i] -= fr * pr - fi * pi;
          ci[i] -= fr * pi + fi * pr;
        }
      }
    }
    __syncthreads();
  }
  // R = the upper triangle of the factored columns (n x n, ld n), zeros below
  for (int e = tid; e < mine * n; e += QT) {
    const int c = e / n, i = e - c * n;
    const int j = rank + CL * c;
    const int64_t g = (int64_t)j * n + i;
    R[g] = i <= j ? Ar[(size_t)c * m + i] : 0.0;
    if (cplx) R[planeR + g] = i <= j ? Ai[(size_t)c * m + i] : 0.0;
  }
  cluster.sync();      // every reflector final before anyone reads them below
  // ---------------------------------------------------------------- Q (zung2r)
  for (int e = tid; e < mine * m; e += QT) {
    Qr[e] = 0.0;
    Qi[e] = 0.0;
  }
  __syncthreads();
  for (int k = n - 1; k >= 0; k--) {
    const int owner = k % CL, lc = k / CL;
    const double* rvr = cluster.map_shared_rank(Ar + (size_t)lc * m, owner);
    const double* rvi = cluster.map_shared_rank(Ai + (size_t)lc * m, owner);
    const double* rtr = cluster.map_shared_rank(tr, owner);
    const double* rti = cluster.map_shared_rank(ti, owner);
    for (int i = k + 1 + tid; i < m; i += QT) {
      vr[i] = rvr[i];
      vi[i] = rvi[i];
    }
    if (tid == 0) {
      vr[k] = 1.0;
      vi[k] = 0.0;
      scal[0] = rtr[k];
      scal[1] = rti[k];
    }
    __syncthreads();
    const double tur = scal[0], tui = scal[1];
    // H_k = I - tau v v^H on the own columns j > k (rows k .. m-1)
    int c0 = (k + 1 - rank + CL - 1) / CL;
    if (k + 1 - rank <= 0) c0 = 0;
    if (tur != 0.0 || tui != 0.0)
      for (int c = c0 + wid; c < mine; c += QT / 32) {
        double* qr = Qr + (size_t)c * m;
        double* qi = Qi + (size_t)c * m;
        double wr = 0.0, wi = 0.0;
        for (int i = k + lane; i < m; i += 32) {
          wr += vr[i] * qr[i] + vi[i] * qi[i];
          wi += vr[i] * qi[i] - vi[i] * qr[i];
        }
        wr = warp_sum_d(wr);
        wi = warp_sum_d(wi);
        const double fr = tur * wr - tui * wi, fi = tur * wi + tui * wr;   // tau w
        for (int i = k + lane; i < m; i += 32) {
          const double pr = vr[i], pi = vi[i];
          qr[i] -= fr * pr - fi * pi;
          qi[i] -= fr * pi + fi * pr;
        }
      }
    // column k itself: e_k - tau v (rows k .. m-1), zero above
    if (rank == owner) {
      double* qr = Qr + (size_t)lc * m;
      double* qi = Qi + (size_t)lc * m;
      for (int i = k + 1 + tid; i < m; i += QT) {
        qr[i] = -(tur * vr[i] - tui * vi[i]);
        qi[i] = -(tur * vi[i] + tui * vr[i]);
      }
      if (tid == 0) {
        qr[k] = 1.0 - tur;
        qi[k] = -tui;
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < mine * m; e += QT) {
    const int c = e / m, i = e - c * m;
    const int64_t g = (int64_t)(rank + CL * c) * m + i;
    Q[g] = Qr[e];
    if (cplx) Q[planeQ + g] = Qi[e];
  }
  cluster.sync();      // no CTA leaves while another may still read its shared memory
}

size_t qr_smem_bytes(int m, int n, int nloc) {
  return sizeof(double) * ((size_t)4 * nloc * m + 2 * (size_t)m + 2 * (size_t)n + QT / 32 + 4);
}

template <int CL>
int qr_launch(fmpt_handle* h, int cplx, int m, int n, const double* M, double* Q, double* R) {
  const int nloc = (n + CL - 1) / CL;
  const size_t smem = qr_smem_bytes(m, n, nloc);
  auto kern = qr_cluster_kernel<CL>;
  if (CL > 8) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
        cudaSuccess) {
      cudaGetLastError();
      return FMPT_ERR_UNSUPPORTED;
    }
  }
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return FMPT_ERR_UNSUPPORTED;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(QT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return FMPT_ERR_UNSUPPORTED;
  }
  FMPT_CUDA(h, cudaLaunchKernelEx(&cfg, kern, cplx, m, n, M, (int64_t)m * n, Q, (int64_t)m * n,
                                  R, (int64_t)n * n, nloc));
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

}  // namespace

// Q (m x n, ld m) and R (n x n, ld n) of M (m x n, ld m, m >= n), split-plane complex when
// cplx.  FMPT_ERR_UNSUPPORTED (nothing launched) when the panel is outside the kernel's
// range or no cluster fits; the caller then takes cuSOLVER.
int qr_small_cluster(fmpt_handle* h, int cplx, int m, int n, const double* M, double* Q,
                     double* R) {
  if (!h->cluster_qr || m < n || n < 1 || m > 1024) return FMPT_ERR_UNSUPPORTED;
  if ((int64_t)m * ((n + 15) / 16) <= QR_MAX_LOCAL) {
    const int st = qr_launch<16>(h, cplx, m, n, M, Q, R);
    if (st != FMPT_ERR_UNSUPPORTED) return st;
  }
  if ((int64_t)m * ((n + 7) / 8) <= QR_MAX_LOCAL) return qr_launch<8>(h, cplx, m, n, M, Q, R);
  return FMPT_ERR_UNSUPPORTED;
}

}  // namespace fmpt
