// Gate action of the TEBD bond evolution (circuit/apply_gates.jl:11-50):
//   y[a, p', b] = sum_p G[p', p] x[a, p, b]
// with p the fused physical index of the n sites the gate acts on (column-major
// fusion, first site fastest) and G the gate as a P x P matrix.  One thread per
// (a, b) pair: consecutive threads take consecutive a, so every load and store
// of x and y is coalesced; the gate (at most a few hundred entries for the
// gates the reference allows) is read through the read-only cache.  The work
// is a memory-bound pass over the two-site tensor; the truncated SVD that
// follows dominates the bond update.
#include <algorithm>

#include "internal.h"

namespace fmpt {
namespace {

__global__ void gate_kernel(int cplx, int Dl, int P, int64_t Dr, const double* __restrict__ G,
                            const double* __restrict__ x, double* __restrict__ y,
                            int64_t plane) {
  const int64_t tot = (int64_t)Dl * Dr;
  const int64_t pg = (int64_t)P * P;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = t % Dl, b = t / Dl;
    const int64_t base = a + (int64_t)Dl * P * b;
    for (int q = 0; q < P; q++) {
      double sr = 0.0, si = 0.0;
      for (int p = 0; p < P; p++) {
        const double gr = __ldg(G + q + (int64_t)P * p);
        const double xr = x[base + (int64_t)Dl * p];
        sr = fma(gr, xr, sr);
        if (cplx) {
          const double gi = __ldg(G + pg + q + (int64_t)P * p);
          const double xi = x[plane + base + (int64_t)Dl * p];
          sr = fma(-gi, xi, sr);
          si = fma(gr, xi, si);
          si = fma(gi, xr, si);
        }
      }
      y[base + (int64_t)Dl * q] = sr;
      if (cplx) y[plane + base + (int64_t)Dl * q] = si;
    }
  }
}

}  // namespace
}  // namespace fmpt

using namespace fmpt;

extern "C" {

int fmpt_apply_gate(fmpt_handle* h, int dtype, const double* G_host, int P, const double* x,
                    double* y, int Dl, int Dr) {
  if (!h) return FMPT_ERR_ARG;
  if (!G_host || !x || !y) return set_error(h, FMPT_ERR_ARG, "apply_gate: null pointer");
  if (P < 1 || P > 4096 || Dl < 1 || Dr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "apply_gate: bad extents");
  if (x == y) return set_error(h, FMPT_ERR_ARG, "apply_gate: out of place only");
  const int cp = dtype == FMPT_C128;
  const size_t gbytes = (size_t)P * P * sizeof(double) * (cp ? 2 : 1);
  DevBuf Gd;
  FMPT_TRY(Gd.alloc(h, gbytes));
  FMPT_CUDA(h, cudaMemcpyAsync(Gd.d(), G_host, gbytes, cudaMemcpyHostToDevice, h->stream));
  const int64_t tot = (int64_t)Dl * Dr;
  const int threads = 128;
  const int blocks =
      (int)std::max<int64_t>(1, std::min<int64_t>((tot + threads - 1) / threads, 16LL * h->sm_count));
  gate_kernel<<<blocks, threads, 0, h->stream>>>(cp, Dl, P, Dr, Gd.d(), x, y,
                                                   (int64_t)Dl * P * Dr);
  FMPT_LAUNCHED(h);
  // the gate buffer is freed stream-ordered; the host copy may be reused once
  // the launch has been queued because cudaMemcpyAsync from pageable memory
  // returns after staging
  return FMPT_OK;
}

}  // extern "C"
