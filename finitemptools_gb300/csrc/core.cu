// Handle, memory and BLAS-1 style entry points of libfmpt.
#include <cmath>
#include <cstring>

#include "internal.h"

namespace fmpt {

int DevBuf::alloc(fmpt_handle* hh, size_t nbytes) {
  release();
  h = hh;
  bytes = nbytes;
  if (nbytes == 0) return FMPT_OK;
  cudaError_t e = cudaMallocAsync(&p, nbytes, h->stream);
  if (e != cudaSuccess) {
    p = nullptr;
    return set_error(h, e == cudaErrorMemoryAllocation ? FMPT_ERR_NOMEM : FMPT_ERR_CUDA,
                     "device allocation of %zu bytes: %s", nbytes, cudaGetErrorString(e));
  }
  return FMPT_OK;
}

void DevBuf::release() {
  if (p && h) cudaFreeAsync(p, h->stream);
  p = nullptr;
  bytes = 0;
}

static cudaEvent_t pool_event(fmpt_handle* h) {
  if (!h->ev_pool.empty()) {
    cudaEvent_t e = h->ev_pool.back();
    h->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(fmpt_handle* hh, int c) : h(hh), cls(c) {
  if (!h || !h->prof) return;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return;   // no timers inside a graph capture
  b = pool_event(h);
  e = pool_event(h);
  cudaEventRecord(b, h->stream);
}

ProfScope::~ProfScope() {
  if (!b) return;
  cudaEventRecord(e, h->stream);
  h->prof_ev[cls].push_back({b, e});
}

int grow_buffer(fmpt_handle* h, void** buf, size_t* cap, size_t bytes) {
  if (*cap >= bytes && *buf) return FMPT_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(h->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return set_error(h, FMPT_ERR_UNSUPPORTED, "buffer growth during stream capture");
  }
  if (*buf) cudaFreeAsync(*buf, h->stream);
  *buf = nullptr;
  *cap = 0;
  FMPT_CUDA(h, cudaMallocAsync(buf, bytes, h->stream));
  *cap = bytes;
  return FMPT_OK;
}

int ensure_pinned(fmpt_handle* h, size_t n) {
  if (h->pinned_len >= n) return FMPT_OK;
  if (h->pinned) {
    cudaStreamSynchronize(h->stream);
    cudaFreeHost(h->pinned);
    h->pinned = nullptr;
    h->pinned_len = 0;
  }
  FMPT_CUDA(h, cudaMallocHost((void**)&h->pinned, n * sizeof(double)));
  h->pinned_len = n;
  return FMPT_OK;
}

int ensure_aux(fmpt_handle* h, int n) {
  if (h->aux_event.empty()) {
    cudaEvent_t e;
    FMPT_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->aux_event.push_back(e);
  }
  while ((int)h->aux_stream.size() < n) {
    cudaStream_t st;
    FMPT_CUDA(h, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cusolverDnHandle_t sv;
    if (cusolverDnCreate(&sv) != CUSOLVER_STATUS_SUCCESS) {
      cudaStreamDestroy(st);
      return set_error(h, FMPT_ERR_CUSOLVER, "aux stream: cusolverDnCreate failed");
    }
    cusolverDnSetStream(sv, st);
    cudaEvent_t e;
    FMPT_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->aux_stream.push_back(st);
    h->aux_solver.push_back(sv);
    h->aux_event.push_back(e);
  }
  return FMPT_OK;
}

int aux_fork(fmpt_handle* h, int n) {
  FMPT_TRY(ensure_aux(h, n));
  FMPT_CUDA(h, cudaEventRecord(h->aux_event[0], h->stream));
  for (int i = 0; i < n; i++) FMPT_CUDA(h, cudaStreamWaitEvent(h->aux_stream[i], h->aux_event[0], 0));
  return FMPT_OK;
}

int aux_join(fmpt_handle* h, int n) {
  for (int i = 0; i < n; i++) {
    FMPT_CUDA(h, cudaEventRecord(h->aux_event[1 + i], h->aux_stream[i]));
    FMPT_CUDA(h, cudaStreamWaitEvent(h->stream, h->aux_event[1 + i], 0));
  }
  return FMPT_OK;
}

namespace {

constexpr int RT = 256;       // threads per reduction block

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum; every thread gets the result
__device__ double block_sum(double v) {
  __shared__ double red[RT / 32];
  __shared__ double total;
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double w = threadIdx.x < RT / 32 ? red[threadIdx.x] : 0.0;
    w = warp_sum(w);
    if (threadIdx.x == 0) total = w;
  }
  __syncthreads();
  double r = total;
  __syncthreads();
  return r;
}

// partial[blockIdx] = sum over a grid-stride slice of conj(x) y (re, im)
__global__ void dot_partial(int cplx, int64_t n, const double* __restrict__ x,
                            const double* __restrict__ y, double* __restrict__ part) {
  double sr = 0.0, si = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * RT + threadIdx.x; i < n; i += (int64_t)gridDim.x * RT) {
    double xr = x[i], yr = y[i];
    sr = fma(xr, yr, sr);
    if (cplx) {
      double xi = x[n + i], yi = y[n + i];
      sr = fma(xi, yi, sr);
      si = fma(xr, yi, si);
      si = fma(-xi, yr, si);
    }
  }
  sr = block_sum(sr);
  if (cplx) si = block_sum(si);
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = sr; part[2 * blockIdx.x + 1] = si; }
}

__global__ void sum_partials(int nparts, const double* __restrict__ part, double* out, int sqrt_re) {
  double sr = 0.0, si = 0.0;
  for (int i = threadIdx.x; i < nparts; i += RT) { sr += part[2 * i]; si += part[2 * i + 1]; }
  sr = block_sum(sr);
  si = block_sum(si);
  if (threadIdx.x == 0) { out[0] = sqrt_re ? sqrt(sr) : sr; out[1] = si; }
}

__global__ void axpy_kernel(int cplx, int64_t n, double ar, double ai, const double* __restrict__ x,
                            double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (cplx) {
      double xr = x[i], xi = x[n + i];
      y[i] += ar * xr - ai * xi;
      y[n + i] += ar * xi + ai * xr;
    } else {
      y[i] = fma(ar, x[i], y[i]);
    }
  }
}

__global__ void scal_kernel(int cplx, int64_t n, double ar, double ai, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (cplx) {
      double xr = x[i], xi = x[n + i];
      x[i] = ar * xr - ai * xi;
      x[n + i] = ar * xi + ai * xr;
    } else {
      x[i] *= ar;
    }
  }
}

__global__ void scale_dim_kernel(int cplx, int side, int m, int n, const double* __restrict__ s,
                                 double* __restrict__ M) {
  int64_t tot = (int64_t)m * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % m), j = (int)(t / m);
    double f = side == 0 ? s[i] : s[j];
    M[t] *= f;
    if (cplx) M[tot + t] *= f;
  }
}

int reduction_grid(fmpt_handle* h, int64_t n) {
  int64_t g = (n + RT - 1) / RT;
  int64_t cap = (int64_t)h->sm_count * 4;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int elementwise_grid(fmpt_handle* h, int64_t n) {
  int64_t g = (n + 255) / 256;
  int64_t cap = (int64_t)h->sm_count * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

int vec_dot_dev(fmpt_handle* h, int cplx, int64_t n, const double* x, const double* y,
                double* out_dev) {
  int G = reduction_grid(h, n);
  DevBuf part;
  FMPT_TRY(part.alloc(h, sizeof(double) * 2 * G));
  dot_partial<<<G, RT, 0, h->stream>>>(cplx, n, x, y, part.d());
  FMPT_LAUNCHED(h);
  sum_partials<<<1, RT, 0, h->stream>>>(G, part.d(), out_dev, 0);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int vec_nrm2_dev(fmpt_handle* h, int cplx, int64_t n, const double* x, double* out_dev) {
  int G = reduction_grid(h, n);
  DevBuf part;
  FMPT_TRY(part.alloc(h, sizeof(double) * 2 * G));
  // ||x||^2 = Re <x, x>; for split planes that is the real dot over 2n values
  dot_partial<<<G, RT, 0, h->stream>>>(0, cplx ? 2 * n : n, x, x, part.d());
  FMPT_LAUNCHED(h);
  sum_partials<<<1, RT, 0, h->stream>>>(G, part.d(), out_dev, 1);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

}  // namespace fmpt

using namespace fmpt;

extern "C" {

int fmpt_version(void) { return 1; }

const char* fmpt_status_string(int s) {
  switch (s) {
    case FMPT_OK: return "ok";
    case FMPT_ERR_ARG: return "invalid argument";
    case FMPT_ERR_SHAPE: return "dimension mismatch";
    case FMPT_ERR_CUDA: return "CUDA error";
    case FMPT_ERR_CUSOLVER: return "cuSOLVER error";
    case FMPT_ERR_TIMEOUT: return "device wait timed out";
    case FMPT_ERR_NONFINITE: return "non-finite value";
    case FMPT_ERR_NOMEM: return "out of device memory";
    case FMPT_ERR_UNSUPPORTED: return "unsupported";
    case FMPT_ERR_NOCONV: return "not converged";
    default: return "unknown status";
  }
}

int fmpt_create(int device, fmpt_handle** out) {
  if (!out) return FMPT_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return FMPT_ERR_CUDA;
  if (device < 0 || device >= ndev) return FMPT_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return FMPT_ERR_CUDA;
  fmpt_handle* h = new fmpt_handle();
  h->device = device;
  cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return FMPT_ERR_CUDA;
  }
  h->stream = h->own_stream;
  // keep freed pool memory cached: the solvers allocate the same sizes every step
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (cusolverDnCreate(&h->solver) != CUSOLVER_STATUS_SUCCESS) {
    cudaStreamDestroy(h->own_stream);
    delete h;
    return FMPT_ERR_CUSOLVER;
  }
  cusolverDnSetStream(h->solver, h->stream);
  *out = h;
  return FMPT_OK;
}

int fmpt_profile_enable(fmpt_handle* h, int on) {
  if (!h) return FMPT_ERR_ARG;
  h->prof = on != 0;
  return FMPT_OK;
}

int fmpt_profile_read(fmpt_handle* h, int cls, int64_t* launches, double* total_ms) {
  if (!h || cls < 0 || cls >= FMPT_K_COUNT) return FMPT_ERR_ARG;
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  double tot = 0.0;
  for (auto& pr : h->prof_ev[cls]) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pr.first, pr.second);
    tot += ms;
    h->ev_pool.push_back(pr.first);
    h->ev_pool.push_back(pr.second);
  }
  if (launches) *launches = (int64_t)h->prof_ev[cls].size();
  if (total_ms) *total_ms = tot;
  h->prof_ev[cls].clear();
  return FMPT_OK;
}

int fmpt_destroy(fmpt_handle* h) {
  if (!h) return FMPT_OK;
  cudaStreamSynchronize(h->stream);
  for (auto& v : h->prof_ev)
    for (auto& pr : v) { h->ev_pool.push_back(pr.first); h->ev_pool.push_back(pr.second); }
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  if (h->solver) cusolverDnDestroy(h->solver);
  for (auto sv : h->aux_solver) cusolverDnDestroy(sv);
  for (auto st : h->aux_stream) cudaStreamDestroy(st);
  for (auto ev : h->aux_event) cudaEventDestroy(ev);
  if (h->lanczos_exec) cudaGraphExecDestroy(h->lanczos_exec);
  for (auto& kv : h->arnoldi_exec) cudaGraphExecDestroy(kv.second);
  if (h->gemm_ws) cudaFree(h->gemm_ws);
  if (h->gemm_cnt) cudaFree(h->gemm_cnt);
  if (h->tc_ws) cudaFree(h->tc_ws);
  if (h->oz_ws) cudaFree(h->oz_ws);
  if (h->gstatus) cudaFree(h->gstatus);
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return FMPT_OK;
}

const char* fmpt_last_error(fmpt_handle* h) { return h ? h->err.c_str() : "null handle"; }

uint64_t fmpt_graph_launch_count(fmpt_handle* h) { return h ? h->graph_launches : 0; }

int fmpt_set_tuning(fmpt_handle* h, int mode) {
  if (!h) return FMPT_ERR_ARG;
  if (mode < 0 || mode > 4)
    return fmpt::set_error(h, FMPT_ERR_ARG, "tuning mode must be 0, 1, 2, 3 or 4");
  h->tune_mode = mode;
  return FMPT_OK;
}

int fmpt_tuning_info(fmpt_handle* h, int* entries, int64_t* timed) {
  if (!h) return FMPT_ERR_ARG;
  if (entries) *entries = (int)h->tune_cache.size();
  if (timed) *timed = (int64_t)h->tune_runs;
  return FMPT_OK;
}

int fmpt_set_svd_method(fmpt_handle* h, int method) {
  if (!h) return FMPT_ERR_ARG;
  if (method < 0 || method > 2) return set_error(h, FMPT_ERR_ARG, "svd method must be 0, 1 or 2");
  h->svd_method = method;
  return FMPT_OK;
}

int fmpt_set_tc_tile(fmpt_handle* h, int mode) {
  if (!h) return FMPT_ERR_ARG;
  if (mode < 0 || mode > 1) return set_error(h, FMPT_ERR_ARG, "tc tile mode must be 0 or 1");
  h->tc_tile = mode;
  return FMPT_OK;
}

int fmpt_set_f64_engine(fmpt_handle* h, int mode) {
  if (!h) return FMPT_ERR_ARG;
  if (mode < 0 || mode > 1) return set_error(h, FMPT_ERR_ARG, "f64 engine mode must be 0 or 1");
  h->f64_tc = mode;
  return FMPT_OK;
}

int fmpt_set_wait_test(fmpt_handle* h, int64_t timeout_ns, int hold) {
  if (!h) return FMPT_ERR_ARG;
  if (timeout_ns < 0 || timeout_ns > 10000000000LL || hold < 0 || hold > 1)
    return set_error(h, FMPT_ERR_ARG, "wait test: timeout 0..1e10 ns, hold 0 or 1");
  h->wait_test_ns = timeout_ns;
  h->wait_test_hold = hold;
  return FMPT_OK;
}

int fmpt_set_graphs(fmpt_handle* h, int on) {
  if (!h) return FMPT_ERR_ARG;
  h->graphs = on != 0;
  return FMPT_OK;
}

int fmpt_set_fused_krylov(fmpt_handle* h, int on) {
  if (!h) return FMPT_ERR_ARG;
  h->fused_gs = on != 0;
  return FMPT_OK;
}

int fmpt_set_cluster_qr(fmpt_handle* h, int on) {
  if (!h) return FMPT_ERR_ARG;
  h->cluster_qr = on != 0;
  return FMPT_OK;
}

int fmpt_synchronize(fmpt_handle* h) {
  if (!h) return FMPT_ERR_ARG;
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  return fmpt::gp_check_status(h);   // a timed-out grouped launch reports here
}

int fmpt_set_stream(fmpt_handle* h, void* s) {
  if (!h) return FMPT_ERR_ARG;
  // the handle's workspaces (GEMM split-K buffer, operator scratch, pinned staging) are
  // reused in stream order: work queued on the old stream must finish before the new
  // stream may touch them
  const cudaStream_t ns = s ? (cudaStream_t)s : h->own_stream;
  if (ns != h->stream) FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stream = ns;
  cusolverDnSetStream(h->solver, h->stream);
  return FMPT_OK;
}

void* fmpt_get_stream(fmpt_handle* h) { return h ? (void*)h->stream : nullptr; }

uint64_t fmpt_launch_count(fmpt_handle* h) { return h ? h->launches : 0; }

int fmpt_malloc(fmpt_handle* h, size_t bytes, void** dptr) {
  if (!h || !dptr) return FMPT_ERR_ARG;
  *dptr = nullptr;
  if (bytes == 0) return FMPT_OK;
  FMPT_CUDA(h, cudaMallocAsync(dptr, bytes, h->stream));
  return FMPT_OK;
}

int fmpt_free(fmpt_handle* h, void* p) {
  if (!h) return FMPT_ERR_ARG;
  if (p) FMPT_CUDA(h, cudaFreeAsync(p, h->stream));
  return FMPT_OK;
}

int fmpt_memcpy_h2d(fmpt_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (!dst && bytes) || (!src && bytes)) return FMPT_ERR_ARG;
  if (bytes) FMPT_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
  return FMPT_OK;
}

int fmpt_memcpy_d2h(fmpt_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (!dst && bytes) || (!src && bytes)) return FMPT_ERR_ARG;
  if (bytes) {
    FMPT_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return FMPT_OK;
}

int fmpt_memcpy_d2d(fmpt_handle* h, void* dst, const void* src, size_t bytes) {
  if (!h || (!dst && bytes) || (!src && bytes)) return FMPT_ERR_ARG;
  if (bytes) FMPT_CUDA(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, h->stream));
  return FMPT_OK;
}

int fmpt_memset_zero(fmpt_handle* h, void* dst, size_t bytes) {
  if (!h || (!dst && bytes)) return FMPT_ERR_ARG;
  if (bytes) FMPT_CUDA(h, cudaMemsetAsync(dst, 0, bytes, h->stream));
  return FMPT_OK;
}

int fmpt_gemm(fmpt_handle* h, int dtype, int ta, int tb, int m, int n, int k,
              const double* alpha, const double* A, int lda, const double* B, int ldb,
              const double* beta, double* C, int ldc) {
  if (!h || !alpha || !beta || (!A && m && k) || (!B && n && k) || (!C && m && n))
    return FMPT_ERR_ARG;
  if (dtype != FMPT_F64 && dtype != FMPT_C128) return set_error(h, FMPT_ERR_ARG, "dtype");
  if (ta < 0 || ta > 3 || tb < 0 || tb > 3) return set_error(h, FMPT_ERR_ARG, "trans code");
  const int cp = dtype == FMPT_C128;
  GemmArgs g{};
  g.cplx = cp; g.ta = ta; g.tb = tb; g.m = m; g.n = n; g.k = k;
  g.alpha[0] = alpha[0]; g.alpha[1] = cp ? alpha[1] : 0.0;
  g.beta[0] = beta[0]; g.beta[1] = cp ? beta[1] : 0.0;
  const bool an = (ta == FMPT_N || ta == FMPT_R), bn = (tb == FMPT_N || tb == FMPT_R);
  g.A = A; g.lda = lda; g.planeA = (int64_t)lda * (an ? k : m);
  g.B = B; g.ldb = ldb; g.planeB = (int64_t)ldb * (bn ? n : k);
  g.C = C; g.ldc = ldc; g.planeC = (int64_t)ldc * n;
  if (lda < (an ? m : k) || ldb < (bn ? k : n) || ldc < m)
    return set_error(h, FMPT_ERR_SHAPE, "gemm: leading dimension too small");
  g.batch = 1;
  return gemm_f64(h, g);
}

int fmpt_dot(fmpt_handle* h, int dtype, int64_t n, const double* x, const double* y,
             double* out) {
  if (!h || !x || !y || !out || n < 0) return FMPT_ERR_ARG;
  FMPT_TRY(ensure_pinned(h, 2));
  DevBuf r;
  FMPT_TRY(r.alloc(h, 2 * sizeof(double)));
  FMPT_TRY(vec_dot_dev(h, dtype == FMPT_C128, n, x, y, r.d()));
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, r.d(), 2 * sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  out[0] = h->pinned[0];
  out[1] = dtype == FMPT_C128 ? h->pinned[1] : 0.0;
  return FMPT_OK;
}

int fmpt_nrm2(fmpt_handle* h, int dtype, int64_t n, const double* x, double* out) {
  if (!h || !x || !out || n < 0) return FMPT_ERR_ARG;
  FMPT_TRY(ensure_pinned(h, 2));
  DevBuf r;
  FMPT_TRY(r.alloc(h, 2 * sizeof(double)));
  FMPT_TRY(vec_nrm2_dev(h, dtype == FMPT_C128, n, x, r.d()));
  FMPT_CUDA(h, cudaMemcpyAsync(h->pinned, r.d(), sizeof(double), cudaMemcpyDeviceToHost,
                               h->stream));
  FMPT_CUDA(h, cudaStreamSynchronize(h->stream));
  out[0] = h->pinned[0];
  return FMPT_OK;
}

int fmpt_axpy(fmpt_handle* h, int dtype, int64_t n, const double* a, const double* x,
              double* y) {
  if (!h || !a || !x || !y || n < 0) return FMPT_ERR_ARG;
  if (n == 0) return FMPT_OK;
  const int cp = dtype == FMPT_C128;
  axpy_kernel<<<elementwise_grid(h, n), 256, 0, h->stream>>>(cp, n, a[0], cp ? a[1] : 0.0, x, y);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int fmpt_scal(fmpt_handle* h, int dtype, int64_t n, const double* a, double* x) {
  if (!h || !a || !x || n < 0) return FMPT_ERR_ARG;
  if (n == 0) return FMPT_OK;
  const int cp = dtype == FMPT_C128;
  scal_kernel<<<elementwise_grid(h, n), 256, 0, h->stream>>>(cp, n, a[0], cp ? a[1] : 0.0, x);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

int fmpt_scale_dim(fmpt_handle* h, int dtype, int side, int m, int n, const double* s,
                   double* M) {
  if (!h || !s || !M || m < 0 || n < 0 || (side != 0 && side != 1)) return FMPT_ERR_ARG;
  int64_t tot = (int64_t)m * n;
  if (tot == 0) return FMPT_OK;
  scale_dim_kernel<<<elementwise_grid(h, tot), 256, 0, h->stream>>>(dtype == FMPT_C128, side, m, n,
                                                                    s, M);
  FMPT_LAUNCHED(h);
  return FMPT_OK;
}

}  // extern "C"
