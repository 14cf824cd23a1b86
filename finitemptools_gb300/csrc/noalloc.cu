// Allocation-free variant of the plain FP64 two-site H_eff*x.
//
// Who needs it: callers that must not allocate device memory while they run --
// applications whose own memory manager owns all device memory (a framework's caching
// allocator, an embedding host that hands the library a fixed arena), and drivers that
// run under a fixed memory budget, where a pool allocation in the middle of a solve can
// fail or stall.  The ordinary fmpt_ac2_prime takes its intermediates (T1, T3) and its
// MPO block table from the stream-ordered pool; this entry point takes them from one
// file-scope device array instead, so the call itself allocates nothing.
//
// The array is FMPT_NOALLOC_SCRATCH_BYTES (64 MiB) and every GPU that loads the library
// holds it until the process exits.  All calls share it and it keeps the last call's
// contents; calls that overlap on the GPU (two streams, two host threads) race on it, so
// the caller must serialise them.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.h"

namespace fmpt {
namespace {

constexpr size_t kScratchDoubles = FMPT_NOALLOC_SCRATCH_BYTES / sizeof(double);

// The scratch itself.  In host code this name is only a stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Once per device, with that device current: resolve the array's device
// address (this also loads the module on that device, which is why the first
// call on a device has to come before any stream capture).
int scratch_for_current_device(fmpt_handle* h, double** out) {
  int dev = 0;
  FMPT_CUDA(h, cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(h, FMPT_ERR_UNSUPPORTED, "noalloc: device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_error(h, FMPT_ERR_CUDA, "noalloc: cudaGetSymbolAddress failed: %s",
                       cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return FMPT_OK;
}

// A piece of the block table passed by value to table_put.
constexpr int kChunkWords = 960;   // 3840 bytes: within the classic 4 KB parameter space
struct TableChunk {
  uint32_t w[kChunkWords];
};

__global__ void table_put(TableChunk c, int n, uint32_t* __restrict__ dst) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = c.w[i];
}

// n 32-bit words from host memory to dst (scratch) through kernel parameters
int upload_words(fmpt_handle* h, const uint32_t* src, size_t n, uint32_t* dst) {
  for (size_t o = 0; o < n; o += kChunkWords) {
    const int k = (int)std::min<size_t>(kChunkWords, n - o);
    TableChunk c;
    std::memcpy(c.w, src + o, (size_t)k * sizeof(uint32_t));
    table_put<<<1, 256, 0, h->stream>>>(c, k, dst + o);
    FMPT_LAUNCHED(h);
  }
  return FMPT_OK;
}

}  // namespace
}  // namespace fmpt

using namespace fmpt;

extern "C" int fmpt_ac2_prime_noalloc(fmpt_handle* h, int dtype, const double* x,
                                      const double* W1, const double* W2, const double* hleft,
                                      const double* hright, double* y, int Dl, int d1, int d2,
                                      int Dr, int wl, int wm, int wr) {
  if (!h) return FMPT_ERR_ARG;
  if (dtype != FMPT_F64 && dtype != FMPT_C128)
    return set_error(h, FMPT_ERR_ARG, "noalloc: unknown dtype %d", dtype);
  if (!x || !W1 || !W2 || !hleft || !hright || !y)
    return set_error(h, FMPT_ERR_ARG, "noalloc: null pointer");
  if (Dl < 1 || Dr < 1 || d1 < 1 || d2 < 1 || wl < 1 || wm < 1 || wr < 1)
    return set_error(h, FMPT_ERR_SHAPE, "noalloc: non-positive dimension");
  const int cp = dtype == FMPT_C128;
  const int P = d1 * d2;
  if (P > 16)
    return set_error(h, FMPT_ERR_UNSUPPORTED, "noalloc: physical dimension product %d > 16", P);

  // ---- MPO block table of the two-site MPO (host): the builder of fmpt_ac2_prime
  MidSchedule sched;
  schedule_ac2_host(cp, W1, W2, d1, d2, wl, wm, wr, sched);
  const std::vector<int>& win = sched.blk_win;
  const std::vector<int>& wstart = sched.wout_start;
  const std::vector<double>& coef = sched.coef;

  // ---- scratch layout (doubles): [ table | T1 | T3 ], every part 256-byte aligned
  auto up32 = [](size_t n) { return (n + 31) / 32 * 32; };
  const size_t t_int = up32((win.size() + wstart.size() + 1) / 2 + 1);   // ints packed in doubles
  const size_t t_coef = up32(coef.size() + 1);
  const int64_t e1 = (int64_t)Dl * wl * P * Dr, e3 = (int64_t)Dl * P * wr * Dr;
  const size_t s1 = up32((size_t)e1 * (cp ? 2 : 1)), s3 = up32((size_t)e3 * (cp ? 2 : 1));
  const size_t need = t_int + t_coef + s1 + s3;
  if (need > kScratchDoubles)
    return set_error(h, FMPT_ERR_SHAPE,
                     "noalloc: this H_eff*x needs %zu bytes of scratch but the static scratch "
                     "holds %zu bytes (FMPT_NOALLOC_SCRATCH_BYTES); use fmpt_ac2_prime",
                     need * sizeof(double), (size_t)FMPT_NOALLOC_SCRATCH_BYTES);
  double* base = nullptr;
  FMPT_TRY(scratch_for_current_device(h, &base));
  int* d_win = reinterpret_cast<int*>(base);
  int* d_wstart = d_win + win.size();
  double* d_coef = base + t_int;
  double* T1 = d_coef + t_coef;
  double* T3 = T1 + s1;
  // The table is the only part that must hold defined values before the kernels run; T1
  // and T3 are written in full (GEMM with beta = 0, every output block of the MPO step)
  // before they are read, so nothing is cleared.  The table reaches the device as kernel
  // parameters (by value, in pieces of TableChunk), not through a host-memory copy.
  FMPT_TRY(upload_words(h, reinterpret_cast<const uint32_t*>(win.data()), win.size(),
                        reinterpret_cast<uint32_t*>(d_win)));
  FMPT_TRY(upload_words(h, reinterpret_cast<const uint32_t*>(wstart.data()), wstart.size(),
                        reinterpret_cast<uint32_t*>(d_wstart)));
  FMPT_TRY(upload_words(h, reinterpret_cast<const uint32_t*>(coef.data()), coef.size() * 2,
                        reinterpret_cast<uint32_t*>(d_coef)));
  sched.d_win = d_win; sched.d_wstart = d_wstart; sched.d_coef = d_coef;

  // ---- the three steps of the plain form (the same kernels as fmpt_ac2_prime)
  const int64_t nx = (int64_t)Dl * P * Dr;
  GemmArgs g{};
  g.cplx = cp; g.alpha[0] = 1.0; g.batch = 1;
  g.nosplit = 1;            // a split-K workspace would be an allocation
  // 1. T1[(a' w), (s b)] = L[(a' w), a] x[a, (s b)]
  g.ta = FMPT_N; g.tb = FMPT_N; g.m = Dl * wl; g.n = P * Dr; g.k = Dl;
  g.A = hleft; g.lda = (int64_t)Dl * wl; g.planeA = (int64_t)Dl * wl * Dl;
  g.B = x; g.ldb = Dl; g.planeB = nx;
  g.C = T1; g.ldc = (int64_t)Dl * wl; g.planeC = e1;
  FMPT_TRY(gemm_f64(h, g));
  // 2. T3[a', s', w2, b] = sum over nonzero blocks O[s', s] T1[a', w, s, b]
  MidStrides si{1, (int64_t)Dl * wl * P, Dl, (int64_t)Dl * wl};
  MidStrides so{1, (int64_t)Dl * P * wr, (int64_t)Dl * P, Dl};
  FMPT_TRY(mid_apply(h, sched, T1, e1, si, T3, e3, so, Dl, Dr));
  // 3. y[(a' s'), b'] = T3[(a' s'), (w2 b)] R[b', (w2 b)]^T
  g.ta = FMPT_N; g.tb = FMPT_T; g.m = Dl * P; g.n = Dr; g.k = wr * Dr;
  g.A = T3; g.lda = (int64_t)Dl * P; g.planeA = e3;
  g.B = hright; g.ldb = Dr; g.planeB = (int64_t)Dr * wr * Dr;
  g.C = y; g.ldc = (int64_t)Dl * P; g.planeC = nx;
  FMPT_TRY(gemm_f64(h, g));
  return FMPT_OK;
}
