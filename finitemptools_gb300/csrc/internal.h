// Internal declarations shared by the libfmpt translation units.
#pragma once

#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/fmpt.h"

struct fmpt_handle {
  int device = 0;
  cudaStream_t stream = nullptr;       // stream in use
  cudaStream_t own_stream = nullptr;   // stream created by fmpt_create
  cusolverDnHandle_t solver = nullptr;
  uint64_t launches = 0;
  std::string err;
  // small pinned host staging area for scalars read back by the solvers
  double* pinned = nullptr;
  size_t pinned_len = 0;
  int sm_count = 0;
  // device timers (fmpt_profile_*)
  bool prof = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[FMPT_K_COUNT];
  std::vector<cudaEvent_t> ev_pool;
  // status word of the grouped block-sparse launches (1 = a grid barrier timed
  // out); allocated on first use, read and cleared by gp_check_status
  int* gstatus = nullptr;
  // auxiliary streams with their own cuSOLVER handles for independent
  // factorisations (created on first use): fork/join through events on `stream`
  std::vector<cudaStream_t> aux_stream;
  std::vector<cusolverDnHandle_t> aux_solver;
  std::vector<cudaEvent_t> aux_event;   // [0] fork, [1 + i] join of aux stream i
  // CUDA graphs for the Krylov solvers of block-sparse operators (fmpt_set_graphs)
  bool graphs = true;
  // Krylov exponentials: one cooperative launch per Arnoldi orthogonalisation step
  // (fmpt_set_fused_krylov; the seven separate launches give bit-identical results)
  int fused_gs = 1;
  // thin QR of small tall panels on one thread-block cluster (fmpt_set_cluster_qr)
  int cluster_qr = 1;
  int svd_method = 0;          // 0 gesvd (bidiagonalisation), 1 gesvdp (polar decomposition)
  int tc_tile = 0;             // tcgen05 GEMM tile: 0 CTA pair where it applies, 1 one CTA
  // split-K workspace of the FP64 GEMM, grown outside stream capture only (stream-ordered
  // reuse on h->stream)
  void* gemm_ws = nullptr;
  size_t gemm_ws_bytes = 0;
  // per-tile arrival counts of the split FP64 GEMM (zero between launches)
  void* gemm_cnt = nullptr;
  size_t gemm_cnt_bytes = 0;
  // partial tiles and arrival counters of the BF16 pair GEMM's K-split last round
  void* tc_ws = nullptr;
  size_t tc_ws_bytes = 0;
  // FP64 GEMMs on the BF16 tensor cores (Ozaki digit planes, exponents, split pieces):
  // f64_tc 1 routes every FP64 GEMM of this handle there when its cost model says it is
  // faster than the CUDA-core kernel (fmpt_set_f64_engine)
  int f64_tc = 0;
  // failure-detection test hook (fmpt_set_wait_test): bound of the grouped kernel's barrier
  // waits (0: 2 s) and extra arrivals they wait for (0 in normal use)
  int64_t wait_test_ns = 0;
  int wait_test_hold = 0;
  void* oz_ws = nullptr;
  size_t oz_ws_bytes = 0;
  // executable graphs of the captured Arnoldi basis, one per operator structure
  std::map<std::string, cudaGraphExec_t> arnoldi_exec;
  cudaGraphExec_t lanczos_exec = nullptr;   // reused through cudaGraphExecUpdate
  uint64_t graph_launches = 0;
  // grouped-kernel tile autotuner (fmpt_set_tuning): 0 measure, 1 force the
  // 32x32 tile, 2 force 64x64; cache: (program kind, work bucket) -> variant
  int tune_mode = 0;
  std::map<int, int> tune_cache;
  uint64_t tune_runs = 0;
};

namespace fmpt {

int set_error(fmpt_handle* h, int status, const char* fmt, ...);

#define FMPT_CUDA(h, expr)                                                              \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return ::fmpt::set_error((h), _e == cudaErrorMemoryAllocation ? FMPT_ERR_NOMEM    \
                                                                    : FMPT_ERR_CUDA,    \
                               "%s:%d %s: %s", __FILE__, __LINE__, #expr,              \
                               cudaGetErrorString(_e));                                 \
  } while (0)

#define FMPT_TRY(expr)          \
  do {                          \
    int _s = (expr);            \
    if (_s != FMPT_OK) return _s; \
  } while (0)

#define FMPT_LAUNCHED(h)                                                                \
  do {                                                                                  \
    (h)->launches++;                                                                    \
    cudaError_t _e = cudaGetLastError();                                                \
    if (_e != cudaSuccess)                                                              \
      return ::fmpt::set_error((h), FMPT_ERR_CUDA, "%s:%d launch: %s", __FILE__,        \
                               __LINE__, cudaGetErrorString(_e));                       \
  } while (0)

// Stream-ordered device scratch owned by a C++ scope.
struct DevBuf {
  fmpt_handle* h = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  int alloc(fmpt_handle* hh, size_t nbytes);
  void release();
  double* d() const { return static_cast<double*>(p); }
};

int ensure_pinned(fmpt_handle* h, size_t n_doubles);
// the FP64 one-/two-site operator application in two halves (heff.cu): head = GEMM 1 and
// the MPO step into the operator's scratch, tail = GEMM 2 into y
int op_fp64_head(fmpt_op* op, const double* x);
int op_fp64_tail(fmpt_op* op, double* y);
// Q (m x n) and R (n x n) of a small tall panel (m >= n) on one thread-block cluster;
// FMPT_ERR_UNSUPPORTED (nothing launched) outside its range (qr_cluster.cu)
int qr_small_cluster(fmpt_handle* h, int cplx, int m, int n, const double* M, double* Q,
                     double* R);
// a device buffer of at least `bytes` held in *buf / *cap (stream-ordered on h->stream);
// growing it while h->stream is being captured returns FMPT_ERR_UNSUPPORTED
int grow_buffer(fmpt_handle* h, void** buf, size_t* cap, size_t bytes);
// At least n auxiliary streams/solvers; aux_fork makes them wait for the work
// queued so far on h->stream, aux_join makes h->stream wait for them.
int ensure_aux(fmpt_handle* h, int n);
int aux_fork(fmpt_handle* h, int n);
int aux_join(fmpt_handle* h, int n);

// Scoped device timer for one launch of a kernel class (no-op unless profiling).
struct ProfScope {
  fmpt_handle* h;
  int cls;
  cudaEvent_t b = nullptr, e = nullptr;
  ProfScope(fmpt_handle* hh, int c);
  ~ProfScope();
};

// Digit planes and exponents of one FP64 GEMM operand for the tensor-core FP64 engine,
// kept across calls by an owner whose operand does not change between them (a prepared
// operator's environments): built on first use, reused while src and shape match.
struct OzCache {
  const double* src = nullptr;
  int64_t key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  void* buf = nullptr;
  size_t bytes = 0;
  bool valid = false;
};
void oz_cache_free(fmpt_handle* h, OzCache& c);

// -------- generic FP64 / split-complex GEMM (gemm_f64.cu)
// C = alpha op(A) op(B) + beta C ; planes: element offsets between re and im planes.
struct GemmArgs {
  int cplx;                 // 0 real, 1 split complex
  int ta, tb;               // fmpt_trans
  int m, n, k;
  double alpha[2], beta[2];
  const double* A; int64_t lda; int64_t planeA;
  const double* B; int64_t ldb; int64_t planeB;
  double* C; int64_t ldc; int64_t planeC;
  int batch;                // batched over blockIdx.z with the strides below
  int64_t strideA, strideB, strideC;
  int nosplit;              // 1: never split K (no workspace allocation)
  int engine;               // 0: the handle's FP64 engine, 1: tensor cores where faster
  OzCache* cacheA;          // optional digit-plane caches of A / B (tensor-core engine)
  OzCache* cacheB;
};
int gemm_f64(fmpt_handle* h, const GemmArgs& g);
// the Ozaki-scheme FP64 GEMM on the BF16 tensor cores (ozaki.cu): whether it applies to g
// (engine requested, shape large enough to win), and the call itself
int gemm_f64_ozaki_possible(fmpt_handle* h, const GemmArgs& g);
int gemm_f64_ozaki(fmpt_handle* h, const GemmArgs& g);
// the handle's device status word (1: a bounded device wait timed out), read and cleared by
// gp_check_status / fmpt_synchronize
int gp_status_word(fmpt_handle* h, int** out);
inline bool prec_is_f64(int precision) {
  return precision == FMPT_PREC_FP64 || precision == FMPT_PREC_FP64_TC;
}

// -------- block-sparse MPO "middle" contraction (heff.cu)
// out[o1, o2, wo, so] = sum_{blocks (wi -> wo)} sum_si coef[so, si] in[o1, o2, wi, si]
constexpr int MS_MAX_OUT = 128, MS_MAX_T = 512;   // sparse MPO-step table capacity
struct MidSchedule {
  int nw_in = 0, nw_out = 0, p_in = 0, p_out = 0, cplx = 0;
  std::vector<int> blk_win;      // per block: input w
  std::vector<int> wout_start;   // nw_out + 1 prefix offsets into the blocks (sorted by wo)
  std::vector<double> coef;      // per block: p_out x p_in (row-major so, si), re then im if cplx
  // the nonzero terms per output (wo, so): prefix offsets, wi * 16 + si, coefficients (re, im
  // pairs if cplx); empty when they exceed the by-value table of the sparse kernel
  std::vector<int> sp_start, sp_idx;
  std::vector<double> sp_coef;
  // device copies
  int* d_win = nullptr;
  int* d_wstart = nullptr;
  double* d_coef = nullptr;
  int nblocks() const { return (int)blk_win.size(); }
};
int mid_upload(fmpt_handle* h, MidSchedule& s);
void mid_free(fmpt_handle* h, MidSchedule& s);
struct MidStrides { int64_t o1, o2, w, s; };
int mid_apply(fmpt_handle* h, const MidSchedule& s, const double* in, int64_t plane_in,
              MidStrides si, double* out, int64_t plane_out, MidStrides so, int n1, int n2);

// Schedules from dense host MPO tensors (W[wl, s_out, wr, s_in]).
int schedule_ac2(fmpt_handle* h, int cplx, const double* W1, const double* W2, int d1, int d2,
                 int wl, int wm, int wr, MidSchedule& s);
// the host part of schedule_ac2: fills s.blk_win / s.wout_start / s.coef, uploads nothing
void schedule_ac2_host(int cplx, const double* W1, const double* W2, int d1, int d2, int wl,
                       int wm, int wr, MidSchedule& s);
int schedule_ac(fmpt_handle* h, int cplx, const double* W, int d, int wl, int wr, MidSchedule& s);
// updateright maps the right index w2 (input) to the left index w (output)
int schedule_env(fmpt_handle* h, int cplx, const double* W, int d, int wl, int wr, bool right,
                 MidSchedule& s);

// -------- grouped persistent block-sparse engine (grouped.cu)
constexpr int GP_MAX_PHASES = 4, GP_SLOTS = 8;
constexpr int GP_VARIANTS = 4;   // (tile, schedule): v & 1 -> 32x32 / 64x64 tiles, v >> 1 -> schedule
enum { GP_GEMM = 0, GP_SUM = 1 };
// One output block: C (m x n, column-major with ldc) at c_off in the phase's C slot.
struct GProblem {
  int64_t c_off, ldc;
  int m, n, seg0, seg1;
};
// One term of a block: coef * op(A) op(B) (GEMM, inner extent k) or coef * A (SUM).
struct GSegment {
  int64_t a_off, lda, b_off, ldb;
  double coef;
  int k, pad;
};
struct GPhaseDesc {
  int type, ta, tb, a_slot, b_slot, c_slot, tile0, tile1;
};
struct GroupedProgram {
  std::vector<GPhaseDesc> phases;
  std::vector<int> phase_prob0;
  std::vector<GProblem> probs;
  std::vector<GSegment> segs;
  std::vector<int> tile_prob, tile_mn;           // the tiles of every variant, one after another
  std::vector<int> vtile0[GP_VARIANTS], vtile1[GP_VARIANTS];   // per variant and phase
  int vgrid[GP_VARIANTS] = {0, 0, 0, 0};
  int variant = 0;                                // the one gp_run launches by default
  double flops = 0.0;       // 2 m n k over the GEMM segments
  double sum_elems = 0.0;   // output elements x terms of the SUM phases
  int64_t slot_elems[GP_SLOTS] = {-1, -1, -1, -1, -1, -1, -1, -1};  // operand extents
  DevBuf dev;
  GProblem* d_probs = nullptr;
  GSegment* d_segs = nullptr;
  int* d_tile_prob = nullptr;
  int* d_tile_mn = nullptr;
  int* d_ctl = nullptr;
  bool ready = false;
};
// Builder: a phase, then its problems, each followed by its segments.
void gp_phase(GroupedProgram& g, int type, int ta, int tb, int a_slot, int b_slot, int c_slot);
int gp_problem(GroupedProgram& g, int64_t c_off, int64_t ldc, int m, int n);
void gp_segment(GroupedProgram& g, int64_t a_off, int64_t lda, int64_t b_off, int64_t ldb, int k,
                double coef);
// Declares how many doubles operand slot `slot` holds; gp_finalize checks every
// block footprint against it (host side, before anything reaches the GPU).
void gp_slot(GroupedProgram& g, int slot, int64_t elems);
int gp_finalize(fmpt_handle* h, GroupedProgram& g);   // bounds check + tiles + upload
// gate: optional device flag; when it is nonzero at launch time every CTA
// returns at once (a solver step after convergence inside a CUDA graph)
int gp_run(fmpt_handle* h, const GroupedProgram& g, double* const* slots, int nslots,
           const int* gate = nullptr, int variant = -1);
int gp_prepare(fmpt_handle* h);   // allocations gp_run needs, done before a stream capture
// Picks g.variant: the handle's cached choice for (kind, work bucket), else
// (tune mode 0) times every variant on these slots -- the program must be
// safe to run repeatedly on them -- and caches the fastest.
enum { GP_KIND_HEFF = 1, GP_KIND_ENV = 2, GP_KIND_OTHER = 3 };
int gp_autotune(fmpt_handle* h, GroupedProgram& g, double* const* slots, int nslots, int kind);
int gp_check_status(fmpt_handle* h);                  // synchronises; FMPT_ERR_TIMEOUT if set

// -------- dense helpers shared with the sector code (linalg.cu)
int copy_mat(fmpt_handle* h, int cplx, int rows, int cols, const double* src, int64_t s_ld,
             int64_t s_plane, int trans, int conj, double* dst, int64_t d_ld, int64_t d_plane);
int svd_tall(fmpt_handle* h, int cplx, int m, int n, double* Awork, double* S, double* U,
             double* VT);

// -------- vector kernels (krylov.cu)
int vec_dot_dev(fmpt_handle* h, int cplx, int64_t n, const double* x, const double* y,
                double* out_dev /* re, im */);
int vec_nrm2_dev(fmpt_handle* h, int cplx, int64_t n, const double* x, double* out_dev);

}  // namespace fmpt

// The opaque operator type of the C ABI.
struct fmpt_op {
  fmpt_handle* h = nullptr;
  int kind = 0;          // 0 ac2, 1 ac, 2 c
  int dtype = FMPT_F64;
  int precision = FMPT_PREC_FP64;
  int Dl = 0, Dr = 0, d1 = 1, d2 = 1, wl = 1, wm = 1, wr = 1;
  const double* hleft = nullptr;
  const double* hright = nullptr;
  fmpt::MidSchedule sched;
  int64_t n = 0;          // vector length (complex elements for C128)
  void* tc = nullptr;     // tensor-core state (mixed precision), owned
  void* u1 = nullptr;     // U(1) block-sparse state (grouped program + scratch), owned
  bool defer_right = false;  // mixed precision: the right environment is converted later
  // FP64 intermediates of one application (T1/T3 or T), grown outside stream capture only
  double* scratch = nullptr;
  // digit planes of the environments for the tensor-core FP64 engine (FP64_TC operators)
  fmpt::OzCache oz_left, oz_right;
  size_t scratch_bytes = 0;
  // projectors of the excited-state sweeps: after every application
  // y -= dot(y, p) p for each p in order (device vectors of n elements, not owned)
  std::vector<const double*> proj;
  double* proj_part = nullptr;   // 2 * proj_G block partials, owned
  int proj_G = 0;
};

namespace fmpt {
int op_apply_fp64(fmpt_op* op, const double* x, double* y);
int op_tc_prepare(fmpt_op* op);
int op_tc_apply(fmpt_op* op, const double* x, double* y);
// split application of a real tensor-core two-site operator (host-buffer pipeline):
// head = x conversion, GEMM 1 and MPO step; tail = GEMM 2; prepare_right converts the
// right environment of an operator created with defer_right
int op_tc_apply_head(fmpt_op* op, const double* x);
int op_tc_apply_tail(fmpt_op* op, double* y);
int op_tc_prepare_right(fmpt_op* op);
// the same for the rows b' in [r0, r1) of the right environment / columns of y
int op_tc_prepare_right_rows(fmpt_op* op, int r0, int r1);
int op_tc_apply_tail_rows(fmpt_op* op, double* y, int r0, int r1);
int op_tc_check(fmpt_op* op);   // reads the device timeout flag (synchronises)
// mixed-precision environment update (real data), FP64 output in the reference layout
int env_update_tc(fmpt_handle* h, bool right, int precision, const double* hold, const double* A,
                  const double* W, const double* B, double* hnew, int Dl, int d, int Dr, int wl,
                  int wr);
void op_tc_free(fmpt_op* op);
int op_u1_apply(fmpt_op* op, const double* x, double* y, const int* gate = nullptr);
// the projections of op->proj applied to y in place (no-op without projectors)
int op_project(fmpt_op* op, double* y, const int* gate = nullptr);
void op_u1_free(fmpt_op* op);

// K-major tensor-core operand: TF32 (float storage) or BF16 plane, optional
// TF32 low plane (3xTF32), row stride and batch stride in elements.
struct TcOperand {
  const void* hi;
  const void* lo;
  int64_t ld;
  int64_t bstride;
};
// C[m, n] (+ batch) = sum_k A[m, k] B[n, k] on tcgen05; mode 0 TF32, 1 3xTF32, 2 BF16;
// C is FP32 (out_f64 = 0), FP64 (1) or, in BF16 mode, BF16 (2); column-major with ldc.
int tc_gemm(fmpt_handle* h, int mode, int M, int N, int K, int batch, const TcOperand& A,
            const TcOperand& B, void* C, int out_f64, int64_t ldc, int64_t strideC, int* err_dev);
}  // namespace fmpt
