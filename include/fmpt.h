/*
 * libfmpt -- GB300 (sm_103a) kernels for the DMRG/TDVP inner loop of
 * FiniteMPTools, behind a plain C ABI.
 *
 * Conventions
 *   - Every entry point returns an int status (FMPT_OK == 0, negative on
 *     error); nothing is thrown across the ABI.  fmpt_last_error() gives the
 *     message of the last failure on a handle.
 *   - Tensor arguments are DEVICE pointers in the reference's column-major
 *     layout and index order (Julia storage of the TensorKit tensors):
 *       MPS site tensor   A[a, s, b]            -> A[a + Dl*(s + d*b)]
 *       MPO site tensor   W[wl, s_out, wr, s_in] (HOST pointer, see below)
 *       environment       L[a', w, a], R[b', w, b] (bra, mpo, ket)
 *       two-site tensor   x[a, s1, s2, b]
 *   - MPO tensors are tiny and are the only HOST pointers: the library
 *     derives the nonzero (w, w') block schedule from them on the host.
 *   - dtype FMPT_F64 is real double; FMPT_C128 is complex double held as
 *     split planes: a tensor of n elements is 2n doubles, the n real parts
 *     followed by the n imaginary parts (also for the host MPO tensors).
 *   - A handle owns one CUDA stream, a cuSOLVER handle and a stream-ordered
 *     memory pool.  It is not thread-safe: use one handle per host thread.
 *     Calls are asynchronous on the handle's stream unless they return a
 *     host scalar (eigenvalues, truncation results), which synchronise.
 */
#ifndef FMPT_H
#define FMPT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fmpt_handle fmpt_handle;
typedef struct fmpt_op fmpt_op;

enum fmpt_status {
  FMPT_OK = 0,
  FMPT_ERR_ARG = -1,          /* bad argument (null pointer, unknown enum)  ~ ArgumentError   */
  FMPT_ERR_SHAPE = -2,        /* inconsistent dimensions                   ~ DimensionMismatch */
  FMPT_ERR_CUDA = -3,         /* CUDA runtime error                                            */
  FMPT_ERR_CUSOLVER = -4,     /* cuSOLVER error or non-converged factorisation                 */
  FMPT_ERR_TIMEOUT = -5,      /* a bounded device wait gave up                                 */
  FMPT_ERR_NONFINITE = -6,    /* NaN/Inf met in a reduction                                    */
  FMPT_ERR_NOMEM = -7,        /* device allocation failed                                      */
  FMPT_ERR_UNSUPPORTED = -8,  /* valid request this build does not implement                   */
  FMPT_ERR_NOCONV = -9        /* Krylov exponential did not reach its tolerance                */
};

enum fmpt_dtype { FMPT_F64 = 0, FMPT_C128 = 1 };

/* Arithmetic of the contractions (H_eff*x and environment updates).
 * FP64 is the plain form (CUDA-core FMA, or the handle's FP64 engine, see
 * fmpt_set_f64_engine).  FP64_TC is the same FP64 contraction with every GEMM
 * large enough to gain run on the BF16 tensor cores by the Ozaki scheme: each
 * FP64 operand row becomes 9 exact base-64 digit planes (every digit within 32,
 * 53 bits below the row maximum), the 45 digit products of levels up to 10 run
 * as tcgen05 MMAs whose FP32 sums over each K chunk are exact, and the level
 * sums are added in FP64 (Frobenius-relative error 1e-15 to 4e-15 against the
 * FP64 kernel on random data, the accuracy class of an FP64 GEMM).  TF32,
 * 3xTF32 and BF16 run on tcgen05 with FP32 accumulation (3xTF32 = hi/lo split
 * products). */
enum fmpt_precision {
  FMPT_PREC_FP64 = 0,
  FMPT_PREC_TF32X3 = 1,
  FMPT_PREC_TF32 = 2,
  FMPT_PREC_BF16 = 3,
  FMPT_PREC_FP64_TC = 4
};

enum fmpt_trans { FMPT_N = 0, FMPT_T = 1, FMPT_C = 2, FMPT_R = 3 /* conj, no transpose */ };

/* ------------------------------------------------------------ handle */
int fmpt_create(int device, fmpt_handle** out);
int fmpt_destroy(fmpt_handle* h);
const char* fmpt_status_string(int status);
const char* fmpt_last_error(fmpt_handle* h);
int fmpt_synchronize(fmpt_handle* h);
/* SVD routine of every truncated split on this handle (fmpt_svd_trunc, the
 * U(1) per-sector SVD, the TEBD bond updates): 0 = cuSOLVER gesvd
 * (bidiagonalisation; the default, as the reference's LAPACK fallback in
 * auxiliary/stable_svd.jl:12-18), 1 = cuSOLVER Xgesvdp (polar decomposition,
 * level-3 bound), 2 = cuSOLVER gesvdj (one-sided Jacobi).  0 and 1 fall back
 * to the Jacobi SVD when they report failure. */
int fmpt_set_svd_method(fmpt_handle* h, int method);

/* CUDA graphs for the Krylov solvers (default on): fmpt_lanczos_ground on a
 * block-sparse (U(1)) operator captures all its iterations into one graph --
 * after convergence a device flag turns the remaining steps into no-ops -- and
 * launches it once, with one host synchronisation per solve instead of one
 * per iteration.  The instantiated graph is reused across solves through
 * cudaGraphExecUpdate.  Off: the host-driven loop.  No counterpart in the
 * reference. */
int fmpt_set_graphs(fmpt_handle* h, int on);
/* Number of CUDA graph launches of this handle's solvers. */
uint64_t fmpt_graph_launch_count(fmpt_handle* h);
/* Krylov exponentials (fmpt_exponentiate, fmpt_expm_nodes): on (default), each
 * Arnoldi vector's two-pass Gram-Schmidt orthogonalisation and normalisation
 * run as ONE cooperative launch with bounded grid barriers instead of seven
 * launches; off, the seven launches.  Both give bit-identical results.  No
 * counterpart in the reference. */
int fmpt_set_fused_krylov(fmpt_handle* h, int on);
/* Thin QR (fmpt_qr, fmpt_lq, leftorth!/rightorth) of small tall panels: on
 * (default), a panel with m >= n and m * ceil(n / 16) <= 4096 (e.g. 128 x 64 at
 * D = 64) runs as ONE launch on a thread-block cluster of 8 or 16 CTAs, with
 * LAPACK's Householder conventions (the same Q and R as geqrf/ungqr to
 * rounding); off, or outside that range, cuSOLVER geqrf + ungqr.  No
 * counterpart in the reference. */
int fmpt_set_cluster_qr(fmpt_handle* h, int on);
/* Autotuner of the grouped block-sparse kernel.  mode 0 (default): the first
 * time a block-sparse operator or environment update of a new work size (kind,
 * half-octave of FLOPs) is built, every kernel variant -- 32x32 or 64x64 output
 * tiles, each with two block schedules (blocks by descending work, or tiles by
 * descending work of their own) -- is timed on it and the fastest is cached in
 * the handle; mode 1 / 2 force the 32x32 / 64x64 tile with the first schedule,
 * mode 3 / 4 the same tiles with the second.
 * All variants sum every output in the same order: the choice never changes
 * results.  No counterpart in the reference. */
int fmpt_set_tuning(fmpt_handle* h, int mode);
/* Output tile of the tensor-core GEMMs (BF16, TF32, 3xTF32).  mode 0 (default):
 * GEMMs of more than 128 rows run 256x256 tiles on two-CTA clusters
 * (tcgen05.mma.cta_group::2), the rest one-CTA tiles (128x256; 128x128 for
 * 3xTF32); mode 1: always the one-CTA tile.  Both accumulate in FP32 over the
 * same K slices; the last bits may differ.  No counterpart in the reference. */
int fmpt_set_tc_tile(fmpt_handle* h, int mode);
/* FP64 engine of every FP64 GEMM this handle runs without a precision argument
 * of its own (FP64 H_eff*x and environment updates, the density-matrix split's
 * Gram matrix, the Krylov solvers' Ritz combinations, fmpt_gemm): mode 0
 * (default) the CUDA cores; mode 1 the BF16 tensor cores by the Ozaki scheme of
 * FMPT_PREC_FP64_TC wherever a cost model of the two kernels says it is faster
 * (large GEMMs; small ones stay on the CUDA cores).  No counterpart in the
 * reference. */
int fmpt_set_f64_engine(fmpt_handle* h, int mode);
/* Failure-detection test hook of the cooperative SIMT launches -- the grouped
 * block-sparse kernel and the fused Krylov orthogonalisation step (no counterpart in the
 * reference).  Every grid barrier of those launches waits at most timeout_ns (0: the
 * default 2 s); then the launch sets the handle's status word and returns, and the next
 * fmpt_synchronize (or solver) reports FMPT_ERR_TIMEOUT while the context stays usable.
 * hold = 1 makes the barriers wait for one arrival that never comes, so that a test can
 * run the wait out; hold = 0 is normal operation.  No other kernel is affected. */
int fmpt_set_wait_test(fmpt_handle* h, int64_t timeout_ns, int hold);
/* Number of cached tuning decisions and of timed tunings so far. */
int fmpt_tuning_info(fmpt_handle* h, int* entries, int64_t* timed);
/* Output tile edge (32 or 64) a block-sparse operator runs with (0: dense op). */
int fmpt_op_tile(fmpt_op* op);
/* Run subsequent work of this handle on an external cudaStream_t (NULL: the
 * handle's own stream). */
int fmpt_set_stream(fmpt_handle* h, void* cuda_stream);
void* fmpt_get_stream(fmpt_handle* h);
/* Number of kernels this handle has launched (own kernels only). */
uint64_t fmpt_launch_count(fmpt_handle* h);
int fmpt_version(void);

/* Device-side timers: while enabled, every launch of the classes below is
 * bracketed by CUDA events on the handle's stream.  fmpt_profile_read
 * synchronises, returns the launch count and summed device milliseconds of
 * one class and clears it.  Classes: */
enum fmpt_kernel_class {
  FMPT_K_TC_GEMM = 0,     /* tcgen05 tensor-core GEMM (mixed precision) */
  FMPT_K_F64_GEMM = 1,    /* FP64 / complex FP64 CUDA-core GEMM         */
  FMPT_K_MPO_STEP = 2,    /* block-sparse MPO contraction step          */
  FMPT_K_CONVERT = 3,     /* operand layout / precision conversion      */
  FMPT_K_GROUPED = 4,     /* grouped block-sparse (U(1)) persistent launch */
  FMPT_K_COUNT = 5
};
int fmpt_profile_enable(fmpt_handle* h, int on);
int fmpt_profile_read(fmpt_handle* h, int kernel_class, int64_t* launches, double* total_ms);

/* ------------------------------------------------------------ memory */
int fmpt_malloc(fmpt_handle* h, size_t bytes, void** dptr);
int fmpt_free(fmpt_handle* h, void* dptr);
int fmpt_memcpy_h2d(fmpt_handle* h, void* dst, const void* src, size_t bytes);
int fmpt_memcpy_d2h(fmpt_handle* h, void* dst, const void* src, size_t bytes);
int fmpt_memcpy_d2d(fmpt_handle* h, void* dst, const void* src, size_t bytes);
int fmpt_memset_zero(fmpt_handle* h, void* dst, size_t bytes);

/* ------------------------------------------------- BLAS-like helpers */
/* C = alpha*op(A)*op(B) + beta*C, column-major, op from fmpt_trans.  For
 * C128 the operands are split planes with plane strides (in elements)
 * given by the matrix extents: A has lda*cols(A) elements per plane, etc.
 * alpha/beta are {re, im}. */
int fmpt_gemm(fmpt_handle* h, int dtype, int transa, int transb, int m, int n, int k,
              const double* alpha, const double* A, int lda, const double* B, int ldb,
              const double* beta, double* C, int ldc);
/* out = <x, y> = sum conj(x_i) y_i, written to HOST out[0..1] (re, im). */
int fmpt_dot(fmpt_handle* h, int dtype, int64_t n, const double* x, const double* y, double* out);
int fmpt_nrm2(fmpt_handle* h, int dtype, int64_t n, const double* x, double* out);
/* y = a*x + y ; x = a*x  (a = {re, im}) */
int fmpt_axpy(fmpt_handle* h, int dtype, int64_t n, const double* a, const double* x, double* y);
int fmpt_scal(fmpt_handle* h, int dtype, int64_t n, const double* a, double* x);
/* M[i, j] *= s[i] (side 0) or s[j] (side 1); s is a real DEVICE vector. */
int fmpt_scale_dim(fmpt_handle* h, int dtype, int side, int m, int n, const double* s, double* M);

/* ------------------------------------------------------ H_eff * x
 * ac2_prime (algorithms/derivatives.jl:20-22):
 *   y[a',s1',s2',b'] = sum L[a',w,a] x[a,s1,s2,b] W1[w,s1',m,s1] W2[m,s2',w2,s2] R[b',w2,b]
 * hleft [Dl, wl, Dl], hright [Dr, wr, Dr], W1 [wl, d1, wm, d1], W2 [wm, d2, wr, d2]. */
int fmpt_ac2_prime(fmpt_handle* h, int dtype, int precision, const double* x,
                   const double* W1_host, const double* W2_host, const double* hleft,
                   const double* hright, double* y, int Dl, int d1, int d2, int Dr,
                   int wl, int wm, int wr);
/* ac2_prime with HOST buffers: x, hleft, hright and y live in host memory, W1/W2 as
 * for fmpt_ac2_prime.  The result is identical to copying in, calling fmpt_ac2_prime
 * and copying out.  For real data in a mixed precision the transfers are pipelined
 * on a second stream (L, then x, then R): the L conversion overlaps the x copy, and
 * the x conversion, GEMM 1 and the MPO step overlap the R copy.  Use page-locked
 * buffers (cudaHostAlloc / cudaHostRegister) for the overlap; pageable memory works
 * but copies synchronously.  Returns after y has been written. */
int fmpt_ac2_prime_host(fmpt_handle* h, int dtype, int precision, const double* x_host,
                        const double* W1_host, const double* W2_host, const double* hleft_host,
                        const double* hright_host, double* y_host, int Dl, int d1, int d2,
                        int Dr, int wl, int wm, int wr);

/* ac_prime (derivatives.jl:2-4): y[a',s',b'] = sum L[a',w,a] x[a,s,b] W[w,s',w2,s] R[b',w2,b] */
int fmpt_ac_prime(fmpt_handle* h, int dtype, int precision, const double* x,
                  const double* W_host, const double* hleft, const double* hright, double* y,
                  int Dl, int d, int Dr, int wl, int wr);
/* c_prime (derivatives.jl:52-54): y[a',b'] = sum L[a',w,a] C[a,b] R[b',w,b] */
int fmpt_c_prime(fmpt_handle* h, int dtype, int precision, const double* C,
                 const double* hleft, const double* hright, double* y, int Dl, int Dr, int w);

/* ------------------------------------------------ environment updates
 * updateleft (mpo/transfer.jl:31-34):
 *   hnew[b',w2,b] = sum hold[a',w,a] B[a,s,b] W[w,s',w2,s] conj(A[a',s',b'])
 *   hold [Dl, wl, Dl], A/B [Dl, d, Dr], hnew [Dr, wr, Dr].
 * updateright (mpo/transfer.jl:26-29):
 *   hnew[a',w,a] = sum hold[b',w2,b] B[a,s,b] W[w,s',w2,s] conj(A[a',s',b'])
 *   hold [Dr, wr, Dr], hnew [Dl, wl, Dl].
 * W_host == NULL selects the operator-less overlap update (transfer.jl:37-45)
 * with wl == wr. */
int fmpt_updateleft(fmpt_handle* h, int dtype, int precision, const double* hold,
                    const double* A, const double* W_host, const double* B, double* hnew,
                    int Dl, int d, int Dr, int wl, int wr);
int fmpt_updateright(fmpt_handle* h, int dtype, int precision, const double* hold,
                     const double* A, const double* W_host, const double* B, double* hnew,
                     int Dl, int d, int Dr, int wl, int wr);

/* ---------------------------------------- prepared operators (solvers)
 * An fmpt_op captures one effective Hamiltonian (its environments are
 * referenced, not copied, and must stay alive and unchanged) so that the
 * Krylov solvers can apply it repeatedly without re-deriving schedules or
 * re-converting operands. */
int fmpt_op_ac2(fmpt_handle* h, int dtype, int precision, const double* W1_host,
                const double* W2_host, const double* hleft, const double* hright, int Dl,
                int d1, int d2, int Dr, int wl, int wm, int wr, fmpt_op** out);
int fmpt_op_ac(fmpt_handle* h, int dtype, int precision, const double* W_host,
               const double* hleft, const double* hright, int Dl, int d, int Dr, int wl,
               int wr, fmpt_op** out);
int fmpt_op_c(fmpt_handle* h, int dtype, int precision, const double* hleft,
              const double* hright, int Dl, int Dr, int w, fmpt_op** out);
int fmpt_op_apply(fmpt_op* op, const double* x, double* y);
int64_t fmpt_op_size(fmpt_op* op);
int fmpt_op_destroy(fmpt_op* op);

/* Projected operator of the excited-state sweeps: after every application
 * (fmpt_op_apply and every solver built on it, the graph-captured Lanczos
 * included) y = y - dot(y, p) p for p = p[0], ..., p[nproj-1] in order, with
 * Julia's dot(y, p) = sum conj(y) p.  This is _project! of
 * algorithms/dmrgexcited.jl:1-6 composed with ac_prime / ac2_prime as in
 * :21 and :102.  p holds nproj device pointers to vectors of fmpt_op_size(op)
 * elements (the c_proj / _c2_prime_2 projections); they are referenced, not
 * copied.  nproj = 0 removes the projectors. */
int fmpt_op_set_projectors(fmpt_op* op, int nproj, const double* const* p);

/* Lowest eigenpair by the reference's plain Lanczos
 * (auxiliary/simple_lanczos.jl:83-120): three-term recurrence, stop when
 * beta < btol, at most kmax Krylov vectors, lowest Ritz pair of the
 * tridiagonal matrix (solved on the device in FP64).  reorth != 0 adds full
 * FP64 reorthogonalisation (not in the reference; off for parity runs).
 * eigval/info/niter are HOST outputs; xout is a device vector. */
int fmpt_lanczos_ground(fmpt_op* op, const double* x0, int kmax, double btol, int reorth,
                        double* eigval, double* xout, int* info, int* niter);

/* One whole DMRG2 sweep: sweep!(m, DMRG2) (algorithms/dmrgexcited.jl:219-223),
 * i.e. leftsweep! over the bonds (1,2) .. (L-2,L-1) then rightsweep! over
 * (L-1,L) .. (1,2) (algorithms/dmrg.jl:89-144).  Each bond: two-site product,
 * fmpt_lanczos_ground on the ac2 operator (eig_maxiter, eig_tol, reorth), the
 * MPSTruncation split (split 0: fmpt_svd_trunc, 1: fmpt_dm_split; maxD, eps),
 * normalize!(s), the fidelity |1 - |<usv, x2>||, and updateleft!/updateright!
 * in env_precision.  The chain stays in caller-owned device buffers:
 *   sites[i]  A_i [bond[i], phys[i], bond[i+1]], capacity site_cap[i] elements;
 *   envs[b]   h_b [bond[b], wbond[b], bond[b]] (envs[0] = l_LL, envs[L] =
 *             r_RR, envs[b] the environment left of site b), capacity env_cap[b];
 *   W_host[i] the HOST MPO tensor of site i [wbond[i], phys[i], wbond[i+1], phys[i]];
 *   svals[b]  optional (NULL, or NULL entries): receives s of bond b on the
 *             right sweep (psi.s[b+1] in the reference's 1-based numbering).
 * bond (HOST, L+1 entries, bond[0] = bond[L] = 1 for a finite chain) is updated
 * bond by bond.  energies (HOST) gets the 2L-3 Ritz values in sweep order and
 * delta (HOST) the largest fidelity delta.  A kept rank that does not fit a
 * buffer returns FMPT_ERR_SHAPE before that bond writes anything (the bonds
 * before it are complete).  No projectors (plain ExpectationCache only). */
int fmpt_dmrg2_sweep(fmpt_handle* h, int dtype, int precision, int env_precision, int L,
                     const int* phys, int* bond, double* const* sites, const int64_t* site_cap,
                     double* const* envs, const int64_t* env_cap, const double* const* W_host,
                     const int* wbond, double* const* svals, int maxD, double eps,
                     int eig_maxiter, double eig_tol, int reorth, int split, double* energies,
                     double* delta);

/* TEBD gate action (the bondmpo contraction of bond_evolution,
 * circuit/apply_gates.jl:11-50): y[a, p', b] = sum_p G[p', p] x[a, p, b] for a
 * device tensor x [Dl, P, Dr] whose middle index fuses the physical indices of
 * the gate's sites (first site fastest) and a HOST gate matrix G [P, P]
 * (column-major, outputs first; C128: real plane then imaginary plane).
 * Out of place. */
int fmpt_apply_gate(fmpt_handle* h, int dtype, const double* G_host, int P, const double* x,
                    double* y, int Dl, int Dr);

/* The num lowest (which 0, "SR") or highest (which 1, "LR") eigenpairs of a
 * Hermitian op: eigsolve(f, x0, num, which, Lanczos()) as
 * exact_diagonalization calls it (algorithms/exactdiag.jl:28).  KrylovKit's
 * Lanczos is not vendored; this is a thick-restart Lanczos (Wu & Simon 2000)
 * with full FP64 reorthogonalisation, a basis of at most krylovdim (2..256)
 * device vectors and at most maxiter restarts.  A Ritz pair has converged when
 * its residual norm is <= tol.  evals/resid (num each) and nconv/napply (the
 * number of converged leading pairs and of operator applications) are HOST
 * outputs; evecs is a device buffer of num vectors of fmpt_op_size(op)
 * elements (complex: split planes per vector), one after the other. */
int fmpt_eigsolve(fmpt_op* op, const double* x0, int num, int krylovdim, int maxiter, double tol,
                  int which, double* evals, double* evecs, double* resid, int* nconv,
                  int* napply);

/* xout = exp(t * op) x  (t = t_re + i t_im) by a Krylov projection of at
 * most krylovdim vectors with adaptive time stepping to ``tol`` (the
 * tolerance _exp_evolve hands KrylovKit.exponentiate, algorithms/tdvp.jl:3-6,
 * already divided by |t|).  The op must be Hermitian.  A complex t needs
 * dtype C128.  info (HOST) = number of Krylov restarts used. */
int fmpt_exponentiate(fmpt_op* op, double t_re, double t_im, const double* x, double* xout,
                      int krylovdim, double tol, int* info);

/* ------------------------------------------ allocation-free H_eff * x
 * No counterpart in the reference.  The plain FP64 two-site H_eff*x of
 * fmpt_ac2_prime (same arguments; the result equals fmpt_ac2_prime's to FP64
 * rounding -- the summation order of the GEMMs may differ) for callers that
 * cannot allocate device memory while they run: applications whose own memory
 * manager owns the device memory (a framework's caching allocator, a host that
 * hands the library a fixed arena) and runs under a fixed memory budget, where
 * a pool allocation in the middle of a solve may fail.  Instead of pool memory
 * it uses one file-scope device array of FMPT_NOALLOC_SCRATCH_BYTES, held by
 * every GPU that loads the library until the process exits; it calls no
 * cudaMalloc/cudaFree and no allocating library routine, and its MPO block
 * table reaches the device as kernel parameters.
 *   - Scratch need: 8*(Dl*wl*P*Dr + Dl*P*wr*Dr) bytes (x2 for C128), P = d1*d2,
 *     plus a small block table; larger problems return FMPT_ERR_SHAPE with
 *     the sizes in fmpt_last_error (use fmpt_ac2_prime for them).
 *   - The first call on a device resolves the array's device address
 *     (cudaGetSymbolAddress, with that device current); make that first call
 *     before any stream capture.
 *   - All calls share the array, which keeps the last call's contents: calls
 *     that overlap on the GPU race on it.  Issue them on one stream (or
 *     serialise them).
 *   - FP64 forms only (dtype F64 or C128), always on the CUDA cores. */
#define FMPT_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int fmpt_ac2_prime_noalloc(fmpt_handle* h, int dtype, const double* x, const double* W1_host,
                           const double* W2_host, const double* hleft, const double* hright,
                           double* y, int Dl, int d1, int d2, int Dr, int wl, int wm, int wr);

/* ------------------------------------------------- dense factorisations
 * Truncated SVD of M (m x n, column-major) with MPSTruncation semantics
 * (auxiliary/truncation.jl:27-47, stable_svd.jl:12-18): drop sigma below
 * eps*||sigma||_2, then keep at most maxD.  U (m x k, ld m), S (k, real),
 * Vt (k x n, ld k) are device buffers sized for k = min(m, n).  k and err
 * (2-norm of the dropped sigma) are HOST outputs. */
int fmpt_svd_trunc(fmpt_handle* h, int dtype, const double* M, int m, int n, int maxD,
                   double eps, double* U, double* S, double* Vt, int* k, double* err);
/* The truncated two-site split through the reduced density matrix (White's
 * DMRG truncation), for the mixed-precision sweeps.  side 0 (left-to-right
 * sweep): rho = M M^H, A = its k leading eigenvectors (orthonormal columns,
 * m x k) and B = A^H M (= s*v, k x n).  side 1 (right-to-left): rho = M^H M,
 * B = the k leading eigenvectors as orthonormal rows (k x n) and A = M B^H
 * (= u*s, m x k).  Everything in FP64 on the device (GEMM + cuSOLVER
 * syevd/heevd); S gets sqrt of the kept eigenvalues, truncated with the
 * MPSTruncation rule of fmpt_svd_trunc.  No factor is divided by s, so the
 * isometric side stays exactly isometric; singular values below
 * ~1e-8*sigma_max are resolved only to the FP64 noise of rho (they are
 * squared).  ~9x faster than gesvd at 2048^2.  No counterpart in the
 * reference (stable_tsvd! always runs an SVD). */
int fmpt_dm_split(fmpt_handle* h, int dtype, const double* M, int m, int n, int maxD,
                  double eps, int side, double* A, double* S, double* B, int* k, double* err);
/* Thin QR (leftorth!, QR()): M (m x n) = Q (m x r) R (r x n), r = min(m, n). */
int fmpt_qr(fmpt_handle* h, int dtype, const double* M, int m, int n, double* Q, double* R);
/* Thin LQ (rightorth, LQ()): M (m x n) = L (m x r) Q (r x n). */
int fmpt_lq(fmpt_handle* h, int dtype, const double* M, int m, int n, double* Lout, double* Q);

/* ------------------------------------------------- U(1) block-sparse path
 * Charge-conserving (U(1), e.g. Sz) tensors, as TensorKit holds them for
 * U1Space legs (the reference's symmetric path: heisenberg_xxz_chain,
 * utilities/models.jl:47, with the charge labels of abelian_matrix_from_dense,
 * auxiliary/abelianmatrix.jl:112-124: physical basis state i has charge i).
 *
 * A virtual leg is a table of sectors (charge, dimension), charges strictly
 * increasing; its basis is charge-sorted, sector by sector.  MPS tensors
 * A[a, s, b] and environments L[a', w, a] are stored DENSE in these sorted
 * bases (the reference's index order and column-major layout) with exact
 * zeros outside the allowed blocks:
 *   A[a, s, b]    nonzero only if q(a) + qp(s)  == q(b)
 *   L[a', w, a]   nonzero only if q(a') == q(a) + qw(w)   (same rule for R[b', w, b])
 *   W[wl, s', wr, s] must satisfy qw(wl) + qp(s') == qw(wr) + qp(s)
 * qp are the physical charges, qw the charges of the MPO bond channels (the
 * charge the operator string to the left of the bond has added).  The
 * two-site vector x[a, s1, s2, b] is PACKED: only its allowed blocks
 * (ia, s, ib), s = s1 + d1*s2, each column-major dim(ia) x dim(ib), in the
 * order ia fastest, then s, then ib.  All of these run FP64 (real only) on the
 * grouped persistent engine: one cooperative launch per contraction, CTAs
 * pulling 32x32 tiles of the uneven blocks from a device work counter, a
 * bounded grid barrier between the three steps (L*x, MPO step, *R). */
typedef struct fmpt_u1_space {
  int nsect;            /* number of sectors                     */
  const int* charge;    /* nsect charges, strictly increasing   */
  const int* dim;       /* nsect dimensions, each >= 1           */
} fmpt_u1_space;

/* Length (elements) of the packed two-site vector (host-only; h may be NULL). */
int fmpt_u1_twosite_size(fmpt_handle* h, const fmpt_u1_space* Vl, const fmpt_u1_space* Vr,
                         int d1, const int* qp1, int d2, const int* qp2, int64_t* n);
/* dense charge-sorted x[a, s1, s2, b] <-> packed (direction 0: pack, 1: unpack;
 * unpack writes the zeros too). */
int fmpt_u1_pack2(fmpt_handle* h, int dtype, const double* src, double* dst,
                  const fmpt_u1_space* Vl, const fmpt_u1_space* Vr, int d1, const int* qp1,
                  int d2, const int* qp2, int direction);
/* Block-sparse two-site H_eff operator (ac2_prime, derivatives.jl:20-22, on
 * U1Space tensors) for the Krylov solvers: fmpt_op_apply maps packed x to
 * packed y, fmpt_op_size is the packed length.  W1/W2 are HOST MPO tensors;
 * qwl/qwm/qwr the channel charges of their bonds; hleft [Dl, wl, Dl] and
 * hright [Dr, wr, Dr] device environments that must outlive the operator. */
int fmpt_u1_op_ac2(fmpt_handle* h, int dtype, const double* W1_host, const double* W2_host,
                   const double* hleft, const double* hright, const fmpt_u1_space* Vl,
                   const fmpt_u1_space* Vr, int d1, const int* qp1, int d2, const int* qp2,
                   int wl, const int* qwl, int wm, const int* qwm, int wr, const int* qwr,
                   fmpt_op** out);
/* Algorithmic FLOPs of one fmpt_op_apply (dense: the pairwise-order count
 * 4 w d^2 D^3-type formula of the operator's shape; U(1): the block-sparse
 * GEMM and MPO-step work of its block lists). */
int fmpt_op_flops(fmpt_op* op, double* flops);
/* x[a, s1, s2, b] (packed) = sum_m A[a, s1, m] B[m, s2, b]  (dmrg.jl:98). */
int fmpt_u1_twosite(fmpt_handle* h, int dtype, const double* A, const double* B, double* x,
                    const fmpt_u1_space* Vl, const fmpt_u1_space* Vm, const fmpt_u1_space* Vr,
                    int d1, const int* qp1, int d2, const int* qp2);
/* Environment updates (mpo/transfer.jl:26-34) on U(1) tensors: hold is
 * [Dl, wl, Dl] (left) or [Dr, wr, Dr] (right); A, B are [Dl, d, Dr]; the
 * output is written in full (zeros outside the allowed blocks). */
int fmpt_u1_updateleft(fmpt_handle* h, int dtype, const double* hold, const double* A,
                       const double* W_host, const double* B, double* hnew,
                       const fmpt_u1_space* Vl, const fmpt_u1_space* Vr, int d, const int* qp,
                       int wl, const int* qwl, int wr, const int* qwr);
int fmpt_u1_updateright(fmpt_handle* h, int dtype, const double* hold, const double* A,
                        const double* W_host, const double* B, double* hnew,
                        const fmpt_u1_space* Vl, const fmpt_u1_space* Vr, int d, const int* qp,
                        int wl, const int* qwl, int wr, const int* qwr);
/* Truncated two-site split of a packed x (stable_tsvd! + MPSTruncation,
 * stable_svd.jl:12-18, truncation.jl:27-47, with TensorKit's cross-sector
 * rule): each charge sector qc of the new bond, rows (s1, a) with
 * q(a) + qp1(s1) == qc and columns (s2, b) with q(b) - qp2(s2) == qc, is
 * factorised by an FP64 SVD on the device; then sigma below eps*||sigma||_2
 * (over all sectors) is dropped and at most maxD values are kept, largest
 * first (ties: lower charge first).  The kept sigma are normalised to unit
 * 2-norm (normalize!(s) of DMRG2) and returned in S; side 0 gives A = u
 * (left isometry) and B = s*v, side 1 gives A = u*s and B = v (right
 * isometry).  A is [Dl, d1, Dm'] and B [Dm', d2, Dr] in the new sorted basis,
 * written in full; size them for Dm' <= min(maxD, Dl*d1, d2*Dr).  HOST
 * outputs: the new leg (nsect_out sectors into charge_out/dim_out, capacity
 * cap) and err (2-norm of the dropped sigma before normalisation).
 * method 0: an SVD per sector (gesvd, gesvdj fallback: the reference's
 * stable_tsvd!).  method 1: the density-matrix form of fmpt_dm_split for
 * every sector at once -- all Gram matrices in one grouped launch, one
 * batched FP64 eigensolve per padded size; the isometric side is the exact
 * eigenvector set and the other factor a product with x (no division by
 * sigma); sigma below ~1e-8*sigma_max is resolved only to the FP64 noise of
 * the Gram matrix.  No counterpart in the reference. */
int fmpt_u1_split(fmpt_handle* h, int dtype, const double* x, const fmpt_u1_space* Vl,
                  const fmpt_u1_space* Vr, int d1, const int* qp1, int d2, const int* qp2,
                  int maxD, double eps, int side, int method, double* A, double* S, double* B,
                  int cap, int* nsect_out, int* charge_out, int* dim_out, double* err);

/* ------------------------------------- adjoint (reverse-mode) building blocks
 * For the differentiable one-site TDVP (gradients of an observable after a
 * TDVP trajectory with respect to the MPO couplings).  The reference has no
 * gradient code (ChainRulesCore is not one of its dependencies); these are the
 * backward counterparts of ac_prime (derivatives.jl:2-4), updateleft/right
 * (mpo/transfer.jl:26-34), leftorth!/rightorth (tdvp.jl:33,55) and the Krylov
 * exponential (tdvp.jl:3-6).  Cotangents follow zbar = dL/dRe z + i dL/dIm z.
 *
 * exp(s_j t H) x for nnodes values s_j (HOST array) from one Krylov space of
 * dimension krylovdim (<= 31) built from x; out holds nnodes vectors of the
 * operator's size one after another; err_est (HOST) the a-posteriori error
 * estimate relative to ||x||. */
int fmpt_expm_nodes(fmpt_op* op, double t_re, double t_im, const double* x, int krylovdim,
                    int nnodes, const double* nodes, double* out, double* err_est);
/* MPO-tensor gradient of Re<a, ac_prime(b, W, L, R)>:
 * out[w, s', w2, s] = conj(sum conj(a[a',s',b']) L[a',w,a] b[a,s,b] R[b',w2,b])
 * (device output, wl*d*wr*d elements). */
int fmpt_wgrad(fmpt_handle* h, int dtype, const double* a, const double* Lenv, const double* b,
               const double* Renv, double* out, int Dl, int d, int Dr, int wl, int wr);
/* dst(i, j) = src(i, j) for an m x n column-major block (leading dimensions lds,
 * ldd; complex split planes at the element offsets plane_src / plane_dst): the
 * catdomain / catcodomain concatenations of the subspace expansion. */
int fmpt_copy2d(fmpt_handle* h, int dtype, int m, int n, const double* src, int64_t lds,
                int64_t plane_src, double* dst, int64_t ldd, int64_t plane_dst);
/* dst[k, j, i] = src[i, j, k], conjugated when conj != 0 (out of place). */
int fmpt_swap13(fmpt_handle* h, int dtype, const double* src, double* dst, int n0, int n1, int n2,
                int conj);
/* Cotangent of M for the thin QR M = Q R (m >= n, real diagonal of R, the
 * fmpt_qr convention) given the cotangents Qbar (m x n) and Rbar (n x n);
 * complex (C128) only. */
int fmpt_qr_adjoint(fmpt_handle* h, int dtype, const double* Q, const double* R, const double* Qbar,
                    const double* Rbar, double* Mbar, int m, int n);

#ifdef __cplusplus
}
#endif
#endif /* FMPT_H */
