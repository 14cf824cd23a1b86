// FP64-accurate GEMM on the BF16 tensor cores (Ozaki scheme).
//
// GB300 runs FP64 on the CUDA cores at about 2 DFMA per clock per SM (~1.2 TFLOP/s for
// the whole chip) while its BF16 tensor cores run three orders of magnitude faster.  The
// plain-FP64 contractions therefore go through the error-free splitting of Ozaki, Ogita,
// Oishi and Rump (Numer. Algorithms 59, 2012):
//
//   1. every row r of op(A) (and every column n of op(B)) gets an exponent e with
//      max |row| < 2^(e - 1) (one bit of headroom), and its entries become NS = 9 balanced
//      base-64 digits,
//        X(r, k) = sum_i sigma_i(r, k) 2^(e_r - 6 i),   sigma_i integer, |sigma_i| <= 32,
//      exact to 2^(e_r - 54) (every FP64 entry in the top binade of its row is represented
//      exactly, smaller ones to 53 bits below the row maximum); the digits are computed with integer arithmetic on the FP64
//      bit pattern (no FP64 instruction; each digit's BF16 encoding comes from one exact
//      FP32 subtraction), and each one is an exact BF16 value;
//   2. the digit planes are multiplied on the tensor cores (tcgen05.mma kind::f16, BF16 x
//      BF16 -> FP32).  All products sigma_i tau_j with the same level l = i + j carry the
//      same scale 2^(e_r + e_n - 6 l), so they share one TMEM accumulator; the 45 products
//      with l <= NS + 1 are formed (the rest lie about 2^-53 below the row and column
//      maxima);
//   3. a level accumulator is an integer sum.  Its terms per k are bounded by
//      (l - 1) * 32 * 32, so over a K-chunk of up to 2^24 / bound(l) (16384 at l = 2 down
//      to 1820 at l = 10) it stays below 2^24 and FP32 accumulation is exact.  A level's K
//      range is cut into equal chunks of at most that length.  The one bit of headroom in
//      the exponent keeps every digit, the leading one included, within 32, which makes
//      these chunks up to 4x longer than with a leading digit of 64 (fewer epilogue
//      passes).  After each (level, chunk) the epilogue warps add the
//      accumulator, scaled by 2^(e_r + e_n - 6 l) (built in the FP64 exponent field with
//      integer operations), into the FP64 output.
//
// The result is op(A) op(B) to about 2^-53 relative to max|row| * max|column| per term:
// the accuracy class of an FP64 GEMM even for rows whose entries span a few decades
// (8 digits, 48 bits, measured 6e-13 on rows spanning e^+-3), at 45 BF16 MMAs per FP64
// multiply-add.  Complex operands use the real embedding [Re -Im; Im Re] x [Re; Im].
//
// Kernels: oz_rowmax / oz_digits (FP64 operand -> row exponents + 9 K-major BF16 digit
// planes, gridded over 32-row strips and 512-column K chunks), oz_gemm_pair (the CTA
// pair tcgen05 kernel of tc_gemm.cu with the (chunk, level, product) sequence and the
// FP64 epilogue), oz_reduce (sums split pieces in a fixed order, applies alpha / beta).
#include <algorithm>
#include <cmath>

#include "tc_ptx.cuh"

namespace fmpt {
namespace oz {

using namespace tc;

constexpr int NS = 9;                 // digits per entry
constexpr int SB = 6;                 // bits per digit
constexpr int NLEV = NS;              // levels 2 .. NS + 1
constexpr int NPROD = NS * (NS + 1) / 2;
constexpr int STAGES = 6;
constexpr int KELEMS = 64;            // BF16 elements per 128-byte K slice
constexpr int GH = 8;                 // tile rows per group of the tile order
constexpr int E_BAD = 1 << 20;        // exponent of a row or column holding Inf / NaN
constexpr int TILE = 256;             // pair tile edge

// Level sets of the pieces a tile's work is cut into (variant v: 1, 3 or 5 pieces; level l
// holds l - 1 digit products): the order the kernel visits the levels of a piece, and the
// piece boundaries in it.  Long and short groups alternate, so the epilogue's drain of one
// level overlaps the MMAs of the next.
constexpr int NVAR = 3;
__constant__ int kOrder[NVAR][NLEV] = {{10, 2, 6, 9, 3, 5, 8, 4, 7},
                                       {10, 2, 6, 9, 3, 5, 8, 4, 7},    // 15, 14, 16 products
                                       {10, 2, 9, 3, 8, 4, 7, 5, 6}};   // 10, 10, 10, 10, 5
__constant__ int kSetStart[NVAR][6] = {{0, 9}, {0, 3, 6, 9}, {0, 2, 4, 6, 8, 9}};
constexpr int kVarPieces[NVAR] = {1, 3, 5};
constexpr int kVarMaxProducts[NVAR] = {45, 16, 10};
static_assert(kVarMaxProducts[0] == NPROD, "one piece holds every digit product");

// ------------------------------------------------------------ digit planes
// op(X)(r, c) of a GEMM operand, real index space: X[r * sr + c * sc] (+ batch stride).
// Complex operands are embedded as real matrices with doubled extents: the A side as
// rows [Re, -Im] over [Im, Re], the B side (rows = output columns) as [Re, Im].
struct SliceSrc {
  const double* p;
  int64_t plane;        // offset of the imaginary plane
  int64_t sr, sc;       // element strides of row and column index
  int64_t bstride;      // batch stride
  int rows, cols;       // real extents of op(X)
  int cplx, role, conj; // role 0: A side, 1: B side
};

__device__ __forceinline__ uint64_t src_bits(const SliceSrc& s, int z, int r2, int c2) {
  int r = r2, c = c2, hr = 0, hc = 0;
  if (s.cplx) {
    if (s.role == 0 && r >= s.rows) { r -= s.rows; hr = 1; }
    if (c >= s.cols) { c -= s.cols; hc = 1; }
  }
  // the imaginary part sits at (hr, hc) = (0, 1) with a minus sign and at (1, 0) on the
  // A side, at hc = 1 on the B side; conj flips its sign once more
  bool im = false, neg = false;
  if (s.cplx) {
    if (s.role == 0) {
      im = hr != hc;
      neg = hr == 0 && hc == 1;
    } else {
      im = hc == 1;
    }
    if (im && s.conj) neg = !neg;
  }
  const double* b = s.p + (int64_t)z * s.bstride + (int64_t)r * s.sr + (int64_t)c * s.sc;
  uint64_t v = (uint64_t)__double_as_longlong(__ldg(b + (im ? s.plane : 0)));
  if (neg) v ^= 0x8000000000000000ull;
  return v;
}

// Balanced digits by offset binary: with B = 32 (2^42 + 2^36 + ... + 2^0), N + B written in
// base 64 has digit words u_i in [0, 64) below the top one, and
//   N = (N + B) >> 48 * 2^48 + sum_{i >= 2} (u_i - 32) 2^(54 - 6 i),
// so sigma_1 = (N + B) >> 48 (|sigma_1| <= 32 for |N| < 2^53) and sigma_i = u_i - 32 in
// [-32, 31]: one 64-bit add and bit-field extracts instead of NS rounding divisions.
constexpr int64_t kDigitBias = 0x820820820820ll;
static_assert(NS == 9 && SB == 6, "the digit extraction below is written for 9 digits of 6 bits");

constexpr int SL_ROWS = 32;           // rows of a slicing block
constexpr int SL_KCH = 512;           // K columns of a slicing block (8 tiles of 64)

// A 32 x 64 tile of op(X) bit patterns: element e = t + 256 q of thread t (q < 8) is
// (row, column) = (e & 31, e >> 5) when rows are contiguous in the source and
// (e >> 6, e & 63) otherwise, so that every warp load is contiguous; zeros outside the
// operand.  The loads go to registers first, so that a block can fetch its next tile
// while it works on the current one.
__device__ __forceinline__ void tile_pos(bool rowfast, int e, int& lr, int& lc) {
  if (rowfast) { lr = e & 31; lc = e >> 5; } else { lc = e & 63; lr = e >> 6; }
}

__device__ __forceinline__ void fetch_tile(const SliceSrc& src, int z, int r0, int c0, int rows_out,
                                           int k_out, uint64_t (&v)[8]) {
  const int t = threadIdx.x;
  const bool rowfast = src.sr == 1;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    int lr, lc;
    tile_pos(rowfast, t + 256 * q, lr, lc);
    const int r = r0 + lr, c = c0 + lc;
    v[q] = (r < rows_out && c < k_out) ? src_bits(src, z, r, c) : 0ull;
  }
}

// Row maxima of |X| on the bit patterns (non-negative IEEE doubles order as their bits):
// block (strip, K chunk, batch) reduces its 32 x SL_KCH part and folds it into mx with an
// atomic max (mx zeroed beforehand).
__global__ void __launch_bounds__(256, 4) oz_rowmax(SliceSrc src, int rows_out, int k_out,
                                                 unsigned long long* __restrict__ mx) {
  __shared__ unsigned long long smax[SL_ROWS];
  const int r0 = blockIdx.x * SL_ROWS, kc0 = blockIdx.y * SL_KCH, z = blockIdx.z;
  const int t = threadIdx.x;
  const bool rowfast = src.sr == 1;
  if (t < SL_ROWS) smax[t] = 0ull;
  // rows of this thread's elements: one row (rowfast) or rows (t >> 6) + 4 q
  uint64_t m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int c1 = min(kc0 + SL_KCH, k_out);
  uint64_t v[8];
  if (kc0 < c1) fetch_tile(src, z, r0, kc0, rows_out, k_out, v);
  for (int c0 = kc0; c0 < c1; c0 += 64) {
    uint64_t cur[8];
#pragma unroll
    for (int q = 0; q < 8; q++) cur[q] = v[q] & 0x7fffffffffffffffull;
    if (c0 + 64 < c1) fetch_tile(src, z, r0, c0 + 64, rows_out, k_out, v);
#pragma unroll
    for (int q = 0; q < 8; q++) m[q] = cur[q] > m[q] ? cur[q] : m[q];
  }
  __syncthreads();
  if (rowfast) {
    uint64_t a = m[0];
#pragma unroll
    for (int q = 1; q < 8; q++) a = m[q] > a ? m[q] : a;
    if (a) atomicMax(&smax[t & 31], (unsigned long long)a);
  } else {
    // the 64 threads of a row group share their rows: fold across the warp's halves
#pragma unroll
    for (int q = 0; q < 8; q++) {
      uint64_t a = m[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_xor_sync(0xffffffffu, a, o);
        a = y > a ? y : a;
      }
      if ((t & 31) == 0 && a) atomicMax(&smax[(t >> 6) + 4 * q], (unsigned long long)a);
    }
  }
  __syncthreads();
  const int r = r0 + t;
  if (t < SL_ROWS && r < rows_out && smax[t] != 0) atomicMax(mx + (int64_t)z * rows_out + r, smax[t]);
}

// Digits: block (strip, K chunk, batch) writes NS BF16 planes of its 32 x SL_KCH part
// (zeros in the padding up to ldk); the chunk-0 blocks write the row exponents.
// S[(z NS + i) rows_out + r][ldk] (K-major), E[z rows_out + r].  Each 32 x 64 tile goes
// through a double-buffered shared tile (one barrier per tile); thread (rr, part) then
// turns 8 consecutive K entries of row rr into 16-byte stores, one per digit plane.
__global__ void __launch_bounds__(256, 3) oz_digits(SliceSrc src, int rows_out, int k_out, int ldk,
                                                 const unsigned long long* __restrict__ mxa,
                                                 uint16_t* __restrict__ S, int* __restrict__ E) {
  __shared__ uint64_t tile[2][SL_ROWS][65];
  const int r0 = blockIdx.x * SL_ROWS, kc0 = blockIdx.y * SL_KCH, z = blockIdx.z;
  const int t = threadIdx.x, rr = t >> 3, part = t & 7;
  const bool rowfast = src.sr == 1;
  const int r = r0 + rr;
  const uint64_t mx = r < rows_out ? mxa[(int64_t)z * rows_out + r] : 0ull;
  const int exm = (int)(mx >> 52);
  const bool bad = exm == 0x7ff;
  // max |row| = f 2^(e - 1) with f in [0.5, 1): e = exm - 1021 for normal numbers (one
  // bit of headroom, so that |N| < 2^53 and every digit lies within 32); the subnormal
  // exponent field 0 behaves as 1 with no implicit bit (then max < 2^-1022)
  const int e = mx == 0 ? 0 : (exm == 0 ? -1020 : exm - 1021);
  if (blockIdx.y == 0 && part == 0 && r < rows_out) E[(int64_t)z * rows_out + r] = bad ? E_BAD : e;
  const int64_t plane_stride = (int64_t)rows_out * ldk;
  uint16_t* out = S + ((int64_t)z * NS * rows_out + r) * ldk;
  const int c1 = min(kc0 + SL_KCH, ldk);
  uint64_t v[8];
  if (kc0 < c1) fetch_tile(src, z, r0, kc0, rows_out, k_out, v);
  int buf = 0;
  for (int c0 = kc0; c0 < c1; c0 += 64, buf ^= 1) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      int lr, lc;
      tile_pos(rowfast, t + 256 * q, lr, lc);
      tile[buf][lr][lc] = v[q];
    }
    __syncthreads();
    if (c0 + 64 < c1) fetch_tile(src, z, r0, c0 + 64, rows_out, k_out, v);
    const int cb = c0 + part * 8;
    if (r < rows_out && cb < ldk) {
      // N + kDigitBias of the 8 entries, N = X 2^(54 - e) as an integer (|N| < 2^54)
      uint64_t Mo[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const uint64_t bits = bad ? 0ull : tile[buf][rr][part * 8 + q];
        const int ex = (int)((bits >> 52) & 0x7ff);
        int64_t N = (int64_t)(bits & 0xfffffffffffffull);
        if (ex) N |= (int64_t)1 << 52;
        const int sh = (ex ? ex : 1) - 1021 - e;          // max(ex, 1) - 1075 + 54 - e
        if (sh >= 0) N <<= sh;                            // sh <= 1
        else N = sh <= -63 ? 0 : (N >> (-sh));
        if (bits >> 63) N = -N;
        Mo[q] = (uint64_t)(N + kDigitBias);
      }
      // digit i of each entry: word 0 the arithmetic top of N + kDigitBias, word i >= 1
      // its bits [54 - 6 (i + 1), + 6) minus 32; the BF16 encoding is the upper half of the
      // exact FP32 value (2^23 + u) - (2^23 + bias)
#pragma unroll
      for (int i = 0; i < NS; i++) {
        uint32_t fb[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          if (i == 0) {
            const int d0 = (int)(uint32_t)(Mo[q] >> 32) >> 16;
            fb[q] = __float_as_uint(__uint_as_float(0x4B000000u | (uint32_t)(d0 + 64)) -
                                    8388672.0f);
          } else {
            const uint32_t u = (uint32_t)(Mo[q] >> (54 - SB * (i + 1))) & 63u;
            fb[q] = __float_as_uint(__uint_as_float(0x4B000000u | u) - 8388640.0f);
          }
        }
        *reinterpret_cast<uint4*>(out + i * plane_stride + cb) =
            make_uint4(__byte_perm(fb[0], fb[1], 0x7632), __byte_perm(fb[2], fb[3], 0x7632),
                       __byte_perm(fb[4], fb[5], 0x7632), __byte_perm(fb[6], fb[7], 0x7632));
      }
    }
  }
}

// ------------------------------------------------------------ fast slicing of real operands
// Real operands whose row or K index has unit stride (with 16-byte aligned rows or columns)
// take these kernels instead of the generic ones above: 16-byte loads, eight independent
// loads in flight per thread and no shared-memory staging for the row maxima, the digits
// of a K-contiguous operand straight from registers.  The generic kernels are bound by
// memory latency (long-scoreboard stalls, 22-37% of DRAM bandwidth).
constexpr int RM_KCH = 128;           // K columns per block, row-contiguous row maxima
constexpr int RK_KCH = 1024;          // K columns per block, K-contiguous row maxima

// rows r, r + 1 of a row-contiguous operand (element (r, c) at p[r + c ld])
__global__ void __launch_bounds__(256) oz_rowmax_rowfast(const double* __restrict__ p, int64_t ld,
                                                         int64_t bstride, int rows, int k,
                                                         unsigned long long* __restrict__ mx) {
  const int z = blockIdx.z;
  const int r = (blockIdx.x * 256 + threadIdx.x) * 2;
  const int c0 = blockIdx.y * RM_KCH, c1 = min(c0 + RM_KCH, k);
  if (r >= rows) return;
  const double* b = p + (int64_t)z * bstride + r;
  uint64_t m0 = 0, m1 = 0;
  for (int c = c0; c < c1; c += 8) {
    double2 v[8];
#pragma unroll
    for (int u = 0; u < 8; u++)
      v[u] = c + u < c1 ? __ldg(reinterpret_cast<const double2*>(b + (int64_t)(c + u) * ld))
                        : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const uint64_t a0 = (uint64_t)__double_as_longlong(v[u].x) & 0x7fffffffffffffffull;
      const uint64_t a1 = (uint64_t)__double_as_longlong(v[u].y) & 0x7fffffffffffffffull;
      m0 = a0 > m0 ? a0 : m0;
      m1 = a1 > m1 ? a1 : m1;
    }
  }
  if (m0) atomicMax(mx + (int64_t)z * rows + r, (unsigned long long)m0);
  if (m1) atomicMax(mx + (int64_t)z * rows + r + 1, (unsigned long long)m1);
}

// one warp per row of a K-contiguous operand (element (r, c) at p[r ld + c])
__global__ void __launch_bounds__(256) oz_rowmax_kfast(const double* __restrict__ p, int64_t ld,
                                                       int64_t bstride, int rows, int k,
                                                       unsigned long long* __restrict__ mx) {
  const int z = blockIdx.z, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= rows) return;                                   // uniform over the warp
  const int c0 = blockIdx.y * RK_KCH, c1 = min(c0 + RK_KCH, k);
  const double* b = p + (int64_t)z * bstride + (int64_t)r * ld;
  uint64_t m = 0;
  for (int c = c0 + 2 * lane; c < c1; c += 64 * 8) {
    double2 v[8];
#pragma unroll
    for (int u = 0; u < 8; u++)
      v[u] = c + 64 * u < c1 ? __ldg(reinterpret_cast<const double2*>(b + c + 64 * u))
                             : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const uint64_t a0 = (uint64_t)__double_as_longlong(v[u].x) & 0x7fffffffffffffffull;
      const uint64_t a1 = (uint64_t)__double_as_longlong(v[u].y) & 0x7fffffffffffffffull;
      m = a0 > m ? a0 : m;
      m = a1 > m ? a1 : m;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  if (lane == 0 && m) atomicMax(mx + (int64_t)z * rows + r, (unsigned long long)m);
}

// exponent of a row from its maximum's bit pattern (as oz_digits): e, and whether the row
// holds Inf/NaN
__device__ __forceinline__ int row_exponent(uint64_t mx, bool& bad) {
  const int exm = (int)(mx >> 52);
  bad = exm == 0x7ff;
  return mx == 0 ? 0 : (exm == 0 ? -1020 : exm - 1021);
}

// the NS digit planes of 8 consecutive K entries of one row: 16-byte stores at out + cb
__device__ __forceinline__ void slice8_store(const uint64_t (&bits8)[8], int e, bool bad,
                                             uint16_t* __restrict__ out, int64_t plane_stride,
                                             int cb) {
  uint64_t Mo[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const uint64_t bits = bad ? 0ull : bits8[q];
    const int ex = (int)((bits >> 52) & 0x7ff);
    int64_t N = (int64_t)(bits & 0xfffffffffffffull);
    if (ex) N |= (int64_t)1 << 52;
    const int sh = (ex ? ex : 1) - 1021 - e;
    if (sh >= 0) N <<= sh;
    else N = sh <= -63 ? 0 : (N >> (-sh));
    if (bits >> 63) N = -N;
    Mo[q] = (uint64_t)(N + kDigitBias);
  }
#pragma unroll
  for (int i = 0; i < NS; i++) {
    uint32_t fb[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (i == 0) {
        const int d0 = (int)(uint32_t)(Mo[q] >> 32) >> 16;
        fb[q] = __float_as_uint(__uint_as_float(0x4B000000u | (uint32_t)(d0 + 64)) - 8388672.0f);
      } else {
        const uint32_t u = (uint32_t)(Mo[q] >> (54 - SB * (i + 1))) & 63u;
        fb[q] = __float_as_uint(__uint_as_float(0x4B000000u | u) - 8388640.0f);
      }
    }
    *reinterpret_cast<uint4*>(out + i * plane_stride + cb) =
        make_uint4(__byte_perm(fb[0], fb[1], 0x7632), __byte_perm(fb[2], fb[3], 0x7632),
                   __byte_perm(fb[4], fb[5], 0x7632), __byte_perm(fb[6], fb[7], 0x7632));
  }
}

// Digits of a K-contiguous operand: thread (rr, part) of a block owns row r0 + rr and, per
// 64-column tile, the 8 entries from part * 8; two tiles' loads are in flight at once.
__global__ void __launch_bounds__(256) oz_digits_kfast(const double* __restrict__ p, int64_t ld,
                                                       int64_t bstride, int rows_out, int k_out,
                                                       int ldk,
                                                       const unsigned long long* __restrict__ mxa,
                                                       uint16_t* __restrict__ S,
                                                       int* __restrict__ E) {
  const int r0 = blockIdx.x * SL_ROWS, kc0 = blockIdx.y * SL_KCH, z = blockIdx.z;
  const int t = threadIdx.x, rr = t >> 3, part = t & 7;
  const int r = r0 + rr;
  if (r >= rows_out) return;
  bool bad;
  const int e = row_exponent(mxa[(int64_t)z * rows_out + r], bad);
  if (blockIdx.y == 0 && part == 0) E[(int64_t)z * rows_out + r] = bad ? E_BAD : e;
  const int64_t plane_stride = (int64_t)rows_out * ldk;
  uint16_t* out = S + ((int64_t)z * NS * rows_out + r) * ldk;
  const double* b = p + (int64_t)z * bstride + (int64_t)r * ld;
  const int c1 = min(kc0 + SL_KCH, ldk);
  for (int c0 = kc0; c0 < c1; c0 += 128) {
    double2 v[2][4];
#pragma unroll
    for (int hh = 0; hh < 2; hh++)
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int cc = c0 + 64 * hh + part * 8 + 2 * u;
        v[hh][u] = cc < k_out ? __ldg(reinterpret_cast<const double2*>(b + cc))
                              : make_double2(0.0, 0.0);
      }
#pragma unroll
    for (int hh = 0; hh < 2; hh++) {
      const int cb = c0 + 64 * hh + part * 8;
      if (cb >= c1) break;
      uint64_t bits8[8];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        bits8[2 * u] = (uint64_t)__double_as_longlong(v[hh][u].x);
        bits8[2 * u + 1] = (uint64_t)__double_as_longlong(v[hh][u].y);
      }
      slice8_store(bits8, e, bad, out, plane_stride, cb);
    }
  }
}

// Digits of a row-contiguous operand (element (r, c) at p[r + c ld]): the 32 x 64 tiles of
// the block's K chunk stream into a 3-stage shared-memory ring by 8-byte cp.async copies
// (two tiles in flight, no registers held for them), and thread (rr, part) turns 8
// consecutive K entries of row rr into one 16-byte store per digit plane.
constexpr int DR_STAGES = 3;
constexpr size_t DR_SMEM = (size_t)DR_STAGES * SL_ROWS * 65 * sizeof(uint64_t);

__device__ __forceinline__ void cp_async8(uint64_t* dst, const double* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(256) oz_digits_rowfast(const double* __restrict__ p, int64_t ld,
                                                         int64_t bstride, int rows_out,
                                                         int k_out, int ldk,
                                                         const unsigned long long* __restrict__ mxa,
                                                         uint16_t* __restrict__ S,
                                                         int* __restrict__ E) {
  extern __shared__ __align__(16) uint64_t dr_smem[];
  auto tile = [&](int st, int lr, int lc) -> uint64_t& {
    return dr_smem[((size_t)st * SL_ROWS + lr) * 65 + lc];
  };
  const int r0 = blockIdx.x * SL_ROWS, kc0 = blockIdx.y * SL_KCH, z = blockIdx.z;
  const int t = threadIdx.x, rr = t >> 3, part = t & 7;
  const int r = r0 + rr;
  bool bad = false;
  const int e = r < rows_out ? row_exponent(mxa[(int64_t)z * rows_out + r], bad) : 0;
  if (blockIdx.y == 0 && part == 0 && r < rows_out) E[(int64_t)z * rows_out + r] = bad ? E_BAD : e;
  const int64_t plane_stride = (int64_t)rows_out * ldk;
  uint16_t* out = S + ((int64_t)z * NS * rows_out + r) * ldk;
  const double* b = p + (int64_t)z * bstride;
  const int c1 = min(kc0 + SL_KCH, ldk);
  const int ntile = (c1 - kc0 + 63) / 64;
  // tile j of the chunk into stage j % DR_STAGES: lanes run along rows (contiguous)
  auto issue = [&](int j) {
    if (j < ntile) {
      const int c0 = kc0 + 64 * j, st = j % DR_STAGES;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int e2 = t + 256 * q, lr = e2 & 31, lc = e2 >> 5;
        const int rg = r0 + lr, cg = c0 + lc;
        if (rg < rows_out && cg < k_out)
          cp_async8(&tile(st, lr, lc), b + rg + (int64_t)cg * ld);
        else
          tile(st, lr, lc) = 0ull;
      }
    }
    cp_async_commit();                      // one group per tile slot (empty past the end)
  };
  issue(0);
  issue(1);
  for (int j = 0; j < ntile; j++) {
    issue(j + 2);
    cp_async_wait<2>();                     // this thread's copies of tile j have landed
    __syncthreads();                        // and every thread's
    const int cb = kc0 + 64 * j + part * 8;
    if (r < rows_out && cb < c1) {
      uint64_t bits8[8];
#pragma unroll
      for (int q = 0; q < 8; q++) bits8[q] = tile(j % DR_STAGES, rr, part * 8 + q);
      slice8_store(bits8, e, bad, out, plane_stride, cb);
    }
    __syncthreads();                        // stage j % 3 is refilled by issue(j + 3)
  }
}

// ------------------------------------------------------------ GEMM kernel
struct OzEpi {
  double* C;            // direct: output; split: workspace tiles [item][256 cols][256 rows]
  int64_t ldc, strideC, planeC;
  int M, N, mh;         // rows >= mh of the real embedding go to the imaginary plane
  const int* ea;        // [batch][M] row exponents
  const int* eb;        // [batch][N] column exponents
  double alpha;         // direct mode only
  int* err;
  int nfast;
  int split;            // pieces per tile: S level sets x Q chunk ranges (1: direct)
  int var, S, Q;        // level-set variant (kOrder / kSetStart), S = its piece count
};

// K slices (of KELEMS) per exactness chunk of a level: the longest run of K over which the
// level's integer sum stays below 2^24 (per-k bound (l - 1) 32 32)
__host__ __device__ constexpr int level_chunk_slices(int level) {
  return (1 << 24) / ((level - 1) * 32 * 32) / KELEMS;
}
static_assert(level_chunk_slices(2) == 256 && level_chunk_slices(10) == 28, "chunk lengths");

// chunk ch of nch equal chunks of the K slices [k0, k1) (nch = ceil((k1 - k0) / kcs), so
// every chunk is at most kcs long and none is a short tail)
__device__ __forceinline__ int level_chunks(int k0, int k1, int kcs) {
  return (k1 - k0 + kcs - 1) / kcs;
}
__device__ __forceinline__ int chunk_edge(int k0, int k1, int nch, int ch) {
  return k0 + (int)((int64_t)(k1 - k0) * ch / nch);
}

// tile unit -> (mt2, nt, z): groups of GH tile rows, column by column inside a group, so the
// clusters running at the same time share the digit planes of few A row blocks and few B
// column blocks in L2
__host__ __device__ inline void oz_tile(int u, int tiles_m2, int tiles_n, int& mt2, int& nt,
                                        int& z) {
  const int per = tiles_m2 * tiles_n;
  z = u / per;
  const int r = u - z * per;
  const int g = r / (GH * tiles_n);
  const int rows = min(GH, tiles_m2 - g * GH);
  const int idx = r - g * GH * tiles_n;
  mt2 = g * GH + idx % rows;
  nt = idx / rows;
}

__host__ __device__ inline int oz_unit(int mt2, int nt, int z, int tiles_m2, int tiles_n) {
  const int g = mt2 / GH;
  const int rows = min(GH, tiles_m2 - g * GH);
  return z * tiles_m2 * tiles_n + g * GH * tiles_n + nt * rows + (mt2 - g * GH);
}

// the levels of piece lp of variant v: kOrder[v][l0 .. l0 + nl)
__device__ __forceinline__ void piece_levels(int v, int lp, int& l0, int& nl) {
  l0 = kSetStart[v][lp];
  nl = kSetStart[v][lp + 1] - l0;
}

// x 2^E of an FP32 integer value outside the exponent range of the fast path
__device__ __noinline__ double scaled_slow(uint32_t u, int E) {
  if ((u << 1) == 0) return 0.0;
  return ldexp((double)__uint_as_float(u), E);
}

// Adds the level accumulator (TMEM lanes of this warp: 32 rows x 256 columns), scaled by
// 2^(e_r + e_n - 6 level), into the FP64 output tile (first group: stores it).  A chunk of
// 32 columns whose row and column exponents all lie in (-400, 400), with every row and
// column inside the output, takes the fast path: the FP64 value is assembled in the
// exponent field with integer operations and no branch, and the only FP64 instruction is
// the add.  Other chunks (a ragged edge, Inf/NaN rows or columns, extreme exponents) take
// the general path.
template <bool SPLIT>
__device__ __forceinline__ void drain(uint32_t tbase, int row, int rloc, int n0, int z,
                                      int level, bool first, bool last, const OzEpi& ep,
                                      double* wtile) {
  const bool live = row < ep.M;
  double* crow;
  int64_t ld;
  if (SPLIT) {
    crow = wtile + rloc;
    ld = TILE;
  } else {
    crow = ep.C + (int64_t)z * ep.strideC + (row < ep.mh ? (int64_t)row : ep.planeC + row - ep.mh);
    ld = ep.ldc;
  }
  const int er = live ? __ldg(ep.ea + (int64_t)z * ep.M + row) : 0;
  const int eb = er - SB * level;
  const bool scale = !SPLIT && last && ep.alpha != 1.0;
  const int lane = threadIdx.x & 31;
#pragma unroll 1
  for (int c0 = 0; c0 < TILE; c0 += 32) {
    uint32_t r[32];
    tmem_ld32_async(tbase + c0, r);
    const int nb = n0 + c0;
    const int ec = nb + lane < ep.N ? __ldg(ep.eb + (int64_t)z * ep.N + nb + lane) : 0;
    const int lim = SPLIT ? 32 : min(32, ep.N - nb);
    double* p = crow + (int64_t)(SPLIT ? c0 : nb) * ld;
    double old[32];
    if (!first && live) {
#pragma unroll
      for (int j = 0; j < 32; j++) old[j] = j < lim ? p[j * ld] : 0.0;
    }
    const bool fast =
        __all_sync(0xffffffffu, live && er > -400 && er < 400 && ec > -400 && ec < 400) &&
        lim == 32;
    tmem_wait_ld(r);
    if (fast) {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int E = eb + __shfl_sync(0xffffffffu, ec, j);
        const uint32_t u = r[j];
        const uint32_t hi = (u & 0x80000000u) |
                            ((((u >> 23) & 0xffu) + (uint32_t)(896 + E)) << 20) |
                            ((u & 0x7fffffu) >> 3);
        double v = (u << 1) == 0 ? 0.0 : __hiloint2double((int)hi, (int)(u << 29));
        if (!first) v += old[j];
        if (scale) v *= ep.alpha;
        p[j * ld] = v;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int ecj = __shfl_sync(0xffffffffu, ec, j);
        if (!live || j >= lim) continue;
        double v;
        if (er >= E_BAD || ecj >= E_BAD) {
          v = __longlong_as_double(0x7ff8000000000000ll);
        } else {
          const int E = eb + ecj;
          const uint32_t u = r[j];
          if (E >= -1000 && E <= 990) {
            const uint32_t hi = (u & 0x80000000u) |
                                ((((u >> 23) & 0xffu) + (uint32_t)(896 + E)) << 20) |
                                ((u & 0x7fffffu) >> 3);
            v = (u << 1) == 0 ? 0.0 : __hiloint2double((int)hi, (int)(u << 29));
          } else {
            v = scaled_slow(u, E);
          }
        }
        if (!first) v += old[j];
        if (scale) v *= ep.alpha;
        p[j * ld] = v;
      }
    }
  }
}

// Persistent over work items (tile, piece); cluster c of two CTAs takes items c, c + ncl..
// Per item the producer and the MMA issuer walk the same sequence:
//   for chunk in the piece's chunk range, for level in its level set, for i in 1..level-1
//   (j = level - i), for the chunk's K slices: A digit plane i-1, B digit plane j-1.
// Each (chunk, level) group accumulates in one TMEM buffer (two, alternating) and is
// drained by the epilogue warps into the FP64 output.
__global__ void __launch_bounds__(NTHREADS, 1)
    oz_gemm_pair(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                 int K, int tiles_m2, int tiles_n, int batch, OzEpi ep) {
  constexpr int A_BYTES = BM * 128, B_BYTES = 128 * 128;
  constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  constexpr int TMEM_COLS = 256;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = bars + 2 * STAGES + 2;
  uint64_t* drainb = bars + 2 * STAGES + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t rank = cluster_rank();
  const bool lead = rank == 0;
  const int cl = blockIdx.x >> 1, ncl = gridDim.x >> 1;
  const int nk = (K + KELEMS - 1) / KELEMS;
  const int units = tiles_m2 * tiles_n * batch;
  const int num_items = units * ep.split;
  auto stageA = [&](int s) { return smem + s * STAGE_BYTES; };
  auto stageB = [&](int s) { return stageA(s) + A_BYTES; };
  // item -> tile unit u, level set [l0, l0 + nl) of kOrder[ep.var], K slices [k0, k1).
  // Items run K-range-major: (K range cq, tile unit u, level set lp), so the clusters that
  // run at one time cover many tiles over ONE K range and read 1/Q of those tiles' digit
  // planes (a split GEMM 2 at D=2048 reads 30 GB from DRAM per launch instead of 42 GB)
  auto item_of = [&](int item, int& u, int& l0, int& nl, int& k0, int& k1) {
    const int us = units * ep.S;
    const int cq = item / us;
    const int rem = item - cq * us;
    u = rem / ep.S;
    const int lp = rem - u * ep.S;
    piece_levels(ep.var, lp, l0, nl);
    k0 = (int)((int64_t)cq * nk / ep.Q);
    k1 = (int)((int64_t)(cq + 1) * nk / ep.Q);
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[STAGES + s]), 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&acc_full[b]), 1);
      mbar_init(smem_u32(&acc_empty[b]), 8);
    }
    mbar_init(smem_u32(drainb), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int it = 0, last = -1;
      bool stop = false;
      for (int item = cl; item < num_items && !stop && !*abort_flag; item += ncl) {
        int u, l0, nl, k0, k1, mt2, nt, z;
        item_of(item, u, l0, nl, k0, k1);
        oz_tile(u, tiles_m2, tiles_n, mt2, nt, z);
        const int m0 = min(mt2 * 2 * BM + (int)rank * BM, ep.M - 1);
        const int n0 = min(nt * TILE + (int)rank * 128, ep.N - 1);
        for (int li = 0; li < nl && !stop; li++) {
          const int level = kOrder[ep.var][l0 + li];
          const int nch = level_chunks(k0, k1, level_chunk_slices(level));
          for (int ch = 0; ch < nch && !stop; ch++) {
            const int kb0 = chunk_edge(k0, k1, nch, ch), kb1 = chunk_edge(k0, k1, nch, ch + 1);
            for (int i = 1; i < level && !stop; i++) {
              const int za = z * NS + i - 1, zb = z * NS + (level - i) - 1;
              for (int kb = kb0; kb < kb1; kb++, it++) {
                const int s = it % STAGES;
                const uint32_t ph = (it / STAGES) & 1;
                if (!mbar_wait(smem_u32(&bars[STAGES + s]), ph ^ 1, abort_flag, ep.err)) {
                  stop = true;
                  break;
                }
                const uint32_t full = smem_u32(&bars[s]);
                if (lead) mbar_expect_tx(full, 2 * STAGE_BYTES);
                const uint32_t full_lead = cluster_addr(full, 0);
                const int kc = kb * KELEMS;
                tma_load_3d_pair(smem_u32(stageA(s)), &mapA, full_lead, kc, m0, za);
                tma_load_3d_pair(smem_u32(stageB(s)), &mapB, full_lead, kc, n0, zb);
                last = it;
              }
            }
          }
        }
      }
      if (*abort_flag && last >= 0) {
        const unsigned long long t0 = globaltimer();
        if (lead) {
          for (int j = max(0, last - STAGES + 1); j <= last; j++) {
            const uint32_t bar = smem_u32(&bars[j % STAGES]);
            while (!mbar_try(bar, (j / STAGES) & 1) && globaltimer() - t0 < WAIT_NS) {
            }
          }
        } else {
          while (globaltimer() - t0 < 1000000ull) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      constexpr uint32_t idesc = make_idesc(BF16, 2 * BM, TILE);
      int it = 0, local = 0;
      bool stop = false;
      for (int item = cl; item < num_items && !stop && !*abort_flag; item += ncl) {
        int u, l0, nl, k0, k1;
        item_of(item, u, l0, nl, k0, k1);
        for (int li = 0; li < nl && !stop; li++) {
          const int level = kOrder[ep.var][l0 + li];
          const int nch = level_chunks(k0, k1, level_chunk_slices(level));
          for (int ch = 0; ch < nch && !stop; ch++, local++) {
            const int kb0 = chunk_edge(k0, k1, nch, ch), kb1 = chunk_edge(k0, k1, nch, ch + 1);
            const int buf = local & 1;
            const uint32_t use = (uint32_t)(local >> 1);
            if (!mbar_wait(smem_u32(&acc_empty[buf]), (use & 1) ^ 1, abort_flag, ep.err)) {
              stop = true;
              break;
            }
            tc_fence_after();
            const uint32_t tacc = tmem + buf * TMEM_COLS;
            for (int i = 1; i < level && !stop; i++) {
              for (int kb = kb0; kb < kb1; kb++, it++) {
                const int s = it % STAGES;
                const uint32_t ph = (it / STAGES) & 1;
                if (!mbar_wait(smem_u32(&bars[s]), ph, abort_flag, ep.err)) {
                  stop = true;
                  break;
                }
                tc_fence_after();
                const uint32_t a0 = smem_u32(stageA(s)), b0 = smem_u32(stageB(s));
#pragma unroll
                for (int ks = 0; ks < 4; ks++) {
                  const uint32_t acc = (i > 1 || kb > kb0 || ks > 0) ? 1u : 0u;
                  mma_pair<BF16>(tacc, smem_desc(a0 + ks * 32), smem_desc(b0 + ks * 32), idesc, acc);
                }
                mma_commit_pair(smem_u32(&bars[STAGES + s]), 3);
              }
            }
            if (!stop) mma_commit_pair(smem_u32(&acc_full[buf]), 3);
          }
        }
      }
    }
  } else {
    const int q = warp & 3;
    int local = 0;
    bool stop = false;
    for (int item = cl; item < num_items && !stop; item += ncl) {
      int u, l0, nl, k0, k1, mt2, nt, z;
      item_of(item, u, l0, nl, k0, k1);
      oz_tile(u, tiles_m2, tiles_n, mt2, nt, z);
      const int rloc = (int)rank * BM + 32 * q + lane;
      const int row = mt2 * 2 * BM + rloc;
      double* wtile = ep.split > 1 || ep.mh < 0 ? ep.C + (int64_t)item * TILE * TILE : nullptr;
      for (int li = 0; li < nl && !stop; li++) {
        const int level = kOrder[ep.var][l0 + li];
        const int nch = level_chunks(k0, k1, level_chunk_slices(level));
        for (int ch = 0; ch < nch; ch++, local++) {
          const int buf = local & 1;
          const uint32_t use = (uint32_t)(local >> 1);
          const bool ok = mbar_wait(smem_u32(&acc_full[buf]), use & 1, abort_flag, ep.err);
          if (!ok || *abort_flag) {
            stop = true;
            break;
          }
          tc_fence_after();
          const uint32_t tbase = tmem + buf * TMEM_COLS + ((uint32_t)(32 * q) << 16);
          const bool first = li == 0 && ch == 0;
          const bool lastg = li == nl - 1 && ch == nch - 1;
          if (wtile)
            drain<true>(tbase, row, rloc, nt * TILE, z, level, first, lastg, ep, wtile);
          else
            drain<false>(tbase, row, rloc, nt * TILE, z, level, first, lastg, ep, nullptr);
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_cluster(cluster_addr(smem_u32(&acc_empty[buf]), 0));
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1 && lead) {
    tc_fence_after();
    if (lane == 0) {
      mma_commit_pair(smem_u32(drainb), 1);
      const unsigned long long t0 = globaltimer();
      while (!mbar_try(smem_u32(drainb), 0) && globaltimer() - t0 < WAIT_NS) {
      }
    }
    __syncwarp();
  }
  cluster_sync();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * TMEM_COLS)
                 : "memory");
  }
}

// C = alpha (sum of the pieces, in piece order) + beta C.  ws holds the pieces of tile
// unit u at items u * split + p, each [256 columns][256 rows] of the real embedding.
struct RedArgs {
  const double* ws;
  double* C;
  int64_t ldc, strideC, planeC;
  int m, n, batch, cplx, split, S, tiles_m2, tiles_n, nfast;
  double alpha[2], beta[2];
};

__device__ __forceinline__ double ws_sum(const RedArgs& a, int z, int r, int c) {
  // unit index of the tile holding (r, c) under the kernel's tile order
  const int mt2 = r / TILE, nt = c / TILE;
  const int units = a.tiles_m2 * a.tiles_n * a.batch;
  const int u = oz_unit(mt2, nt, z, a.tiles_m2, a.tiles_n);
  const double* w = a.ws + (int64_t)(c % TILE) * TILE + r % TILE;
  // piece p = lp + S cq of unit u sits at item (cq units + u) S + lp (K-range-major);
  // summed in piece order
  double s = 0.0;
  for (int p = 0; p < a.split; p++) {
    const int lp = p % a.S, cq = p / a.S;
    const int64_t item = ((int64_t)cq * units + u) * a.S + lp;
    s += w[item * TILE * TILE];
  }
  return s;
}

__global__ void oz_reduce(RedArgs a) {
  const int64_t mn = (int64_t)a.m * a.n;
  const int64_t total = mn * a.batch;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(t / mn);
    const int64_t rem = t - z * mn;
    const int r = (int)(rem % a.m), c = (int)(rem / a.m);
    double* C = a.C + z * a.strideC;
    const int64_t idx = (int64_t)r + (int64_t)c * a.ldc;
    const bool has_beta = a.beta[0] != 0.0 || a.beta[1] != 0.0;
    if (a.cplx) {
      const double sr = ws_sum(a, z, r, c), si = ws_sum(a, z, r + a.m, c);
      double re = a.alpha[0] * sr - a.alpha[1] * si;
      double im = a.alpha[0] * si + a.alpha[1] * sr;
      if (has_beta) {
        const double cr = C[idx], ci = C[a.planeC + idx];
        re += a.beta[0] * cr - a.beta[1] * ci;
        im += a.beta[0] * ci + a.beta[1] * cr;
      }
      C[idx] = re;
      C[a.planeC + idx] = im;
    } else {
      double v = a.alpha[0] * ws_sum(a, z, r, c);
      if (has_beta) v += a.beta[0] * C[idx];
      C[idx] = v;
    }
  }
}

// ------------------------------------------------------------ host side
constexpr int SMEM = STAGES * (BM * 128 + 128 * 128) + 1024 + 256;
static_assert(SMEM <= 227 * 1024, "shared memory");

struct Plan {
  int var = 0, S = 1, Q = 1;
  double t_oz = 0.0;
};

}  // namespace oz

// estimated device seconds of the digit GEMM with the piece split (S level sets, Q chunk
// ranges) on `cl` resident clusters, against the CUDA-core FP64 kernel
static oz::Plan oz_plan(int64_t M2, int64_t N, int64_t K2, int batch, int cl) {
  using namespace oz;
  const int64_t tiles = ((M2 + TILE - 1) / TILE) * ((N + TILE - 1) / TILE) * batch;
  const int64_t nk = (K2 + KELEMS - 1) / KELEMS;
  const int nch = (int)nk;          // Q splits the K slices
  // one digit product of a pair tile: 256 x 256 x K on two SMs at ~1.75 PFLOP/s / 76 pairs
  const double prod_s = 2.0 * TILE * TILE * (double)(nk * KELEMS) / (1.75e15 / 76.0);
  Plan best;
  best.t_oz = 1e30;
  for (int v = 0; v < NVAR; v++)
    for (int Q = 1; Q <= std::min(nch, 8); Q *= 2) {
      const int S = kVarPieces[v];
      const int64_t items = tiles * S * Q;
      const int64_t rounds = (items + cl - 1) / cl;
      // an item: its level set's products over 1/Q of the K chunks
      double t = rounds * prod_s * kVarMaxProducts[v] / Q;
      if (S * Q > 1) t += (double)items * TILE * TILE * 8.0 * 2.0 / 5e12 + 4e-6;   // reduce
      if (t < best.t_oz * 0.97) {
        best.t_oz = t;
        best.var = v;
        best.S = S;
        best.Q = Q;
      }
    }
  // digit planes: read FP64 twice, write 16 B per element; launch overheads
  best.t_oz += (double)(M2 + N) * K2 * batch * 32.0 / 5e12 + 15e-6;
  return best;
}

int gemm_f64_ozaki_possible(fmpt_handle* h, const GemmArgs& g) {
  if (!h->f64_tc && !g.engine) return 0;
  if (g.m < 32 || g.n < 32 || g.k < 16) return 0;
  const int cp = g.cplx ? 2 : 1;
  const double flops = 2.0 * g.m * g.n * (double)g.k * g.batch * cp * cp;
  const double t_simt = flops / 1.1e12;
  oz::Plan p = oz_plan((int64_t)g.m * cp, g.n, (int64_t)g.k * cp, g.batch,
                       std::max(1, h->sm_count / 2));
  return p.t_oz < t_simt ? 1 : 0;
}

int gemm_f64_ozaki(fmpt_handle* h, const GemmArgs& g) {
  using namespace oz;
  const int cp = g.cplx ? 1 : 0;
  const int M2 = g.m * (cp ? 2 : 1), K2 = g.k * (cp ? 2 : 1), N = g.n;
  const int ldk = (K2 + 7) / 8 * 8;
  const int batch = g.batch;
  if ((int64_t)batch * NS > INT32_MAX / 2) return set_error(h, FMPT_ERR_SHAPE, "ozaki: batch");
  // workspace: digit planes of A and B, exponents, then the split pieces
  const size_t planesA = (size_t)batch * NS * M2 * ldk * 2, planesB = (size_t)batch * NS * N * ldk * 2;
  const size_t expA = (size_t)batch * M2 * 4, expB = (size_t)batch * N * 4;
  auto al = [](size_t b) { return (b + 255) / 256 * 256; };
  const int tiles_m2 = (M2 + TILE - 1) / TILE, tiles_n = (N + TILE - 1) / TILE;
  const int64_t units = (int64_t)tiles_m2 * tiles_n * batch;
  if (units > INT32_MAX / 64) return set_error(h, FMPT_ERR_SHAPE, "ozaki: too many tiles");
  // resident clusters of the kernel
  static int clusters = -1;
  cudaLaunchConfig_t cfg{};
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = SMEM;
  cfg.stream = h->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (clusters < 0) {
    FMPT_CUDA(h, cudaFuncSetAttribute(oz_digits_rowfast,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DR_SMEM));
    FMPT_CUDA(h, cudaFuncSetAttribute(oz_gemm_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    cfg.gridDim = dim3(2 * std::max(1, h->sm_count / 2));
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, oz_gemm_pair, &cfg) != cudaSuccess) {
      (void)cudaGetLastError();
      n = 0;
    }
    clusters = n;
  }
  if (clusters <= 0) return set_error(h, FMPT_ERR_UNSUPPORTED, "ozaki: no 2-CTA cluster fits");
  const Plan plan = oz_plan(M2, N, K2, batch, clusters);
  const int split = plan.S * plan.Q;
  const bool direct = split == 1 && g.beta[0] == 0.0 && g.beta[1] == 0.0 && g.alpha[1] == 0.0;
  const size_t wsb = direct ? 0 : (size_t)units * split * TILE * TILE * sizeof(double);
  const size_t mxb = (size_t)batch * (M2 + N) * sizeof(uint64_t);
  // an operand with a cache keeps its planes there (built once while its key holds)
  const int64_t keyA[8] = {M2, K2, ldk, g.ta, cp, batch, g.lda, g.strideA};
  const int64_t keyB[8] = {N, K2, ldk, g.tb, cp, batch, g.ldb, g.strideB};
  auto cache_hit = [](const OzCache* c, const double* src, const int64_t* key) {
    if (!c || !c->valid || c->src != src) return false;
    for (int i = 0; i < 8; i++)
      if (c->key[i] != key[i]) return false;
    return true;
  };
  const bool hitA = cache_hit(g.cacheA, g.A, keyA), hitB = cache_hit(g.cacheB, g.B, keyB);
  const bool inA = g.cacheA != nullptr, inB = g.cacheB != nullptr;
  const size_t need = (inA ? 0 : al(planesA) + al(expA)) + (inB ? 0 : al(planesB) + al(expB)) +
                      al(mxb) + wsb;
  FMPT_TRY(grow_buffer(h, &h->oz_ws, &h->oz_ws_bytes, need));
  for (int side = 0; side < 2; side++) {
    OzCache* c = side == 0 ? g.cacheA : g.cacheB;
    if (!c || (side == 0 ? hitA : hitB)) continue;
    const size_t want = side == 0 ? al(planesA) + al(expA) : al(planesB) + al(expB);
    c->valid = false;
    FMPT_TRY(grow_buffer(h, &c->buf, &c->bytes, want));
  }
  char* base = static_cast<char*>(h->oz_ws);
  char* pa = inA ? static_cast<char*>(g.cacheA->buf) : base;
  if (!inA) base += al(planesA) + al(expA);
  char* pb = inB ? static_cast<char*>(g.cacheB->buf) : base;
  if (!inB) base += al(planesB) + al(expB);
  uint16_t* SA = reinterpret_cast<uint16_t*>(pa);
  int* EA = reinterpret_cast<int*>(pa + al(planesA));
  uint16_t* SBp = reinterpret_cast<uint16_t*>(pb);
  int* EB = reinterpret_cast<int*>(pb + al(planesB));
  unsigned long long* MX = reinterpret_cast<unsigned long long*>(base);
  double* WS = reinterpret_cast<double*>(base + al(mxb));

  // digit planes (A side: op(A), m x k; B side: op(B)^T, n x k)
  SliceSrc sa{}, sb{};
  sa.p = g.A; sa.plane = g.planeA; sa.bstride = g.strideA; sa.rows = g.m; sa.cols = g.k;
  sa.cplx = cp; sa.role = 0; sa.conj = (g.ta == FMPT_C || g.ta == FMPT_R);
  if (g.ta == FMPT_N || g.ta == FMPT_R) { sa.sr = 1; sa.sc = g.lda; } else { sa.sr = g.lda; sa.sc = 1; }
  sb.p = g.B; sb.plane = g.planeB; sb.bstride = g.strideB; sb.rows = g.n; sb.cols = g.k;
  sb.cplx = cp; sb.role = 1; sb.conj = (g.tb == FMPT_C || g.tb == FMPT_R);
  // op(B)(c, n) = B[c + n ldb] (N, R) or B[n + c ldb] (T, C)
  if (g.tb == FMPT_N || g.tb == FMPT_R) { sb.sr = g.ldb; sb.sc = 1; } else { sb.sr = 1; sb.sc = g.ldb; }
  {
    ProfScope prof(h, FMPT_K_CONVERT);
    FMPT_CUDA(h, cudaMemsetAsync(MX, 0, (size_t)batch * (M2 + N) * sizeof(uint64_t), h->stream));
    const unsigned kch = (unsigned)((ldk + SL_KCH - 1) / SL_KCH);
    const dim3 ga((M2 + SL_ROWS - 1) / SL_ROWS, kch, batch), gb((N + SL_ROWS - 1) / SL_ROWS, kch, batch);
    // the fast kernels need a real operand with a unit-stride index, 16-byte aligned rows
    // or columns and an even extent along the unit-stride index
    auto aligned = [](const SliceSrc& x, int64_t ld) {
      return !x.cplx && (reinterpret_cast<uintptr_t>(x.p) & 15) == 0 && (ld & 1) == 0 &&
             (x.bstride & 1) == 0;
    };
    auto slice = [&](const SliceSrc& x, int rows, const dim3& grid, unsigned long long* mx,
                     uint16_t* planes, int* ex) -> int {
      if (x.sr == 1 && aligned(x, x.sc) && (rows & 1) == 0) {
        const dim3 g1((unsigned)((rows / 2 + 255) / 256), (unsigned)((K2 + RM_KCH - 1) / RM_KCH),
                      (unsigned)batch);
        oz_rowmax_rowfast<<<g1, 256, 0, h->stream>>>(x.p, x.sc, x.bstride, rows, K2, mx);
      } else if (x.sc == 1 && aligned(x, x.sr) && (K2 & 1) == 0) {
        const dim3 g1((unsigned)((rows + 7) / 8), (unsigned)((K2 + RK_KCH - 1) / RK_KCH),
                      (unsigned)batch);
        oz_rowmax_kfast<<<g1, 256, 0, h->stream>>>(x.p, x.sr, x.bstride, rows, K2, mx);
      } else {
        oz_rowmax<<<grid, 256, 0, h->stream>>>(x, rows, K2, mx);
      }
      FMPT_LAUNCHED(h);
      if (x.sc == 1 && aligned(x, x.sr) && (K2 & 1) == 0)
        oz_digits_kfast<<<grid, 256, 0, h->stream>>>(x.p, x.sr, x.bstride, rows, K2, ldk, mx,
                                                      planes, ex);
      else if (x.sr == 1 && !x.cplx)
        oz_digits_rowfast<<<grid, 256, DR_SMEM, h->stream>>>(x.p, x.sc, x.bstride, rows, K2,
                                                              ldk, mx, planes, ex);
      else
        oz_digits<<<grid, 256, 0, h->stream>>>(x, rows, K2, ldk, mx, planes, ex);
      FMPT_LAUNCHED(h);
      return FMPT_OK;
    };
    if (!hitA) FMPT_TRY(slice(sa, M2, ga, MX, SA, EA));
    if (!hitB) FMPT_TRY(slice(sb, N, gb, MX + (size_t)batch * M2, SBp, EB));
  }
  for (int side = 0; side < 2; side++) {
    OzCache* c = side == 0 ? g.cacheA : g.cacheB;
    if (!c || (side == 0 ? hitA : hitB)) continue;
    c->src = side == 0 ? g.A : g.B;
    for (int i = 0; i < 8; i++) c->key[i] = side == 0 ? keyA[i] : keyB[i];
    c->valid = true;
  }
  CUtensorMap ma, mb;
  FMPT_TRY(make_map(h, &ma, SA, BF16, K2, M2, ldk, (int64_t)batch * NS, (int64_t)M2 * ldk, BM));
  FMPT_TRY(make_map(h, &mb, SBp, BF16, K2, N, ldk, (int64_t)batch * NS, (int64_t)N * ldk, 128));

  OzEpi ep{};
  ep.M = M2;
  ep.N = N;
  ep.ea = EA;
  ep.eb = EB;
  FMPT_TRY(gp_status_word(h, &ep.err));
  ep.nfast = M2 > N ? 1 : 0;
  ep.split = split;
  ep.var = plan.var;
  ep.S = plan.S;
  ep.Q = plan.Q;
  if (direct) {
    ep.C = g.C;
    ep.ldc = g.ldc;
    ep.strideC = g.strideC;
    ep.planeC = g.planeC;
    ep.mh = cp ? g.m : INT32_MAX;
    ep.alpha = g.alpha[0];
  } else {
    ep.C = WS;
    ep.mh = -1;        // workspace tiles
    ep.alpha = 1.0;
  }
  const int64_t items = units * split;
  cfg.gridDim = dim3((unsigned)(2 * std::min<int64_t>(items, clusters)));
  {
    ProfScope prof(h, FMPT_K_TC_GEMM);
    FMPT_CUDA(h, cudaLaunchKernelEx(&cfg, oz_gemm_pair, ma, mb, K2, tiles_m2, tiles_n, batch, ep));
    FMPT_LAUNCHED(h);
  }
  if (!direct) {
    RedArgs ra{};
    ra.ws = WS;
    ra.C = g.C;
    ra.ldc = g.ldc;
    ra.strideC = g.strideC;
    ra.planeC = g.planeC;
    ra.m = g.m;
    ra.n = g.n;
    ra.batch = batch;
    ra.cplx = cp;
    ra.split = split;
    ra.S = plan.S;
    ra.tiles_m2 = tiles_m2;
    ra.tiles_n = tiles_n;
    ra.nfast = ep.nfast;
    ra.alpha[0] = g.alpha[0];
    ra.alpha[1] = g.alpha[1];
    ra.beta[0] = g.beta[0];
    ra.beta[1] = g.beta[1];
    const int64_t total = (int64_t)g.m * g.n * batch;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 8LL * h->sm_count));
    oz_reduce<<<blocks, 256, 0, h->stream>>>(ra);
    FMPT_LAUNCHED(h);
  }
  return FMPT_OK;
}

void oz_cache_free(fmpt_handle* h, OzCache& c) {
  if (c.buf) cudaFreeAsync(c.buf, h->stream);
  c.buf = nullptr;
  c.bytes = 0;
  c.valid = false;
  c.src = nullptr;
}

}  // namespace fmpt
