// FP64-accurate Legendre sums on the tensor cores: fixed-point BF16 slices
// with exact FP32 accumulation (the error-free splitting of Ozaki, Ogita,
// Oishi and Rump, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012).
//
// Every table row (one (m, theta) of P or dP for the synthesis, one (m, l)
// for the analysis) and every data column (one (m, column) over all K) is
// scaled by a power of two so that its entries lie in (-1, 1) (in the
// synthesis after exact per-degree weights, see deg_shift), then written as
// seven signed base-256 digits:
//     x 2^-E = sum_{i<7} d_i 2^(-7-8i),   d_i integer, |d_i| <= 128,
// each exact in BF16.  A product of two digits is an integer of at most 2^14
// in magnitude, and
//     sum_K a b = 2^(Ea+Eb-14) sum_{i+j<=6} 2^(-8(i+j)) (A_i B_j)
// keeps 28 of the 49 digit products in seven tensor-memory accumulators
// C_d = sum_{i+j=d} A_i B_j.  C_d adds (d+1) K-sums and stays an exact FP32
// integer while (d+1) K 2^14 <= 2^24: K <= 1024, 512, 341 for C_0, C_1, C_2
// (C_3..C_6 enter at 2^-24 and below and need not be exact).  K is at most
// (l_max+2)/2 degrees of one parity (synthesis) or n_theta/2 colatitudes
// (analysis); beyond 341 the worst case rounds C_2 at 2^-40 of the scales.
// The dropped digits and products leave a relative error near 2^-55 of the
// row and column scales.  Six digits (2^-47) measured 1e-13 normwise at
// l_max = 255 and up to 5e-11 on an output 600x smaller than its call's
// others (the spheroidal part of a curl); seven bring the sums below the
// double-float FFTs' own error.  The epilogue sums the accumulators in
// double-float arithmetic (dfloat.cuh) and writes double-float half spectra
// for the double-float FFTs (synthesis) or FP64 spectra (analysis).
//
// Structure (as the 3xBF16 persistent kernels of legendre_tcp.cu): a pack
// kernel builds the data digits in the exact shared-memory image of the
// MMA's K-major, 128-byte-swizzled operand, one CTA per (m, column tile),
// first finding each column's scale over all of K; a persistent CTA per SM
// takes output tiles from a global counter, warp 0 bulk-copies table and data
// tiles into shared-memory rings, one thread of warp 1 issues tcgen05.mma,
// warps 2..9 drain the accumulators.  Per table and K step of 16 the MMA
// thread issues, for digit i of the table,
//     A_i x [B_0 | ... | B_{6-i}]  ->  [C_i | ... | C_6]     (N = 32 (7 - i))
// because the data digits of a tile lie one after the other along N.
#include <algorithm>
#include <type_traits>
#include <vector>
#include <cuda_bf16.h>
#include "common.cuh"
#include "cplx.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace {

// Digits per operand S: 7 (MAGIC_SHT_FP64TC) or 5 (MAGIC_SHT_BF16X5); every
// kernel below is a template on S, with kS = S, kTS its data-tile bytes and
// kFix its fixed-point position.
constexpr int kNC = 32;                  // real data columns per tile (16 complex)
// data tile: S digit blocks of 32 rows x 64 K bf16 (4 KB each)
__host__ __device__ constexpr uint32_t tile_bytes(int S) { return (uint32_t)S * kNC * 128; }
#define OZ_DIGITS(S)                          \
  constexpr int kS = (S);                     \
  constexpr uint32_t kTS = tile_bytes(S);     \
  constexpr int kFix = 8 * (S) - 1;           \
  (void)kTS;                                  \
  (void)kFix
constexpr int kThreads = 320;            // 10 warps
constexpr int kEpiThreads = 256;         // warps 2..9
constexpr int kPackThreads = 256;
constexpr int kPack1Threads = 512;       // the one-pass synthesis pack: one complex column per warp
constexpr int kNTR = 4;                  // tile-index ring

__device__ __forceinline__ unsigned char* align1k(unsigned char* p) {
  return (unsigned char*)(((uintptr_t)p + 1023) & ~(uintptr_t)1023);
}

// ------------------------------------------------------------ digits
// round(x 2^sh) as a 64-bit integer, with integer instructions only
// (|x| 2^sh < 2^62 assumed; round half away from zero).
__device__ __forceinline__ long long fixed_from_double(double x, int sh) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0x7FF) return 0;  // Inf / NaN: no digits (the scale is not finite either)
  unsigned long long m = b & ((1ull << 52) - 1);
  if (ex) m |= 1ull << 52;
  const int s = (ex ? ex : 1) - 1075 + sh;  // x = m 2^(s - sh)
  long long F;
  if (s >= 0) F = (long long)(m << s);
  else if (s <= -54) F = 0;
  else F = (long long)((m + (1ull << (-s - 1))) >> (-s));
  return (long long)(b >> 63) ? -F : F;
}
__device__ __forceinline__ long long fixed_from_float(float x, int sh) {
  const unsigned int b = __float_as_uint(x);
  const int ex = (int)((b >> 23) & 0xFF);
  if (ex == 0xFF) return 0;
  unsigned long long m = b & 0x7FFFFFu;
  if (ex) m |= 0x800000u;
  const int s = (ex ? ex : 1) - 150 + sh;
  long long F;
  if (s >= 0) F = (long long)(m << s);
  else if (s <= -25) F = 0;
  else F = (long long)((m + (1ull << (-s - 1))) >> (-s));
  return (b >> 31) ? -F : F;
}
// The S balanced base-256 digits of F as FP32 values (exact small integers;
// d_0 the most significant), with one byte permute and one FP32 subtraction
// per digit: every byte of U = F + 0x80...80 (a bias of 128 in each of the S
// bytes) is u = d + 128 with d in [-128, 127], and the top digit is
// (U >> 8(S-1)) - 128 in [-128, 128] (|F| <= 2^(8S-1) keeps U in
// [0, 2^(8S) + 2^(8S-8)]).  A byte u placed in the mantissa of 0x4B400000 is
// the float 1.5 2^23 + u.
template <int S>
__device__ __forceinline__ void digitsf(long long F, float (&f)[S]) {
  static_assert(S >= 5 && S <= 7, "five to seven digits");
  constexpr unsigned long long kBias = 0x8080808080808080ull >> (8 * (8 - S));
  const unsigned long long U = (unsigned long long)F + kBias;
  const uint32_t lo = (uint32_t)U, hi = (uint32_t)(U >> 32);
  constexpr uint32_t kMag = 0x4B400000u;
  constexpr float kOff = 12583040.0f;  // 1.5 2^23 + 128
#pragma unroll
  for (int b = 0; b < S - 1; ++b)  // byte b of U: digit S-1-b
    f[S - 1 - b] = __uint_as_float(__byte_perm(b < 4 ? lo : hi, kMag, 0x7640u | (uint32_t)(b & 3))) - kOff;
  // bytes S-1 and S of U (in hi: S >= 5)
  constexpr uint32_t kTop = 0x7600u | ((uint32_t)(S - 4) << 4) | (uint32_t)(S - 5);
  f[0] = __uint_as_float(__byte_perm(hi, kMag, kTop)) - kOff;
}
// two FP32 values (small integers, exact) as one bf16x2 word, lo at the lower address
__device__ __forceinline__ uint32_t bf16x2_of(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo in the low half
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ uint16_t bf16_bits(float x) { return (uint16_t)(bf16x2_of(x, 0.f) & 0xFFFFu); }
// Synthesis degree weights: the table is stored times w_l and the spectra
// divided by w_l, w_l = 2^-k(l), k(l) = floor(log2(l+1)) (exact, cancels in
// the sum).  dP grows about like l along a table row while the spectra fall
// off, so without the weights the fixed-point digits of a row, scaled to its
// largest (high-l) entry, would keep too few bits of the low-l entries that
// dominate the sum (1e-11 instead of 2e-13 at l_max = 255).
__device__ __forceinline__ int deg_shift(int l) { return 31 - __clz(l + 1); }
// e with |x| < 2^e (frexp exponent) from the bits; -4096 for zero
__device__ __forceinline__ int exp_bound(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b << 1) == 0) return -4096;
  const int ex = (int)((b >> 52) & 0x7FF);
  return (ex ? ex : 1) - 1022;
}
// exponent E with |x| < 2^E for every x of magnitude <= mx (0 for mx = 0)
__device__ __forceinline__ int scale_exp(double mx) {
  int e = 0;
  if (mx > 0.0 && mx <= 1.79e308) frexp(mx, &e);
  return e;
}
// digits of x scaled by 2^-E (|x| < 2^E), as BF16 bit patterns; fixed-point
// position F = round(x 2^(kFix - E))
template <int S>
__device__ __forceinline__ void digits_of(double x, int E, uint16_t (&d)[S]) {
  OZ_DIGITS(S);
  float f[kS];
  digitsf<S>(fixed_from_double(x, kFix - E), f);
#pragma unroll
  for (int i = 0; i < kS; ++i) d[i] = bf16_bits(f[i]);
}
// the digits of one row at the even index k (f[0]) and k + 1 (f[1]): one
// 32-bit store per digit block
template <int S>
__device__ __forceinline__ void store_digit_pairs(unsigned char* tile, int row, int k, const float (&f)[2][S]) {
  constexpr int kS = S;
#pragma unroll
  for (int i = 0; i < kS; ++i) *(uint32_t*)(tile + tc::sw128_offset(i * kNC + row, k)) = bf16x2_of(f[0][i], f[1][i]);
}

// ------------------------------------------------------------ accumulators
// C_0..C_{S-1} of 16 columns (this thread's TMEM lane) at `col` (digit block
// d at col + d * kNC), summed into double-float.  The balanced digits do not
// shrink with their position, so every C_d is about as large as C_0: only
// C_4..C_6 (weights 2^-32 and below) may be added in FP32, whose rounding at
// 2^-24 of C_4 is 2^-56 of C_0; C_3, C_2, C_1 and C_0 enter with error-free
// additions (an FP32 sum from C_3 on measured 2e-14 instead of 1e-15).
template <int S>
__device__ __forceinline__ void drain16(uint32_t col, dfl (&v)[16]) {
  static_assert(S >= 5 && S <= 7, "five to seven accumulators");
  uint32_t a[16], b[16];
  float t[16];
  if constexpr (S == 7) {
    tc::tmem_ld16_nw(col + 6 * kNC, a);
    tc::tmem_ld16_nw(col + 5 * kNC, b);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = __fmaf_rn(__uint_as_float(a[i]), 0.00390625f, __uint_as_float(b[i]));
    tc::tmem_ld16_nw(col + 4 * kNC, a);
    tc::tmem_ld16_nw(col + 3 * kNC, b);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = __fmaf_rn(t[i], 0.00390625f, __uint_as_float(a[i]));  // C4 + 2^-8 C5 + 2^-16 C6
  } else if constexpr (S == 6) {
    tc::tmem_ld16_nw(col + 5 * kNC, a);
    tc::tmem_ld16_nw(col + 4 * kNC, b);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = __fmaf_rn(__uint_as_float(a[i]), 0.00390625f, __uint_as_float(b[i]));
    tc::tmem_ld16_nw(col + 3 * kNC, b);
    tc::tmem_wait_ld();
  } else {
    tc::tmem_ld16_nw(col + 4 * kNC, a);
    tc::tmem_ld16_nw(col + 3 * kNC, b);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = __uint_as_float(a[i]);  // C4
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    float s, e;
    two_sum(__uint_as_float(b[i]), __fmul_rn(t[i], 0.00390625f), s, e);  // C3 + 2^-8 (...), exact
    v[i] = mkdf(s, e);
  }
#pragma unroll
  for (int d = 2; d >= 0; --d) {
    tc::tmem_ld16_nw(col + d * kNC, a);
    tc::tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      // C_d + 2^-8 v (the scaling by 2^-8 is exact)
      float s, e;
      two_sum(__uint_as_float(a[i]), __fmul_rn(v[i].h, 0.00390625f), s, e);
      v[i] = fast_two_sum(s, __fmaf_rn(v[i].l, 0.00390625f, e));
    }
  }
}

// ------------------------------------------------------------ rings
__device__ __forceinline__ bool wait_full(uint64_t* bar, uint32_t use, uint32_t ring) {
  return tc::mbar_wait(bar, (use / ring) & 1u);
}
__device__ __forceinline__ bool wait_empty(uint64_t* bar, uint32_t use, uint32_t ring) {
  return tc::mbar_wait(bar, ((use / ring) & 1u) ^ 1u);
}
template <int N>
__device__ __forceinline__ void drain_copies(uint64_t* full, uint32_t use) {
  for (uint32_t u = use > N ? use - N : 0; u < use; ++u) wait_full(&full[u % N], u, N);
}
struct TileRing {
  int* idx;
  uint64_t* full;
  uint64_t* empty;
};
__device__ __forceinline__ bool ring_push(const TileRing& R, uint32_t& use, int ix) {
  const uint32_t slot = use % kNTR;
  if (!wait_empty(&R.empty[slot], use, kNTR)) return false;
  R.idx[slot] = ix;
  tc::mbar_arrive(&R.full[slot]);
  ++use;
  return true;
}
__device__ __forceinline__ bool ring_pop(const TileRing& R, uint32_t& use, int& ix) {
  const uint32_t slot = use % kNTR;
  if (!wait_full(&R.full[slot], use, kNTR)) return false;
  ix = R.idx[slot];
  tc::mbar_arrive(&R.empty[slot]);
  ++use;
  return true;
}

// MMAs of table digit u against the stacked data digits: K = 16 per MMA, the
// first nks (<= 4) of a 64-wide chunk (the K rows past a synthesis order's
// degrees are zero in both operands and are skipped); table tb's
// accumulators at acc + tb * kS * kNC.
template <int NT, int S>
__device__ __forceinline__ void issue_digit(uint32_t acc, const unsigned char* A, const unsigned char* B, int u,
                                            bool first_chunk, uint32_t bstride_tb, int nks, int tb0, int tb1) {
  constexpr int kS = S;
  const uint64_t a0 = tc::sw128_desc(tc::smem_u32(A));
  const uint64_t b0 = tc::sw128_desc(tc::smem_u32(B));
  const uint32_t idesc = tc::idesc_bf16(128, (kS - u) * kNC);
#pragma unroll
  for (int ks = 0; ks < 4; ++ks)
#pragma unroll
    for (int tb = 0; tb < NT; ++tb) {
      if (ks >= nks || tb < tb0 || tb >= tb1) continue;  // tb0..tb1-1: this MMA thread's tables
      const uint32_t d = acc + (uint32_t)((tb * kS + u) * kNC);
      const uint64_t ad = a0 + (uint64_t)((tb * 16384 + ks * 32) >> 4);
      const uint64_t bd = b0 + (uint64_t)((tb * bstride_tb + ks * 32) >> 4);
      tc::mma_bf16(d, ad, bd, idesc, (u != 0 || !first_chunk || ks) ? 1u : 0u);
    }
}

// Bytes of a 128-row table block that hold its first `rows` rows (8-row
// groups of 1 KB in the 128-byte-swizzled layout).  The rows past a block's
// colatitudes (synthesis) or degrees (analysis) are zero and are not loaded:
// the MMA reads whatever the ring slot held there into accumulator rows that
// the epilogue does not store.
__device__ __forceinline__ uint32_t table_rows_bytes(int rows) { return (uint32_t)((min(rows, 128) + 7) >> 3) << 10; }

// ------------------------------------------------------------ instances
// (tile_inst / block_inst of common.cuh: one instance, or several with MULTI)
using OzInv = LegInst<InvSet>;
using OzFwd = LegInst<FwdSet>;

template <typename P>
__device__ __forceinline__ P* shfl_ptr(P* p, int src) {
  const unsigned long long v = (unsigned long long)p;
  const unsigned lo = __shfl_sync(0xffffffffu, (unsigned)v, src);
  const unsigned hi = __shfl_sync(0xffffffffu, (unsigned)(v >> 32), src);
  return (P*)(((unsigned long long)hi << 32) | lo);
}

// CTAs per SM and TMEM columns: one table (224 accumulator columns) two
// CTAs per SM with 256 columns each; two tables (448) one CTA with 512.  MMA
// threads: one per CTA, but one per table in the two-table analysis (warps 1
// and 10; 4% faster there, 13% slower in the synthesis, whose two tables
// share the data tiles).
template <bool VEC, bool INV>
struct Occ {
  static constexpr int CPS = VEC ? 1 : 2;
  static constexpr int TCOLS = VEC ? 512 : 256;
  static constexpr int NISS = (VEC && !INV) ? 2 : 1;
  static constexpr int THREADS = kThreads + 32 * (NISS - 1);
};
// ring depths: A = one table digit of one K chunk (NT x 16 KB), B = data
// tiles (a fifth table slot for the two-table kernels measured no faster)
template <bool VEC, bool INV>
struct Rings {
  static constexpr int NA = VEC ? (INV ? 4 : 3) : 3;
  static constexpr int NB = 2;
};

// ------------------------------------------------------------ table images
// Synthesis block (m, theta tile, table, parity, chunk, digit), 128 rows =
// colatitudes, 64 columns = degrees l = m + p + 2 l'; analysis block
// (m, parity, l' tile, table, theta chunk, digit), 128 rows = degrees, 64
// columns = colatitudes.  Row exponents in inv_exp [2][n_m][ntt*128] and
// fwd_exp [2][lm_max].
template <int S>
__global__ void build_inv_oz_kernel(const ShtGeom g, TcTables t, unsigned char* img, short* rexp) {
  OZ_DIGITS(S);
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int NHP = t.ntt * 128;
  if (idx >= (long long)g.n_m * 2 * NHP) return;
  const int j = (int)(idx % NHP);
  const int tb = (int)((idx / NHP) % 2);
  const int mc = (int)(idx / (2LL * NHP));
  const int m = mc * g.minc, n_l = g.l_max - m + 1, lm0 = g.lmoff[mc];
  const double* tab = tb ? g.dP64 : g.P64;
  const bool valid = j < g.nh;
  double mx = 0.0;
  if (valid)
    for (int l = 0; l < n_l; ++l) mx = fmax(mx, ldexp(fabs(tab[(size_t)(lm0 + l) * g.nh + j]), -deg_shift(m + l)));
  const int E = scale_exp(mx);
  rexp[((size_t)tb * g.n_m + mc) * NHP + j] = (short)E;
  const int nch = tc_nch(n_l);
  const int tt = j / 128, row = j % 128;
  for (int p = 0; p < 2; ++p)
    for (int lp = 0; lp < nch * 64; ++lp) {
      const int loff = p + 2 * lp;
      const double v =
          (valid && loff < n_l) ? ldexp(tab[(size_t)(lm0 + loff) * g.nh + j], -deg_shift(m + loff)) : 0.0;
      uint16_t d[kS];
      digits_of(v, E, d);
      const long long blk0 = t.inv_blk0[mc] + ((((long long)tt * 2 + tb) * 2 + p) * nch + lp / 64) * kS;
      for (int i = 0; i < kS; ++i) *(uint16_t*)(img + (blk0 + i) * 16384 + tc::sw128_offset(row, lp % 64)) = d[i];
    }
}

template <int S>
__global__ void build_fwd_oz_kernel(const ShtGeom g, TcTables t, unsigned char* img, short* rexp) {
  OZ_DIGITS(S);
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int NLP = t.nlt * 128;
  if (idx >= (long long)g.n_m * 2 * 2 * NLP) return;
  const int lpad = (int)(idx % NLP);
  const int p = (int)((idx / NLP) % 2);
  const int tb = (int)((idx / (2LL * NLP)) % 2);
  const int mc = (int)(idx / (4LL * NLP));
  const int m = mc * g.minc, n_l = g.l_max - m + 1, lm0 = g.lmoff[mc];
  const double* tab = tb ? g.dP64 : g.P64;
  const int loff = p + 2 * lpad;
  const bool valid = loff < n_l;
  double mx = 0.0;
  if (valid)
    for (int j = 0; j < g.nh; ++j) mx = fmax(mx, fabs(tab[(size_t)(lm0 + loff) * g.nh + j]));
  const int E = scale_exp(mx);
  if (valid) rexp[(size_t)tb * g.lm_max + lm0 + loff] = (short)E;
  const int lt = lpad / 128, row = lpad % 128;
  for (int j = 0; j < t.ncj * 64; ++j) {
    const double v = (valid && j < g.nh) ? tab[(size_t)(lm0 + loff) * g.nh + j] : 0.0;
    uint16_t d[kS];
    digits_of(v, E, d);
    const long long blk0 = t.fwd_blk0[mc] + ((((long long)p * t.nlt + lt) * 2 + tb) * t.ncj + j / 64) * kS;
    for (int i = 0; i < kS; ++i) *(uint16_t*)(img + (blk0 + i) * 16384 + tc::sw128_offset(row, j % 64)) = d[i];
  }
}

// ------------------------------------------------------------ packing
// Synthesis data of one (column tile ct, order mc): 16 complex columns
// (scalar: (level, field); vector: (level, field, S|T)) over all degrees of
// that order.  Pass 1 finds each real column's scale over l; pass 2 writes
// the digit tiles of every (parity, chunk), double-buffered in shared memory
// and stored with bulk copies.  Column exponents: cexp[mc][ct * kNC + row].
__device__ __forceinline__ double2 oz_operand(const SpecOperand& op, int r, int lm0, int loff, int l, int m,
                                             double or2) {
  const long long base = (long long)r * op.ld + lm0 + loff;
  const double2 a = __ldg(op.A + base);
  switch (op.op) {
    case OP_COPY: return a;
    case OP_DLH: {
      const double d = (double)(l * (l + 1));
      return make_double2(d * a.x, d * a.y);
    }
    case OP_CURLT: {
      const double2 b = __ldg(op.B + base);
      const double d = or2 * (double)(l * (l + 1));
      return make_double2(d * a.x - b.x, d * a.y - b.y);
    }
    case OP_IM: return make_double2(-(double)m * a.y, (double)m * a.x);
    default: return make_double2(0.0, 0.0);
  }
}

struct PackCol {
  SpecOperand op;  // op.op == OP_ZERO: a zero column
  int r, lc;
  double or2;
};

template <bool VEC>
__device__ __forceinline__ PackCol pack_col(const ShtGeom& g, const InvSet& s, int q, int ncplx) {
  PackCol c;
  c.op = SpecOperand{nullptr, nullptr, 0, OP_ZERO, 0};
  c.r = 0;
  c.lc = -1;
  c.or2 = 0.0;
  if (q >= ncplx) return c;
  const int pair = VEC ? (q >> 1) : q;
  const int r = pair / s.nf, f = pair - r * s.nf;
  const SpecOperand op = (VEC && (q & 1)) ? s.f[f].x1 : s.f[f].x0;
  if (op.op == OP_ZERO || op.A == nullptr || (op.op == OP_CURLT && op.B == nullptr)) return c;
  c.op = op;
  c.r = r;
  c.lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
  c.or2 = (op.op == OP_CURLT) ? (s.or2 ? s.or2[r] : s.or2_0) : 0.0;
  return c;
}

template <bool VEC, bool MULTI, int S>
__global__ void __launch_bounds__(kPackThreads, 3) pack_inv_oz(const __grid_constant__ OzInv one,
                                                            const OzInv* __restrict__ many,
                                                            const __grid_constant__ InstIndex X) {
  extern __shared__ unsigned char smem_raw[];
  OZ_DIGITS(S);
  unsigned char* buf = align1k(smem_raw);  // two tiles of kTS bytes
  __shared__ int sE[kNC];
  int ct, mc, c_unused;
  const OzInv& I = block_inst<MULTI>(one, many, X, ct, mc, c_unused);
  const ShtGeom& g = I.g;
  const InvSet& s = I.s;
  const TcTables& t = I.t;
  unsigned char* __restrict__ bimg = I.bimg;
  short* __restrict__ cexp = I.cexp;
  const int nct = I.nct;
  const int m = mc * g.minc, n_l = g.l_max - m + 1, lm0 = g.lmoff[mc];
  const int nch = tc_nch(n_l);
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  const int tid = threadIdx.x;
  // pass 1: 16 threads per complex column, strided over l
  {
    const int ql = tid >> 4, li = tid & 15;
    const PackCol c = pack_col<VEC>(g, s, ct * (kNC / 2) + ql, ncplx);
    // largest exponent of x 2^k(l) (the spectra divided by the degree weights)
    int er = -4096, ei = -4096;
    if (c.op.op != OP_ZERO) {
      const int nl = min(n_l, c.lc - m + 1);
      // eight independent loads per thread in flight before their exponents are taken
      for (int l0 = li; l0 < nl; l0 += 16 * 8) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int loff = l0 + 16 * u;
          v[u] = loff < nl ? oz_operand(c.op, c.r, lm0, loff, m + loff, m, c.or2) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = deg_shift(m + l0 + 16 * u);
          er = max(er, exp_bound(v[u].x) + k);
          ei = max(ei, exp_bound(v[u].y) + k);
        }
      }
    }
#pragma unroll
    for (int d = 8; d >= 1; d >>= 1) {
      er = max(er, __shfl_xor_sync(0xffffffffu, er, d));
      ei = max(ei, __shfl_xor_sync(0xffffffffu, ei, d));
    }
    if (er < -3000) er = 0;
    if (ei < -3000) ei = 0;
    if (li == 0) {
      sE[2 * ql] = er;
      sE[2 * ql + 1] = ei;
      cexp[(long long)mc * nct * kNC + ct * kNC + 2 * ql] = (short)er;
      cexp[(long long)mc * nct * kNC + ct * kNC + 2 * ql + 1] = (short)ei;
    }
  }
  __syncthreads();
  // pass 2: thread = (degree indices 2 kp, 2 kp + 1 of the chunk, column group qg)
  const int kp = tid & 31, qg = tid >> 5;
  PackCol cols[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) cols[i] = pack_col<VEC>(g, s, ct * (kNC / 2) + qg + 8 * i, ncplx);
  int nb = 0;
  for (int p = 0; p < 2; ++p)
    for (int c = 0; c < nch; ++c, ++nb) {
      unsigned char* B = buf + (nb & 1) * kTS;
      if (nb >= 2) {  // the bulk store that read this buffer has finished
        if (tid == 0) tc::bulk_wait_read<1>();
        __syncthreads();
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int ql = qg + 8 * i;
        double2 v[2];
        int kw[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int loff = p + 2 * (64 * c + 2 * kp + h);
          const int l = m + loff;
          v[h] = make_double2(0.0, 0.0);
          if (cols[i].op.op != OP_ZERO && loff < n_l && l <= cols[i].lc)
            v[h] = oz_operand(cols[i].op, cols[i].r, lm0, loff, l, m, cols[i].or2);
          kw[h] = deg_shift(l);  // x 2^k(l): the spectra divided by the degree weight
        }
        float d[2][kS];
#pragma unroll
        for (int h = 0; h < 2; ++h) digitsf<S>(fixed_from_double(v[h].x, kFix - sE[2 * ql] + kw[h]), d[h]);
        store_digit_pairs(B, 2 * ql, 2 * kp, d);
#pragma unroll
        for (int h = 0; h < 2; ++h) digitsf<S>(fixed_from_double(v[h].y, kFix - sE[2 * ql + 1] + kw[h]), d[h]);
        store_digit_pairs(B, 2 * ql + 1, 2 * kp, d);
      }
      tc::fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
        const long long pc = t.bpc0[mc] + p * nch + c;
        tc::bulk_s2g(bimg + (pc * nct + ct) * (long long)kTS, B, kTS);
        tc::bulk_commit();
      }
    }
  if (tid == 0) tc::bulk_wait<0>();
}

// The same pack in one pass, for orders of at most two 64-degree chunks per
// parity (l_max <= 255): warp qg owns complex columns qg and qg + 8 over all
// degrees of the order (lane kp: degree indices 2 kp, 2 kp + 1 of every
// chunk), so it loads all of them into registers at once (16 loads in
// flight per thread), takes each column's scale by a warp reduction and
// writes the digits from registers: the spectra are read once, with one
// memory latency per CTA instead of one per pass and chunk.  The digits are
// those of pack_inv_oz (same scales, same rounding).
template <bool VEC, bool MULTI, int S>
__global__ void __launch_bounds__(kPack1Threads, 2) pack_inv_oz1(const __grid_constant__ OzInv one,
                                                              const OzInv* __restrict__ many,
                                                              const __grid_constant__ InstIndex X) {
  extern __shared__ unsigned char smem_raw[];
  OZ_DIGITS(S);
  unsigned char* buf = align1k(smem_raw);  // two tiles of kTS bytes
  int ct, mc, c_unused;
  const OzInv& I = block_inst<MULTI>(one, many, X, ct, mc, c_unused);
  const ShtGeom& g = I.g;
  const InvSet& s = I.s;
  const TcTables& t = I.t;
  unsigned char* __restrict__ bimg = I.bimg;
  short* __restrict__ cexp = I.cexp;
  const int nct = I.nct;
  const int m = mc * g.minc, n_l = g.l_max - m + 1, lm0 = g.lmoff[mc];
  const int nch = tc_nch(n_l);  // <= 2
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  // sixteen warps, one complex column (two real rows of the tile) each
  const int tid = threadIdx.x, kp = tid & 31, ql = tid >> 5;
  const PackCol col = pack_col<VEC>(g, s, ct * (kNC / 2) + ql, ncplx);
  // v[p][c][h]: parity p, chunk c, degree index 64 c + 2 kp + h
  double2 v[2][2][2];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int loff = p + 2 * (64 * c + 2 * kp + h);
        const int l = m + loff;
        v[p][c][h] = make_double2(0.0, 0.0);
        if (col.op.op != OP_ZERO && c < nch && loff < n_l && l <= col.lc)
          v[p][c][h] = oz_operand(col.op, col.r, lm0, loff, l, m, col.or2);
      }
  // largest exponent of x 2^k(l) per real column (the spectra divided by the degree weights)
  int E0, E1;
  {
    int er = -4096, ei = -4096;
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int k = deg_shift(m + p + 2 * (64 * c + 2 * kp + h));
          er = max(er, exp_bound(v[p][c][h].x) + k);
          ei = max(ei, exp_bound(v[p][c][h].y) + k);
        }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
      er = max(er, __shfl_xor_sync(0xffffffffu, er, d));
      ei = max(ei, __shfl_xor_sync(0xffffffffu, ei, d));
    }
    E0 = er < -3000 ? 0 : er;
    E1 = ei < -3000 ? 0 : ei;
    if (kp == 0) {
      cexp[(long long)mc * nct * kNC + ct * kNC + 2 * ql] = (short)E0;
      cexp[(long long)mc * nct * kNC + ct * kNC + 2 * ql + 1] = (short)E1;
    }
  }
  int nb = 0;
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      if (c >= nch) continue;
      unsigned char* B = buf + (nb & 1) * kTS;
      if (nb >= 2) {  // the bulk store that read this buffer has finished
        if (tid == 0) tc::bulk_wait_read<1>();
        __syncthreads();
      }
      int kw[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) kw[h] = deg_shift(m + p + 2 * (64 * c + 2 * kp + h));
      float d[2][kS];
#pragma unroll
      for (int h = 0; h < 2; ++h) digitsf<S>(fixed_from_double(v[p][c][h].x, kFix - E0 + kw[h]), d[h]);
      store_digit_pairs(B, 2 * ql, 2 * kp, d);
#pragma unroll
      for (int h = 0; h < 2; ++h) digitsf<S>(fixed_from_double(v[p][c][h].y, kFix - E1 + kw[h]), d[h]);
      store_digit_pairs(B, 2 * ql + 1, 2 * kp, d);
      tc::fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
        const long long pc = t.bpc0[mc] + p * nch + c;
        tc::bulk_s2g(bimg + (pc * nct + ct) * (long long)kTS, B, kTS);
        tc::bulk_commit();
      }
      ++nb;
    }
  if (tid == 0) tc::bulk_wait<0>();
}

// Analysis data of one (column tile ct, order mc): the double-float (ES, EA)
// half spectra of 16 complex columns over the nh colatitudes.  Exponents per
// (ES | EA, real column): cexp[mc][2][nct * kNC]; tiles [mc][chunk][ct][ES|EA].
template <bool VEC, bool MULTI, int S>
__global__ void __launch_bounds__(kPackThreads, 3) pack_fwd_oz(const __grid_constant__ OzFwd one,
                                                            const OzFwd* __restrict__ many,
                                                            const __grid_constant__ InstIndex X) {
  extern __shared__ unsigned char smem_raw[];
  // one (ES, EA) tile pair (56 KB): three CTAs per SM; the next chunk waits for
  // the bulk store of the previous one (two pairs measured 1 CTA per SM, 1.8 ms)
  OZ_DIGITS(S);
  unsigned char* buf = align1k(smem_raw);
  __shared__ int sE[2][kNC];
  int ct, mc, c_unused;
  const OzFwd& I = block_inst<MULTI>(one, many, X, ct, mc, c_unused);
  const ShtGeom& g = I.g;
  const FwdSet& s = I.s;
  const TcTables& t = I.t;
  unsigned char* __restrict__ bimg = I.bimg;
  short* __restrict__ cexp = I.cexp;
  const int nct = I.nct;
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  const int tid = threadIdx.x;
  auto src_of = [&](int q) -> const dfl2* {
    if (q >= ncplx) return nullptr;
    const int pair = VEC ? (q >> 1) : q;
    const int r = pair / s.nf, f = pair - r * s.nf;
    const dfl2* base = (const dfl2*)((VEC && (q & 1)) ? s.f[f].in1 : s.f[f].in0);
    return base + (long long)r * s.f[f].in_ld + (long long)mc * g.nh * 2;  // (ES, EA) at 2j, 2j+1
  };
  {
    const int ql = tid >> 4, li = tid & 15;
    const dfl2* src = src_of(ct * (kNC / 2) + ql);
    float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
    // only the hi words set the scale: twelve colatitudes per thread in flight
    // (every colatitude of nh <= 192 in one round), four floats each
    if (src)
      for (int j0 = li; j0 < g.nh; j0 += 16 * 12) {
        float hw[12][4];
#pragma unroll
        for (int u = 0; u < 12; ++u) {
          const int j = j0 + 16 * u;
          const float* q = (const float*)(src + 2 * j);  // es.x.h, es.y.h, ea.x.h, ea.y.h at 0, 2, 4, 6
#pragma unroll
          for (int w = 0; w < 4; ++w) hw[u][w] = j < g.nh ? __ldg(q + 2 * w) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 12; ++u) {
          m0 = fmaxf(m0, fabsf(hw[u][0]));
          m1 = fmaxf(m1, fabsf(hw[u][1]));
          m2 = fmaxf(m2, fabsf(hw[u][2]));
          m3 = fmaxf(m3, fabsf(hw[u][3]));
        }
      }
#pragma unroll
    for (int d = 8; d >= 1; d >>= 1) {
      m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, d));
      m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, d));
      m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, d));
      m3 = fmaxf(m3, __shfl_xor_sync(0xffffffffu, m3, d));
    }
    if (li == 0) {
      const int e[4] = {scale_exp(m0), scale_exp(m1), scale_exp(m2), scale_exp(m3)};
      const long long b = (long long)mc * 2 * nct * kNC + ct * kNC + 2 * ql;
      sE[0][2 * ql] = e[0];
      sE[0][2 * ql + 1] = e[1];
      sE[1][2 * ql] = e[2];
      sE[1][2 * ql + 1] = e[3];
      cexp[b] = (short)e[0];
      cexp[b + 1] = (short)e[1];
      cexp[b + (long long)nct * kNC] = (short)e[2];
      cexp[b + (long long)nct * kNC + 1] = (short)e[3];
    }
  }
  __syncthreads();
  // pass 2: thread = (colatitudes 2 kp, 2 kp + 1 of the chunk, column group qg)
  const int kp = tid & 31, qg = tid >> 5;
  const dfl2* srcs[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) srcs[i] = src_of(ct * (kNC / 2) + qg + 8 * i);
  // values of chunk c: es / ea [column][colatitude 2 kp + h]; the loads of
  // chunk c + 1 are issued before chunk c's barrier and bulk store
  dfl2 es[2][2], ea[2][2];
  auto load_chunk = [&](int c) {
    const int j0 = 64 * c + 2 * kp;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        es[i][h] = {dfl(0), dfl(0)};
        ea[i][h] = es[i][h];
        if (srcs[i] && c < t.ncj && j0 + h < g.nh) {
          es[i][h] = srcs[i][2 * (j0 + h)];
          ea[i][h] = srcs[i][2 * (j0 + h) + 1];
        }
      }
  };
  load_chunk(0);
  for (int c = 0; c < t.ncj; ++c) {
    unsigned char* B = buf;
    if (c >= 1) {
      if (tid == 0) tc::bulk_wait_read<0>();
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int ql = qg + 8 * i;
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int which = w >> 1, row = 2 * ql + (w & 1);
        const int sh = kFix - sE[which][row];
        float d[2][kS];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const dfl v = w == 0 ? es[i][h].x : w == 1 ? es[i][h].y : w == 2 ? ea[i][h].x : ea[i][h].y;
          digitsf<S>(fixed_from_float(v.h, sh) + fixed_from_float(v.l, sh), d[h]);
        }
        store_digit_pairs(B + which * kTS, row, 2 * kp, d);
      }
    }
    load_chunk(c + 1);
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::bulk_s2g(bimg + (((long long)mc * t.ncj + c) * nct + ct) * (2LL * kTS), B, 2 * kTS);
      tc::bulk_commit();
    }
  }
  if (tid == 0) tc::bulk_wait<0>();
}

// ------------------------------------------------------------ synthesis
struct InvTile {
  int mc, p, tt, ct, nch, nchp, nlp;
  __device__ void decode(const ShtGeom& g, const TcTables& t, int nct, int ix) {
    int rest;
    if (t.order == 0) {
      ct = ix % nct;
      rest = ix / nct;
      tt = rest % t.ntt;
      rest /= t.ntt;
    } else {
      tt = ix % t.ntt;
      rest = ix / t.ntt;
      ct = rest % nct;
      rest /= nct;
    }
    p = rest & 1;
    mc = rest >> 1;
    const int n_l = g.l_max - mc * g.minc + 1;
    nch = tc_nch(n_l);
    nlp = (n_l + 1 - p) / 2;
    nchp = (nlp + 63) / 64;
  }
};

// 2^e as an FP32 factor (e clamped to the normal range: smaller factors flush
// the contribution to zero, larger ones overflow as the true value would)
__device__ __forceinline__ float pow2f(int e) {
  e = max(-127, min(e, 128));
  if (e == -127) return 0.f;
  if (e == 128) return __int_as_float(0x7F800000);
  return __int_as_float((e + 127) << 23);
}

template <bool VEC, bool MULTI, int S>
__global__ void __launch_bounds__(Occ<VEC, true>::THREADS, Occ<VEC, true>::CPS)
    inv_leg_oz(const __grid_constant__ OzInv one, const OzInv* __restrict__ many,
               const __grid_constant__ InstIndex X, int ntiles) {
  OZ_DIGITS(S);
  constexpr int NT = VEC ? 2 : 1;
  constexpr int NA = Rings<VEC, true>::NA, NB = Rings<VEC, true>::NB;
  constexpr uint32_t ASZ = NT * 16384;
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t a_full[NA], a_empty[NA], b_full[NB], b_empty[NB], acc_full, acc_empty, fin;
  __shared__ uint64_t tr_full[kNTR], tr_empty[kNTR];
  __shared__ int tr_idx[kNTR];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  unsigned char* sA = align1k(smem_raw);
  unsigned char* sB = sA + NA * ASZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    constexpr int NI = Occ<VEC, true>::NISS;  // every MMA thread commits to the empty / full barriers
    for (int i = 0; i < NA; ++i) { tc::mbar_init(&a_full[i], 1); tc::mbar_init(&a_empty[i], NI); }
    for (int i = 0; i < NB; ++i) { tc::mbar_init(&b_full[i], 1); tc::mbar_init(&b_empty[i], NI); }
    tc::mbar_init(&acc_full, NI);
    tc::mbar_init(&acc_empty, kEpiThreads);
    tc::mbar_init(&fin, NI);
    for (int i = 0; i < kNTR; ++i) { tc::mbar_init(&tr_full[i], 1); tc::mbar_init(&tr_empty[i], NI + kEpiThreads); }
    s_fail = 0;
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, Occ<VEC, true>::TCOLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  const TileRing R{tr_idx, tr_full, tr_empty};
  bool ok = true;
  InvTile T;

  if (warp == 0) {
    if (lane == 0) {  // ---------------------------------------- loader
      uint32_t a_use = 0, b_use = 0, tr = 0;
      int ix = blockIdx.x;
      while (ok) {
        if (!ring_push(R, tr, ix < ntiles ? ix : -1)) { ok = false; break; }
        if (ix >= ntiles) break;
        const int next = atomicAdd(one.t.tile_ctr, 1) + (int)gridDim.x;
        int lix = ix;
        const OzInv& I = tile_inst<MULTI>(one, many, X, lix);
        const ShtGeom& g = I.g;
        const TcTables& t = I.t;
        const int nct = I.nct;
        T.decode(g, t, nct, lix);
        ix = next;
        if (T.nlp == 0) continue;
        for (int c = 0; c < T.nchp && ok; ++c) {
          const uint32_t bslot = b_use % NB;
          if (!wait_empty(&b_empty[bslot], b_use, NB)) { ok = false; break; }
          tc::mbar_expect_tx(&b_full[bslot], kTS);
          tc::bulk_g2s(sB + bslot * kTS, I.bimg + ((t.bpc0[T.mc] + T.p * T.nch + c) * nct + T.ct) * (long long)kTS,
                       kTS, &b_full[bslot]);
          ++b_use;
          const uint32_t abytes = table_rows_bytes(g.nh - T.tt * 128);
          for (int u = 0; u < kS; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_empty(&a_empty[slot], a_use, NA)) { ok = false; break; }
            tc::mbar_expect_tx(&a_full[slot], NT * abytes);
            for (int tb = 0; tb < NT; ++tb) {
              const long long blk =
                  t.inv_blk0[T.mc] + ((((long long)T.tt * 2 + tb) * 2 + T.p) * T.nch + c) * kS + u;
              tc::bulk_g2s(sA + slot * ASZ + tb * 16384, t.inv_img + blk * 16384, abytes, &a_full[slot]);
            }
          }
        }
      }
      drain_copies<NA>(a_full, a_use);
      drain_copies<NB>(b_full, b_use);
    }
  } else if (warp == 1 || (Occ<VEC, true>::NISS == 2 && warp == 2 + kEpiThreads / 32)) {
    if (lane == 0) {  // ---------------------------------------- MMA issuer(s)
      const int tb0 = warp == 1 ? 0 : 1, tb1 = Occ<VEC, true>::NISS == 2 ? tb0 + 1 : NT;
      uint32_t a_use = 0, b_use = 0, acc_use = 0, tr = 0;
      while (ok) {
        int ix;
        if (!ring_pop(R, tr, ix)) { ok = false; break; }
        if (ix < 0) break;
        const OzInv& I = tile_inst<MULTI>(one, many, X, ix);
        T.decode(I.g, I.t, I.nct, ix);
        if (T.nlp == 0) continue;
        if (!wait_empty(&acc_empty, acc_use, 1)) { ok = false; break; }
        tc::tc_fence_after();
        for (int c = 0; c < T.nchp && ok; ++c, ++b_use) {
          const uint32_t bslot = b_use % NB;
          if (!wait_full(&b_full[bslot], b_use, NB)) { ok = false; break; }
          const int nks = min(4, (T.nlp - 64 * c + 15) >> 4);  // K steps holding degrees of the order
          for (int u = 0; u < kS; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_full(&a_full[slot], a_use, NA)) { ok = false; break; }
            tc::tc_fence_after();
            issue_digit<NT, S>(tmem, sA + slot * ASZ, sB + bslot * kTS, u, c == 0, 0, nks, tb0, tb1);
            tc::mma_commit(&a_empty[slot]);
          }
          tc::mma_commit(&b_empty[bslot]);
        }
        tc::mma_commit(&acc_full);
        ++acc_use;
      }
      tc::mma_commit(&fin);
      if (!tc::mbar_wait(&fin, 0)) ok = false;
    }
  } else if (warp < 2 + kEpiThreads / 32) {  // ------------------ epilogue
    const int q4 = warp & 3, half = (warp - 2) >> 2;
    const int cc0 = half * (kNC / 2);  // this warp's 16 real columns
    const int jl = 32 * q4 + lane;
    const uint32_t lane_off = (uint32_t)(32 * q4) << 16;
    uint32_t acc_use = 0, tr = 0;
    while (ok) {
      int ix;
      if (!ring_pop(R, tr, ix)) { ok = false; break; }
      if (ix < 0) break;
      const OzInv& I = tile_inst<MULTI>(one, many, X, ix);
      const ShtGeom& g = I.g;
      const InvSet& s = I.s;
      const TcTables& t = I.t;
      const int nct = I.nct;
      const int npair = s.nf * s.nlev;
      const int ncplx = npair * (VEC ? 2 : 1);
      const int NHP = t.ntt * 128;
      T.decode(g, t, nct, ix);
      const int jg = T.tt * 128 + jl;
      const bool row_ok = jg < g.nh;
      // output column bases, one per lane (scalar: lane q < 8 holds complex
      // column q of this warp; vector: lane q < 4 the v_theta array of pair q,
      // lane 4 + q its v_phi array; E at +0, F at +nh)
      dfl2* cb = nullptr;
      {
        const long long per_p = VEC ? 2LL * g.nh : (long long)g.nh;
        const long long moff = ((long long)T.mc * 2 + T.p) * per_p;
        if (!VEC && lane < 8) {
          const int cq = T.ct * (kNC / 2) + cc0 / 2 + lane;
          if (cq < ncplx) {
            const int r = cq / s.nf, f = cq - r * s.nf;
            cb = (dfl2*)s.f[f].out0 + (long long)r * s.f[f].out_ld + moff;
          }
        } else if (VEC && lane < 8) {
          const int pr = T.ct * (kNC / 4) + cc0 / 4 + (lane & 3);
          if (pr < npair) {
            const int r = pr / s.nf, f = pr - r * s.nf;
            cb = (dfl2*)(lane < 4 ? s.f[f].out0 : s.f[f].out1) + (long long)r * s.f[f].out_ld + moff;
          }
        }
      }
      const dfl2 z2 = {dfl(0), dfl(0)};
      if (T.nlp == 0) {  // odd parity of m = l_max: zeros
        for (int q = 0; q < 8; ++q) {
          dfl2* b = shfl_ptr(cb, q);
          if (b && row_ok) {
            b[jg] = z2;
            if (VEC) b[g.nh + jg] = z2;
          }
        }
        continue;
      }
      // exponents: this thread's row (both tables) and the warp's 16 columns
      const int erow0 = row_ok ? t.inv_exp[(size_t)T.mc * NHP + jg] : 0;
      const int erow1 = (VEC && row_ok) ? t.inv_exp[((size_t)g.n_m + T.mc) * NHP + jg] : 0;
      const short* ce = I.cexp + (long long)T.mc * nct * kNC + T.ct * kNC + cc0;
      if (!wait_full(&acc_full, acc_use, 1)) { ok = false; break; }
      tc::tc_fence_after();
      const uint32_t acc = tmem + lane_off + cc0;
      dfl P[16], D[16];
      drain16<S>(acc, P);
      if (VEC) drain16<S>(acc + kS * kNC, D);
      tc::tc_fence_before();
      tc::mbar_arrive(&acc_empty);  // tensor memory free for the next tile
      ++acc_use;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int ec = ce[i];
        P[i] = P[i] * pow2f(erow0 + ec - 14);
        if (VEC) D[i] = D[i] * pow2f(erow1 + ec - 14);
      }
      // every lane takes part in the pointer shuffles; rows past nh only skip the stores
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          dfl2* b = shfl_ptr(cb, q);
          dfl2 v;
          v.x = P[2 * q];
          v.y = P[2 * q + 1];
          if (b && row_ok) b[jg] = v;
        }
      } else {
        const float dm = (float)(T.mc * g.minc);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          dfl2* bt = shfl_ptr(cb, q);
          dfl2* bp = shfl_ptr(cb, 4 + q);
          // C = sum S P, B = sum T P; A = sum S dP, D = sum T dP
          const dfl Cr = P[4 * q], Ci = P[4 * q + 1], Br = P[4 * q + 2], Bi = P[4 * q + 3];
          const dfl Ar = D[4 * q], Ai = D[4 * q + 1], Dr = D[4 * q + 2], Di = D[4 * q + 3];
          // v_theta: U = i m B, W = A;   v_phi: U = i m C, W = -D
          const dfl Utr = -(Bi * dm), Uti = Br * dm;
          const dfl Upr = -(Ci * dm), Upi = Cr * dm;
          if (bt && row_ok) {
            dfl2 e, f;
            e.x = Utr + Ar; e.y = Uti + Ai;
            f.x = Utr - Ar; f.y = Uti - Ai;
            bt[jg] = e;
            bt[g.nh + jg] = f;
            e.x = Upr - Dr; e.y = Upi - Di;
            f.x = Upr + Dr; f.y = Upi + Di;
            bp[jg] = e;
            bp[g.nh + jg] = f;
          }
        }
      }
    }
  }
  if (!ok) atomicExch(&s_fail, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 0 && s_fail && one.t.err) atomicExch(one.t.err, 1);
  if (warp == 0) tc::tmem_dealloc(tmem, Occ<VEC, true>::TCOLS);
}

// ------------------------------------------------------------ analysis
struct FwdTile {
  int mc, p, lt, ct, nlp;
  __device__ void decode(const ShtGeom& g, const TcTables& t, int nct, int ix) {
    int rest;
    if (t.order == 0) {
      ct = ix % nct;
      rest = ix / nct;
      lt = rest % t.nlt;
      rest /= t.nlt;
    } else {
      lt = ix % t.nlt;
      rest = ix / t.nlt;
      ct = rest % nct;
      rest /= nct;
    }
    p = rest & 1;
    mc = rest >> 1;
    const int n_l = g.l_max - mc * g.minc + 1;
    nlp = (n_l + 1 - p) / 2;
  }
};

template <bool VEC, bool MULTI, int S>
__global__ void __launch_bounds__(Occ<VEC, false>::THREADS, Occ<VEC, false>::CPS)
    fwd_leg_oz(const __grid_constant__ OzFwd one, const OzFwd* __restrict__ many,
               const __grid_constant__ InstIndex X, int ntiles) {
  OZ_DIGITS(S);
  constexpr int NT = VEC ? 2 : 1;
  constexpr int NA = Rings<VEC, false>::NA, NB = Rings<VEC, false>::NB;
  constexpr uint32_t ASZ = NT * 16384;
  constexpr uint32_t BSZ = NT * kTS;  // mine (and other)
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t a_full[NA], a_empty[NA], b_full[NB], b_empty[NB], acc_full, acc_empty, fin;
  __shared__ uint64_t tr_full[kNTR], tr_empty[kNTR];
  __shared__ int tr_idx[kNTR];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail;
  unsigned char* sA = align1k(smem_raw);
  unsigned char* sB = sA + NA * ASZ;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    constexpr int NI = Occ<VEC, false>::NISS;  // every MMA thread commits to the empty / full barriers
    for (int i = 0; i < NA; ++i) { tc::mbar_init(&a_full[i], 1); tc::mbar_init(&a_empty[i], NI); }
    for (int i = 0; i < NB; ++i) { tc::mbar_init(&b_full[i], 1); tc::mbar_init(&b_empty[i], NI); }
    tc::mbar_init(&acc_full, NI);
    tc::mbar_init(&acc_empty, kEpiThreads);
    tc::mbar_init(&fin, NI);
    for (int i = 0; i < kNTR; ++i) { tc::mbar_init(&tr_full[i], 1); tc::mbar_init(&tr_empty[i], NI + kEpiThreads); }
    s_fail = 0;
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, Occ<VEC, false>::TCOLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  const TileRing R{tr_idx, tr_full, tr_empty};
  bool ok = true;
  FwdTile T;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t a_use = 0, b_use = 0, tr = 0;
      int ix = blockIdx.x;
      while (ok) {
        if (!ring_push(R, tr, ix < ntiles ? ix : -1)) { ok = false; break; }
        if (ix >= ntiles) break;
        const int next = atomicAdd(one.t.tile_ctr, 1) + (int)gridDim.x;
        int lix = ix;
        const OzFwd& I = tile_inst<MULTI>(one, many, X, lix);
        const TcTables& t = I.t;
        const int nct = I.nct;
        T.decode(I.g, t, nct, lix);
        ix = next;
        if (T.lt * 128 >= T.nlp) continue;
        for (int c = 0; c < t.ncj && ok; ++c) {
          const uint32_t bslot = b_use % NB;
          if (!wait_empty(&b_empty[bslot], b_use, NB)) { ok = false; break; }
          tc::mbar_expect_tx(&b_full[bslot], BSZ);
          const unsigned char* img = I.bimg + (((long long)T.mc * t.ncj + c) * nct + T.ct) * (2LL * kTS);
          tc::bulk_g2s(sB + bslot * BSZ, img + T.p * kTS, kTS, &b_full[bslot]);                     // mine
          if (VEC) tc::bulk_g2s(sB + bslot * BSZ + kTS, img + (1 - T.p) * kTS, kTS, &b_full[bslot]);  // other
          ++b_use;
          const uint32_t abytes = table_rows_bytes(T.nlp - T.lt * 128);
          for (int u = 0; u < kS; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_empty(&a_empty[slot], a_use, NA)) { ok = false; break; }
            tc::mbar_expect_tx(&a_full[slot], NT * abytes);
            for (int tb = 0; tb < NT; ++tb) {
              const long long blk =
                  t.fwd_blk0[T.mc] + ((((long long)T.p * t.nlt + T.lt) * 2 + tb) * t.ncj + c) * kS + u;
              tc::bulk_g2s(sA + slot * ASZ + tb * 16384, t.fwd_img + blk * 16384, abytes, &a_full[slot]);
            }
          }
        }
      }
      drain_copies<NA>(a_full, a_use);
      drain_copies<NB>(b_full, b_use);
    }
  } else if (warp == 1 || (Occ<VEC, false>::NISS == 2 && warp == 2 + kEpiThreads / 32)) {
    if (lane == 0) {  // MMA issuer(s)
      const int tb0 = warp == 1 ? 0 : 1, tb1 = Occ<VEC, false>::NISS == 2 ? tb0 + 1 : NT;
      uint32_t a_use = 0, b_use = 0, acc_use = 0, tr = 0;
      while (ok) {
        int ix;
        if (!ring_pop(R, tr, ix)) { ok = false; break; }
        if (ix < 0) break;
        const OzFwd& I = tile_inst<MULTI>(one, many, X, ix);
        T.decode(I.g, I.t, I.nct, ix);
        if (T.lt * 128 >= T.nlp) continue;
        if (!wait_empty(&acc_empty, acc_use, 1)) { ok = false; break; }
        tc::tc_fence_after();
        for (int c = 0; c < I.t.ncj && ok; ++c, ++b_use) {
          const uint32_t bslot = b_use % NB;
          if (!wait_full(&b_full[bslot], b_use, NB)) { ok = false; break; }
          for (int u = 0; u < kS; ++u, ++a_use) {
            const uint32_t slot = a_use % NA;
            if (!wait_full(&a_full[slot], a_use, NA)) { ok = false; break; }
            tc::tc_fence_after();
            issue_digit<NT, S>(tmem, sA + slot * ASZ, sB + bslot * BSZ, u, c == 0, kTS, 4, tb0, tb1);
            tc::mma_commit(&a_empty[slot]);
          }
          tc::mma_commit(&b_empty[bslot]);
        }
        tc::mma_commit(&acc_full);
        ++acc_use;
      }
      tc::mma_commit(&fin);
      if (!tc::mbar_wait(&fin, 0)) ok = false;
    }
  } else if (warp < 2 + kEpiThreads / 32) {  // epilogue
    const int q4 = warp & 3, half = (warp - 2) >> 2;
    const int cc0 = half * (kNC / 2);
    const int lr = 32 * q4 + lane;
    const uint32_t lane_off = (uint32_t)(32 * q4) << 16;
    uint32_t acc_use = 0, tr = 0;
    while (ok) {
      int ix;
      if (!ring_pop(R, tr, ix)) { ok = false; break; }
      if (ix < 0) break;
      const OzFwd& I = tile_inst<MULTI>(one, many, X, ix);
      const ShtGeom& g = I.g;
      const FwdSet& s = I.s;
      const TcTables& t = I.t;
      const int nct = I.nct;
      const int npair = s.nf * s.nlev;
      const int ncplx = npair * (VEC ? 2 : 1);
      T.decode(g, t, nct, ix);
      if (T.lt * 128 >= T.nlp) continue;
      const int m = T.mc * g.minc;
      const int lp = T.lt * 128 + lr;
      const int l = m + T.p + 2 * lp;
      const bool valid = lp < T.nlp;
      const int lm = g.lmoff[T.mc] + l - m;
      // per-column output bases and cut-offs (scalar: lane q < 8 complex column
      // q of this warp; vector: lane q < 4 pair q's S array, lane 4 + q its T array)
      double2* cb = nullptr;
      int clc = -1;
      if (lane < 8) {
        const int q = VEC ? (lane & 3) : lane;
        const int cq = VEC ? T.ct * (kNC / 4) + cc0 / 4 + q : T.ct * (kNC / 2) + cc0 / 2 + q;
        if (cq < (VEC ? npair : ncplx)) {
          const int r = cq / s.nf, f = cq - r * s.nf;
          cb = (VEC && lane >= 4 ? s.f[f].out1 : s.f[f].out0) + (long long)r * s.f[f].out_ld;
          clc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
        }
      }
      const int erow0 = valid ? t.fwd_exp[lm] : 0;
      const int erow1 = (VEC && valid) ? t.fwd_exp[(size_t)g.lm_max + lm] : 0;
      const short* ce = I.cexp + (long long)T.mc * 2 * nct * kNC + T.ct * kNC + cc0;
      const short* ce_mine = ce + (long long)T.p * nct * kNC;
      const short* ce_other = ce + (long long)(1 - T.p) * nct * kNC;
      if (!wait_full(&acc_full, acc_use, 1)) { ok = false; break; }
      tc::tc_fence_after();
      const uint32_t acc = tmem + lane_off + cc0;
      dfl D0[16], D1[16];
      drain16<S>(acc, D0);
      if (VEC) drain16<S>(acc + kS * kNC, D1);
      tc::tc_fence_before();
      tc::mbar_arrive(&acc_empty);
      ++acc_use;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        D0[i] = D0[i] * pow2f(erow0 + ce_mine[i] - 14);
        if (VEC) D1[i] = D1[i] * pow2f(erow1 + ce_other[i] - 14);
      }
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          double2* b = shfl_ptr(cb, q);
          const int lc = __shfl_sync(0xffffffffu, clc, q);
          if (b && valid)
            b[lm] = (l <= lc) ? make_double2(df_to_double(D0[2 * q]), df_to_double(D0[2 * q + 1]))
                              : make_double2(0.0, 0.0);
        }
      } else {
        const float dm = (float)m;
        // 1/(l(l+1)) as a double-float (l = 0 only has S = T = 0 inputs)
        const dfl inv_ll = df_from_double(l > 0 ? 1.0 / ((double)l * (double)(l + 1)) : 1.0);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          double2* bs = shfl_ptr(cb, q);
          double2* bt = shfl_ptr(cb, 4 + q);
          const int lc = __shfl_sync(0xffffffffu, clc, q);
          // A = sum F1_mine P, D = sum F2_mine P, C = sum F1_other dP, B = sum F2_other dP
          const dfl Ar = D0[4 * q], Ai = D0[4 * q + 1], Dr = D0[4 * q + 2], Di = D0[4 * q + 3];
          const dfl Cr = D1[4 * q], Ci = D1[4 * q + 1], Br = D1[4 * q + 2], Bi = D1[4 * q + 3];
          // S = (-i m A + B) / (l(l+1)),  T = (-C - i m D) / (l(l+1))
          const dfl Sr = (Ai * dm + Br) * inv_ll, Si = (Bi - Ar * dm) * inv_ll;
          const dfl Tr = (Di * dm - Cr) * inv_ll, Ti = -(Ci + Dr * dm) * inv_ll;
          double2 Sv = make_double2(df_to_double(Sr), df_to_double(Si));
          double2 Tv = make_double2(df_to_double(Tr), df_to_double(Ti));
          if (l > lc) { Sv = make_double2(0.0, 0.0); Tv = Sv; }
          if (bs && valid) {
            bs[lm] = Sv;
            bt[lm] = Tv;
          }
        }
      }
    }
  }
  if (!ok) atomicExch(&s_fail, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 0 && s_fail && one.t.err) atomicExch(one.t.err, 1);
  if (warp == 0) tc::tmem_dealloc(tmem, Occ<VEC, false>::TCOLS);
}

size_t align256_oz(size_t x) { return (x + 255) & ~(size_t)255; }
size_t oz_tiles_bytes_inv(const TcTables& t, int nct) { return align256_oz((size_t)t.npc * nct * tile_bytes(t.ndig)); }
size_t oz_tiles_bytes_fwd(const ShtGeom& g, const TcTables& t, int nct) {
  return align256_oz((size_t)g.n_m * t.ncj * nct * 2 * tile_bytes(t.ndig));
}

int num_sms_oz() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

long long oz_nct(int ncplx) { return (ncplx + kNC / 2 - 1) / (kNC / 2); }

// tiles of the persistent kernels and blocks of the pack kernels of one instance
long long oz_inv_tiles(const ShtGeom& g, const TcTables& t, int nct) { return (long long)nct * t.ntt * 2 * g.n_m; }
long long oz_fwd_tiles(const ShtGeom& g, const TcTables& t, int nct) { return (long long)nct * t.nlt * 2 * g.n_m; }

template <bool VEC, bool MULTI, int S>
cudaError_t launch_inv_oz_s(const OzInv& one, const OzInv* many, const InstIndex& X, long long nblocks,
                            long long ntiles, int lmax, cudaStream_t st) {
  constexpr int NT = VEC ? 2 : 1, NA = Rings<VEC, true>::NA, NB = Rings<VEC, true>::NB;
  constexpr uint32_t kTS = tile_bytes(S);
  if (ntiles <= 0) return cudaSuccess;
  const size_t psmem = 1024 + 2 * (size_t)kTS;
  const dim3 pgrid = MULTI ? dim3((unsigned)nblocks) : dim3(one.nct, one.g.n_m);
  // one pass when every order of every instance has at most two chunks per parity
  if (tc_nch(lmax + 1) > 2) {
    CUDA_TRY(cudaFuncSetAttribute(pack_inv_oz<VEC, MULTI, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
    pack_inv_oz<VEC, MULTI, S><<<pgrid, kPackThreads, psmem, st>>>(one, many, X);
  } else {
    CUDA_TRY(cudaFuncSetAttribute(pack_inv_oz1<VEC, MULTI, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
    pack_inv_oz1<VEC, MULTI, S><<<pgrid, kPack1Threads, psmem, st>>>(one, many, X);
  }
  CUDA_TRY(cudaGetLastError());
  const size_t smem = 1024 + (size_t)NA * NT * 16384 + (size_t)NB * kTS;
  CUDA_TRY(cudaFuncSetAttribute(inv_leg_oz<VEC, MULTI, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (int)std::min<long long>(ntiles, (long long)num_sms_oz() * Occ<VEC, true>::CPS);
  CUDA_TRY(cudaMemsetAsync(one.t.tile_ctr, 0, sizeof(int), st));
  inv_leg_oz<VEC, MULTI, S><<<grid, Occ<VEC, true>::THREADS, smem, st>>>(one, many, X, (int)ntiles);
  return cudaGetLastError();
}

template <bool VEC, bool MULTI, int S>
cudaError_t launch_fwd_oz_s(const OzFwd& one, const OzFwd* many, const InstIndex& X, long long nblocks,
                            long long ntiles, cudaStream_t st) {
  constexpr int NT = VEC ? 2 : 1, NA = Rings<VEC, false>::NA, NB = Rings<VEC, false>::NB;
  constexpr uint32_t kTS = tile_bytes(S);
  if (ntiles <= 0) return cudaSuccess;
  const size_t psmem = 1024 + 2 * (size_t)kTS;
  CUDA_TRY(cudaFuncSetAttribute(pack_fwd_oz<VEC, MULTI, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
  const dim3 pgrid = MULTI ? dim3((unsigned)nblocks) : dim3(one.nct, one.g.n_m);
  pack_fwd_oz<VEC, MULTI, S><<<pgrid, kPackThreads, psmem, st>>>(one, many, X);
  CUDA_TRY(cudaGetLastError());
  const size_t smem = 1024 + (size_t)NA * NT * 16384 + (size_t)NB * NT * kTS;
  CUDA_TRY(cudaFuncSetAttribute(fwd_leg_oz<VEC, MULTI, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (int)std::min<long long>(ntiles, (long long)num_sms_oz() * Occ<VEC, false>::CPS);
  CUDA_TRY(cudaMemsetAsync(one.t.tile_ctr, 0, sizeof(int), st));
  fwd_leg_oz<VEC, MULTI, S><<<grid, Occ<VEC, false>::THREADS, smem, st>>>(one, many, X, (int)ntiles);
  return cudaGetLastError();
}

// the digit count of the tables (t.ndig: 7 or 5) selects the instantiation
// lmax: the largest l_max of the launch's instances
template <bool VEC, bool MULTI>
cudaError_t launch_inv_oz(const OzInv& one, const OzInv* many, const InstIndex& X, long long nblocks, long long ntiles,
                          int lmax, cudaStream_t st) {
  if (one.t.ndig == 7) return launch_inv_oz_s<VEC, MULTI, 7>(one, many, X, nblocks, ntiles, lmax, st);
  if (one.t.ndig == 5) return launch_inv_oz_s<VEC, MULTI, 5>(one, many, X, nblocks, ntiles, lmax, st);
  return cudaErrorInvalidValue;
}
template <bool VEC, bool MULTI>
cudaError_t launch_fwd_oz(const OzFwd& one, const OzFwd* many, const InstIndex& X, long long nblocks, long long ntiles,
                          cudaStream_t st) {
  if (one.t.ndig == 7) return launch_fwd_oz_s<VEC, MULTI, 7>(one, many, X, nblocks, ntiles, st);
  if (one.t.ndig == 5) return launch_fwd_oz_s<VEC, MULTI, 5>(one, many, X, nblocks, ntiles, st);
  return cudaErrorInvalidValue;
}

}  // namespace

// Data-image bytes of one call: the digit tiles, then the column exponents.
size_t oz_data_bytes(const ShtGeom& g, const TcTables& t, int ncplx, bool inverse) {
  const long long nct = oz_nct(ncplx);
  const size_t tiles = inverse ? oz_tiles_bytes_inv(t, (int)nct) : oz_tiles_bytes_fwd(g, t, (int)nct);
  const size_t ex = (size_t)g.n_m * (inverse ? 1 : 2) * nct * kNC * sizeof(short);
  return tiles + ex;
}

void oz_table_layout(const ShtGeom& g, int digits, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
                     std::vector<long long>& fwd_blk0, long long* inv_blocks, long long* fwd_blocks) {
  tc_table_layout_bpc(g, digits, ntt, nlt, ncj, inv_blk0, fwd_blk0, inv_blocks, fwd_blocks);
}

template <int S>
cudaError_t build_oz_images_s(const ShtGeom& g, const TcTables& t, unsigned char* inv_img, short* inv_exp,
                              unsigned char* fwd_img, short* fwd_exp, cudaStream_t st) {
  {
    const long long n = (long long)g.n_m * 2 * t.ntt * 128;
    build_inv_oz_kernel<S><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(g, t, inv_img, inv_exp);
    CUDA_TRY(cudaGetLastError());
  }
  {
    const long long n = (long long)g.n_m * 4 * t.nlt * 128;
    build_fwd_oz_kernel<S><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(g, t, fwd_img, fwd_exp);
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

cudaError_t build_oz_images(const ShtGeom& g, const TcTables& t, unsigned char* inv_img, short* inv_exp,
                            unsigned char* fwd_img, short* fwd_exp, cudaStream_t st) {
  if (t.ndig == 7) return build_oz_images_s<7>(g, t, inv_img, inv_exp, fwd_img, fwd_exp, st);
  if (t.ndig == 5) return build_oz_images_s<5>(g, t, inv_img, inv_exp, fwd_img, fwd_exp, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_inv_legendre_oz(const ShtGeom& g, const InvSet& s, bool vec, const TcTables& t,
                                   unsigned char* bimg, cudaStream_t st) {
  std::vector<OzInv> one(1);
  one[0].g = g;
  one[0].s = s;
  one[0].t = t;
  one[0].bimg = bimg;
  long long nblocks = 0, ntiles = 0;
  oz_layout_insts(one.data(), 1, vec, &nblocks, &ntiles);
  InstIndex X{};
  return vec ? launch_inv_oz<true, false>(one[0], nullptr, X, nblocks, ntiles, g.l_max, st)
             : launch_inv_oz<false, false>(one[0], nullptr, X, nblocks, ntiles, g.l_max, st);
}

cudaError_t launch_fwd_legendre_oz(const ShtGeom& g, const FwdSet& s, bool vec, const TcTables& t,
                                   unsigned char* bimg, cudaStream_t st) {
  std::vector<OzFwd> one(1);
  one[0].g = g;
  one[0].s = s;
  one[0].t = t;
  one[0].bimg = bimg;
  long long nblocks = 0, ntiles = 0;
  oz_layout_insts(one.data(), 1, vec, &nblocks, &ntiles);
  InstIndex X{};
  return vec ? launch_fwd_oz<true, false>(one[0], nullptr, X, nblocks, ntiles, st)
             : launch_fwd_oz<false, false>(one[0], nullptr, X, nblocks, ntiles, st);
}

template <class Set>
void oz_layout_insts(LegInst<Set>* inst, int n, bool vec, long long* nblocks, long long* ntiles) {
  constexpr bool INV = std::is_same<Set, InvSet>::value;
  long long nb = 0, nt = 0;
  for (int i = 0; i < n; ++i) {
    LegInst<Set>& I = inst[i];
    const int ncplx = I.s.nf * I.s.nlev * (vec ? 2 : 1);
    I.nct = (int)oz_nct(ncplx > 0 ? ncplx : 0);
    I.cexp = (short*)(I.bimg + (INV ? oz_tiles_bytes_inv(I.t, I.nct) : oz_tiles_bytes_fwd(I.g, I.t, I.nct)));
    I.blk0 = (int)nb;
    I.tile0 = (int)nt;
    I.pad_ = 0;
    nb += (long long)I.nct * I.g.n_m;
    nt += INV ? oz_inv_tiles(I.g, I.t, I.nct) : oz_fwd_tiles(I.g, I.t, I.nct);
  }
  *nblocks = nb;
  *ntiles = nt;
}
template void oz_layout_insts<InvSet>(LegInst<InvSet>*, int, bool, long long*, long long*);
template void oz_layout_insts<FwdSet>(LegInst<FwdSet>*, int, bool, long long*, long long*);

cudaError_t launch_inv_legendre_oz_multi(const LegInst<InvSet>* inst, const LegInst<InvSet>* d_inst, int n,
                                         bool vec, long long nblocks, long long ntiles, cudaStream_t st) {
  if (n < 1 || n > kMaxGroupInst) return cudaErrorInvalidValue;
  const InstIndex X = inst_index(inst, n);
  int lmax = 0;
  for (int i = 0; i < n; ++i) lmax = std::max(lmax, inst[i].g.l_max);
  return vec ? launch_inv_oz<true, true>(inst[0], d_inst, X, nblocks, ntiles, lmax, st)
             : launch_inv_oz<false, true>(inst[0], d_inst, X, nblocks, ntiles, lmax, st);
}

cudaError_t launch_fwd_legendre_oz_multi(const LegInst<FwdSet>* inst, const LegInst<FwdSet>* d_inst, int n,
                                         bool vec, long long nblocks, long long ntiles, cudaStream_t st) {
  if (n < 1 || n > kMaxGroupInst) return cudaErrorInvalidValue;
  const InstIndex X = inst_index(inst, n);
  return vec ? launch_fwd_oz<true, true>(inst[0], d_inst, X, nblocks, ntiles, st)
             : launch_fwd_oz<false, true>(inst[0], d_inst, X, nblocks, ntiles, st);
}
