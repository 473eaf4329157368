// Double-float ("float-float") arithmetic on the FP32 pipes: a value is the
// unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, about
// 48 significant bits.  GB300 runs FP32 at ~74x its FP64 rate, so the
// azimuthal FFTs of the FP64-accurate tensor-core form compute in this type.
//
// Algorithms: Knuth's TwoSum and Dekker's FastTwoSum for the error-free
// additions, the FMA-based TwoProd for products (the "sloppy" double-float
// addition and multiplication of Dekker 1971 and Hida, Li and Bailey's QD
// library).  Every operation goes through __fadd_rn / __fmul_rn / __fmaf_rn
// so that the compiler neither contracts nor reorders the error terms.
//
// Range: the FP32 exponent range.  Magnitudes must stay below 2^127; values
// below ~2^-100 lose relative precision (their lo parts underflow).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

struct dfl {
  float h, l;
  dfl() = default;
  __host__ __device__ constexpr dfl(float a, float b) : h(a), l(b) {}
  // small integers and literal constants (folded at compile time)
  __host__ __device__ constexpr dfl(int x) : h((float)x), l(0.f) {}
  __host__ __device__ explicit dfl(double x) : h((float)x), l((float)(x - (double)(float)x)) {}
};
struct dfl2 {
  dfl x, y;
};

__device__ __forceinline__ dfl mkdf(float h, float l) { return dfl(h, l); }

// s + e = a + b exactly (|a| >= |b| not required)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// h + l = s + e, normalized (requires |s| >= |e| or s == 0)
__device__ __forceinline__ dfl fast_two_sum(float s, float e) {
  const float h = __fadd_rn(s, e);
  return mkdf(h, __fsub_rn(e, __fsub_rn(h, s)));
}

// The arithmetic is "lazy": sums and products return the unevaluated pair
// (leading result, error terms) without the final FastTwoSum, so lo may
// exceed ulp(hi)/2 by a few units.  The represented value keeps an absolute
// error near 2^-48 of the operands, which is what the FFTs' normwise bound
// needs, at ~20% fewer operations; df_norm restores the normalized form.
__device__ __forceinline__ dfl df_norm(dfl a) { return fast_two_sum(a.h, a.l); }
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return mkdf(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return mkdf(-a.h, -a.l); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return mkdf(p, e);
}
// by an FP32 number
__device__ __forceinline__ dfl operator*(dfl a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return mkdf(p, e);
}
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl& operator*=(dfl& a, dfl b) { return a = a * b; }
// exact scaling by a power of two
__device__ __forceinline__ dfl df_ldexp(dfl a, int e) { return mkdf(ldexpf(a.h, e), ldexpf(a.l, e)); }

// FP64 <-> double-float with integer instructions (the FP64 pipe of GB300
// is narrow).  From FP64: the 53-bit mantissa is T 2^29 + R with T its top
// 24 bits; hi = T rounded to nearest even (T + 1 and R - 2^29 when rounding
// up), lo = R 2^(e-1075) rounded to FP32 by one integer -> float conversion
// and moved to its exponent by an integer add (lo = RN(x - hi), |R| <= 2^28).
// Below 2^-126 hi (and lo) are signed zeros, a lo below 2^-126 is zero; above
// the FP32 range hi is Inf (NaN for NaN) and lo zero.  Back: hi + lo rounded
// to FP64 (one FP64 add).
__device__ __forceinline__ double f2d_exact_int(float x);
__device__ __forceinline__ dfl df_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int whi = (unsigned int)(b >> 32), wlo = (unsigned int)b;
  const unsigned int sign = whi & 0x80000000u;
  const int e = (int)((whi >> 20) & 0x7FF);
  if (e < 1023 - 126) return mkdf(__uint_as_float(sign), __uint_as_float(sign));
  if (e > 1023 + 127) {
    const bool nan = e == 0x7FF && ((whi & 0xFFFFFu) | wlo) != 0u;
    return mkdf(__uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u)), 0.f);
  }
  unsigned int T = 0x800000u | ((whi & 0xFFFFFu) << 3) | (wlo >> 29);
  int R = (int)(wlo & 0x1FFFFFFFu);
  const bool up = R > 0x10000000 || (R == 0x10000000 && (T & 1u));
  T += up ? 1u : 0u;
  R -= up ? 0x20000000 : 0;
  // T = 2^24 after rounding carries into the exponent field (Inf past the range)
  const unsigned int hb = sign | (((unsigned int)(e - 1023 + 127) << 23) + (T - 0x800000u));
  const float rf = __int2float_rn(sign ? -R : R);
  unsigned int lb = __float_as_uint(rf);
  const int sh = e - 1075;
  lb = (rf != 0.f && (int)((lb >> 23) & 0xFFu) + sh > 0) ? lb + ((unsigned int)sh << 23) : (lb & 0x80000000u);
  return mkdf(__uint_as_float(hb), __uint_as_float(lb));
}
__device__ __forceinline__ double df_to_double(dfl a) { return f2d_exact_int(a.h) + f2d_exact_int(a.l); }

// exact for normal numbers, zero, Inf and NaN (FP32 subnormals flush to zero)
__device__ __forceinline__ double f2d_exact_int(float x) {
  const unsigned int u = __float_as_uint(x);
  const unsigned int a = u & 0x7FFFFFFFu;
  unsigned int hi = (a >> 3) + 0x38000000u;
  unsigned int lo = u << 29;
  if (a >= 0x7F800000u) hi |= 0x7FF00000u;
  if (a < 0x00800000u) hi = lo = 0u;
  return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}

// Complex double-float: the real and imaginary parts of a product each take
// one TwoSum of the two leading products and one normalization.
__device__ __forceinline__ dfl df_dot2_sub(dfl a, dfl b, dfl c, dfl d) {  // a b - c d
  const float p1 = __fmul_rn(a.h, b.h), p2 = __fmul_rn(c.h, d.h);
  const float e1 = __fmaf_rn(a.h, b.h, -p1), e2 = __fmaf_rn(c.h, d.h, -p2);
  float s, t;
  two_sum(p1, -p2, s, t);
  float lo = __fadd_rn(t, __fsub_rn(e1, e2));
  lo = __fmaf_rn(a.h, b.l, lo);
  lo = __fmaf_rn(a.l, b.h, lo);
  lo = __fmaf_rn(-c.h, d.l, lo);
  lo = __fmaf_rn(-c.l, d.h, lo);
  return mkdf(s, lo);
}
__device__ __forceinline__ dfl df_dot2_add(dfl a, dfl b, dfl c, dfl d) {  // a b + c d
  return df_dot2_sub(a, b, -c, d);
}
