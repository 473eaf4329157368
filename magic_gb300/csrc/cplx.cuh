// Small complex helpers for double2 / float2 (device only).
#pragma once
#include <cuda_runtime.h>
#include "dfloat.cuh"

template <typename T> struct V2;
template <> struct V2<double> { typedef double2 t; };
template <> struct V2<float> { typedef float2 t; };
template <> struct V2<dfl> { typedef dfl2 t; };

template <typename T2> struct ScalarOf;
template <> struct ScalarOf<double2> { typedef double t; };
template <> struct ScalarOf<float2> { typedef float t; };
template <> struct ScalarOf<dfl2> { typedef dfl t; };

__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ dfl2 mk2(dfl a, dfl b) { dfl2 r; r.x = a; r.y = b; return r; }

template <typename T2> __device__ __forceinline__ T2 zero2() {
  T2 z; z.x = 0; z.y = 0; return z;
}
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { T2 r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { T2 r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  T2 r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <> __device__ __forceinline__ dfl2 cmul<dfl2>(dfl2 a, dfl2 b) {
  dfl2 r; r.x = df_dot2_sub(a.x, b.x, a.y, b.y); r.y = df_dot2_add(a.x, b.y, a.y, b.x); return r;
}
template <typename T2> __device__ __forceinline__ T2 cconj(T2 a) { a.y = -a.y; return a; }
// multiply by +i (s>0) or -i (s<0)
template <typename T2> __device__ __forceinline__ T2 cmuli(T2 a, int s) {
  T2 r; if (s > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; } return r;
}
template <typename T2, typename S> __device__ __forceinline__ T2 cscale(T2 a, S s) {
  T2 r; r.x = a.x * s; r.y = a.y * s; return r;
}


template <typename T2> __device__ __forceinline__ T2 shfl_xor2(T2 v, int d) {
  T2 r; r.x = __shfl_xor_sync(0xffffffffu, v.x, d); r.y = __shfl_xor_sync(0xffffffffu, v.y, d); return r;
}
template <> __device__ __forceinline__ dfl2 shfl_xor2<dfl2>(dfl2 v, int d) {
  dfl2 r;
  r.x.h = __shfl_xor_sync(0xffffffffu, v.x.h, d); r.x.l = __shfl_xor_sync(0xffffffffu, v.x.l, d);
  r.y.h = __shfl_xor_sync(0xffffffffu, v.y.h, d); r.y.l = __shfl_xor_sync(0xffffffffu, v.y.l, d);
  return r;
}
// b + sg a for sg = +-1 (the cross-lane butterflies of the FFT)
template <typename T> __device__ __forceinline__ T add_signed(T sg, T a, T b) { return fma(sg, a, b); }
template <> __device__ __forceinline__ dfl add_signed<dfl>(dfl sg, dfl a, dfl b) {
  return b + (sg.h < 0.f ? -a : a);
}

// FP64 <-> FP32 conversions with integer instructions only (the FP64 pipe of
// GB300 is narrow; these conversions run on the integer/FP32 pipes).
// d2f: round to nearest even; magnitudes below 2^-126 flush to zero, beyond
// the FP32 range give +-Inf, NaN stays NaN.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int hi = (unsigned int)(b >> 32), lo = (unsigned int)b;
  const int e = (int)((hi >> 20) & 0x7FF);
  const unsigned int sign = hi & 0x80000000u;
  if (e < 1023 - 126) return __uint_as_float(sign);
  const unsigned int mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  if (e > 1023 + 127) {
    const bool nan = e == 0x7FF && ((hi & 0xFFFFFu) | lo) != 0u;
    return __uint_as_float(sign | 0x7F800000u | (nan ? 0x400000u : 0u));
  }
  unsigned int f = sign | ((unsigned int)(e - 1023 + 127) << 23) | mant;
  const unsigned int rbit = (lo >> 28) & 1u;
  const unsigned int sticky = (lo & 0x0FFFFFFFu) != 0u;
  if (rbit && (sticky || (mant & 1u))) f += 1u;  // a carry may round up to Inf: correct
  return __uint_as_float(f);
}
// exact widening (normal numbers, zero, Inf and NaN; FP32 subnormals flush to zero)
// on 32-bit halves: the magnitude shifted right by 3 puts the exponent and the
// top 20 mantissa bits in place, + (1023 - 127) << 20 rebiases the exponent
__device__ __forceinline__ double f2d_int(float x) {
  const unsigned int u = __float_as_uint(x);
  const unsigned int a = u & 0x7FFFFFFFu;
  unsigned int hi = (a >> 3) + 0x38000000u;
  unsigned int lo = u << 29;
  if (a >= 0x7F800000u) hi |= 0x7FF00000u;  // Inf, NaN (payload kept)
  if (a < 0x00800000u) hi = lo = 0u;        // zero, subnormals
  return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}

// Conversions between a transform's working type T and the FP64 of the
// grids and spectra: identity for double, integer-only for float.
template <typename T> __device__ __forceinline__ double to_f64(T x);
template <> __device__ __forceinline__ double to_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ double to_f64<float>(float x) { return f2d_int(x); }
template <> __device__ __forceinline__ double to_f64<dfl>(dfl x) { return df_to_double(x); }
template <typename T> __device__ __forceinline__ T from_f64(double x);
template <> __device__ __forceinline__ double from_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ float from_f64<float>(double x) { return d2f_int(x); }
template <> __device__ __forceinline__ dfl from_f64<dfl>(double x) { return df_from_double(x); }

template <typename T2> __device__ __forceinline__ T2 cvt2(double2 a);
template <> __device__ __forceinline__ double2 cvt2<double2>(double2 a) { return a; }
template <> __device__ __forceinline__ float2 cvt2<float2>(double2 a) { return make_float2(d2f_int(a.x), d2f_int(a.y)); }
template <> __device__ __forceinline__ dfl2 cvt2<dfl2>(double2 a) { dfl2 r; r.x = df_from_double(a.x); r.y = df_from_double(a.y); return r; }
__device__ __forceinline__ double2 to_d2(double2 a) { return a; }
__device__ __forceinline__ double2 to_d2(float2 a) { return make_double2(f2d_int(a.x), f2d_int(a.y)); }
__device__ __forceinline__ double2 to_d2(dfl2 a) { return make_double2(df_to_double(a.x), df_to_double(a.y)); }

// A grid value read in FP64 into a transform's working type: plain
// conversion for float and double, the double-float split for dfl.
template <typename T> __device__ __forceinline__ T cvt_in(double x) { return (T)x; }
template <> __device__ __forceinline__ dfl cvt_in<dfl>(double x) { return df_from_double(x); }
