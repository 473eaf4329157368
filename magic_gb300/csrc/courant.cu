// Courant condition of the radial loop on the device: courant.f90:54-278, the
// branch the reference compiles (XSH_COURANT == 0, :193-276).  Per radial
// level, the maxima over the (theta, phi) grid of
//   vr2 = or4 (cf2 vflr2 + af2 valr^2 / (valr + valri2)),
//   vh2 = or2 (cf2 vflh2 + af2 valh^2 / (valh + valhi2)),
//   vflr2 = orho2 vr^2,  valr = LFfac orho1 br^2,
//   vflh2 = (vt^2 + vp^2) / sin^2(theta) orho2,  valh = LFfac (bt^2 + bp^2) / sin^2(theta) orho1,
// (without the Lorentz force: vr2 = cf2 or4 vflr2, vh2 = cf2 or2 vflh2), then
// dtrkc = min(dtrkc, sqrt(delxr2 / vr2max)) and the same for dthkc, where the
// maximum is not 0.  Products and sums are rounded one by one in the
// reference's order (no fused multiply-adds), so a CPU restatement evaluated
// the same way differs only through its own 1/sin^2(theta) table.  A term
// that is 0/0 (valr = valri2 = 0) does not enter the maximum.
#include "common.cuh"
#include "internal.h"

namespace {

constexpr int kCourThreads = 256;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ double block_max(double v, double* red) {
  for (int d = 16; d >= 1; d >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, d));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  v = 0.0;
  if (threadIdx.x < kCourThreads / 32) v = red[threadIdx.x];
  if (warp == 0)
    for (int d = 16; d >= 1; d >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, d));
  __syncthreads();
  return v;
}

// Per-level constants of both forms of a point's two Courant terms.
struct CourLevel {
  double orho1, orho2, o2, o4, cf2, af2, LFfac, valri2, valhi2;
  // FP32 estimate: a_r = A1 vr^2 [+ A2 v v / (v + RI), v = KV br^2],
  //                a_h = B1 s (vt^2 + vp^2) [+ B2 w w / (w + HI), w = KV s (bt^2 + bp^2)]
  float A1, A2, KV, RI, B1, B2, HI;
  bool fast;  // every FP32 constant is 0 or in [2^-30, 2^30]
};

__device__ __forceinline__ bool in_window(float c) { return c == 0.0f || (c >= 0x1p-30f && c <= 0x1p30f); }

__device__ __forceinline__ CourLevel level_constants(const CourantArgs& a, int lev, bool mag) {
  CourLevel c;
  c.orho1 = a.orho1[lev]; c.orho2 = a.orho2[lev]; c.o2 = a.or2[lev]; c.o4 = a.or4[lev];
  c.cf2 = mul(a.courfac, a.courfac); c.af2 = mul(a.alffac, a.alffac); c.LFfac = a.LFfac;
  c.valri2 = 0.0; c.valhi2 = 0.0;
  if (a.alf_damp) {
    const double h = mul(0.5, add(1.0, a.opm));
    c.valri2 = mul(h, h) / a.delxr2[lev];
    c.valhi2 = mul(h, h) / a.delxh2[lev];
  }
  if (mag) {
    c.A1 = (float)(c.o4 * c.cf2 * c.orho2); c.A2 = (float)(c.o4 * c.af2);
    c.B1 = (float)(c.o2 * c.cf2 * c.orho2); c.B2 = (float)(c.o2 * c.af2);
  } else {
    c.A1 = (float)(c.cf2 * c.o4 * c.orho2); c.A2 = 0.0f;
    c.B1 = (float)(c.cf2 * c.o2 * c.orho2); c.B2 = 0.0f;
  }
  c.KV = (float)(c.LFfac * c.orho1); c.RI = (float)c.valri2; c.HI = (float)c.valhi2;
  c.fast = in_window(c.A1) && in_window(c.A2) && in_window(c.B1) && in_window(c.B2) &&
           (!mag || (in_window(c.KV) && in_window(c.RI) && in_window(c.HI)));
  return c;
}

// The reference's terms of one point, rounded one by one in its order.
template <bool MAG>
__device__ __forceinline__ double exact_r(const CourLevel& c, double vr, double br) {
  const double vflr2 = mul(mul(c.orho2, vr), vr);
  if (!MAG) return mul(mul(c.cf2, c.o4), vflr2);
  const double valr = mul(mul(mul(br, br), c.LFfac), c.orho1);
  const double valr2 = mul(valr, valr) / add(valr, c.valri2);
  return mul(c.o4, add(mul(c.cf2, vflr2), mul(c.af2, valr2)));
}
template <bool MAG>
__device__ __forceinline__ double exact_h(const CourLevel& c, double vt, double vp, double bt, double bp, double os2) {
  const double vflh2 = mul(mul(add(mul(vt, vt), mul(vp, vp)), os2), c.orho2);
  if (!MAG) return mul(mul(c.cf2, c.o2), vflh2);
  const double valh2 = mul(mul(mul(add(mul(bt, bt), mul(bp, bp)), c.LFfac), os2), c.orho1);
  const double valh2m = mul(valh2, valh2) / add(valh2, c.valhi2);
  return mul(c.o2, add(mul(c.cf2, vflh2), mul(c.af2, valh2m)));
}

// |x| as FP32 from the high word of x (mantissa truncated to 20 bits, relative
// error below 2^-20): below 2^-126 it gives at most 2^-126, from 2^128 (and
// for Inf / NaN) +Inf.  Integer operations only.
__device__ __forceinline__ float hi_abs_f32(double x) {
  unsigned m = (unsigned)__double2hiint(x) & 0x7FFFFFFFu;
  m = min(max(m, 0x38000000u), 0x47F00000u);
  return __uint_as_float((m - 0x38000000u) << 3);
}

template <bool MAG>
__device__ __forceinline__ float approx_r(const CourLevel& c, float vr, float br) {
  float a = c.A1 * (vr * vr);
  if (MAG) {
    const float v = c.KV * (br * br);
    a += c.A2 * (v * (v / (v + c.RI)));  // v (v / (v + RI)): no underflow of v^2
  }
  return a;
}
template <bool MAG>
__device__ __forceinline__ float approx_h(const CourLevel& c, float vt, float vp, float bt, float bp, float s) {
  float a = c.B1 * (s * (vt * vt + vp * vp));
  if (MAG) {
    const float w = c.KV * (s * (bt * bt + bp * bp));
    a += c.B2 * (w * (w / (w + c.HI)));
  }
  return a;
}

__device__ __forceinline__ float finite_or_zero(float a) { return a < __int_as_float(0x7F800000) ? a : 0.0f; }

// Maxima over the grid of one level (blockIdx.y) of the two Courant terms.
// Evaluating a point's terms in FP64 in the reference's order costs about
// 45 FP64 operations (two divisions), which bounds the kernel by the FP64
// pipe on this GPU; so every point first gets an FP32 estimate a of each term
// from the high words of its inputs (integer and FP32 operations only).  With
// constants in [2^-30, 2^30] and every term a sum of non-negative products,
// |a - e| <= 2^-16 e + 2^-50 for the FP64 value e whenever a is finite (no
// overflow; underflow contributes the absolute part).  If p is the point of
// the largest e, then for every point q with finite a_q,
//   a_p >= (1 - 2^-15) a_q - 2^-49,
// so a point whose estimate is below (1 - 2^-13) M - 2^-49, M the largest
// finite estimate seen so far in the block, cannot hold the maximum and is
// skipped; every other point (and every point with an infinite or NaN
// estimate, and every point of a level whose constants leave the window) is
// evaluated exactly.  The maxima are therefore the reference's values, bit
// for bit; M is shared by the block's warps through shared memory, so only
// a few points per warp take the FP64 path.  Threads handle pairs of rows
// (2j, 2j+1: one theta_j); PAIR loads them as 16-byte pairs.
template <bool MAG, bool PAIR>
__global__ void __launch_bounds__(kCourThreads) courant_reduce(const ShtGeom g, const CourantArgs a,
                                                               unsigned long long* mx) {
  __shared__ double red[kCourThreads / 32];
  __shared__ unsigned m_r, m_h;  // bits of the largest finite estimates (non-negative floats order as integers)
  const int lev = blockIdx.y, lane = threadIdx.x & 31;
  const CourLevel c = level_constants(a, lev, MAG);
  if (threadIdx.x == 0) { m_r = 0u; m_h = 0u; }
  __syncthreads();
  const long long o0 = (long long)lev * a.ld;
  const unsigned nh = (unsigned)(g.n_theta / 2), total = nh * (unsigned)g.n_phi;
  const unsigned stride = gridDim.x * blockDim.x;
  const float kfac = 1.0f - 0x1p-13f, tau2 = 0x1p-49f;
  double vr2max = 0.0, vh2max = 0.0;
  for (unsigned base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total; base += stride) {
    const unsigned i = base + lane;
    const bool valid = i < total;
    double vr[2] = {0.0, 0.0}, vt[2] = {0.0, 0.0}, vp[2] = {0.0, 0.0};
    double br[2] = {0.0, 0.0}, bt[2] = {0.0, 0.0}, bp[2] = {0.0, 0.0};
    double os2 = 0.0;
    if (valid) {
      const unsigned ph = i / nh, j = i - ph * nh;
      const long long o = o0 + (long long)ph * g.ld + 2 * j;
      os2 = g.osin2[j];
      const double* const src[6] = {a.vr, a.vt, a.vp, a.br, a.bt, a.bp};
      double* const dst[6] = {vr, vt, vp, br, bt, bp};
#pragma unroll
      for (int f = 0; f < (MAG ? 6 : 3); ++f) {
        if (PAIR) {
          const double2 v = __ldg(reinterpret_cast<const double2*>(src[f] + o));
          dst[f][0] = v.x; dst[f][1] = v.y;
        } else {
          dst[f][0] = __ldg(src[f] + o); dst[f][1] = __ldg(src[f] + o + 1);
        }
      }
    }
    // FP32 estimates; a pair whose 1/sin^2 exceeds 2^24 is evaluated exactly
    const float s = hi_abs_f32(os2);
    const bool s_ok = s <= 0x1p24f;
    float ar[2], ah[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      ar[k] = approx_r<MAG>(c, hi_abs_f32(vr[k]), hi_abs_f32(br[k]));
      ah[k] = approx_h<MAG>(c, hi_abs_f32(vt[k]), hi_abs_f32(vp[k]), hi_abs_f32(bt[k]), hi_abs_f32(bp[k]), s);
    }
    const unsigned wr = __reduce_max_sync(0xffffffffu, valid ? __float_as_uint(fmaxf(finite_or_zero(ar[0]),
                                                                                      finite_or_zero(ar[1]))) : 0u);
    const unsigned wh = __reduce_max_sync(0xffffffffu, valid ? __float_as_uint(fmaxf(finite_or_zero(ah[0]),
                                                                                      finite_or_zero(ah[1]))) : 0u);
    unsigned cr = *(volatile unsigned*)&m_r, ch = *(volatile unsigned*)&m_h;
    if (wr > cr) { if (lane == 0) atomicMax(&m_r, wr); cr = wr; }
    if (wh > ch) { if (lane == 0) atomicMax(&m_h, wh); ch = wh; }
    const float thr_r = kfac * __uint_as_float(cr) - tau2, thr_h = kfac * __uint_as_float(ch) - tau2;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      // !(a < thr) also holds for an infinite or NaN estimate
      if (valid && (!c.fast || !(ar[k] < thr_r))) vr2max = fmax(vr2max, exact_r<MAG>(c, vr[k], br[k]));
      if (valid && (!c.fast || !s_ok || !(ah[k] < thr_h)))
        vh2max = fmax(vh2max, exact_h<MAG>(c, vt[k], vp[k], bt[k], bp[k], os2));
    }
  }
  // maxima are >= +0, so their bit patterns order like the values
  vr2max = block_max(vr2max, red);
  vh2max = block_max(vh2max, red);
  if (threadIdx.x == 0) {
    atomicMax(&mx[2 * lev], (unsigned long long)__double_as_longlong(vr2max));
    atomicMax(&mx[2 * lev + 1], (unsigned long long)__double_as_longlong(vh2max));
  }
}

__global__ void courant_finish(const CourantArgs a, int nlev, const unsigned long long* mx, double* dtrkc,
                               double* dthkc) {
  const int lev = blockIdx.x * blockDim.x + threadIdx.x;
  if (lev >= nlev) return;
  const double vr2max = __longlong_as_double((long long)mx[2 * lev]);
  const double vh2max = __longlong_as_double((long long)mx[2 * lev + 1]);
  if (vr2max != 0.0) dtrkc[lev] = fmin(dtrkc[lev], sqrt(a.delxr2[lev] / vr2max));
  if (vh2max != 0.0) dthkc[lev] = fmin(dthkc[lev], sqrt(a.delxh2[lev] / vh2max));
}

}  // namespace

cudaError_t launch_courant(const ShtGeom& g, const CourantArgs& a, int nlev, unsigned long long* mx, double* dtrkc,
                           double* dthkc, cudaStream_t st) {
  if (nlev <= 0) return cudaSuccess;
  CUDA_TRY(cudaMemsetAsync(mx, 0, (size_t)nlev * 2 * sizeof(unsigned long long), st));
  const long long npts = (long long)g.n_phi * (g.n_theta / 2);  // pairs of rows
  int dev = 0, nsm = 1;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int gx = (4 * nsm + nlev - 1) / nlev;  // about four blocks per SM in all
  const int need = (int)((npts + kCourThreads - 1) / kCourThreads);
  if (gx > need) gx = need;
  if (gx < 1) gx = 1;
  const bool mag = a.br != nullptr;
  const bool pair = ((g.ld | a.ld) & 1) == 0 && (((uintptr_t)a.vr | (uintptr_t)a.vt | (uintptr_t)a.vp |
                                                   (uintptr_t)a.br | (uintptr_t)a.bt | (uintptr_t)a.bp) & 15) == 0;
  const dim3 grid(gx, nlev);
  if (mag && pair) courant_reduce<true, true><<<grid, kCourThreads, 0, st>>>(g, a, mx);
  else if (mag) courant_reduce<true, false><<<grid, kCourThreads, 0, st>>>(g, a, mx);
  else if (pair) courant_reduce<false, true><<<grid, kCourThreads, 0, st>>>(g, a, mx);
  else courant_reduce<false, false><<<grid, kCourThreads, 0, st>>>(g, a, mx);
  CUDA_TRY(cudaGetLastError());
  courant_finish<<<(nlev + 127) / 128, 128, 0, st>>>(a, nlev, mx, dtrkc, dthkc);
  return cudaGetLastError();
}
