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

__global__ void __launch_bounds__(kCourThreads) courant_reduce(const ShtGeom g, const CourantArgs a,
                                                               unsigned long long* mx) {
  __shared__ double red[kCourThreads / 32];
  const int lev = blockIdx.y;
  const long long o0 = (long long)lev * a.ld;
  const double orho1 = a.orho1[lev], orho2 = a.orho2[lev], o2 = a.or2[lev], o4 = a.or4[lev];
  const double cf2 = mul(a.courfac, a.courfac), af2 = mul(a.alffac, a.alffac);
  double valri2 = 0.0, valhi2 = 0.0;
  if (a.alf_damp) {
    const double h = mul(0.5, add(1.0, a.opm));
    valri2 = mul(h, h) / a.delxr2[lev];
    valhi2 = mul(h, h) / a.delxh2[lev];
  }
  const bool mag = a.br != nullptr;
  double vr2max = 0.0, vh2max = 0.0;
  const long long npts = (long long)g.n_phi * g.n_theta;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts;
       p += (long long)gridDim.x * blockDim.x) {
    const int ph = (int)(p / g.n_theta), th = (int)(p - (long long)ph * g.n_theta);
    const long long o = o0 + (long long)ph * g.ld + th;
    const double os2 = g.osin2[th >> 1];  // scrambled rows 2j, 2j+1 share theta_j
    const double vr = a.vr[o], vt = a.vt[o], vp = a.vp[o];
    const double vflr2 = mul(mul(orho2, vr), vr);
    const double vflh2 = mul(mul(add(mul(vt, vt), mul(vp, vp)), os2), orho2);
    if (mag) {
      const double br = a.br[o], bt = a.bt[o], bp = a.bp[o];
      const double valr = mul(mul(mul(br, br), a.LFfac), orho1);
      const double valr2 = mul(valr, valr) / add(valr, valri2);
      vr2max = fmax(vr2max, mul(o4, add(mul(cf2, vflr2), mul(af2, valr2))));
      const double valh2 = mul(mul(mul(add(mul(bt, bt), mul(bp, bp)), a.LFfac), os2), orho1);
      const double valh2m = mul(valh2, valh2) / add(valh2, valhi2);
      vh2max = fmax(vh2max, mul(o2, add(mul(cf2, vflh2), mul(af2, valh2m))));
    } else {
      vr2max = fmax(vr2max, mul(mul(cf2, o4), vflr2));
      vh2max = fmax(vh2max, mul(mul(cf2, o2), vflh2));
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
  const long long npts = (long long)g.n_phi * g.n_theta;
  int dev = 0, nsm = 1;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int gx = (4 * nsm + nlev - 1) / nlev;  // about four blocks per SM in all
  const int need = (int)((npts + kCourThreads - 1) / kCourThreads);
  if (gx > need) gx = need;
  if (gx < 1) gx = 1;
  courant_reduce<<<dim3(gx, nlev), kCourThreads, 0, st>>>(g, a, mx);
  CUDA_TRY(cudaGetLastError());
  courant_finish<<<(nlev + 127) / 128, 128, 0, st>>>(a, nlev, mx, dtrkc, dthkc);
  return cudaGetLastError();
}
