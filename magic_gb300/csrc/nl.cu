// Grid-space nonlinear products of the radial loop (get_nl.f90:213-441 and
// the Lorentz-force addition of rIter.f90:650-655): the grids that
// transform_to_lm_space transforms, computed from the grids of
// transform_to_grid_space.  Boussinesq form (orho1 = 1), curl form of the
// advection (l_adv_curl), magnetic field and heat equation on, unit physical
// constants (LFfac = OhmLossFac = 1, otemp1 = lambda = 1); heatTerms holds the
// ohmic-loss part (get_nl.f90:424-429).  Elementwise: FP64 arithmetic in the
// FP64 form, FP32 arithmetic (FP64 grids in and out) in the reduced forms.
#include <algorithm>
#include "common.cuh"
#include "cplx.cuh"
#include "internal.h"

namespace {

__device__ __forceinline__ double2 ld2(const double* p, long long o) {
  return __ldg(reinterpret_cast<const double2*>(p + o));
}
__device__ __forceinline__ void st2(double* p, long long o, double a, double b) {
  *reinterpret_cast<double2*>(p + o) = make_double2(a, b);
}

// one thread per (level, phi, pair of theta rows 2j, 2j+1); rows of a pair
// share theta_j in the scrambled north/south order.  T is the arithmetic:
// double (the FP64 form), or float for the reduced forms, whose grids carry
// errors far above FP32 rounding: the FP64 grids are narrowed and the
// products widened with integer instructions (d2f_int / f2d_int), so the
// float kernel runs on the FP32 and integer pipes and is bound by HBM, while
// the FP64 one is bound by the FP64 pipe (about 40 FP64 operations a point).
template <typename T>
__global__ void __launch_bounds__(256) get_nl_kernel(const ShtGeom g, const NlGrids in, NlGrids out,
                                                     const double* __restrict__ or2, double or2_0, int r0) {
  const int r = r0 + blockIdx.y;
  const unsigned nh = (unsigned)(g.n_theta / 2), per_level = (unsigned)g.n_phi * nh;
  const double o2d = or2 ? or2[r] : or2_0;
  const T o2 = from_f64<T>(o2d), o4 = from_f64<T>(o2d * o2d);
  const long long b_in = (long long)r * in.ld, b_out = (long long)r * out.ld;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < per_level; i += gridDim.x * blockDim.x) {
    const unsigned ph = i / nh, j = i - ph * nh;
    const long long o_in = b_in + (long long)ph * g.ld + 2 * j;
    const long long o_out = b_out + (long long)ph * g.ld + 2 * j;
    const T sn2 = from_f64<T>(g.osin2[j]);  // 1 / sin^2 theta_j
    double2 x[NL_NIN];
#pragma unroll
    for (int k = 0; k < NL_NIN; ++k) x[k] = ld2(in.p[k], o_in);
    T res[NL_NOUT][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      auto v = [&](int k) { return from_f64<T>(h ? x[k].y : x[k].x); };
      const T Vr = v(NL_VR), Vt = v(NL_VT), Vp = v(NL_VP);
      const T Wr = v(NL_CVR), Wt = v(NL_CVT), Wp = v(NL_CVP);
      const T Br = v(NL_BR), Bt = v(NL_BT), Bp = v(NL_BP);
      const T Jr = v(NL_CBR), Jt = v(NL_CBT), Jp = v(NL_CBP);
      const T S = v(NL_S);
      // Lorentz force (get_nl.f90:243-256)
      const T LFr = sn2 * (Jt * Bp - Jp * Bt);
      const T LFt = o4 * (Jp * Br - Jr * Bp);
      const T LFp = o4 * (Jr * Bt - Jt * Br);
      // advection, curl form (get_nl.f90:262-272), plus the Lorentz force
      res[NL_ADVR][h] = -sn2 * (Wt * Vp - Wp * Vt) + LFr;
      res[NL_ADVT][h] = -o4 * (Wp * Vr - Wr * Vp) + LFt;
      res[NL_ADVP][h] = -o4 * (Wr * Vt - Wt * Vr) + LFp;
      // entropy advection (get_nl.f90:318-322)
      res[NL_VSR][h] = Vr * S;
      res[NL_VST][h] = o2 * Vt * S;
      res[NL_VSP][h] = o2 * Vp * S;
      // induction (get_nl.f90:377-388)
      res[NL_VXBR][h] = sn2 * (Vt * Bp - Vp * Bt);
      res[NL_VXBT][h] = o4 * (Vp * Br - Vr * Bp);
      res[NL_VXBP][h] = o4 * (Vr * Bt - Vt * Br);
      // ohmic losses (get_nl.f90:424-429)
      res[NL_HEAT][h] = o2 * (o2 * Jr * Jr + sn2 * Jt * Jt + sn2 * Jp * Jp);
    }
#pragma unroll
    for (int k = 0; k < NL_NOUT; ++k) st2(out.p[k], o_out, to_f64<T>(res[k][0]), to_f64<T>(res[k][1]));
  }
}

}  // namespace

cudaError_t launch_get_nl(const ShtGeom& g, const NlGrids& in, const NlGrids& out, const double* or2,
                          double or2_0, int nlev, bool f32, cudaStream_t st) {
  const long long per_level = (long long)g.n_phi * (g.n_theta / 2);
  if (nlev <= 0 || per_level <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int need = (int)((per_level + 255) / 256);
  for (int r0 = 0; r0 < nlev; r0 += 65535) {
    const int nl = std::min(nlev - r0, 65535);
    const int gx = std::max(1, std::min(need, (8 * nsm + nl - 1) / nl));  // about eight blocks per SM in all
    if (f32) get_nl_kernel<float><<<dim3(gx, nl), 256, 0, st>>>(g, in, out, or2, or2_0, r0);
    else get_nl_kernel<double><<<dim3(gx, nl), 256, 0, st>>>(g, in, out, or2, or2_0, r0);
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}
