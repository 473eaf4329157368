// Grid-space nonlinear products of the radial loop (get_nl.f90:213-441 and
// the Lorentz-force addition of rIter.f90:650-655): the grids that
// transform_to_lm_space transforms, computed from the grids of
// transform_to_grid_space.  Boussinesq form (orho1 = 1), curl form of the
// advection (l_adv_curl), magnetic field and heat equation on, unit physical
// constants (LFfac = OhmLossFac = 1, otemp1 = lambda = 1); heatTerms holds the
// ohmic-loss part (get_nl.f90:424-429).  Elementwise, FP64, HBM-bound.
#include <algorithm>
#include "common.cuh"
#include "internal.h"

namespace {

__device__ __forceinline__ double2 ld2(const double* p, long long o) {
  return __ldg(reinterpret_cast<const double2*>(p + o));
}
__device__ __forceinline__ void st2(double* p, long long o, double a, double b) {
  *reinterpret_cast<double2*>(p + o) = make_double2(a, b);
}

// one thread per (level, phi, pair of theta rows 2j, 2j+1); rows of a pair
// share theta_j in the scrambled north/south order
__global__ void __launch_bounds__(256) get_nl_kernel(const ShtGeom g, const NlGrids in, NlGrids out,
                                                     const double* __restrict__ or2, double or2_0, int nlev) {
  const int nh = g.n_theta / 2;
  const long long per_level = (long long)g.n_phi * nh;
  const long long total = per_level * nlev;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / per_level);
    const long long rem = i - (long long)r * per_level;
    const int ph = (int)(rem / nh), j = (int)(rem - (long long)ph * nh);
    const long long o_in = (long long)r * in.ld + (long long)ph * g.ld + 2 * j;
    const long long o_out = (long long)r * out.ld + (long long)ph * g.ld + 2 * j;
    const double o2 = or2 ? or2[r] : or2_0, o4 = o2 * o2;
    const double sn2 = g.osin2[j];  // 1 / sin^2 theta_j
    const double2 vr = ld2(in.p[NL_VR], o_in), vt = ld2(in.p[NL_VT], o_in), vp = ld2(in.p[NL_VP], o_in);
    const double2 cvr = ld2(in.p[NL_CVR], o_in), cvt = ld2(in.p[NL_CVT], o_in), cvp = ld2(in.p[NL_CVP], o_in);
    const double2 br = ld2(in.p[NL_BR], o_in), bt = ld2(in.p[NL_BT], o_in), bp = ld2(in.p[NL_BP], o_in);
    const double2 cbr = ld2(in.p[NL_CBR], o_in), cbt = ld2(in.p[NL_CBT], o_in), cbp = ld2(in.p[NL_CBP], o_in);
    const double2 sc = ld2(in.p[NL_S], o_in);
    double res[NL_NOUT][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const double Vr = h ? vr.y : vr.x, Vt = h ? vt.y : vt.x, Vp = h ? vp.y : vp.x;
      const double Wr = h ? cvr.y : cvr.x, Wt = h ? cvt.y : cvt.x, Wp = h ? cvp.y : cvp.x;
      const double Br = h ? br.y : br.x, Bt = h ? bt.y : bt.x, Bp = h ? bp.y : bp.x;
      const double Jr = h ? cbr.y : cbr.x, Jt = h ? cbt.y : cbt.x, Jp = h ? cbp.y : cbp.x;
      const double S = h ? sc.y : sc.x;
      // Lorentz force (get_nl.f90:243-256)
      const double LFr = sn2 * (Jt * Bp - Jp * Bt);
      const double LFt = o4 * (Jp * Br - Jr * Bp);
      const double LFp = o4 * (Jr * Bt - Jt * Br);
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
    for (int k = 0; k < NL_NOUT; ++k) st2(out.p[k], o_out, res[k][0], res[k][1]);
  }
}

}  // namespace

cudaError_t launch_get_nl(const ShtGeom& g, const NlGrids& in, const NlGrids& out, const double* or2,
                          double or2_0, int nlev, cudaStream_t st) {
  const long long total = (long long)nlev * g.n_phi * (g.n_theta / 2);
  if (total <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = std::min<long long>((total + 255) / 256, (long long)nsm * 8);
  get_nl_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, in, out, or2, or2_0, nlev);
  return cudaGetLastError();
}
