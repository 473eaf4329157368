// Grid-space nonlinear products of the radial loop (get_nl.f90:213-441 and
// the Lorentz-force addition of rIter.f90:650-655): the grids that
// transform_to_lm_space transforms, computed from the grids of
// transform_to_grid_space.  Boussinesq form (orho1 = 1), curl form of the
// advection (l_adv_curl), magnetic field and heat equation on, unit physical
// constants (LFfac = OhmLossFac = 1, otemp1 = lambda = 1); heatTerms holds the
// ohmic-loss part (get_nl.f90:424-429).  Elementwise: FP64 arithmetic in the
// FP64 form, double-float arithmetic on the FP32 pipe in the FP64-accurate
// form (about 2^-48 per operation), FP32 arithmetic in the reduced forms (FP64
// grids in and out in all of them).
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
                          double or2_0, int nlev, int arith, cudaStream_t st) {
  const long long per_level = (long long)g.n_phi * (g.n_theta / 2);
  if (nlev <= 0 || per_level <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int need = (int)((per_level + 255) / 256);
  for (int r0 = 0; r0 < nlev; r0 += 65535) {
    const int nl = std::min(nlev - r0, 65535);
    const int gx = std::max(1, std::min(need, (8 * nsm + nl - 1) / nl));  // about eight blocks per SM in all
    if (arith == FFT_ARITH_F32) get_nl_kernel<float><<<dim3(gx, nl), 256, 0, st>>>(g, in, out, or2, or2_0, r0);
    else if (arith == FFT_ARITH_DF) get_nl_kernel<dfl><<<dim3(gx, nl), 256, 0, st>>>(g, in, out, or2, or2_0, r0);
    else get_nl_kernel<double><<<dim3(gx, nl), 256, 0, st>>>(g, in, out, or2, or2_0, r0);
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

// ------------------------------------------------- the general get_nl
// get_nl.f90:213-441 with the reference's switches and radial functions and
// the Lorentz-force combination of transform_to_lm_space
// (rIter.f90:645-662).  Per level: the Lorentz force where l_mag_LF, nBc = 0
// and outside the low-conductivity region; the advection in the curl form
// (:260-272) or as u.grad u (:274-302) where l_conv_nl and nBc = 0; V S, V Xi
// where nBc = 0; V x B in its bulk, stress-free (nBc = 1 or inside the
// region) or rigid (nBc = 2) form; heatTerms (viscous heating and ohmic
// losses, :398-432) where l_anel and nBc = 0.  Outputs a level does not
// produce are left untouched, as the reference leaves them.
namespace {

template <typename T>
__global__ void __launch_bounds__(256) get_nl_full_kernel(const ShtGeom g, const NlFull a, const double* __restrict__ cosn2,
                                                          int r0) {
  const int r = r0 + blockIdx.y;
  const unsigned nh = (unsigned)(g.n_theta / 2), per_level = (unsigned)g.n_phi * nh;
  const NlOpts& o = a.o;
  const int nbc = o.nbc ? o.nbc[r] : 0;
  const bool bulk = nbc == 0, lcr = o.lcr && o.lcr[r] != 0;
  const double rd = o.r[r], o1d = 1.0 / rd, o2d = o1d * o1d;
  const T rr = from_f64<T>(rd), o1 = from_f64<T>(o1d), o2 = from_f64<T>(o2d), o4 = from_f64<T>(o2d * o2d);
  const T oh = from_f64<T>(o.orho1 ? o.orho1[r] : 1.0), bt = from_f64<T>(o.beta ? o.beta[r] : 0.0);
  const T ot = from_f64<T>(o.otemp1 ? o.otemp1[r] : 1.0), vi = from_f64<T>(o.visc ? o.visc[r] : 1.0);
  const T la = from_f64<T>(o.lambda ? o.lambda[r] : 1.0);
  const T LFfac = from_f64<T>(o.LFfac), VHF = from_f64<T>(o.ViscHeatFac), OLF = from_f64<T>(o.OhmLossFac);
  const bool do_lf = o.lf && bulk && !lcr;
  const bool do_adv = bulk && (o.conv || o.lf);
  const bool do_vs = o.heat && bulk, do_vxi = o.chem && bulk, do_heat = o.anel && bulk;
  const int vxb = !o.mag ? 0 : (bulk && !lcr) ? 1 : (nbc == 1 || lcr) ? 2 : (nbc == 2) ? 3 : 0;
  const T two = (T)2, third = (T)(1.0 / 3.0);
  const long long b_in = (long long)r * a.ld_in, b_out = (long long)r * a.ld_out;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < per_level; i += gridDim.x * blockDim.x) {
    const unsigned ph = i / nh, j = i - ph * nh;
    const long long oi = b_in + (long long)ph * g.ld + 2 * j;
    const long long oo = b_out + (long long)ph * g.ld + 2 * j;
    const T sn2 = from_f64<T>(g.osin2[j]);
    const T cn2n = from_f64<T>(cosn2[j]);  // cos/sin^2 of the northern row; the southern row has -cos
    auto ld = [&](int k) { return __ldg(reinterpret_cast<const double2*>(a.in[k] + oi)); };
    double2 x[NLF_NIN];
#pragma unroll
    for (int k = 0; k < NLF_NIN; ++k) x[k] = a.in[k] ? ld(k) : make_double2(0.0, 0.0);
    T res[NLF_NOUT][2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      auto v = [&](int k) { return from_f64<T>(h ? x[k].y : x[k].x); };
      const T cn2 = h ? -cn2n : cn2n;
      const T vr = v(NLF_VR), vt = v(NLF_VT), vp = v(NLF_VP);
      const T br = v(NLF_BR), btt = v(NLF_BT), bp = v(NLF_BP);
      const T jr = v(NLF_CBR), jt = v(NLF_CBT), jp = v(NLF_CBP);
      T ar = 0, at = 0, ap = 0;
      if (o.conv) {
        if (o.curl) {
          const T wr = v(NLF_CVR), wt = v(NLF_CVT), wp = v(NLF_CVP);
          ar = -sn2 * (wt * vp - wp * vt);
          at = -o4 * (wp * vr - wr * vp);
          ap = -o4 * (wr * vt - wt * vr);
        } else {
          const T drr = v(NLF_DVRDR), dtr = v(NLF_DVTDR), dpr = v(NLF_DVPDR);
          const T drt = v(NLF_DVRDT), drp = v(NLF_DVRDP), dtp = v(NLF_DVTDP), dpp = v(NLF_DVPDP);
          const T wr = v(NLF_CVR);
          ar = -o2 * oh * (vr * (drr - (two * o1 + bt) * vr) + sn2 * (vt * (drt - rr * vt) + vp * (drp - rr * vp)));
          at = o4 * oh * (-vr * (dtr - bt * vt) + vt * (cn2 * vt + dpp + drr) + vp * (cn2 * vp - dtp));
          ap = o4 * oh * (-vr * (dpr - bt * vp) - vt * (dtp + wr) - vp * dpp);
        }
      }
      if (do_lf) {
        ar += LFfac * sn2 * (jt * bp - jp * btt);
        at += LFfac * o4 * (jp * br - jr * bp);
        ap += LFfac * o4 * (jr * btt - jt * br);
      }
      res[NLF_ADVR][h] = ar;
      res[NLF_ADVT][h] = at;
      res[NLF_ADVP][h] = ap;
      const T s = v(NLF_S), xi = v(NLF_XI);
      res[NLF_VSR][h] = vr * s;
      res[NLF_VST][h] = o2 * vt * s;
      res[NLF_VSP][h] = o2 * vp * s;
      res[NLF_VXIR][h] = vr * xi;
      res[NLF_VXIT][h] = o2 * vt * xi;
      res[NLF_VXIP][h] = o2 * vp * xi;
      if (vxb == 1) {
        res[NLF_VXBR][h] = oh * sn2 * (vt * bp - vp * btt);
        res[NLF_VXBT][h] = oh * o4 * (vp * br - vr * bp);
        res[NLF_VXBP][h] = oh * o4 * (vr * btt - vt * br);
      } else {
        res[NLF_VXBR][h] = 0;
        res[NLF_VXBT][h] = o4 * oh * vp * br;
        res[NLF_VXBP][h] = vxb == 2 ? -o4 * oh * vt * br : (T)0;
      }
      T heat = 0;
      if (do_heat) {
        const T drr = v(NLF_DVRDR), dtr = v(NLF_DVTDR), dpr = v(NLF_DVPDR);
        const T drt = v(NLF_DVRDT), drp = v(NLF_DVRDP), dtp = v(NLF_DVTDP), dpp = v(NLF_DVPDP);
        const T wr = v(NLF_CVR);
        const T e1 = drr - (two * o1 + bt) * vr;
        const T e2 = cn2 * vt + dpp + drr - o1 * vr;
        const T e3 = dpp + cn2 * vt + o1 * vr;
        const T e6 = two * dtp + wr - two * cn2 * vp;
        const T e4 = rr * dtr - (two + bt * rr) * vt + o1 * drt;
        const T e5 = rr * dpr - (two + bt * rr) * vp + o1 * drp;
        heat = VHF * o4 * oh * ot * vi *
               (two * e1 * e1 + two * e2 * e2 + two * e3 * e3 + e6 * e6 + sn2 * (e4 * e4 + e5 * e5) -
                two * third * (bt * vr) * (bt * vr));
        if (o.mag && !lcr) heat += OLF * o2 * ot * la * (o2 * jr * jr + sn2 * jt * jt + sn2 * jp * jp);
      }
      res[NLF_HEAT][h] = heat;
    }
    auto st = [&](int k) {
      *reinterpret_cast<double2*>(a.out[k] + oo) = make_double2(to_f64<T>(res[k][0]), to_f64<T>(res[k][1]));
    };
    if (do_adv && a.out[NLF_ADVR]) { st(NLF_ADVR); st(NLF_ADVT); st(NLF_ADVP); }
    if (do_vs && a.out[NLF_VSR]) { st(NLF_VSR); st(NLF_VST); st(NLF_VSP); }
    if (do_vxi && a.out[NLF_VXIR]) { st(NLF_VXIR); st(NLF_VXIT); st(NLF_VXIP); }
    if (vxb == 1 && a.out[NLF_VXBR]) st(NLF_VXBR);
    if (vxb && a.out[NLF_VXBT]) { st(NLF_VXBT); st(NLF_VXBP); }
    if (do_heat && a.out[NLF_HEAT]) st(NLF_HEAT);
  }
}

__global__ void cosn2_kernel(int nh, const double* __restrict__ theta, double* __restrict__ cosn2) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nh) {
    const double s = sin(theta[j]);
    cosn2[j] = cos(theta[j]) / s / s;  // horizontal.f90:156
  }
}

}  // namespace

cudaError_t build_cosn2(const ShtGeom& g, const double* theta, double* cosn2, cudaStream_t st) {
  const int nh = g.n_theta / 2;
  cosn2_kernel<<<(nh + 127) / 128, 128, 0, st>>>(nh, theta, cosn2);
  return cudaGetLastError();
}

cudaError_t launch_get_nl_full(const ShtGeom& g, const NlFull& a, const double* cosn2, int nlev, int arith,
                               cudaStream_t st) {
  const long long per_level = (long long)g.n_phi * (g.n_theta / 2);
  if (nlev <= 0 || per_level <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int need = (int)((per_level + 255) / 256);
  for (int r0 = 0; r0 < nlev; r0 += 65535) {
    const int nl = std::min(nlev - r0, 65535);
    const int gx = std::max(1, std::min(need, (8 * nsm + nl - 1) / nl));
    if (arith == FFT_ARITH_F32) get_nl_full_kernel<float><<<dim3(gx, nl), 256, 0, st>>>(g, a, cosn2, r0);
    else if (arith == FFT_ARITH_DF) get_nl_full_kernel<dfl><<<dim3(gx, nl), 256, 0, st>>>(g, a, cosn2, r0);
    else get_nl_full_kernel<double><<<dim3(gx, nl), 256, 0, st>>>(g, a, cosn2, r0);
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}
