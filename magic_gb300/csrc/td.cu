// Spectral assembly of the explicit time derivatives at the radial levels
// (get_td.f90:133-208 get_dwdt, :311-379 get_dpdt, :381-457 get_dzdt,
// :459-521 get_dsdt, :558-619 get_dbdt) from the analysis outputs of the
// radial loop: Boussinesq form, Coriolis force on, magnetic field and heat
// equation on, no double-curl form.  At a boundary level (nbc != 0) only
// dVxBhLM is written; the other outputs are left as they are, as the
// reference leaves them.  One thread per (level, lm); the l-1 and l+1
// neighbours of lm in the m-major order are lm-1 and lm+1.  The per-lm
// coefficients are tabulated once per handle (td_coef_kernel), so the
// kernel spends its FP64 operations on the assembly alone.
// Operator coefficients as in horizontal.f90:204-229:
//   clm(l,m) = sqrt((l+m)(l-m) / ((2l-1)(2l+1))), dLh = l(l+1), dPhi = i m,
//   dTheta2S = (l-1) clm(l,m),  dTheta2A = (l+2) clm(l+1,m),
//   dTheta3S = (l-1)(l+1) clm(l,m),  dTheta3A = l(l+2) clm(l+1,m),
//   dTheta4S = (l+1) clm(l,m) (l-1) l,  dTheta4A = l clm(l+1,m) (l+1)(l+2).
#include <algorithm>
#include "common.cuh"
#include "cplx.cuh"
#include "internal.h"

namespace {

__device__ __forceinline__ double clm(int l, int m) {
  return sqrt((double)((l + m) * (l - m)) / (double)((2 * l - 1) * (2 * l + 1)));
}

// Level-independent coefficients of each lm, four double2 per lm:
//   {t2A, t2S}, {t3A, t3S}, {t4A, t4S}, {dLh, m}
// with t2A = (l+2) clm(l+1,m), t2S = (l-1) clm(l,m), t3A = l(l+2) clm(l+1,m),
// t3S = (l-1)(l+1) clm(l,m), t4A = l clm(l+1,m) (l+1)(l+2), t4S = (l+1) clm(l,m) (l-1) l,
// and lq[lm] = l | m << 16.
__global__ void td_coef_kernel(const ShtGeom g, double2* coef, int* lq) {
  const int lm = blockIdx.x * blockDim.x + threadIdx.x;
  if (lm >= g.lm_max) return;
  int lo = 0, hi = g.n_m - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.lmoff[mid] <= lm) lo = mid;
    else hi = mid - 1;
  }
  const int m = lo * g.minc, l = m + (lm - g.lmoff[lo]);
  const double cS = l > m ? clm(l, m) : 0.0, cA = clm(l + 1, m);
  coef[4 * lm + 0] = make_double2((l + 2) * cA, (l - 1) * cS);
  coef[4 * lm + 1] = make_double2((double)l * (l + 2) * cA, (double)(l - 1) * (l + 1) * cS);
  coef[4 * lm + 2] = make_double2((double)l * cA * (double)(l + 1) * (l + 2), (double)(l + 1) * cS * (double)(l - 1) * l);
  coef[4 * lm + 3] = make_double2((double)l * (l + 1), (double)m);
  lq[lm] = l | (m << 16);
}

// One block row (blockIdx.y) per radial level, threads over lm; the
// coefficients come from the tables of td_coef_kernel (L2-resident).  T is
// the arithmetic: double in the FP64 form (about 60 FP64 operations per lm,
// which bound the kernel by the FP64 pipe), float in the reduced forms, whose
// spectra carry errors far above FP32 rounding (FP64 spectra narrowed and the
// results widened with integer instructions; bound by HBM).
template <typename T>
__global__ void __launch_bounds__(256) get_td_kernel(const ShtGeom g, const TdArgs a, int r0) {
  typedef typename V2<T>::t T2;
  const int r = r0 + blockIdx.y;
  const double rrd = a.r[r], or1d = 1.0 / rrd, or2d = or1d * or1d;
  const T rr = from_f64<T>(rrd), or1 = from_f64<T>(or1d), or2 = from_f64<T>(or2d), or4 = from_f64<T>(or2d * or2d);
  const int lR = a.lcut ? min(a.lcut[r], g.l_max) : g.l_max;
  const bool boundary = a.nbc && a.nbc[r] != 0;
  const T two_cor = from_f64<T>(2.0 * a.cor_fac);
  const T2 zero = zero2<T2>();
  const long long o0 = (long long)r * a.ld;
  auto ld = [&](const double2* p, long long o) { return cvt2<T2>(p[o]); };
  for (int lm = blockIdx.x * blockDim.x + threadIdx.x; lm < g.lm_max; lm += gridDim.x * blockDim.x) {
    const long long o = o0 + lm;
    const double2 c3 = a.coef[4 * lm + 3];
    const T dLh = from_f64<T>(c3.x), dm = from_f64<T>(c3.y);
    if (boundary) {  // boundary level: only get_dbdt's dVxBhLM (get_td.f90:598-612)
      a.dVxBh[o] = to_d2(cscale(ld(a.VxBt, o), -dLh * rr * rr));
      continue;
    }
    const int q = a.lq[lm], l = q & 0xFFFF, m = q >> 16;
    const bool hasS = l > m, hasA = l < lR;  // l-1 and l+1 terms (clm(m,m) = 0; l = l_R drops l+1)
    const double2 c0 = a.coef[4 * lm + 0], c1 = a.coef[4 * lm + 1];
    const T2 w = ld(a.w, o), dw = ld(a.dw, o), z = ld(a.z, o);
    const T2 zS = hasS ? ld(a.z, o - 1) : zero, zA = hasA ? ld(a.z, o + 1) : zero;
    const T2 dwS = hasS ? ld(a.dw, o - 1) : zero, dwA = hasA ? ld(a.dw, o + 1) : zero;
    const T2 wS = hasS ? ld(a.w, o - 1) : zero, wA = hasA ? ld(a.w, o + 1) : zero;
    const bool inside = l <= lR;
    // dPhi * x = i m x
    auto iphi = [&](T2 x) { return mk2(-dm * x.y, dm * x.x); };
    // ---- get_dwdt: or2 AdvrLM + 2 CorFac or1 (dPhi dw + dTheta2A z(l+1) - dTheta2S z(l-1))
    T2 dwdt = cscale(ld(a.Advr, o), or2);
    if (inside) {
      const T t2A = from_f64<T>(c0.x), t2S = from_f64<T>(c0.y);
      const T2 p = iphi(dw);
      const T2 c = mk2(p.x + t2A * zA.x - t2S * zS.x, p.y + t2A * zA.y - t2S * zS.y);
      if (l > 0) dwdt = cadd(dwdt, cscale(c, two_cor * or1));
      else dwdt = cadd(dwdt, cscale(mk2(t2A * zA.x, t2A * zA.y), two_cor * or1));  // lm = 1
    }
    // ---- get_dzdt: dLh AdvpLM + 2 CorFac or2 (dPhi z + dTheta3A dw(l+1) + or1 dTheta4A w(l+1)
    //                                           + dTheta3S dw(l-1) - or1 dTheta4S w(l-1))
    T2 dzdt = l > 0 ? cscale(ld(a.Advp, o), dLh) : zero;
    const T t3A = from_f64<T>(c1.x), t3S = from_f64<T>(c1.y);
    if (inside) {
      const double2 c2 = a.coef[4 * lm + 2];
      const T t4A = from_f64<T>(c2.x), t4S = from_f64<T>(c2.y);
      T2 c = mk2(t3A * dwA.x + or1 * t4A * wA.x + t3S * dwS.x - or1 * t4S * wS.x,
                 t3A * dwA.y + or1 * t4A * wA.y + t3S * dwS.y - or1 * t4S * wS.y);
      if (l > 0) c = cadd(c, iphi(z));
      dzdt = cadd(dzdt, cscale(c, two_cor * or2));
    }
    // ---- get_dpdt: -dLh AdvtLM + 2 CorFac or2 (-dPhi (dw + or1 dLh w) + dTheta3A z(l+1) + dTheta3S z(l-1))
    T2 dpdt = zero;
    if (l > 0) {
      dpdt = cscale(ld(a.Advt, o), -dLh);
      if (inside) {
        const T2 qq = iphi(mk2(dw.x + or1 * dLh * w.x, dw.y + or1 * dLh * w.y));
        const T2 c = mk2(-qq.x + t3A * zA.x + t3S * zS.x, -qq.y + t3A * zA.y + t3S * zS.y);
        dpdt = cadd(dpdt, cscale(c, two_cor * or2));
      }
    }
    // ---- get_dsdt (Boussinesq): dLh VStLM; l = 0: the internal heating epsc
    const double2 dsdt = l > 0 ? to_d2(cscale(ld(a.VSt, o), dLh)) : make_double2(a.epsc ? a.epsc[r] : 0.0, 0.0);
    // ---- get_dbdt
    const T2 dbdt = cscale(ld(a.VxBp, o), dLh);
    const T2 dVxBh = cscale(ld(a.VxBt, o), -dLh * rr * rr);
    const T2 djdt = cscale(ld(a.VxBr, o), dLh * or4);
    a.dwdt[o] = to_d2(dwdt);
    a.dzdt[o] = to_d2(dzdt);
    a.dpdt[o] = to_d2(dpdt);
    a.dsdt[o] = dsdt;
    a.dbdt[o] = to_d2(dbdt);
    a.djdt[o] = to_d2(djdt);
    a.dVxBh[o] = to_d2(dVxBh);
  }
}

}  // namespace

cudaError_t build_td_coef(const ShtGeom& g, double2* coef, int* lq, cudaStream_t st) {
  if (g.lm_max <= 0) return cudaSuccess;
  td_coef_kernel<<<(g.lm_max + 255) / 256, 256, 0, st>>>(g, coef, lq);
  return cudaGetLastError();
}

cudaError_t launch_get_td(const ShtGeom& g, const TdArgs& a, int nlev, int arith, cudaStream_t st) {
  if (nlev <= 0 || g.lm_max <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int need = (g.lm_max + 255) / 256;
  for (int r0 = 0; r0 < nlev; r0 += 65535) {
    const int nl = std::min(nlev - r0, 65535);
    const int gx = std::max(1, std::min(need, (8 * nsm + nl - 1) / nl));  // about eight blocks per SM in all
    // FP64 also for the FP64-accurate form: in double-float arithmetic this
    // kernel measured slower (0.56 against 0.47 ms at 129 levels)
    if (arith == FFT_ARITH_F32) get_td_kernel<float><<<dim3(gx, nl), 256, 0, st>>>(g, a, r0);
    else get_td_kernel<double><<<dim3(gx, nl), 256, 0, st>>>(g, a, r0);
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

// ------------------------------------------------- the general get_td
// get_td.f90 with the reference's switches, as the radial loop calls it
// (rIter.f90:410-428): get_dzdt, get_dwdt or get_dwdt_double_curl (with
// dVxVhLM), get_dpdt, get_dsdt (anelastic heatTermsLM, temp0 of the
// anelastic-liquid form), get_dxidt, get_dbdt (zeros without l_mag_nl).  An
// output is computed when its pointer is non-null (its equation is on); at
// a boundary level only dVxBhLM, dVxVhLM (double curl), dVSrLM and dVXirLM
// are written (get_td.f90:298-306, :512-519, :548-554, :598-612).  Entries
// the reference does not set (dpdt and dVxVhLM at l = 0) are left untouched.
namespace {

template <typename T>
__global__ void __launch_bounds__(256) get_td_full_kernel(const ShtGeom g, const TdFull a, int r0) {
  typedef typename V2<T>::t T2;
  const int r = r0 + blockIdx.y;
  const TdOpts& o = a.o;
  const double rrd = o.r[r], or1d = 1.0 / rrd, or2d = or1d * or1d;
  const T rr = from_f64<T>(rrd), or1 = from_f64<T>(or1d), or2 = from_f64<T>(or2d), or4 = from_f64<T>(or2d * or2d);
  const T oh = from_f64<T>(o.orho1 ? o.orho1[r] : 1.0), be = from_f64<T>(o.beta ? o.beta[r] : 0.0);
  const T t0 = from_f64<T>((o.anel && o.liquid && o.temp0) ? o.temp0[r] : 1.0);
  const int lR = o.lcut ? min(o.lcut[r], g.l_max) : g.l_max;
  const bool bulk = !(o.nbc && o.nbc[r] != 0);
  const T two_cor = from_f64<T>(2.0 * o.cor_fac);
  const T2 zero = zero2<T2>();
  const long long o0 = (long long)r * a.ld;
  auto ld = [&](const double2* p, long long oo) { return cvt2<T2>(p[oo]); };
  auto iphi = [&](T2 x, T dm) { return mk2(-dm * x.y, dm * x.x); };
  for (int lm = blockIdx.x * blockDim.x + threadIdx.x; lm < g.lm_max; lm += gridDim.x * blockDim.x) {
    const long long oo = o0 + lm;
    const double2 c3 = a.coef[4 * lm + 3];
    const T dLh = from_f64<T>(c3.x), dm = from_f64<T>(c3.y);
    if (!bulk) {
      if (o.dcurl && a.dVxVh) a.dVxVh[oo] = make_double2(0.0, 0.0);
      if (a.dsdt && a.dVSr) a.dVSr[oo] = make_double2(0.0, 0.0);
      if (a.dxidt && a.dVXir) a.dVXir[oo] = make_double2(0.0, 0.0);
      if (a.dVxBh) a.dVxBh[oo] = (o.mag_nl && lm > 0) ? to_d2(cscale(ld(a.VxBt, oo), -dLh * rr * rr)) : make_double2(0.0, 0.0);
      continue;
    }
    const int q = a.lq[lm], l = q & 0xFFFF, m = q >> 16;
    const bool hasS = l > m, hasA = l < lR;
    const bool inside = l <= lR;
    const double2 c0 = a.coef[4 * lm + 0], c1 = a.coef[4 * lm + 1], c2 = a.coef[4 * lm + 2];
    const T t2A = from_f64<T>(c0.x), t2S = from_f64<T>(c0.y), t3A = from_f64<T>(c1.x), t3S = from_f64<T>(c1.y);
    const T t4A = from_f64<T>(c2.x), t4S = from_f64<T>(c2.y);
    const bool need_vel = o.corr && (a.dwdt || a.dzdt || a.dpdt);
    T2 w = zero, dw = zero, z = zero, zS = zero, zA = zero, dwS = zero, dwA = zero, wS = zero, wA = zero;
    if (need_vel) {
      w = ld(a.w, oo); dw = ld(a.dw, oo); z = ld(a.z, oo);
      if (hasS) { zS = ld(a.z, oo - 1); dwS = ld(a.dw, oo - 1); wS = ld(a.w, oo - 1); }
      if (hasA) { zA = ld(a.z, oo + 1); dwA = ld(a.dw, oo + 1); wA = ld(a.w, oo + 1); }
    }
    // ---- get_dzdt (get_td.f90:381-457)
    if (a.dzdt) {
      T2 d = (o.conv && l > 0) ? cscale(ld(a.Advp, oo), dLh) : zero;
      if (o.corr && inside) {
        T2 c = mk2(t3A * dwA.x + or1 * t4A * wA.x + t3S * dwS.x - or1 * t4S * wS.x,
                   t3A * dwA.y + or1 * t4A * wA.y + t3S * dwS.y - or1 * t4S * wS.y);
        if (l > 0) c = cadd(c, iphi(z, dm));
        d = cadd(d, cscale(c, two_cor * or2));
      }
      a.dzdt[oo] = to_d2(d);
    }
    // ---- get_dwdt (:133-208) / get_dwdt_double_curl (:210-309)
    if (a.dwdt) {
      T2 d;
      if (l == 0) {  // lm = 1
        d = o.conv ? cscale(ld(a.Advr, oo), or2) : zero;
        if (o.corr && !o.single_matrix) d = cadd(d, cscale(zA, t2A * two_cor * or1));
      } else if (!o.dcurl) {
        d = o.conv ? cscale(ld(a.Advr, oo), or2) : zero;
        if (o.corr && inside) {
          const T2 p = iphi(dw, dm);
          const T2 c = mk2(p.x + t2A * zA.x - t2S * zS.x, p.y + t2A * zA.y - t2S * zS.y);
          d = cadd(d, cscale(c, two_cor * or1));
        }
      } else {
        d = o.conv ? cscale(ld(a.Advr, oo), dLh * or4 * oh) : zero;
        if (a.dVxVh) a.dVxVh[oo] = o.conv ? to_d2(cscale(ld(a.Advt, oo), -oh * rr * rr * dLh)) : make_double2(0.0, 0.0);
        if (o.corr && inside) {
          const T2 ddw = ld(a.ddw, oo);
          const T2 dzS = hasS ? ld(a.dz, oo - 1) : zero, dzA = hasA ? ld(a.dz, oo + 1) : zero;
          const T k = be * or1 + or2;
          const T2 p = iphi(mk2(-ddw.x + be * dw.x + k * dLh * w.x, -ddw.y + be * dw.y + k * dLh * w.y), dm);
          const T2 c = mk2(p.x + t3A * (dzA.x - be * zA.x) + t3S * (dzS.x - be * zS.x) + or1 * (t4A * zA.x - t4S * zS.x),
                           p.y + t3A * (dzA.y - be * zA.y) + t3S * (dzS.y - be * zS.y) + or1 * (t4A * zA.y - t4S * zS.y));
          d = cadd(d, cscale(c, two_cor * or2 * oh));
        }
      }
      a.dwdt[oo] = to_d2(d);
    }
    // ---- get_dpdt (:311-379); lm = 1 is left as it is
    if (a.dpdt && l > 0) {
      T2 d = o.conv ? cscale(ld(a.Advt, oo), -dLh) : zero;
      if (o.corr && inside) {
        const T2 qq = iphi(mk2(dw.x + or1 * dLh * w.x, dw.y + or1 * dLh * w.y), dm);
        const T2 c = mk2(-qq.x + t3A * zA.x + t3S * zS.x, -qq.y + t3A * zA.y + t3S * zS.y);
        d = cadd(d, cscale(c, two_cor * or2));
      }
      a.dpdt[oo] = to_d2(d);
    }
    // ---- get_dsdt (:459-521)
    if (a.dsdt) {
      T2 d = l > 0 ? cscale(ld(a.VSt, oo), dLh) : mk2(from_f64<T>(o.epsc ? o.epsc[r] : 0.0), (T)0);
      if (o.anel) d = cadd(d, cscale(ld(a.heat, oo), t0));
      a.dsdt[oo] = to_d2(d);
    }
    // ---- get_dxidt (:523-556)
    if (a.dxidt) a.dxidt[oo] = l > 0 ? to_d2(cscale(ld(a.VXit, oo), dLh)) : make_double2(o.epscXi, 0.0);
    // ---- get_dbdt (:558-619)
    if (o.mag_nl) {
      if (a.dbdt) a.dbdt[oo] = to_d2(cscale(ld(a.VxBp, oo), dLh));
      if (a.dVxBh) a.dVxBh[oo] = to_d2(cscale(ld(a.VxBt, oo), -dLh * rr * rr));
      if (a.djdt) a.djdt[oo] = to_d2(cscale(ld(a.VxBr, oo), dLh * or4));
    } else {
      if (a.dbdt) a.dbdt[oo] = make_double2(0.0, 0.0);
      if (a.dVxBh) a.dVxBh[oo] = make_double2(0.0, 0.0);
      if (a.djdt) a.djdt[oo] = make_double2(0.0, 0.0);
    }
  }
}

}  // namespace

cudaError_t launch_get_td_full(const ShtGeom& g, const TdFull& a, int nlev, int arith, cudaStream_t st) {
  if (nlev <= 0 || g.lm_max <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int need = (g.lm_max + 255) / 256;
  for (int r0 = 0; r0 < nlev; r0 += 65535) {
    const int nl = std::min(nlev - r0, 65535);
    const int gx = std::max(1, std::min(need, (8 * nsm + nl - 1) / nl));
    if (arith == FFT_ARITH_F32) get_td_full_kernel<float><<<dim3(gx, nl), 256, 0, st>>>(g, a, r0);
    else get_td_full_kernel<double><<<dim3(gx, nl), 256, 0, st>>>(g, a, r0);  // as launch_get_td
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}
