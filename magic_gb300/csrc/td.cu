// Spectral assembly of the explicit time derivatives at the radial levels
// (get_td.f90:133-208 get_dwdt, :311-379 get_dpdt, :381-457 get_dzdt,
// :459-521 get_dsdt, :558-619 get_dbdt) from the analysis outputs of the
// radial loop: Boussinesq form, Coriolis force on, magnetic field and heat
// equation on, no double-curl form.  At a boundary level (nbc != 0) only
// dVxBhLM is written; the other outputs are left as they are, as the
// reference leaves them.  One thread per (level, lm); the l-1 and l+1
// neighbours of lm in the m-major order are lm-1 and lm+1.
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

__global__ void __launch_bounds__(256) get_td_kernel(const ShtGeom g, const TdArgs a, int nlev) {
  const long long total = (long long)nlev * g.lm_max;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / g.lm_max);
    const int lm = (int)(i - (long long)r * g.lm_max);
    // order index by binary search in the m-major offsets
    int lo = 0, hi = g.n_m - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (g.lmoff[mid] <= lm) lo = mid;
      else hi = mid - 1;
    }
    const int m = lo * g.minc, l = m + (lm - g.lmoff[lo]);
    const long long o = (long long)r * a.ld + lm;
    const double rr = a.r[r], or1 = 1.0 / rr, or2 = or1 * or1, or4 = or2 * or2;
    const int lR = a.lcut ? min(a.lcut[r], g.l_max) : g.l_max;
    const double dLh = (double)l * (l + 1);
    if (a.nbc && a.nbc[r] != 0) {  // boundary level: only get_dbdt's dVxBhLM (get_td.f90:598-612)
      a.dVxBh[o] = cscale(a.VxBt[o], -dLh * rr * rr);
      continue;
    }
    const double two_cor = 2.0 * a.cor_fac;
    const bool hasS = l > m, hasA = l < lR;  // l-1 and l+1 terms (clm(m,m) = 0; l = l_R drops l+1)
    const double cS = hasS ? clm(l, m) : 0.0, cA = hasA ? clm(l + 1, m) : 0.0;
    const double2 zero = make_double2(0.0, 0.0);
    const double2 w = a.w[o], dw = a.dw[o], z = a.z[o];
    const double2 zS = hasS ? a.z[o - 1] : zero, zA = hasA ? a.z[o + 1] : zero;
    const double2 dwS = hasS ? a.dw[o - 1] : zero, dwA = hasA ? a.dw[o + 1] : zero;
    const double2 wS = hasS ? a.w[o - 1] : zero, wA = hasA ? a.w[o + 1] : zero;
    const bool inside = l <= lR;
    const double dm = (double)m;
    // dPhi * x = i m x
    auto iphi = [&](double2 x) { return make_double2(-dm * x.y, dm * x.x); };
    // ---- get_dwdt: or2 AdvrLM + 2 CorFac or1 (dPhi dw + dTheta2A z(l+1) - dTheta2S z(l-1))
    double2 dwdt = cscale(a.Advr[o], or2);
    if (inside) {
      const double t2A = (l + 2) * cA, t2S = (l - 1) * cS;
      const double2 p = iphi(dw);
      const double2 c = make_double2(p.x + t2A * zA.x - t2S * zS.x, p.y + t2A * zA.y - t2S * zS.y);
      if (l > 0) dwdt = cadd(dwdt, cscale(c, two_cor * or1));
      else dwdt = cadd(dwdt, cscale(make_double2(t2A * zA.x, t2A * zA.y), two_cor * or1));  // lm = 1
    }
    // ---- get_dzdt: dLh AdvpLM + 2 CorFac or2 (dPhi z + dTheta3A dw(l+1) + or1 dTheta4A w(l+1)
    //                                           + dTheta3S dw(l-1) - or1 dTheta4S w(l-1))
    double2 dzdt = l > 0 ? cscale(a.Advp[o], dLh) : zero;
    if (inside) {
      const double t3A = (double)l * (l + 2) * cA, t3S = (double)(l - 1) * (l + 1) * cS;
      const double t4A = (double)l * cA * (double)(l + 1) * (l + 2), t4S = (double)(l + 1) * cS * (double)(l - 1) * l;
      double2 c = make_double2(t3A * dwA.x + or1 * t4A * wA.x + t3S * dwS.x - or1 * t4S * wS.x,
                               t3A * dwA.y + or1 * t4A * wA.y + t3S * dwS.y - or1 * t4S * wS.y);
      if (l > 0) c = cadd(c, iphi(z));
      dzdt = cadd(dzdt, cscale(c, two_cor * or2));
    }
    // ---- get_dpdt: -dLh AdvtLM + 2 CorFac or2 (-dPhi (dw + or1 dLh w) + dTheta3A z(l+1) + dTheta3S z(l-1))
    double2 dpdt = zero;
    if (l > 0) {
      dpdt = cscale(a.Advt[o], -dLh);
      if (inside) {
        const double t3A = (double)l * (l + 2) * cA, t3S = (double)(l - 1) * (l + 1) * cS;
        const double2 q = iphi(make_double2(dw.x + or1 * dLh * w.x, dw.y + or1 * dLh * w.y));
        const double2 c = make_double2(-q.x + t3A * zA.x + t3S * zS.x, -q.y + t3A * zA.y + t3S * zS.y);
        dpdt = cadd(dpdt, cscale(c, two_cor * or2));
      }
    }
    // ---- get_dsdt (Boussinesq): dLh VStLM; l = 0: the internal heating epsc
    const double2 dsdt = l > 0 ? cscale(a.VSt[o], dLh) : make_double2(a.epsc ? a.epsc[r] : 0.0, 0.0);
    // ---- get_dbdt
    const double2 dbdt = cscale(a.VxBp[o], dLh);
    const double2 dVxBh = cscale(a.VxBt[o], -dLh * rr * rr);
    const double2 djdt = cscale(a.VxBr[o], dLh * or4);
    a.dwdt[o] = dwdt;
    a.dzdt[o] = dzdt;
    a.dpdt[o] = dpdt;
    a.dsdt[o] = dsdt;
    a.dbdt[o] = dbdt;
    a.djdt[o] = djdt;
    a.dVxBh[o] = dVxBh;
  }
}

}  // namespace

cudaError_t launch_get_td(const ShtGeom& g, const TdArgs& a, int nlev, cudaStream_t st) {
  const long long total = (long long)nlev * g.lm_max;
  if (total <= 0) return cudaSuccess;
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = std::min<long long>((total + 255) / 256, (long long)nsm * 8);
  get_td_kernel<<<(unsigned)blocks, 256, 0, st>>>(g, a, nlev);
  return cudaGetLastError();
}
