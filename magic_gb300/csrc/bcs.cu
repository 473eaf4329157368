// Boundary pieces of the radial loop (nonlinear_bcs.f90) on the device, one
// radial level each.  Grids are f(ld, n_phi) with theta fastest and the rows
// scrambled north/south: rows 2j and 2j+1 sit at colatitudes theta_j and
// pi - theta_j, so sin(theta) is shared and cos(theta) changes sign
// (horizontal.f90:145-159); phi_k = 2 pi k / (n_phi minc) (horizontal.f90:186-187).
#include "common.cuh"
#include "internal.h"

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;

struct RowTrig {
  double s, c;  // sin, cos of the row's colatitude
};
__device__ __forceinline__ RowTrig row_trig(const double* theta, int th) {
  const double colat = theta[th >> 1];
  double s, c;
  sincos(colat, &s, &c);
  return {s, (th & 1) ? -c : c};
}

// v_rigid_boundary (nonlinear_bcs.f90:120-175): a rigid boundary rotating at
// omega: vr = 0 (unless keep_vr), vt = 0, vp = r^2 rho0 sin^2(theta) omega; with
// the derivative grids, cvr = 2 r^2 rho0 cos(theta) omega and the four angular
// derivatives 0.
__global__ void rigid_kernel(const ShtGeom g, const double* theta, BcGrids a, double r2rho0, double omega,
                             int keep_vr) {
  const long long n = (long long)g.n_phi * g.n_theta;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int ph = (int)(p / g.n_theta), th = (int)(p - (long long)ph * g.n_theta);
    const long long o = (long long)ph * g.ld + th;
    const RowTrig t = row_trig(theta, th);
    if (!keep_vr && a.p[0]) a.p[0][o] = 0.0;
    if (a.p[1]) a.p[1][o] = 0.0;
    if (a.p[2]) a.p[2][o] = r2rho0 * (t.s * t.s) * omega;
    if (a.p[3]) a.p[3][o] = r2rho0 * 2.0 * t.c * omega;
    for (int i = 4; i < 8; ++i)
      if (a.p[i]) a.p[i][o] = 0.0;
  }
}

// v_center_sphere (nonlinear_bcs.f90:177-224): the l = 1 flow through the
// centre of a full sphere from ddw(l=1, m=0) and ddw(l=1, m=1) (minc = 1).
__global__ void center_kernel(const ShtGeom g, const double* theta, const double2* ddw, int lm11, double* vr,
                              double* vt, double* vp) {
  const double y10 = 0.5 * sqrt(3.0 / kPi), y11 = 0.5 * sqrt(1.5 / kPi);  // preCalculations.f90:313-314
  const double d10 = ddw[1].x;                                           // lm2(1,0): the second entry
  const double2 d11 = lm11 >= 0 ? ddw[lm11] : make_double2(0.0, 0.0);
  const double dphi = 2.0 * kPi / (double)(g.n_phi * g.minc);
  const long long n = (long long)g.n_phi * g.n_theta;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int ph = (int)(p / g.n_theta), th = (int)(p - (long long)ph * g.n_theta);
    const long long o = (long long)ph * g.ld + th;
    const RowTrig t = row_trig(theta, th);
    if (lm11 >= 0) {
      double sp, cp;
      sincos(ph * dphi, &sp, &cp);
      const double c = d11.x * cp - d11.y * sp;
      vr[o] = y10 * d10 * t.c + 2.0 * y11 * t.s * c;
      vt[o] = t.s * (-y10 * d10 * t.s + 2.0 * y11 * t.c * c);
      vp[o] = -2.0 * y11 * t.s * (d11.x * sp + d11.y * cp);
    } else {
      vr[o] = y10 * d10 * t.c;
      vt[o] = -t.s * y10 * d10 * t.s;
      vp[o] = 0.0;
    }
  }
}

// grid products of get_br_v_bcs (nonlinear_bcs.f90:24-69):
//   br_vt = fac br vt,  br_vp = br (fac vp - omega sin^2(theta)),  fac = or2 orho1
__global__ void br_v_kernel(const ShtGeom g, const double* theta, const double* br, const double* vt,
                            const double* vp, double fac, double omega, double* out_t, double* out_p) {
  const long long n = (long long)g.n_phi * g.ld;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const int th = (int)(p % g.ld);
    if (th >= g.n_theta) {
      out_t[p] = 0.0;
      out_p[p] = 0.0;
      continue;
    }
    const RowTrig t = row_trig(theta, th);
    out_t[p] = fac * br[p] * vt[p];
    out_p[p] = br[p] * (fac * vp[p] - omega * (t.s * t.s));
  }
}

// get_b_nl_bcs (nonlinear_bcs.f90:71-118): x(lm) = -fac y(lm), x(l=0) = 0
__global__ void b_nl_kernel(int K, double fac, const double2* y, double2* x) {
  const int lm = blockIdx.x * blockDim.x + threadIdx.x;
  if (lm >= K) return;
  x[lm] = lm == 0 ? make_double2(0.0, 0.0) : make_double2(-fac * y[lm].x, -fac * y[lm].y);
}

int grid_blocks(const ShtGeom& g) {
  const long long n = (long long)g.n_phi * g.ld;
  long long b = (n + 255) / 256;
  return (int)(b < 2048 ? b : 2048);
}

// Lorentz torque on a rotating, conducting boundary (get_lorentz_torque,
// outRot.f90:423-483): LFfac 2 pi / n_phi times the sum over one level's grid
// of gauss(theta) (br - b0 cos(theta)) bp.  Deterministic: block b sums the
// phi rows [b n_phi / nblk, (b+1) n_phi / nblk) (threads over the colatitude
// pairs j: rows 2j and 2j+1 at theta_j and pi - theta_j share the weight
// 2 pi w_j), and one thread adds the block sums in order.
__global__ void __launch_bounds__(256) torque_partial_kernel(const ShtGeom g, const double* __restrict__ theta,
                                                             const double* __restrict__ br,
                                                             const double* __restrict__ bp, double b0,
                                                             double* __restrict__ partial) {
  __shared__ double red[256 / 32];
  const int p0 = (int)((long long)blockIdx.x * g.n_phi / gridDim.x);
  const int p1 = (int)((long long)(blockIdx.x + 1) * g.n_phi / gridDim.x);
  double acc = 0.0;
  for (int j = threadIdx.x; j < g.nh; j += blockDim.x) {
    const double c = b0 != 0.0 ? b0 * cos(theta[j]) : 0.0;  // b0r of row 2j; row 2j+1 has -c
    double sj = 0.0;
    for (int ph = p0; ph < p1; ++ph) {
      const long long o = (long long)ph * g.ld + 2 * j;
      sj += (br[o] - c) * bp[o] + (br[o + 1] + c) * bp[o + 1];
    }
    acc += g.wgt[j] * sj;
  }
  for (int d = 16; d >= 1; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    partial[blockIdx.x] = t;
  }
}

__global__ void torque_finish_kernel(const double* __restrict__ partial, int n, double fac, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < n; ++i) t += partial[i];
    out[0] = fac * t;
  }
}

}  // namespace

int lorentz_torque_blocks(const ShtGeom& g) { return g.n_phi < 128 ? g.n_phi : 128; }

cudaError_t launch_lorentz_torque(const ShtGeom& g, const double* theta, const double* br, const double* bp,
                                  double LFfac, double b0, double* partial, double* out, cudaStream_t st) {
  const int nblk = lorentz_torque_blocks(g);
  torque_partial_kernel<<<nblk, 256, 0, st>>>(g, theta, br, bp, b0, partial);
  CUDA_TRY(cudaGetLastError());
  // the 2 pi of LFfac 2 pi / n_phi is already inside g.wgt (2 pi w_j, built
  // by the table kernels), so the remaining factor is LFfac / n_phi
  torque_finish_kernel<<<1, 32, 0, st>>>(partial, nblk, LFfac / (double)g.n_phi, out);
  return cudaGetLastError();
}

cudaError_t launch_v_rigid_boundary(const ShtGeom& g, const double* theta, const BcGrids& a, double r2rho0,
                                    double omega, int keep_vr, cudaStream_t st) {
  rigid_kernel<<<grid_blocks(g), 256, 0, st>>>(g, theta, a, r2rho0, omega, keep_vr);
  return cudaGetLastError();
}

cudaError_t launch_v_center_sphere(const ShtGeom& g, const double* theta, const double2* ddw, int lm11, double* vr,
                                   double* vt, double* vp, cudaStream_t st) {
  center_kernel<<<grid_blocks(g), 256, 0, st>>>(g, theta, ddw, lm11, vr, vt, vp);
  return cudaGetLastError();
}

cudaError_t launch_br_v_products(const ShtGeom& g, const double* theta, const double* br, const double* vt,
                                 const double* vp, double fac, double omega, double* out_t, double* out_p,
                                 cudaStream_t st) {
  br_v_kernel<<<grid_blocks(g), 256, 0, st>>>(g, theta, br, vt, vp, fac, omega, out_t, out_p);
  return cudaGetLastError();
}

cudaError_t launch_b_nl_bcs(int K, double fac, const double2* y, double2* x, cudaStream_t st) {
  b_nl_kernel<<<(K + 255) / 256, 256, 0, st>>>(K, fac, y, x);
  return cudaGetLastError();
}
