// Init-time FP64 tables on the GPU: Gauss-Legendre colatitudes/weights and the
// orthonormal associated Legendre functions P_lm(cos theta) and
// sin(theta) dP_lm/dtheta for the northern colatitudes.
//
//   gauleg:     src/horizontal.f90:279-340 (Newton iteration on P_N, eps = 10*eps)
//   plm_theta:  src/plms.f90:14-189 with norm=2 (x 1/sqrt(4 pi)), no Condon-
//               Shortley phase, the same three-term recurrence in l, the
//               same extra l = l_max+1 value for the derivative recurrence.
//   tables:     src/shtransforms.f90:67-77 (Plm, dPlm for n_theta/2 points).
//
// Layout: P[lm][j] with j (northern colatitude index) fastest; one thread
// per (m, j) runs the recurrence in l, so consecutive threads write
// consecutive j.
#include <cmath>
#include "common.cuh"
#include "internal.h"

namespace {

__global__ void gauleg_kernel(int n, double* theta, double* w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1-based root index
  const int mroots = (n + 1) / 2;
  if (i > mroots) return;
  const double pi = 3.141592653589793238462643383279502884;
  const double eps = 10.0 * 2.220446049250313e-16;
  double z = cos(pi * (((double)i - 0.25) / ((double)n + 0.5)));
  double z1 = z + 10.0 * eps;
  double p1 = 0, p2 = 0, p3 = 0, pp = 0;
  int it = 0;
  while (fabs(z - z1) > eps && it < 100) {  // bounded: Newton converges in < 10 steps
    p1 = 1.0; p2 = 0.0;
    for (int j = 1; j <= n; ++j) {
      p3 = p2; p2 = p1;
      p1 = ((double)(2 * j - 1) * z * p2 - (double)(j - 1) * p3) / (double)j;
    }
    pp = (double)n * (z * p1 - p2) / (z * z - 1.0);
    z1 = z;
    z = z1 - p1 / pp;
    ++it;
  }
  theta[i - 1] = acos(z);
  theta[n - i] = acos(-z);
  w[i - 1] = 2.0 / ((1.0 - z * z) * pp * pp);
  w[n - i] = w[i - 1];
}

__global__ void plm_kernel(int l_max, int m_max, int minc, int nh, const int* __restrict__ lmoff,
                           const double* __restrict__ theta, double* __restrict__ P,
                           double* __restrict__ dP) {
  const int n_m = m_max / minc + 1;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n_m * nh) return;
  const int j = (int)(idx % nh);
  const int mc = (int)(idx / nh);
  const int m = mc * minc;
  const int lm0 = lmoff[mc];
  const double th = theta[j];
  const double dnorm = 1.0 / sqrt(4.0 * 3.141592653589793238462643383279502884);
  const double ct = cos(th), st = sin(th);
  double fac = 1.0;
  for (int jj = 3; jj <= 2 * m + 1; jj += 2) fac = fac * (double)jj / (double)(jj - 1);
  double plm = sqrt(fac);
  if (st != 0.0) plm = plm * pow(st, (double)m);
  else if (m != 0) plm = 0.0;
  P[(size_t)lm0 * nh + j] = dnorm * plm;
  double plm1 = 0.0, plm2 = 0.0;
  for (int l = m + 1; l <= l_max; ++l) {
    plm2 = plm1; plm1 = plm;
    plm = ct * sqrt((double)((2 * l - 1) * (2 * l + 1)) / (double)((l - m) * (l + m))) * plm1 -
          sqrt(((double)(2 * l + 1) * (double)(l + m - 1) * (double)(l - m - 1)) /
               ((double)(2 * l - 3) * (double)(l - m) * (double)(l + m))) * plm2;
    P[(size_t)(lm0 + l - m) * nh + j] = dnorm * plm;
  }
  double pextra;  // P_{l_max+1, m}
  {
    const int l = l_max + 1;
    plm2 = plm1; plm1 = plm;
    plm = ct * sqrt((double)((2 * l - 1) * (2 * l + 1)) / (double)((l - m) * (l + m))) * plm1 -
          sqrt((double)((2 * l + 1) * (l + m - 1) * (l - m - 1)) /
               (double)((2 * l - 3) * (l - m) * (l + m))) * plm2;
    pextra = dnorm * plm;
  }
  // sin(theta) dP/dtheta from the l-1 / l+1 neighbours (plms.f90:120-187)
  double pm1 = 0.0;
  double p0 = P[(size_t)lm0 * nh + j];
  for (int l = m; l <= l_max; ++l) {
    const double pp1 = (l < l_max) ? P[(size_t)(lm0 + l - m + 1) * nh + j] : pextra;
    double d;
    if (l == m) {
      d = l / sqrt((double)(2 * l + 3)) * pp1;
    } else {
      d = l * sqrt((double)((l + m + 1) * (l - m + 1)) / (double)((2 * l + 1) * (2 * l + 3))) * pp1 -
          (l + 1) * sqrt((double)((l + m) * (l - m)) / (double)((2 * l - 1) * (2 * l + 1))) * pm1;
    }
    dP[(size_t)(lm0 + l - m) * nh + j] = d;
    pm1 = p0;
    p0 = pp1;
  }
}

__global__ void aux_kernel(int nh, const double* __restrict__ theta, const double* __restrict__ gauss,
                           double* wgt, double* osin2) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nh) return;
  const double s = sin(theta[j]);
  wgt[j] = 2.0 * 3.141592653589793238462643383279502884 * gauss[j];
  osin2[j] = 1.0 / (s * s);
}

__global__ void to_fp32_kernel(const double* a, const double* b, float* a32, float* b32, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    a32[i] = (float)a[i];
    b32[i] = (float)b[i];
  }
}

}  // namespace

cudaError_t build_tables_fp64(int l_max, int m_max, int minc, int n_theta, const int* d_lmoff,
                              double* d_theta, double* d_gauss, double* d_P, double* d_dP,
                              double* d_wgt, double* d_osin2, cudaStream_t st) {
  const int nh = n_theta / 2;
  const int roots = (n_theta + 1) / 2;
  gauleg_kernel<<<(roots + 127) / 128, 128, 0, st>>>(n_theta, d_theta, d_gauss);
  CUDA_TRY(cudaGetLastError());
  const int n_m = m_max / minc + 1;
  const long long nthr = (long long)n_m * nh;
  plm_kernel<<<(unsigned)((nthr + 127) / 128), 128, 0, st>>>(l_max, m_max, minc, nh, d_lmoff,
                                                              d_theta, d_P, d_dP);
  CUDA_TRY(cudaGetLastError());
  aux_kernel<<<(nh + 127) / 128, 128, 0, st>>>(nh, d_theta, d_gauss, d_wgt, d_osin2);
  return cudaGetLastError();
}

cudaError_t convert_tables_fp32(const double* P, const double* dP, float* P32, float* dP32,
                                size_t n, cudaStream_t st) {
  to_fp32_kernel<<<1024, 256, 0, st>>>(P, dP, P32, dP32, n);
  return cudaGetLastError();
}
