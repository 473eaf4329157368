// ---------------------------------------------------------------------------
// ORACLE — test infrastructure only.
//
// A CPU FP64 restatement of MagIC's native spherical-harmonic transforms
// (module `sht` in src/sht_native.f90 over module `shtransforms` in
// src/shtransforms.f90, Legendre tables from src/plms.f90, Gauss nodes from
// src/horizontal.f90, azimuthal FFT conventions from src/fft.f90).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
// this library, and only as the checker / the timed CPU reference.  The GPU
// product never calls it.
//
// The reference itself is Fortran and cannot be compiled in this environment
// (no Fortran compiler), so this file follows its loops statement by
// statement; each routine cites the reference lines it restates.  The FFT is
// our own mixed-radix (2,3,4,5) Stockham FFT that implements the transform
// *definition* of fft991 (src/fft.f90:262-268): the inverse is unnormalised
// and ignores Im(c_0), Im(c_{n/2}); the forward carries the 1/n factor and
// returns Im(c_0) = Im(c_{n/2}) = 0.
//
// Layouts (identical to the reference): spectral arrays are complex(8) in
// st_map order (m-major, l inner: src/blocking.f90:309-317); grid arrays are
// real(8) f(n_theta_max, n_phi_max) column-major with theta fastest and the
// theta rows scrambled north/south (row 2j north, 2j+1 south, 0-based;
// src/sht_native.f90:29, src/horizontal.f90:145-157).
// ---------------------------------------------------------------------------
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

typedef std::complex<double> cplx;
static const double PI = 4.0 * std::atan(1.0);            // constants.f90:17
static const cplx CI(0.0, 1.0);

// ----------------------------------------------------------------- FFT ----
// Complex Stockham FFT, radices 4,2,3,5, length n.  sign=-1 forward.
struct CFFT {
  int n = 0;
  std::vector<int> radix;
  std::vector<cplx> wfwd;  // e^{-2 pi i k / n}
  void init(int n_) {
    n = n_;
    radix.clear();
    int r = n;
    while (r % 4 == 0) { radix.push_back(4); r /= 4; }
    while (r % 2 == 0) { radix.push_back(2); r /= 2; }
    while (r % 3 == 0) { radix.push_back(3); r /= 3; }
    while (r % 5 == 0) { radix.push_back(5); r /= 5; }
    if (r != 1) { radix.clear(); n = -1; return; }
    wfwd.resize(n);
    for (int k = 0; k < n; ++k) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * k / n;
      wfwd[k] = cplx((double)cosl(a), (double)sinl(a));
    }
  }
  // in/out may alias `a`; `work` is scratch of length n.
  void run(cplx* a, cplx* work, int sign) const {
    cplx* src = a;
    cplx* dst = work;
    int Ns = 1;
    for (int R : radix) {
      const int nR = n / R;
      const int tstep = n / (Ns * R);
      for (int j = 0; j < nR; ++j) {
        const int k = j % Ns;
        cplx v[5];
        for (int q = 0; q < R; ++q) {
          cplx w = wfwd[(k * q * tstep) % n];
          if (sign > 0) w = std::conj(w);
          v[q] = src[j + q * nR] * w;
        }
        cplx o[5];
        for (int p = 0; p < R; ++p) {
          cplx s = 0.0;
          for (int q = 0; q < R; ++q) {
            cplx w = wfwd[((p * q) % R) * (n / R)];
            if (sign > 0) w = std::conj(w);
            s += v[q] * w;
          }
          o[p] = s;
        }
        const int idxD = (j / Ns) * Ns * R + k;
        for (int p = 0; p < R; ++p) dst[idxD + p * Ns] = o[p];
      }
      std::swap(src, dst);
      Ns *= R;
    }
    if (src != a) std::memcpy(a, src, sizeof(cplx) * n);
  }
};

// Real <-> half-complex transform of length P (P multiple of 4), fft991
// definition (src/fft.f90:262-268).
struct RFFT {
  int P = 0, nh = 0;
  CFFT c;
  std::vector<cplx> wP;  // e^{+2 pi i k / P}
  void init(int P_) {
    P = P_; nh = P / 2; c.init(nh);
    wP.resize(nh + 1);
    for (int k = 0; k <= nh; ++k) {
      long double a = 2.0L * 3.14159265358979323846264338327950288L * k / P;
      wP[k] = cplx((double)cosl(a), (double)sinl(a));
    }
  }
  // isign=+1: x(j) = sum_k c_k e^{2 pi i j k / P} with hermitian extension.
  void inverse(const cplx* cin, double* x, cplx* buf, cplx* work) const {
    for (int k = 0; k < nh; ++k) {
      cplx ck = cin[k];
      cplx cn = cin[nh - k];
      if (k == 0) { ck = cplx(ck.real(), 0.0); cn = cplx(cn.real(), 0.0); }
      cplx E = ck + std::conj(cn);
      cplx O = (ck - std::conj(cn)) * wP[k];
      buf[k] = E + CI * O;
    }
    c.run(buf, work, +1);
    for (int j = 0; j < nh; ++j) { x[2 * j] = buf[j].real(); x[2 * j + 1] = buf[j].imag(); }
  }
  // isign=-1: c_k = (1/P) sum_j x_j e^{-2 pi i j k / P}, k=0..P/2.
  void forward(const double* x, cplx* cout, cplx* buf, cplx* work) const {
    for (int j = 0; j < nh; ++j) buf[j] = cplx(x[2 * j], x[2 * j + 1]);
    c.run(buf, work, -1);
    const double sc = 1.0 / P;
    for (int k = 0; k <= nh; ++k) {
      cplx Zk = buf[k % nh];
      cplx Zn = std::conj(buf[(nh - k) % nh]);
      cplx X = 0.5 * (Zk + Zn) - 0.5 * CI * std::conj(wP[k]) * (Zk - Zn);
      cout[k] = X * sc;
    }
    cout[0] = cplx(cout[0].real(), 0.0);
    cout[nh] = cplx(cout[nh].real(), 0.0);
  }
};

// ------------------------------------------------------------- Oracle ----
struct Oracle {
  int l_max, m_min, m_max, minc, n_theta, n_phi, n_m_max, lm_max, nh;
  std::vector<double> theta_ord, gauss;            // gauleg, north -> south
  std::vector<double> Plm, dPlm, wPlm, wdPlm;      // [nh][lm_max], lm fastest
  std::vector<int> lStart, lStop;                  // 0-based, inclusive
  std::vector<double> D_mc2m;
  std::vector<int> lm2l, lm2m;
  std::vector<double> dLh, O_sin_theta_E2;         // O_sin_theta_E2 scrambled
  RFFT fft;
};

// gauleg: src/horizontal.f90:279-340 (NR Newton iteration on P_N).
static void gauleg(double sinThMin, double sinThMax, int n_th_max, double* theta_ord,
                   double* gauss) {
  const double eps = 10.0 * 2.220446049250313e-16;  // 10*epsilon(one)
  const int m = (n_th_max + 1) / 2;
  const double sinThMean = 0.5 * (sinThMax + sinThMin);
  const double sinThDiff = 0.5 * (sinThMax - sinThMin);
  for (int i = 1; i <= m; ++i) {
    double z = std::cos(PI * (((double)i - 0.25) / ((double)n_th_max + 0.5)));
    double z1 = z + 10.0 * eps;
    double p1 = 0, p2 = 0, p3 = 0, pp = 0;
    while (std::fabs(z - z1) > eps) {
      p1 = 1.0; p2 = 0.0;
      for (int j = 1; j <= n_th_max; ++j) {
        p3 = p2; p2 = p1;
        p1 = ((double)(2 * j - 1) * z * p2 - (double)(j - 1) * p3) / (double)j;
      }
      pp = (double)n_th_max * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    }
    theta_ord[i - 1] = std::acos(sinThMean + sinThDiff * z);
    theta_ord[n_th_max - i] = std::acos(sinThMean - sinThDiff * z);
    gauss[i - 1] = 2.0 * sinThDiff / ((1.0 - z * z) * pp * pp);
    gauss[n_th_max - i] = gauss[i - 1];
  }
}

// plm_theta with norm=2: src/plms.f90:14-189.  plma/dtheta_plma are m-major.
static void plm_theta(double theta, int max_degree, int min_order, int max_order, int m0,
                      double* plma, double* dtheta_plma) {
  const double dnorm = 1.0 / std::sqrt(4.0 * PI);  // osq4pi, constants.f90:19
  int pos = 0;
  for (int m = min_order; m <= max_order; m += m0) {
    double fac = 1.0;
    for (int j = 3; j <= 2 * m + 1; j += 2) fac = fac * (double)j / (double)(j - 1);
    double plm = std::sqrt(fac);
    if (std::sin(theta) != 0.0) plm = plm * std::pow(std::sin(theta), m);
    else if (m != 0) plm = 0.0;
    plma[pos++] = dnorm * plm;
    double plm1 = 0.0, plm2 = 0.0;
    for (int l = m + 1; l <= max_degree; ++l) {
      plm2 = plm1; plm1 = plm;
      plm = std::cos(theta) * std::sqrt((double)((2 * l - 1) * (2 * l + 1)) /
                                        (double)((l - m) * (l + m))) * plm1 -
            std::sqrt(((double)(2 * l + 1) * (double)(l + m - 1) * (double)(l - m - 1)) /
                      ((double)(2 * l - 3) * (double)(l - m) * (double)(l + m))) * plm2;
      plma[pos++] = dnorm * plm;
    }
    // extra l = max_degree+1 value kept in dtheta_plma(pos) (plms.f90:102-113)
    const int l = max_degree + 1;
    plm2 = plm1; plm1 = plm;
    plm = std::cos(theta) * std::sqrt((double)((2 * l - 1) * (2 * l + 1)) /
                                      (double)((l - m) * (l + m))) * plm1 -
          std::sqrt((double)((2 * l + 1) * (l + m - 1) * (l - m - 1)) /
                    (double)((2 * l - 3) * (l - m) * (l + m))) * plm2;
    dtheta_plma[pos - 1] = dnorm * plm;
  }
  pos = 0;
  for (int m = min_order; m <= max_order; m += m0) {
    int l = m;
    pos++;
    if (m < max_degree) {
      dtheta_plma[pos - 1] = l / std::sqrt((double)(2 * l + 3)) * plma[pos];
    } else {
      dtheta_plma[pos - 1] = l / std::sqrt((double)(2 * l + 3)) * dtheta_plma[pos - 1];
    }
    for (l = m + 1; l <= max_degree - 1; ++l) {
      pos++;
      dtheta_plma[pos - 1] =
          l * std::sqrt((double)((l + m + 1) * (l - m + 1)) / (double)((2 * l + 1) * (2 * l + 3))) *
              plma[pos] -
          (l + 1) * std::sqrt((double)((l + m) * (l - m)) / (double)((2 * l - 1) * (2 * l + 1))) *
              plma[pos - 2];
    }
    if (m < max_degree) {
      l = max_degree;
      pos++;
      dtheta_plma[pos - 1] =
          l * std::sqrt((double)((l + m + 1) * (l - m + 1)) / (double)((2 * l + 1) * (2 * l + 3))) *
              dtheta_plma[pos - 1] -
          (l + 1) * std::sqrt((double)((l + m) * (l - m)) / (double)((2 * l - 1) * (2 * l + 1))) *
              plma[pos - 2];
    }
  }
}

// get_openmp_blocks: src/parallel.f90:94-146 (0-based, inclusive bounds).
static void omp_block(int gStart, int gStop, int& nStart, int& nStop) {
  int n_points = gStop - gStart + 1;
  int nthr = omp_get_num_threads(), tid = omp_get_thread_num();
  nStart = gStart; nStop = gStop;
  if (n_points == 1) return;
  int per, left;
  if (n_points < nthr) { per = 1; left = 0; if (tid >= n_points) { nStart = 1; nStop = 0; return; } }
  else { per = n_points / nthr; left = n_points - nthr * per; }
  if (tid + 1 <= left) { nStart = gStart + tid * per + tid; nStop = nStart + per; }
  else { nStart = gStart + tid * per + left; nStop = nStart + per - 1; }
}

extern "C" {

int oracle_version() { return 1; }
void oracle_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }
int oracle_max_threads() { return omp_get_max_threads(); }

void oracle_gauleg(int n, double* theta, double* w) { gauleg(-1.0, 1.0, n, theta, w); }

void oracle_plm_theta(double theta, int l_max, int m_min, int m_max, int minc, double* plma,
                      double* dplma) {
  plm_theta(theta, l_max, m_min, m_max, minc, plma, dplma);
}

// Grid sizing from l_max (src/truncation.f90:50-124 with nalias, prime
// decomposition :162-192).  out = {n_theta_max, n_phi_tot, n_phi_max, m_max, n_m_max, lm_max}
void oracle_truncation(int l_max, int nalias, int minc, int* out) {
  int n_theta = (30 * l_max) / nalias;
  int nlon = 2 * n_theta;
  double dist_min = 100.0; int i0 = 0, j0 = 0, k0 = 0;
  for (int i = 0; i <= 12; ++i)
    for (int j = 0; j <= 6; ++j)
      for (int k = 0; k <= 6; ++k) {
        double res = std::pow(2.0, i) * std::pow(3.0, j) * std::pow(5.0, k);
        double dist = res - nlon;
        if (dist >= 0 && dist < dist_min) { i0 = i; j0 = j; k0 = k; dist_min = dist; }
      }
  int n_phi_tot = (int)(std::pow(2.0, i0) * std::pow(3.0, j0) * std::pow(5.0, k0) + 0.5);
  int n_phi_max = n_phi_tot / minc;
  n_theta = n_phi_tot / 2;
  int m_max = (l_max / minc) * minc;
  if (m_max > l_max) m_max = l_max;
  int n_m_max = m_max / minc + 1;
  int lm_max = 0;
  for (int m = 0; m <= m_max; m += minc) lm_max += l_max - m + 1;
  out[0] = n_theta; out[1] = n_phi_tot; out[2] = n_phi_max; out[3] = m_max; out[4] = n_m_max;
  out[5] = lm_max;
}

// initialize_transforms (src/shtransforms.f90:38-91) + the horizontal()
// pieces the transforms use (src/horizontal.f90:141-157, :216).
void* oracle_init(int l_max, int minc, int n_theta, int n_phi_max, int m_max) {
  if (n_theta % 4 != 0 || n_phi_max % 4 != 0 || minc < 1 || l_max < 1) return nullptr;
  Oracle* o = new Oracle();
  o->l_max = l_max; o->minc = minc; o->n_theta = n_theta; o->n_phi = n_phi_max;
  o->m_min = 0;
  if (m_max <= 0) m_max = (l_max / minc) * minc;
  if (m_max > l_max) m_max = l_max;
  o->m_max = m_max;
  o->n_m_max = m_max / minc + 1;
  int lm = 0;
  for (int m = 0; m <= m_max; m += minc) lm += l_max - m + 1;
  o->lm_max = lm;
  o->nh = n_theta / 2;
  o->theta_ord.resize(n_theta); o->gauss.resize(n_theta);
  gauleg(-1.0, 1.0, n_theta, o->theta_ord.data(), o->gauss.data());
  const int K = o->lm_max, nh = o->nh;
  o->Plm.resize((size_t)K * nh); o->dPlm.resize((size_t)K * nh);
  o->wPlm.resize((size_t)K * nh); o->wdPlm.resize((size_t)K * nh);
  std::vector<double> plma(K + 1), dplma(K + 1);
  for (int j = 0; j < nh; ++j) {
    plm_theta(o->theta_ord[j], l_max, 0, m_max, minc, plma.data(), dplma.data());
    for (int i = 0; i < K; ++i) {
      o->Plm[(size_t)j * K + i] = plma[i];
      o->dPlm[(size_t)j * K + i] = dplma[i];
      o->wPlm[(size_t)j * K + i] = 2.0 * PI * o->gauss[j] * plma[i];
      o->wdPlm[(size_t)j * K + i] = 2.0 * PI * o->gauss[j] * dplma[i];
    }
  }
  o->lStart.resize(o->n_m_max); o->lStop.resize(o->n_m_max); o->D_mc2m.resize(o->n_m_max);
  o->lStart[0] = 0; o->lStop[0] = l_max; o->D_mc2m[0] = 0.0;
  for (int mc = 1; mc < o->n_m_max; ++mc) {
    int m = mc * minc;
    o->D_mc2m[mc] = (double)m;
    o->lStart[mc] = o->lStop[mc - 1] + 1;
    o->lStop[mc] = o->lStart[mc] + l_max - m;
  }
  o->lm2l.resize(K); o->lm2m.resize(K); o->dLh.resize(K);
  lm = 0;
  for (int m = 0; m <= m_max; m += minc)
    for (int l = m; l <= l_max; ++l) {
      o->lm2l[lm] = l; o->lm2m[lm] = m; o->dLh[lm] = (double)(l * (l + 1)); ++lm;
    }
  o->O_sin_theta_E2.resize(n_theta);
  for (int j = 0; j < nh; ++j) {
    double colat = o->theta_ord[j];
    o->O_sin_theta_E2[2 * j] = 1.0 / (std::sin(colat) * std::sin(colat));
    o->O_sin_theta_E2[2 * j + 1] = 1.0 / (std::sin(colat) * std::sin(colat));
  }
  o->fft.init(n_phi_max);
  if (o->fft.c.n < 0) { delete o; return nullptr; }
  return o;
}

void oracle_free(void* h) { delete (Oracle*)h; }

// {l_max, m_max, minc, n_theta, n_phi_max, n_m_max, lm_max}
void oracle_sizes(void* h, int* out) {
  Oracle* o = (Oracle*)h;
  out[0] = o->l_max; out[1] = o->m_max; out[2] = o->minc; out[3] = o->n_theta;
  out[4] = o->n_phi; out[5] = o->n_m_max; out[6] = o->lm_max;
}

// Copies of the tables (for tests): theta_ord/gauss (n_theta), Plm/dPlm
// as [nh][lm_max].
void oracle_tables(void* h, double* theta, double* gauss, double* plm, double* dplm) {
  Oracle* o = (Oracle*)h;
  if (theta) std::memcpy(theta, o->theta_ord.data(), sizeof(double) * o->n_theta);
  if (gauss) std::memcpy(gauss, o->gauss.data(), sizeof(double) * o->n_theta);
  if (plm) std::memcpy(plm, o->Plm.data(), sizeof(double) * o->Plm.size());
  if (dplm) std::memcpy(dplm, o->dPlm.data(), sizeof(double) * o->dPlm.size());
}

}  // extern "C"

// ---------------------------------------------------- FFT over theta rows ----
// ifft_many / fft_many (src/fft.f90:164-252): theta-fastest arrays,
// tmp(n_theta, n_phi/2+1) complex <-> g(n_theta, n_phi) real.
static void ifft_many(const Oracle* o, const cplx* tmp, double* g) {
  const int N = o->n_theta, P = o->n_phi, nh = P / 2;
#pragma omp parallel
  {
    std::vector<cplx> cin(nh + 1), buf(nh), work(nh);
    std::vector<double> x(P);
#pragma omp for schedule(static)
    for (int t = 0; t < N; ++t) {
      for (int k = 0; k <= nh; ++k) cin[k] = tmp[(size_t)k * N + t];
      o->fft.inverse(cin.data(), x.data(), buf.data(), work.data());
      for (int p = 0; p < P; ++p) g[(size_t)p * N + t] = x[p];
    }
  }
}

static void fft_many(const Oracle* o, const double* g, cplx* tmp) {
  const int N = o->n_theta, P = o->n_phi, nh = P / 2;
#pragma omp parallel
  {
    std::vector<cplx> cout(nh + 1), buf(nh), work(nh);
    std::vector<double> x(P);
#pragma omp for schedule(static)
    for (int t = 0; t < N; ++t) {
      for (int p = 0; p < P; ++p) x[p] = g[(size_t)p * N + t];
      o->fft.forward(x.data(), cout.data(), buf.data(), work.data());
      for (int k = 0; k <= nh; ++k) tmp[(size_t)k * N + t] = cout[k];
    }
  }
}

// ------------------------------------------------------- native routines ----
// native_qst_to_spat: src/shtransforms.f90:103-245.
static void native_qst_to_spat(const Oracle* o, const cplx* Qlm, const cplx* Slm,
                               const cplx* Tlm, double* brc, double* btc, double* bpc,
                               int lcut) {
  const int N = o->n_theta, nhp = o->n_phi / 2 + 1, K = o->lm_max;
  std::vector<cplx> bhG(K), bhC(K);
  std::vector<cplx> tmpr((size_t)N * nhp), tmpt((size_t)N * nhp), tmpp((size_t)N * nhp);
  bhG[0] = 0.0; bhC[0] = 0.0;
  for (int lm = 1; lm < K; ++lm) { bhG[lm] = Slm[lm] - CI * Tlm[lm]; bhC[lm] = Slm[lm] + CI * Tlm[lm]; }
#pragma omp parallel
  {
    std::vector<double> PlmG(K), PlmC(K);
    int s0, s1;
    omp_block(0, N / 2 - 1, s0, s1);
    for (int mc = 0; mc < o->n_m_max; ++mc) {
      const int m = mc * o->minc;
      if (m > lcut) {
        for (int j = s0; j <= s1; ++j)
          for (int r = 0; r < 2; ++r) {
            tmpr[(size_t)mc * N + 2 * j + r] = 0.0;
            tmpt[(size_t)mc * N + 2 * j + r] = 0.0;
            tmpp[(size_t)mc * N + 2 * j + r] = 0.0;
          }
        continue;
      }
      const double dm = o->D_mc2m[mc];
      const int lmS = o->lStop[mc] + lcut - o->l_max;
      const bool l_Odd = ((lmS - o->lStart[mc]) % 2 == 0);
      for (int j = s0; j <= s1; ++j) {
        const double* P = &o->Plm[(size_t)j * K];
        const double* dP = &o->dPlm[(size_t)j * K];
        cplx brES = 0.0, brEA = 0.0;
        int lm;
        for (lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          brES += Qlm[lm] * P[lm];
          brEA += Qlm[lm + 1] * P[lm + 1];
          PlmG[lm] = dP[lm] - dm * P[lm];
          PlmC[lm] = dP[lm] + dm * P[lm];
          PlmG[lm + 1] = dP[lm + 1] - dm * P[lm + 1];
          PlmC[lm + 1] = dP[lm + 1] + dm * P[lm + 1];
        }
        if (l_Odd) {
          brES += Qlm[lmS] * P[lmS];
          PlmG[lmS] = dP[lmS] - dm * P[lmS];
          PlmC[lmS] = dP[lmS] + dm * P[lmS];
        }
        tmpr[(size_t)mc * N + 2 * j] = brES + brEA;
        tmpr[(size_t)mc * N + 2 * j + 1] = brES - brEA;
        cplx bhN1 = 0.0, bhS1 = 0.0, bhN2 = 0.0, bhS2 = 0.0;
        for (lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          bhN1 = bhN1 + bhG[lm] * PlmG[lm] + bhG[lm + 1] * PlmG[lm + 1];
          bhS1 = bhS1 - bhG[lm] * PlmC[lm] + bhG[lm + 1] * PlmC[lm + 1];
          bhN2 = bhN2 + bhC[lm] * PlmC[lm] + bhC[lm + 1] * PlmC[lm + 1];
          bhS2 = bhS2 - bhC[lm] * PlmG[lm] + bhC[lm + 1] * PlmG[lm + 1];
        }
        if (l_Odd) {
          bhN1 = bhN1 + bhG[lmS] * PlmG[lmS];
          bhS1 = bhS1 - bhG[lmS] * PlmC[lmS];
          bhN2 = bhN2 + bhC[lmS] * PlmC[lmS];
          bhS2 = bhS2 - bhC[lmS] * PlmG[lmS];
        }
        cplx bhN1M = 0.5 * bhN1, bhS1M = 0.5 * bhS1, bhN2M = 0.5 * bhN2, bhS2M = 0.5 * bhS2;
        tmpt[(size_t)mc * N + 2 * j] = bhN1M + bhN2M;
        cplx bhN = bhN1M - bhN2M;
        tmpt[(size_t)mc * N + 2 * j + 1] = bhS1M + bhS2M;
        cplx bhS = bhS1M - bhS2M;
        tmpp[(size_t)mc * N + 2 * j] = -CI * bhN;
        tmpp[(size_t)mc * N + 2 * j + 1] = -CI * bhS;
      }
    }
  }
  for (int mc = o->n_m_max; mc < nhp; ++mc)
    for (int t = 0; t < N; ++t) {
      tmpr[(size_t)mc * N + t] = 0.0; tmpt[(size_t)mc * N + t] = 0.0; tmpp[(size_t)mc * N + t] = 0.0;
    }
  ifft_many(o, tmpr.data(), brc);
  ifft_many(o, tmpt.data(), btc);
  ifft_many(o, tmpp.data(), bpc);
}

// native_sphtor_to_spat: src/shtransforms.f90:247-372.
static void native_sphtor_to_spat(const Oracle* o, const cplx* Slm, const cplx* Tlm,
                                  double* btc, double* bpc, int lcut) {
  const int N = o->n_theta, nhp = o->n_phi / 2 + 1, K = o->lm_max;
  std::vector<cplx> bhG(K), bhC(K);
  std::vector<cplx> tmpt((size_t)N * nhp), tmpp((size_t)N * nhp);
  for (int lm = 0; lm < K; ++lm) { bhG[lm] = Slm[lm] - CI * Tlm[lm]; bhC[lm] = Slm[lm] + CI * Tlm[lm]; }
#pragma omp parallel
  {
    std::vector<double> PlmG(K), PlmC(K);
    int s0, s1;
    omp_block(0, N / 2 - 1, s0, s1);
    for (int mc = 0; mc < o->n_m_max; ++mc) {
      const double dm = o->D_mc2m[mc];
      const int lmS = o->lStop[mc] - o->l_max + lcut;
      const bool l_Odd = ((lmS - o->lStart[mc]) % 2 == 0);
      const int m = mc * o->minc;
      if (m > lcut) {
        for (int j = s0; j <= s1; ++j)
          for (int r = 0; r < 2; ++r) {
            tmpt[(size_t)mc * N + 2 * j + r] = 0.0;
            tmpp[(size_t)mc * N + 2 * j + r] = 0.0;
          }
        continue;
      }
      for (int j = s0; j <= s1; ++j) {
        const double* P = &o->Plm[(size_t)j * K];
        const double* dP = &o->dPlm[(size_t)j * K];
        int lm;
        for (lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          PlmG[lm] = dP[lm] - dm * P[lm];
          PlmC[lm] = dP[lm] + dm * P[lm];
          PlmG[lm + 1] = dP[lm + 1] - dm * P[lm + 1];
          PlmC[lm + 1] = dP[lm + 1] + dm * P[lm + 1];
        }
        if (l_Odd) {
          PlmG[lmS] = dP[lmS] - dm * P[lmS];
          PlmC[lmS] = dP[lmS] + dm * P[lmS];
        }
        cplx bhN1 = 0.0, bhS1 = 0.0, bhN2 = 0.0, bhS2 = 0.0;
        for (lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          bhN1 = bhN1 + bhG[lm] * PlmG[lm] + bhG[lm + 1] * PlmG[lm + 1];
          bhS1 = bhS1 - bhG[lm] * PlmC[lm] + bhG[lm + 1] * PlmC[lm + 1];
          bhN2 = bhN2 + bhC[lm] * PlmC[lm] + bhC[lm + 1] * PlmC[lm + 1];
          bhS2 = bhS2 - bhC[lm] * PlmG[lm] + bhC[lm + 1] * PlmG[lm + 1];
        }
        if (l_Odd) {
          bhN1 = bhN1 + bhG[lmS] * PlmG[lmS];
          bhS1 = bhS1 - bhG[lmS] * PlmC[lmS];
          bhN2 = bhN2 + bhC[lmS] * PlmC[lmS];
          bhS2 = bhS2 - bhC[lmS] * PlmG[lmS];
        }
        cplx bhN1M = 0.5 * bhN1, bhS1M = 0.5 * bhS1, bhN2M = 0.5 * bhN2, bhS2M = 0.5 * bhS2;
        tmpt[(size_t)mc * N + 2 * j] = bhN1M + bhN2M;
        cplx bhN = bhN1M - bhN2M;
        tmpt[(size_t)mc * N + 2 * j + 1] = bhS1M + bhS2M;
        cplx bhS = bhS1M - bhS2M;
        tmpp[(size_t)mc * N + 2 * j] = -CI * bhN;
        tmpp[(size_t)mc * N + 2 * j + 1] = -CI * bhS;
      }
    }
  }
  for (int mc = o->n_m_max; mc < nhp; ++mc)
    for (int t = 0; t < N; ++t) { tmpt[(size_t)mc * N + t] = 0.0; tmpp[(size_t)mc * N + t] = 0.0; }
  ifft_many(o, tmpt.data(), btc);
  ifft_many(o, tmpp.data(), bpc);
}

// native_axi_to_spat: src/shtransforms.f90:374-403 (output sc(n_theta)).
static void native_axi_to_spat(const Oracle* o, const cplx* Slm, double* sc) {
  const int K = o->lm_max;
  for (int j = 0; j < o->n_theta / 2; ++j) {
    const double* P = &o->Plm[(size_t)j * K];
    cplx sES = 0.0, sEA = 0.0;
    const int lmS = o->lStop[0];
    for (int lm = o->lStart[0]; lm <= lmS - 1; lm += 2) {
      sES += Slm[lm] * P[lm];
      sEA += Slm[lm + 1] * P[lm + 1];
    }
    if (o->l_max % 2 == 0) sES += Slm[lmS] * P[lmS];
    sc[2 * j] = (sES + sEA).real();
    sc[2 * j + 1] = (sES - sEA).real();
  }
}

// native_toraxi_to_spat: src/shtransforms.f90:405-491.
static void native_toraxi_to_spat(const Oracle* o, const cplx* Tlm, double* btc, double* bpc,
                                  int lcut) {
  const int K = o->lm_max, L1 = o->l_max + 1;
  std::vector<cplx> bhG(L1), bhC(L1);
  for (int l = 0; l < L1; ++l) {
    if (l > lcut) { bhG[l] = 0.0; bhC[l] = 0.0; }
    else { bhG[l] = -CI * Tlm[l]; bhC[l] = CI * Tlm[l]; }
  }
  for (int j = 0; j < o->n_theta / 2; ++j) {
    const double* dP = &o->dPlm[(size_t)j * K];
    const int lmS = o->lStop[0];
    cplx bhN1 = 0.0, bhS1 = 0.0, bhN2 = 0.0, bhS2 = 0.0;
    for (int lm = o->lStart[0]; lm <= lmS - 1; lm += 2) {
      bhN1 = bhN1 + bhG[lm] * dP[lm] + bhG[lm + 1] * dP[lm + 1];
      bhS1 = bhS1 - bhG[lm] * dP[lm] + bhG[lm + 1] * dP[lm + 1];
      bhN2 = bhN2 + bhC[lm] * dP[lm] + bhC[lm + 1] * dP[lm + 1];
      bhS2 = bhS2 - bhC[lm] * dP[lm] + bhC[lm + 1] * dP[lm + 1];
    }
    if (o->l_max % 2 == 0) {
      bhN1 = bhN1 + bhG[lmS] * dP[lmS];
      bhS1 = bhS1 - bhG[lmS] * dP[lmS];
      bhN2 = bhN2 + bhC[lmS] * dP[lmS];
      bhS2 = bhS2 - bhC[lmS] * dP[lmS];
    }
    cplx bhN1M = 0.5 * bhN1, bhS1M = 0.5 * bhS1, bhN2M = 0.5 * bhN2, bhS2M = 0.5 * bhS2;
    btc[2 * j] = (bhN1M + bhN2M).real();
    cplx bhN = bhN1M - bhN2M;
    btc[2 * j + 1] = (bhS1M + bhS2M).real();
    cplx bhS = bhS1M - bhS2M;
    bpc[2 * j] = (-CI * bhN).real();
    bpc[2 * j + 1] = (-CI * bhS).real();
  }
}

// native_sph_to_spat: src/shtransforms.f90:493-561.
static void native_sph_to_spat(const Oracle* o, const cplx* Slm, double* sc, int lcut) {
  const int N = o->n_theta, nhp = o->n_phi / 2 + 1, K = o->lm_max;
  std::vector<cplx> tmp((size_t)N * nhp);
#pragma omp parallel
  {
    int s0, s1;
    omp_block(0, N / 2 - 1, s0, s1);
    for (int mc = 0; mc < o->n_m_max; ++mc) {
      const int m = mc * o->minc;
      const int lmS = o->lStop[mc] - o->l_max + lcut;
      const bool l_Odd = ((lmS - o->lStart[mc]) % 2 == 0);
      if (m > lcut) {
        for (int j = s0; j <= s1; ++j) { tmp[(size_t)mc * N + 2 * j] = 0.0; tmp[(size_t)mc * N + 2 * j + 1] = 0.0; }
        continue;
      }
      for (int j = s0; j <= s1; ++j) {
        const double* P = &o->Plm[(size_t)j * K];
        cplx sES = 0.0, sEA = 0.0;
        for (int lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          sES += Slm[lm] * P[lm];
          sEA += Slm[lm + 1] * P[lm + 1];
        }
        if (l_Odd) sES += Slm[lmS] * P[lmS];
        tmp[(size_t)mc * N + 2 * j] = sES + sEA;
        tmp[(size_t)mc * N + 2 * j + 1] = sES - sEA;
      }
    }
  }
  for (int mc = o->n_m_max; mc < nhp; ++mc)
    for (int t = 0; t < N; ++t) tmp[(size_t)mc * N + t] = 0.0;
  ifft_many(o, tmp.data(), sc);
}

// native_sph_to_grad_spat: src/shtransforms.f90:563-646.
static void native_sph_to_grad_spat(const Oracle* o, const cplx* Slm, double* gradtc,
                                    double* gradpc, int lcut) {
  const int N = o->n_theta, nhp = o->n_phi / 2 + 1, K = o->lm_max;
  std::vector<cplx> tmpt((size_t)N * nhp), tmpp((size_t)N * nhp);
#pragma omp parallel
  {
    int s0, s1;
    omp_block(0, N / 2 - 1, s0, s1);
    for (int mc = 0; mc < o->n_m_max; ++mc) {
      const double dm = o->D_mc2m[mc];
      const int lmS = o->lStop[mc] - o->l_max + lcut;
      const bool l_Odd = ((lmS - o->lStart[mc]) % 2 == 0);
      const int m = mc * o->minc;
      if (m > lcut) {
        for (int j = s0; j <= s1; ++j)
          for (int r = 0; r < 2; ++r) { tmpt[(size_t)mc * N + 2 * j + r] = 0.0; tmpp[(size_t)mc * N + 2 * j + r] = 0.0; }
        continue;
      }
      for (int j = s0; j <= s1; ++j) {
        const double* P = &o->Plm[(size_t)j * K];
        const double* dP = &o->dPlm[(size_t)j * K];
        cplx sES = 0.0, sEA = 0.0, gES = 0.0, gEA = 0.0;
        for (int lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          gEA = gEA + Slm[lm] * dP[lm];
          gES = gES + Slm[lm + 1] * dP[lm + 1];
          sES = sES + Slm[lm] * P[lm];
          sEA = sEA + Slm[lm + 1] * P[lm + 1];
        }
        if (l_Odd) {
          gEA = gEA + Slm[lmS] * dP[lmS];
          sES = sES + Slm[lmS] * P[lmS];
        }
        tmpt[(size_t)mc * N + 2 * j] = gES + gEA;
        tmpt[(size_t)mc * N + 2 * j + 1] = gES - gEA;
        tmpp[(size_t)mc * N + 2 * j] = dm * CI * (sES + sEA);
        tmpp[(size_t)mc * N + 2 * j + 1] = dm * CI * (sES - sEA);
      }
    }
  }
  for (int mc = o->n_m_max; mc < nhp; ++mc)
    for (int t = 0; t < N; ++t) { tmpt[(size_t)mc * N + t] = 0.0; tmpp[(size_t)mc * N + t] = 0.0; }
  ifft_many(o, tmpt.data(), gradtc);
  ifft_many(o, tmpp.data(), gradpc);
}

// native_spat_to_sph: src/shtransforms.f90:648-729.
static void native_spat_to_sph(const Oracle* o, const double* scal, cplx* f1LM, int lcut) {
  const int N = o->n_theta, nhp = o->n_phi / 2 + 1, K = o->lm_max, nmm = o->n_m_max;
  std::vector<cplx> f1TM((size_t)N * nhp);
  fft_many(o, scal, f1TM.data());
  for (int i = 0; i < K; ++i) f1LM[i] = 0.0;
  const int mlim = std::min(o->m_max, lcut);
#pragma omp parallel
  {
    std::vector<cplx> acc(K, cplx(0.0, 0.0));
    std::vector<cplx> f1ES((size_t)(N / 2) * nmm), f1EA((size_t)(N / 2) * nmm);
    int b0, b1;
    omp_block(0, N / 4 - 1, b0, b1);
    const int t1s = 2 * b0, t1e = 2 * b1 + 1;   // NHS thetas (0-based)
    for (int mc = 0; mc < nmm; ++mc) {
      const int lmS = o->lStop[mc] - o->l_max + lcut;
      const bool l_Odd = ((lmS - o->lStart[mc]) % 2 == 0);
      const int m = mc * o->minc;
      const bool zero = (m > mlim);
      for (int j = t1s; j <= t1e; ++j) {
        cplx fN = zero ? cplx(0.0) : f1TM[(size_t)mc * N + 2 * j];
        cplx fS = zero ? cplx(0.0) : f1TM[(size_t)mc * N + 2 * j + 1];
        f1ES[(size_t)mc * (N / 2) + j] = fN + fS;
        f1EA[(size_t)mc * (N / 2) + j] = fN - fS;
      }
      if (zero) continue;  // all terms below would add exact zeros
      for (int j1 = t1s; j1 <= t1e; j1 += 2) {
        const int j2 = j1 + 1;
        const cplx e1 = f1ES[(size_t)mc * (N / 2) + j1], e2 = f1ES[(size_t)mc * (N / 2) + j2];
        const cplx a1 = f1EA[(size_t)mc * (N / 2) + j1], a2 = f1EA[(size_t)mc * (N / 2) + j2];
        const double* w1 = &o->wPlm[(size_t)j1 * K];
        const double* w2 = &o->wPlm[(size_t)j2 * K];
        for (int lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          acc[lm] = acc[lm] + e1 * w1[lm] + e2 * w2[lm];
          acc[lm + 1] = acc[lm + 1] + a1 * w1[lm + 1] + a2 * w2[lm + 1];
        }
        if (l_Odd) acc[lmS] = acc[lmS] + e1 * w1[lmS] + e2 * w2[lmS];
      }
    }
#pragma omp critical
    for (int i = 0; i < K; ++i) f1LM[i] += acc[i];
  }
}

// native_spat_to_sph_tor: src/shtransforms.f90:731-872.
static void native_spat_to_sph_tor(const Oracle* o, const double* vt, const double* vp,
                                   cplx* f1LM, cplx* f2LM, int lcut) {
  const int N = o->n_theta, nhp = o->n_phi / 2 + 1, K = o->lm_max, nmm = o->n_m_max;
  std::vector<cplx> f1TM((size_t)N * nhp), f2TM((size_t)N * nhp);
  fft_many(o, vt, f2TM.data());   // the crossing of the reference (:764-767)
  fft_many(o, vp, f1TM.data());
  for (int i = 0; i < K; ++i) { f1LM[i] = 0.0; f2LM[i] = 0.0; }
  for (int mc = 0; mc < nhp; ++mc)
    for (int t = 0; t < N; ++t) {
      f1TM[(size_t)mc * N + t] *= o->O_sin_theta_E2[t];
      f2TM[(size_t)mc * N + t] *= o->O_sin_theta_E2[t];
    }
  const int mlim = std::min(o->m_max, lcut);
#pragma omp parallel
  {
    std::vector<cplx> acc1(K, cplx(0.0)), acc2(K, cplx(0.0));
    std::vector<cplx> f1ES((size_t)(N / 2) * nmm), f1EA((size_t)(N / 2) * nmm);
    std::vector<cplx> f2ES((size_t)(N / 2) * nmm), f2EA((size_t)(N / 2) * nmm);
    int b0, b1;
    omp_block(0, N / 4 - 1, b0, b1);
    const int t1s = 2 * b0, t1e = 2 * b1 + 1;
    for (int mc = 0; mc < nmm; ++mc) {
      const int lmS = o->lStop[mc] - o->l_max + lcut;
      const bool l_Odd = ((lmS - o->lStart[mc]) % 2 == 0);
      const double dm = o->D_mc2m[mc];
      const int m = mc * o->minc;
      const bool zero = (m > mlim);
      const size_t base = (size_t)mc * (N / 2);
      for (int j = t1s; j <= t1e; ++j) {
        cplx a = zero ? cplx(0.0) : f1TM[(size_t)mc * N + 2 * j];
        cplx b = zero ? cplx(0.0) : f1TM[(size_t)mc * N + 2 * j + 1];
        cplx c = zero ? cplx(0.0) : f2TM[(size_t)mc * N + 2 * j];
        cplx d = zero ? cplx(0.0) : f2TM[(size_t)mc * N + 2 * j + 1];
        f1ES[base + j] = a + b; f1EA[base + j] = a - b;
        f2ES[base + j] = c + d; f2EA[base + j] = c - d;
      }
      if (zero) continue;
      for (int j1 = t1s; j1 <= t1e; j1 += 2) {
        const int j2 = j1 + 1;
        const cplx f1ES1 = f1ES[base + j1], f1ES2 = f1ES[base + j2];
        const cplx f1EA1 = f1EA[base + j1], f1EA2 = f1EA[base + j2];
        const cplx f2ES1 = f2ES[base + j1], f2ES2 = f2ES[base + j2];
        const cplx f2EA1 = f2EA[base + j1], f2EA2 = f2EA[base + j2];
        const double* w1 = &o->wPlm[(size_t)j1 * K];
        const double* w2 = &o->wPlm[(size_t)j2 * K];
        const double* d1 = &o->wdPlm[(size_t)j1 * K];
        const double* d2 = &o->wdPlm[(size_t)j2 * K];
        const cplx cim = -CI * dm;
        for (int lm = o->lStart[mc]; lm <= lmS - 1; lm += 2) {
          acc1[lm] = acc1[lm] + cim * f1ES1 * w1[lm] + cim * f1ES2 * w2[lm] + f2EA1 * d1[lm] +
                     f2EA2 * d2[lm];
          acc1[lm + 1] = acc1[lm + 1] + cim * f1EA1 * w1[lm + 1] + cim * f1EA2 * w2[lm + 1] +
                         f2ES1 * d1[lm + 1] + f2ES2 * d2[lm + 1];
          acc2[lm] = acc2[lm] - f1EA1 * d1[lm] - f1EA2 * d2[lm] + cim * f2ES1 * w1[lm] +
                     cim * f2ES2 * w2[lm];
          acc2[lm + 1] = acc2[lm + 1] - f1ES1 * d1[lm + 1] - f1ES2 * d2[lm + 1] +
                         cim * f2EA1 * w1[lm + 1] + cim * f2EA2 * w2[lm + 1];
        }
        if (l_Odd) {
          acc1[lmS] = acc1[lmS] + cim * f1ES1 * w1[lmS] + cim * f1ES2 * w2[lmS] + f2EA1 * d1[lmS] +
                      f2EA2 * d2[lmS];
          acc2[lmS] = acc2[lmS] - f1EA1 * d1[lmS] - f1EA2 * d2[lmS] + cim * f2ES1 * w1[lmS] +
                      cim * f2ES2 * w2[lmS];
        }
      }
    }
#pragma omp critical
    for (int i = 0; i < K; ++i) { f1LM[i] += acc1[i]; f2LM[i] += acc2[i]; }
  }
  for (int lm = 1; lm < K; ++lm) {
    const int l = o->lm2l[lm];
    f1LM[lm] = f1LM[lm] / (double)(l * (l + 1));
    f2LM[lm] = f2LM[lm] / (double)(l * (l + 1));
  }
}

// ------------------------------------------------------- facade (sht) ------
// Public names of src/sht_native.f90:16-20 (prefixed).  Complex arrays are
// interleaved (re,im) doubles; grids are f[n_phi_max][n_theta].
extern "C" {

#define OR(h) ((const Oracle*)(h))
#define CP(x) ((const cplx*)(x))

void oracle_scal_to_spat(void* h, const double* Slm, double* f, int lcut) {  // :40-52
  native_sph_to_spat(OR(h), CP(Slm), f, lcut);
}
void oracle_scal_to_grad_spat(void* h, const double* Slm, double* gt, double* gp, int lcut) {  // :54-68
  native_sph_to_grad_spat(OR(h), CP(Slm), gt, gp, lcut);
}
void oracle_pol_to_grad_spat(void* h, const double* Slm, double* gt, double* gp, int lcut) {  // :70-97
  const Oracle* o = OR(h);
  std::vector<cplx> Q(o->lm_max);
  for (int lm = 0; lm < o->lm_max; ++lm)
    Q[lm] = (o->lm2l[lm] <= lcut) ? o->dLh[lm] * CP(Slm)[lm] : cplx(0.0);
  native_sph_to_grad_spat(o, Q.data(), gt, gp, lcut);
}
void oracle_torpol_to_spat(void* h, const double* W, const double* dW, const double* Z,
                           double* vr, double* vt, double* vp, int lcut) {  // :99-127
  const Oracle* o = OR(h);
  std::vector<cplx> Q(o->lm_max);
  for (int lm = 0; lm < o->lm_max; ++lm)
    Q[lm] = (o->lm2l[lm] <= lcut) ? o->dLh[lm] * CP(W)[lm] : cplx(0.0);
  native_qst_to_spat(o, Q.data(), CP(dW), CP(Z), vr, vt, vp, lcut);
}
void oracle_sphtor_to_spat(void* h, const double* dW, const double* Z, double* vt, double* vp,
                           int lcut) {  // :129-141
  native_sphtor_to_spat(OR(h), CP(dW), CP(Z), vt, vp, lcut);
}
void oracle_torpol_to_curl_spat_IC(void* h, double r, double r_ICB, const double* dB,
                                   const double* ddB, const double* J, const double* dJ,
                                   double* cbr, double* cbt, double* cbp) {  // :143-186
  const Oracle* o = OR(h);
  const int K = o->lm_max, L = o->l_max;
  std::vector<double> rDep(L + 1), rDep2(L + 1);
  const double rRatio = r / r_ICB;
  rDep[0] = rRatio; rDep2[0] = 1.0 / r_ICB;
  for (int l = 1; l <= L; ++l) { rDep[l] = rDep[l - 1] * rRatio; rDep2[l] = rDep2[l - 1] * rRatio; }
  std::vector<cplx> Q(K), S(K), T(K);
  for (int lm = 0; lm < K; ++lm) {
    const int l = o->lm2l[lm];
    Q[lm] = rDep[l] * o->dLh[lm] * CP(J)[lm];
    S[lm] = rDep2[l] * ((double)(l + 1) * CP(J)[lm] + r * CP(dJ)[lm]);
    T[lm] = -rDep2[l] * (2.0 * (double)(l + 1) * CP(dB)[lm] + r * CP(ddB)[lm]);
  }
  native_qst_to_spat(o, Q.data(), S.data(), T.data(), cbr, cbt, cbp, L);
}
void oracle_torpol_to_spat_IC(void* h, double r, double r_ICB, const double* W,
                              const double* dW, const double* Z, double* Br, double* Bt,
                              double* Bp) {  // :188-229
  const Oracle* o = OR(h);
  const int K = o->lm_max, L = o->l_max;
  std::vector<double> rDep(L + 1), rDep2(L + 1);
  const double rRatio = r / r_ICB;
  rDep[0] = rRatio; rDep2[0] = 1.0 / r_ICB;
  for (int l = 1; l <= L; ++l) { rDep[l] = rDep[l - 1] * rRatio; rDep2[l] = rDep2[l - 1] * rRatio; }
  std::vector<cplx> Q(K), S(K), T(K);
  for (int lm = 0; lm < K; ++lm) {
    const int l = o->lm2l[lm];
    Q[lm] = rDep[l] * o->dLh[lm] * CP(W)[lm];
    S[lm] = rDep2[l] * ((double)(l + 1) * CP(W)[lm] + r * CP(dW)[lm]);
    T[lm] = rDep[l] * CP(Z)[lm];
  }
  native_qst_to_spat(o, Q.data(), S.data(), T.data(), Br, Bt, Bp, L);
}
void oracle_torpol_to_dphspat(void* h, const double* dW, const double* Z, double* dvtdp,
                              double* dvpdp, int lcut) {  // :231-272
  const Oracle* o = OR(h);
  const int K = o->lm_max, N = o->n_theta, P = o->n_phi;
  std::vector<cplx> S(K), T(K);
  for (int lm = 0; lm < K; ++lm) {
    const double m = (double)o->lm2m[lm];
    if (o->lm2l[lm] <= lcut) { S[lm] = CI * m * CP(dW)[lm]; T[lm] = CI * m * CP(Z)[lm]; }
    else { S[lm] = 0.0; T[lm] = 0.0; }
  }
  native_sphtor_to_spat(o, S.data(), T.data(), dvtdp, dvpdp, lcut);
  for (int ip = 0; ip < P; ++ip)
    for (int t = 0; t < N; ++t) {
      dvtdp[(size_t)ip * N + t] *= o->O_sin_theta_E2[t];
      dvpdp[(size_t)ip * N + t] *= o->O_sin_theta_E2[t];
    }
}
void oracle_pol_to_curlr_spat(void* h, const double* Qlm, double* cvr, int lcut) {  // :274-300
  const Oracle* o = OR(h);
  std::vector<cplx> dQ(o->lm_max);
  for (int lm = 0; lm < o->lm_max; ++lm)
    dQ[lm] = (o->lm2l[lm] <= lcut) ? o->dLh[lm] * CP(Qlm)[lm] : cplx(0.0);
  native_sph_to_spat(o, dQ.data(), cvr, lcut);
}
void oracle_torpol_to_curl_spat(void* h, double or2, const double* B, const double* ddB,
                                const double* J, const double* dJ, double* cvr, double* cvt,
                                double* cvp, int lcut) {  // :302-336
  const Oracle* o = OR(h);
  std::vector<cplx> Q(o->lm_max), T(o->lm_max);
  for (int lm = 0; lm < o->lm_max; ++lm) {
    if (o->lm2l[lm] <= lcut) {
      Q[lm] = o->dLh[lm] * CP(J)[lm];
      T[lm] = or2 * o->dLh[lm] * CP(B)[lm] - CP(ddB)[lm];
    } else { Q[lm] = 0.0; T[lm] = 0.0; }
  }
  native_qst_to_spat(o, Q.data(), CP(dJ), T.data(), cvr, cvt, cvp, lcut);
}
void oracle_scal_to_SH(void* h, const double* f, double* fLM, int lcut) {  // :338-346
  native_spat_to_sph(OR(h), f, (cplx*)fLM, lcut);
}
void oracle_spat_to_qst(void* h, const double* f, const double* g, const double* hh,
                        double* qLM, double* sLM, double* tLM, int lcut) {  // :348-364
  native_spat_to_sph(OR(h), f, (cplx*)qLM, lcut);
  native_spat_to_sph_tor(OR(h), g, hh, (cplx*)sLM, (cplx*)tLM, lcut);
}
void oracle_spat_to_sphertor(void* h, const double* f, const double* g, double* fLM,
                             double* gLM, int lcut) {  // :366-379
  native_spat_to_sph_tor(OR(h), f, g, (cplx*)fLM, (cplx*)gLM, lcut);
}
void oracle_axi_to_spat(void* h, const double* fl_ax, double* f) {  // :381-391
  native_axi_to_spat(OR(h), CP(fl_ax), f);
}
void oracle_toraxi_to_spat(void* h, const double* fl_ax, double* ft, double* fp, int lcut) {  // :393-405
  native_toraxi_to_spat(OR(h), CP(fl_ax), ft, fp, lcut);
}

// Raw FFT conventions (for tests): c (n_phi/2+1 complex) <-> x (n_phi real).
void oracle_rfft_inverse(int P, const double* c, double* x) {
  RFFT f; f.init(P);
  std::vector<cplx> buf(P / 2), work(P / 2);
  f.inverse(CP(c), x, buf.data(), work.data());
}
void oracle_rfft_forward(int P, const double* x, double* c) {
  RFFT f; f.init(P);
  std::vector<cplx> buf(P / 2), work(P / 2);
  f.forward(x, (cplx*)c, buf.data(), work.data());
}

}  // extern "C"
