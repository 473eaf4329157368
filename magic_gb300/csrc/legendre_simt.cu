// Legendre sums over the triangular (l,m) layout on the SIMT pipes.
//
// FP64 instantiation: the parity ("plain") form of the native transforms
//   native_sph_to_spat / native_qst_to_spat / native_sphtor_to_spat /
//   native_sph_to_grad_spat   (src/shtransforms.f90:103-372, :493-646)
//   native_spat_to_sph / native_spat_to_sph_tor  (src/shtransforms.f90:648-872)
// FP32 instantiation: the same sums with FP32 tables and accumulators.
//
// Both directions are per-m dense contractions, batched over many columns
// (radial level x field):
//   synthesis  t(theta_j, m)[c] = sum_l P(l,m,theta_j) X(l,m)[c]
//   analysis   f(l, m)[c]       = sum_j P(l,m,theta_j) F(theta_j, m)[c]
// and use the equatorial symmetry of P (even/odd l-m) so that only the
// northern colatitudes are contracted (ES/EA split of the reference).
//
// CTA tile: 8 warps; lanes run along theta (synthesis) or l (analysis), the
// warps split into TW "tile" warps x CW "column" warps, each thread holds TC
// columns in registers.  The table tile and the spectral/half-spectrum tile
// are staged through shared memory; spectral operands are pre-scaled while
// staged (dLh, curl and i*m combinations of src/sht_native.f90).
#include "common.cuh"
#include "cplx.cuh"
#include "internal.h"

namespace {

constexpr int LC = 32;  // l chunk of the synthesis (even: keeps the parity aligned)

__device__ __forceinline__ double2 load_operand(const SpecOperand& o, int r, int lm, int l, int m,
                                                double or2) {
  if (o.op == OP_ZERO || o.A == nullptr) return make_double2(0.0, 0.0);
  const long long base = (long long)r * o.ld + lm;
  double2 a = o.A[base];
  switch (o.op) {
    case OP_COPY: return a;
    case OP_DLH: {
      const double d = (double)(l * (l + 1));
      return make_double2(d * a.x, d * a.y);
    }
    case OP_CURLT: {
      const double2 b = o.B[base];
      const double d = or2 * (double)(l * (l + 1));
      return make_double2(d * a.x - b.x, d * a.y - b.y);
    }
    case OP_IM: {
      const double dm = (double)m;
      return make_double2(-dm * a.y, dm * a.x);
    }
    default: return make_double2(0.0, 0.0);
  }
}

// ---------------------------------------------------------------- synthesis
template <typename T, bool VEC, int TW, int CW, int TC>
__global__ void __launch_bounds__(256) inv_legendre_kernel(const ShtGeom g, const InvSet s) {
  typedef typename V2<T>::t T2;
  constexpr int TJ = TW * 32;   // theta points per CTA
  constexpr int CC = CW * TC;   // columns per CTA
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // layout (see inv_smem_bytes): Xs, Ys (T2) | s_or2 (double) | Ps, dPs (T) | s_lcut (int)
  T2 (*Xs)[CC] = reinterpret_cast<T2 (*)[CC]>(smem_raw);
  T2 (*Ys)[CC] = reinterpret_cast<T2 (*)[CC]>(smem_raw + sizeof(T2) * LC * CC);
  double* s_or2 = reinterpret_cast<double*>(smem_raw + sizeof(T2) * LC * CC * (VEC ? 2 : 1));
  T (*Ps)[TJ] = reinterpret_cast<T (*)[TJ]>(reinterpret_cast<unsigned char*>(s_or2) + sizeof(double) * CC);
  T (*dPs)[TJ] = reinterpret_cast<T (*)[TJ]>(reinterpret_cast<unsigned char*>(Ps) + sizeof(T) * LC * TJ);
  int* s_lcut = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(Ps) + sizeof(T) * LC * TJ * (VEC ? 2 : 1));

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wj = warp % TW, wc = warp / TW;
  const int mc = blockIdx.x;
  const int m = mc * g.minc;
  const int n_l = g.l_max - m + 1;
  const int lm0 = g.lmoff[mc];
  const int jt0 = blockIdx.z * TJ;
  if (jt0 >= g.nh) return;
  const int j = jt0 + wj * 32 + lane;
  const int ncol = s.nf * s.nlev;
  const int colbase = blockIdx.y * CC;
  const T* __restrict__ Ptab = sizeof(T) == 8 ? (const T*)g.P64 : (const T*)g.P32;
  const T* __restrict__ dPtab = sizeof(T) == 8 ? (const T*)g.dP64 : (const T*)g.dP32;

  if (threadIdx.x < CC) {
    const int c = colbase + threadIdx.x;
    int lc = -1;
    double o2 = 0.0;
    if (c < ncol) {
      const int r = c / s.nf;
      lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
      o2 = s.or2 ? s.or2[r] : s.or2_0;
    }
    s_lcut[threadIdx.x] = lc;
    s_or2[threadIdx.x] = o2;
  }

  T2 ae[TC], ao[TC];
  T2 be[VEC ? TC : 1], bo[VEC ? TC : 1], ce[VEC ? TC : 1], co[VEC ? TC : 1],
      de[VEC ? TC : 1], dO[VEC ? TC : 1];
#pragma unroll
  for (int q = 0; q < TC; ++q) {
    ae[q] = zero2<T2>(); ao[q] = zero2<T2>();
    if (VEC) { be[q] = zero2<T2>(); bo[q] = zero2<T2>(); ce[q] = zero2<T2>();
               co[q] = zero2<T2>(); de[q] = zero2<T2>(); dO[q] = zero2<T2>(); }
  }
  __syncthreads();

  for (int l0 = 0; l0 < n_l; l0 += LC) {
    // table tile: rows l0..l0+LC-1 of this m block, theta jt0..jt0+TJ-1
    for (int i = threadIdx.x; i < LC * TJ; i += blockDim.x) {
      const int li = i / TJ, jj = i - li * TJ;
      const int jg = jt0 + jj;
      T pv = 0, dv = 0;
      if (l0 + li < n_l && jg < g.nh) {
        const size_t idx = (size_t)(lm0 + l0 + li) * g.nh + jg;
        pv = Ptab[idx];
        if (VEC) dv = dPtab[idx];
      }
      Ps[li][jj] = pv;
      if (VEC) dPs[li][jj] = dv;
    }
    // spectral tile: each thread walks one column along l
    for (int i = threadIdx.x; i < LC * CC; i += blockDim.x) {
      const int cc = i % CC, li = i / CC;
      const int c = colbase + cc;
      const int l = m + l0 + li;
      double2 x = make_double2(0.0, 0.0), y = make_double2(0.0, 0.0);
      if (c < ncol && l0 + li < n_l && l <= s_lcut[cc]) {
        const int r = c / s.nf, f = c - r * s.nf;
        x = load_operand(s.f[f].x0, r, lm0 + l0 + li, l, m, s_or2[cc]);
        if (VEC) y = load_operand(s.f[f].x1, r, lm0 + l0 + li, l, m, s_or2[cc]);
      }
      Xs[li][cc] = cvt2<T2>(x);
      if (VEC) Ys[li][cc] = cvt2<T2>(y);
    }
    __syncthreads();
    const int lmax_chunk = min(LC, n_l - l0);
#pragma unroll 2
    for (int i = 0; i < lmax_chunk; i += 2) {
      const T pe = Ps[i][wj * 32 + lane];
      const T po = Ps[i + 1][wj * 32 + lane];
      T dpe = 0, dpo = 0;
      if (VEC) { dpe = dPs[i][wj * 32 + lane]; dpo = dPs[i + 1][wj * 32 + lane]; }
#pragma unroll
      for (int q = 0; q < TC; ++q) {
        const int cc = wc * TC + q;
        const T2 xe = Xs[i][cc], xo = Xs[i + 1][cc];
        if (!VEC) {
          ae[q].x += pe * xe.x; ae[q].y += pe * xe.y;
          ao[q].x += po * xo.x; ao[q].y += po * xo.y;
        } else {
          const T2 ye = Ys[i][cc], yo = Ys[i + 1][cc];
          // A = sum S dP, B = sum T P, C = sum S P, D = sum T dP
          ae[q].x += dpe * xe.x; ae[q].y += dpe * xe.y;
          ao[q].x += dpo * xo.x; ao[q].y += dpo * xo.y;
          be[q].x += pe * ye.x;  be[q].y += pe * ye.y;
          bo[q].x += po * yo.x;  bo[q].y += po * yo.y;
          ce[q].x += pe * xe.x;  ce[q].y += pe * xe.y;
          co[q].x += po * xo.x;  co[q].y += po * xo.y;
          de[q].x += dpe * ye.x; de[q].y += dpe * ye.y;
          dO[q].x += dpo * yo.x; dO[q].y += dpo * yo.y;
        }
      }
    }
    __syncthreads();
  }

  if (j >= g.nh) return;
  const T dm = (T)m;
#pragma unroll
  for (int q = 0; q < TC; ++q) {
    const int cc = wc * TC + q;
    const int c = colbase + cc;
    if (c >= ncol) continue;
    const int r = c / s.nf, f = c - r * s.nf;
    const long long o = (long long)r * s.f[f].out_ld + (long long)mc * g.n_theta + 2 * j;
    T2* out0 = (T2*)s.f[f].out0;
    if (!VEC) {
      out0[o] = cadd(ae[q], ao[q]);
      out0[o + 1] = csub(ae[q], ao[q]);
    } else {
      T2* out1 = (T2*)s.f[f].out1;
      // north: vt = (A_e+A_o) + i m (B_e+B_o);  vp = i m (C_e+C_o) - (D_e+D_o)
      // south: vt = (A_o-A_e) + i m (B_e-B_o);  vp = i m (C_e-C_o) + (D_e-D_o)
      const T2 bN = cadd(be[q], bo[q]), bS = csub(be[q], bo[q]);
      const T2 cN = cadd(ce[q], co[q]), cS = csub(ce[q], co[q]);
      T2 vtN, vtS, vpN, vpS;
      vtN.x = ae[q].x + ao[q].x - dm * bN.y;  vtN.y = ae[q].y + ao[q].y + dm * bN.x;
      vtS.x = ao[q].x - ae[q].x - dm * bS.y;  vtS.y = ao[q].y - ae[q].y + dm * bS.x;
      vpN.x = -dm * cN.y - (de[q].x + dO[q].x); vpN.y = dm * cN.x - (de[q].y + dO[q].y);
      vpS.x = -dm * cS.y + (de[q].x - dO[q].x); vpS.y = dm * cS.x + (de[q].y - dO[q].y);
      out0[o] = vtN; out0[o + 1] = vtS;
      out1[o] = vpN; out1[o + 1] = vpS;
    }
  }
}

// ----------------------------------------------------------------- analysis
template <typename T, bool VEC, int LW, int CW, int TC, int JC>
__global__ void __launch_bounds__(256) fwd_legendre_kernel(const ShtGeom g, const FwdSet s) {
  typedef typename V2<T>::t T2;
  constexpr int TLL = LW * 32;  // l values per CTA
  constexpr int CC = CW * TC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // layout (see fwd_smem_bytes): F1s, F2s (T2) | Pt, dPt (T)
  T2 (*F1s)[JC][2] = reinterpret_cast<T2 (*)[JC][2]>(smem_raw);
  T2 (*F2s)[JC][2] = reinterpret_cast<T2 (*)[JC][2]>(smem_raw + sizeof(T2) * CC * JC * 2);
  T (*Pt)[TLL + 1] = reinterpret_cast<T (*)[TLL + 1]>(smem_raw + sizeof(T2) * CC * JC * 2 * (VEC ? 2 : 1));
  T (*dPt)[TLL + 1] = reinterpret_cast<T (*)[TLL + 1]>(reinterpret_cast<unsigned char*>(Pt) + sizeof(T) * JC * (TLL + 1));

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wl = warp % LW, wc = warp / LW;
  const int mc = blockIdx.x;
  const int m = mc * g.minc;
  const int n_l = g.l_max - m + 1;
  const int lt0 = blockIdx.z * TLL;
  if (lt0 >= n_l) return;
  const int lm0 = g.lmoff[mc];
  const int loff = lt0 + wl * 32 + lane;  // l - m
  const int par = loff & 1;
  const int ncol = s.nf * s.nlev;
  const int colbase = blockIdx.y * CC;
  const T* __restrict__ Ptab = sizeof(T) == 8 ? (const T*)g.P64 : (const T*)g.P32;
  const T* __restrict__ dPtab = sizeof(T) == 8 ? (const T*)g.dP64 : (const T*)g.dP32;

  T2 A[TC], B[VEC ? TC : 1], C[VEC ? TC : 1], D[VEC ? TC : 1];
#pragma unroll
  for (int q = 0; q < TC; ++q) {
    A[q] = zero2<T2>();
    if (VEC) { B[q] = zero2<T2>(); C[q] = zero2<T2>(); D[q] = zero2<T2>(); }
  }

  for (int j0 = 0; j0 < g.nh; j0 += JC) {
    // table tile, transposed to [j][l]
    for (int i = threadIdx.x; i < JC * TLL; i += blockDim.x) {
      const int li = i / JC, jj = i - li * JC;
      T pv = 0, dv = 0;
      if (lt0 + li < n_l && j0 + jj < g.nh) {
        const size_t idx = (size_t)(lm0 + lt0 + li) * g.nh + j0 + jj;
        pv = Ptab[idx];
        if (VEC) dv = dPtab[idx];
      }
      Pt[jj][li] = pv;
      if (VEC) dPt[jj][li] = dv;
    }
    // half-spectrum tile (ES/EA pairs)
    for (int i = threadIdx.x; i < CC * JC * 2; i += blockDim.x) {
      const int cc = i / (JC * 2), rem = i - cc * (JC * 2);
      const int jj = rem >> 1, e = rem & 1;
      const int c = colbase + cc;
      T2 v1 = zero2<T2>(), v2 = zero2<T2>();
      if (c < ncol && j0 + jj < g.nh) {
        const int r = c / s.nf, f = c - r * s.nf;
        const long long o = (long long)r * s.f[f].in_ld +
                            ((long long)mc * g.nh + j0 + jj) * 2 + e;
        v1 = ((const T2*)s.f[f].in0)[o];
        if (VEC) v2 = ((const T2*)s.f[f].in1)[o];
      }
      F1s[cc][jj][e] = v1;
      if (VEC) F2s[cc][jj][e] = v2;
    }
    __syncthreads();
    const int jmax = min(JC, g.nh - j0);
#pragma unroll 4
    for (int jj = 0; jj < jmax; ++jj) {
      const T p = Pt[jj][wl * 32 + lane];
      T d = 0;
      if (VEC) d = dPt[jj][wl * 32 + lane];
#pragma unroll
      for (int q = 0; q < TC; ++q) {
        const int cc = wc * TC + q;
        const T2 f1m = F1s[cc][jj][par];
        if (!VEC) {
          A[q].x += p * f1m.x; A[q].y += p * f1m.y;
        } else {
          const T2 f1o = F1s[cc][jj][par ^ 1];
          const T2 f2m = F2s[cc][jj][par];
          const T2 f2o = F2s[cc][jj][par ^ 1];
          A[q].x += p * f1m.x; A[q].y += p * f1m.y;   // sum F1_mine  P
          B[q].x += d * f2o.x; B[q].y += d * f2o.y;   // sum F2_other dP
          C[q].x += d * f1o.x; C[q].y += d * f1o.y;   // sum F1_other dP
          D[q].x += p * f2m.x; D[q].y += p * f2m.y;   // sum F2_mine  P
        }
      }
    }
    __syncthreads();
  }

  if (loff >= n_l) return;
  const int l = m + loff;
  const double dm = (double)m;
#pragma unroll
  for (int q = 0; q < TC; ++q) {
    const int c = colbase + wc * TC + q;
    if (c >= ncol) continue;
    const int r = c / s.nf, f = c - r * s.nf;
    const int lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
    const bool keep = (l <= lc);
    const long long o = (long long)r * s.f[f].out_ld + lm0 + loff;
    if (!VEC) {
      s.f[f].out0[o] = keep ? to_d2(A[q]) : make_double2(0.0, 0.0);
    } else {
      // S = (-i m A + B) / (l(l+1)),  T = (-C - i m D) / (l(l+1))   (l>0)
      const double2 a = to_d2(A[q]), b = to_d2(B[q]), cc2 = to_d2(C[q]), dd = to_d2(D[q]);
      double2 Sv = make_double2(dm * a.y + b.x, -dm * a.x + b.y);
      double2 Tv = make_double2(-cc2.x + dm * dd.y, -cc2.y - dm * dd.x);
      if (l > 0) {
        const double inv = 1.0 / (double)(l * (l + 1));
        Sv.x *= inv; Sv.y *= inv; Tv.x *= inv; Tv.y *= inv;
      }
      s.f[f].out0[o] = keep ? Sv : make_double2(0.0, 0.0);
      s.f[f].out1[o] = keep ? Tv : make_double2(0.0, 0.0);
    }
  }
}

template <typename T, bool VEC, int TW, int CW, int TC>
constexpr size_t inv_smem_bytes() {
  typedef typename V2<T>::t T2;
  return sizeof(T2) * LC * CW * TC * (VEC ? 2 : 1) + sizeof(double) * CW * TC +
         sizeof(T) * LC * TW * 32 * (VEC ? 2 : 1) + sizeof(int) * CW * TC;
}

template <typename T, bool VEC, int LW, int CW, int TC, int JC>
constexpr size_t fwd_smem_bytes() {
  typedef typename V2<T>::t T2;
  return sizeof(T2) * CW * TC * JC * 2 * (VEC ? 2 : 1) + sizeof(T) * JC * (LW * 32 + 1) * (VEC ? 2 : 1);
}

template <typename T, bool VEC, int TW, int CW, int TC>
cudaError_t launch_inv_cfg(const ShtGeom& g, const InvSet& s, cudaStream_t st) {
  const int ncol = s.nf * s.nlev;
  constexpr int CC = CW * TC;
  constexpr size_t smem = inv_smem_bytes<T, VEC, TW, CW, TC>();
  static_assert(smem <= 227 * 1024, "shared memory");
  auto k = inv_legendre_kernel<T, VEC, TW, CW, TC>;
  CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(g.n_m, (ncol + CC - 1) / CC, (g.nh + TW * 32 - 1) / (TW * 32));
  k<<<grid, 256, smem, st>>>(g, s);
  return cudaGetLastError();
}

template <typename T, bool VEC, int LW, int CW, int TC, int JC>
cudaError_t launch_fwd_cfg(const ShtGeom& g, const FwdSet& s, cudaStream_t st) {
  const int ncol = s.nf * s.nlev;
  constexpr int CC = CW * TC;
  constexpr size_t smem = fwd_smem_bytes<T, VEC, LW, CW, TC, JC>();
  static_assert(smem <= 227 * 1024, "shared memory");
  auto k = fwd_legendre_kernel<T, VEC, LW, CW, TC, JC>;
  CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(g.n_m, (ncol + CC - 1) / CC, (g.l_max + 1 + LW * 32 - 1) / (LW * 32));
  k<<<grid, 256, smem, st>>>(g, s);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_inv_t(const ShtGeom& g, const InvSet& s, bool vec, cudaStream_t st) {
  const int ncol = s.nf * s.nlev;
  if (ncol <= 0) return cudaSuccess;
  if (!vec) {
    if (ncol >= 256) return launch_inv_cfg<T, false, 1, 8, 8>(g, s, st);
    if (ncol >= 8) return launch_inv_cfg<T, false, 2, 4, 2>(g, s, st);
    return launch_inv_cfg<T, false, 8, 1, 1>(g, s, st);
  } else {
    if (ncol >= 64) return launch_inv_cfg<T, true, 1, 8, 2>(g, s, st);
    if (ncol >= 4) return launch_inv_cfg<T, true, 2, 4, 1>(g, s, st);
    return launch_inv_cfg<T, true, 8, 1, 1>(g, s, st);
  }
}

template <typename T>
cudaError_t launch_fwd_t(const ShtGeom& g, const FwdSet& s, bool vec, cudaStream_t st) {
  const int ncol = s.nf * s.nlev;
  if (ncol <= 0) return cudaSuccess;
  if (!vec) {
    if (ncol >= 128) return launch_fwd_cfg<T, false, 1, 8, 4, 32>(g, s, st);
    if (ncol >= 8) return launch_fwd_cfg<T, false, 2, 4, 2, 32>(g, s, st);
    return launch_fwd_cfg<T, false, 8, 1, 1, 32>(g, s, st);
  } else {
    if (ncol >= 64) return launch_fwd_cfg<T, true, 1, 8, 2, 16>(g, s, st);
    if (ncol >= 4) return launch_fwd_cfg<T, true, 2, 4, 1, 16>(g, s, st);
    return launch_fwd_cfg<T, true, 8, 1, 1, 16>(g, s, st);
  }
}

}  // namespace

cudaError_t launch_inv_legendre_simt(const ShtGeom& g, const InvSet& s, bool vec, bool fp64,
                                     cudaStream_t st) {
  return fp64 ? launch_inv_t<double>(g, s, vec, st) : launch_inv_t<float>(g, s, vec, st);
}

cudaError_t launch_fwd_legendre_simt(const ShtGeom& g, const FwdSet& s, bool vec, bool fp64,
                                     cudaStream_t st) {
  return fp64 ? launch_fwd_t<double>(g, s, vec, st) : launch_fwd_t<float>(g, s, vec, st);
}
