// Azimuthal real FFTs over phi, batched over theta rows, radial levels and
// fields.  Transform definition of MagIC's fft991 (src/fft.f90:262-268):
//   inverse (ifft_many, :211-252): x_j = sum_k c_k e^{+2 pi i j k / P},
//     hermitian extension, Im(c_0) and Im(c_{P/2}) ignored, unnormalised;
//   forward (fft_many, :164-209): c_k = (1/P) sum_j x_j e^{-2 pi i j k / P}.
// Grids are theta-fastest (P rows of ld doubles), as in the reference.
//
// A real FFT of length P runs as a complex FFT of length n = P/2 plus the
// usual even/odd pre/post-processing.  Fast path (n = 32*S, S in
// {1,2,3,4,5,6,8,10,12,16,20,24}): each warp owns one theta row; lane l holds
// z[S*l + q], q < S; a 32-point radix-2 DIF network runs across the lanes with
// warp shuffles, then the four-step twiddle, then a length-S FFT in registers
// (warp_fft).  Rows are staged through shared memory so that global loads and
// stores stay coalesced along theta.  Other sizes use a per-warp
// shared-memory Stockham FFT.
//
// Forward epilogue (fused): 1/sin^2 theta (spat_to_sph_tor,
// src/shtransforms.f90:789-794), the Gauss weight 2 pi w_j, and the
// north/south -> ES/EA combination (src/shtransforms.f90:704-709, :811-818).
#include <type_traits>
#include <vector>
#include "common.cuh"
#include "cplx.cuh"
#include "internal.h"

namespace {

// Twiddle table e^{+2 pi i k / P} in the working type of a transform.
template <typename T> struct Tw;
template <> struct Tw<float> { static __device__ __forceinline__ const float2* get(const ShtGeom& g) { return g.tw32; } };
template <> struct Tw<double> { static __device__ __forceinline__ const double2* get(const ShtGeom& g) { return g.tw64; } };
template <> struct Tw<dfl> {
  static __device__ __forceinline__ const dfl2* get(const ShtGeom& g) { return (const dfl2*)g.twdf; }
};

// The double-float rows of 24 points per lane fill 101.5 KB of shared memory
// per CTA: their twiddle tables (TwTab layout, 15.5 KB) are read from a copy
// in device memory (through L1) so that two CTAs fit on an SM.
template <typename T, int S> struct GlobalTw { static constexpr bool v = std::is_same<T, dfl>::value && S >= 24; };

// CTAs per SM of the fast path: FP32 three (two for the longest rows), FP64
// one, double-float two (its rows are twice the FP32 size, its arithmetic
// needs the latency hiding of a second CTA)
template <typename T, int S, int RT> struct FftOcc { static constexpr int v = S >= 20 ? 2 : 3; };
template <int S, int RT> struct FftOcc<double, S, RT> { static constexpr int v = 1; };
// double-float: the forward kernel at 12 points per lane and 8 rows runs three
// CTAs per SM (80 registers)
template <int S, int RT> struct FftOcc<dfl, S, RT> { static constexpr int v = (S == 12 && RT == 8) ? 3 : 2; };

// Half-spectrum entries of the double-float transforms may be held in FP64
// (FFT_HS_F64: the FP64 SIMT Legendre sums on either side); the other forms
// read and write their own type.
template <typename T2> __device__ __forceinline__ T2 ld_hs(const T2* p, bool) { return *p; }
template <> __device__ __forceinline__ dfl2 ld_hs<dfl2>(const dfl2* p, bool f64) {
  return f64 ? cvt2<dfl2>(*(const double2*)p) : *p;
}
template <typename T2> __device__ __forceinline__ void st_hs(T2* p, T2 v, bool) { *p = v; }
template <> __device__ __forceinline__ void st_hs<dfl2>(dfl2* p, dfl2 v, bool f64) {
  if (f64) {
    *(double2*)p = to_d2(v);
  } else {
    // normalized pairs: the tensor-core analysis scales its digits by max |hi|
    v.x = df_norm(v.x);
    v.y = df_norm(v.y);
    *p = v;
  }
}

template <typename T2, int R> struct Bfly;
template <typename T2> struct Bfly<T2, 2> {
  static __device__ __forceinline__ void run(T2* v, int) {
    const T2 a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  }
};
template <typename T2> struct Bfly<T2, 3> {
  static __device__ __forceinline__ void run(T2* v, int s) {
    typedef typename ScalarOf<T2>::t T;
    const T h = (T)0.5, r3 = (T)0.86602540378443864676372317075294;
    const T2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
    T2 m1; m1.x = v[0].x - h * t1.x; m1.y = v[0].y - h * t1.y;
    const T2 m2 = cscale(cmuli(t2, s), r3);
    v[0] = cadd(v[0], t1); v[1] = cadd(m1, m2); v[2] = csub(m1, m2);
  }
};
template <typename T2> struct Bfly<T2, 4> {
  static __device__ __forceinline__ void run(T2* v, int s) {
    const T2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    const T2 b0 = cadd(v[1], v[3]), b1 = cmuli(csub(v[1], v[3]), s);
    v[0] = cadd(a0, b0); v[2] = csub(a0, b0);
    v[1] = cadd(a1, b1); v[3] = csub(a1, b1);
  }
};
template <typename T2> struct Bfly<T2, 5> {
  static __device__ __forceinline__ void run(T2* v, int s) {
    typedef typename ScalarOf<T2>::t T;
    const T c1 = (T)0.30901699437494742410229341718282;    // cos(2pi/5)
    const T c2 = (T)-0.80901699437494742410229341718282;   // cos(4pi/5)
    const T s1 = (T)0.95105651629515357211643933337938;    // sin(2pi/5)
    const T s2 = (T)0.58778525229247312916870595463907;    // sin(4pi/5)
    const T2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    const T2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    T2 a1, a2, u1, u2;
    a1.x = v[0].x + c1 * t1.x + c2 * t2.x; a1.y = v[0].y + c1 * t1.y + c2 * t2.y;
    a2.x = v[0].x + c2 * t1.x + c1 * t2.x; a2.y = v[0].y + c2 * t1.y + c1 * t2.y;
    u1.x = s1 * t3.x + s2 * t4.x; u1.y = s1 * t3.y + s2 * t4.y;
    u2.x = s2 * t3.x - s1 * t4.x; u2.y = s2 * t3.y - s1 * t4.y;
    const T2 b1 = cmuli(u1, s), b2 = cmuli(u2, s);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a1, b1); v[4] = csub(a1, b1);
    v[2] = cadd(a2, b2); v[3] = csub(a2, b2);
  }
};

// twiddle e^{s 2 pi i e / P} from the table of e^{+2 pi i k / P}
template <typename T2>
__device__ __forceinline__ T2 twid(const T2* __restrict__ tw, int e, int s) {
  T2 w = tw[e];
  if (s < 0) w.y = -w.y;
  return w;
}

// One Stockham stage of radix R on a length-S register array.
template <typename T2, int S, int R, int Ns>
__device__ __forceinline__ void reg_stage(T2 (&a)[S], const T2* __restrict__ tw, int pstride, int s) {
  T2 b[S];
  constexpr int nR = S / R;
#pragma unroll
  for (int j = 0; j < nR; ++j) {
    const int k = j % Ns;
    T2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      v[q] = a[j + q * nR];
      const int e = (k * q * (S / (Ns * R))) % S;
      if (e != 0) v[q] = cmul(v[q], twid(tw, e * pstride, s));
    }
    Bfly<T2, R>::run(v, s);
    const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int p = 0; p < R; ++p) b[idxD + p * Ns] = v[p];
  }
#pragma unroll
  for (int i = 0; i < S; ++i) a[i] = b[i];
}

// root[e] = e^{+2 pi i e / S}
template <typename T2, int S>
__device__ __forceinline__ void reg_fft(T2 (&a)[S], const T2* __restrict__ tw, int s) {
  constexpr int ps = 1;
  if constexpr (S == 2) { reg_stage<T2, S, 2, 1>(a, tw, ps, s); }
  else if constexpr (S == 3) { reg_stage<T2, S, 3, 1>(a, tw, ps, s); }
  else if constexpr (S == 4) { reg_stage<T2, S, 4, 1>(a, tw, ps, s); }
  else if constexpr (S == 5) { reg_stage<T2, S, 5, 1>(a, tw, ps, s); }
  else if constexpr (S == 6) { reg_stage<T2, S, 2, 1>(a, tw, ps, s); reg_stage<T2, S, 3, 2>(a, tw, ps, s); }
  else if constexpr (S == 8) { reg_stage<T2, S, 4, 1>(a, tw, ps, s); reg_stage<T2, S, 2, 4>(a, tw, ps, s); }
  else if constexpr (S == 10) { reg_stage<T2, S, 2, 1>(a, tw, ps, s); reg_stage<T2, S, 5, 2>(a, tw, ps, s); }
  else if constexpr (S == 12) { reg_stage<T2, S, 4, 1>(a, tw, ps, s); reg_stage<T2, S, 3, 4>(a, tw, ps, s); }
  else if constexpr (S == 16) { reg_stage<T2, S, 4, 1>(a, tw, ps, s); reg_stage<T2, S, 4, 4>(a, tw, ps, s); }
  else if constexpr (S == 20) { reg_stage<T2, S, 4, 1>(a, tw, ps, s); reg_stage<T2, S, 5, 4>(a, tw, ps, s); }
  else if constexpr (S == 24) {
    reg_stage<T2, S, 4, 1>(a, tw, ps, s); reg_stage<T2, S, 2, 4>(a, tw, ps, s);
    reg_stage<T2, S, 3, 8>(a, tw, ps, s);
  }
}

// Complex FFT of length n = 32*S held by one warp, four-step with the
// 32-point radix-2 DIF across lanes first and the length-S DFT in registers
// last:  input a[q] = z[S*lane + q],  output a[k2] = Z[brev5(lane) + 32*k2]
// (brev5(hx_pos(lane)) in the half-exchange form of the double-float
// transforms).  Outputs of one register are therefore 32 consecutive indices
// across the warp, which keeps the shared-memory write-back free of bank
// conflicts.
__host__ __device__ __forceinline__ int brev5(int x) {
#ifdef __CUDA_ARCH__
  return __brev(x) >> 27;
#else
  return ((x & 1) << 4) | ((x & 2) << 2) | (x & 4) | ((x & 8) >> 2) | ((x & 16) >> 4);
#endif
}

// Twiddle tables of the fast path in shared memory, laid out so that every
// warp-wide read is either 32 consecutive entries (one per lane) or one entry
// for all lanes (P = 2n = 64 S):
//   lanew[st][l] = e^{+2 pi i (l mod d) / (2d)}, d = 16 >> st  (cross-lane stages, st < 4)
//   post[q][l]   = e^{+2 pi i q brev5(l) / n}                   (four-step twiddles, q < S)
//   root[e]      = e^{+2 pi i e / S}                            (register DFT, e < S)
//   lo[q]        = e^{+2 pi i q / P},  hi[j] = e^{+2 pi i j KS / P}  (real <-> half-length
//   complex twiddle e^{2 pi i k / P} as a per-thread factor times one of these)
template <int S>
struct TwTab {
  static constexpr int kLane = 0, kPost = 128, kRoot = 128 + 32 * S, kLo = kRoot + S, kHi = kLo + S;
  static constexpr int size = kHi + S + 1;
  // index into the table e^{+2 pi i k / P} (k < P) of entry i; KS = order stride of the forward epilogue
  static __host__ __device__ __forceinline__ int src(int i, int KS) {
    constexpr int P = 64 * S;
    if (i < kPost) {
      const int st = i >> 5, l = i & 31, d = 16 >> st;
      return (l & (d - 1)) * (P / (2 * d));
    }
    if (i < kRoot) {
      const int q = (i - kPost) >> 5, l = (i - kPost) & 31;
      return (2 * q * brev5(l)) % P;  // e^{2 pi i q k1 / n} = e^{2 pi i 2 q k1 / P}
    }
    if (i < kLo) return (i - kRoot) * (P / S);
    if (i < kHi) return i - kLo;
    const int j = i - kHi;
    return KS * j < P ? KS * j : 0;  // entries past P are never read
  }
};

// One cross-lane radix-2 DIF stage of distance d (d = 16, 8, 4, 2, 1).
template <typename T2, int S>
__device__ __forceinline__ void lane_stage(T2 (&a)[S], const T2* __restrict__ tab, int s, int d, int lane) {
  typedef TwTab<S> TT;
  typedef typename ScalarOf<T2>::t T;
  const bool up = (lane & d) != 0;
  const T sg = up ? (T)-1 : (T)1;
  T2 w;
  if (d > 1) {
    const int st = d == 16 ? 0 : d == 8 ? 1 : d == 4 ? 2 : 3;
    w = twid(tab + TT::kLane, st * 32 + lane, s);
    if (!up) { w.x = (T)1; w.y = (T)0; }
  }
#pragma unroll
  for (int q = 0; q < S; ++q) {
    const T2 b = shfl_xor2(a[q], d);
    T2 t;
    t.x = add_signed(sg, a[q].x, b.x);
    t.y = add_signed(sg, a[q].y, b.y);
    a[q] = d > 1 ? cmul(t, w) : t;
  }
}

// Double-float cross-lane stages as half exchanges (S even, H = S/2).  In the
// stage of lane bit d the lane with that bit clear combines the pairs held in
// its registers 0..H-1, its partner the pairs in H..S-1: each lane sends and
// receives H values instead of S and twiddles H differences instead of S
// values (half of which the full exchange multiplies by 1).  Sums go to
// register j, differences to j + H, so a stage swaps lane bit d with the
// register half: after the five stages lane bits 4..0 hold (q / H, l4, l3,
// l2, l1) of the DIF position l and of the register index q, the register
// half holds l0.  One more exchange across lane bit 16 gives every lane all S
// values of the position hx_pos(lane).  The upper lane of a pair forms
// own - received = -(lower - upper): its sign is folded into the twiddle.
// The d = 2 twiddles are 1 and s i, applied as a swap and signs.
__device__ __forceinline__ int hx_pos(int lane) { return ((lane & 15) << 1) | (lane >> 4); }
__device__ __forceinline__ dfl df_sgn(dfl a, float g) { return mkdf(a.h * g, a.l * g); }  // g = +-1: exact

template <int S>
__device__ __forceinline__ void warp_fft_hx(dfl2 (&a)[S], const dfl2* __restrict__ tab, int s, int lane) {
  typedef TwTab<S> TT;
  constexpr int H = S / 2;
#pragma unroll 1
  for (int d = 16; d >= 1; d >>= 1) {
    const bool up = (lane & d) != 0;
    const float g = up ? -1.f : 1.f;
    if (d >= 4) {
      const int st = d == 16 ? 0 : d == 8 ? 1 : 2;
      dfl2 w = twid(tab + TT::kLane, st * 32 + lane, s);
      w.x = df_sgn(w.x, g);
      w.y = df_sgn(w.y, g);
#pragma unroll
      for (int j = 0; j < H; ++j) {
        const dfl2 snd = up ? a[j] : a[j + H];
        const dfl2 own = up ? a[j + H] : a[j];
        const dfl2 rcv = shfl_xor2(snd, d);
        a[j] = cadd(own, rcv);
        a[j + H] = cmul(csub(own, rcv), w);
      }
    } else {
      // d = 2: t (g s i) on odd lanes = g s (-t.y, t.x), t g on even lanes; d = 1: t g
      const bool sw = d == 2 && (lane & 1);
      const float fx = sw ? -g * (float)s : g, fy = sw ? g * (float)s : g;
#pragma unroll
      for (int j = 0; j < H; ++j) {
        const dfl2 snd = up ? a[j] : a[j + H];
        const dfl2 own = up ? a[j + H] : a[j];
        const dfl2 rcv = shfl_xor2(snd, d);
        a[j] = cadd(own, rcv);
        const dfl2 t = csub(own, rcv);
        dfl2 r;
        r.x = df_sgn(sw ? t.y : t.x, fx);
        r.y = df_sgn(sw ? t.x : t.y, fy);
        a[j + H] = r;
      }
    }
  }
  // lane bit 16 <-> register half: the lower lane keeps l0 = 0, the upper l0 = 1
  const bool up4 = (lane & 16) != 0;
#pragma unroll
  for (int j = 0; j < H; ++j) {
    const dfl2 snd = up4 ? a[j] : a[j + H];
    const dfl2 rcv = shfl_xor2(snd, 16);
    a[j] = up4 ? rcv : a[j];
    a[j + H] = up4 ? a[j + H] : rcv;
  }
  const int pl = hx_pos(lane);
#pragma unroll
  for (int q = 1; q < S; ++q) a[q] = cmul(a[q], twid(tab + TT::kPost, q * 32 + pl, s));
  reg_fft<dfl2, S>(a, tab + TT::kRoot, s);
}

// DIF position held by a lane after warp_fft: output a[k2] = Z[brev5(pos) + 32 k2]
template <typename T2, int S>
__device__ __forceinline__ int fft_pos(int lane) {
  if constexpr (std::is_same<T2, dfl2>::value && S % 2 == 0) return hx_pos(lane);
  else return lane;
}

template <typename T2, int S>
__device__ __forceinline__ void warp_fft(T2 (&a)[S], const T2* __restrict__ tab, int s) {
  typedef TwTab<S> TT;
  const int lane = threadIdx.x & 31;
  if constexpr (std::is_same<T2, dfl2>::value && S % 2 == 0) {
    warp_fft_hx<S>(a, tab, s, lane);
    return;
  } else if constexpr (std::is_same<T2, dfl2>::value) {
    // double-float: the five cross-lane stages as a loop (the unrolled code
    // stalled on instruction fetch), then the same four-step twiddles and
    // register FFT
#pragma unroll 1
    for (int d = 16; d >= 1; d >>= 1) lane_stage<T2, S>(a, tab, s, d, lane);
#pragma unroll
    for (int q = 1; q < S; ++q) a[q] = cmul(a[q], twid(tab + TT::kPost, q * 32 + lane, s));
    reg_fft<T2, S>(a, tab + TT::kRoot, s);
    return;
  }
  typedef typename ScalarOf<T2>::t T;
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) {
    // lower lane: a + b;  upper lane: (b - a) * w  -> t = b + sg*a, a = t * w
    // (the last stage, d = 1, has w = 1 on every lane)
    const bool up = (lane & d) != 0;
    const T sg = up ? (T)-1 : (T)1;
    T2 w;
    if (d > 1) {
      const int st = d == 16 ? 0 : d == 8 ? 1 : d == 4 ? 2 : 3;
      w = twid(tab + TT::kLane, st * 32 + lane, s);
      if (!up) { w.x = (T)1; w.y = (T)0; }
    }
#pragma unroll
    for (int q = 0; q < S; ++q) {
      const T2 b = shfl_xor2(a[q], d);
      T2 t;
      t.x = add_signed(sg, a[q].x, b.x);
      t.y = add_signed(sg, a[q].y, b.y);
      a[q] = d > 1 ? cmul(t, w) : t;
    }
  }
#pragma unroll
  for (int q = 1; q < S; ++q) a[q] = cmul(a[q], twid(tab + TT::kPost, q * 32 + lane, s));  // omega_n^{q k1}
  reg_fft<T2, S>(a, tab + TT::kRoot, s);
}

// Shared-memory row layouts of the fast path (row pitch KP = 33 S + 1, odd):
// input position of index k (digit swap k = S*i1 + q -> 33 q + i1: the lanes
// of a half warp storing neighbouring k, or reading one q, hit distinct banks)
template <int S>
__device__ __forceinline__ int pin(int k) { return (k % S) * 33 + k / S; }
// output position of the natural index k = k1 + 32 k2 (k1 < 32): the
// bit-reversed lanes of a half warp write the even or the odd k1 of one
// block, which pos() spreads over distinct banks
__device__ __forceinline__ int pos(int k) { return (k & 31) + ((k >> 4) & 1) + 33 * (k >> 5); }

// ------------------------------------------------------------ fast path ----
// Stage-in of the inverse fast path: the spectra of RT theta rows into the
// pin() layout, and the twiddle table into shared memory.  All loads of a
// batch of NB orders (E at both parities, and F for vector fields), and of
// the twiddle table, are issued before the first shared-memory store, so that
// a thread waits for one memory latency per batch.
template <typename T2, int S, int RT, int NB, bool STAGE_TW>
__device__ __forceinline__ void inv_stage(const ShtGeom& g, const T2* __restrict__ in, bool in_parity,
                                          bool has_f, bool hs64, long long per_p, const T2* __restrict__ twg, T2* sm,
                                          T2* stw, int rp, int kq, int rowg, bool row_ok) {
  constexpr int KP = 33 * S + 1, KS = 256 / (RT / 2), NT = TwTab<S>::size, NTW = (NT + 255) / 256;
  const int n_m = g.n_m;
  T2 twr[NTW];
  if constexpr (STAGE_TW) {
#pragma unroll
    for (int i = 0; i < NTW; ++i)
      if (threadIdx.x + 256 * i < NT) twr[i] = twg[TwTab<S>::src(threadIdx.x + 256 * i, KS)];
  }
  for (int kb = 0; kb < n_m; kb += KS * NB) {
    T2 x[NB][4];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int k = kb + kq + KS * b;
#pragma unroll
      for (int j = 0; j < 4; ++j) x[b][j] = zero2<T2>();
      if (row_ok && k < n_m) {
        if (in_parity) {
          const T2* b0 = in + (long long)k * 2 * per_p + (rowg >> 1);
          x[b][0] = ld_hs(b0, hs64);
          x[b][1] = ld_hs(b0 + per_p, hs64);
          if (has_f) {
            x[b][2] = ld_hs(b0 + g.nh, hs64);
            x[b][3] = ld_hs(b0 + per_p + g.nh, hs64);
          }
        } else {
          const T2* p = in + (long long)k * g.n_theta + rowg;
          x[b][0] = ld_hs(p, hs64);
          x[b][1] = ld_hs(p + 1, hs64);
        }
      }
    }
    if (STAGE_TW && kb == 0) {  // n_m >= 1: the first batch always runs
#pragma unroll
      for (int i = 0; i < NTW; ++i)
        if (threadIdx.x + 256 * i < NT) stw[threadIdx.x + 256 * i] = twr[i];
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int k = kb + kq + KS * b;
      if (k >= n_m) continue;
      T2 v0 = x[b][0], v1 = x[b][1];
      if (in_parity) {  // rows 2j, 2j + 1: north = ES + EA, south = ES - EA
        v0 = cadd(x[b][0], x[b][1]);
        v1 = has_f ? csub(x[b][2], x[b][3]) : csub(x[b][0], x[b][1]);
      }
      sm[rp * KP + pin<S>(k)] = v0;
      sm[(rp + 1) * KP + pin<S>(k)] = v1;
    }
  }
}

// One CTA = RT consecutive theta rows of one (level, field) column; 8 warps,
// each owning RT/8 rows in turn.  FP32: three CTAs per SM (80 registers per
// thread); four CTAs at 64 registers measured 14% slower (inverse) and 3%
// (forward).  Shared memory holds the RT rows with an
// odd pitch KP = 33 S + 1 and the layouts pin() / pos(), so that row-parallel
// and index-parallel accesses both spread over the banks.
template <typename T, int S, int RT>
__global__ void __launch_bounds__(256, FftOcc<T, S, RT>::v) fft_inv_fast(const ShtGeom g, const FftSet s) {
  typedef typename V2<T>::t T2;
  constexpr int n = 32 * S, KP = 33 * S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* sm = (T2*)smem_raw;
  const int col = blockIdx.y;
  const int r = col / s.nf, f = col - r * s.nf;
  const FftField& fd = s.f[f];
  const int row0 = blockIdx.x * RT;
  const T2* __restrict__ twg = Tw<T>::get(g);
  T2* stw = sm + RT * KP;  // twiddle tables (TwTab), or their copy in device memory
  const T2* tab = GlobalTw<T, S>::v ? (const T2*)g.twr : stw;
  const T2* __restrict__ in = (const T2*)fd.in + (long long)r * fd.in_ld;
  const int n_m = g.n_m;
  const bool in_parity = (fd.flags & (FFT_IN_E | FFT_IN_EF)) != 0;
  const bool has_f = (fd.flags & FFT_IN_EF) != 0;
  const long long per_p = has_f ? 2LL * g.nh : (long long)g.nh;
  // Each thread owns the row pair (rp, rp + 1) (16 B for FP32 half spectra;
  // n_theta is even) and the orders k = kq + KS j.
  constexpr int RT2 = RT / 2, KS = 256 / RT2;
  const int rp = 2 * (threadIdx.x % RT2), kq = threadIdx.x / RT2;
  const int rowg = row0 + rp;
  const bool row_ok = rowg < g.n_theta;
  const bool hs64 = (fd.flags & FFT_HS_F64) != 0;
  inv_stage<T2, S, RT, sizeof(T) == 4 ? 4 : 2, !GlobalTw<T, S>::v>(g, in, in_parity, has_f, hs64, per_p, twg, sm,
                                                                   stw, rp, kq, rowg, row_ok);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T2 base = twg[S * lane];  // e^{2 pi i S lane / P}: times lo[q] gives e^{2 pi i k / P}, k = S lane + q
  T2 wq[S];  // the same for both rows of the warp
#pragma unroll
  for (int q = 0; q < S; ++q) wq[q] = q == 0 ? base : cmul(base, tab[TwTab<S>::kLo + q]);
  for (int rr = warp; rr < RT; rr += 8) {
    T2* row = sm + rr * KP;
    T2 a[S];
#pragma unroll
    for (int q = 0; q < S; ++q) {
      // k = S*lane + q sits at pin(k) = 33q + lane; n - k at 33(S-q) + 31 - lane
      // (q > 0) or 32 - lane (q = 0; k = 0 has no partner)
      const int k = S * lane + q;
      T2 ck = zero2<T2>(), cn = zero2<T2>();
      if (k < n_m) ck = row[33 * q + lane];
      const int kn = n - k;
      if (kn < n_m) cn = row[q == 0 ? 32 - lane : 33 * (S - q) + 31 - lane];
      if (k == 0) { ck.y = 0; cn.y = 0; }
      const T2 E = cadd(ck, cconj(cn));
      const T2 O = cmul(csub(ck, cconj(cn)), wq[q]);
      a[q].x = E.x - O.y;
      a[q].y = E.y + O.x;
    }
    __syncwarp();
    warp_fft<T2, S>(a, tab, +1);
    const int k1 = brev5(fft_pos<T2, S>(lane));
#pragma unroll
    for (int k2 = 0; k2 < S; ++k2) row[pos(k1 + 32 * k2)] = a[k2];  // z_j = x_{2j} + i x_{2j+1}
    __syncwarp();
  }
  __syncthreads();
  double* out = (double*)fd.out + (long long)r * fd.out_ld;
  const bool vec = (g.ld % 2) == 0;  // 16-byte stores of two rows need an even pitch
  if (!row_ok) return;
  // the row pair (rp, rp + 1) of this thread shares theta_j, j = rowg / 2
  const T o = (fd.flags & FFT_OSIN2) ? from_f64<T>(g.osin2[rowg >> 1]) : (T)1;
#pragma unroll (sizeof(T) == 4 ? 4 : 2)
  const T2* s0 = sm + rp * KP + pos(kq);  // pos(kk + 32 j) = pos(kk) + 33 j
  const long long dstep = 2LL * KS * g.ld;
  double* dst = out + (long long)(2 * kq) * g.ld + rowg;
  for (int kk = kq; kk < n; kk += KS, s0 += 33 * (KS / 32), dst += dstep) {
    T2 v0 = s0[0], v1 = s0[KP];  // phi = 2kk (x) and 2kk+1 (y) of rows rp, rp + 1
    if constexpr (std::is_same<T, dfl>::value) {
      // a double-float product costs ~10 FP32 operations: only the 1/sin^2 fields pay it
      if (fd.flags & FFT_OSIN2) {
        v0 = cscale(v0, o);
        v1 = cscale(v1, o);
      }
    } else {
      v0 = cscale(v0, o);
      v1 = cscale(v1, o);
    }
    // row rp widens on the FP64 pipe (idle in this kernel), row rp + 1 with
    // integer instructions: splitting the conversions between the two pipes
    // measured faster than either alone.  Both are exact; FP32 subnormals
    // (below 1.2e-38) are kept by the first and flushed to zero by the second.
    double x0, y0;
    if constexpr (std::is_same<T, dfl>::value) {
      x0 = to_f64<T>(v0.x);
      y0 = to_f64<T>(v0.y);
    } else {
      x0 = (double)v0.x;
      y0 = (double)v0.y;
    }
    if (vec) {
      *reinterpret_cast<double2*>(dst) = make_double2(x0, to_f64<T>(v1.x));
      *reinterpret_cast<double2*>(dst + g.ld) = make_double2(y0, to_f64<T>(v1.y));
    } else {
      dst[0] = x0;
      dst[1] = to_f64<T>(v1.x);
      dst[g.ld] = y0;
      dst[g.ld + 1] = to_f64<T>(v1.y);
    }
  }
}

template <typename T, int S, int RT>
__global__ void __launch_bounds__(256, FftOcc<T, S, RT>::v) fft_fwd_fast(const ShtGeom g, const FftSet s) {
  typedef typename V2<T>::t T2;
  constexpr int n = 32 * S, KP = 33 * S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* sm = (T2*)smem_raw;
  const int col = blockIdx.y;
  const int r = col / s.nf, f = col - r * s.nf;
  const FftField& fd = s.f[f];
  const int row0 = blockIdx.x * RT;
  const T2* __restrict__ twg = Tw<T>::get(g);
  T2* stw = sm + RT * KP;  // twiddle tables (TwTab), or their copy in device memory
  constexpr bool kStage = !GlobalTw<T, S>::v;
  const T2* tab = kStage ? stw : (const T2*)g.twr;
  const double* __restrict__ in = (const double*)fd.in + (long long)r * fd.in_ld;
  // Each thread owns the row pair (rp, rp + 1) and the indices kk = kq + KS j
  // (phi = 2kk, 2kk + 1); the loads of a batch of NB indices, and of the
  // twiddle tables, are all issued before the first shared-memory store.
  constexpr int RT2 = RT / 2, KS = 256 / RT2, NB = 6, NT = TwTab<S>::size, NTW = (NT + 255) / 256;
  const int rp = 2 * (threadIdx.x % RT2), kq = threadIdx.x / RT2;
  const int rowg = row0 + rp;
  const bool row_ok = rowg < g.n_theta;
  const bool vec = (g.ld % 2) == 0;
  T2 twr[NTW];
  if constexpr (kStage) {
#pragma unroll
    for (int i = 0; i < NTW; ++i)
      if (threadIdx.x + 256 * i < NT) twr[i] = twg[TwTab<S>::src(threadIdx.x + 256 * i, KS)];
  }
  for (int kb = 0; kb < n; kb += KS * NB) {
    double2 u[NB], w[NB];  // (row rp | rp+1) at phi 2kk (u) and 2kk+1 (w)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int kk = kb + kq + KS * b;
      u[b] = w[b] = make_double2(0.0, 0.0);
      if (row_ok && kk < n) {
        const double* src = in + (long long)(2 * kk) * g.ld + rowg;
        if (vec) {
          u[b] = *reinterpret_cast<const double2*>(src);
          w[b] = *reinterpret_cast<const double2*>(src + g.ld);
        } else {
          u[b] = make_double2(src[0], src[1]);
          w[b] = make_double2(src[g.ld], src[g.ld + 1]);
        }
      }
    }
    if (kStage && kb == 0) {
#pragma unroll
      for (int i = 0; i < NTW; ++i)
        if (threadIdx.x + 256 * i < NT) stw[threadIdx.x + 256 * i] = twr[i];
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int kk = kb + kq + KS * b;
      if (kk >= n) continue;
      const int pj = pin<S>(kk);
      T2 z0, z1;
      z0.x = cvt_in<T>(u[b].x); z0.y = cvt_in<T>(w[b].x);
      z1.x = cvt_in<T>(u[b].y); z1.y = cvt_in<T>(w[b].y);
      sm[rp * KP + pj] = z0;
      sm[(rp + 1) * KP + pj] = z1;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int rr = warp; rr < RT; rr += 8) {
    T2* row = sm + rr * KP;
    T2 a[S];
#pragma unroll
    for (int q = 0; q < S; ++q) a[q] = row[q * 33 + lane];  // = z[S*lane + q]
    __syncwarp();
    warp_fft<T2, S>(a, tab, -1);
    const int k1 = brev5(fft_pos<T2, S>(lane));
#pragma unroll
    for (int k2 = 0; k2 < S; ++k2) row[pos(k1 + 32 * k2)] = a[k2];
    __syncwarp();
  }
  __syncthreads();
  // X_k = (Z_k + conj Z_{n-k})/2 - i e^{-2 pi i k/P} (Z_k - conj Z_{n-k})/2, then ES/EA
  typedef T Tt;
  T2* out = (T2*)fd.out + (long long)r * fd.out_ld;
  const bool hs64 = (fd.flags & FFT_HS_F64) != 0;
  // this thread's colatitude pair jp (rows 2jp, 2jp + 1) and orders k = kq + KS j
  const int jp = threadIdx.x % RT2, jg = (row0 >> 1) + jp;
  if (jg >= g.nh) return;
  Tt fac = (Tt)(1.0 / (double)g.n_phi);
  if (fd.flags & FFT_OSIN2) fac *= from_f64<Tt>(g.osin2[jg]);
  if (fd.flags & FFT_WEIGHT) fac *= from_f64<Tt>(g.wgt[jg]);
  const T2 base = twg[kq];  // e^{2 pi i kq / P}: times hi[j] gives e^{2 pi i k / P}, k = kq + KS j
  for (int k = kq, j = 0; k < g.n_m; k += KS, ++j) {
    const T2 tk = j == 0 ? base : cmul(base, tab[TwTab<S>::kHi + j]);
    T2 c[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const T2* row = sm + (2 * jp + h) * KP;
      const T2 Zk = row[pos(k)];
      const T2 Zn = cconj(row[pos(k == 0 ? 0 : n - k)]);
      const T2 D = csub(Zk, Zn);
      const T2 u = cmul(cconj(tk), D);
      T2 X;
      X.x = (Tt)0.5 * (Zk.x + Zn.x + u.y);
      X.y = (Tt)0.5 * (Zk.y + Zn.y - u.x);
      if (k == 0) X.y = 0;
      c[h] = X;
    }
    c[0] = cscale(c[0], fac);
    c[1] = cscale(c[1], fac);
    const long long o = ((long long)k * g.nh + jg) * 2;
    st_hs(out + o, cadd(c[0], c[1]), hs64);
    st_hs(out + o + 1, csub(c[0], c[1]), hs64);
  }
}

// ---------------------------------------------------- shared staging code ----
template <typename T2>
__device__ __forceinline__ void stage_spectrum(const ShtGeom& g, const T2* __restrict__ in,
                                               int row0, int RT, int RP, T2* sm, int flags) {
  const bool in_parity = (flags & (FFT_IN_E | FFT_IN_EF)) != 0;
  const bool has_f = (flags & FFT_IN_EF) != 0;
  const bool hs64 = (flags & FFT_HS_F64) != 0;
  const long long per_p = has_f ? 2LL * g.nh : (long long)g.nh;
  for (int i = threadIdx.x; i < g.n_m * RT; i += blockDim.x) {
    const int k = i / RT, rr = i - k * RT;
    const int row = row0 + rr;
    T2 v = zero2<T2>();
    if (row < g.n_theta) {
      if (in_parity) {
        const int jg = row >> 1;
        const T2* b0 = in + (long long)k * 2 * per_p;
        const T2* b1 = b0 + per_p;
        if ((row & 1) == 0) v = cadd(ld_hs(b0 + jg, hs64), ld_hs(b1 + jg, hs64));
        else v = has_f ? csub(ld_hs(b0 + g.nh + jg, hs64), ld_hs(b1 + g.nh + jg, hs64))
                       : csub(ld_hs(b0 + jg, hs64), ld_hs(b1 + jg, hs64));
      } else {
        v = ld_hs(in + (long long)k * g.n_theta + row, hs64);
      }
    }
    sm[k * RP + rr] = v;
  }
}

// Z_k = E_k + i O_k for the half-length complex inverse (k = 32q + lane)
template <typename T2>
__device__ __forceinline__ T2 inv_pre(const ShtGeom& g, const T2* sm, int RP, int rr, int k, int n,
                                      const T2* __restrict__ tw) {
  T2 ck = zero2<T2>(), cn = zero2<T2>();
  if (k < g.n_m) ck = sm[k * RP + rr];
  const int kn = n - k;
  if (kn < g.n_m) cn = sm[kn * RP + rr];
  if (k == 0) { ck.y = 0; cn.y = 0; }
  const T2 E = cadd(ck, cconj(cn));
  const T2 O = cmul(csub(ck, cconj(cn)), tw[k]);
  T2 z; z.x = E.x - O.y; z.y = E.y + O.x;
  return z;
}

template <typename T2>
__device__ __forceinline__ void store_grid(const ShtGeom& g, const FftField& fd, double* out,
                                           int row0, int RT, int RP, const T2* sm) {
  for (int i = threadIdx.x; i < g.n_phi * RT; i += blockDim.x) {
    const int ph = i / RT, rr = i - ph * RT;
    const int row = row0 + rr;
    if (row >= g.n_theta) continue;
    typedef typename ScalarOf<T2>::t T;
    const T2 v = sm[(ph >> 1) * RP + rr];
    T x = (ph & 1) ? v.y : v.x;
    if (fd.flags & FFT_OSIN2) x *= from_f64<T>(g.osin2[row >> 1]);
    out[(long long)ph * g.ld + row] = to_f64<T>(x);
  }
}

template <typename T2>
__device__ __forceinline__ void stage_grid(const ShtGeom& g, const double* __restrict__ in, int row0,
                                           int RT, int RP, T2* sm) {
  typedef typename ScalarOf<T2>::t T;
  T* smr = (T*)sm;
  for (int i = threadIdx.x; i < g.n_phi * RT; i += blockDim.x) {
    const int ph = i / RT, rr = i - ph * RT;
    const int row = row0 + rr;
    double x = 0.0;
    if (row < g.n_theta) x = in[(long long)ph * g.ld + row];
    smr[((ph >> 1) * RP + rr) * 2 + (ph & 1)] = cvt_in<T>(x);
  }
}

// X_k from the half-length forward spectrum Z (in smem), then ES/EA output.
template <typename T2>
__device__ __forceinline__ void fwd_post(const ShtGeom& g, const FftField& fd, T2* out, int row0,
                                         int RT, int RP, const T2* sm, const T2* __restrict__ tw) {
  typedef typename ScalarOf<T2>::t T;
  const int n = g.n_phi / 2;
  const T scale = (T)(1.0 / (double)g.n_phi);
  const int npair = RT / 2;
  for (int i = threadIdx.x; i < g.n_m * npair; i += blockDim.x) {
    const int k = i / npair, jp = i - k * npair;
    const int jg = (row0 >> 1) + jp;
    if (jg >= g.nh) continue;
    T2 c[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int rr = 2 * jp + h;
      const T2 Zk = sm[k * RP + rr];
      const T2 Zn = cconj(sm[((n - k) % n) * RP + rr]);
      const T2 D = csub(Zk, Zn);
      const T2 u = cmul(cconj(tw[k]), D);
      T2 X;
      X.x = (T)0.5 * (Zk.x + Zn.x + u.y);
      X.y = (T)0.5 * (Zk.y + Zn.y - u.x);
      X.x *= scale; X.y *= scale;
      if (k == 0) X.y = 0;
      c[h] = X;
    }
    T fac = 1;
    if (fd.flags & FFT_OSIN2) fac *= from_f64<T>(g.osin2[jg]);
    if (fd.flags & FFT_WEIGHT) fac *= from_f64<T>(g.wgt[jg]);
    c[0] = cscale(c[0], fac); c[1] = cscale(c[1], fac);
    const long long o = ((long long)k * g.nh + jg) * 2;
    const bool hs64 = (fd.flags & FFT_HS_F64) != 0;
    st_hs(out + o, cadd(c[0], c[1]), hs64);
    st_hs(out + o + 1, csub(c[0], c[1]), hs64);
  }
}

// ------------------------------------------------------- general sizes ----
struct Radices { int n; int r[24]; };

template <typename T2>
__device__ void warp_stockham(T2* src, T2* dst, int n, const Radices& rad, const T2* __restrict__ tw,
                              int P, int s) {
  // result ends in `src` (buffers swapped internally an even/odd number of times)
  const int lane = threadIdx.x & 31;
  int Ns = 1;
  T2* a = src;
  T2* b = dst;
  for (int st = 0; st < rad.n; ++st) {
    const int R = rad.r[st];
    const int nR = n / R;
    const int tstride = n / (Ns * R);
    for (int j = lane; j < nR; j += 32) {
      const int k = j % Ns;
      T2 v[5];
      for (int q = 0; q < R; ++q) {
        v[q] = a[j + q * nR];
        const int e = (k * q * tstride) % n;
        if (e) v[q] = cmul(v[q], twid(tw, 2 * e, s));
      }
      if (R == 2) Bfly<T2, 2>::run(v, s);
      else if (R == 3) Bfly<T2, 3>::run(v, s);
      else if (R == 4) Bfly<T2, 4>::run(v, s);
      else Bfly<T2, 5>::run(v, s);
      const int idxD = (j / Ns) * Ns * R + k;
      for (int p = 0; p < R; ++p) b[idxD + p * Ns] = v[p];
    }
    __syncwarp();
    T2* t = a; a = b; b = t;
    Ns *= R;
  }
  if (a != src) {
    for (int i = lane; i < n; i += 32) src[i] = a[i];
    __syncwarp();
  }
}

template <typename T>
__global__ void __launch_bounds__(256) fft_inv_gen(const ShtGeom g, const FftSet s, const Radices rad) {
  typedef typename V2<T>::t T2;
  constexpr int RT = 8, RP = RT + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* sm = (T2*)smem_raw;
  const int n = g.n_phi / 2;
  const int nstage = (g.n_m > n ? g.n_m : n) * RP;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T2* wa = sm + nstage + warp * 2 * n;
  T2* wb = wa + n;
  const int col = blockIdx.y;
  const int r = col / s.nf, f = col - r * s.nf;
  const FftField& fd = s.f[f];
  const int row0 = blockIdx.x * RT;
  const T2* __restrict__ tw = Tw<T>::get(g);
  stage_spectrum<T2>(g, (const T2*)fd.in + (long long)r * fd.in_ld, row0, RT, RP, sm, fd.flags);
  __syncthreads();
  for (int k = lane; k < n; k += 32) wa[k] = inv_pre<T2>(g, sm, RP, warp, k, n, tw);
  __syncwarp();
  warp_stockham<T2>(wa, wb, n, rad, tw, g.n_phi, +1);
  __syncthreads();
  for (int k = lane; k < n; k += 32) sm[k * RP + warp] = wa[k];
  __syncthreads();
  store_grid<T2>(g, fd, (double*)fd.out + (long long)r * fd.out_ld, row0, RT, RP, sm);
}

template <typename T>
__global__ void __launch_bounds__(256) fft_fwd_gen(const ShtGeom g, const FftSet s, const Radices rad) {
  typedef typename V2<T>::t T2;
  constexpr int RT = 8, RP = RT + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T2* sm = (T2*)smem_raw;
  const int n = g.n_phi / 2;
  const int nstage = (g.n_m > n ? g.n_m : n) * RP;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T2* wa = sm + nstage + warp * 2 * n;
  T2* wb = wa + n;
  const int col = blockIdx.y;
  const int r = col / s.nf, f = col - r * s.nf;
  const FftField& fd = s.f[f];
  const int row0 = blockIdx.x * RT;
  const T2* __restrict__ tw = Tw<T>::get(g);
  stage_grid<T2>(g, (const double*)fd.in + (long long)r * fd.in_ld, row0, RT, RP, sm);
  __syncthreads();
  for (int k = lane; k < n; k += 32) wa[k] = sm[k * RP + warp];
  __syncwarp();
  warp_stockham<T2>(wa, wb, n, rad, tw, g.n_phi, -1);
  __syncthreads();
  for (int k = lane; k < n; k += 32) sm[k * RP + warp] = wa[k];
  __syncthreads();
  fwd_post<T2>(g, fd, (T2*)fd.out + (long long)r * fd.out_ld, row0, RT, RP, sm, tw);
}

bool factorize(int n, Radices& rad) {
  rad.n = 0;
  while (n % 4 == 0 && rad.n < 24) { rad.r[rad.n++] = 4; n /= 4; }
  while (n % 2 == 0 && rad.n < 24) { rad.r[rad.n++] = 2; n /= 2; }
  while (n % 3 == 0 && rad.n < 24) { rad.r[rad.n++] = 3; n /= 3; }
  while (n % 5 == 0 && rad.n < 24) { rad.r[rad.n++] = 5; n /= 5; }
  return n == 1;
}

template <typename T, int S, int RT>
cudaError_t launch_rt(const ShtGeom& g, const FftSet& s, bool inverse, cudaStream_t st) {
  typedef typename V2<T>::t T2;
  constexpr int KP = 33 * S + 1;
  // the device-memory tables are built for 8-row CTAs (fft_df_global_twiddles)
  static_assert(!GlobalTw<T, S>::v || (RT == 8 && S == 24), "device-memory twiddle tables: S = 24, 8 rows");
  const size_t smem = ((size_t)RT * KP + (GlobalTw<T, S>::v ? 0 : TwTab<S>::size)) * sizeof(T2);
  dim3 grid((g.n_theta + RT - 1) / RT, s.nf * s.nlev);
  auto k = inverse ? fft_inv_fast<T, S, RT> : fft_fwd_fast<T, S, RT>;
  CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k<<<grid, 256, smem, st>>>(g, s);
  return cudaGetLastError();
}

// rows: theta rows per CTA, 8 or 16 (FP32; the FP64 kernels keep the size
// rule), 0 = 16, or 8 where 16 would leave one CTA per SM
template <typename T, int S>
cudaError_t launch_fast(const ShtGeom& g, const FftSet& s, bool inverse, int rows, cudaStream_t st) {
  typedef typename V2<T>::t T2;
  constexpr int KP = 33 * S + 1;
  constexpr int RT = (sizeof(T2) * 16 * KP > 100 * 1024) ? 8 : 16;
  if constexpr (sizeof(T) == 4) {
    if (rows == 8) return launch_rt<T, S, 8>(g, s, inverse, st);
    if (rows == 16) return launch_rt<T, S, 16>(g, s, inverse, st);
  }
  // double-float forward at 12 points per lane: 8 rows, three CTAs per SM
  // (3.76 -> 3.64 ms for the 10 analysis grids of 129 levels at n_phi = 768;
  // the inverse stays at 16 rows, 4.90 against 5.28 ms at 8)
  if constexpr (std::is_same<T, dfl>::value && S == 12)
    if (!inverse) return launch_rt<T, S, 8>(g, s, inverse, st);
  return launch_rt<T, S, RT>(g, s, inverse, st);
}

template <typename T>
cudaError_t launch_gen(const ShtGeom& g, const FftSet& s, bool inverse, cudaStream_t st) {
  typedef typename V2<T>::t T2;
  const int n = g.n_phi / 2;
  Radices rad;
  if (!factorize(n, rad)) return cudaErrorInvalidValue;
  const size_t smem = ((size_t)(g.n_m > n ? g.n_m : n) * 9 + (size_t)8 * 2 * n) * sizeof(T2);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  dim3 grid((g.n_theta + 7) / 8, s.nf * s.nlev);
  if (inverse) {
    CUDA_TRY(cudaFuncSetAttribute(fft_inv_gen<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fft_inv_gen<T><<<grid, 256, smem, st>>>(g, s, rad);
  } else {
    CUDA_TRY(cudaFuncSetAttribute(fft_fwd_gen<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fft_fwd_gen<T><<<grid, 256, smem, st>>>(g, s, rad);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_any(const ShtGeom& g, const FftSet& s, bool inverse, int rows, cudaStream_t st) {
  if (s.nf * s.nlev <= 0) return cudaSuccess;
  const int n = g.n_phi / 2;
  if (n % 32 == 0) {
    switch (n / 32) {
      case 1: return launch_fast<T, 1>(g, s, inverse, rows, st);
      case 2: return launch_fast<T, 2>(g, s, inverse, rows, st);
      case 3: return launch_fast<T, 3>(g, s, inverse, rows, st);
      case 4: return launch_fast<T, 4>(g, s, inverse, rows, st);
      case 5: return launch_fast<T, 5>(g, s, inverse, rows, st);
      case 6: return launch_fast<T, 6>(g, s, inverse, rows, st);
      case 8: return launch_fast<T, 8>(g, s, inverse, rows, st);
      case 10: return launch_fast<T, 10>(g, s, inverse, rows, st);
      case 12: return launch_fast<T, 12>(g, s, inverse, rows, st);
      case 16: return launch_fast<T, 16>(g, s, inverse, rows, st);
      case 20: return launch_fast<T, 20>(g, s, inverse, rows, st);
      case 24: return launch_fast<T, 24>(g, s, inverse, rows, st);
      default: break;
    }
  }
  return launch_gen<T>(g, s, inverse, st);
}

}  // namespace

// The twiddle tables the double-float fast path reads from device memory
// (GlobalTw): TwTab<24> at the order stride of 8-row CTAs, from the
// double-float table e^{+2 pi i k / P}; empty for the other lengths.
std::vector<float4> fft_df_global_twiddles(int n_phi, const std::vector<float4>& twdf) {
  std::vector<float4> out;
  if (n_phi != 64 * 24 || (int)twdf.size() != n_phi) return out;
  typedef TwTab<24> TT;
  constexpr int KS = 256 / (8 / 2);
  out.resize(TT::size);
  for (int i = 0; i < TT::size; ++i) out[i] = twdf[TT::src(i, KS)];
  return out;
}

bool fft_fast_path(int n_phi) {
  const int n = n_phi / 2;
  if (n % 32) return false;
  switch (n / 32) {
    case 1: case 2: case 3: case 4: case 5: case 6: case 8: case 10: case 12: case 16:
    case 20: case 24: return true;
    default: return false;
  }
}

cudaError_t launch_fft_inverse(const ShtGeom& g, const FftSet& s, int arith, int rows, cudaStream_t st) {
  if (arith == FFT_ARITH_DF) return launch_any<dfl>(g, s, true, rows, st);
  return arith == FFT_ARITH_F64 ? launch_any<double>(g, s, true, rows, st) : launch_any<float>(g, s, true, rows, st);
}

cudaError_t launch_fft_forward(const ShtGeom& g, const FftSet& s, int arith, int rows, cudaStream_t st) {
  if (arith == FFT_ARITH_DF) return launch_any<dfl>(g, s, false, rows, st);
  return arith == FFT_ARITH_F64 ? launch_any<double>(g, s, false, rows, st) : launch_any<float>(g, s, false, rows, st);
}
