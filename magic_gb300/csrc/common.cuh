// Shared device/host definitions for the GB300 spherical-harmonic transform
// library (libmagic_sht).  Everything here is internal; the public C ABI is
// include/magic_sht.h.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#define MAGIC_MAX_FIELDS 16

// Pre-scaling applied to a spectral operand while it is staged into shared
// memory (the O(lm_max) loops of src/sht_native.f90:84-93, 114-123,
// 249-260, 287-296, 320-330 fused into the Legendre prologue).
enum SpecOp : int {
  OP_ZERO = 0,   // X = 0
  OP_COPY = 1,   // X = A
  OP_DLH = 2,    // X = l(l+1) A                      (dLh, horizontal.f90:216)
  OP_CURLT = 3,  // X = or2(level) l(l+1) A - B       (torpol_to_curl_spat T)
  OP_IM = 4,     // X = i m A                         (torpol_to_dphspat)
};

// One spectral operand: X = op(A, B), level stride `ld` (complex elements).
struct SpecOperand {
  const double2* A;
  const double2* B;
  long long ld;
  int op;
  int pad_;
};

// Legendre synthesis field (spectral -> (theta,m) half spectrum).
//   SCALAR: out0 = sum_l P X0
//   VECTOR: (S=X0, T=X1) -> out0 = v_theta, out1 = v_phi (Robert form)
struct InvField {
  SpecOperand x0, x1;
  void* out0;  // T2 [n_m][n_theta] per level
  void* out1;
  long long out_ld;  // complex elements between levels
};

struct InvSet {
  InvField f[MAGIC_MAX_FIELDS];
  int nf;
  int nlev;
  const int* lcut;    // device [nlev] or null (then lcut0 for every level)
  const double* or2;  // device [nlev] or null (then or2_0; only OP_CURLT uses it)
  int lcut0;
  int pad_;
  double or2_0;
};

// Legendre analysis field ((theta,m) ES/EA half spectrum -> spectral).
//   SCALAR: out0(l,m) = sum_j F_{mine}(j) P(l,m,j)
//   VECTOR: in0 = F1 (from v_phi), in1 = F2 (from v_theta) -> out0 = S, out1 = T
struct FwdField {
  const void* in0;  // T2 [n_m][n_theta/2][2] per level (ES, EA pairs), weighted
  const void* in1;
  long long in_ld;   // complex elements between levels
  double2* out0;     // complex128 [lm_max] per level
  double2* out1;
  long long out_ld;  // complex elements between levels
};

struct FwdSet {
  FwdField f[MAGIC_MAX_FIELDS];
  int nf;
  int nlev;
  const int* lcut;    // device [nlev] or null (then lcut0)
  int lcut0;
  int pad_;
};

// Azimuthal FFT field.
enum FftFlags : int {
  FFT_OSIN2 = 1,    // inverse: multiply grid rows by 1/sin^2 theta (dphspat)
                    // forward: multiply spectrum rows by 1/sin^2 theta (sphtor)
  FFT_WEIGHT = 2,   // forward: multiply by 2 pi w_j (Gauss weight) for the Legendre sums
  // inverse input in the parity-separated layout of the tensor-core synthesis:
  // per m, parity p = 0,1: E_p[nh] (and F_p[nh] with FFT_IN_EF); rows are
  // N = E_0 + E_1, S = F_0 - F_1 (F = E with FFT_IN_E)
  FFT_IN_E = 4,
  FFT_IN_EF = 8,
  // double-float transforms: the half spectra (inverse input, forward output)
  // are FP64 instead of double-float pairs
  FFT_HS_F64 = 16,
};

// arithmetic of the azimuthal FFTs
enum FftArith : int { FFT_ARITH_F32 = 0, FFT_ARITH_F64 = 1, FFT_ARITH_DF = 2 };

struct FftField {
  const void* in;
  void* out;
  long long in_ld;   // elements (complex T for spectra, double for grids) between levels
  long long out_ld;
  int flags;
  int pad_;
};

struct FftSet {
  FftField f[MAGIC_MAX_FIELDS];
  int nf;
  int nlev;
};

// Grid geometry and device tables of one transform instance.
struct ShtGeom {
  int l_max, m_max, minc, n_m;   // n_m = m_max/minc + 1
  int n_theta, nh;               // nh = n_theta/2 (north points)
  int n_phi;                     // n_phi_max = n_phi_tot/minc
  int lm_max;
  int ld;                        // leading dimension (nlat_padded) of grid arrays
  int pad_;
  const int* lmoff;              // device [n_m] start of each m block (st_map)
  const double* P64;             // device [lm_max][nh]
  const double* dP64;
  const float* P32;
  const float* dP32;
  const double* wgt;             // device [nh]  2 pi w_j
  const double* osin2;           // device [nh]  1/sin^2 theta_j
  const double2* tw64;           // device [n_phi]  e^{+2 pi i k/n_phi}
  const float2* tw32;
  const void* twdf;              // device [n_phi]  the same as double-float pairs (hi, lo) x (re, im)
  const void* twr;               // device: the fast-path twiddle tables of the double-float FFT at 24
                                 // points per lane (read from L1 instead of shared memory), else null
};

// Pre-split (3xBF16) and pre-tiled Legendre tables of the tensor-core form.
// Every block is the exact shared-memory image of one 128-row x 64-column
// K-major operand tile with the 128-byte swizzle (16 KB).
//   synthesis block  (m, theta tile tt, table tb, parity p, l' chunk c, split s):
//     rows = 128 northern colatitudes, columns = 64 degrees l = m + p + 2 l'
//   analysis block   (m, parity p, l' tile lt, table tb, theta chunk c, split s):
//     rows = 128 degrees l = m + p + 2 l', columns = 64 northern colatitudes
// Rows are scaled by powers of two (scale tables hold the inverse factors).
struct TcTables {
  const unsigned char* inv_img;
  const long long* inv_blk0;  // [n_m] first synthesis block of each m
  const float* inv_scale;     // [2][n_m][ntt*128]
  const unsigned char* fwd_img;
  const long long* fwd_blk0;  // [n_m]
  const float* fwd_scale;     // [2][lm_max]
  const short* inv_exp;       // FP64-accurate form: row exponents [2][n_m][ntt*128] (the scales are 2^exp)
  const short* fwd_exp;       // [2][lm_max]
  int* err;                   // device error word (bounded waits that gave up)
  const long long* bpc0;      // [n_m] first (parity, chunk) pair of each m in the synthesis data images
  long long npc;              // total (parity, chunk) pairs over all m
  int* tile_ctr;              // tile counter of the persistent kernels (reset before each launch)
  int ntt;                    // theta tiles of 128 northern points
  int nlt;                    // l' tiles of 128 rows per parity
  int ncj;                    // theta chunks of 64 (analysis K)
  int order;                  // tile order of the persistent kernels: 0 = consecutive tiles
                              // share the table block, 1 = they share the data block
  int ndig;                   // fixed-point digits per operand of the FP64TC / BF16X5 forms (7 / 5)
  int pad_;
};

// grids of the nonlinear products (nl.cu): inputs from the synthesis set,
// outputs for the analysis set; ld = doubles between levels
enum NlIn : int { NL_VR, NL_VT, NL_VP, NL_CVR, NL_CVT, NL_CVP, NL_BR, NL_BT, NL_BP,
                  NL_CBR, NL_CBT, NL_CBP, NL_S, NL_NIN };
enum NlOut : int { NL_ADVR, NL_ADVT, NL_ADVP, NL_VSR, NL_VST, NL_VSP, NL_VXBR, NL_VXBT, NL_VXBP,
                   NL_HEAT, NL_NOUT };
struct NlGrids {
  double* p[NL_NIN];
  long long ld;
};

// the general get_nl (nl.cu): the reference's switches and radial functions
// (device arrays of the levels; null: the Boussinesq default, r required)
struct NlOpts {
  int conv, curl, lf, heat, chem, mag, anel, pad_;
  double LFfac, ViscHeatFac, OhmLossFac;
  const double *r, *orho1, *beta, *otemp1, *visc, *lambda;
  const int *nbc, *lcr;
};
enum NlfIn : int { NLF_VR, NLF_VT, NLF_VP, NLF_CVR, NLF_CVT, NLF_CVP, NLF_DVRDR, NLF_DVTDR, NLF_DVPDR,
                   NLF_DVRDT, NLF_DVRDP, NLF_DVTDP, NLF_DVPDP, NLF_BR, NLF_BT, NLF_BP, NLF_CBR, NLF_CBT,
                   NLF_CBP, NLF_S, NLF_XI, NLF_NIN };
enum NlfOut : int { NLF_ADVR, NLF_ADVT, NLF_ADVP, NLF_VSR, NLF_VST, NLF_VSP, NLF_VXIR, NLF_VXIT, NLF_VXIP,
                    NLF_VXBR, NLF_VXBT, NLF_VXBP, NLF_HEAT, NLF_NOUT };
struct NlFull {
  NlOpts o;
  const double* in[NLF_NIN];  // null: not needed by the switches
  double* out[NLF_NOUT];
  long long ld_in, ld_out;    // doubles between levels
};

// spectral assembly of the time derivatives (td.cu); arrays [level][ld] complex
struct TdArgs {
  const double2 *w, *dw, *z;                                   // radial-loop spectra
  const double2 *Advr, *Advt, *Advp, *VSt, *VxBr, *VxBt, *VxBp;  // analysis outputs
  double2 *dwdt, *dzdt, *dpdt, *dsdt, *dbdt, *djdt, *dVxBh;     // outputs
  long long ld;
  const double* r;      // [level] radius
  const int* lcut;      // [level] l_R, or null (= l_max)
  const double* epsc;   // [level] internal heating of dsdt(l=0), or null (= 0)
  const int* nbc;       // [level] boundary flag (nBc != 0), or null (all interior)
  double cor_fac;       // CorFac (1/E)
  const double2* coef;  // [lm][4] level-independent coefficients (build_td_coef)
  const int* lq;        // [lm] l | m << 16
};

// the general get_td (td.cu): the reference's switches; null outputs are skipped
struct TdOpts {
  int conv, corr, dcurl, single_matrix, anel, liquid, mag_nl, pad_;
  double cor_fac, epscXi;
  const double *r, *orho1, *beta, *temp0, *epsc;  // [level]; r required
  const int *lcut, *nbc;                          // [level] or null
};
struct TdFull {
  TdOpts o;
  const double2 *w, *dw, *ddw, *z, *dz;
  const double2 *Advr, *Advt, *Advp, *VSt, *heat, *VXit, *VxBr, *VxBt, *VxBp;
  double2 *dwdt, *dzdt, *dpdt, *dsdt, *dxidt, *dbdt, *djdt, *dVxBh, *dVxVh, *dVSr, *dVXir;
  long long ld;
  const double2* coef;
  const int* lq;
};

// Courant condition (courant.cu); grids [level][ld], radial functions [level]
struct CourantArgs {
  const double *vr, *vt, *vp, *br, *bt, *bp;  // br = null: no Lorentz-force term
  long long ld;
  const double *orho1, *orho2, *or2, *or4, *delxr2, *delxh2;
  double courfac, alffac, LFfac, opm;
  int alf_damp;
};

// grids of one level written at a rigid boundary (bcs.cu): vr, vt, vp, cvr,
// dvrdt, dvrdp, dvtdp, dvpdp; null entries are skipped
struct BcGrids {
  double* p[8];
};

// One transform instance of a persistent tensor-core launch: its geometry,
// its field set (InvSet or FwdSet), its table images and its data-operand
// images (`bimg`, column exponents `cexp` after the tiles), with `nct` column
// tiles.  A launch over several instances (magic_sht_group_*) takes an array
// of them: tile0 / blk0 are the instance's first tile of the persistent
// kernel and first block of the pack kernel, and the instances' tiles follow
// each other in the array's order.
template <class Set>
struct LegInst {
  ShtGeom g;
  Set s;
  TcTables t;
  unsigned char* bimg;
  short* cexp;
  int nct;
  int tile0;
  int blk0;
  int pad_;
};

// First tile / pack block of each instance of a launch over several
// instances, passed as a kernel parameter (constant bank: the per-tile lookup
// reads no global memory).
constexpr int kMaxGroupInst = 64;
struct InstIndex {
  int n;
  int tile0[kMaxGroupInst];
  int blk0[kMaxGroupInst];
};

template <class Set>
inline InstIndex inst_index(const LegInst<Set>* inst, int n) {
  InstIndex X{};
  X.n = n;
  for (int i = 0; i < n && i < kMaxGroupInst; ++i) {
    X.tile0[i] = inst[i].tile0;
    X.blk0[i] = inst[i].blk0;
  }
  return X;
}

#ifdef __CUDACC__
// the last instance whose first index (tile or block) is <= x
__device__ __forceinline__ int inst_search(const int* first, int n, int x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
// A persistent launch covers one instance (the kernel parameter `one`) or,
// with MULTI, the X.n instances of `many` (device memory), whose tiles and
// pack blocks follow each other; `one` then holds the first instance (the
// tile counter and the error word of the launch).
// The instance of persistent-kernel tile `ix`; ix becomes the tile within it.
template <bool MULTI, class I>
__device__ __forceinline__ const I& tile_inst(const I& one, const I* many, const InstIndex& X, int& ix) {
  if constexpr (!MULTI) {
    return one;
  } else {
    const int k = inst_search(X.tile0, X.n, ix);
    ix -= X.tile0[k];
    return many[k];
  }
}
// The instance, column tile ct, order mc and chunk c of this pack-kernel
// block: a 3-D grid (ct, mc, c) for one instance; with MULTI a 1-D grid whose
// blocks of one instance run column tile fastest, then order, then chunk.
template <bool MULTI, class I>
__device__ __forceinline__ const I& block_inst(const I& one, const I* many, const InstIndex& X, int& ct, int& mc,
                                               int& c) {
  if constexpr (!MULTI) {
    ct = blockIdx.x;
    mc = blockIdx.y;
    c = blockIdx.z;
    return one;
  } else {
    const int b = blockIdx.x;
    const int k = inst_search(X.blk0, X.n, b);
    const I& in = many[k];
    int r = b - X.blk0[k];
    ct = r % in.nct;
    r /= in.nct;
    mc = r % in.g.n_m;
    c = r / in.g.n_m;
    return in;
  }
}
#endif

__host__ __device__ inline int tc_nch(int n_l) { return ((n_l + 1) / 2 + 63) / 64; }

#define CUDA_TRY(x)                                                        \
  do {                                                                     \
    cudaError_t _e = (x);                                                  \
    if (_e != cudaSuccess) return _e;                                      \
  } while (0)
