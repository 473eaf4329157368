/*
 * magic_sht.h — C ABI of the GB300 (sm_103a) spherical-harmonic transform
 * library that replaces MagIC's `module sht` (src/sht_native.f90 over
 * src/shtransforms.f90, src/plms.f90 and src/fft.f90) as a drop-in.
 *
 * Conventions (identical to the reference):
 *   - spectral arrays: complex(8) in st_map order (m-major, l inner,
 *     src/blocking.f90:309-317), passed as interleaved (re, im) doubles;
 *   - grid arrays: real(8) f(nlat_padded, n_phi_max), column-major (theta
 *     fastest), theta rows scrambled north/south (row 2j-1 north, 2j south,
 *     1-based; initialize_sht returns l_scrambled_theta = .true.,
 *     src/sht_native.f90:29);
 *   - vector outputs in Robert form (x sin theta); forward FFT carries 1/n_phi.
 * Every pointer may be host memory (pageable or pinned: staged through the
 * device, the call returns after the results are back on the host) or device
 * memory (the call is asynchronous on the handle's stream).
 * Every function returns MAGIC_SHT_OK (0) or a MAGIC_SHT_ERR_* code; the
 * reference has no return codes and aborts (abortRun) on bad sizes
 * (src/truncation.f90:126-160, src/fft.f90:55-65).  magic_sht_last_error()
 * returns the message of the calling thread's last failure.
 */
#ifndef MAGIC_SHT_H
#define MAGIC_SHT_H

#ifdef __cplusplus
extern "C" {
#endif

#define MAGIC_SHT_OK 0
#define MAGIC_SHT_ERR_ARG 1         /* null handle/pointer, n_levels < 0, bad stride */
#define MAGIC_SHT_ERR_SIZE 2        /* grid/truncation rejected (truncation.f90:126-160) */
#define MAGIC_SHT_ERR_LCUT 3        /* lcut outside [0, l_max] */
#define MAGIC_SHT_ERR_CUDA 4        /* a CUDA runtime call failed */
#define MAGIC_SHT_ERR_UNSUPPORTED 5 /* precision/mode not available on this device */
#define MAGIC_SHT_ERR_NOMEM 6       /* device allocation failed */
#define MAGIC_SHT_ERR_TIMEOUT 7     /* a bounded device wait gave up */

/* Arithmetic forms of the Legendre sums and FFTs. */
#define MAGIC_SHT_FP64 0    /* FP64 everywhere: the parity form */
#define MAGIC_SHT_FP32 1    /* FP32 tables, FFTs and accumulation */
#define MAGIC_SHT_BF16X3 2  /* tensor cores: 3xBF16 split products, FP32 accumulate, FP32 FFT */
#define MAGIC_SHT_TF32X2 3  /* tensor cores: 2xTF32 split products (hi*hi, hi*lo, lo*hi), FP32 accumulate,
                               FP32 FFT; persistent kernels only (no scal_to_spat_noalloc) */
#define MAGIC_SHT_FP64TC 4  /* FP64-accurate on tensor cores: seven fixed-point BF16 digits per operand, 28 digit
                               products accumulated exactly in FP32, double-float (FP32-pair) FFTs and
                               half spectra, FP64 radial-loop kernels; values within the FP32 exponent range */
#define MAGIC_SHT_BF16X5 5  /* the same tensor-core form with five fixed-point BF16 digits per operand (15 digit
                               products, the dropped digits below 2^-39 of the row and column scales): double-float
                               FFTs and half spectra, FP64 radial-loop kernels, the FP32 exponent range */

typedef struct magic_sht_desc {
  int l_max;       /* truncation degree (truncation.f90 l_max) */
  int m_max;       /* 0 -> (l_max/minc)*minc (truncation.f90:75) */
  int minc;        /* azimuthal symmetry; n_phi_max = n_phi_tot/minc */
  int n_theta_max; /* Gauss points, multiple of 4 (truncation.f90:150) */
  int n_phi_max;   /* longitudes per symmetry sector, multiple of 4, 2^i 3^j 5^k */
  int nlat_padded; /* leading dimension of grid arrays; 0 -> n_theta_max */
  int precision;   /* MAGIC_SHT_FP64 | _FP32 | _BF16X3 | _TF32X2 | _FP64TC | _BF16X5 */
  int device;      /* CUDA device ordinal; -1 -> current device */
} magic_sht_desc;

typedef struct magic_sht_handle magic_sht_handle;
typedef struct magic_sht_graph magic_sht_graph;

/* ---- set-up: replaces initialize_sht / finalize_sht (sht_native.f90:24-38)
 * and initialize_transforms (shtransforms.f90:38-91): Gauss nodes, P_lm and
 * sin(theta) dP_lm/dtheta tables are built in FP64 on the GPU. */
int magic_sht_init(const magic_sht_desc* desc, magic_sht_handle** handle);
int magic_sht_finalize(magic_sht_handle* handle);
const char* magic_sht_last_error(void);
/* l_scrambled_theta of initialize_sht (sht_native.f90:29): always 1. */
int magic_sht_scrambled_theta(const magic_sht_handle* handle, int* l_scrambled_theta);
/* out[0..7] = {l_max, m_max, minc, n_theta_max, n_phi_max, nlat_padded, n_m_max, lm_max} */
int magic_sht_get_sizes(const magic_sht_handle* handle, int* out8);
/* Gauss-Legendre colatitudes (north -> south) and weights, n_theta_max each
 * (gauleg, horizontal.f90:279-340). Host pointers. */
int magic_sht_gauss_grid(magic_sht_handle* handle, double* theta_ord, double* gauss);
/* Run on an external CUDA stream (cudaStream_t passed as void*); NULL selects
 * the legacy default stream.  The handle starts on a stream of its own. */
int magic_sht_set_stream(magic_sht_handle* handle, void* cuda_stream);
int magic_sht_synchronize(magic_sht_handle* handle);
/* Pre-size the device workspace for batched calls of up to n_levels levels
 * (required before capturing a graph). */
int magic_sht_reserve(magic_sht_handle* handle, int n_levels);

/* ---- spectral -> grid, one radial level (sht_native.f90 public names) ---- */
int magic_sht_scal_to_spat(magic_sht_handle* h, const double* Slm, double* fieldc,
                           int lcut);                                   /* :40-52   */
int magic_sht_scal_to_grad_spat(magic_sht_handle* h, const double* Slm, double* gradtc,
                                double* gradpc, int lcut);              /* :54-68   */
int magic_sht_pol_to_grad_spat(magic_sht_handle* h, const double* Slm, double* gradtc,
                               double* gradpc, int lcut);               /* :70-97   */
int magic_sht_torpol_to_spat(magic_sht_handle* h, const double* Wlm, const double* dWlm,
                             const double* Zlm, double* vrc, double* vtc, double* vpc,
                             int lcut);                                 /* :99-127  */
int magic_sht_sphtor_to_spat(magic_sht_handle* h, const double* dWlm, const double* Zlm,
                             double* vtc, double* vpc, int lcut);       /* :129-141 */
int magic_sht_torpol_to_curl_spat_IC(magic_sht_handle* h, double r, double r_ICB,
                                     const double* dBlm, const double* ddBlm,
                                     const double* Jlm, const double* dJlm, double* cbr,
                                     double* cbt, double* cbp);         /* :143-186 */
int magic_sht_torpol_to_spat_IC(magic_sht_handle* h, double r, double r_ICB,
                                const double* Wlm, const double* dWlm, const double* Zlm,
                                double* Br, double* Bt, double* Bp);    /* :188-229 */
int magic_sht_torpol_to_dphspat(magic_sht_handle* h, const double* dWlm, const double* Zlm,
                                double* dvtdp, double* dvpdp, int lcut); /* :231-272 */
int magic_sht_pol_to_curlr_spat(magic_sht_handle* h, const double* Qlm, double* cvrc,
                                int lcut);                              /* :274-300 */
int magic_sht_torpol_to_curl_spat(magic_sht_handle* h, double or2, const double* Blm,
                                  const double* ddBlm, const double* Jlm, const double* dJlm,
                                  double* cvrc, double* cvtc, double* cvpc,
                                  int lcut);                            /* :302-336 */
int magic_sht_axi_to_spat(magic_sht_handle* h, const double* fl_ax,
                          double* f);                                   /* :381-391 */
int magic_sht_toraxi_to_spat(magic_sht_handle* h, const double* fl_ax, double* ft, double* fp,
                             int lcut);                                 /* :393-405 */

/* Allocation-free variant of magic_sht_scal_to_spat.  It has no counterpart
 * in the reference.  It is meant for callers that must not allocate device
 * memory while they run: applications whose free GPU memory is owned by a
 * pool allocator (a raw cudaMalloc there fails or fragments the pool), and
 * time-critical loops where cudaMalloc/cudaFree would stall on their
 * implicit device synchronization.  The ordinary entry points may grow the
 * handle's workspace with cudaMalloc; this one calls no allocating routine:
 * its only scratch (the (theta, m) half spectrum) is a static 4 MiB device
 * array that every GPU loading the library holds until the process exits.
 *   - Slm and fieldc must be device pointers (MAGIC_SHT_ERR_ARG otherwise);
 *     the call is asynchronous on the handle's stream.
 *   - Limit: n_m_max * n_theta_max * 16 bytes (FP64 form; 8 bytes for the
 *     other forms) must not exceed 4 MiB, else MAGIC_SHT_ERR_SIZE; e.g.
 *     l_max=255 with 384 Gauss points uses 1.5 MiB.
 *   - magic_sht_init loads the library's module on its device and looks
 *     up the array's device address there (cudaGetSymbolAddress, with that
 *     device current), so the array is reserved when the first handle on a
 *     device is created, not by this call; this call only reads the cached
 *     address.
 *   - Every call shares the one array, which keeps the last call's contents
 *     (each call overwrites all of it before reading it); calls that overlap
 *     on the GPU (other streams, other handles on the same device) race. */
int magic_sht_scal_to_spat_noalloc(magic_sht_handle* h, const double* Slm, double* fieldc, int lcut);

/* ---- grid -> spectral, one radial level ---- */
int magic_sht_scal_to_SH(magic_sht_handle* h, const double* f, double* fLM,
                         int lcut);                                     /* :338-346 */
int magic_sht_spat_to_qst(magic_sht_handle* h, const double* f, const double* g,
                          const double* hh, double* qLM, double* sLM, double* tLM,
                          int lcut);                                    /* :348-364 */
int magic_sht_spat_to_sphertor(magic_sht_handle* h, const double* f, const double* g,
                               double* fLM, double* gLM, int lcut);     /* :366-379 */

/* ---- the radial loop's transform set, many radial levels per call ----
 * transform_to_grid_space (rIter.f90:466-622) and transform_to_lm_space
 * (rIter.f90:624-712) for levels nR = 1..n_levels at once.  Spectral arrays
 * are laid out like the reference's R-distributed fields f_Rloc(lm_max, nR):
 * level k starts at ptr + 2*k*spec_ld doubles; grids at ptr + k*grid_ld
 * doubles.  A NULL input/output pointer skips that field (and its outputs).
 * or2 (1/r^2 per level) and lcut (l_R(nR) per level) may be NULL (0 and
 * l_max).  Host pointers are staged; device pointers stay asynchronous. */
typedef struct magic_sht_grid_space_args {
  /* spectral inputs, complex [n_levels][spec_ld] */
  const double *s, *p, *xi;                 /* scal_to_spat (rIter.f90:485,503,506) */
  const double *w, *dw, *ddw, *z, *dz;      /* torpol_to_spat + torpol_to_curl_spat (:516,:522) */
  const double *b, *db, *ddb, *aj, *dj;     /* torpol_to_spat + torpol_to_curl_spat (:606,:610) */
  long long spec_ld;                        /* complex elements between levels (>= lm_max) */
  /* grid outputs, [n_levels][grid_ld] doubles, each level f(nlat_padded, n_phi_max) */
  double *sc, *pc, *xic;
  double *vrc, *vtc, *vpc, *cvrc, *cvtc, *cvpc;
  double *brc, *btc, *bpc, *cbrc, *cbtc, *cbpc;
  long long grid_ld;                        /* doubles between levels (>= nlat_padded*n_phi_max) */
  /* velocity derivatives of the u.grad u advection and the anelastic viscous
   * heating (rIter.f90:527-545), at grid_ld; NULL skips them:
   * torpol_to_spat(dw, ddw, dz) -> dvrdrc, dvtdrc, dvpdrc;
   * pol_to_grad_spat(w) -> dvrdtc, dvrdpc; torpol_to_dphspat(dw, z) -> dvtdpc, dvpdpc.
   * cvrc alone (without cvtc, cvpc) is pol_to_curlr_spat(z) (rIter.f90:540). */
  double *dvrdrc, *dvtdrc, *dvpdrc, *dvrdtc, *dvrdpc, *dvtdpc, *dvpdpc;
} magic_sht_grid_space_args;

typedef struct magic_sht_lm_space_args {
  /* grid inputs */
  const double *Advr, *Advt, *Advp;         /* spat_to_qst (rIter.f90:682) */
  const double *VSr, *VSt, *VSp;            /* spat_to_qst (:688) */
  const double *VxBr, *VxBt, *VxBp;         /* spat_to_qst (:701) */
  const double *heatTerms;                  /* scal_to_SH (:691) */
  long long grid_ld;
  /* spectral outputs */
  double *AdvrLM, *AdvtLM, *AdvpLM;
  double *VSrLM, *VStLM, *VSpLM;
  double *VxBrLM, *VxBtLM, *VxBpLM;
  double *heatTermsLM;
  long long spec_ld;
  /* composition (l_chemical_conv): spat_to_qst of V Xi (rIter.f90:699-702);
   * grid inputs at grid_ld, spectral outputs at spec_ld; NULL skips them */
  const double *VXir, *VXit, *VXip;
  double *VXirLM, *VXitLM, *VXipLM;
} magic_sht_lm_space_args;

int magic_sht_transform_to_grid_space(magic_sht_handle* h, int n_levels, const double* or2,
                                      const int* lcut, const magic_sht_grid_space_args* a);
int magic_sht_transform_to_lm_space(magic_sht_handle* h, int n_levels, const int* lcut,
                                    const magic_sht_lm_space_args* a);

/* ---- any facade routines, many radial levels per call ----
 * Each job is one facade routine of module sht (sht_native.f90:16-20) applied
 * to every level of its arrays, with the routine's own argument order:
 * in[] its array inputs, out[] its outputs (spectra complex, spec_ld apart per
 * level; grids grid_ld doubles apart), unused slots NULL.  All jobs of one call
 * share one batched Legendre launch per field kind and one FFT launch per
 * direction.  lcut (per level, NULL = l_max) applies to every job; or2 (per
 * level) is the or2 argument of torpol_to_curl_spat jobs (required when one is
 * present).  Inputs may be shared between jobs; outputs must be distinct.
 * Host pointers are staged (pipelined over chunks of levels when every array
 * is in host memory); device pointers stay asynchronous.  Errors:
 * MAGIC_SHT_ERR_ARG for an unknown routine, a job of the other direction, a
 * missing array, repeated outputs or a curl job without or2. */
enum {
  /* synthesis (magic_sht_inv_batch): in[] -> out[] */
  MAGIC_SHT_JOB_SCAL_TO_SPAT = 1,        /* Slm -> fieldc */
  MAGIC_SHT_JOB_SCAL_TO_GRAD_SPAT = 2,   /* Slm -> gradtc, gradpc */
  MAGIC_SHT_JOB_POL_TO_GRAD_SPAT = 3,    /* Slm -> gradtc, gradpc */
  MAGIC_SHT_JOB_TORPOL_TO_SPAT = 4,      /* Wlm, dWlm, Zlm -> vrc, vtc, vpc */
  MAGIC_SHT_JOB_SPHTOR_TO_SPAT = 5,      /* dWlm, Zlm -> vtc, vpc */
  MAGIC_SHT_JOB_TORPOL_TO_CURL_SPAT = 6, /* Blm, ddBlm, Jlm, dJlm -> cvrc, cvtc, cvpc (or2 per level) */
  MAGIC_SHT_JOB_POL_TO_CURLR_SPAT = 7,   /* Qlm -> cvrc */
  MAGIC_SHT_JOB_TORPOL_TO_DPHSPAT = 8,   /* dWlm, Zlm -> dvtdp, dvpdp */
  /* analysis (magic_sht_fwd_batch) */
  MAGIC_SHT_JOB_SCAL_TO_SH = 101,        /* f -> fLM */
  MAGIC_SHT_JOB_SPAT_TO_QST = 102,       /* f, g, h -> qLM, sLM, tLM */
  MAGIC_SHT_JOB_SPAT_TO_SPHERTOR = 103   /* f, g -> fLM, gLM */
};
typedef struct magic_sht_job {
  int routine;                              /* MAGIC_SHT_JOB_* */
  int pad_;
  const double *in[4];
  double *out[3];
} magic_sht_job;
int magic_sht_inv_batch(magic_sht_handle* h, int n_levels, const double* or2, const int* lcut,
                        long long spec_ld, long long grid_ld, const magic_sht_job* jobs, int n_jobs);
int magic_sht_fwd_batch(magic_sht_handle* h, int n_levels, const int* lcut, long long grid_ld,
                        long long spec_ld, const magic_sht_job* jobs, int n_jobs);

/* ---- asynchronous host-buffer batches.  With on != 0, a batched call whose
 * arrays are all in host memory and that spans more than 16 levels returns once
 * its chunked copies and kernels are queued (instead of when the host outputs
 * are written); its host arrays must stay valid and untouched until
 * magic_sht_synchronize(h).  Consecutive such calls overlap one call's
 * device-to-host copies with the next call's host-to-device copies.  Off by
 * default (the reference's calls return with their results). */
int magic_sht_set_host_async(magic_sht_handle* h, int on);

/* ---- runtime tuning of one handle (magic_gb300/autotune.py searches these
 * per geometry and caches the choice).  Results do not depend on them except
 * tc_kernel, which selects between two kernels of the same arithmetic form,
 * and fft_rows, whose forward FFT factors its twiddles e^(2 pi i k / n_phi)
 * differently (spectra differ at FP32 rounding, grids are identical); graphs
 * captured earlier keep the settings they were captured with.
 *   tc_kernel:  tensor-core forms, 0 persistent kernels, 1 one tile per CTA
 *               (3xBF16) or the FP64 SIMT Legendre sums (FP64TC, with its
 *               double-float FFTs)
 *   tc_order:   persistent kernels' tile order, 0 consecutive tiles share the
 *               table blocks, 1 they share the data tiles
 *   pipe_chunk: radial levels per chunk of the host-buffer pipeline (1..1024)
 *   fft_rows:   theta rows per CTA of the FP32 azimuthal FFT, 8 or 16
 *               (0 = by size; the double-float FFTs choose their own: 8 rows
 *               where 16 would not fit two CTAs per SM, and for the forward at
 *               n_phi = 768) */
typedef struct magic_sht_tuning {
  int tc_kernel, tc_order, pipe_chunk, fft_rows;
} magic_sht_tuning;
int magic_sht_set_tuning(magic_sht_handle* h, const magic_sht_tuning* t);
int magic_sht_get_tuning(const magic_sht_handle* h, magic_sht_tuning* t);

/* ---- grid-space nonlinear products between the two transform sets
 * (get_nl.f90:213-441 and the Lorentz-force addition of rIter.f90:650-655).
 * Reads the grids transform_to_grid_space writes (vrc..vpc, cvrc..cvpc,
 * brc..bpc, cbrc..cbpc, sc of `g`) and writes the grids
 * transform_to_lm_space reads (Advr..heatTerms of `nl`; their const
 * qualifiers are cast away: they are this call's outputs).  Boussinesq form,
 * curl-form advection, magnetic field and heat equation on, unit physical
 * constants; heatTerms receives the ohmic losses.  Device pointers only,
 * 16-byte aligned, even grid_ld and nlat_padded; or2 = 1/r^2 per level (host
 * or device array of n_levels; NULL = 1).  Arithmetic: FP64 on an FP64
 * handle; FP32 (FP64 grids in and out) on the reduced-precision forms. */
int magic_sht_get_nl(magic_sht_handle* h, int n_levels, const double* or2, const magic_sht_grid_space_args* g,
                     const magic_sht_lm_space_args* nl);

/* ---- the grid-space nonlinear products with the reference's switches and
 * physical parameters (get_nl.f90:213-441) and the Lorentz-force combination
 * of transform_to_lm_space (rIter.f90:645-662).  Per level:
 *   Adv (where nBc = 0 and l_conv_nl or l_mag_LF): the advection, curl form
 *     (l_adv_curl, :260-272) or u.grad u (:274-302), when l_conv_nl, plus
 *     LFfac times the Lorentz force (:243-256) when l_mag_LF and the level is
 *     outside the low-conductivity region;
 *   VS, VXi (where nBc = 0 and l_heat_nl / l_chemical_conv, :316-327);
 *   VxB (l_mag_nl, :376-395): the full product where nBc = 0 outside the
 *     region; VxBt, VxBp of the stress-free form where nBc = 1 or inside the
 *     region; of the rigid form (VxBp = 0) where nBc = 2; VxBr is written
 *     with the full product only;
 *   heatTerms (where nBc = 0 and l_anel, :398-432): viscous heating plus, with
 *     l_mag_nl outside the region, ohmic losses.
 * Outputs a level does not produce are left untouched (the reference leaves
 * them as they were).  Grids: device pointers, 16-byte aligned, even grid_ld
 * and nlat_padded; the inputs each enabled term needs must be non-NULL
 * (velocity and vorticity; the derivative grids for u.grad u and l_anel;
 * B and curl B for the Lorentz force, the induction and the ohmic losses; s,
 * xi).  Per-level arrays: host or device, n_levels entries; r is required,
 * NULL orho1 / beta / otemp1 / visc / lambda / nbc / lcr mean 1 / 0 / 1 /
 * 1 / 1 / 0 / 0.  Arithmetic: FP64 on the FP64 and FP64-accurate tensor-core
 * handles, FP32 (FP64 grids in and out) on the reduced forms. */
typedef struct magic_sht_nl_opts {
  int l_conv_nl, l_adv_curl, l_mag_LF, l_heat_nl, l_chemical_conv, l_mag_nl, l_anel, pad_;
  double LFfac, ViscHeatFac, OhmLossFac;
  const double *r, *orho1, *beta, *otemp1, *visc, *lambda;
  const int *nbc;   /* nBc per level */
  const int *lcr;   /* nonzero: nR <= n_r_LCR (inside the low-conductivity region) */
} magic_sht_nl_opts;
typedef struct magic_sht_nl_grids {
  const double *vrc, *vtc, *vpc, *cvrc, *cvtc, *cvpc;
  const double *dvrdrc, *dvtdrc, *dvpdrc, *dvrdtc, *dvrdpc, *dvtdpc, *dvpdpc;
  const double *brc, *btc, *bpc, *cbrc, *cbtc, *cbpc;
  const double *sc, *xic;
  long long grid_ld;
} magic_sht_nl_grids;
typedef struct magic_sht_nl_out {
  double *Advr, *Advt, *Advp, *VSr, *VSt, *VSp, *VXir, *VXit, *VXip, *VxBr, *VxBt, *VxBp, *heatTerms;
  long long grid_ld;
} magic_sht_nl_out;
int magic_sht_get_nl_opts(magic_sht_handle* h, int n_levels, const magic_sht_nl_opts* opts,
                          const magic_sht_nl_grids* in, const magic_sht_nl_out* out);

/* ---- spectral assembly of the explicit time derivatives at interior radial
 * levels (get_td.f90: get_dwdt :133-208, get_dpdt :311-379, get_dzdt
 * :381-457, get_dsdt :459-521, get_dbdt :558-619) from the analysis outputs
 * and the radial-loop spectra: Boussinesq form, Coriolis force (cor_fac =
 * CorFac), magnetic field and heat equation on, no double-curl form.  Device
 * arrays [n_levels][spec_ld] complex; r (radius), lcut (l_R, NULL = l_max) and
 * epsc (internal heating added to dsdt at l = 0, NULL = 0) are per-level host
 * or device arrays.  dpdt at l = 0 is set to 0 (the reference leaves it).
 * Arithmetic: FP64 on an FP64 handle; FP32 (FP64 spectra in and out) on the
 * reduced-precision forms. */
typedef struct magic_sht_td_args {
  const double *w, *dw, *z;                                           /* spectra */
  const double *AdvrLM, *AdvtLM, *AdvpLM, *VStLM, *VxBrLM, *VxBtLM, *VxBpLM;  /* analysis out */
  double *dwdt, *dzdt, *dpdt, *dsdt, *dbdt, *djdt, *dVxBhLM;           /* outputs */
  long long spec_ld;
} magic_sht_td_args;
int magic_sht_get_td(magic_sht_handle* h, int n_levels, const double* r, const int* lcut, double cor_fac,
                     const double* epsc, const magic_sht_td_args* a);
/* The same with a boundary flag per level (nbc, host or device int array of
 * n_levels; nBc of rIter.f90:193-215): at a level with nbc != 0 only dVxBhLM
 * is written (get_td.f90:598-612) and the other outputs are left untouched. */
int magic_sht_get_td_nbc(magic_sht_handle* h, int n_levels, const double* r, const int* lcut, double cor_fac,
                         const double* epsc, const int* nbc, const magic_sht_td_args* a);

/* ---- the spectral assembly with the reference's switches, as the radial
 * loop calls it (rIter.f90:410-428): get_dzdt (get_td.f90:381-457),
 * get_dwdt (:133-208) or, with l_double_curl, get_dwdt_double_curl
 * (:210-309, also dVxVhLM), get_dpdt (:311-379), get_dsdt (:459-521: the
 * anelastic heatTermsLM, times temp0 in the anelastic-liquid form), get_dxidt
 * (:523-556), get_dbdt (:558-619; zeros without l_mag_nl).  An output is
 * computed where its pointer is non-NULL (its equation is on) and left
 * untouched otherwise; at a level with nbc != 0 only dVxBhLM, dVxVhLM (double
 * curl; zero), dVSrLM (with dsdt; zero) and dVXirLM (with dxidt; zero) are
 * written; dpdt and dVxVhLM at l = 0 are never written (the reference leaves
 * them).  Spectra: device arrays [n_levels][spec_ld] complex; per-level
 * arrays host or device (r required; NULL orho1 / beta / temp0 / epsc / lcut
 * / nbc mean 1 / 0 / 1 / 0 / l_max / 0).  Arithmetic as magic_sht_get_td. */
typedef struct magic_sht_td_opts {
  int l_conv_nl, l_corr, l_double_curl, l_single_matrix, l_anel, l_anelastic_liquid, l_mag_nl, pad_;
  double cor_fac, epscXi;
  const double *r, *orho1, *beta, *temp0, *epsc;
  const int *lcut, *nbc;
} magic_sht_td_opts;
typedef struct magic_sht_td_in {
  const double *w, *dw, *ddw, *z, *dz;
  const double *AdvrLM, *AdvtLM, *AdvpLM, *VStLM, *heatTermsLM, *VXitLM, *VxBrLM, *VxBtLM, *VxBpLM;
  long long spec_ld;
} magic_sht_td_in;
typedef struct magic_sht_td_out {
  double *dwdt, *dzdt, *dpdt, *dsdt, *dxidt, *dbdt, *djdt, *dVxBhLM, *dVxVhLM, *dVSrLM, *dVXirLM;
  long long spec_ld;
} magic_sht_td_out;
int magic_sht_get_td_opts(magic_sht_handle* h, int n_levels, const magic_sht_td_opts* opts,
                          const magic_sht_td_in* in, const magic_sht_td_out* out);

/* ---- Courant condition of the radial loop (courant.f90:54-278, the branch
 * the reference compiles): per level, the maxima over the grid of the radial
 * and horizontal velocity terms (fluid + damped Alfven velocity with the
 * Lorentz force), then dtrkc = min(dtrkc, sqrt(delxr2 / vr2max)) and
 * dthkc = min(dthkc, sqrt(delxh2 / vh2max)); a level whose maximum is 0 keeps
 * its values.  Grids: device pointers as transform_to_grid_space writes them
 * (level stride grid_ld); br = bt = bp = NULL drops the Lorentz-force term
 * (l_mag_LF off or l_mag_kin).  Radial functions: arrays of n_levels (host or
 * device); dtrkc, dthkc: in/out arrays of n_levels (host or device; the
 * radial loop starts them at 1e10).  The maxima are the FP64 values of the
 * reference's expressions in every precision form (an FP32 estimate only
 * selects the points that can hold them). */
typedef struct magic_sht_courant_args {
  const double *vr, *vt, *vp, *br, *bt, *bp;
  long long grid_ld;
  const double *orho1, *orho2, *or2, *or4, *delxr2, *delxh2;
  double courfac, alffac, LFfac, opm;
  int l_cour_alf_damp;
} magic_sht_courant_args;
int magic_sht_courant(magic_sht_handle* h, int n_levels, const magic_sht_courant_args* a, double* dtrkc,
                      double* dthkc);

/* ---- new time step from the Courant steps (dt_courant, courant.f90:280-346,
 * without its log lines): host arrays of n_levels; *l_new_dt = 1 and *dt_new
 * the new step when dt > dtMax, dt > min(dtrkc, dthkc), or 2 dt < that
 * minimum (and dt < dtMax); otherwise 0 and dt.  Needs no GPU. */
int magic_sht_dt_courant(int n_levels, const double* dtrkc, const double* dthkc, double dt, double dtMax,
                         int* l_new_dt, double* dt_new);

/* ---- boundary pieces of the radial loop (nonlinear_bcs.f90), one radial
 * level each; grids f(nlat_padded, n_phi_max) like the facade routines, host
 * or device pointers.
 * v_rigid_boundary (:120-175): a rigid boundary rotating at omega, with
 * r2_rho0 = r^2 rho0 at that boundary: vr = 0 (kept when keep_vr, l_vr_cmb /
 * l_vr_icb), vt = 0, vp = r2_rho0 sin^2(theta) omega; when lDeriv, cvr =
 * 2 r2_rho0 cos(theta) omega and dvrdt, dvrdp, dvtdp, dvpdp = 0.  NULL grids
 * are skipped (vr, vt, vp are required). */
typedef struct magic_sht_rigid_args {
  double *vr, *vt, *vp;                    /* required */
  double *cvr, *dvrdt, *dvrdp, *dvtdp, *dvpdp; /* written when non-NULL (lDeriv) */
} magic_sht_rigid_args;
int magic_sht_v_rigid_boundary(magic_sht_handle* h, double r2_rho0, double omega, int keep_vr,
                               const magic_sht_rigid_args* a);
/* v_center_sphere (:177-224): the l = 1 flow at the centre of a full sphere
 * from the spectrum ddw (lm_max complex; uses l = 1, m = 0 and m = 1). */
int magic_sht_v_center_sphere(magic_sht_handle* h, const double* ddw, double* vr, double* vt, double* vp);
/* get_br_v_bcs (:24-69): spat_to_sphertor of br vt / (r^2 sin^2) and
 * br (vp / (r^2 sin^2) - omega), i.e. of fac br vt and br (fac vp - omega
 * sin^2(theta)) with fac = or2 orho1, into br_vt_lm, br_vp_lm (lm_max complex). */
int magic_sht_get_br_v_bcs(magic_sht_handle* h, const double* br, const double* vt, const double* vp, double omega,
                           double or2, double orho1, double* br_vt_lm, double* br_vp_lm);
/* ---- Lorentz torque on a rotating, conducting mantle or inner core
 * (get_lorentz_torque, outRot.f90:423-483) from one boundary level's grids
 * br (r^2 B_r) and bp (r sin(theta) B_phi) as transform_to_grid_space writes
 * them: *torque = LFfac 2 pi / n_phi_max times the sum over the grid of
 * gauss(theta) (br - b0 cos(theta)) bp, with b0 = 2 BIC r_icb^2 (times
 * r_icb / r_cmb at the outer boundary) in the Grenoble setup and 0 otherwise.
 * Grids and *torque host or device.  The radial loop uses the value at the
 * inner boundary and minus the value at the outer one (rIter.f90:278-292,
 * :462). */
int magic_sht_lorentz_torque(magic_sht_handle* h, const double* br, const double* bp, double LFfac, double b0,
                             double* torque);
/* get_b_nl_bcs (:71-118): b_nl_bc = -fac br_vt_lm and aj_nl_bc = -fac br_vp_lm
 * for l > 0, 0 at l = m = 0; fac = conductance_ma prmag at the CMB (both
 * outputs), sigma_ratio prmag at the ICB (b_nl_bc = NULL: aj only). */
int magic_sht_get_b_nl_bcs(magic_sht_handle* h, double fac, const double* br_vt_lm, const double* br_vp_lm,
                           double* b_nl_bc, double* aj_nl_bc);

/* ---- CUDA-graph capture of a device-pointer call sequence on the handle's
 * stream (e.g. the radial loop's transform set), replayed with one launch. */
int magic_sht_graph_begin(magic_sht_handle* h);
int magic_sht_graph_end(magic_sht_handle* h, magic_sht_graph** graph);
int magic_sht_graph_launch(magic_sht_handle* h, const magic_sht_graph* graph);
int magic_sht_graph_destroy(magic_sht_graph* graph);

/* ---- several independent instances in one launch per kind.  A group holds
 * handles of different l_max / minc / grids (each its own initialize_transforms,
 * all MAGIC_SHT_FP64TC, all MAGIC_SHT_BF16X5 or all MAGIC_SHT_BF16X3, with the
 * persistent tensor-core kernels, one device).
 * A group call runs the batched call of every instance (argument i for handle
 * i, the same meaning as magic_sht_transform_to_grid_space /
 * magic_sht_transform_to_lm_space), but the Legendre sums of all instances go
 * into one pack and one persistent tensor-core launch per direction and field
 * kind (scalar, vector), the instances with the largest l_max first, with the
 * FFTs of every instance after them (synthesis) or before them (analysis).
 * The results equal those of the separate calls bit for bit.  The reference
 * runs one instance per process and loops its radial levels (rIter.f90:190);
 * this is the batching form of the same per-level set.
 * Device arrays only for spectra and grids (or2 / lcut may be host arrays);
 * every handle must be bound to one stream (magic_sht_set_stream), on which
 * the call is asynchronous and may be captured with magic_sht_graph_begin on
 * the first handle: make the same calls once before capturing (they size the
 * workspaces and reserve room for the per-instance tables of captured calls,
 * which the group keeps until magic_sht_group_destroy; uncaptured calls reuse
 * a fixed device ring for theirs).  A handle belongs to at most one group call
 * at a time; n_levels, or2, lcut and args are arrays of n_handles entries
 * (or2 / lcut may be NULL for all). */
typedef struct magic_sht_group magic_sht_group;
int magic_sht_group_create(magic_sht_handle* const* handles, int n_handles, magic_sht_group** group);
int magic_sht_group_destroy(magic_sht_group* group);
int magic_sht_group_transform_to_grid_space(magic_sht_group* group, const int* n_levels,
                                            const double* const* or2, const int* const* lcut,
                                            const magic_sht_grid_space_args* args);
int magic_sht_group_transform_to_lm_space(magic_sht_group* group, const int* n_levels, const int* const* lcut,
                                          const magic_sht_lm_space_args* args);

/* ---- per-phase timing: CUDA events recorded on the handle's stream around
 * every kernel launch while profiling is on (timer counterpart of the
 * reference's lm2phy/phy2lm counters, timing.f90:17-163). */
#define MAGIC_SHT_PHASE_INV_LEG_SCALAR 0
#define MAGIC_SHT_PHASE_INV_LEG_VECTOR 1
#define MAGIC_SHT_PHASE_FFT_INV 2
#define MAGIC_SHT_PHASE_FFT_FWD 3
#define MAGIC_SHT_PHASE_FWD_LEG_SCALAR 4
#define MAGIC_SHT_PHASE_FWD_LEG_VECTOR 5
#define MAGIC_SHT_PHASE_NL 6      /* magic_sht_get_nl */
#define MAGIC_SHT_PHASE_COURANT 7 /* magic_sht_courant (two kernels) */
#define MAGIC_SHT_PHASE_TD 8      /* magic_sht_get_td / magic_sht_get_td_nbc */
#define MAGIC_SHT_PHASE_BCS 9     /* the boundary kernels of nonlinear_bcs.f90 */
#define MAGIC_SHT_N_PHASES 10
int magic_sht_set_profiling(magic_sht_handle* h, int on);
/* accumulated ms and launch counts per phase (arrays of MAGIC_SHT_N_PHASES) */
int magic_sht_phase_times(magic_sht_handle* h, double* ms, long long* launches, int reset);
/* MAGIC_SHT_ERR_TIMEOUT if a bounded device wait of an earlier kernel gave
 * up (synchronizes the handle's stream); clear != 0 resets the flag. */
int magic_sht_device_status(magic_sht_handle* h, int clear);
/* total kernel launches issued by this handle */
int magic_sht_launch_count(const magic_sht_handle* h, long long* n);

/* ---- measurement helper: FMA throughput of the device in GFLOP/s for
 * precision MAGIC_SHT_FP64 or MAGIC_SHT_FP32, the roofline denominators of
 * the FP64 and FP32 forms of the Legendre sums. */
int magic_sht_measure_gflops(int device, int precision, double* gflops);

/* ---- diagnostics: one tcgen05 (tensor-core) GEMM D = A B^T with M=128,
 * N = n (32/64/128/256), K = 64*kchunks (1 or 2) on bf16-exact inputs,
 * checked on the host; returns the max error relative to max |D|. */
int magic_sht_tc_selftest(int device, int n, int kchunks, double* max_rel_err);
/* Failure-detection check of the kernels' bounded waits: a one-thread kernel
 * waits on an mbarrier that is (arrive != 0) or is never (arrive == 0)
 * completed, giving up after max_cycles SM cycles (1 .. 2^31).  Returns
 * MAGIC_SHT_ERR_TIMEOUT when the wait gave up (the device stays usable),
 * MAGIC_SHT_OK when it completed. */
int magic_sht_wait_selftest(int device, long long max_cycles, int arrive);
/* the same with tf32 operands (kind::tf32), K = 32*kchunks */
int magic_sht_tc_selftest_tf32(int device, int n, int kchunks, double* max_rel_err);

#ifdef __cplusplus
}
#endif
#endif /* MAGIC_SHT_H */
