// C ABI of the library (include/magic_sht.h): handle life cycle, host/device
// pointer staging, the public names of MagIC's `module sht`
// (src/sht_native.f90:16-20) and the batched radial-loop transform set
// (src/rIter.f90:466-712).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/magic_sht.h"
#include "common.cuh"
#include "internal.h"

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;

static int set_err(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess)                                                         \
      return set_err(_e == cudaErrorMemoryAllocation ? MAGIC_SHT_ERR_NOMEM         \
                                                     : MAGIC_SHT_ERR_CUDA,         \
                     "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),       \
                     __FILE__, __LINE__);                                          \
  } while (0)

#define TRY(x)               \
  do {                       \
    int _rc = (x);           \
    if (_rc) return _rc;     \
  } while (0)

extern "C" const char* magic_sht_last_error(void) { return g_err.c_str(); }

// ------------------------------------------------------------------ handle
struct magic_sht_handle {
  int device = 0;
  int precision = MAGIC_SHT_FP64;
  ShtGeom g{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool capturing = false;
  int* d_lmoff = nullptr;
  double2* d_tdcoef = nullptr;  // get_td coefficients [lm][4]
  int* d_tdlq = nullptr;        // [lm] l | m << 16
  double *d_theta = nullptr, *d_gauss = nullptr, *d_P = nullptr, *d_dP = nullptr;
  double *d_wgt = nullptr, *d_osin2 = nullptr;
  float *d_P32 = nullptr, *d_dP32 = nullptr;
  double2* d_tw64 = nullptr;
  float2* d_tw32 = nullptr;
  float4* d_twdf = nullptr;  // e^{+2 pi i k/P} as double-float (hi re, lo re, hi im, lo im)
  float4* d_twr = nullptr;   // the double-float fast path's twiddle tables in device memory (n_phi = 1536)
  short* d_inv_exp = nullptr;  // FP64-accurate tensor-core form: table row exponents
  short* d_fwd_exp = nullptr;
  double* d_cosn2 = nullptr;  // cos / sin^2 of the northern colatitudes (general get_nl)
  // tensor-core form: pre-split table images
  TcTables tct{};
  unsigned char* d_inv_img = nullptr;
  unsigned char* d_fwd_img = nullptr;
  long long* d_inv_blk0 = nullptr;
  long long* d_fwd_blk0 = nullptr;
  long long* d_bpc0 = nullptr;
  int* d_tile_ctr = nullptr;
  unsigned char* d_bimg = nullptr;  // data-operand images of the persistent tensor-core kernels
  size_t bimg_bytes = 0;
  float* d_inv_scale = nullptr;
  float* d_fwd_scale = nullptr;
  int* d_err = nullptr;
  bool tc_persistent = true;  // MAGIC_SHT_TC_KERNEL=tiled selects the one-tile-per-CTA kernels
  // runtime tuning (magic_sht_set_tuning): levels per host-pipeline chunk
  // (default 16: at l_max = 255, 8 measured 2% slower end to end and 4 5%
  // slower) and theta rows per CTA of the fast FFT (0 = by size); the
  // persistent kernels' tile order lives in tct.order
  int pipe_chunk = 16;
  int fft_rows = 0;
  char* ws = nullptr;
  size_t ws_bytes = 0;
  std::vector<int> lmoff;
  // host-buffer pipeline of the batched calls: two staging slots, two copy streams
  // Staging for the host-buffer pipeline: two pools that consecutive calls
  // alternate, so one call's host->device copies never wait for the previous
  // call's device->host copies.  A pool holds 2 chunk slots (synchronous
  // calls) or one slot per chunk (asynchronous calls: the uploads then run
  // ahead of the previous call's downloads instead of waiting for slot reuse).
  struct StagePool {
    char* buf = nullptr;
    size_t bytes = 0, stride = 0;
    std::vector<cudaEvent_t> ev_in, ev_comp, ev_out;
    std::vector<char> used;
  } pools[2];
  int pool = 0;
  cudaStream_t cpy_in = nullptr, cpy_out = nullptr;
  // magic_sht_set_host_async: pipelined host-buffer calls return once queued
  bool host_async = false;
  // pinned ring for small host inputs (per-level arrays such as or2, r,
  // lcut): their copies are issued from pinned memory, asynchronously, so a
  // call whose only host arrays are such inputs needs no synchronisation
  char* pin = nullptr;
  size_t pin_cap = 0, pin_off = 0;
  cudaEvent_t pin_ev = nullptr;
  // per-phase CUDA-event timing (magic_sht_set_profiling)
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_marks;
  double phase_ms[MAGIC_SHT_N_PHASES] = {0};
  long long phase_launches[MAGIC_SHT_N_PHASES] = {0};
  long long launches = 0;
  // a group call (magic_sht_group_*) collects this handle's tensor-core
  // Legendre and FFT launches here instead of issuing them; defer_bimg counts
  // the data-image bytes its collected Legendre launches need
  struct Deferred* defer = nullptr;
  size_t defer_bimg = 0;
};

// Launches of the handles of one group call, held back so that the Legendre
// launches of every instance run as one pack + one persistent kernel per kind.
struct Deferred {
  struct Leg {
    magic_sht_handle* h;
    bool inverse, vec;
    InvSet inv;
    FwdSet fwd;
    size_t bimg_off;  // in h->d_bimg
  };
  struct Fft {
    magic_sht_handle* h;
    bool inverse;
    FftSet fs;
  };
  std::vector<Leg> leg;
  std::vector<Fft> fft;
};

struct magic_sht_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {
// device address of the allocation-free entry point's static scratch (defined at the end of this file)
int noalloc_scratch(int dev, void** out);
}  // namespace

namespace {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

bool smooth235(int n) {
  if (n <= 0) return false;
  for (int f : {2, 3, 5})
    while (n % f == 0) n /= f;
  return n == 1;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int ensure_ws(magic_sht_handle* h, size_t bytes) {
  if (bytes <= h->ws_bytes) return MAGIC_SHT_OK;
  if (h->capturing)
    return set_err(MAGIC_SHT_ERR_NOMEM,
                   "workspace of %zu bytes needed during graph capture; call "
                   "magic_sht_reserve first",
                   bytes);
  if (h->ws) {
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaFree(h->ws));
    h->ws = nullptr;
    h->ws_bytes = 0;
  }
  const size_t nb = align256(bytes + bytes / 8);
  CK(cudaMalloc((void**)&h->ws, nb));
  h->ws_bytes = nb;
  return MAGIC_SHT_OK;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// page-locked host memory (cudaHostAlloc / cudaHostRegister): asynchronous copies from it do not block the host
bool is_pinned_host(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

bool fp64_pipes(const magic_sht_handle* h) { return h->precision == MAGIC_SHT_FP64; }
// the FP64-accurate tensor-core form: Legendre sums of fixed-point BF16 digits
// (or, with tc_kernel = 1, the FP64 SIMT sums) and double-float FFTs
// (also MAGIC_SHT_BF16X5: the same form with five digits per operand)
bool oz_form(const magic_sht_handle* h) {
  return h->precision == MAGIC_SHT_FP64TC || h->precision == MAGIC_SHT_BF16X5;
}
int oz_digits(const magic_sht_handle* h) { return h->precision == MAGIC_SHT_BF16X5 ? 5 : 7; }
// FP64 arithmetic in the SIMT Legendre sums and the radial-loop kernels
bool f64_sums(const magic_sht_handle* h) { return fp64_pipes(h) || oz_form(h); }
size_t t2_bytes(const magic_sht_handle* h) { return f64_sums(h) ? 16 : 8; }
int fft_arith(const magic_sht_handle* h) {
  return fp64_pipes(h) ? FFT_ARITH_F64 : oz_form(h) ? FFT_ARITH_DF : FFT_ARITH_F32;
}

size_t hs_bytes(const magic_sht_handle* h, int nlev) {
  return (size_t)nlev * h->g.n_m * h->g.n_theta * t2_bytes(h);
}

// Synthesis half spectra of a vector component in the tensor-core form hold
// E and F for both parities: twice the entries of the N/S layout.
// The split-product forms (3xBF16, 2xTF32) always; the FP64-accurate form when
// its tensor-core kernels run (tc_kernel = 0).
bool split_form(const magic_sht_handle* h) {
  return h->precision == MAGIC_SHT_BF16X3 || h->precision == MAGIC_SHT_TF32X2;
}
bool tc_form(const magic_sht_handle* h) { return split_form(h) || (oz_form(h) && h->tc_persistent); }
// FP64 half spectra between the FP64 SIMT Legendre sums and the double-float FFTs
int fft_hs_flag(const magic_sht_handle* h) { return (oz_form(h) && !h->tc_persistent) ? FFT_HS_F64 : 0; }
bool tf32_form(const magic_sht_handle* h) { return h->precision == MAGIC_SHT_TF32X2; }
// data-operand images of the persistent tensor-core kernels (grown like the workspace)
int ensure_bimg(magic_sht_handle* h, size_t bytes) {
  if (bytes <= h->bimg_bytes) return MAGIC_SHT_OK;
  if (h->capturing)
    return set_err(MAGIC_SHT_ERR_NOMEM,
                   "tensor-core data images of %zu bytes needed during graph capture; call "
                   "magic_sht_reserve first",
                   bytes);
  if (h->d_bimg) {
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaFree(h->d_bimg));
    h->d_bimg = nullptr;
    h->bimg_bytes = 0;
  }
  const size_t nb = align256(bytes);
  CK(cudaMalloc((void**)&h->d_bimg, nb));
  h->bimg_bytes = nb;
  return MAGIC_SHT_OK;
}
// a Legendre launch of a group call: recorded with its data-image offset
int defer_leg(magic_sht_handle* h, const InvSet* inv, const FwdSet* fwd, bool vec) {
  Deferred::Leg j{};
  j.h = h;
  j.inverse = inv != nullptr;
  j.vec = vec;
  if (inv) j.inv = *inv;
  if (fwd) j.fwd = *fwd;
  const int ncplx = inv ? inv->nf * inv->nlev * (vec ? 2 : 1) : fwd->nf * fwd->nlev * (vec ? 2 : 1);
  j.bimg_off = h->defer_bimg;
  h->defer_bimg += align256(oz_form(h) ? oz_data_bytes(h->g, h->tct, ncplx, inv != nullptr)
                                       : tcp_data_bytes(h->g, h->tct, ncplx, vec, inv != nullptr, tf32_form(h)));
  h->defer->leg.push_back(j);
  return MAGIC_SHT_OK;
}
int inv_tc(magic_sht_handle* h, const ShtGeom& g, const InvSet& s, bool vec) {
  if (h->defer) return defer_leg(h, &s, nullptr, vec);
  if (oz_form(h)) {
    TRY(ensure_bimg(h, oz_data_bytes(g, h->tct, s.nf * s.nlev * (vec ? 2 : 1), true)));
    h->launches++;  // pack kernel + persistent kernel
    CK(launch_inv_legendre_oz(g, s, vec, h->tct, h->d_bimg, h->stream));
    return MAGIC_SHT_OK;
  }
  if (!h->tc_persistent) {
    CK(launch_inv_legendre_tc(g, s, vec, h->tct, h->stream));
    return MAGIC_SHT_OK;
  }
  TRY(ensure_bimg(h, tcp_data_bytes(g, h->tct, s.nf * s.nlev * (vec ? 2 : 1), vec, true, tf32_form(h))));
  h->launches++;  // pack kernel + persistent kernel
  CK(launch_inv_legendre_tcp(g, s, vec, tf32_form(h), h->tct, h->d_bimg, h->stream));
  return MAGIC_SHT_OK;
}
int fwd_tc(magic_sht_handle* h, const ShtGeom& g, const FwdSet& s, bool vec) {
  if (h->defer) return defer_leg(h, nullptr, &s, vec);
  if (oz_form(h)) {
    TRY(ensure_bimg(h, oz_data_bytes(g, h->tct, s.nf * s.nlev * (vec ? 2 : 1), false)));
    h->launches++;  // pack kernel + persistent kernel
    CK(launch_fwd_legendre_oz(g, s, vec, h->tct, h->d_bimg, h->stream));
    return MAGIC_SHT_OK;
  }
  if (!h->tc_persistent) {
    CK(launch_fwd_legendre_tc(g, s, vec, h->tct, h->stream));
    return MAGIC_SHT_OK;
  }
  TRY(ensure_bimg(h, tcp_data_bytes(g, h->tct, s.nf * s.nlev * (vec ? 2 : 1), vec, false, tf32_form(h))));
  h->launches++;  // pack kernel + persistent kernel
  CK(launch_fwd_legendre_tcp(g, s, vec, tf32_form(h), h->tct, h->d_bimg, h->stream));
  return MAGIC_SHT_OK;
}
size_t hs_inv_bytes(const magic_sht_handle* h, int nlev, bool vec) {
  return hs_bytes(h, nlev) * ((vec && tc_form(h)) ? 2 : 1);
}
long long hs_inv_ld(const magic_sht_handle* h, bool vec) {
  return (long long)h->g.n_m * h->g.n_theta * ((vec && tc_form(h)) ? 2 : 1);
}

cudaEvent_t next_event(magic_sht_handle* h) {
  if (h->ev_used == h->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    h->ev_pool.push_back(e);
  }
  return h->ev_pool[h->ev_used++];
}

// Brackets one kernel launch: counts it and, when profiling, records an
// event pair on the launching stream.
struct PhaseScope {
  magic_sht_handle* h;
  int ph;
  cudaEvent_t e1 = nullptr;
  // `nk` kernels launched inside the scope (timed together)
  PhaseScope(magic_sht_handle* h_, int ph_, int nk = 1) : h(h_), ph(ph_) {
    if (h->defer) return;  // collected for a group launch: counted there
    h->launches += nk;
    h->phase_launches[ph] += nk;
    if (h->profiling && !h->capturing) {
      cudaEvent_t e0 = next_event(h);
      e1 = next_event(h);
      if (e0 && e1) {
        cudaEventRecord(e0, h->stream);
        h->ev_marks.push_back({ph, {e0, e1}});
      } else {
        e1 = nullptr;
      }
    }
  }
  ~PhaseScope() {
    if (e1) cudaEventRecord(e1, h->stream);
  }
};

constexpr size_t kPinRing = 1 << 20, kPinMax = 64 << 10;

// Copies a small host input into the pinned ring and returns its slot, or
// null (too large, or no pinned memory: the caller copies from the pageable
// array).  A slot is written again only after every copy of the previous lap
// has completed (all of them were issued on the handle's stream, and binding
// another stream synchronises the old one).
const void* pin_stage(magic_sht_handle* h, const void* src, size_t bytes) {
  const size_t need = (bytes + 255) & ~(size_t)255;
  if (need > kPinMax) return nullptr;
  if (!h->pin) {
    if (cudaHostAlloc((void**)&h->pin, kPinRing, cudaHostAllocDefault) != cudaSuccess) {
      h->pin = nullptr;
      cudaGetLastError();
      return nullptr;
    }
    if (cudaEventCreateWithFlags(&h->pin_ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaFreeHost(h->pin);
      h->pin = nullptr;
      h->pin_ev = nullptr;
      cudaGetLastError();
      return nullptr;
    }
    h->pin_cap = kPinRing;
    h->pin_off = 0;
  }
  if (h->pin_off + need > h->pin_cap) {
    if (cudaEventRecord(h->pin_ev, h->stream) != cudaSuccess || cudaEventSynchronize(h->pin_ev) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    h->pin_off = 0;
  }
  char* p = h->pin + h->pin_off;
  memcpy(p, src, bytes);
  h->pin_off += need;
  return p;
}

// One call's device buffers: host arrays are staged, device arrays are used
// in place, temporaries come from the handle's workspace.  Small host inputs
// of raw_in go through the pinned ring; a call with any other host array
// synchronises its stream before returning.
class CallCtx {
 public:
  enum Kind { IN = 0, OUT = 1, TMP = 2, INOUT = 3 };
  CallCtx(magic_sht_handle* h) : h_(h) {}

  // grid arrays: nlev levels of n_phi rows of ld doubles, level stride `lds`
  int grid_in(const double* p, int nlev, long long lds) { return add(p, IN, nlev, lds, true); }
  int grid_out(double* p, int nlev, long long lds) { return add(p, OUT, nlev, lds, true); }
  // spectral arrays: nlev levels of lm_max complex, level stride `lds` complex
  int spec_in(const double* p, int nlev, long long lds) { return add(p, IN, nlev, lds, false); }
  int spec_out(double* p, int nlev, long long lds) { return add(p, OUT, nlev, lds, false); }
  int raw_in(const void* p, size_t bytes) {
    Ent e;
    e.host = p; e.kind = IN; e.bytes = bytes; e.raw = true;
    ents_.push_back(e);
    return (int)ents_.size() - 1;
  }
  // staged in before the kernels and back after them when `p` is host memory
  int raw_inout(void* p, size_t bytes) {
    Ent e;
    e.host = p; e.kind = INOUT; e.bytes = bytes; e.raw = true;
    ents_.push_back(e);
    return (int)ents_.size() - 1;
  }
  int tmp(size_t bytes) {
    Ent e;
    e.kind = TMP; e.bytes = bytes;
    ents_.push_back(e);
    return (int)ents_.size() - 1;
  }

  int prepare() {
    size_t total = 0;
    bool host = false;
    for (auto& e : ents_) {
      if (e.kind != TMP) e.is_dev = is_device_ptr(e.host);
      if (e.kind == TMP || !e.is_dev) total += align256(e.bytes);
      if (e.kind != TMP && !e.is_dev && e.host) host = true;
    }
    if (host && h_->capturing)
      return set_err(MAGIC_SHT_ERR_ARG, "host arrays in a captured call: pass device arrays while capturing");
    TRY(ensure_ws(h_, total));
    size_t off = 0;
    for (auto& e : ents_) {
      if (e.kind != TMP && e.is_dev) {
        e.dev = const_cast<void*>(e.host);
        continue;
      }
      e.dev = h_->ws + off;
      off += align256(e.bytes);
      if (e.kind == TMP) continue;
      const void* src = (e.raw && e.kind == IN && e.bytes) ? pin_stage(h_, e.host, e.bytes) : nullptr;
      if (!src) any_host_ = true;
      if ((e.kind == IN || e.kind == INOUT) && e.bytes)
        CK(cudaMemcpyAsync(e.dev, src ? src : e.host, e.bytes, cudaMemcpyHostToDevice, h_->stream));
    }
    return MAGIC_SHT_OK;
  }

  void* dev(int i) const { return i < 0 ? nullptr : ents_[i].dev; }

  int finish() {
    const ShtGeom& g = h_->g;
    for (auto& e : ents_) {
      if ((e.kind != OUT && e.kind != INOUT) || e.is_dev || !e.host) continue;
      if (e.grid && g.ld > g.n_theta) {
        for (int r = 0; r < e.nlev; ++r)
          CK(cudaMemcpy2DAsync((char*)e.host + (size_t)r * e.lds * 8, (size_t)g.ld * 8,
                               (char*)e.dev + (size_t)r * e.lds * 8, (size_t)g.ld * 8,
                               (size_t)g.n_theta * 8, g.n_phi, cudaMemcpyDeviceToHost, h_->stream));
      } else {
        CK(cudaMemcpyAsync(const_cast<void*>(e.host), e.dev, e.bytes, cudaMemcpyDeviceToHost, h_->stream));
      }
    }
    if (any_host_) CK(cudaStreamSynchronize(h_->stream));
    return MAGIC_SHT_OK;
  }

 private:
  struct Ent {
    const void* host = nullptr;
    void* dev = nullptr;
    size_t bytes = 0;
    int kind = 0;
    bool is_dev = false;
    bool grid = false;
    bool raw = false;
    int nlev = 0;
    long long lds = 0;
  };
  int add(const void* p, int kind, int nlev, long long lds, bool grid) {
    if (!p) return -1;
    const ShtGeom& g = h_->g;
    Ent e;
    e.host = p; e.kind = kind; e.grid = grid; e.nlev = nlev; e.lds = lds;
    const size_t last = grid ? (size_t)g.n_phi * g.ld * 8 : (size_t)g.lm_max * 16;
    const size_t unit = grid ? 8 : 16;
    e.bytes = (size_t)(nlev - 1) * (size_t)lds * unit + last;
    ents_.push_back(e);
    return (int)ents_.size() - 1;
  }
  magic_sht_handle* h_;
  std::vector<Ent> ents_;
  bool any_host_ = false;
};

// ---------------------------------------------------------- transform jobs
struct SpecRef {  // operand: op(A, B) with ctx indices
  int op = OP_ZERO;
  int a = -1, b = -1;
};
struct ScalarInv { SpecRef x; int out = -1; int flags = 0; };
struct VectorInv { SpecRef s, t; int out_t = -1, out_p = -1; int flags = 0; };
struct ScalarFwd { int in = -1; int out = -1; };
struct VectorFwd { int in_t = -1, in_p = -1; int out_s = -1, out_t = -1; };

struct LevelCtl {
  int nlev = 1;
  int lcut0 = 0;
  double or2_0 = 0.0;
  int lcut_idx = -1;  // ctx index of device int[nlev]
  int or2_idx = -1;
  long long spec_ld = 0;  // complex
  long long grid_ld = 0;  // doubles
};

SpecOperand make_operand(const CallCtx& cx, const SpecRef& r, long long ld) {
  SpecOperand o;
  o.A = (const double2*)cx.dev(r.a);
  o.B = (const double2*)cx.dev(r.b);
  o.ld = ld;
  o.op = (r.a < 0) ? OP_ZERO : r.op;
  o.pad_ = 0;
  return o;
}

// Synthesis: Legendre sums into half spectra, then inverse FFTs.  The
// half-spectrum temporaries must have been registered in `cx` before
// prepare(); `hs` holds their ctx indices (one per output grid, in order).
int run_inverse(magic_sht_handle* h, CallCtx& cx, const LevelCtl& lv,
                const std::vector<ScalarInv>& sc, const std::vector<VectorInv>& vc,
                const std::vector<int>& hs_sc, const std::vector<int>& hs_vc) {
  const ShtGeom& g = h->g;
  const long long hs_ld = hs_inv_ld(h, false), hs_ld_v = hs_inv_ld(h, true);
  const int hsf = fft_hs_flag(h);
  const int flag_s = (tc_form(h) ? FFT_IN_E : 0) | hsf, flag_v = (tc_form(h) ? FFT_IN_EF : 0) | hsf;
  const bool f64 = f64_sums(h);
  const int* d_lcut = (const int*)cx.dev(lv.lcut_idx);
  const double* d_or2 = (const double*)cx.dev(lv.or2_idx);
  FftSet fs{};
  fs.nlev = lv.nlev;
  auto flush_fft = [&]() -> int {
    if (fs.nf && h->defer) {
      h->defer->fft.push_back({h, true, fs});
      fs.nf = 0;
    }
    if (fs.nf) {
      PhaseScope ps(h, MAGIC_SHT_PHASE_FFT_INV);
      CK(launch_fft_inverse(g, fs, fft_arith(h), h->fft_rows, h->stream));
      fs.nf = 0;
    }
    return MAGIC_SHT_OK;
  };
  auto add_fft = [&](void* in, int out_idx, int flags, long long in_ld) -> int {
    if (fs.nf == MAGIC_MAX_FIELDS) TRY(flush_fft());
    FftField& f = fs.f[fs.nf++];
    f.in = in; f.out = cx.dev(out_idx); f.in_ld = in_ld; f.out_ld = lv.grid_ld;
    f.flags = flags; f.pad_ = 0;
    return MAGIC_SHT_OK;
  };
  for (size_t i0 = 0; i0 < sc.size(); i0 += MAGIC_MAX_FIELDS) {
    InvSet s{};
    s.nlev = lv.nlev; s.lcut = d_lcut; s.or2 = d_or2; s.lcut0 = lv.lcut0; s.or2_0 = lv.or2_0;
    for (size_t i = i0; i < sc.size() && i < i0 + MAGIC_MAX_FIELDS; ++i) {
      InvField& f = s.f[s.nf++];
      f.x0 = make_operand(cx, sc[i].x, lv.spec_ld);
      f.x1 = SpecOperand{nullptr, nullptr, 0, OP_ZERO, 0};
      f.out0 = cx.dev(hs_sc[i]); f.out1 = nullptr; f.out_ld = hs_ld;
    }
    PhaseScope ps(h, MAGIC_SHT_PHASE_INV_LEG_SCALAR);
    if (tc_form(h)) TRY(inv_tc(h, g, s, false));
    else CK(launch_inv_legendre_simt(g, s, false, f64, h->stream));
  }
  for (size_t i0 = 0; i0 < vc.size(); i0 += MAGIC_MAX_FIELDS) {
    InvSet s{};
    s.nlev = lv.nlev; s.lcut = d_lcut; s.or2 = d_or2; s.lcut0 = lv.lcut0; s.or2_0 = lv.or2_0;
    for (size_t i = i0; i < vc.size() && i < i0 + MAGIC_MAX_FIELDS; ++i) {
      InvField& f = s.f[s.nf++];
      f.x0 = make_operand(cx, vc[i].s, lv.spec_ld);
      f.x1 = make_operand(cx, vc[i].t, lv.spec_ld);
      f.out0 = cx.dev(hs_vc[2 * i]); f.out1 = cx.dev(hs_vc[2 * i + 1]); f.out_ld = hs_ld_v;
    }
    PhaseScope ps(h, MAGIC_SHT_PHASE_INV_LEG_VECTOR);
    if (tc_form(h)) TRY(inv_tc(h, g, s, true));
    else CK(launch_inv_legendre_simt(g, s, true, f64, h->stream));
  }
  for (size_t i = 0; i < sc.size(); ++i) TRY(add_fft(cx.dev(hs_sc[i]), sc[i].out, sc[i].flags | flag_s, hs_ld));
  for (size_t i = 0; i < vc.size(); ++i) {
    TRY(add_fft(cx.dev(hs_vc[2 * i]), vc[i].out_t, vc[i].flags | flag_v, hs_ld_v));
    TRY(add_fft(cx.dev(hs_vc[2 * i + 1]), vc[i].out_p, vc[i].flags | flag_v, hs_ld_v));
  }
  return flush_fft();
}

// Vector Legendre analysis of the radial set (after the vector FFTs).
int run_forward_vectors(magic_sht_handle* h, CallCtx& cx, const LevelCtl& lv, const std::vector<VectorFwd>& vc,
                        const std::vector<int>& hs_vc, const int* d_lcut) {
  const ShtGeom& g = h->g;
  const long long hs_ld = (long long)g.n_m * g.n_theta;
  const bool f64 = f64_sums(h);
  for (size_t i0 = 0; i0 < vc.size(); i0 += MAGIC_MAX_FIELDS) {
    FwdSet s{};
    s.nlev = lv.nlev; s.lcut = d_lcut; s.lcut0 = lv.lcut0;
    for (size_t i = i0; i < vc.size() && i < i0 + MAGIC_MAX_FIELDS; ++i) {
      FwdField& f = s.f[s.nf++];
      // F1 from v_phi, F2 from v_theta (the crossing of shtransforms.f90:764-767)
      f.in0 = cx.dev(hs_vc[2 * i + 1]); f.in1 = cx.dev(hs_vc[2 * i]); f.in_ld = hs_ld;
      f.out0 = (double2*)cx.dev(vc[i].out_s); f.out1 = (double2*)cx.dev(vc[i].out_t);
      f.out_ld = lv.spec_ld;
    }
    PhaseScope ps(h, MAGIC_SHT_PHASE_FWD_LEG_VECTOR);
    if (tc_form(h)) TRY(fwd_tc(h, g, s, true));
    else CK(launch_fwd_legendre_simt(g, s, true, f64, h->stream));
  }
  return MAGIC_SHT_OK;
}

// Analysis: forward FFTs into ES/EA half spectra, then Legendre sums.
int run_forward(magic_sht_handle* h, CallCtx& cx, const LevelCtl& lv,
                const std::vector<ScalarFwd>& sc, const std::vector<VectorFwd>& vc,
                const std::vector<int>& hs_sc, const std::vector<int>& hs_vc) {
  const ShtGeom& g = h->g;
  const long long hs_ld = (long long)g.n_m * g.n_theta;
  const bool f64 = f64_sums(h);
  const int hsf = fft_hs_flag(h);
  const int* d_lcut = (const int*)cx.dev(lv.lcut_idx);
  FftSet fs{};
  fs.nlev = lv.nlev;
  auto flush_fft = [&]() -> int {
    if (fs.nf && h->defer) {
      h->defer->fft.push_back({h, false, fs});
      fs.nf = 0;
    }
    if (fs.nf) {
      PhaseScope ps(h, MAGIC_SHT_PHASE_FFT_FWD);
      CK(launch_fft_forward(g, fs, fft_arith(h), h->fft_rows, h->stream));
      fs.nf = 0;
    }
    return MAGIC_SHT_OK;
  };
  auto add_fft = [&](int in_idx, void* out, int flags) -> int {
    if (fs.nf == MAGIC_MAX_FIELDS) TRY(flush_fft());
    FftField& f = fs.f[fs.nf++];
    f.in = cx.dev(in_idx); f.out = out; f.in_ld = lv.grid_ld; f.out_ld = hs_ld;
    f.flags = flags; f.pad_ = 0;
    return MAGIC_SHT_OK;
  };
  for (size_t i = 0; i < sc.size(); ++i) TRY(add_fft(sc[i].in, cx.dev(hs_sc[i]), FFT_WEIGHT | hsf));
  for (size_t i = 0; i < vc.size(); ++i) {
    TRY(add_fft(vc[i].in_t, cx.dev(hs_vc[2 * i]), FFT_WEIGHT | FFT_OSIN2 | hsf));
    TRY(add_fft(vc[i].in_p, cx.dev(hs_vc[2 * i + 1]), FFT_WEIGHT | FFT_OSIN2 | hsf));
  }
  TRY(flush_fft());
  for (size_t i0 = 0; i0 < sc.size(); i0 += MAGIC_MAX_FIELDS) {
    FwdSet s{};
    s.nlev = lv.nlev; s.lcut = d_lcut; s.lcut0 = lv.lcut0;
    for (size_t i = i0; i < sc.size() && i < i0 + MAGIC_MAX_FIELDS; ++i) {
      FwdField& f = s.f[s.nf++];
      f.in0 = cx.dev(hs_sc[i]); f.in1 = nullptr; f.in_ld = hs_ld;
      f.out0 = (double2*)cx.dev(sc[i].out); f.out1 = nullptr; f.out_ld = lv.spec_ld;
    }
    PhaseScope ps(h, MAGIC_SHT_PHASE_FWD_LEG_SCALAR);
    if (tc_form(h)) TRY(fwd_tc(h, g, s, false));
    else CK(launch_fwd_legendre_simt(g, s, false, f64, h->stream));
  }
  return run_forward_vectors(h, cx, lv, vc, hs_vc, d_lcut);
}

int check_handle(const magic_sht_handle* h) {
  if (!h) return set_err(MAGIC_SHT_ERR_ARG, "null handle");
  return MAGIC_SHT_OK;
}

int check_lcut(const magic_sht_handle* h, int lcut) {
  if (lcut < 0 || lcut > h->g.l_max)
    return set_err(MAGIC_SHT_ERR_LCUT, "lcut=%d outside [0, l_max=%d]", lcut, h->g.l_max);
  return MAGIC_SHT_OK;
}



// Single-level synthesis helper.
int inverse_one(magic_sht_handle* h, int lcut, double or2, const std::vector<const double*>& specs,
                const std::vector<double*>& grids,
                // builds the jobs from ctx indices of specs / grids
                void (*build)(const std::vector<int>&, const std::vector<int>&,
                              std::vector<ScalarInv>&, std::vector<VectorInv>&)) {
  TRY(check_handle(h));
  TRY(check_lcut(h, lcut));
  for (auto p : specs) if (!p) return set_err(MAGIC_SHT_ERR_ARG, "null spectral pointer");
  for (auto p : grids) if (!p) return set_err(MAGIC_SHT_ERR_ARG, "null grid pointer");
  DeviceGuard dg(h->device);
  CallCtx cx(h);
  std::vector<int> si, gi;
  for (auto p : specs) si.push_back(cx.spec_in(p, 1, h->g.lm_max));
  for (auto p : grids) gi.push_back(cx.grid_out(p, 1, (long long)h->g.n_phi * h->g.ld));
  std::vector<ScalarInv> sc;
  std::vector<VectorInv> vc;
  build(si, gi, sc, vc);
  std::vector<int> hs_sc, hs_vc;
  for (size_t i = 0; i < sc.size(); ++i) hs_sc.push_back(cx.tmp(hs_bytes(h, 1)));
  for (size_t i = 0; i < 2 * vc.size(); ++i) hs_vc.push_back(cx.tmp(hs_inv_bytes(h, 1, true)));
  TRY(cx.prepare());
  LevelCtl lv;
  lv.nlev = 1; lv.lcut0 = lcut; lv.or2_0 = or2;
  lv.spec_ld = h->g.lm_max; lv.grid_ld = (long long)h->g.n_phi * h->g.ld;
  TRY(run_inverse(h, cx, lv, sc, vc, hs_sc, hs_vc));
  return cx.finish();
}

int forward_one(magic_sht_handle* h, int lcut, const std::vector<const double*>& grids,
                const std::vector<double*>& specs,
                void (*build)(const std::vector<int>&, const std::vector<int>&,
                              std::vector<ScalarFwd>&, std::vector<VectorFwd>&)) {
  TRY(check_handle(h));
  TRY(check_lcut(h, lcut));
  for (auto p : specs) if (!p) return set_err(MAGIC_SHT_ERR_ARG, "null spectral pointer");
  for (auto p : grids) if (!p) return set_err(MAGIC_SHT_ERR_ARG, "null grid pointer");
  DeviceGuard dg(h->device);
  CallCtx cx(h);
  std::vector<int> gi, si;
  for (auto p : grids) gi.push_back(cx.grid_in(p, 1, (long long)h->g.n_phi * h->g.ld));
  for (auto p : specs) si.push_back(cx.spec_out(p, 1, h->g.lm_max));
  std::vector<ScalarFwd> sc;
  std::vector<VectorFwd> vc;
  build(gi, si, sc, vc);
  std::vector<int> hs_sc, hs_vc;
  for (size_t i = 0; i < sc.size(); ++i) hs_sc.push_back(cx.tmp(hs_bytes(h, 1)));
  for (size_t i = 0; i < 2 * vc.size(); ++i) hs_vc.push_back(cx.tmp(hs_bytes(h, 1)));
  TRY(cx.prepare());
  LevelCtl lv;
  lv.nlev = 1; lv.lcut0 = lcut;
  lv.spec_ld = h->g.lm_max; lv.grid_ld = (long long)h->g.n_phi * h->g.ld;
  TRY(run_forward(h, cx, lv, sc, vc, hs_sc, hs_vc));
  return cx.finish();
}

SpecRef ref(int op, int a, int b = -1) {
  SpecRef r;
  r.op = op; r.a = a; r.b = b;
  return r;
}

__global__ void ic_prescale_kernel(int K, const int* __restrict__ lm2l, const double* __restrict__ ca,
                                   const double* __restrict__ cb, const double2* __restrict__ A,
                                   const double2* __restrict__ B, double2* __restrict__ X) {
  const int lm = blockIdx.x * blockDim.x + threadIdx.x;
  if (lm >= K) return;
  const int l = lm2l[lm];
  const double2 a = A[lm];
  double2 x = make_double2(ca[l] * a.x, ca[l] * a.y);
  if (B) {
    const double2 b = B[lm];
    x.x += cb[l] * b.x;
    x.y += cb[l] * b.y;
  }
  X[lm] = x;
}

__global__ void axi_kernel(int l_max, int nh, const double* __restrict__ P, const double* __restrict__ dP,
                           const double2* __restrict__ S, int lcut, int tor, double* a, double* b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nh) return;
  // m = 0 block occupies lm = 0..l_max (native_axi_to_spat, shtransforms.f90:374-403;
  // native_toraxi_to_spat, :405-491).  Only real parts enter for m = 0.
  double es = 0.0, ea = 0.0;
  for (int l = 0; l <= l_max; ++l) {
    if (tor && l > lcut) continue;
    const double v = S[l].x * (tor ? dP[(size_t)l * nh + j] : P[(size_t)l * nh + j]);
    if (l & 1) ea += v; else es += v;
  }
  if (!tor) {
    a[2 * j] = es + ea;
    a[2 * j + 1] = es - ea;
  } else {
    // bhG = -iT, bhC = iT: the theta component cancels, v_phi = -sum T dP
    // with dP odd under theta -> pi - theta for even l.
    a[2 * j] = 0.0;
    a[2 * j + 1] = 0.0;
    b[2 * j] = -(es + ea);
    b[2 * j + 1] = es - ea;
  }
}

}  // namespace

// ============================================================ public ABI ==
extern "C" {

int magic_sht_init(const magic_sht_desc* d, magic_sht_handle** out) {
  if (!d || !out) return set_err(MAGIC_SHT_ERR_ARG, "null descriptor or output pointer");
  *out = nullptr;
  const int L = d->l_max, minc = d->minc, N = d->n_theta_max, P = d->n_phi_max;
  if (L < 1 || L > 32767) return set_err(MAGIC_SHT_ERR_SIZE, "l_max=%d must be in [1, 32767]", L);
  if (minc < 1) return set_err(MAGIC_SHT_ERR_SIZE, "minc=%d must be > 0", minc);
  if (N <= 2 || N % 4) return set_err(MAGIC_SHT_ERR_SIZE, "n_theta_max=%d must be a multiple of 4 and > 2", N);
  if (P % 4 || P / 2 <= 2) return set_err(MAGIC_SHT_ERR_SIZE, "n_phi_max=%d must be a multiple of 4 and > 4", P);
  if (!smooth235(P)) return set_err(MAGIC_SHT_ERR_SIZE, "n_phi_max=%d must factor into 2, 3 and 5", P);
  int m_max = d->m_max > 0 ? d->m_max : (L / minc) * minc;
  if (m_max > L) m_max = L;
  if (m_max % minc) return set_err(MAGIC_SHT_ERR_SIZE, "m_max=%d not a multiple of minc=%d", m_max, minc);
  const int n_m = m_max / minc + 1;
  if (n_m > P / 2) return set_err(MAGIC_SHT_ERR_SIZE, "m_max/minc+1=%d exceeds n_phi_max/2=%d (aliasing)", n_m, P / 2);
  const int ld = d->nlat_padded > 0 ? d->nlat_padded : N;
  if (ld < N) return set_err(MAGIC_SHT_ERR_SIZE, "nlat_padded=%d < n_theta_max=%d", ld, N);
  if (d->precision != MAGIC_SHT_FP64 && d->precision != MAGIC_SHT_FP32 && d->precision != MAGIC_SHT_BF16X3 &&
      d->precision != MAGIC_SHT_TF32X2 && d->precision != MAGIC_SHT_FP64TC && d->precision != MAGIC_SHT_BF16X5)
    return set_err(MAGIC_SHT_ERR_ARG, "unknown precision %d", d->precision);

  int dev = d->device;
  if (dev < 0) CK(cudaGetDevice(&dev));
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (dev >= ndev) return set_err(MAGIC_SHT_ERR_ARG, "device %d not present (%d devices)", dev, ndev);
  DeviceGuard dg(dev);
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev));
  if (prop.major < 10)
    return set_err(MAGIC_SHT_ERR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a",
                   dev, prop.major, prop.minor);

  magic_sht_handle* h = new magic_sht_handle();
  h->device = dev;
  h->precision = d->precision;
  ShtGeom& g = h->g;
  g.l_max = L; g.m_max = m_max; g.minc = minc; g.n_m = n_m;
  g.n_theta = N; g.nh = N / 2; g.n_phi = P; g.ld = ld;
  h->lmoff.resize(n_m);
  int K = 0;
  for (int mc = 0; mc < n_m; ++mc) { h->lmoff[mc] = K; K += L - mc * minc + 1; }
  g.lm_max = K;
  int rc = MAGIC_SHT_OK;
  auto fail = [&](int code) { magic_sht_finalize(h); return code; };
  cudaError_t e;
#define INIT_CK(x)                                                                     \
  do {                                                                                 \
    e = (x);                                                                           \
    if (e != cudaSuccess) {                                                            \
      rc = set_err(e == cudaErrorMemoryAllocation ? MAGIC_SHT_ERR_NOMEM : MAGIC_SHT_ERR_CUDA, \
                   "init: %s: %s", #x, cudaGetErrorString(e));                         \
      return fail(rc);                                                                 \
    }                                                                                  \
  } while (0)
  INIT_CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  h->own_stream = true;
  const size_t tab = (size_t)K * g.nh;
  INIT_CK(cudaMalloc((void**)&h->d_lmoff, sizeof(int) * n_m));
  INIT_CK(cudaMalloc((void**)&h->d_theta, sizeof(double) * N));
  INIT_CK(cudaMalloc((void**)&h->d_gauss, sizeof(double) * N));
  INIT_CK(cudaMalloc((void**)&h->d_wgt, sizeof(double) * g.nh));
  INIT_CK(cudaMalloc((void**)&h->d_osin2, sizeof(double) * g.nh));
  INIT_CK(cudaMalloc((void**)&h->d_P, sizeof(double) * tab));
  INIT_CK(cudaMalloc((void**)&h->d_dP, sizeof(double) * tab));
  INIT_CK(cudaMalloc((void**)&h->d_tw64, sizeof(double2) * P));
  INIT_CK(cudaMalloc((void**)&h->d_tw32, sizeof(float2) * P));
  INIT_CK(cudaMalloc((void**)&h->d_twdf, sizeof(float4) * P));
  if (h->precision == MAGIC_SHT_FP32) {
    INIT_CK(cudaMalloc((void**)&h->d_P32, sizeof(float) * tab));
    INIT_CK(cudaMalloc((void**)&h->d_dP32, sizeof(float) * tab));
  }
  INIT_CK(cudaMalloc((void**)&h->d_tdcoef, sizeof(double2) * 4 * (size_t)K));
  INIT_CK(cudaMalloc((void**)&h->d_tdlq, sizeof(int) * (size_t)K));
  INIT_CK(cudaMalloc((void**)&h->d_err, sizeof(int)));
  INIT_CK(cudaMemset(h->d_err, 0, sizeof(int)));
  INIT_CK(cudaMemcpyAsync(h->d_lmoff, h->lmoff.data(), sizeof(int) * n_m, cudaMemcpyHostToDevice, h->stream));
  {
    std::vector<double2> tw(P);
    std::vector<float2> tw32(P);
    std::vector<float4> twdf(P);
    for (int k = 0; k < P; ++k) {
      const long double a = 2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)P;
      tw[k] = make_double2((double)cosl(a), (double)sinl(a));
      tw32[k] = make_float2((float)tw[k].x, (float)tw[k].y);
      const float ch = (float)cosl(a), sh = (float)sinl(a);
      twdf[k] = make_float4(ch, (float)(cosl(a) - (long double)ch), sh, (float)(sinl(a) - (long double)sh));
    }
    INIT_CK(cudaMemcpyAsync(h->d_tw64, tw.data(), sizeof(double2) * P, cudaMemcpyHostToDevice, h->stream));
    INIT_CK(cudaMemcpyAsync(h->d_tw32, tw32.data(), sizeof(float2) * P, cudaMemcpyHostToDevice, h->stream));
    INIT_CK(cudaMemcpyAsync(h->d_twdf, twdf.data(), sizeof(float4) * P, cudaMemcpyHostToDevice, h->stream));
    const std::vector<float4> twr = fft_df_global_twiddles(P, twdf);
    if (!twr.empty()) {
      INIT_CK(cudaMalloc((void**)&h->d_twr, sizeof(float4) * twr.size()));
      INIT_CK(cudaMemcpyAsync(h->d_twr, twr.data(), sizeof(float4) * twr.size(), cudaMemcpyHostToDevice,
                              h->stream));
    }
    INIT_CK(cudaStreamSynchronize(h->stream));
  }
  INIT_CK(build_tables_fp64(L, m_max, minc, N, h->d_lmoff, h->d_theta, h->d_gauss, h->d_P, h->d_dP,
                            h->d_wgt, h->d_osin2, h->stream));
  if (h->precision == MAGIC_SHT_FP32)
    INIT_CK(convert_tables_fp32(h->d_P, h->d_dP, h->d_P32, h->d_dP32, tab, h->stream));
  g.lmoff = h->d_lmoff;
  INIT_CK(build_td_coef(g, h->d_tdcoef, h->d_tdlq, h->stream));
  INIT_CK(cudaMalloc((void**)&h->d_cosn2, sizeof(double) * g.nh));
  INIT_CK(build_cosn2(g, h->d_theta, h->d_cosn2, h->stream));
  INIT_CK(cudaStreamSynchronize(h->stream));
  g.P64 = h->d_P; g.dP64 = h->d_dP; g.P32 = h->d_P32; g.dP32 = h->d_dP32;
  g.wgt = h->d_wgt; g.osin2 = h->d_osin2; g.tw64 = h->d_tw64; g.tw32 = h->d_tw32; g.twdf = h->d_twdf;
  g.twr = h->d_twr;
  if (oz_form(h)) {
    if (prop.major != 10)
      return fail(set_err(MAGIC_SHT_ERR_UNSUPPORTED, "the tensor-core form needs tcgen05 (sm_10x)"));
    h->tc_persistent = true;
    TcTables& t = h->tct;
    std::vector<long long> ib, fb;
    long long ninv = 0, nfwd = 0;
    t.ndig = oz_digits(h);
    oz_table_layout(g, t.ndig, &t.ntt, &t.nlt, &t.ncj, ib, fb, &ninv, &nfwd);
    INIT_CK(cudaMalloc((void**)&h->d_inv_img, (size_t)ninv * 16384));
    INIT_CK(cudaMalloc((void**)&h->d_fwd_img, (size_t)nfwd * 16384));
    INIT_CK(cudaMalloc((void**)&h->d_inv_blk0, sizeof(long long) * n_m));
    INIT_CK(cudaMalloc((void**)&h->d_fwd_blk0, sizeof(long long) * n_m));
    INIT_CK(cudaMalloc((void**)&h->d_inv_exp, sizeof(short) * 2 * n_m * t.ntt * 128));
    INIT_CK(cudaMalloc((void**)&h->d_fwd_exp, sizeof(short) * 2 * (size_t)K));
    INIT_CK(cudaMemcpy(h->d_inv_blk0, ib.data(), sizeof(long long) * n_m, cudaMemcpyHostToDevice));
    INIT_CK(cudaMemcpy(h->d_fwd_blk0, fb.data(), sizeof(long long) * n_m, cudaMemcpyHostToDevice));
    std::vector<long long> pc(n_m);
    t.npc = 0;
    for (int mc = 0; mc < n_m; ++mc) {
      pc[mc] = t.npc;
      t.npc += 2LL * tc_nch(L - mc * minc + 1);
    }
    INIT_CK(cudaMalloc((void**)&h->d_bpc0, sizeof(long long) * n_m));
    INIT_CK(cudaMalloc((void**)&h->d_tile_ctr, 256));
    t.tile_ctr = h->d_tile_ctr;
    INIT_CK(cudaMemcpy(h->d_bpc0, pc.data(), sizeof(long long) * n_m, cudaMemcpyHostToDevice));
    t.bpc0 = h->d_bpc0;
    INIT_CK(cudaMemset(h->d_fwd_exp, 0, sizeof(short) * 2 * (size_t)K));
    t.inv_img = h->d_inv_img; t.fwd_img = h->d_fwd_img;
    t.inv_blk0 = h->d_inv_blk0; t.fwd_blk0 = h->d_fwd_blk0;
    t.inv_exp = h->d_inv_exp; t.fwd_exp = h->d_fwd_exp;
    t.err = h->d_err;
    INIT_CK(build_oz_images(g, t, h->d_inv_img, h->d_inv_exp, h->d_fwd_img, h->d_fwd_exp, h->stream));
    INIT_CK(cudaStreamSynchronize(h->stream));
  }
  if (split_form(h)) {
    if (prop.major != 10)
      return fail(set_err(MAGIC_SHT_ERR_UNSUPPORTED, "the tensor-core form needs tcgen05 (sm_10x)"));
    const char* kern = getenv("MAGIC_SHT_TC_KERNEL");
    // the TF32 form exists only in the persistent kernels
    h->tc_persistent = tf32_form(h) || !(kern && strcmp(kern, "tiled") == 0);
    TcTables& t = h->tct;
    std::vector<long long> ib, fb;
    long long ninv = 0, nfwd = 0;
    tc_table_layout(g, tf32_form(h), &t.ntt, &t.nlt, &t.ncj, ib, fb, &ninv, &nfwd);
    INIT_CK(cudaMalloc((void**)&h->d_inv_img, (size_t)ninv * 16384));
    INIT_CK(cudaMalloc((void**)&h->d_fwd_img, (size_t)nfwd * 16384));
    INIT_CK(cudaMalloc((void**)&h->d_inv_blk0, sizeof(long long) * n_m));
    INIT_CK(cudaMalloc((void**)&h->d_fwd_blk0, sizeof(long long) * n_m));
    INIT_CK(cudaMalloc((void**)&h->d_inv_scale, sizeof(float) * 2 * n_m * t.ntt * 128));
    INIT_CK(cudaMalloc((void**)&h->d_fwd_scale, sizeof(float) * 2 * (size_t)K));
    INIT_CK(cudaMemcpy(h->d_inv_blk0, ib.data(), sizeof(long long) * n_m, cudaMemcpyHostToDevice));
    INIT_CK(cudaMemcpy(h->d_fwd_blk0, fb.data(), sizeof(long long) * n_m, cudaMemcpyHostToDevice));
    std::vector<long long> pc(n_m);
    t.npc = 0;
    for (int mc = 0; mc < n_m; ++mc) {
      pc[mc] = t.npc;
      t.npc += 2LL * tc_nch(L - mc * minc + 1);
    }
    INIT_CK(cudaMalloc((void**)&h->d_bpc0, sizeof(long long) * n_m));
    INIT_CK(cudaMalloc((void**)&h->d_tile_ctr, 256));
    t.tile_ctr = h->d_tile_ctr;
    INIT_CK(cudaMemcpy(h->d_bpc0, pc.data(), sizeof(long long) * n_m, cudaMemcpyHostToDevice));
    t.bpc0 = h->d_bpc0;
    INIT_CK(cudaMemset(h->d_fwd_scale, 0, sizeof(float) * 2 * (size_t)K));
    t.inv_img = h->d_inv_img; t.fwd_img = h->d_fwd_img;
    t.inv_blk0 = h->d_inv_blk0; t.fwd_blk0 = h->d_fwd_blk0;
    t.inv_scale = h->d_inv_scale; t.fwd_scale = h->d_fwd_scale;
    t.err = h->d_err;
    INIT_CK(build_tc_images(g, t, tf32_form(h), h->d_inv_img, h->d_inv_scale, h->d_fwd_img, h->d_fwd_scale,
                            h->stream));
    INIT_CK(cudaStreamSynchronize(h->stream));
  }
#undef INIT_CK
  {
    // Load this file's module on the device now and resolve the static
    // scratch of magic_sht_scal_to_spat_noalloc: with lazy module loading the
    // first use of the module reserves its 4 MiB array, and that reservation
    // belongs here, not inside the allocation-free call.
    void* scratch = nullptr;
    rc = noalloc_scratch(dev, &scratch);
    if (rc != MAGIC_SHT_OK) return fail(rc);
  }
  *out = h;
  return MAGIC_SHT_OK;
}

int magic_sht_finalize(magic_sht_handle* h) {
  if (!h) return MAGIC_SHT_OK;
  DeviceGuard dg(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  void* ptrs[] = {h->d_lmoff, h->d_theta, h->d_gauss, h->d_P, h->d_dP, h->d_wgt, h->d_osin2,
                  h->d_P32, h->d_dP32, h->d_tw64, h->d_tw32, h->ws, h->d_inv_img, h->d_fwd_img,
                  h->d_inv_blk0, h->d_fwd_blk0, h->d_inv_scale, h->d_fwd_scale, h->d_err,
                  h->d_bpc0, h->d_bimg, h->d_tile_ctr, h->d_tdcoef, h->d_tdlq, h->d_twdf,
                  h->d_inv_exp, h->d_fwd_exp, h->d_cosn2, h->d_twr};
  for (void* p : ptrs) if (p) cudaFree(p);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  if (h->pin) cudaFreeHost(h->pin);
  if (h->pin_ev) cudaEventDestroy(h->pin_ev);
  for (auto& P : h->pools) {
    if (P.buf) cudaFree(P.buf);
    for (auto* v : {&P.ev_in, &P.ev_comp, &P.ev_out})
      for (cudaEvent_t e : *v) cudaEventDestroy(e);
  }
  if (h->cpy_in) cudaStreamDestroy(h->cpy_in);
  if (h->cpy_out) cudaStreamDestroy(h->cpy_out);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return MAGIC_SHT_OK;
}

int magic_sht_scrambled_theta(const magic_sht_handle* h, int* l_scrambled_theta) {
  TRY(check_handle(h));
  if (!l_scrambled_theta) return set_err(MAGIC_SHT_ERR_ARG, "null output");
  *l_scrambled_theta = 1;
  return MAGIC_SHT_OK;
}

int magic_sht_get_sizes(const magic_sht_handle* h, int* o) {
  TRY(check_handle(h));
  if (!o) return set_err(MAGIC_SHT_ERR_ARG, "null output");
  const ShtGeom& g = h->g;
  o[0] = g.l_max; o[1] = g.m_max; o[2] = g.minc; o[3] = g.n_theta; o[4] = g.n_phi;
  o[5] = g.ld; o[6] = g.n_m; o[7] = g.lm_max;
  return MAGIC_SHT_OK;
}

int magic_sht_gauss_grid(magic_sht_handle* h, double* theta_ord, double* gauss) {
  TRY(check_handle(h));
  DeviceGuard dg(h->device);
  if (theta_ord) CK(cudaMemcpy(theta_ord, h->d_theta, sizeof(double) * h->g.n_theta, cudaMemcpyDeviceToHost));
  if (gauss) CK(cudaMemcpy(gauss, h->d_gauss, sizeof(double) * h->g.n_theta, cudaMemcpyDeviceToHost));
  return MAGIC_SHT_OK;
}

int magic_sht_set_stream(magic_sht_handle* h, void* s) {
  TRY(check_handle(h));
  if ((cudaStream_t)s == h->stream && !h->own_stream) return MAGIC_SHT_OK;
  if (h->capturing) return set_err(MAGIC_SHT_ERR_ARG, "cannot change the stream during capture");
  DeviceGuard dg(h->device);
  CK(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  // NULL selects the legacy default stream (the CUDA convention), so the
  // library orders with every other default-stream user.
  h->stream = (cudaStream_t)s;
  h->own_stream = false;
  return MAGIC_SHT_OK;
}

int magic_sht_synchronize(magic_sht_handle* h) {
  TRY(check_handle(h));
  DeviceGuard dg(h->device);
  CK(cudaStreamSynchronize(h->stream));
  if (h->cpy_in) CK(cudaStreamSynchronize(h->cpy_in));
  if (h->cpy_out) CK(cudaStreamSynchronize(h->cpy_out));
  return MAGIC_SHT_OK;
}

int magic_sht_set_host_async(magic_sht_handle* h, int on) {
  TRY(check_handle(h));
  if (!on && h->host_async) TRY(magic_sht_synchronize(h));
  h->host_async = on != 0;
  return MAGIC_SHT_OK;
}

int magic_sht_set_tuning(magic_sht_handle* h, const magic_sht_tuning* t) {
  TRY(check_handle(h));
  if (!t) return set_err(MAGIC_SHT_ERR_ARG, "null tuning");
  if (t->tc_kernel < 0 || t->tc_kernel > 1 || t->tc_order < 0 || t->tc_order > 1)
    return set_err(MAGIC_SHT_ERR_ARG, "tc_kernel and tc_order are 0 or 1");
  if (t->pipe_chunk < 1 || t->pipe_chunk > 1024) return set_err(MAGIC_SHT_ERR_ARG, "pipe_chunk outside [1, 1024]");
  if (t->fft_rows != 0 && t->fft_rows != 8 && t->fft_rows != 16)
    return set_err(MAGIC_SHT_ERR_ARG, "fft_rows is 0, 8 or 16");
  if (t->tc_kernel == 1 && tf32_form(h))
    return set_err(MAGIC_SHT_ERR_UNSUPPORTED, "the TF32 form has only the persistent kernels");
  if (split_form(h) || oz_form(h)) h->tc_persistent = t->tc_kernel == 0;
  h->tct.order = t->tc_order;
  h->pipe_chunk = t->pipe_chunk;
  h->fft_rows = t->fft_rows;
  return MAGIC_SHT_OK;
}

int magic_sht_get_tuning(const magic_sht_handle* h, magic_sht_tuning* t) {
  TRY(check_handle(h));
  if (!t) return set_err(MAGIC_SHT_ERR_ARG, "null tuning");
  t->tc_kernel = h->tc_persistent ? 0 : 1;
  t->tc_order = h->tct.order;
  t->pipe_chunk = h->pipe_chunk;
  t->fft_rows = h->fft_rows;
  return MAGIC_SHT_OK;
}

int magic_sht_reserve(magic_sht_handle* h, int n) {
  TRY(check_handle(h));
  if (n < 1) return set_err(MAGIC_SHT_ERR_ARG, "n_levels=%d", n);
  DeviceGuard dg(h->device);
  // the radial set needs 15 inverse half spectra (the forward set needs 10)
  // plus per-level lcut/or2 staging
  const size_t need = (tc_form(h) ? 23 : 15) * align256(hs_bytes(h, n)) + 4 * align256((size_t)n * 8) + 4096;
  TRY(ensure_ws(h, need));
  if (oz_form(h) && h->tc_persistent) {
    const ShtGeom& g = h->g;
    size_t b = oz_data_bytes(g, h->tct, 7 * n, true);
    b = std::max(b, oz_data_bytes(g, h->tct, 4 * n * 2, true));
    b = std::max(b, oz_data_bytes(g, h->tct, n, false));
    b = std::max(b, oz_data_bytes(g, h->tct, 3 * n * 2, false));
    TRY(ensure_bimg(h, b));
  } else if (tc_form(h) && h->tc_persistent) {
    // data images of the radial set's largest tensor-core launch (7 scalar + 4 vector
    // syntheses, 1 scalar + 3 vector analyses per level)
    const ShtGeom& g = h->g;
    const bool f = tf32_form(h);
    size_t b = tcp_data_bytes(g, h->tct, 7 * n, false, true, f);
    b = std::max(b, tcp_data_bytes(g, h->tct, 4 * n * 2, true, true, f));
    b = std::max(b, tcp_data_bytes(g, h->tct, n, false, false, f));
    b = std::max(b, tcp_data_bytes(g, h->tct, 3 * n * 2, true, false, f));
    TRY(ensure_bimg(h, b));
  }
  return MAGIC_SHT_OK;
}

// ----------------------------------------------------- single-level facade
int magic_sht_scal_to_spat(magic_sht_handle* h, const double* Slm, double* f, int lcut) {
  return inverse_one(h, lcut, 0.0, {Slm}, {f},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>& sc,
                        std::vector<VectorInv>&) { sc.push_back({ref(OP_COPY, s[0]), g[0], 0}); });
}

int magic_sht_pol_to_curlr_spat(magic_sht_handle* h, const double* Qlm, double* f, int lcut) {
  return inverse_one(h, lcut, 0.0, {Qlm}, {f},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>& sc,
                        std::vector<VectorInv>&) { sc.push_back({ref(OP_DLH, s[0]), g[0], 0}); });
}

int magic_sht_scal_to_grad_spat(magic_sht_handle* h, const double* Slm, double* gt, double* gp, int lcut) {
  return inverse_one(h, lcut, 0.0, {Slm}, {gt, gp},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>&,
                        std::vector<VectorInv>& vc) {
                       vc.push_back({ref(OP_COPY, s[0]), SpecRef(), g[0], g[1], 0});
                     });
}

int magic_sht_pol_to_grad_spat(magic_sht_handle* h, const double* Slm, double* gt, double* gp, int lcut) {
  return inverse_one(h, lcut, 0.0, {Slm}, {gt, gp},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>&,
                        std::vector<VectorInv>& vc) {
                       vc.push_back({ref(OP_DLH, s[0]), SpecRef(), g[0], g[1], 0});
                     });
}

int magic_sht_torpol_to_spat(magic_sht_handle* h, const double* W, const double* dW, const double* Z,
                             double* vr, double* vt, double* vp, int lcut) {
  return inverse_one(h, lcut, 0.0, {W, dW, Z}, {vr, vt, vp},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>& sc,
                        std::vector<VectorInv>& vc) {
                       sc.push_back({ref(OP_DLH, s[0]), g[0], 0});
                       vc.push_back({ref(OP_COPY, s[1]), ref(OP_COPY, s[2]), g[1], g[2], 0});
                     });
}

int magic_sht_sphtor_to_spat(magic_sht_handle* h, const double* dW, const double* Z, double* vt,
                             double* vp, int lcut) {
  return inverse_one(h, lcut, 0.0, {dW, Z}, {vt, vp},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>&,
                        std::vector<VectorInv>& vc) {
                       vc.push_back({ref(OP_COPY, s[0]), ref(OP_COPY, s[1]), g[0], g[1], 0});
                     });
}

int magic_sht_torpol_to_dphspat(magic_sht_handle* h, const double* dW, const double* Z, double* dvtdp,
                                double* dvpdp, int lcut) {
  return inverse_one(h, lcut, 0.0, {dW, Z}, {dvtdp, dvpdp},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>&,
                        std::vector<VectorInv>& vc) {
                       vc.push_back({ref(OP_IM, s[0]), ref(OP_IM, s[1]), g[0], g[1], FFT_OSIN2});
                     });
}

int magic_sht_torpol_to_curl_spat(magic_sht_handle* h, double or2, const double* B, const double* ddB,
                                  const double* J, const double* dJ, double* cvr, double* cvt,
                                  double* cvp, int lcut) {
  return inverse_one(h, lcut, or2, {B, ddB, J, dJ}, {cvr, cvt, cvp},
                     [](const std::vector<int>& s, const std::vector<int>& g, std::vector<ScalarInv>& sc,
                        std::vector<VectorInv>& vc) {
                       sc.push_back({ref(OP_DLH, s[2]), g[0], 0});
                       vc.push_back({ref(OP_COPY, s[3]), ref(OP_CURLT, s[0], s[1]), g[1], g[2], 0});
                     });
}

// Inner-core variants (rare diagnostics): the r-dependent prescaling is a
// small kernel writing Q,S,T into the workspace, then the QST synthesis.
static int ic_qst(magic_sht_handle* h, double r, double r_ICB, const double* A0, const double* A1,
                  const double* A2, const double* A3, double* o0, double* o1, double* o2, bool curl) {
  TRY(check_handle(h));
  if (!A0 || !A1 || !A2 || (curl && !A3) || !o0 || !o1 || !o2)
    return set_err(MAGIC_SHT_ERR_ARG, "null pointer");
  if (r_ICB == 0.0) return set_err(MAGIC_SHT_ERR_ARG, "r_ICB must be non-zero");
  DeviceGuard dg(h->device);
  const ShtGeom& g = h->g;
  const int L = g.l_max, K = g.lm_max;
  // coefficient tables (src/sht_native.f90:166-182, :209-225)
  std::vector<double> rDep(L + 1), rDep2(L + 1);
  const double rRatio = r / r_ICB;
  rDep[0] = rRatio; rDep2[0] = 1.0 / r_ICB;
  for (int l = 1; l <= L; ++l) { rDep[l] = rDep[l - 1] * rRatio; rDep2[l] = rDep2[l - 1] * rRatio; }
  std::vector<double> cq(L + 1), cs_a(L + 1), cs_b(L + 1), ct_a(L + 1), ct_b(L + 1);
  for (int l = 0; l <= L; ++l) {
    cq[l] = rDep[l] * (double)(l * (l + 1));
    cs_a[l] = rDep2[l] * (double)(l + 1);
    cs_b[l] = rDep2[l] * r;
    if (curl) { ct_a[l] = -rDep2[l] * 2.0 * (double)(l + 1); ct_b[l] = -rDep2[l] * r; }
    else { ct_a[l] = rDep[l]; ct_b[l] = 0.0; }
  }
  std::vector<int> lm2l(K);
  for (int mc = 0; mc < g.n_m; ++mc)
    for (int l = mc * g.minc; l <= L; ++l) lm2l[h->lmoff[mc] + l - mc * g.minc] = l;
  CallCtx cx(h);
  // curl: Q from J (A2), S from J,dJ (A2,A3), T from dB,ddB (A0,A1)
  // plain: Q from W (A0), S from W,dW (A0,A1), T from Z (A2)
  const double* qa = curl ? A2 : A0;
  const double* sa = curl ? A2 : A0;
  const double* sb = curl ? A3 : A1;
  const double* ta = curl ? A0 : A2;
  const double* tb = curl ? A1 : nullptr;
  const int iqa = cx.spec_in(qa, 1, K), isa = cx.spec_in(sa, 1, K), isb = cx.spec_in(sb, 1, K);
  const int ita = cx.spec_in(ta, 1, K), itb = tb ? cx.spec_in(tb, 1, K) : -1;
  const int ilm = cx.tmp(sizeof(int) * K);
  const int icf = cx.tmp(sizeof(double) * 5 * (L + 1));
  const int iQ = cx.tmp(16 * (size_t)K), iS = cx.tmp(16 * (size_t)K), iT = cx.tmp(16 * (size_t)K);
  const long long gl = (long long)g.n_phi * g.ld;
  const int g0 = cx.grid_out(o0, 1, gl), g1 = cx.grid_out(o1, 1, gl), g2 = cx.grid_out(o2, 1, gl);
  const int hs0 = cx.tmp(hs_bytes(h, 1)), hs1 = cx.tmp(hs_inv_bytes(h, 1, true)), hs2 = cx.tmp(hs_inv_bytes(h, 1, true));
  TRY(cx.prepare());
  std::vector<double> cf;
  cf.insert(cf.end(), cq.begin(), cq.end());
  cf.insert(cf.end(), cs_a.begin(), cs_a.end());
  cf.insert(cf.end(), cs_b.begin(), cs_b.end());
  cf.insert(cf.end(), ct_a.begin(), ct_a.end());
  cf.insert(cf.end(), ct_b.begin(), ct_b.end());
  double* dcf = (double*)cx.dev(icf);
  CK(cudaMemcpyAsync(cx.dev(ilm), lm2l.data(), sizeof(int) * K, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dcf, cf.data(), sizeof(double) * cf.size(), cudaMemcpyHostToDevice, h->stream));
  const int nb = (K + 255) / 256;
  const int* dlm = (const int*)cx.dev(ilm);
  ic_prescale_kernel<<<nb, 256, 0, h->stream>>>(K, dlm, dcf, nullptr, (const double2*)cx.dev(iqa), nullptr,
                                                (double2*)cx.dev(iQ));
  ic_prescale_kernel<<<nb, 256, 0, h->stream>>>(K, dlm, dcf + (L + 1), dcf + 2 * (L + 1),
                                                (const double2*)cx.dev(isa), (const double2*)cx.dev(isb),
                                                (double2*)cx.dev(iS));
  ic_prescale_kernel<<<nb, 256, 0, h->stream>>>(K, dlm, dcf + 3 * (L + 1), dcf + 4 * (L + 1),
                                                (const double2*)cx.dev(ita),
                                                itb >= 0 ? (const double2*)cx.dev(itb) : nullptr,
                                                (double2*)cx.dev(iT));
  CK(cudaGetLastError());
  // The synchronous host copies above use pageable vectors; make sure they
  // have been consumed before the vectors go out of scope.
  CK(cudaStreamSynchronize(h->stream));
  std::vector<ScalarInv> sc{{ref(OP_COPY, iQ), g0, 0}};
  std::vector<VectorInv> vc{{ref(OP_COPY, iS), ref(OP_COPY, iT), g1, g2, 0}};
  LevelCtl lv;
  lv.nlev = 1; lv.lcut0 = L; lv.spec_ld = K; lv.grid_ld = gl;
  TRY(run_inverse(h, cx, lv, sc, vc, {hs0}, {hs1, hs2}));
  return cx.finish();
}

int magic_sht_torpol_to_spat_IC(magic_sht_handle* h, double r, double r_ICB, const double* W,
                                const double* dW, const double* Z, double* Br, double* Bt, double* Bp) {
  return ic_qst(h, r, r_ICB, W, dW, Z, nullptr, Br, Bt, Bp, false);
}

int magic_sht_torpol_to_curl_spat_IC(magic_sht_handle* h, double r, double r_ICB, const double* dB,
                                     const double* ddB, const double* J, const double* dJ, double* cbr,
                                     double* cbt, double* cbp) {
  return ic_qst(h, r, r_ICB, dB, ddB, J, dJ, cbr, cbt, cbp, true);
}

// m = 0 only transforms (native_axi_to_spat / native_toraxi_to_spat), grids of n_theta.
static int axi_common(magic_sht_handle* h, const double* fl, double* a, double* b, int lcut, int tor) {
  TRY(check_handle(h));
  if (!fl || !a || (tor && !b)) return set_err(MAGIC_SHT_ERR_ARG, "null pointer");
  if (tor) TRY(check_lcut(h, lcut));
  DeviceGuard dg(h->device);
  const ShtGeom& g = h->g;
  CallCtx cx(h);
  const int iin = cx.raw_in(fl, sizeof(double) * 2 * (g.l_max + 1));
  const int ia = cx.tmp(sizeof(double) * g.n_theta), ib = cx.tmp(sizeof(double) * g.n_theta);
  TRY(cx.prepare());
  axi_kernel<<<(g.nh + 127) / 128, 128, 0, h->stream>>>(g.l_max, g.nh, g.P64, g.dP64,
                                                        (const double2*)cx.dev(iin), lcut, tor,
                                                        (double*)cx.dev(ia), (double*)cx.dev(ib));
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(a, cx.dev(ia), sizeof(double) * g.n_theta, cudaMemcpyDefault, h->stream));
  if (tor) CK(cudaMemcpyAsync(b, cx.dev(ib), sizeof(double) * g.n_theta, cudaMemcpyDefault, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return cx.finish();
}

int magic_sht_axi_to_spat(magic_sht_handle* h, const double* fl_ax, double* f) {
  return axi_common(h, fl_ax, f, nullptr, 0, 0);
}

int magic_sht_toraxi_to_spat(magic_sht_handle* h, const double* fl_ax, double* ft, double* fp, int lcut) {
  return axi_common(h, fl_ax, ft, fp, lcut, 1);
}

// -------------------------------------------------------- analysis facade
int magic_sht_scal_to_SH(magic_sht_handle* h, const double* f, double* fLM, int lcut) {
  return forward_one(h, lcut, {f}, {fLM},
                     [](const std::vector<int>& g, const std::vector<int>& s, std::vector<ScalarFwd>& sc,
                        std::vector<VectorFwd>&) { sc.push_back({g[0], s[0]}); });
}

int magic_sht_spat_to_qst(magic_sht_handle* h, const double* f, const double* gg, const double* hh,
                          double* qLM, double* sLM, double* tLM, int lcut) {
  return forward_one(h, lcut, {f, gg, hh}, {qLM, sLM, tLM},
                     [](const std::vector<int>& g, const std::vector<int>& s, std::vector<ScalarFwd>& sc,
                        std::vector<VectorFwd>& vc) {
                       sc.push_back({g[0], s[0]});
                       vc.push_back({g[1], g[2], s[1], s[2]});
                     });
}

int magic_sht_spat_to_sphertor(magic_sht_handle* h, const double* f, const double* gg, double* fLM,
                               double* gLM, int lcut) {
  return forward_one(h, lcut, {f, gg}, {fLM, gLM},
                     [](const std::vector<int>& g, const std::vector<int>& s, std::vector<ScalarFwd>&,
                        std::vector<VectorFwd>& vc) { vc.push_back({g[0], g[1], s[0], s[1]}); });
}

// ------------------------------------------- host-buffer level pipeline
// Batched calls with host arrays run in chunks of levels: chunk c is copied in
// on one copy stream, transformed on the handle's stream and copied out on a
// second copy stream, through two device staging slots, so that copies in
// both directions overlap each other and the kernels.
struct PipeArray {
  const void* host;   // level 0 of the host array
  size_t lds;         // bytes between levels
  size_t last;        // bytes of one level
  bool out;
  size_t slot_off;    // offset in a staging slot
};

static int pipelined_levels(magic_sht_handle* h, int n, int chunk, std::vector<PipeArray>& arrs,
                            const std::function<int(int, int, const std::vector<char*>&)>& compute) {
  // A copy from pageable memory returns only once the copy stream has reached
  // it, which would hold the host at every chunk: small pageable inputs (the
  // per-level radii, or2, lcut) are staged once in the pinned ring and copied
  // from there.
  for (auto& a : arrs) {
    if (a.out) continue;
    const size_t all = (size_t)(n - 1) * a.lds + a.last;
    if (!is_pinned_host(a.host))
      if (const void* pinned = pin_stage(h, a.host, all)) a.host = pinned;
  }
  size_t slot = 0;
  for (auto& a : arrs) {
    a.slot_off = slot;
    slot += align256((size_t)(chunk - 1) * a.lds + a.last);
  }
  const int nchunks = (n + chunk - 1) / chunk;
  const int ns = h->host_async ? nchunks : 2;
  auto& P = h->pools[h->pool];
  h->pool ^= 1;
  if (!h->cpy_in) {
    CK(cudaStreamCreateWithFlags(&h->cpy_in, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&h->cpy_out, cudaStreamNonBlocking));
  }
  if ((size_t)ns * slot > P.bytes || slot != P.stride) {
    // new layout of this pool: its previous slots must be drained first
    if ((size_t)ns * slot > P.bytes) {
      CK(cudaDeviceSynchronize());
      if (P.buf) CK(cudaFree(P.buf));
      P.buf = nullptr;
      P.bytes = 0;
      CK(cudaMalloc((void**)&P.buf, (size_t)ns * slot));
      P.bytes = (size_t)ns * slot;
    } else {
      for (size_t k = 0; k < P.used.size(); ++k)
        if (P.used[k]) {
          CK(cudaStreamWaitEvent(h->cpy_in, P.ev_out[k], 0));
          CK(cudaStreamWaitEvent(h->stream, P.ev_out[k], 0));
        }
    }
    P.stride = slot;
    std::fill(P.used.begin(), P.used.end(), 0);
  }
  while ((int)P.used.size() < ns) {
    cudaEvent_t e[3];
    for (auto& x : e) CK(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    P.ev_in.push_back(e[0]);
    P.ev_comp.push_back(e[1]);
    P.ev_out.push_back(e[2]);
    P.used.push_back(0);
  }
  // A slot is reused once the copies out of its previous use (in this call or
  // an earlier one) are done; the host arrays need no other ordering.
  for (int c = 0; c < nchunks; ++c) {
    const int sl = c % ns, r0 = c * chunk, nr = std::min(chunk, n - r0);
    char* base = P.buf + (size_t)sl * P.stride;
    const bool reuse = P.used[sl] != 0;
    if (reuse) CK(cudaStreamWaitEvent(h->cpy_in, P.ev_out[sl], 0));  // slot drained
    std::vector<char*> dev(arrs.size());
    for (size_t i = 0; i < arrs.size(); ++i) {
      const PipeArray& a = arrs[i];
      dev[i] = base + a.slot_off;
      if (!a.out)
        CK(cudaMemcpyAsync(dev[i], (const char*)a.host + (size_t)r0 * a.lds, (size_t)(nr - 1) * a.lds + a.last,
                           cudaMemcpyHostToDevice, h->cpy_in));
    }
    CK(cudaEventRecord(P.ev_in[sl], h->cpy_in));
    CK(cudaStreamWaitEvent(h->stream, P.ev_in[sl], 0));
    if (reuse) CK(cudaStreamWaitEvent(h->stream, P.ev_out[sl], 0));  // previous outputs copied
    TRY(compute(r0, nr, dev));
    CK(cudaEventRecord(P.ev_comp[sl], h->stream));
    CK(cudaStreamWaitEvent(h->cpy_out, P.ev_comp[sl], 0));
    for (size_t i = 0; i < arrs.size(); ++i) {
      const PipeArray& a = arrs[i];
      if (a.out)
        CK(cudaMemcpyAsync((char*)a.host + (size_t)r0 * a.lds, dev[i], (size_t)(nr - 1) * a.lds + a.last,
                           cudaMemcpyDeviceToHost, h->cpy_out));
    }
    CK(cudaEventRecord(P.ev_out[sl], h->cpy_out));
    P.used[sl] = 1;
  }
  if (!h->host_async) {
    CK(cudaStreamSynchronize(h->cpy_out));
    CK(cudaStreamSynchronize(h->stream));
  }
  return MAGIC_SHT_OK;
}

// the host-buffer pipeline runs when every given array is in host memory
static bool all_host_v(const std::vector<const void*>& ptrs) {
  bool any = false;
  for (const void* p : ptrs) {
    if (!p) continue;
    if (is_device_ptr(p)) return false;
    any = true;
  }
  return any;
}
static bool all_host(std::initializer_list<const void*> ptrs) { return all_host_v(std::vector<const void*>(ptrs)); }

// ------------------------------------------------------ radial-loop sets
static int level_ctl(magic_sht_handle* h, CallCtx& cx, int n, const int* lcut, const double* or2,
                     LevelCtl& lv, std::vector<int>& lcut_copy) {
  lv.nlev = n;
  lv.lcut0 = h->g.l_max;
  lv.or2_0 = 0.0;
  if (lcut) {
    if (!is_device_ptr(lcut)) {
      for (int i = 0; i < n; ++i)
        if (lcut[i] < 0 || lcut[i] > h->g.l_max)
          return set_err(MAGIC_SHT_ERR_LCUT, "lcut[%d]=%d outside [0, %d]", i, lcut[i], h->g.l_max);
    }
    lv.lcut_idx = cx.raw_in(lcut, sizeof(int) * n);
  }
  if (or2) lv.or2_idx = cx.raw_in(or2, sizeof(double) * n);
  (void)lcut_copy;
  return MAGIC_SHT_OK;
}

int magic_sht_transform_to_grid_space(magic_sht_handle* h, int n, const double* or2, const int* lcut,
                                      const magic_sht_grid_space_args* a) {
  TRY(check_handle(h));
  if (!a || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  const ShtGeom& g = h->g;
  if (a->spec_ld < g.lm_max || a->grid_ld < (long long)g.n_phi * g.ld)
    return set_err(MAGIC_SHT_ERR_ARG, "spec_ld/grid_ld smaller than one level");
  DeviceGuard dg(h->device);
  if (n > h->pipe_chunk && !h->capturing &&
      all_host({a->s, a->p, a->xi, a->w, a->dw, a->ddw, a->z, a->dz, a->b, a->db, a->ddb, a->aj, a->dj,
                a->sc, a->pc, a->xic, a->vrc, a->vtc, a->vpc, a->cvrc, a->cvtc, a->cvpc, a->brc, a->btc,
                a->bpc, a->cbrc, a->cbtc, a->cbpc, a->dvrdrc, a->dvtdrc, a->dvpdrc, a->dvrdtc, a->dvrdpc,
                a->dvtdpc, a->dvpdpc, lcut, or2})) {
    if (lcut)
      for (int i = 0; i < n; ++i)
        if (!is_device_ptr(lcut) && (lcut[i] < 0 || lcut[i] > g.l_max))
          return set_err(MAGIC_SHT_ERR_LCUT, "lcut[%d]=%d outside [0, %d]", i, lcut[i], g.l_max);
    const double* const ins[13] = {a->s, a->p, a->xi, a->w, a->dw, a->ddw, a->z, a->dz,
                                   a->b, a->db, a->ddb, a->aj, a->dj};
    constexpr int NO = 22;
    double* const outs[NO] = {a->sc,     a->pc,     a->xic,    a->vrc,    a->vtc,    a->vpc,    a->cvrc,
                              a->cvtc,   a->cvpc,   a->brc,    a->btc,    a->bpc,    a->cbrc,   a->cbtc,
                              a->cbpc,   a->dvrdrc, a->dvtdrc, a->dvpdrc, a->dvrdtc, a->dvrdpc, a->dvtdpc,
                              a->dvpdpc};
    std::vector<PipeArray> arrs;
    std::vector<int> idx_in(13, -1), idx_out(NO, -1);
    const size_t sb = (size_t)a->spec_ld * 16, gb = (size_t)a->grid_ld * 8;
    for (int i = 0; i < 13; ++i)
      if (ins[i]) { idx_in[i] = (int)arrs.size(); arrs.push_back({ins[i], sb, (size_t)g.lm_max * 16, false, 0}); }
    for (int i = 0; i < NO; ++i)
      if (outs[i]) { idx_out[i] = (int)arrs.size(); arrs.push_back({outs[i], gb, (size_t)g.n_phi * g.ld * 8, true, 0}); }
    if (or2) arrs.push_back({or2, 8, 8, false, 0});
    if (lcut) arrs.push_back({lcut, 4, 4, false, 0});
    const int i_or2 = or2 ? (int)arrs.size() - (lcut ? 2 : 1) : -1;
    const int i_lc = lcut ? (int)arrs.size() - 1 : -1;
    return pipelined_levels(h, n, h->pipe_chunk, arrs, [&](int r0, int nr, const std::vector<char*>& d) {
      magic_sht_grid_space_args b = *a;
      double** pin[13] = {(double**)&b.s, (double**)&b.p, (double**)&b.xi, (double**)&b.w, (double**)&b.dw,
                          (double**)&b.ddw, (double**)&b.z, (double**)&b.dz, (double**)&b.b, (double**)&b.db,
                          (double**)&b.ddb, (double**)&b.aj, (double**)&b.dj};
      double** pout[NO] = {&b.sc,     &b.pc,     &b.xic,    &b.vrc,    &b.vtc,    &b.vpc,    &b.cvrc,
                           &b.cvtc,   &b.cvpc,   &b.brc,    &b.btc,    &b.bpc,    &b.cbrc,   &b.cbtc,
                           &b.cbpc,   &b.dvrdrc, &b.dvtdrc, &b.dvpdrc, &b.dvrdtc, &b.dvrdpc, &b.dvtdpc,
                           &b.dvpdpc};
      for (int i = 0; i < 13; ++i) *pin[i] = idx_in[i] >= 0 ? (double*)d[idx_in[i]] : nullptr;
      for (int i = 0; i < NO; ++i) *pout[i] = idx_out[i] >= 0 ? (double*)d[idx_out[i]] : nullptr;
      (void)r0;
      return magic_sht_transform_to_grid_space(h, nr, i_or2 >= 0 ? (const double*)d[i_or2] : nullptr,
                                               i_lc >= 0 ? (const int*)d[i_lc] : nullptr, &b);
    });
  }
  CallCtx cx(h);
  LevelCtl lv;
  std::vector<int> lc;
  TRY(level_ctl(h, cx, n, lcut, or2, lv, lc));
  lv.spec_ld = a->spec_ld;
  lv.grid_ld = a->grid_ld;
  auto si = [&](const double* p) { return cx.spec_in(p, n, a->spec_ld); };
  auto go = [&](double* p) { return cx.grid_out(p, n, a->grid_ld); };
  std::vector<ScalarInv> sc;
  std::vector<VectorInv> vc;
  // scalars: s, p, xi (rIter.f90:485, 503, 506)
  if (a->s && a->sc) sc.push_back({ref(OP_COPY, si(a->s)), go(a->sc), 0});
  if (a->p && a->pc) sc.push_back({ref(OP_COPY, si(a->p)), go(a->pc), 0});
  if (a->xi && a->xic) sc.push_back({ref(OP_COPY, si(a->xi)), go(a->xic), 0});
  // velocity and vorticity (rIter.f90:516, 522)
  int iw = -1, idw = -1, iddw = -1, iz = -1, idz = -1;
  if (a->w) iw = si(a->w);
  if (a->dw) idw = si(a->dw);
  if (a->ddw) iddw = si(a->ddw);
  if (a->z) iz = si(a->z);
  if (a->dz) idz = si(a->dz);
  if (iw >= 0 && idw >= 0 && iz >= 0 && a->vrc && a->vtc && a->vpc) {
    sc.push_back({ref(OP_DLH, iw), go(a->vrc), 0});
    vc.push_back({ref(OP_COPY, idw), ref(OP_COPY, iz), go(a->vtc), go(a->vpc), 0});
  }
  if (iw >= 0 && iddw >= 0 && iz >= 0 && idz >= 0 && a->cvrc && a->cvtc && a->cvpc) {
    sc.push_back({ref(OP_DLH, iz), go(a->cvrc), 0});
    vc.push_back({ref(OP_COPY, idz), ref(OP_CURLT, iw, iddw), go(a->cvtc), go(a->cvpc), 0});
  } else if (iz >= 0 && a->cvrc && !a->cvtc && !a->cvpc) {
    sc.push_back({ref(OP_DLH, iz), go(a->cvrc), 0});  // pol_to_curlr_spat(z) of the u.grad u set (:540)
  }
  // velocity derivatives (rIter.f90:527-545): torpol_to_spat(dw, ddw, dz),
  // pol_to_grad_spat(w), torpol_to_dphspat(dw, z)
  if (idw >= 0 && iddw >= 0 && idz >= 0 && a->dvrdrc && a->dvtdrc && a->dvpdrc) {
    sc.push_back({ref(OP_DLH, idw), go(a->dvrdrc), 0});
    vc.push_back({ref(OP_COPY, iddw), ref(OP_COPY, idz), go(a->dvtdrc), go(a->dvpdrc), 0});
  }
  if (iw >= 0 && a->dvrdtc && a->dvrdpc) vc.push_back({ref(OP_DLH, iw), SpecRef(), go(a->dvrdtc), go(a->dvrdpc), 0});
  if (idw >= 0 && iz >= 0 && a->dvtdpc && a->dvpdpc)
    vc.push_back({ref(OP_IM, idw), ref(OP_IM, iz), go(a->dvtdpc), go(a->dvpdpc), FFT_OSIN2});
  // magnetic field and current (rIter.f90:606, 610)
  int ib = -1, idb = -1, iddb = -1, iaj = -1, idj = -1;
  if (a->b) ib = si(a->b);
  if (a->db) idb = si(a->db);
  if (a->ddb) iddb = si(a->ddb);
  if (a->aj) iaj = si(a->aj);
  if (a->dj) idj = si(a->dj);
  if (ib >= 0 && idb >= 0 && iaj >= 0 && a->brc && a->btc && a->bpc) {
    sc.push_back({ref(OP_DLH, ib), go(a->brc), 0});
    vc.push_back({ref(OP_COPY, idb), ref(OP_COPY, iaj), go(a->btc), go(a->bpc), 0});
  }
  if (ib >= 0 && iddb >= 0 && iaj >= 0 && idj >= 0 && a->cbrc && a->cbtc && a->cbpc) {
    sc.push_back({ref(OP_DLH, iaj), go(a->cbrc), 0});
    vc.push_back({ref(OP_COPY, idj), ref(OP_CURLT, ib, iddb), go(a->cbtc), go(a->cbpc), 0});
  }
  std::vector<int> hs_sc, hs_vc;
  for (size_t i = 0; i < sc.size(); ++i) hs_sc.push_back(cx.tmp(hs_bytes(h, n)));
  for (size_t i = 0; i < 2 * vc.size(); ++i) hs_vc.push_back(cx.tmp(hs_inv_bytes(h, n, true)));
  TRY(cx.prepare());
  TRY(run_inverse(h, cx, lv, sc, vc, hs_sc, hs_vc));
  return cx.finish();
}

int magic_sht_get_nl(magic_sht_handle* h, int n, const double* or2, const magic_sht_grid_space_args* gin,
                     const magic_sht_lm_space_args* nl) {
  TRY(check_handle(h));
  if (!gin || !nl || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  const ShtGeom& g = h->g;
  if (gin->grid_ld < (long long)g.n_phi * g.ld || nl->grid_ld < (long long)g.n_phi * g.ld)
    return set_err(MAGIC_SHT_ERR_ARG, "grid_ld smaller than one level");
  if ((gin->grid_ld | nl->grid_ld | (long long)g.ld) & 1)
    return set_err(MAGIC_SHT_ERR_ARG, "get_nl needs even grid_ld and nlat_padded (16-byte pairs of rows)");
  DeviceGuard dg(h->device);
  NlGrids in{}, out{};
  const double* const ins[NL_NIN] = {gin->vrc, gin->vtc, gin->vpc, gin->cvrc, gin->cvtc, gin->cvpc,
                                     gin->brc, gin->btc, gin->bpc, gin->cbrc, gin->cbtc, gin->cbpc, gin->sc};
  const double* const outs[NL_NOUT] = {nl->Advr, nl->Advt, nl->Advp, nl->VSr, nl->VSt, nl->VSp,
                                       nl->VxBr, nl->VxBt, nl->VxBp, nl->heatTerms};
  for (int i = 0; i < NL_NIN; ++i) {
    if (!ins[i] || !is_device_ptr(ins[i]) || ((uintptr_t)ins[i] & 15))
      return set_err(MAGIC_SHT_ERR_ARG, "get_nl input grid %d: null, host or not 16-byte aligned", i);
    in.p[i] = const_cast<double*>(ins[i]);
  }
  for (int i = 0; i < NL_NOUT; ++i) {
    if (!outs[i] || !is_device_ptr(outs[i]) || ((uintptr_t)outs[i] & 15))
      return set_err(MAGIC_SHT_ERR_ARG, "get_nl output grid %d: null, host or not 16-byte aligned", i);
    out.p[i] = const_cast<double*>(outs[i]);  // the analysis inputs are written here
  }
  in.ld = gin->grid_ld;
  out.ld = nl->grid_ld;
  CallCtx cx(h);
  const int i_or2 = or2 ? cx.raw_in(or2, (size_t)n * 8) : -1;
  TRY(cx.prepare());
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_NL);
    CK(launch_get_nl(g, in, out, (const double*)cx.dev(i_or2), 1.0, n, fft_arith(h), h->stream));
  }
  return cx.finish();
}

int magic_sht_get_nl_opts(magic_sht_handle* h, int n, const magic_sht_nl_opts* o, const magic_sht_nl_grids* gin,
                          const magic_sht_nl_out* gout) {
  TRY(check_handle(h));
  if (!o || !gin || !gout || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  if (!o->r) return set_err(MAGIC_SHT_ERR_ARG, "get_nl_opts needs the radius of every level (opts->r)");
  const ShtGeom& g = h->g;
  if (gin->grid_ld < (long long)g.n_phi * g.ld || gout->grid_ld < (long long)g.n_phi * g.ld)
    return set_err(MAGIC_SHT_ERR_ARG, "grid_ld smaller than one level");
  if ((gin->grid_ld | gout->grid_ld | (long long)g.ld) & 1)
    return set_err(MAGIC_SHT_ERR_ARG, "get_nl needs even grid_ld and nlat_padded (16-byte pairs of rows)");
  DeviceGuard dg(h->device);
  NlFull a{};
  const double* const ins[NLF_NIN] = {gin->vrc,   gin->vtc,    gin->vpc,    gin->cvrc,   gin->cvtc,   gin->cvpc,
                                      gin->dvrdrc, gin->dvtdrc, gin->dvpdrc, gin->dvrdtc, gin->dvrdpc, gin->dvtdpc,
                                      gin->dvpdpc, gin->brc,    gin->btc,    gin->bpc,    gin->cbrc,   gin->cbtc,
                                      gin->cbpc,   gin->sc,     gin->xic};
  double* const outs[NLF_NOUT] = {gout->Advr, gout->Advt, gout->Advp, gout->VSr,  gout->VSt,
                                  gout->VSp,  gout->VXir, gout->VXit, gout->VXip, gout->VxBr,
                                  gout->VxBt, gout->VxBp, gout->heatTerms};
  // inputs each enabled term reads (get_nl.f90:241-432)
  bool need[NLF_NIN] = {};
  const bool conv = o->l_conv_nl, anel = o->l_anel, mag = o->l_mag_nl, lf = o->l_mag_LF;
  if (conv || o->l_heat_nl || o->l_chemical_conv || mag || anel) need[NLF_VR] = need[NLF_VT] = need[NLF_VP] = true;
  if (conv && o->l_adv_curl) need[NLF_CVR] = need[NLF_CVT] = need[NLF_CVP] = true;
  if ((conv && !o->l_adv_curl) || anel) {
    for (int k : {NLF_DVRDR, NLF_DVTDR, NLF_DVPDR, NLF_DVRDT, NLF_DVRDP, NLF_DVTDP, NLF_DVPDP, NLF_CVR}) need[k] = true;
  }
  if (lf || mag) need[NLF_BR] = need[NLF_BT] = need[NLF_BP] = true;
  if (lf || (anel && mag)) need[NLF_CBR] = need[NLF_CBT] = need[NLF_CBP] = true;
  if (o->l_heat_nl) need[NLF_S] = true;
  if (o->l_chemical_conv) need[NLF_XI] = true;
  for (int i = 0; i < NLF_NIN; ++i) {
    if (!ins[i]) {
      if (need[i]) return set_err(MAGIC_SHT_ERR_ARG, "get_nl_opts: input grid %d is needed by the switches", i);
      continue;
    }
    if (!is_device_ptr(ins[i]) || ((uintptr_t)ins[i] & 15))
      return set_err(MAGIC_SHT_ERR_ARG, "get_nl_opts input grid %d: host or not 16-byte aligned", i);
    if (need[i]) a.in[i] = ins[i];
  }
  for (int i = 0; i < NLF_NOUT; ++i) {
    if (!outs[i]) continue;
    if (!is_device_ptr(outs[i]) || ((uintptr_t)outs[i] & 15))
      return set_err(MAGIC_SHT_ERR_ARG, "get_nl_opts output grid %d: host or not 16-byte aligned", i);
    a.out[i] = outs[i];
  }
  a.ld_in = gin->grid_ld;
  a.ld_out = gout->grid_ld;
  a.o.conv = conv; a.o.curl = o->l_adv_curl; a.o.lf = lf; a.o.heat = o->l_heat_nl;
  a.o.chem = o->l_chemical_conv; a.o.mag = mag; a.o.anel = anel;
  a.o.LFfac = o->LFfac; a.o.ViscHeatFac = o->ViscHeatFac; a.o.OhmLossFac = o->OhmLossFac;
  CallCtx cx(h);
  const size_t nb = (size_t)n * 8, ni = (size_t)n * 4;
  const int i_r = cx.raw_in(o->r, nb);
  const int i_rho = o->orho1 ? cx.raw_in(o->orho1, nb) : -1, i_beta = o->beta ? cx.raw_in(o->beta, nb) : -1;
  const int i_ot = o->otemp1 ? cx.raw_in(o->otemp1, nb) : -1, i_vi = o->visc ? cx.raw_in(o->visc, nb) : -1;
  const int i_la = o->lambda ? cx.raw_in(o->lambda, nb) : -1;
  const int i_nbc = o->nbc ? cx.raw_in(o->nbc, ni) : -1, i_lcr = o->lcr ? cx.raw_in(o->lcr, ni) : -1;
  TRY(cx.prepare());
  a.o.r = (const double*)cx.dev(i_r);
  a.o.orho1 = (const double*)cx.dev(i_rho);
  a.o.beta = (const double*)cx.dev(i_beta);
  a.o.otemp1 = (const double*)cx.dev(i_ot);
  a.o.visc = (const double*)cx.dev(i_vi);
  a.o.lambda = (const double*)cx.dev(i_la);
  a.o.nbc = (const int*)cx.dev(i_nbc);
  a.o.lcr = (const int*)cx.dev(i_lcr);
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_NL);
    CK(launch_get_nl_full(g, a, h->d_cosn2, n, fft_arith(h), h->stream));
  }
  return cx.finish();
}

int magic_sht_get_td_opts(magic_sht_handle* h, int n, const magic_sht_td_opts* o, const magic_sht_td_in* in,
                          const magic_sht_td_out* out) {
  TRY(check_handle(h));
  if (!o || !in || !out || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  if (!o->r) return set_err(MAGIC_SHT_ERR_ARG, "get_td_opts needs the radius of every level (opts->r)");
  const ShtGeom& g = h->g;
  if (in->spec_ld < g.lm_max || out->spec_ld < g.lm_max || in->spec_ld != out->spec_ld)
    return set_err(MAGIC_SHT_ERR_ARG, "spec_ld must be >= lm_max and equal for inputs and outputs");
  DeviceGuard dg(h->device);
  TdFull t{};
  t.o.conv = o->l_conv_nl; t.o.corr = o->l_corr; t.o.dcurl = o->l_double_curl;
  t.o.single_matrix = o->l_single_matrix; t.o.anel = o->l_anel; t.o.liquid = o->l_anelastic_liquid;
  t.o.mag_nl = o->l_mag_nl; t.o.cor_fac = o->cor_fac; t.o.epscXi = o->epscXi;
  double2** const outs[] = {&t.dwdt, &t.dzdt, &t.dpdt, &t.dsdt, &t.dxidt, &t.dbdt, &t.djdt, &t.dVxBh,
                            &t.dVxVh, &t.dVSr, &t.dVXir};
  double* const outp[] = {out->dwdt, out->dzdt, out->dpdt, out->dsdt, out->dxidt, out->dbdt, out->djdt,
                          out->dVxBhLM, out->dVxVhLM, out->dVSrLM, out->dVXirLM};
  for (int i = 0; i < 11; ++i) {
    if (outp[i] && !is_device_ptr(outp[i])) return set_err(MAGIC_SHT_ERR_ARG, "get_td_opts output %d: host pointer", i);
    *outs[i] = (double2*)outp[i];
  }
  // inputs each computed output reads
  const bool vel = o->l_corr && (out->dwdt || out->dzdt || out->dpdt);
  struct In { const double* p; const double2** dst; bool need; const char* name; } ins[] = {
      {in->w, &t.w, vel, "w"}, {in->dw, &t.dw, vel, "dw"}, {in->z, &t.z, vel, "z"},
      {in->ddw, &t.ddw, vel && o->l_double_curl && out->dwdt, "ddw"},
      {in->dz, &t.dz, vel && o->l_double_curl && out->dwdt, "dz"},
      {in->AdvrLM, &t.Advr, o->l_conv_nl && out->dwdt, "AdvrLM"},
      {in->AdvtLM, &t.Advt, o->l_conv_nl && (out->dpdt || (o->l_double_curl && out->dVxVhLM)), "AdvtLM"},
      {in->AdvpLM, &t.Advp, o->l_conv_nl && out->dzdt, "AdvpLM"},
      {in->VStLM, &t.VSt, out->dsdt != nullptr, "VStLM"},
      {in->heatTermsLM, &t.heat, o->l_anel && out->dsdt, "heatTermsLM"},
      {in->VXitLM, &t.VXit, out->dxidt != nullptr, "VXitLM"},
      {in->VxBrLM, &t.VxBr, o->l_mag_nl && out->djdt, "VxBrLM"},
      {in->VxBtLM, &t.VxBt, o->l_mag_nl && out->dVxBhLM, "VxBtLM"},
      {in->VxBpLM, &t.VxBp, o->l_mag_nl && out->dbdt, "VxBpLM"}};
  for (auto& x : ins) {
    if (!x.need) continue;
    if (!x.p || !is_device_ptr(x.p))
      return set_err(MAGIC_SHT_ERR_ARG, "get_td_opts: input %s is needed (a device array)", x.name);
    *x.dst = (const double2*)x.p;
  }
  t.ld = in->spec_ld;
  t.coef = h->d_tdcoef;
  t.lq = h->d_tdlq;
  CallCtx cx(h);
  const size_t nb = (size_t)n * 8, ni = (size_t)n * 4;
  const int i_r = cx.raw_in(o->r, nb);
  const int i_rho = o->orho1 ? cx.raw_in(o->orho1, nb) : -1, i_beta = o->beta ? cx.raw_in(o->beta, nb) : -1;
  const int i_t0 = o->temp0 ? cx.raw_in(o->temp0, nb) : -1, i_ep = o->epsc ? cx.raw_in(o->epsc, nb) : -1;
  const int i_lc = o->lcut ? cx.raw_in(o->lcut, ni) : -1, i_nbc = o->nbc ? cx.raw_in(o->nbc, ni) : -1;
  TRY(cx.prepare());
  t.o.r = (const double*)cx.dev(i_r);
  t.o.orho1 = (const double*)cx.dev(i_rho);
  t.o.beta = (const double*)cx.dev(i_beta);
  t.o.temp0 = (const double*)cx.dev(i_t0);
  t.o.epsc = (const double*)cx.dev(i_ep);
  t.o.lcut = (const int*)cx.dev(i_lc);
  t.o.nbc = (const int*)cx.dev(i_nbc);
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_TD);
    CK(launch_get_td_full(g, t, n, fft_arith(h), h->stream));
  }
  return cx.finish();
}

int magic_sht_get_td(magic_sht_handle* h, int n, const double* r, const int* lcut, double cor_fac,
                     const double* epsc, const magic_sht_td_args* a) {
  return magic_sht_get_td_nbc(h, n, r, lcut, cor_fac, epsc, nullptr, a);
}

int magic_sht_get_td_nbc(magic_sht_handle* h, int n, const double* r, const int* lcut, double cor_fac,
                         const double* epsc, const int* nbc, const magic_sht_td_args* a) {
  TRY(check_handle(h));
  if (!a || !r || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args/r or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  const ShtGeom& g = h->g;
  if (a->spec_ld < g.lm_max) return set_err(MAGIC_SHT_ERR_ARG, "spec_ld smaller than lm_max");
  DeviceGuard dg(h->device);
  const void* const arrs[17] = {a->w, a->dw, a->z, a->AdvrLM, a->AdvtLM, a->AdvpLM, a->VStLM, a->VxBrLM,
                                a->VxBtLM, a->VxBpLM, a->dwdt, a->dzdt, a->dpdt, a->dsdt, a->dbdt, a->djdt,
                                a->dVxBhLM};
  for (int i = 0; i < 17; ++i)
    if (!arrs[i] || !is_device_ptr(arrs[i]) || ((uintptr_t)arrs[i] & 15))
      return set_err(MAGIC_SHT_ERR_ARG, "get_td array %d: null, host or not 16-byte aligned", i);
  if (lcut && !is_device_ptr(lcut))
    for (int i = 0; i < n; ++i)
      if (lcut[i] < 0 || lcut[i] > g.l_max)
        return set_err(MAGIC_SHT_ERR_LCUT, "lcut[%d]=%d outside [0, %d]", i, lcut[i], g.l_max);
  CallCtx cx(h);
  const int i_r = cx.raw_in(r, (size_t)n * 8);
  const int i_lc = lcut ? cx.raw_in(lcut, (size_t)n * 4) : -1;
  const int i_ep = epsc ? cx.raw_in(epsc, (size_t)n * 8) : -1;
  const int i_bc = nbc ? cx.raw_in(nbc, (size_t)n * 4) : -1;
  TRY(cx.prepare());
  TdArgs t{};
  t.w = (const double2*)a->w; t.dw = (const double2*)a->dw; t.z = (const double2*)a->z;
  t.Advr = (const double2*)a->AdvrLM; t.Advt = (const double2*)a->AdvtLM; t.Advp = (const double2*)a->AdvpLM;
  t.VSt = (const double2*)a->VStLM; t.VxBr = (const double2*)a->VxBrLM; t.VxBt = (const double2*)a->VxBtLM;
  t.VxBp = (const double2*)a->VxBpLM;
  t.dwdt = (double2*)a->dwdt; t.dzdt = (double2*)a->dzdt; t.dpdt = (double2*)a->dpdt; t.dsdt = (double2*)a->dsdt;
  t.dbdt = (double2*)a->dbdt; t.djdt = (double2*)a->djdt; t.dVxBh = (double2*)a->dVxBhLM;
  t.ld = a->spec_ld;
  t.r = (const double*)cx.dev(i_r);
  t.lcut = (const int*)cx.dev(i_lc);
  t.epsc = (const double*)cx.dev(i_ep);
  t.nbc = (const int*)cx.dev(i_bc);
  t.cor_fac = cor_fac;
  t.coef = h->d_tdcoef;
  t.lq = h->d_tdlq;
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_TD);
    CK(launch_get_td(g, t, n, fft_arith(h), h->stream));
  }
  return cx.finish();
}

int magic_sht_courant(magic_sht_handle* h, int n, const magic_sht_courant_args* a, double* dtrkc, double* dthkc) {
  TRY(check_handle(h));
  if (!a || !dtrkc || !dthkc || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args/dtrkc/dthkc or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  const ShtGeom& g = h->g;
  if (a->grid_ld < (long long)g.n_phi * g.ld) return set_err(MAGIC_SHT_ERR_ARG, "grid_ld smaller than one level");
  const bool mag = a->br || a->bt || a->bp;
  const double* const grids[6] = {a->vr, a->vt, a->vp, a->br, a->bt, a->bp};
  for (int i = 0; i < (mag ? 6 : 3); ++i)
    if (!grids[i] || !is_device_ptr(grids[i]))
      return set_err(MAGIC_SHT_ERR_ARG, "courant grid %d: null or host pointer (device grids only)", i);
  const double* const rf[6] = {a->orho1, a->orho2, a->or2, a->or4, a->delxr2, a->delxh2};
  for (int i = 0; i < 6; ++i)
    if (!rf[i]) return set_err(MAGIC_SHT_ERR_ARG, "courant radial function %d is null", i);
  DeviceGuard dg(h->device);
  CallCtx cx(h);
  int irf[6];
  for (int i = 0; i < 6; ++i) irf[i] = cx.raw_in(rf[i], (size_t)n * 8);
  const int i_r = cx.raw_inout(dtrkc, (size_t)n * 8), i_h = cx.raw_inout(dthkc, (size_t)n * 8);
  const int i_mx = cx.tmp((size_t)n * 16);
  TRY(cx.prepare());
  CourantArgs c{};
  c.vr = a->vr; c.vt = a->vt; c.vp = a->vp;
  if (mag) { c.br = a->br; c.bt = a->bt; c.bp = a->bp; }
  c.ld = a->grid_ld;
  c.orho1 = (const double*)cx.dev(irf[0]); c.orho2 = (const double*)cx.dev(irf[1]);
  c.or2 = (const double*)cx.dev(irf[2]); c.or4 = (const double*)cx.dev(irf[3]);
  c.delxr2 = (const double*)cx.dev(irf[4]); c.delxh2 = (const double*)cx.dev(irf[5]);
  c.courfac = a->courfac; c.alffac = a->alffac; c.LFfac = a->LFfac; c.opm = a->opm;
  c.alf_damp = a->l_cour_alf_damp;
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_COURANT, 2);
    CK(launch_courant(g, c, n, (unsigned long long*)cx.dev(i_mx), (double*)cx.dev(i_r), (double*)cx.dev(i_h),
                      h->stream));
  }
  return cx.finish();
}

int magic_sht_v_rigid_boundary(magic_sht_handle* h, double r2_rho0, double omega, int keep_vr,
                               const magic_sht_rigid_args* a) {
  TRY(check_handle(h));
  if (!a || !a->vr || !a->vt || !a->vp) return set_err(MAGIC_SHT_ERR_ARG, "null args or vr/vt/vp");
  DeviceGuard dg(h->device);
  const long long gl = (long long)h->g.n_phi * h->g.ld;
  double* const ps[8] = {a->vr, a->vt, a->vp, a->cvr, a->dvrdt, a->dvrdp, a->dvtdp, a->dvpdp};
  CallCtx cx(h);
  int idx[8];
  // vr is read back unchanged when it is kept, so it is staged both ways
  for (int i = 0; i < 8; ++i) idx[i] = (i == 0 && keep_vr) ? cx.grid_in(ps[i], 1, gl) : cx.grid_out(ps[i], 1, gl);
  TRY(cx.prepare());
  BcGrids b{};
  for (int i = 0; i < 8; ++i) b.p[i] = (i == 0 && keep_vr) ? nullptr : (double*)cx.dev(idx[i]);
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_BCS);
    CK(launch_v_rigid_boundary(h->g, h->d_theta, b, r2_rho0, omega, keep_vr, h->stream));
  }
  return cx.finish();
}

int magic_sht_v_center_sphere(magic_sht_handle* h, const double* ddw, double* vr, double* vt, double* vp) {
  TRY(check_handle(h));
  if (!ddw || !vr || !vt || !vp) return set_err(MAGIC_SHT_ERR_ARG, "null argument");
  if (h->g.l_max < 1) return set_err(MAGIC_SHT_ERR_SIZE, "v_center_sphere needs l_max >= 1");
  DeviceGuard dg(h->device);
  const long long gl = (long long)h->g.n_phi * h->g.ld;
  CallCtx cx(h);
  const int i_s = cx.spec_in(ddw, 1, h->g.lm_max);
  const int i_r = cx.grid_out(vr, 1, gl), i_t = cx.grid_out(vt, 1, gl), i_p = cx.grid_out(vp, 1, gl);
  TRY(cx.prepare());
  const int lm11 = (h->g.minc == 1 && h->g.n_m > 1) ? h->lmoff[1] : -1;
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_BCS);
    CK(launch_v_center_sphere(h->g, h->d_theta, (const double2*)cx.dev(i_s), lm11, (double*)cx.dev(i_r),
                              (double*)cx.dev(i_t), (double*)cx.dev(i_p), h->stream));
  }
  return cx.finish();
}

int magic_sht_get_br_v_bcs(magic_sht_handle* h, const double* br, const double* vt, const double* vp, double omega,
                           double or2, double orho1, double* br_vt_lm, double* br_vp_lm) {
  TRY(check_handle(h));
  if (!br || !vt || !vp || !br_vt_lm || !br_vp_lm) return set_err(MAGIC_SHT_ERR_ARG, "null argument");
  DeviceGuard dg(h->device);
  const ShtGeom& g = h->g;
  const long long gl = (long long)g.n_phi * g.ld;
  CallCtx cx(h);
  const int i_b = cx.grid_in(br, 1, gl), i_t = cx.grid_in(vt, 1, gl), i_p = cx.grid_in(vp, 1, gl);
  const int t_t = cx.tmp((size_t)gl * 8), t_p = cx.tmp((size_t)gl * 8);
  const int o_t = cx.spec_out(br_vt_lm, 1, g.lm_max), o_p = cx.spec_out(br_vp_lm, 1, g.lm_max);
  std::vector<int> hs_vc = {cx.tmp(hs_bytes(h, 1)), cx.tmp(hs_bytes(h, 1))};
  TRY(cx.prepare());
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_BCS);
    CK(launch_br_v_products(g, h->d_theta, (const double*)cx.dev(i_b), (const double*)cx.dev(i_t),
                            (const double*)cx.dev(i_p), or2 * orho1, omega, (double*)cx.dev(t_t),
                            (double*)cx.dev(t_p), h->stream));
  }
  LevelCtl lv;
  lv.nlev = 1; lv.lcut0 = g.l_max;
  lv.spec_ld = g.lm_max; lv.grid_ld = gl;
  std::vector<ScalarFwd> sc;
  std::vector<VectorFwd> vc = {{t_t, t_p, o_t, o_p}};
  TRY(run_forward(h, cx, lv, sc, vc, {}, hs_vc));
  return cx.finish();
}

int magic_sht_lorentz_torque(magic_sht_handle* h, const double* br, const double* bp, double LFfac, double b0,
                             double* torque) {
  TRY(check_handle(h));
  if (!br || !bp || !torque) return set_err(MAGIC_SHT_ERR_ARG, "null argument");
  DeviceGuard dg(h->device);
  const ShtGeom& g = h->g;
  const long long gl = (long long)g.n_phi * g.ld;
  CallCtx cx(h);
  const int i_r = cx.grid_in(br, 1, gl), i_p = cx.grid_in(bp, 1, gl);
  const int i_part = cx.tmp(sizeof(double) * (size_t)lorentz_torque_blocks(g));
  const int i_t = cx.raw_inout(torque, sizeof(double));
  TRY(cx.prepare());
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_BCS, 2);
    CK(launch_lorentz_torque(g, h->d_theta, (const double*)cx.dev(i_r), (const double*)cx.dev(i_p), LFfac, b0,
                             (double*)cx.dev(i_part), (double*)cx.dev(i_t), h->stream));
  }
  return cx.finish();
}

int magic_sht_get_b_nl_bcs(magic_sht_handle* h, double fac, const double* br_vt_lm, const double* br_vp_lm,
                           double* b_nl_bc, double* aj_nl_bc) {
  TRY(check_handle(h));
  if (!br_vp_lm || !aj_nl_bc || (b_nl_bc && !br_vt_lm)) return set_err(MAGIC_SHT_ERR_ARG, "null argument");
  DeviceGuard dg(h->device);
  const int K = h->g.lm_max;
  CallCtx cx(h);
  const int i_vt = b_nl_bc ? cx.spec_in(br_vt_lm, 1, K) : -1, i_vp = cx.spec_in(br_vp_lm, 1, K);
  const int o_b = b_nl_bc ? cx.spec_out(b_nl_bc, 1, K) : -1, o_j = cx.spec_out(aj_nl_bc, 1, K);
  TRY(cx.prepare());
  {
    PhaseScope sc(h, MAGIC_SHT_PHASE_BCS, b_nl_bc ? 2 : 1);
    if (b_nl_bc) CK(launch_b_nl_bcs(K, fac, (const double2*)cx.dev(i_vt), (double2*)cx.dev(o_b), h->stream));
    CK(launch_b_nl_bcs(K, fac, (const double2*)cx.dev(i_vp), (double2*)cx.dev(o_j), h->stream));
  }
  return cx.finish();
}

int magic_sht_dt_courant(int n, const double* dtrkc, const double* dthkc, double dt, double dtMax,
                         int* l_new_dt, double* dt_new) {
  if (!dtrkc || !dthkc || !l_new_dt || !dt_new || n < 0)
    return set_err(MAGIC_SHT_ERR_ARG, "null argument or n_levels < 0");
  const double dt_fac = 2.0;
  double dt_r = 1000.0 * dtMax, dt_h = 1000.0 * dtMax;
  for (int i = 0; i < n; ++i) {
    dt_r = std::min(dtrkc[i], dt_r);
    dt_h = std::min(dthkc[i], dt_h);
  }
  const double dtMin = std::min(dt_r, dt_h);
  const double dt_2 = std::min(0.5 * (1.0 / dt_fac + 1.0) * dtMin, dtMax);
  if (dt > dtMax) {
    *l_new_dt = 1;
    *dt_new = dtMax;
  } else if (dt > dtMin) {
    *l_new_dt = 1;
    *dt_new = dt_2;
  } else if (dt_fac * dt < dtMin && dt < dtMax) {
    *l_new_dt = 1;
    *dt_new = dt_2;
  } else {
    *l_new_dt = 0;
    *dt_new = dt;
  }
  return MAGIC_SHT_OK;
}

int magic_sht_transform_to_lm_space(magic_sht_handle* h, int n, const int* lcut,
                                    const magic_sht_lm_space_args* a) {
  TRY(check_handle(h));
  if (!a || n < 0) return set_err(MAGIC_SHT_ERR_ARG, "null args or n_levels < 0");
  if (n == 0) return MAGIC_SHT_OK;
  const ShtGeom& g = h->g;
  if (a->spec_ld < g.lm_max || a->grid_ld < (long long)g.n_phi * g.ld)
    return set_err(MAGIC_SHT_ERR_ARG, "spec_ld/grid_ld smaller than one level");
  DeviceGuard dg(h->device);
  if (n > h->pipe_chunk && !h->capturing &&
      all_host({lcut, a->Advr, a->Advt, a->Advp, a->VSr, a->VSt, a->VSp, a->VxBr, a->VxBt, a->VxBp, a->heatTerms,
                a->AdvrLM, a->AdvtLM, a->AdvpLM, a->VSrLM, a->VStLM, a->VSpLM, a->VxBrLM, a->VxBtLM,
                a->VxBpLM, a->heatTermsLM, a->VXir, a->VXit, a->VXip, a->VXirLM, a->VXitLM, a->VXipLM})) {
    if (lcut)
      for (int i = 0; i < n; ++i)
        if (!is_device_ptr(lcut) && (lcut[i] < 0 || lcut[i] > g.l_max))
          return set_err(MAGIC_SHT_ERR_LCUT, "lcut[%d]=%d outside [0, %d]", i, lcut[i], g.l_max);
    constexpr int NF = 13;
    const double* const ins[NF] = {a->Advr, a->Advt, a->Advp, a->VSr, a->VSt, a->VSp, a->VxBr,
                                   a->VxBt, a->VxBp, a->heatTerms, a->VXir, a->VXit, a->VXip};
    double* const outs[NF] = {a->AdvrLM, a->AdvtLM, a->AdvpLM, a->VSrLM, a->VStLM, a->VSpLM, a->VxBrLM,
                              a->VxBtLM, a->VxBpLM, a->heatTermsLM, a->VXirLM, a->VXitLM, a->VXipLM};
    std::vector<PipeArray> arrs;
    std::vector<int> idx_in(NF, -1), idx_out(NF, -1);
    const size_t sb = (size_t)a->spec_ld * 16, gb = (size_t)a->grid_ld * 8;
    for (int i = 0; i < NF; ++i)
      if (ins[i]) { idx_in[i] = (int)arrs.size(); arrs.push_back({ins[i], gb, (size_t)g.n_phi * g.ld * 8, false, 0}); }
    for (int i = 0; i < NF; ++i)
      if (outs[i]) { idx_out[i] = (int)arrs.size(); arrs.push_back({outs[i], sb, (size_t)g.lm_max * 16, true, 0}); }
    if (lcut) arrs.push_back({lcut, 4, 4, false, 0});
    const int i_lc = lcut ? (int)arrs.size() - 1 : -1;
    return pipelined_levels(h, n, h->pipe_chunk, arrs, [&](int r0, int nr, const std::vector<char*>& d) {
      magic_sht_lm_space_args b = *a;
      const double** pin[NF] = {&b.Advr, &b.Advt, &b.Advp, &b.VSr, &b.VSt, &b.VSp, &b.VxBr, &b.VxBt,
                                &b.VxBp, &b.heatTerms, &b.VXir, &b.VXit, &b.VXip};
      double** pout[NF] = {&b.AdvrLM, &b.AdvtLM, &b.AdvpLM, &b.VSrLM, &b.VStLM, &b.VSpLM, &b.VxBrLM,
                           &b.VxBtLM, &b.VxBpLM, &b.heatTermsLM, &b.VXirLM, &b.VXitLM, &b.VXipLM};
      for (int i = 0; i < NF; ++i) *pin[i] = idx_in[i] >= 0 ? (const double*)d[idx_in[i]] : nullptr;
      for (int i = 0; i < NF; ++i) *pout[i] = idx_out[i] >= 0 ? (double*)d[idx_out[i]] : nullptr;
      (void)r0;
      return magic_sht_transform_to_lm_space(h, nr, i_lc >= 0 ? (const int*)d[i_lc] : nullptr, &b);
    });
  }
  CallCtx cx(h);
  LevelCtl lv;
  std::vector<int> lc;
  TRY(level_ctl(h, cx, n, lcut, nullptr, lv, lc));
  lv.spec_ld = a->spec_ld;
  lv.grid_ld = a->grid_ld;
  auto gi = [&](const double* p) { return cx.grid_in(p, n, a->grid_ld); };
  auto so = [&](double* p) { return cx.spec_out(p, n, a->spec_ld); };
  std::vector<ScalarFwd> sc;
  std::vector<VectorFwd> vc;
  struct Q { const double *f, *g, *h; double *q, *s, *t; };
  const Q qs[4] = {{a->Advr, a->Advt, a->Advp, a->AdvrLM, a->AdvtLM, a->AdvpLM},
                   {a->VSr, a->VSt, a->VSp, a->VSrLM, a->VStLM, a->VSpLM},
                   {a->VxBr, a->VxBt, a->VxBp, a->VxBrLM, a->VxBtLM, a->VxBpLM},
                   {a->VXir, a->VXit, a->VXip, a->VXirLM, a->VXitLM, a->VXipLM}};
  for (const Q& q : qs) {
    if (q.f && q.q) sc.push_back({gi(q.f), so(q.q)});
    if (q.g && q.h && q.s && q.t) vc.push_back({gi(q.g), gi(q.h), so(q.s), so(q.t)});
  }
  if (a->heatTerms && a->heatTermsLM) sc.push_back({gi(a->heatTerms), so(a->heatTermsLM)});
  std::vector<int> hs_sc, hs_vc;
  for (size_t i = 0; i < sc.size(); ++i) hs_sc.push_back(cx.tmp(hs_bytes(h, n)));
  for (size_t i = 0; i < 2 * vc.size(); ++i) hs_vc.push_back(cx.tmp(hs_bytes(h, n)));
  TRY(cx.prepare());
  TRY(run_forward(h, cx, lv, sc, vc, hs_sc, hs_vc));
  return cx.finish();
}

// ------------------------------------------------ batched facade jobs
// Any facade routines over many levels in one call: each job becomes the
// scalar / vector jobs its single-level routine builds (above), and all of
// them go through one run_inverse / run_forward.
namespace {
struct JobShape {
  int n_in, n_out;
  bool inv;
};
bool job_shape(int routine, JobShape& s) {
  switch (routine) {
    case MAGIC_SHT_JOB_SCAL_TO_SPAT: s = {1, 1, true}; return true;
    case MAGIC_SHT_JOB_SCAL_TO_GRAD_SPAT: s = {1, 2, true}; return true;
    case MAGIC_SHT_JOB_POL_TO_GRAD_SPAT: s = {1, 2, true}; return true;
    case MAGIC_SHT_JOB_TORPOL_TO_SPAT: s = {3, 3, true}; return true;
    case MAGIC_SHT_JOB_SPHTOR_TO_SPAT: s = {2, 2, true}; return true;
    case MAGIC_SHT_JOB_TORPOL_TO_CURL_SPAT: s = {4, 3, true}; return true;
    case MAGIC_SHT_JOB_POL_TO_CURLR_SPAT: s = {1, 1, true}; return true;
    case MAGIC_SHT_JOB_TORPOL_TO_DPHSPAT: s = {2, 2, true}; return true;
    case MAGIC_SHT_JOB_SCAL_TO_SH: s = {1, 1, false}; return true;
    case MAGIC_SHT_JOB_SPAT_TO_QST: s = {3, 3, false}; return true;
    case MAGIC_SHT_JOB_SPAT_TO_SPHERTOR: s = {2, 2, false}; return true;
    default: return false;
  }
}
}  // namespace

static int batch_jobs(magic_sht_handle* h, bool inv, int n, const double* or2, const int* lcut, long long spec_ld,
                      long long grid_ld, const magic_sht_job* jobs, int n_jobs) {
  TRY(check_handle(h));
  if (n < 0 || n_jobs < 0 || (n_jobs > 0 && !jobs)) return set_err(MAGIC_SHT_ERR_ARG, "null jobs or negative counts");
  if (n == 0 || n_jobs == 0) return MAGIC_SHT_OK;
  const ShtGeom& g = h->g;
  if (spec_ld < g.lm_max || grid_ld < (long long)g.n_phi * g.ld)
    return set_err(MAGIC_SHT_ERR_ARG, "spec_ld/grid_ld smaller than one level");
  bool curl = false;
  std::vector<const void*> all;
  std::vector<const double*> ins, outs;
  for (int j = 0; j < n_jobs; ++j) {
    JobShape s;
    if (!job_shape(jobs[j].routine, s) || s.inv != inv)
      return set_err(MAGIC_SHT_ERR_ARG, "job %d: routine %d is not a %s routine", j, jobs[j].routine,
                     inv ? "synthesis" : "analysis");
    for (int k = 0; k < 4; ++k)
      if ((k < s.n_in) != (jobs[j].in[k] != nullptr))
        return set_err(MAGIC_SHT_ERR_ARG, "job %d: input %d %s", j, k, k < s.n_in ? "missing" : "not used (NULL)");
    for (int k = 0; k < 3; ++k)
      if ((k < s.n_out) != (jobs[j].out[k] != nullptr))
        return set_err(MAGIC_SHT_ERR_ARG, "job %d: output %d %s", j, k, k < s.n_out ? "missing" : "not used (NULL)");
    for (int k = 0; k < s.n_in; ++k) { ins.push_back(jobs[j].in[k]); all.push_back(jobs[j].in[k]); }
    for (int k = 0; k < s.n_out; ++k) { outs.push_back(jobs[j].out[k]); all.push_back(jobs[j].out[k]); }
    curl = curl || jobs[j].routine == MAGIC_SHT_JOB_TORPOL_TO_CURL_SPAT;
  }
  if (curl && !or2) return set_err(MAGIC_SHT_ERR_ARG, "torpol_to_curl_spat jobs need or2 per level");
  {
    std::vector<const double*> o = outs;
    std::sort(o.begin(), o.end());
    if (std::adjacent_find(o.begin(), o.end()) != o.end()) return set_err(MAGIC_SHT_ERR_ARG, "repeated output array");
    for (const double* p : ins)
      if (std::binary_search(o.begin(), o.end(), p)) return set_err(MAGIC_SHT_ERR_ARG, "an output is also an input");
  }
  DeviceGuard dg(h->device);
  const size_t sb = (size_t)spec_ld * 16, gb = (size_t)grid_ld * 8;
  const size_t s_last = (size_t)g.lm_max * 16, g_last = (size_t)g.n_phi * g.ld * 8;
  all.push_back(lcut);
  all.push_back(or2);
  if (n > h->pipe_chunk && !h->capturing && all_host_v(all)) {
    if (lcut)
      for (int i = 0; i < n; ++i)
        if (lcut[i] < 0 || lcut[i] > g.l_max)
          return set_err(MAGIC_SHT_ERR_LCUT, "lcut[%d]=%d outside [0, %d]", i, lcut[i], g.l_max);
    // one pipelined array per distinct input and per output
    std::vector<PipeArray> arrs;
    std::map<const double*, int> seen;
    std::vector<std::array<int, 4>> iin(n_jobs);
    std::vector<std::array<int, 3>> iout(n_jobs);
    for (int j = 0; j < n_jobs; ++j) {
      JobShape s;
      job_shape(jobs[j].routine, s);
      for (int k = 0; k < s.n_in; ++k) {
        const double* p = jobs[j].in[k];
        auto it = seen.find(p);
        if (it == seen.end()) {
          it = seen.emplace(p, (int)arrs.size()).first;
          arrs.push_back({p, inv ? sb : gb, inv ? s_last : g_last, false, 0});
        }
        iin[j][k] = it->second;
      }
      for (int k = 0; k < s.n_out; ++k) {
        iout[j][k] = (int)arrs.size();
        arrs.push_back({jobs[j].out[k], inv ? gb : sb, inv ? g_last : s_last, true, 0});
      }
    }
    const int i_or2 = or2 ? (int)arrs.size() : -1;
    if (or2) arrs.push_back({or2, 8, 8, false, 0});
    const int i_lc = lcut ? (int)arrs.size() : -1;
    if (lcut) arrs.push_back({lcut, 4, 4, false, 0});
    return pipelined_levels(h, n, h->pipe_chunk, arrs, [&](int r0, int nr, const std::vector<char*>& d) {
      std::vector<magic_sht_job> b(jobs, jobs + n_jobs);
      for (int j = 0; j < n_jobs; ++j) {
        JobShape s;
        job_shape(jobs[j].routine, s);
        for (int k = 0; k < s.n_in; ++k) b[j].in[k] = (const double*)d[iin[j][k]];
        for (int k = 0; k < s.n_out; ++k) b[j].out[k] = (double*)d[iout[j][k]];
      }
      (void)r0;
      return batch_jobs(h, inv, nr, i_or2 >= 0 ? (const double*)d[i_or2] : nullptr,
                        i_lc >= 0 ? (const int*)d[i_lc] : nullptr, spec_ld, grid_ld, b.data(), n_jobs);
    });
  }
  CallCtx cx(h);
  LevelCtl lv;
  std::vector<int> lc;
  TRY(level_ctl(h, cx, n, lcut, or2, lv, lc));
  lv.spec_ld = spec_ld;
  lv.grid_ld = grid_ld;
  std::map<const double*, int> seen;
  auto in_idx = [&](const double* p) {
    auto it = seen.find(p);
    if (it != seen.end()) return it->second;
    const int i = inv ? cx.spec_in(p, n, spec_ld) : cx.grid_in(p, n, grid_ld);
    seen.emplace(p, i);
    return i;
  };
  std::vector<int> hs_sc, hs_vc;
  if (inv) {
    std::vector<ScalarInv> sc;
    std::vector<VectorInv> vc;
    for (int j = 0; j < n_jobs; ++j) {
      JobShape sh;
      job_shape(jobs[j].routine, sh);
      int s[4], o[3];
      for (int k = 0; k < sh.n_in; ++k) s[k] = in_idx(jobs[j].in[k]);
      for (int k = 0; k < sh.n_out; ++k) o[k] = cx.grid_out(jobs[j].out[k], n, grid_ld);
      switch (jobs[j].routine) {  // as the single-level routines above
        case MAGIC_SHT_JOB_SCAL_TO_SPAT: sc.push_back({ref(OP_COPY, s[0]), o[0], 0}); break;
        case MAGIC_SHT_JOB_POL_TO_CURLR_SPAT: sc.push_back({ref(OP_DLH, s[0]), o[0], 0}); break;
        case MAGIC_SHT_JOB_SCAL_TO_GRAD_SPAT: vc.push_back({ref(OP_COPY, s[0]), SpecRef(), o[0], o[1], 0}); break;
        case MAGIC_SHT_JOB_POL_TO_GRAD_SPAT: vc.push_back({ref(OP_DLH, s[0]), SpecRef(), o[0], o[1], 0}); break;
        case MAGIC_SHT_JOB_TORPOL_TO_SPAT:
          sc.push_back({ref(OP_DLH, s[0]), o[0], 0});
          vc.push_back({ref(OP_COPY, s[1]), ref(OP_COPY, s[2]), o[1], o[2], 0});
          break;
        case MAGIC_SHT_JOB_SPHTOR_TO_SPAT: vc.push_back({ref(OP_COPY, s[0]), ref(OP_COPY, s[1]), o[0], o[1], 0}); break;
        case MAGIC_SHT_JOB_TORPOL_TO_DPHSPAT:
          vc.push_back({ref(OP_IM, s[0]), ref(OP_IM, s[1]), o[0], o[1], FFT_OSIN2});
          break;
        case MAGIC_SHT_JOB_TORPOL_TO_CURL_SPAT:
          sc.push_back({ref(OP_DLH, s[2]), o[0], 0});
          vc.push_back({ref(OP_COPY, s[3]), ref(OP_CURLT, s[0], s[1]), o[1], o[2], 0});
          break;
        default: break;
      }
    }
    for (size_t i = 0; i < sc.size(); ++i) hs_sc.push_back(cx.tmp(hs_bytes(h, n)));
    for (size_t i = 0; i < 2 * vc.size(); ++i) hs_vc.push_back(cx.tmp(hs_inv_bytes(h, n, true)));
    TRY(cx.prepare());
    TRY(run_inverse(h, cx, lv, sc, vc, hs_sc, hs_vc));
  } else {
    std::vector<ScalarFwd> sc;
    std::vector<VectorFwd> vc;
    for (int j = 0; j < n_jobs; ++j) {
      JobShape sh;
      job_shape(jobs[j].routine, sh);
      int gi[4], so[3];
      for (int k = 0; k < sh.n_in; ++k) gi[k] = in_idx(jobs[j].in[k]);
      for (int k = 0; k < sh.n_out; ++k) so[k] = cx.spec_out(jobs[j].out[k], n, spec_ld);
      switch (jobs[j].routine) {
        case MAGIC_SHT_JOB_SCAL_TO_SH: sc.push_back({gi[0], so[0]}); break;
        case MAGIC_SHT_JOB_SPAT_TO_QST:
          sc.push_back({gi[0], so[0]});
          vc.push_back({gi[1], gi[2], so[1], so[2]});
          break;
        case MAGIC_SHT_JOB_SPAT_TO_SPHERTOR: vc.push_back({gi[0], gi[1], so[0], so[1]}); break;
        default: break;
      }
    }
    for (size_t i = 0; i < sc.size(); ++i) hs_sc.push_back(cx.tmp(hs_bytes(h, n)));
    for (size_t i = 0; i < 2 * vc.size(); ++i) hs_vc.push_back(cx.tmp(hs_bytes(h, n)));
    TRY(cx.prepare());
    TRY(run_forward(h, cx, lv, sc, vc, hs_sc, hs_vc));
  }
  return cx.finish();
}

int magic_sht_inv_batch(magic_sht_handle* h, int n, const double* or2, const int* lcut, long long spec_ld,
                        long long grid_ld, const magic_sht_job* jobs, int n_jobs) {
  return batch_jobs(h, true, n, or2, lcut, spec_ld, grid_ld, jobs, n_jobs);
}

int magic_sht_fwd_batch(magic_sht_handle* h, int n, const int* lcut, long long grid_ld, long long spec_ld,
                        const magic_sht_job* jobs, int n_jobs) {
  return batch_jobs(h, false, n, nullptr, lcut, spec_ld, grid_ld, jobs, n_jobs);
}

// ------------------------------------------------------------ graphs
int magic_sht_graph_begin(magic_sht_handle* h) {
  TRY(check_handle(h));
  if (h->capturing) return set_err(MAGIC_SHT_ERR_ARG, "capture already active");
  if (h->stream == nullptr)
    return set_err(MAGIC_SHT_ERR_ARG, "graph capture needs a non-default stream (magic_sht_set_stream)");
  DeviceGuard dg(h->device);
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  h->capturing = true;
  return MAGIC_SHT_OK;
}

int magic_sht_graph_end(magic_sht_handle* h, magic_sht_graph** out) {
  TRY(check_handle(h));
  if (!out) return set_err(MAGIC_SHT_ERR_ARG, "null output");
  if (!h->capturing) return set_err(MAGIC_SHT_ERR_ARG, "no capture active");
  DeviceGuard dg(h->device);
  h->capturing = false;
  magic_sht_graph* gr = new magic_sht_graph();
  cudaError_t e = cudaStreamEndCapture(h->stream, &gr->graph);
  if (e != cudaSuccess) {
    delete gr;
    return set_err(MAGIC_SHT_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&gr->exec, gr->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(gr->graph);
    delete gr;
    return set_err(MAGIC_SHT_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
  }
  *out = gr;
  return MAGIC_SHT_OK;
}

int magic_sht_graph_launch(magic_sht_handle* h, const magic_sht_graph* gr) {
  TRY(check_handle(h));
  if (!gr) return set_err(MAGIC_SHT_ERR_ARG, "null graph");
  DeviceGuard dg(h->device);
  CK(cudaGraphLaunch(gr->exec, h->stream));
  return MAGIC_SHT_OK;
}

int magic_sht_graph_destroy(magic_sht_graph* gr) {
  if (!gr) return MAGIC_SHT_OK;
  if (gr->exec) cudaGraphExecDestroy(gr->exec);
  if (gr->graph) cudaGraphDestroy(gr->graph);
  delete gr;
  return MAGIC_SHT_OK;
}

}  // extern "C"

// ------------------------------------------------------------ groups
// Several instances (handles of different l_max, minc and grids, all in the
// FP64-accurate or all in the 3xBF16 tensor-core form) transformed together: each handle builds
// its call as usual, but its Legendre and FFT launches are collected
// (magic_sht_handle::defer); then one pack + one persistent tensor-core launch
// per direction and field kind covers the tiles of every instance, heaviest
// instances first, and the FFTs follow (synthesis) or precede (analysis).
struct magic_sht_group {
  std::vector<magic_sht_handle*> h;
  int device = 0;
  // Device copies of the launches' instance arrays.  A call captured into a
  // graph takes new kept slots: append-only while the group lives, copied by
  // the graph itself (a memcpy node from pinned memory that is never
  // rewritten), so every replay reads what was captured and nothing outside
  // that graph reads them (their device copies exist only once it runs).
  // Other calls take a slot of a device ring written from pageable memory on
  // the group's stream (the copy is staged before it returns, and stream
  // order puts it after every earlier launch that read the slot), so repeated
  // calls with new arrays reuse the same memory.
  struct Chunk {
    char* host = nullptr;  // pinned: the source of the asynchronous copies
    char* dev = nullptr;
    size_t cap = 0, used = 0;
  };
  std::vector<Chunk> chunks;
  char* ring = nullptr;
  size_t ring_cap = 0, ring_off = 0;
  // the FFTs of different instances run on these streams, forked from and
  // joined back into the call's stream (one event each way per stream)
  static constexpr int kFftStreams = 4;
  cudaStream_t fft_st[kFftStreams] = {};
  cudaEvent_t fork = nullptr, join[kFftStreams] = {};
};

namespace {


constexpr size_t kGroupChunk = 1 << 20;  // kept copies for captured calls
constexpr size_t kGroupRing = 2 << 20;   // ring of the uncaptured calls (many calls' arrays)

// a kept chunk with `need` free bytes (allocated outside a capture only)
int group_chunk(magic_sht_group* G, size_t need, bool capturing) {
  if (!G->chunks.empty() && G->chunks.back().used + need <= G->chunks.back().cap) return MAGIC_SHT_OK;
  if (capturing)
    return set_err(MAGIC_SHT_ERR_NOMEM,
                   "group instance tables for captured calls are full: make a group call outside the capture "
                   "first (it reserves room for them)");
  magic_sht_group::Chunk c;
  c.cap = std::max(kGroupChunk, need);
  CK(cudaHostAlloc((void**)&c.host, c.cap, cudaHostAllocDefault));
  if (cudaMalloc((void**)&c.dev, c.cap) != cudaSuccess) {
    cudaFreeHost(c.host);
    cudaGetLastError();
    return set_err(MAGIC_SHT_ERR_NOMEM, "group instance tables: cudaMalloc of %zu bytes failed", c.cap);
  }
  G->chunks.push_back(c);
  return MAGIC_SHT_OK;
}

int group_upload(magic_sht_group* G, const void* p, size_t bytes, bool capturing, cudaStream_t st,
                 const void** out) {
  const size_t need = align256(bytes);
  if (!capturing) {
    // room for the kept copies of a capture that may follow
    TRY(group_chunk(G, 2 * kMaxGroupInst * sizeof(LegInst<InvSet>), false));
    if (need > G->ring_cap) {
      if (G->ring) {
        CK(cudaStreamSynchronize(st));
        CK(cudaFree(G->ring));
        G->ring = nullptr;
        G->ring_cap = 0;
      }
      const size_t cap = std::max(kGroupRing, 4 * need);
      CK(cudaMalloc((void**)&G->ring, cap));
      G->ring_cap = cap;
      G->ring_off = 0;
    }
    if (G->ring_off + need > G->ring_cap) G->ring_off = 0;
    char* dp = G->ring + G->ring_off;
    G->ring_off += need;
    CK(cudaMemcpyAsync(dp, p, bytes, cudaMemcpyHostToDevice, st));  // pageable: staged before it returns
    *out = dp;
    return MAGIC_SHT_OK;
  }
  TRY(group_chunk(G, need, true));
  magic_sht_group::Chunk& c = G->chunks.back();
  char* hp = c.host + c.used;
  char* dp = c.dev + c.used;
  c.used += need;
  memcpy(hp, p, bytes);
  CK(cudaMemcpyAsync(dp, hp, bytes, cudaMemcpyHostToDevice, st));
  *out = dp;
  return MAGIC_SHT_OK;
}

// one pack + one persistent launch over the collected Legendre launches of
// one direction and field kind
template <class Set>
int group_legendre(magic_sht_group* G, const Deferred& D, bool inverse, bool vec, bool capturing, cudaStream_t st) {
  std::vector<LegInst<Set>> v;
  for (const auto& j : D.leg) {
    if (j.inverse != inverse || j.vec != vec) continue;
    LegInst<Set> I;
    memset(&I, 0, sizeof(I));
    I.g = j.h->g;
    if constexpr (std::is_same<Set, InvSet>::value) I.s = j.inv;
    else I.s = j.fwd;
    I.t = j.h->tct;
    I.bimg = j.h->d_bimg + j.bimg_off;
    if (I.s.nf * I.s.nlev > 0) v.push_back(I);
  }
  if (v.empty()) return MAGIC_SHT_OK;
  if (v.size() > (size_t)kMaxGroupInst)
    return set_err(MAGIC_SHT_ERR_SIZE, "group call of %zu instance sets of one kind (at most %d)", v.size(),
                   kMaxGroupInst);
  // the heaviest tiles (the largest l_max) are handed out first
  std::stable_sort(v.begin(), v.end(),
                   [](const LegInst<Set>& a, const LegInst<Set>& b) { return a.g.l_max > b.g.l_max; });
  magic_sht_handle* h0 = G->h[0];
  const bool oz = oz_form(h0);
  long long nblocks = 0, ntiles = 0;
  if (oz) oz_layout_insts(v.data(), (int)v.size(), vec, &nblocks, &ntiles);
  else tcp_layout_insts(v.data(), (int)v.size(), vec, &nblocks, &ntiles);
  if (ntiles >= (1LL << 31) || nblocks >= (1LL << 31))
    return set_err(MAGIC_SHT_ERR_SIZE, "group call of %lld tiles: split it", ntiles);
  const void* dv = nullptr;
  TRY(group_upload(G, v.data(), v.size() * sizeof(LegInst<Set>), capturing, st, &dv));
  const int ph = inverse ? (vec ? MAGIC_SHT_PHASE_INV_LEG_VECTOR : MAGIC_SHT_PHASE_INV_LEG_SCALAR)
                         : (vec ? MAGIC_SHT_PHASE_FWD_LEG_VECTOR : MAGIC_SHT_PHASE_FWD_LEG_SCALAR);
  PhaseScope ps(h0, ph, 2);
  const int n = (int)v.size();
  if constexpr (std::is_same<Set, InvSet>::value) {
    const LegInst<InvSet>* d = (const LegInst<InvSet>*)dv;
    CK(oz ? launch_inv_legendre_oz_multi(v.data(), d, n, vec, nblocks, ntiles, st)
          : launch_inv_legendre_tcp_multi(v.data(), d, n, vec, nblocks, ntiles, st));
  } else {
    const LegInst<FwdSet>* d = (const LegInst<FwdSet>*)dv;
    CK(oz ? launch_fwd_legendre_oz_multi(v.data(), d, n, vec, nblocks, ntiles, st)
          : launch_fwd_legendre_tcp_multi(v.data(), d, n, vec, nblocks, ntiles, st));
  }
  return MAGIC_SHT_OK;
}

// The FFT launches of the instances: consecutive instances on different
// streams forked from `st`, so that the FFTs of small instances overlap the
// others' (each launch counted in its handle's phase counters, untimed: the
// phase events are recorded on the handle's stream only).
int group_ffts(magic_sht_group* G, const Deferred& D, bool inverse, cudaStream_t st) {
  constexpr int K = magic_sht_group::kFftStreams;
  int n = 0;
  for (const auto& f : D.fft) n += f.inverse == inverse;
  if (n == 0) return MAGIC_SHT_OK;
  CK(cudaEventRecord(G->fork, st));
  const int ns = std::min(n, K);
  for (int k = 0; k < ns; ++k) CK(cudaStreamWaitEvent(G->fft_st[k], G->fork, 0));
  int i = 0;
  magic_sht_handle* prev = nullptr;
  for (const auto& f : D.fft) {
    if (f.inverse != inverse) continue;
    magic_sht_handle* h = f.h;
    if (prev && h != prev) ++i;  // the FFT batches of one instance stay on one stream
    prev = h;
    const int ph = inverse ? MAGIC_SHT_PHASE_FFT_INV : MAGIC_SHT_PHASE_FFT_FWD;
    h->launches++;
    h->phase_launches[ph]++;
    cudaStream_t s = G->fft_st[i % ns];
    if (inverse) CK(launch_fft_inverse(h->g, f.fs, fft_arith(h), h->fft_rows, s));
    else CK(launch_fft_forward(h->g, f.fs, fft_arith(h), h->fft_rows, s));
  }
  for (int k = 0; k < ns; ++k) {
    CK(cudaEventRecord(G->join[k], G->fft_st[k]));
    CK(cudaStreamWaitEvent(st, G->join[k], 0));
  }
  return MAGIC_SHT_OK;
}

// a group call: the checks, then every instance's call with its launches
// collected, then the group launches
int group_call(magic_sht_group* G, bool inverse, const std::vector<const void*>& arrays,
               const std::function<int(int)>& call) {
  if (!G) return set_err(MAGIC_SHT_ERR_ARG, "null group");
  magic_sht_handle* h0 = G->h[0];
  const cudaStream_t st = h0->stream;
  for (magic_sht_handle* h : G->h) {
    if (h->stream != st)
      return set_err(MAGIC_SHT_ERR_ARG, "the handles of a group share one stream (magic_sht_set_stream)");
    if (!h->tc_persistent)
      return set_err(MAGIC_SHT_ERR_UNSUPPORTED, "group calls need the persistent tensor-core kernels (tc_kernel 0)");
  }
  for (const void* p : arrays)
    if (p && !is_device_ptr(p))
      return set_err(MAGIC_SHT_ERR_ARG, "group calls take device arrays for the spectra and grids");
  DeviceGuard dg(G->device);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(st, &cs));
  const bool capturing = cs == cudaStreamCaptureStatusActive;
  Deferred D;
  std::vector<char> was(G->h.size());
  for (size_t i = 0; i < G->h.size(); ++i) was[i] = G->h[i]->capturing;
  int rc = MAGIC_SHT_OK;
  for (size_t i = 0; i < G->h.size() && rc == MAGIC_SHT_OK; ++i) {
    magic_sht_handle* h = G->h[i];
    h->capturing = h->capturing || capturing;
    h->defer = &D;
    h->defer_bimg = 0;
    rc = call((int)i);
    h->defer = nullptr;
  }
  for (size_t i = 0; i < G->h.size() && rc == MAGIC_SHT_OK; ++i)
    if (G->h[i]->defer_bimg) rc = ensure_bimg(G->h[i], G->h[i]->defer_bimg);
  if (rc == MAGIC_SHT_OK) {
    if (inverse) {
      rc = group_legendre<InvSet>(G, D, true, false, capturing, st);
      if (!rc) rc = group_legendre<InvSet>(G, D, true, true, capturing, st);
      if (!rc) rc = group_ffts(G, D, true, st);
    } else {
      rc = group_ffts(G, D, false, st);
      if (!rc) rc = group_legendre<FwdSet>(G, D, false, false, capturing, st);
      if (!rc) rc = group_legendre<FwdSet>(G, D, false, true, capturing, st);
    }
  }
  for (size_t i = 0; i < G->h.size(); ++i) G->h[i]->capturing = was[i];
  return rc;
}

}  // namespace

extern "C" {

int magic_sht_group_create(magic_sht_handle* const* handles, int n, magic_sht_group** out) {
  if (!handles || !out || n <= 0) return set_err(MAGIC_SHT_ERR_ARG, "null handles/output or n <= 0");
  if (n > kMaxGroupInst) return set_err(MAGIC_SHT_ERR_SIZE, "a group holds at most %d handles", kMaxGroupInst);
  for (int i = 0; i < n; ++i) {
    if (!handles[i]) return set_err(MAGIC_SHT_ERR_ARG, "null handle %d", i);
    if (handles[i]->device != handles[0]->device)
      return set_err(MAGIC_SHT_ERR_ARG, "the handles of a group are on one device");
    const int pr = handles[i]->precision;
    if (pr != MAGIC_SHT_FP64TC && pr != MAGIC_SHT_BF16X5 && pr != MAGIC_SHT_BF16X3)
      return set_err(MAGIC_SHT_ERR_UNSUPPORTED, "group calls need a persistent tensor-core form (handle %d)", i);
    if (pr != handles[0]->precision)
      return set_err(MAGIC_SHT_ERR_ARG, "the handles of a group share one arithmetic form (handle %d)", i);
    for (int k = 0; k < i; ++k)
      if (handles[k] == handles[i]) return set_err(MAGIC_SHT_ERR_ARG, "handle %d appears twice in the group", i);
  }
  DeviceGuard dg(handles[0]->device);
  magic_sht_group* G = new magic_sht_group();
  G->h.assign(handles, handles + n);
  G->device = handles[0]->device;
  bool ok = cudaEventCreateWithFlags(&G->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < magic_sht_group::kFftStreams && ok; ++k)
    ok = cudaStreamCreateWithFlags(&G->fft_st[k], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&G->join[k], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    magic_sht_group_destroy(G);
    return set_err(MAGIC_SHT_ERR_CUDA, "group: stream or event creation failed");
  }
  *out = G;
  return MAGIC_SHT_OK;
}

int magic_sht_group_destroy(magic_sht_group* G) {
  if (!G) return MAGIC_SHT_OK;
  DeviceGuard dg(G->device);
  cudaDeviceSynchronize();
  for (auto& c : G->chunks) {
    if (c.dev) cudaFree(c.dev);
    if (c.host) cudaFreeHost(c.host);
  }
  if (G->ring) cudaFree(G->ring);
  for (int k = 0; k < magic_sht_group::kFftStreams; ++k) {
    if (G->fft_st[k]) cudaStreamDestroy(G->fft_st[k]);
    if (G->join[k]) cudaEventDestroy(G->join[k]);
  }
  if (G->fork) cudaEventDestroy(G->fork);
  delete G;
  return MAGIC_SHT_OK;
}

int magic_sht_group_transform_to_grid_space(magic_sht_group* G, const int* n_levels, const double* const* or2,
                                            const int* const* lcut, const magic_sht_grid_space_args* a) {
  if (!G || !n_levels || !a) return set_err(MAGIC_SHT_ERR_ARG, "null group, n_levels or args");
  std::vector<const void*> arr;
  for (size_t i = 0; i < G->h.size(); ++i) {
    const magic_sht_grid_space_args& b = a[i];
    for (const void* p : {(const void*)b.s, (const void*)b.p, (const void*)b.xi, (const void*)b.w,
                          (const void*)b.dw, (const void*)b.ddw, (const void*)b.z, (const void*)b.dz,
                          (const void*)b.b, (const void*)b.db, (const void*)b.ddb, (const void*)b.aj,
                          (const void*)b.dj, (const void*)b.sc, (const void*)b.pc, (const void*)b.xic,
                          (const void*)b.vrc, (const void*)b.vtc, (const void*)b.vpc, (const void*)b.cvrc,
                          (const void*)b.cvtc, (const void*)b.cvpc, (const void*)b.brc, (const void*)b.btc,
                          (const void*)b.bpc, (const void*)b.cbrc, (const void*)b.cbtc, (const void*)b.cbpc,
                          (const void*)b.dvrdrc, (const void*)b.dvtdrc, (const void*)b.dvpdrc,
                          (const void*)b.dvrdtc, (const void*)b.dvrdpc, (const void*)b.dvtdpc,
                          (const void*)b.dvpdpc})
      arr.push_back(p);
  }
  return group_call(G, true, arr, [&](int i) {
    return magic_sht_transform_to_grid_space(G->h[i], n_levels[i], or2 ? or2[i] : nullptr,
                                             lcut ? lcut[i] : nullptr, &a[i]);
  });
}

int magic_sht_group_transform_to_lm_space(magic_sht_group* G, const int* n_levels, const int* const* lcut,
                                          const magic_sht_lm_space_args* a) {
  if (!G || !n_levels || !a) return set_err(MAGIC_SHT_ERR_ARG, "null group, n_levels or args");
  std::vector<const void*> arr;
  for (size_t i = 0; i < G->h.size(); ++i) {
    const magic_sht_lm_space_args& b = a[i];
    for (const void* p :
         {(const void*)b.Advr, (const void*)b.Advt, (const void*)b.Advp, (const void*)b.VSr, (const void*)b.VSt,
          (const void*)b.VSp, (const void*)b.VxBr, (const void*)b.VxBt, (const void*)b.VxBp,
          (const void*)b.heatTerms, (const void*)b.AdvrLM, (const void*)b.AdvtLM, (const void*)b.AdvpLM,
          (const void*)b.VSrLM, (const void*)b.VStLM, (const void*)b.VSpLM, (const void*)b.VxBrLM,
          (const void*)b.VxBtLM, (const void*)b.VxBpLM, (const void*)b.heatTermsLM, (const void*)b.VXir,
          (const void*)b.VXit, (const void*)b.VXip, (const void*)b.VXirLM, (const void*)b.VXitLM,
          (const void*)b.VXipLM})
      arr.push_back(p);
  }
  return group_call(G, false, arr, [&](int i) {
    return magic_sht_transform_to_lm_space(G->h[i], n_levels[i], lcut ? lcut[i] : nullptr, &a[i]);
  });
}

// ------------------------------------------------------------ profiling
int magic_sht_set_profiling(magic_sht_handle* h, int on) {
  TRY(check_handle(h));
  h->profiling = on != 0;
  return MAGIC_SHT_OK;
}

int magic_sht_phase_times(magic_sht_handle* h, double* ms, long long* launches, int reset) {
  TRY(check_handle(h));
  DeviceGuard dg(h->device);
  CK(cudaStreamSynchronize(h->stream));
  for (auto& m : h->ev_marks) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, m.second.first, m.second.second));
    h->phase_ms[m.first] += t;
  }
  h->ev_marks.clear();
  h->ev_used = 0;
  for (int i = 0; i < MAGIC_SHT_N_PHASES; ++i) {
    if (ms) ms[i] = h->phase_ms[i];
    if (launches) launches[i] = h->phase_launches[i];
    if (reset) { h->phase_ms[i] = 0.0; h->phase_launches[i] = 0; }
  }
  return MAGIC_SHT_OK;
}

int magic_sht_device_status(magic_sht_handle* h, int clear) {
  TRY(check_handle(h));
  DeviceGuard dg(h->device);
  int v = 0;
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(&v, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (clear) CK(cudaMemset(h->d_err, 0, sizeof(int)));
  if (v) return set_err(MAGIC_SHT_ERR_TIMEOUT, "a bounded device wait gave up in a tensor-core kernel");
  return MAGIC_SHT_OK;
}

int magic_sht_launch_count(const magic_sht_handle* h, long long* n) {
  TRY(check_handle(h));
  if (!n) return set_err(MAGIC_SHT_ERR_ARG, "null output");
  *n = h->launches;
  return MAGIC_SHT_OK;
}

// ------------------------------------------------------------ self-test
static int tc_selftest(int device, int n, int kchunks, bool tf32, double* max_rel_err) {
  if (!max_rel_err) return set_err(MAGIC_SHT_ERR_ARG, "null output");
  if (!(n == 32 || n == 64 || n == 128 || n == 256) || kchunks < 1 || kchunks > 2)
    return set_err(MAGIC_SHT_ERR_ARG, "n must be 32/64/128/256 and kchunks 1 or 2");
  if (device < 0) CK(cudaGetDevice(&device));
  DeviceGuard dg(device);
  const int K = (tf32 ? 32 : 64) * kchunks;
  std::vector<float> A((size_t)128 * K), B((size_t)n * K), D((size_t)128 * n);
  unsigned s = 12345u;
  auto rnd = [&]() {  // small integers times powers of two: exact in bf16 and tf32
    s = s * 1664525u + 1013904223u;
    const int v = (int)((s >> 9) % 255) - 127;
    const int e = (int)((s >> 20) % 7) - 3;
    return std::ldexp((float)v, e);
  };
  for (auto& x : A) x = rnd();
  for (auto& x : B) x = rnd();
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* derr = nullptr;
  CK(cudaMalloc((void**)&dA, A.size() * 4));
  CK(cudaMalloc((void**)&dB, B.size() * 4));
  CK(cudaMalloc((void**)&dD, D.size() * 4));
  CK(cudaMalloc((void**)&derr, 4));
  CK(cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemset(dD, 0, D.size() * 4));
  CK(cudaMemset(derr, 0, 4));
  CK(launch_tc_selftest(n, kchunks, tf32, dA, dB, dD, derr, 0));
  CK(cudaDeviceSynchronize());
  int herr = 0;
  CK(cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
  cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(derr);
  if (herr) return set_err(MAGIC_SHT_ERR_TIMEOUT, "tcgen05 self-test: MMA completion wait gave up");
  double worst = 0.0, scale = 0.0;
  for (int i = 0; i < 128; ++i)
    for (int j = 0; j < n; ++j) {
      double ref = 0.0;
      for (int k = 0; k < K; ++k) ref += (double)A[(size_t)i * K + k] * (double)B[(size_t)j * K + k];
      worst = std::fmax(worst, std::fabs(ref - (double)D[(size_t)i * n + j]));
      scale = std::fmax(scale, std::fabs(ref));
    }
  *max_rel_err = worst / (scale > 0 ? scale : 1.0);
  return MAGIC_SHT_OK;
}

int magic_sht_wait_selftest(int device, long long max_cycles, int arrive) {
  if (max_cycles < 1 || max_cycles > (1LL << 31)) return set_err(MAGIC_SHT_ERR_ARG, "max_cycles outside [1, 2^31]");
  int cur = 0;
  CK(cudaGetDevice(&cur));
  if (device >= 0) CK(cudaSetDevice(device));
  int* derr = nullptr;
  CK(cudaMalloc((void**)&derr, 4));
  CK(cudaMemset(derr, 0, 4));
  CK(launch_wait_selftest(max_cycles, arrive, derr, 0));
  CK(cudaDeviceSynchronize());
  int herr = 0;
  CK(cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost));
  cudaFree(derr);
  if (device >= 0) CK(cudaSetDevice(cur));
  if (herr) return set_err(MAGIC_SHT_ERR_TIMEOUT, "bounded device wait gave up after %lld cycles", max_cycles);
  return MAGIC_SHT_OK;
}

int magic_sht_tc_selftest(int device, int n, int kchunks, double* max_rel_err) {
  return tc_selftest(device, n, kchunks, false, max_rel_err);
}

int magic_sht_tc_selftest_tf32(int device, int n, int kchunks, double* max_rel_err) {
  return tc_selftest(device, n, kchunks, true, max_rel_err);
}

// ------------------------------------------------------------ measurement
int magic_sht_measure_gflops(int device, int precision, double* gflops) {
  if (!gflops) return set_err(MAGIC_SHT_ERR_ARG, "null output");
  if (precision != MAGIC_SHT_FP64 && precision != MAGIC_SHT_FP32)
    return set_err(MAGIC_SHT_ERR_ARG, "precision must be MAGIC_SHT_FP64 or MAGIC_SHT_FP32");
  const bool f64 = precision == MAGIC_SHT_FP64;
  if (device < 0) CK(cudaGetDevice(&device));
  DeviceGuard dg(device);
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  const int blocks = prop.multiProcessorCount * 8;
  const int iters = f64 ? 256 : 4096;
  double* d = nullptr;
  CK(cudaMalloc((void**)&d, sizeof(double) * (blocks + 1)));
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int w = 0; w < 2; ++w) CK(launch_fma_peak(d, f64, blocks, iters, st));
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    CK(cudaEventRecord(e0, st));
    CK(launch_fma_peak(d, f64, blocks, iters, st));
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  const double flops = (double)blocks * 256.0 * iters * 16 * 8 * 2;
  *gflops = flops / (best * 1e-3) / 1e9;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  cudaFree(d);
  return MAGIC_SHT_OK;
}

}  // extern "C"

// ============================================== allocation-free scal_to_spat
// A variant of magic_sht_scal_to_spat for callers that must not allocate
// device memory while they run: the (theta, m) half spectrum between the
// Legendre sums and the inverse FFT lives in this file-scope array instead
// of the handle's workspace.  Every GPU that loads the library holds the
// array until the process exits.
#define MAGIC_SHT_NOALLOC_SCRATCH_BYTES (4u << 20)
static __device__ __align__(256) unsigned char g_noalloc_scratch[MAGIC_SHT_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on `dev` (which must be current).  In
// host code the symbol names a host-side stand-in, so the address is looked
// up once per device and cached.
int noalloc_scratch(int dev, void** out) {
  if (dev < 0 || dev >= kMaxDevices) return set_err(MAGIC_SHT_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_err(MAGIC_SHT_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed: %s",
                     cudaGetErrorString(e));
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return MAGIC_SHT_OK;
}
}  // namespace

extern "C" int magic_sht_scal_to_spat_noalloc(magic_sht_handle* h, const double* Slm, double* fieldc,
                                              int lcut) {
  TRY(check_handle(h));
  TRY(check_lcut(h, lcut));
  if (!Slm || !fieldc) return set_err(MAGIC_SHT_ERR_ARG, "null pointer");
  DeviceGuard dg(h->device);
  if (!is_device_ptr(Slm) || !is_device_ptr(fieldc))
    return set_err(MAGIC_SHT_ERR_ARG,
                   "scal_to_spat_noalloc takes device pointers only (host arrays would need staging buffers)");
  if (tf32_form(h))
    return set_err(MAGIC_SHT_ERR_UNSUPPORTED,
                   "scal_to_spat_noalloc: the TF32 form has no allocation-free kernel (its data images need a buffer)");
  const ShtGeom& g = h->g;
  const size_t need = (size_t)g.n_m * g.n_theta * t2_bytes(h);
  if (need > MAGIC_SHT_NOALLOC_SCRATCH_BYTES)
    return set_err(MAGIC_SHT_ERR_SIZE,
                   "half spectrum of %zu bytes (n_m_max=%d x n_theta_max=%d) exceeds the %u-byte static "
                   "scratch of scal_to_spat_noalloc",
                   need, g.n_m, g.n_theta, MAGIC_SHT_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  TRY(noalloc_scratch(h->device, &scratch));
  const long long hs_ld = (long long)g.n_m * g.n_theta;
  InvSet s{};
  s.nf = 1;
  s.nlev = 1;
  s.lcut0 = lcut;
  s.f[0].x0 = SpecOperand{(const double2*)Slm, nullptr, (long long)g.lm_max, OP_COPY, 0};
  s.f[0].x1 = SpecOperand{nullptr, nullptr, 0, OP_ZERO, 0};
  s.f[0].out0 = scratch;
  s.f[0].out1 = nullptr;
  s.f[0].out_ld = hs_ld;
  // the one-tile-per-CTA tensor-core kernel needs no data-image buffer
  {
    PhaseScope ps(h, MAGIC_SHT_PHASE_INV_LEG_SCALAR);
    if (h->precision == MAGIC_SHT_BF16X3) CK(launch_inv_legendre_tc(g, s, false, h->tct, h->stream));
    else CK(launch_inv_legendre_simt(g, s, false, f64_sums(h), h->stream));
  }
  FftSet fs{};
  fs.nf = 1;
  fs.nlev = 1;
  fs.f[0].in = scratch;
  fs.f[0].out = fieldc;
  fs.f[0].in_ld = hs_ld;
  fs.f[0].out_ld = (long long)g.n_phi * g.ld;
  // parity-separated synthesis output of the 3xBF16 one-tile kernel; FP64 half
  // spectra into the double-float FFT of the FP64-accurate form
  fs.f[0].flags = (h->precision == MAGIC_SHT_BF16X3 ? FFT_IN_E : 0) | (oz_form(h) ? FFT_HS_F64 : 0);
  {
    PhaseScope ps(h, MAGIC_SHT_PHASE_FFT_INV);
    CK(launch_fft_inverse(g, fs, fft_arith(h), h->fft_rows, h->stream));
  }
  return MAGIC_SHT_OK;
}
