// Tensor-core (tcgen05) form of the Legendre sums: 3xBF16 split products
// with FP32 accumulation in tensor memory.
//
// This file holds the tcgen05 GEMM self-test used to validate the operand
// layout and descriptor encodings on the device before the split-precision
// Legendre kernels use them.
#include <cuda_bf16.h>
#include <vector>
#include "common.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace {

// D[128][N] = A[128][K] * B[N][K]^T, K = 64*kchunks, one CTA of 4 warps.
template <int N>
__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A,
                                                          const float* __restrict__ B, float* __restrict__ D,
                                                          int kchunks, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;                       // kchunks x [128][64] bf16
  unsigned char* sB = sA + 16384 * kchunks;       // kchunks x [N][64] bf16
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int K = 64 * kchunks;
  constexpr uint32_t NCOL = N < 32 ? 32 : N;
  for (int i = tid; i < 128 * K; i += 128) {
    const int r = i / K, k = i - r * K;
    *(__nv_bfloat16*)(sA + (k >> 6) * 16384 + tc::sw128_offset(r, k & 63)) = __float2bfloat16_rn(A[i]);
  }
  for (int i = tid; i < N * K; i += 128) {
    const int r = i / K, k = i - r * K;
    *(__nv_bfloat16*)(sB + (k >> 6) * (N * 128) + tc::sw128_offset(r, k & 63)) = __float2bfloat16_rn(B[i]);
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, NCOL);
    tc::tmem_relinquish();
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  if (tid == 0) {
    constexpr uint32_t idesc = tc::idesc_bf16(128, N);
    for (int c = 0; c < kchunks; ++c)
      for (int ks = 0; ks < 4; ++ks) {
        const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA + c * 16384) + ks * 32);
        const uint64_t bd = tc::sw128_desc(tc::smem_u32(sB + c * (N * 128)) + ks * 32);
        tc::mma_bf16(tmem, ad, bd, idesc, (c | ks) ? 1u : 0u);
      }
    tc::mma_commit(&bar);
  }
  const bool ok = tc::mbar_wait(&bar, 0);
  if (!ok && lane == 0) atomicExch(err, 1);
  tc::tc_fence_after();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 32; ++i) D[(size_t)(32 * warp + lane) * N + c0 + i] = v[i];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, NCOL);
}

template <int N>
cudaError_t launch_selftest(const float* A, const float* B, float* D, int kchunks, int* err, cudaStream_t st) {
  const size_t smem = 1024 + (size_t)kchunks * (16384 + N * 128);
  CUDA_TRY(cudaFuncSetAttribute(tc_selftest_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tc_selftest_kernel<N><<<1, 128, smem, st>>>(A, B, D, kchunks, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tc_selftest(int n, int kchunks, const float* A, const float* B, float* D, int* err,
                               cudaStream_t st) {
  if (kchunks < 1 || kchunks > 2) return cudaErrorInvalidValue;
  switch (n) {
    case 32: return launch_selftest<32>(A, B, D, kchunks, err, st);
    case 64: return launch_selftest<64>(A, B, D, kchunks, err, st);
    case 128: return launch_selftest<128>(A, B, D, kchunks, err, st);
    case 256: return launch_selftest<256>(A, B, D, kchunks, err, st);
    default: return cudaErrorInvalidValue;
  }
}

// =====================================================================
// Split-precision Legendre sums on the tensor cores.
//
// Synthesis (native_sph_to_spat / native_qst_to_spat / native_sphtor_to_spat,
// src/shtransforms.f90:103-372, :493-646), per order m and parity of l-m:
//   D[theta][col] = sum_l P(l,m,theta) X(l,m)[col]     (M = 128 colatitudes,
//   N = 128 real columns, K = degrees of one parity)
// Analysis (native_spat_to_sph / native_spat_to_sph_tor, :648-872):
//   D[l][col] = sum_theta P(l,m,theta) F(theta,m)[col] (M = 128 degrees of one
//   parity, N = 128 real columns, K = northern colatitudes)
// Both operands are split into three bf16 parts (hi+mid+lo ~ 24 bits); the
// six products with i+j <= 2 are accumulated in fp32 in tensor memory.  The
// table operand is pre-split and pre-tiled (TcTables) and arrives by bulk
// copy; the data operand is split on the fly while staged.
// =====================================================================
namespace {

constexpr int TC_THREADS = 128;
constexpr uint32_t TC_IDESC = tc::idesc_bf16(128, 128);
__constant__ int kSplitPairs[6][2] = {{0, 0}, {0, 1}, {1, 0}, {0, 2}, {1, 1}, {2, 0}};

__device__ __forceinline__ unsigned char* align1024(unsigned char* p) {
  return (unsigned char*)(((uintptr_t)p + 1023) & ~(uintptr_t)1023);
}

__device__ __forceinline__ double2 tc_load_operand(const SpecOperand& o, int r, int lm, int l, int m,
                                                   double or2) {
  if (o.op == OP_ZERO || o.A == nullptr) return make_double2(0.0, 0.0);
  const long long base = (long long)r * o.ld + lm;
  const double2 a = o.A[base];
  switch (o.op) {
    case OP_COPY: return a;
    case OP_DLH: { const double d = (double)(l * (l + 1)); return make_double2(d * a.x, d * a.y); }
    case OP_CURLT: {
      const double2 b = o.B[base];
      const double d = or2 * (double)(l * (l + 1));
      return make_double2(d * a.x - b.x, d * a.y - b.y);
    }
    case OP_IM: { const double dm = (double)m; return make_double2(-dm * a.y, dm * a.x); }
    default: return make_double2(0.0, 0.0);
  }
}

// 8 values -> three 16-byte chunks (hi, mid, lo) at the swizzled position
__device__ __forceinline__ void store_split8(unsigned char* tile0, uint32_t off, const float (&v)[8]) {
  __nv_bfloat16 h[8], md[8], lo[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) tc::split3(v[i], h[i], md[i], lo[i]);
  *(uint4*)(tile0 + off) = *(const uint4*)h;
  *(uint4*)(tile0 + 16384 + off) = *(const uint4*)md;
  *(uint4*)(tile0 + 2 * 16384 + off) = *(const uint4*)lo;
}

__device__ __forceinline__ void tc_record_error(int* err) {
  if (err) atomicExch(err, 1);
}

template <bool VEC>
__global__ void __launch_bounds__(TC_THREADS, 1) inv_leg_tc(const ShtGeom g, const InvSet s, const TcTables t) {
  constexpr int NT = VEC ? 2 : 1;
  constexpr uint32_t TMEM_COLS = VEC ? 512 : 256;
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t barA, barM;
  __shared__ uint32_t tmem_base;
  unsigned char* base = align1024(smem_raw);
  unsigned char* sA = base;                        // [NT][3] x 16 KB
  unsigned char* sB = sA + NT * 3 * 16384;         // [3] x 16 KB
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tt = blockIdx.x, ct = blockIdx.y, mc = blockIdx.z;
  const int m = mc * g.minc;
  const int n_l = g.l_max - m + 1;
  const int lm0 = g.lmoff[mc];
  const int nch = tc_nch(n_l);
  const int npair = s.nf * s.nlev;                 // columns groups (level, field)
  const int ncplx = npair * (VEC ? 2 : 1);         // complex source columns
  if (ct * 64 >= ncplx) return;

  if (tid == 0) {
    tc::mbar_init(&barA, 1);
    tc::mbar_init(&barM, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;

  bool ok = true;
  int stage = 0;
  for (int p = 0; p < 2; ++p) {
    const int nlp = (n_l + 1 - p) / 2;
    const int nchp = (nlp + 63) / 64;
    for (int c = 0; c < nchp; ++c, ++stage) {
      if (stage > 0 && !tc::mbar_wait(&barM, (stage - 1) & 1)) ok = false;
      if (!__syncthreads_and(ok)) { ok = false; break; }
      if (tid == 0) {
        tc::mbar_expect_tx(&barA, NT * 3 * 16384);
        for (int tb = 0; tb < NT; ++tb)
          for (int sp = 0; sp < 3; ++sp) {
            const long long blk = t.inv_blk0[mc] + ((((long long)tt * 2 + tb) * 2 + p) * nch + c) * 3 + sp;
            tc::bulk_g2s(sA + (tb * 3 + sp) * 16384, t.inv_img + blk * 16384, 16384, &barA);
          }
      }
      // data operand: 64 complex columns x 64 degrees of parity p
      for (int u = tid; u < 64 * 8; u += TC_THREADS) {
        const int ql = u >> 3, kg = u & 7;
        const int q = ct * 64 + ql;
        float re[8], im[8];
        if (q < ncplx) {
          const int pair = VEC ? (q >> 1) : q;
          const int r = pair / s.nf, f = pair - r * s.nf;
          const int lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
          const double o2 = s.or2 ? s.or2[r] : s.or2_0;
          const SpecOperand& op = (VEC && (q & 1)) ? s.f[f].x1 : s.f[f].x0;
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int lp = 64 * c + 8 * kg + i;
            const int l = m + p + 2 * lp;
            double2 x = make_double2(0.0, 0.0);
            if (l <= lc) x = tc_load_operand(op, r, lm0 + l - m, l, m, o2);
            re[i] = (float)x.x;
            im[i] = (float)x.y;
          }
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) { re[i] = 0.f; im[i] = 0.f; }
        }
        store_split8(sB, tc::sw128_offset(2 * ql, 8 * kg), re);
        store_split8(sB, tc::sw128_offset(2 * ql + 1, 8 * kg), im);
      }
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        if (!tc::mbar_wait(&barA, stage & 1)) {
          ok = false;
        } else {
          tc::tc_fence_after();
          for (int ks = 0; ks < 4; ++ks)
            for (int tb = 0; tb < NT; ++tb) {
              const uint32_t d = tmem + (uint32_t)((tb * 2 + p) * 128);
              for (int pr = 0; pr < 6; ++pr) {
                const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA + (tb * 3 + kSplitPairs[pr][0]) * 16384) + ks * 32);
                const uint64_t bd = tc::sw128_desc(tc::smem_u32(sB + kSplitPairs[pr][1] * 16384) + ks * 32);
                tc::mma_bf16(d, ad, bd, TC_IDESC, (c | ks | pr) ? 1u : 0u);
              }
            }
        }
        tc::mma_commit(&barM);  // arrives also when nothing was issued
      }
    }
    if (!ok) break;
  }
  if (stage > 0 && !tc::mbar_wait(&barM, (stage - 1) & 1)) ok = false;
  ok = __syncthreads_and(ok);
  tc::tc_fence_after();
  if (!ok) {
    if (tid == 0) tc_record_error(t.err);
  } else {
    const int jl = 32 * warp + lane;
    const int jg = tt * 128 + jl;
    const int NHP = t.ntt * 128;
    const float sP = t.inv_scale[(size_t)mc * NHP + jg];
    const float sdP = VEC ? t.inv_scale[((size_t)g.n_m + mc) * NHP + jg] : 0.f;
    const bool odd_ok = n_l >= 2;
    const uint32_t lane_off = (uint32_t)(32 * warp) << 16;
    const float dm = (float)m;
    for (int cc0 = 0; cc0 < 128; cc0 += 32) {
      float Pe[32], Po[32];
      tc::tmem_ld32(tmem + lane_off + 0 * 128 + cc0, Pe);
      tc::tmem_ld32(tmem + lane_off + 1 * 128 + cc0, Po);
      if (!odd_ok)
#pragma unroll
        for (int i = 0; i < 32; ++i) Po[i] = 0.f;
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int cq = ct * 64 + cc0 / 2 + q;
          if (cq >= ncplx || jg >= g.nh) continue;
          const int r = cq / s.nf, f = cq - r * s.nf;
          const float2 es = make_float2(Pe[2 * q] * sP, Pe[2 * q + 1] * sP);
          const float2 ea = make_float2(Po[2 * q] * sP, Po[2 * q + 1] * sP);
          float2* o = (float2*)s.f[f].out0 + (long long)r * s.f[f].out_ld + (long long)mc * g.n_theta + 2 * jg;
          o[0] = make_float2(es.x + ea.x, es.y + ea.y);
          o[1] = make_float2(es.x - ea.x, es.y - ea.y);
        }
      } else {
        float De[32], Do[32];
        tc::tmem_ld32(tmem + lane_off + 2 * 128 + cc0, De);
        tc::tmem_ld32(tmem + lane_off + 3 * 128 + cc0, Do);
        if (!odd_ok)
#pragma unroll
          for (int i = 0; i < 32; ++i) Do[i] = 0.f;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int pair = ct * 32 + cc0 / 4 + q;
          if (pair >= npair || jg >= g.nh) continue;
          const int r = pair / s.nf, f = pair - r * s.nf;
          // C = sum S P, B = sum T P, A = sum S dP, D = sum T dP (even/odd)
          const float Cer = Pe[4 * q] * sP, Cei = Pe[4 * q + 1] * sP;
          const float Ber = Pe[4 * q + 2] * sP, Bei = Pe[4 * q + 3] * sP;
          const float Cor = Po[4 * q] * sP, Coi = Po[4 * q + 1] * sP;
          const float Bor = Po[4 * q + 2] * sP, Boi = Po[4 * q + 3] * sP;
          const float Aer = De[4 * q] * sdP, Aei = De[4 * q + 1] * sdP;
          const float Der = De[4 * q + 2] * sdP, Dei = De[4 * q + 3] * sdP;
          const float Aor = Do[4 * q] * sdP, Aoi = Do[4 * q + 1] * sdP;
          const float Dor = Do[4 * q + 2] * sdP, Doi = Do[4 * q + 3] * sdP;
          const float bNr = Ber + Bor, bNi = Bei + Boi, bSr = Ber - Bor, bSi = Bei - Boi;
          const float cNr = Cer + Cor, cNi = Cei + Coi, cSr = Cer - Cor, cSi = Cei - Coi;
          const float2 vtN = make_float2(Aer + Aor - dm * bNi, Aei + Aoi + dm * bNr);
          const float2 vtS = make_float2(Aor - Aer - dm * bSi, Aoi - Aei + dm * bSr);
          const float2 vpN = make_float2(-dm * cNi - (Der + Dor), dm * cNr - (Dei + Doi));
          const float2 vpS = make_float2(-dm * cSi + (Der - Dor), dm * cSr + (Dei - Doi));
          const long long o = (long long)r * s.f[f].out_ld + (long long)mc * g.n_theta + 2 * jg;
          float2* o0 = (float2*)s.f[f].out0 + o;
          float2* o1 = (float2*)s.f[f].out1 + o;
          o0[0] = vtN; o0[1] = vtS;
          o1[0] = vpN; o1[1] = vpS;
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

template <bool VEC>
__global__ void __launch_bounds__(TC_THREADS, 1) fwd_leg_tc(const ShtGeom g, const FwdSet s, const TcTables t) {
  constexpr int NT = VEC ? 2 : 1;
  constexpr uint32_t TMEM_COLS = VEC ? 256 : 128;
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t barA, barM;
  __shared__ uint32_t tmem_base;
  unsigned char* base = align1024(smem_raw);
  unsigned char* sA = base;                      // [NT][3] x 16 KB
  unsigned char* sB = sA + NT * 3 * 16384;       // [NT][3] x 16 KB (mine, other)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ct = blockIdx.x, lt = blockIdx.y;
  const int mc = blockIdx.z >> 1, p = blockIdx.z & 1;
  const int m = mc * g.minc;
  const int n_l = g.l_max - m + 1;
  const int nlp = (n_l + 1 - p) / 2;
  const int lm0 = g.lmoff[mc];
  const int npair = s.nf * s.nlev;
  const int ncplx = npair * (VEC ? 2 : 1);
  if (lt * 128 >= nlp || ct * 64 >= ncplx) return;

  if (tid == 0) {
    tc::mbar_init(&barA, 1);
    tc::mbar_init(&barM, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  const int mine = p, other = p ^ 1;  // 0 = ES, 1 = EA

  bool ok = true;
  int stage = 0;
  for (int c = 0; c < t.ncj; ++c, ++stage) {
    if (stage > 0 && !tc::mbar_wait(&barM, (stage - 1) & 1)) ok = false;
    if (!__syncthreads_and(ok)) { ok = false; break; }
    if (tid == 0) {
      tc::mbar_expect_tx(&barA, NT * 3 * 16384);
      for (int tb = 0; tb < NT; ++tb)
        for (int sp = 0; sp < 3; ++sp) {
          const long long blk =
              t.fwd_blk0[mc] + ((((long long)p * t.nlt + lt) * 2 + tb) * t.ncj + c) * 3 + sp;
          tc::bulk_g2s(sA + (tb * 3 + sp) * 16384, t.fwd_img + blk * 16384, 16384, &barA);
        }
    }
    for (int u = tid; u < 64 * 8; u += TC_THREADS) {
      const int ql = u >> 3, kg = u & 7;
      const int q = ct * 64 + ql;
      float mr[8], mi[8], orr[8], oi[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) { mr[i] = mi[i] = orr[i] = oi[i] = 0.f; }
      if (q < ncplx) {
        const int pair = VEC ? (q >> 1) : q;
        const int r = pair / s.nf, f = pair - r * s.nf;
        const float2* src = (const float2*)((VEC && (q & 1)) ? s.f[f].in1 : s.f[f].in0) +
                            (long long)r * s.f[f].in_ld + (long long)mc * g.nh * 2;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int j = 64 * c + 8 * kg + i;
          if (j < g.nh) {
            const float4 v = *(const float4*)(src + 2 * j);  // (ES, EA) of colatitude j
            const float2 es = make_float2(v.x, v.y), ea = make_float2(v.z, v.w);
            const float2 a = mine ? ea : es, b = mine ? es : ea;
            mr[i] = a.x; mi[i] = a.y; orr[i] = b.x; oi[i] = b.y;
          }
        }
      }
      store_split8(sB, tc::sw128_offset(2 * ql, 8 * kg), mr);
      store_split8(sB, tc::sw128_offset(2 * ql + 1, 8 * kg), mi);
      if (VEC) {
        store_split8(sB + 3 * 16384, tc::sw128_offset(2 * ql, 8 * kg), orr);
        store_split8(sB + 3 * 16384, tc::sw128_offset(2 * ql + 1, 8 * kg), oi);
      }
    }
    (void)other;
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      if (!tc::mbar_wait(&barA, stage & 1)) {
        ok = false;
      } else {
        tc::tc_fence_after();
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {
            // P x mine -> D0,  dP x other -> D1
            const uint32_t d = tmem + (uint32_t)(tb * 128);
            for (int pr = 0; pr < 6; ++pr) {
              const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA + (tb * 3 + kSplitPairs[pr][0]) * 16384) + ks * 32);
              const uint64_t bd =
                  tc::sw128_desc(tc::smem_u32(sB + (tb * 3 + kSplitPairs[pr][1]) * 16384) + ks * 32);
              tc::mma_bf16(d, ad, bd, TC_IDESC, (c | ks | pr) ? 1u : 0u);
            }
          }
      }
      tc::mma_commit(&barM);
    }
  }
  if (stage > 0 && !tc::mbar_wait(&barM, (stage - 1) & 1)) ok = false;
  ok = __syncthreads_and(ok);
  tc::tc_fence_after();
  if (!ok) {
    if (tid == 0) tc_record_error(t.err);
  } else {
    const int lr = 32 * warp + lane;
    const int lp = lt * 128 + lr;
    const int l = m + p + 2 * lp;
    const bool valid = lp < nlp;
    const int lm = lm0 + l - m;
    const float sP = valid ? t.fwd_scale[lm] : 0.f;
    const float sdP = (VEC && valid) ? t.fwd_scale[(size_t)g.lm_max + lm] : 0.f;
    const uint32_t lane_off = (uint32_t)(32 * warp) << 16;
    const double dm = (double)m;
    const double inv_ll = l > 0 ? 1.0 / (double)(l * (l + 1)) : 1.0;
    for (int cc0 = 0; cc0 < 128; cc0 += 32) {
      float D0[32];
      tc::tmem_ld32(tmem + lane_off + cc0, D0);
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int cq = ct * 64 + cc0 / 2 + q;
          if (cq >= ncplx || !valid) continue;
          const int r = cq / s.nf, f = cq - r * s.nf;
          const int lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
          const double2 v = (l <= lc) ? make_double2((double)(D0[2 * q] * sP), (double)(D0[2 * q + 1] * sP))
                                      : make_double2(0.0, 0.0);
          s.f[f].out0[(long long)r * s.f[f].out_ld + lm] = v;
        }
      } else {
        float D1[32];
        tc::tmem_ld32(tmem + lane_off + 128 + cc0, D1);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int pair = ct * 32 + cc0 / 4 + q;
          if (pair >= npair || !valid) continue;
          const int r = pair / s.nf, f = pair - r * s.nf;
          const int lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
          // A = sum F1_mine P, D = sum F2_mine P, C = sum F1_other dP, B = sum F2_other dP
          const double Ar = D0[4 * q] * sP, Ai = D0[4 * q + 1] * sP;
          const double Dr = D0[4 * q + 2] * sP, Di = D0[4 * q + 3] * sP;
          const double Cr = D1[4 * q] * sdP, Ci = D1[4 * q + 1] * sdP;
          const double Br = D1[4 * q + 2] * sdP, Bi = D1[4 * q + 3] * sdP;
          double2 Sv = make_double2((dm * Ai + Br) * inv_ll, (-dm * Ar + Bi) * inv_ll);
          double2 Tv = make_double2((-Cr + dm * Di) * inv_ll, (-Ci - dm * Dr) * inv_ll);
          if (l > lc) { Sv = make_double2(0.0, 0.0); Tv = Sv; }
          const long long o = (long long)r * s.f[f].out_ld + lm;
          s.f[f].out0[o] = Sv;
          s.f[f].out1[o] = Tv;
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// ------------------------------------------------------- table images
__global__ void build_inv_img_kernel(const ShtGeom g, TcTables t, unsigned char* img, float* scale) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int NHP = t.ntt * 128;
  if (idx >= (long long)g.n_m * 2 * NHP) return;
  const int j = (int)(idx % NHP);
  const int tb = (int)((idx / NHP) % 2);
  const int mc = (int)(idx / (2LL * NHP));
  const int m = mc * g.minc, n_l = g.l_max - m + 1, lm0 = g.lmoff[mc];
  const double* tab = tb ? g.dP64 : g.P64;
  const bool valid = j < g.nh;
  double mx = 0.0;
  if (valid)
    for (int l = 0; l < n_l; ++l) mx = fmax(mx, fabs(tab[(size_t)(lm0 + l) * g.nh + j]));
  // Rows whose largest |P| is below 1e-250 contribute nothing at FP32
  // precision; they are stored as zeros (their 2^-e factor would overflow).
  int e = 0;
  const bool live = mx > 1e-250;
  if (live) frexp(mx, &e);
  scale[((size_t)tb * g.n_m + mc) * NHP + j] = live ? ldexpf(1.0f, e) : 0.0f;
  const double inv = live ? ldexp(1.0, -e) : 0.0;
  const int nch = tc_nch(n_l);
  const int tt = j / 128, row = j % 128;
  for (int p = 0; p < 2; ++p)
    for (int lp = 0; lp < nch * 64; ++lp) {
      const int loff = p + 2 * lp;
      const double v = (valid && loff < n_l) ? tab[(size_t)(lm0 + loff) * g.nh + j] * inv : 0.0;
      __nv_bfloat16 h[3];
      tc::split3((float)v, h[0], h[1], h[2]);
      for (int sp = 0; sp < 3; ++sp) {
        const long long blk = t.inv_blk0[mc] + ((((long long)tt * 2 + tb) * 2 + p) * nch + lp / 64) * 3 + sp;
        *(__nv_bfloat16*)(img + blk * 16384 + tc::sw128_offset(row, lp % 64)) = h[sp];
      }
    }
}

__global__ void build_fwd_img_kernel(const ShtGeom g, TcTables t, unsigned char* img, float* scale) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int NLP = t.nlt * 128;
  if (idx >= (long long)g.n_m * 2 * 2 * NLP) return;
  const int lpad = (int)(idx % NLP);
  const int p = (int)((idx / NLP) % 2);
  const int tb = (int)((idx / (2LL * NLP)) % 2);
  const int mc = (int)(idx / (4LL * NLP));
  const int m = mc * g.minc, n_l = g.l_max - m + 1, lm0 = g.lmoff[mc];
  const double* tab = tb ? g.dP64 : g.P64;
  const int loff = p + 2 * lpad;
  const bool valid = loff < n_l;
  double mx = 0.0;
  if (valid)
    for (int j = 0; j < g.nh; ++j) mx = fmax(mx, fabs(tab[(size_t)(lm0 + loff) * g.nh + j]));
  int e = 0;
  const bool live = mx > 1e-250;
  if (live) frexp(mx, &e);
  if (valid) scale[(size_t)tb * g.lm_max + lm0 + loff] = live ? ldexpf(1.0f, e) : 0.0f;
  const double inv = live ? ldexp(1.0, -e) : 0.0;
  const int lt = lpad / 128, row = lpad % 128;
  for (int j = 0; j < t.ncj * 64; ++j) {
    const double v = (valid && j < g.nh) ? tab[(size_t)(lm0 + loff) * g.nh + j] * inv : 0.0;
    __nv_bfloat16 h[3];
    tc::split3((float)v, h[0], h[1], h[2]);
    for (int sp = 0; sp < 3; ++sp) {
      const long long blk = t.fwd_blk0[mc] + ((((long long)p * t.nlt + lt) * 2 + tb) * t.ncj + j / 64) * 3 + sp;
      *(__nv_bfloat16*)(img + blk * 16384 + tc::sw128_offset(row, j % 64)) = h[sp];
    }
  }
}

template <bool VEC>
cudaError_t launch_inv_tc_t(const ShtGeom& g, const InvSet& s, const TcTables& t, cudaStream_t st) {
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  if (ncplx <= 0) return cudaSuccess;
  const size_t smem = 1024 + (size_t)((VEC ? 2 : 1) * 3 + 3) * 16384;
  CUDA_TRY(cudaFuncSetAttribute(inv_leg_tc<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(t.ntt, (ncplx + 63) / 64, g.n_m);
  inv_leg_tc<VEC><<<grid, TC_THREADS, smem, st>>>(g, s, t);
  return cudaGetLastError();
}

template <bool VEC>
cudaError_t launch_fwd_tc_t(const ShtGeom& g, const FwdSet& s, const TcTables& t, cudaStream_t st) {
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  if (ncplx <= 0) return cudaSuccess;
  const size_t smem = 1024 + (size_t)((VEC ? 2 : 1) * 6) * 16384;
  CUDA_TRY(cudaFuncSetAttribute(fwd_leg_tc<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((ncplx + 63) / 64, t.nlt, g.n_m * 2);
  fwd_leg_tc<VEC><<<grid, TC_THREADS, smem, st>>>(g, s, t);
  return cudaGetLastError();
}

}  // namespace

void tc_table_layout(const ShtGeom& g, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
                     std::vector<long long>& fwd_blk0, long long* inv_blocks, long long* fwd_blocks) {
  *ntt = (g.nh + 127) / 128;
  *nlt = ((g.l_max + 2) / 2 + 127) / 128;
  *ncj = (g.nh + 63) / 64;
  inv_blk0.resize(g.n_m);
  fwd_blk0.resize(g.n_m);
  long long bi = 0, bf = 0;
  for (int mc = 0; mc < g.n_m; ++mc) {
    const int n_l = g.l_max - mc * g.minc + 1;
    inv_blk0[mc] = bi;
    bi += (long long)(*ntt) * 2 * 2 * tc_nch(n_l) * 3;
    fwd_blk0[mc] = bf;
    bf += 2LL * (*nlt) * 2 * (*ncj) * 3;
  }
  *inv_blocks = bi;
  *fwd_blocks = bf;
}

cudaError_t build_tc_images(const ShtGeom& g, const TcTables& t, unsigned char* inv_img, float* inv_scale,
                            unsigned char* fwd_img, float* fwd_scale, cudaStream_t st) {
  {
    const long long n = (long long)g.n_m * 2 * t.ntt * 128;
    build_inv_img_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(g, t, inv_img, inv_scale);
    CUDA_TRY(cudaGetLastError());
  }
  {
    const long long n = (long long)g.n_m * 4 * t.nlt * 128;
    build_fwd_img_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(g, t, fwd_img, fwd_scale);
    CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

cudaError_t launch_inv_legendre_tc(const ShtGeom& g, const InvSet& s, bool vec, const TcTables& t,
                                   cudaStream_t st) {
  return vec ? launch_inv_tc_t<true>(g, s, t, st) : launch_inv_tc_t<false>(g, s, t, st);
}

cudaError_t launch_fwd_legendre_tc(const ShtGeom& g, const FwdSet& s, bool vec, const TcTables& t,
                                   cudaStream_t st) {
  return vec ? launch_fwd_tc_t<true>(g, s, t, st) : launch_fwd_tc_t<false>(g, s, t, st);
}
