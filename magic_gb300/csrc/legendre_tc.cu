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
#include "cplx.cuh"
#include "tc_build.cuh"

namespace {

// D[128][N] = A[128][K] * B[N][K]^T, K = 64*kchunks, one CTA of 4 warps.
// TF32 = false: bf16 operands, K tiles of 64 (kind::f16, K = 16 per MMA);
// true: tf32 operands, K tiles of 32 (kind::tf32, K = 8 per MMA).
template <int N, bool TF32>
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
  constexpr int KW = TF32 ? 32 : 64;  // K per 128-byte tile row
  const int K = KW * kchunks;
  constexpr uint32_t NCOL = N < 32 ? 32 : N;
  for (int i = tid; i < 128 * K; i += 128) {
    const int r = i / K, k = i - r * K;
    if (TF32) *(float*)(sA + (k / KW) * 16384 + tc::sw128_offset32(r, k % KW)) = A[i];
    else *(__nv_bfloat16*)(sA + (k / KW) * 16384 + tc::sw128_offset(r, k % KW)) = __float2bfloat16_rn(A[i]);
  }
  for (int i = tid; i < N * K; i += 128) {
    const int r = i / K, k = i - r * K;
    if (TF32) *(float*)(sB + (k / KW) * (N * 128) + tc::sw128_offset32(r, k % KW)) = B[i];
    else *(__nv_bfloat16*)(sB + (k / KW) * (N * 128) + tc::sw128_offset(r, k % KW)) = __float2bfloat16_rn(B[i]);
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
    constexpr uint32_t idesc = TF32 ? tc::idesc_tf32(128, N) : tc::idesc_bf16(128, N);
    for (int c = 0; c < kchunks; ++c)
      for (int ks = 0; ks < 4; ++ks) {  // 32 bytes of K per MMA in both formats
        const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA + c * 16384) + ks * 32);
        const uint64_t bd = tc::sw128_desc(tc::smem_u32(sB + c * (N * 128)) + ks * 32);
        if (TF32) tc::mma_tf32(tmem, ad, bd, idesc, (c | ks) ? 1u : 0u);
        else tc::mma_bf16(tmem, ad, bd, idesc, (c | ks) ? 1u : 0u);
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
cudaError_t launch_selftest(const float* A, const float* B, float* D, int kchunks, bool tf32, int* err,
                            cudaStream_t st) {
  const size_t smem = 1024 + (size_t)kchunks * (16384 + N * 128);
  if (tf32) {
    CUDA_TRY(cudaFuncSetAttribute(tc_selftest_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tc_selftest_kernel<N, true><<<1, 128, smem, st>>>(A, B, D, kchunks, err);
  } else {
    CUDA_TRY(cudaFuncSetAttribute(tc_selftest_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tc_selftest_kernel<N, false><<<1, 128, smem, st>>>(A, B, D, kchunks, err);
  }
  return cudaGetLastError();
}

}  // namespace

// Failure-detection check of the bounded waits: one thread waits on an
// mbarrier that is (arrive != 0) or is not (arrive == 0) completed; a wait that
// gives up after max_cycles sets *err and the kernel returns normally.
__global__ void wait_selftest_kernel(long long max_cycles, int arrive, int* err) {
  __shared__ uint64_t bar;
  tc::mbar_init(&bar, 1);
  tc::fence_mbar_init();
  if (arrive) tc::mbar_arrive(&bar);
  if (!tc::mbar_wait(&bar, 0, max_cycles)) *err = 1;
}

cudaError_t launch_wait_selftest(long long max_cycles, int arrive, int* err, cudaStream_t st) {
  wait_selftest_kernel<<<1, 1, 0, st>>>(max_cycles, arrive, err);
  return cudaGetLastError();
}

cudaError_t launch_tc_selftest(int n, int kchunks, bool tf32, const float* A, const float* B, float* D, int* err,
                               cudaStream_t st) {
  if (kchunks < 1 || kchunks > 2) return cudaErrorInvalidValue;
  switch (n) {
    case 32: return launch_selftest<32>(A, B, D, kchunks, tf32, err, st);
    case 64: return launch_selftest<64>(A, B, D, kchunks, tf32, err, st);
    case 128: return launch_selftest<128>(A, B, D, kchunks, tf32, err, st);
    case 256: return launch_selftest<256>(A, B, D, kchunks, tf32, err, st);
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

__device__ __forceinline__ unsigned char* align1024(unsigned char* p) {
  return (unsigned char*)(((uintptr_t)p + 1023) & ~(uintptr_t)1023);
}

__device__ __forceinline__ void tc_record_error(int* err) {
  if (err) atomicExch(err, 1);
}

// Synthesis, one (m, parity, theta tile, column tile) per CTA.  The CTA
// writes, for each output field, E_p = U + W and F_p = U - W where U holds the
// P-terms and W the dP-terms of its parity (scalar fields: E_p only); the
// inverse FFT forms the north/south rows N = E_0 + E_1, S = F_0 - F_1
// (P is even and sin(theta) dP/dtheta odd under theta -> pi - theta for
// even l-m).  Accumulators: hi*hi and the five cross products apart, so the
// large partial sums take one rounding per k-step.
template <bool VEC>
__global__ void __launch_bounds__(TC_THREADS, 2) inv_leg_tc(const ShtGeom g, const InvSet s, const TcTables t) {
  constexpr int NT = VEC ? 2 : 1;
  constexpr int NC = 64;                       // real columns per CTA
  constexpr int BT = NC * 128;                 // bytes of one B split tile
  constexpr uint32_t TMEM_COLS = NT * 2 * NC;  // (table) x (hi, cross)
  constexpr uint32_t IDESC = tc::idesc_bf16(128, NC);
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t barA0, barA1, barF0, barM;
  __shared__ uint32_t tmem_base;
  unsigned char* base = align1024(smem_raw);
  unsigned char* sA0 = base;                   // slot 0: NT x 16 KB
  unsigned char* sA1 = sA0 + NT * 16384;       // slot 1
  unsigned char* sB = sA1 + NT * 16384;        // 3 x BT
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tt = blockIdx.x, ct = blockIdx.y;
  const int mc = blockIdx.z >> 1, p = blockIdx.z & 1;
  const int m = mc * g.minc;
  const int n_l = g.l_max - m + 1;
  const int lm0 = g.lmoff[mc];
  const int nch = tc_nch(n_l);
  const int nlp = (n_l + 1 - p) / 2;
  const int nchp = (nlp + 63) / 64;
  const int npair = s.nf * s.nlev;
  const int ncplx = npair * (VEC ? 2 : 1);
  if (ct * (NC / 2) >= ncplx) return;
  const int jl = 32 * warp + lane;
  const int jg = tt * 128 + jl;
  // output element (field f, level r, parity p, E/F) of this thread's colatitude
  auto out_ptr = [&](void* base_ptr, int r, int f, int ef) -> float2* {
    const long long per_p = VEC ? 2LL * g.nh : (long long)g.nh;
    return (float2*)base_ptr + (long long)r * s.f[f].out_ld + ((long long)mc * 2 + p) * per_p +
           (long long)ef * g.nh + jg;
  };
  if (nlp == 0) {  // m = l_max, odd parity: nothing to sum, contribute zeros
    if (jg < g.nh)
      for (int q = 0; q < NC / 2; ++q) {
        const int cq = ct * (NC / 2) + q;
        if (cq >= ncplx) break;
        if (!VEC) {
          const int r = cq / s.nf, f = cq - r * s.nf;
          *out_ptr(s.f[f].out0, r, f, 0) = make_float2(0.f, 0.f);
        } else if ((cq & 1) == 0) {
          const int pair = cq >> 1, r = pair / s.nf, f = pair - r * s.nf;
          for (int ef = 0; ef < 2; ++ef) {
            *out_ptr(s.f[f].out0, r, f, ef) = make_float2(0.f, 0.f);
            *out_ptr(s.f[f].out1, r, f, ef) = make_float2(0.f, 0.f);
          }
        }
      }
    return;
  }

  if (tid == 0) {
    tc::mbar_init(&barA0, 1);
    tc::mbar_init(&barA1, 1);
    tc::mbar_init(&barF0, 1);
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
  uint32_t ph_a0 = 0, ph_a1 = 0, ph_f0 = 0;
  bool ok = true;
  auto issue_split = [&](int c, int sp, unsigned char* slot, uint64_t* bar) {
    tc::mbar_expect_tx(bar, NT * 16384);
    for (int tb = 0; tb < NT; ++tb) {
      const long long blk = t.inv_blk0[mc] + ((((long long)tt * 2 + tb) * 2 + p) * nch + c) * 3 + sp;
      tc::bulk_g2s(slot + tb * 16384, t.inv_img + blk * 16384, 16384, bar);
    }
  };
  for (int c = 0; c < nchp; ++c) {
    if (c > 0 && !tc::mbar_wait(&barM, (c - 1) & 1)) ok = false;
    if (!__syncthreads_and(ok)) { ok = false; break; }
    if (tid == 0) {
      issue_split(c, 0, sA0, &barA0);
      issue_split(c, 1, sA1, &barA1);
    }
    // data operand: 32 complex columns x 64 degrees of parity p
    inv_build_tile<VEC, NC, 4>(g, s, sB, ct, ncplx, m, lm0, p, c, warp, TC_THREADS / 32, lane);
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      bool good = tc::mbar_wait(&barA0, ph_a0);
      ph_a0 ^= 1;
      tc::tc_fence_after();
      if (good) {
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {
            const uint32_t hi = tmem + (uint32_t)((tb * 2 + 0) * NC), cr = tmem + (uint32_t)((tb * 2 + 1) * NC);
            const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA0 + tb * 16384) + ks * 32);
            const uint32_t first = (c | ks) ? 1u : 0u;
            tc::mma_bf16(hi, ad, tc::sw128_desc(tc::smem_u32(sB) + ks * 32), IDESC, first);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(sB + BT) + ks * 32), IDESC, first);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(sB + 2 * BT) + ks * 32), IDESC, 1u);
          }
      }
      tc::mma_commit(&barF0);
      good = good && tc::mbar_wait(&barA1, ph_a1);
      ph_a1 ^= 1;
      tc::tc_fence_after();
      if (good) {
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {
            const uint32_t cr = tmem + (uint32_t)((tb * 2 + 1) * NC);
            const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA1 + tb * 16384) + ks * 32);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(sB) + ks * 32), IDESC, 1u);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(sB + BT) + ks * 32), IDESC, 1u);
          }
      }
      good = good && tc::mbar_wait(&barF0, ph_f0);  // slot 0 free again
      ph_f0 ^= 1;
      if (good) issue_split(c, 2, sA0, &barA0);
      good = good && tc::mbar_wait(&barA0, ph_a0);
      ph_a0 ^= 1;
      tc::tc_fence_after();
      if (good) {
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {
            const uint32_t cr = tmem + (uint32_t)((tb * 2 + 1) * NC);
            const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA0 + tb * 16384) + ks * 32);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(sB) + ks * 32), IDESC, 1u);
          }
      }
      if (!good) ok = false;
      tc::mma_commit(&barM);
    }
  }
  if (nchp > 0 && !tc::mbar_wait(&barM, (nchp - 1) & 1)) ok = false;
  ok = __syncthreads_and(ok);
  tc::tc_fence_after();
  if (!ok) {
    if (tid == 0) tc_record_error(t.err);
  } else {
    const int NHP = t.ntt * 128;
    const float sP = t.inv_scale[(size_t)mc * NHP + jg];
    const float sdP = VEC ? t.inv_scale[((size_t)g.n_m + mc) * NHP + jg] : 0.f;
    const uint32_t lane_off = (uint32_t)(32 * warp) << 16;
    const float dm = (float)m;
    for (int cc0 = 0; cc0 < NC; cc0 += 32) {
      float P[32], X[32];
      tc::tmem_ld32(tmem + lane_off + 0 * NC + cc0, P);
      tc::tmem_ld32(tmem + lane_off + 1 * NC + cc0, X);
#pragma unroll
      for (int i = 0; i < 32; ++i) P[i] = (P[i] + X[i]) * sP;
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int cq = ct * (NC / 2) + cc0 / 2 + q;
          if (cq >= ncplx || jg >= g.nh) continue;
          const int r = cq / s.nf, f = cq - r * s.nf;
          *out_ptr(s.f[f].out0, r, f, 0) = make_float2(P[2 * q], P[2 * q + 1]);
        }
      } else {
        float D[32];
        tc::tmem_ld32(tmem + lane_off + 2 * NC + cc0, D);
        tc::tmem_ld32(tmem + lane_off + 3 * NC + cc0, X);
#pragma unroll
        for (int i = 0; i < 32; ++i) D[i] = (D[i] + X[i]) * sdP;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int pair = ct * (NC / 4) + cc0 / 4 + q;
          if (pair >= npair || jg >= g.nh) continue;
          const int r = pair / s.nf, f = pair - r * s.nf;
          // C = sum S P, B = sum T P (columns S, T of the pair against P);
          // A = sum S dP, D = sum T dP (against dP)
          const float Cr = P[4 * q], Ci = P[4 * q + 1], Br = P[4 * q + 2], Bi = P[4 * q + 3];
          const float Ar = D[4 * q], Ai = D[4 * q + 1], Dr = D[4 * q + 2], Di = D[4 * q + 3];
          // v_theta: U = i m B, W = A;   v_phi: U = i m C, W = -D
          const float2 Ut = make_float2(-dm * Bi, dm * Br), Wt = make_float2(Ar, Ai);
          const float2 Up = make_float2(-dm * Ci, dm * Cr), Wp = make_float2(-Dr, -Di);
          *out_ptr(s.f[f].out0, r, f, 0) = make_float2(Ut.x + Wt.x, Ut.y + Wt.y);
          *out_ptr(s.f[f].out0, r, f, 1) = make_float2(Ut.x - Wt.x, Ut.y - Wt.y);
          *out_ptr(s.f[f].out1, r, f, 0) = make_float2(Up.x + Wp.x, Up.y + Wp.y);
          *out_ptr(s.f[f].out1, r, f, 1) = make_float2(Up.x - Wp.x, Up.y - Wp.y);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// Analysis, one (m, parity, l' tile, column tile) per CTA.  P x (ES or EA of
// the same parity) and, for vector fields, dP x (the other one); hi*hi and
// cross products in separate accumulators; table splits through a 2-slot
// ring as in the synthesis.
template <bool VEC>
__global__ void __launch_bounds__(TC_THREADS, 2) fwd_leg_tc(const ShtGeom g, const FwdSet s, const TcTables t) {
  constexpr int NT = VEC ? 2 : 1;
  constexpr int NC = VEC ? 64 : 128;
  constexpr int BT = NC * 128;
  constexpr uint32_t TMEM_COLS = NT * 2 * NC;  // 256
  constexpr uint32_t IDESC = tc::idesc_bf16(128, NC);
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t barA0, barA1, barF0, barM;
  __shared__ uint32_t tmem_base;
  unsigned char* base = align1024(smem_raw);
  unsigned char* sA0 = base;
  unsigned char* sA1 = sA0 + NT * 16384;
  unsigned char* sB = sA1 + NT * 16384;        // [NT][3] x BT (mine, other)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ct = blockIdx.x, lt = blockIdx.y;
  const int mc = blockIdx.z >> 1, p = blockIdx.z & 1;
  const int m = mc * g.minc;
  const int n_l = g.l_max - m + 1;
  const int nlp = (n_l + 1 - p) / 2;
  const int lm0 = g.lmoff[mc];
  const int npair = s.nf * s.nlev;
  const int ncplx = npair * (VEC ? 2 : 1);
  if (lt * 128 >= nlp || ct * (NC / 2) >= ncplx) return;

  if (tid == 0) {
    tc::mbar_init(&barA0, 1);
    tc::mbar_init(&barA1, 1);
    tc::mbar_init(&barF0, 1);
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
  const int mine = p;  // 0 = ES, 1 = EA
  uint32_t ph_a0 = 0, ph_a1 = 0, ph_f0 = 0;
  bool ok = true;
  auto issue_split = [&](int c, int sp, unsigned char* slot, uint64_t* bar) {
    tc::mbar_expect_tx(bar, NT * 16384);
    for (int tb = 0; tb < NT; ++tb) {
      const long long blk = t.fwd_blk0[mc] + ((((long long)p * t.nlt + lt) * 2 + tb) * t.ncj + c) * 3 + sp;
      tc::bulk_g2s(slot + tb * 16384, t.fwd_img + blk * 16384, 16384, bar);
    }
  };
  for (int c = 0; c < t.ncj; ++c) {
    if (c > 0 && !tc::mbar_wait(&barM, (c - 1) & 1)) ok = false;
    if (!__syncthreads_and(ok)) { ok = false; break; }
    if (tid == 0) {
      issue_split(c, 0, sA0, &barA0);
      issue_split(c, 1, sA1, &barA1);
    }
    fwd_build_tile<VEC, NC, 4>(g, s, sB, ct, ncplx, mc, mine, c, warp, TC_THREADS / 32, lane);
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      bool good = tc::mbar_wait(&barA0, ph_a0);
      ph_a0 ^= 1;
      tc::tc_fence_after();
      if (good) {
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {  // tb 0: P x mine, tb 1: dP x other
            const uint32_t hi = tmem + (uint32_t)((tb * 2 + 0) * NC), cr = tmem + (uint32_t)((tb * 2 + 1) * NC);
            const unsigned char* b = sB + tb * 3 * BT;
            const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA0 + tb * 16384) + ks * 32);
            const uint32_t first = (c | ks) ? 1u : 0u;
            tc::mma_bf16(hi, ad, tc::sw128_desc(tc::smem_u32(b) + ks * 32), IDESC, first);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(b + BT) + ks * 32), IDESC, first);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(b + 2 * BT) + ks * 32), IDESC, 1u);
          }
      }
      tc::mma_commit(&barF0);
      good = good && tc::mbar_wait(&barA1, ph_a1);
      ph_a1 ^= 1;
      tc::tc_fence_after();
      if (good) {
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {
            const uint32_t cr = tmem + (uint32_t)((tb * 2 + 1) * NC);
            const unsigned char* b = sB + tb * 3 * BT;
            const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA1 + tb * 16384) + ks * 32);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(b) + ks * 32), IDESC, 1u);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(b + BT) + ks * 32), IDESC, 1u);
          }
      }
      good = good && tc::mbar_wait(&barF0, ph_f0);
      ph_f0 ^= 1;
      if (good) issue_split(c, 2, sA0, &barA0);
      good = good && tc::mbar_wait(&barA0, ph_a0);
      ph_a0 ^= 1;
      tc::tc_fence_after();
      if (good) {
        for (int ks = 0; ks < 4; ++ks)
          for (int tb = 0; tb < NT; ++tb) {
            const uint32_t cr = tmem + (uint32_t)((tb * 2 + 1) * NC);
            const unsigned char* b = sB + tb * 3 * BT;
            const uint64_t ad = tc::sw128_desc(tc::smem_u32(sA0 + tb * 16384) + ks * 32);
            tc::mma_bf16(cr, ad, tc::sw128_desc(tc::smem_u32(b) + ks * 32), IDESC, 1u);
          }
      }
      if (!good) ok = false;
      tc::mma_commit(&barM);
    }
  }
  if (t.ncj > 0 && !tc::mbar_wait(&barM, (t.ncj - 1) & 1)) ok = false;
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
    const float dm = (float)m;
    const float inv_ll = l > 0 ? 1.0f / (float)(l * (l + 1)) : 1.0f;
    for (int cc0 = 0; cc0 < NC; cc0 += 32) {
      float D0[32], X[32];
      tc::tmem_ld32(tmem + lane_off + 0 * NC + cc0, D0);
      tc::tmem_ld32(tmem + lane_off + 1 * NC + cc0, X);
#pragma unroll
      for (int i = 0; i < 32; ++i) D0[i] = (D0[i] + X[i]) * sP;
      if (!VEC) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int cq = ct * (NC / 2) + cc0 / 2 + q;
          if (cq >= ncplx || !valid) continue;
          const int r = cq / s.nf, f = cq - r * s.nf;
          const int lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
          const double2 v = (l <= lc) ? make_double2(f2d_int(D0[2 * q]), f2d_int(D0[2 * q + 1]))
                                      : make_double2(0.0, 0.0);
          s.f[f].out0[(long long)r * s.f[f].out_ld + lm] = v;
        }
      } else {
        float D1[32];
        tc::tmem_ld32(tmem + lane_off + 2 * NC + cc0, D1);
        tc::tmem_ld32(tmem + lane_off + 3 * NC + cc0, X);
#pragma unroll
        for (int i = 0; i < 32; ++i) D1[i] = (D1[i] + X[i]) * sdP;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int pair = ct * (NC / 4) + cc0 / 4 + q;
          if (pair >= npair || !valid) continue;
          const int r = pair / s.nf, f = pair - r * s.nf;
          const int lc = min(s.lcut ? s.lcut[r] : s.lcut0, g.l_max);
          // A = sum F1_mine P, D = sum F2_mine P, C = sum F1_other dP, B = sum F2_other dP
          const float Ar = D0[4 * q], Ai = D0[4 * q + 1], Dr = D0[4 * q + 2], Di = D0[4 * q + 3];
          const float Cr = D1[4 * q], Ci = D1[4 * q + 1], Br = D1[4 * q + 2], Bi = D1[4 * q + 3];
          double2 Sv = make_double2(f2d_int((dm * Ai + Br) * inv_ll), f2d_int((-dm * Ar + Bi) * inv_ll));
          double2 Tv = make_double2(f2d_int((-Cr + dm * Di) * inv_ll), f2d_int((-Ci - dm * Dr) * inv_ll));
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
// TF32 = false: 3 bf16 splits per 64-wide K chunk (3 blocks); true: 2 TF32
// splits x 2 K tiles of 32 (4 blocks, block = 2 * split + K tile).
template <bool TF32>
__device__ __forceinline__ void store_table_value(unsigned char* img, long long blk0, int row, int k, double v) {
  if (!TF32) {
    __nv_bfloat16 h[3];
    tc::split3((float)v, h[0], h[1], h[2]);
    for (int sp = 0; sp < 3; ++sp) *(__nv_bfloat16*)(img + (blk0 + sp) * 16384 + tc::sw128_offset(row, k)) = h[sp];
  } else {
    float h[2];
    tc::split_tf32((float)v, h[0], h[1]);
    for (int sp = 0; sp < 2; ++sp)
      *(float*)(img + (blk0 + 2 * sp + (k >> 5)) * 16384 + tc::sw128_offset32(row, k & 31)) = h[sp];
  }
}

template <bool TF32>
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
  constexpr int BPC = TF32 ? 4 : 3;  // 16 KB blocks per chunk
  for (int p = 0; p < 2; ++p)
    for (int lp = 0; lp < nch * 64; ++lp) {
      const int loff = p + 2 * lp;
      const double v = (valid && loff < n_l) ? tab[(size_t)(lm0 + loff) * g.nh + j] * inv : 0.0;
      const long long blk0 = t.inv_blk0[mc] + ((((long long)tt * 2 + tb) * 2 + p) * nch + lp / 64) * BPC;
      store_table_value<TF32>(img, blk0, row, lp % 64, v);
    }
}

template <bool TF32>
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
  constexpr int BPC = TF32 ? 4 : 3;
  for (int j = 0; j < t.ncj * 64; ++j) {
    const double v = (valid && j < g.nh) ? tab[(size_t)(lm0 + loff) * g.nh + j] * inv : 0.0;
    const long long blk0 = t.fwd_blk0[mc] + ((((long long)p * t.nlt + lt) * 2 + tb) * t.ncj + j / 64) * BPC;
    store_table_value<TF32>(img, blk0, row, j % 64, v);
  }
}

template <bool VEC>
cudaError_t launch_inv_tc_t(const ShtGeom& g, const InvSet& s, const TcTables& t, cudaStream_t st) {
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  if (ncplx <= 0) return cudaSuccess;
  const size_t smem = 1024 + (size_t)(VEC ? 2 : 1) * 2 * 16384 + 3 * 64 * 128;
  CUDA_TRY(cudaFuncSetAttribute(inv_leg_tc<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(t.ntt, (ncplx + 31) / 32, g.n_m * 2);
  inv_leg_tc<VEC><<<grid, TC_THREADS, smem, st>>>(g, s, t);
  return cudaGetLastError();
}

template <bool VEC>
cudaError_t launch_fwd_tc_t(const ShtGeom& g, const FwdSet& s, const TcTables& t, cudaStream_t st) {
  const int ncplx = s.nf * s.nlev * (VEC ? 2 : 1);
  if (ncplx <= 0) return cudaSuccess;
  constexpr int NC = VEC ? 64 : 128;
  const size_t smem = 1024 + (size_t)(VEC ? 2 : 1) * 2 * 16384 + (size_t)(VEC ? 2 : 1) * 3 * NC * 128;
  CUDA_TRY(cudaFuncSetAttribute(fwd_leg_tc<VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((ncplx + NC / 2 - 1) / (NC / 2), t.nlt, g.n_m * 2);
  fwd_leg_tc<VEC><<<grid, TC_THREADS, smem, st>>>(g, s, t);
  return cudaGetLastError();
}

}  // namespace

void tc_table_layout(const ShtGeom& g, bool tf32, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
                     std::vector<long long>& fwd_blk0, long long* inv_blocks, long long* fwd_blocks) {
  tc_table_layout_bpc(g, tf32 ? 4 : 3, ntt, nlt, ncj, inv_blk0, fwd_blk0, inv_blocks, fwd_blocks);
}

void tc_table_layout_bpc(const ShtGeom& g, int bpc, int* ntt, int* nlt, int* ncj, std::vector<long long>& inv_blk0,
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
    bi += (long long)(*ntt) * 2 * 2 * tc_nch(n_l) * bpc;
    fwd_blk0[mc] = bf;
    bf += 2LL * (*nlt) * 2 * (*ncj) * bpc;
  }
  *inv_blocks = bi;
  *fwd_blocks = bf;
}

cudaError_t build_tc_images(const ShtGeom& g, const TcTables& t, bool tf32, unsigned char* inv_img,
                            float* inv_scale, unsigned char* fwd_img, float* fwd_scale, cudaStream_t st) {
  {
    const long long n = (long long)g.n_m * 2 * t.ntt * 128;
    const unsigned nb = (unsigned)((n + 127) / 128);
    if (tf32) build_inv_img_kernel<true><<<nb, 128, 0, st>>>(g, t, inv_img, inv_scale);
    else build_inv_img_kernel<false><<<nb, 128, 0, st>>>(g, t, inv_img, inv_scale);
    CUDA_TRY(cudaGetLastError());
  }
  {
    const long long n = (long long)g.n_m * 4 * t.nlt * 128;
    const unsigned nb = (unsigned)((n + 127) / 128);
    if (tf32) build_fwd_img_kernel<true><<<nb, 128, 0, st>>>(g, t, fwd_img, fwd_scale);
    else build_fwd_img_kernel<false><<<nb, 128, 0, st>>>(g, t, fwd_img, fwd_scale);
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
