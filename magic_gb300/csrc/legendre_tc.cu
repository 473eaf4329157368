// Tensor-core (tcgen05) form of the Legendre sums: 3xBF16 split products
// with FP32 accumulation in tensor memory.
//
// This file holds the tcgen05 GEMM self-test used to validate the operand
// layout and descriptor encodings on the device before the split-precision
// Legendre kernels use them.
#include <cuda_bf16.h>
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
