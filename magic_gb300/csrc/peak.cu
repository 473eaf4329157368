// FMA throughput probes (FP64 and FP32).  The FP64 form of the Legendre sums
// is bound by the FP64 pipe of the GPU (not by HBM), the FP32 form by the
// FP32 pipe, so their roofline denominators are the FMA rates measured here
// on the same device and in the same process.  Each thread runs 8
// independent FMA chains; the result is written so the work cannot be
// removed.
#include "common.cuh"
#include "internal.h"

namespace {
template <typename T>
__global__ void __launch_bounds__(256) fma_kernel(T* out, int iters) {
  T a0 = threadIdx.x * (T)1e-9, a1 = a0 + (T)1e-9, a2 = a0 + (T)2e-9, a3 = a0 + (T)3e-9;
  T a4 = a0 + (T)4e-9, a5 = a0 + (T)5e-9, a6 = a0 + (T)6e-9, a7 = a0 + (T)7e-9;
  const T b = (T)0.999999999, c = (T)1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
      a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
  }
  const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == (T)12345.678) out[blockIdx.x] = s;  // practically never; keeps the chains live
  if (threadIdx.x == 0 && blockIdx.x == 0) out[gridDim.x] = s;
}
}  // namespace

// flops per launch = blocks * 256 threads * iters * 16 * 8 FMA * 2
cudaError_t launch_fma_peak(void* out, bool fp64, int blocks, int iters, cudaStream_t st) {
  if (fp64) fma_kernel<double><<<blocks, 256, 0, st>>>((double*)out, iters);
  else fma_kernel<float><<<blocks, 256, 0, st>>>((float*)out, iters);
  return cudaGetLastError();
}
