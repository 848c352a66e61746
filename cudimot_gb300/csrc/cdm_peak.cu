// cdm_peak.cu - FP32 FMA throughput probe used as the roofline peak of the
// FP32-pipe-bound fitting kernels. Each thread runs 8 independent FMA
// chains (enough independent work to cover the FMA latency); the grid is a
// multiple of the SM count. FLOPs = 2 per FMA.
#include <cuda_runtime.h>

__global__ void __launch_bounds__(256) cdm_ffma_probe_kernel(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the loop live
}

extern "C" int cdm_ffma_probe(float* out, int iters, int blocks, void* stream) {
  cdm_ffma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-7f);
  return (int)cudaGetLastError();
}

// FMAs issued by one launch.
extern "C" double cdm_ffma_probe_fmas(int iters, int blocks) {
  return (double)blocks * 256.0 * (double)iters * 16.0 * 8.0;
}
