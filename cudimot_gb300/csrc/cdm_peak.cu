// cdm_peak.cu - FP32 FMA throughput probes used as the roofline peak of the
// FP32-pipe-bound fitting kernels. Each thread runs 8 independent FMA
// chains (enough independent work to cover the FMA latency); the grid is a
// multiple of the SM count. FLOPs = 2 per FMA. The paired probe issues the
// same chains as FFMA2 (two FMAs per instruction, __ffma2_rn), the form the
// kernels' paired cost loops use.
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

__global__ void __launch_bounds__(256) cdm_ffma2_probe_kernel(float* out, int iters, float a, float b) {
  const float t = threadIdx.x * 1e-3f;
  float2 x0 = make_float2(t, t + 0.5f), x1 = make_float2(t + 1, t + 1.5f);
  float2 x2 = make_float2(t + 2, t + 2.5f), x3 = make_float2(t + 3, t + 3.5f);
  float2 x4 = make_float2(t + 4, t + 4.5f), x5 = make_float2(t + 5, t + 5.5f);
  float2 x6 = make_float2(t + 6, t + 6.5f), x7 = make_float2(t + 7, t + 7.5f);
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      x0 = __ffma2_rn(x0, a2, b2); x1 = __ffma2_rn(x1, a2, b2); x2 = __ffma2_rn(x2, a2, b2);
      x3 = __ffma2_rn(x3, a2, b2); x4 = __ffma2_rn(x4, a2, b2); x5 = __ffma2_rn(x5, a2, b2);
      x6 = __ffma2_rn(x6, a2, b2); x7 = __ffma2_rn(x7, a2, b2);
    }
  }
  const float s = x0.x + x0.y + x1.x + x1.y + x2.x + x2.y + x3.x + x3.y + x4.x + x4.y + x5.x +
                  x5.y + x6.x + x6.y + x7.x + x7.y;
  if (s == 1234.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Same FMA count as cdm_ffma_probe (iters x 16 x 8 per thread) as FFMA2.
extern "C" int cdm_ffma2_probe(float* out, int iters, int blocks, void* stream) {
  cdm_ffma2_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-7f);
  return (int)cudaGetLastError();
}

extern "C" int cdm_ffma_probe(float* out, int iters, int blocks, void* stream) {
  cdm_ffma_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-7f);
  return (int)cudaGetLastError();
}

// FMAs issued by one launch.
extern "C" double cdm_ffma_probe_fmas(int iters, int blocks) {
  return (double)blocks * 256.0 * (double)iters * 16.0 * 8.0;
}
