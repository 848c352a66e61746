// cdm_synth.cuh - kernels of the learned initialiser that need the plugin:
// synthetic signals (Predicted_Signal on given parameters + Rician noise),
// network targets from parameters and parameters from network outputs.
#pragma once
#include <cuda_bf16.h>
#include "cdm_common.cuh"
#include "philox.h"

// Counter slots of the synthetic-signal draws (third Philox word).
#define CDM_RNG_SLOT_SYNTH_SNR 0xFFFFFF00u
#define CDM_RNG_SLOT_SYNTH_NOISE 0xFFFFFF01u


// One warp per voxel: clean signal for every measurement, sigma = mean
// clean b = 0 signal / SNR (SNR uniform in [snr_lo, snr_hi] per voxel; the
// largest clean signal when the protocol has no b = 0 rows),
// y = |S + sigma (n1 + i n2)|. Draws: Philox(seed; voxel, measurement,
// slot), so a voxel's noise does not depend on the launch shape, and the
// b = 0 rows can be drawn twice (first for S0, then for the outputs).
__device__ __forceinline__ float cdm_synth_noisy(const cdm_synth_args& a, int v, int m, float s,
                                                 float sigma) {
  const cdm_u32x4 r = cdm_philox4x32_10({(uint32_t)v, (uint32_t)m, CDM_RNG_SLOT_SYNTH_NOISE, 0u},
                                        (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
  const float rad = sqrtf(-2.0f * logf(cdm_u01_open0(r.x)));
  const float u = cdm_u01_open1(r.y);
  const float re = s + sigma * rad * cospif(2.0f * u), im = sigma * rad * sinpif(2.0f * u);
  return sqrtf(re * re + im * im);
}

CDM_KERNEL(CDM_NT) cdm_synth_kernel(CDM_KARG(cdm_synth_args) a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int lane = threadIdx.x & 31;
  cdm_real P[kNPS], FixP[kNFIX];
  cdm_load_params(a.params + (size_t)v * kNP, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_update_derived(P, FixP);
  const cdm_u32x4 rs = cdm_philox4x32_10({(uint32_t)v, 0u, CDM_RNG_SLOT_SYNTH_SNR, 0u},
                                         (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
  const float snr = a.snr_lo + (a.snr_hi - a.snr_lo) * cdm_u01_open1(rs.x);
  // pass 1: clean b = 0 level (sigma), then the noisy b = 0 mean (S0)
  float b0 = 0.0f, smax = 0.0f;
  int nb0 = 0;
  for (int m = lane; m < a.nmeas; m += 32) {
    cdm_real cf[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
    const bool is_b0 = a.b_col >= 0 && (float)cf[a.b_col] == 0.0f;
    if (is_b0 || a.b_col < 0) {
      const float s = (float)Predicted_Signal(NPARAMS, P, cf, FixP);
      smax = fmaxf(smax, s);
      if (is_b0) {
        b0 += s;
        nb0++;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    b0 += __shfl_xor_sync(0xFFFFFFFFu, b0, o);
    nb0 += __shfl_xor_sync(0xFFFFFFFFu, nb0, o);
    smax = fmaxf(smax, __shfl_xor_sync(0xFFFFFFFFu, smax, o));
  }
  if (nb0 == 0 && a.b_col >= 0) {  // no b = 0 rows: largest clean signal
    for (int m = lane; m < a.nmeas; m += 32) {
      cdm_real cf[kNCOLS];
      cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
      smax = fmaxf(smax, (float)Predicted_Signal(NPARAMS, P, cf, FixP));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = fmaxf(smax, __shfl_xor_sync(0xFFFFFFFFu, smax, o));
  }
  const float sigma = (nb0 > 0 ? b0 / (float)nb0 : smax) / snr;
  float ysum = 0.0f;
  if (nb0 > 0) {
    for (int m = lane; m < a.nmeas; m += 32) {
      cdm_real cf[kNCOLS];
      cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
      if ((float)cf[a.b_col] == 0.0f)
        ysum += cdm_synth_noisy(a, v, m, (float)Predicted_Signal(NPARAMS, P, cf, FixP), sigma);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ysum += __shfl_xor_sync(0xFFFFFFFFu, ysum, o);
  }
  const float s0 = nb0 > 0 ? ysum / (float)nb0 : 1.0f;
  if (lane == 0 && a.s0_est) a.s0_est[v] = (double)s0;
  // pass 2: every measurement
  const float inv = s0 > 0.0f ? 1.0f / s0 : 1.0f;
  for (int m = lane; m < a.nmeas; m += 32) {
    cdm_real cf[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
    const float y = cdm_synth_noisy(a, v, m, (float)Predicted_Signal(NPARAMS, P, cf, FixP), sigma);
    if (a.meas) a.meas[(size_t)v * a.nmeas + m] = (double)y;
    if (a.x) a.x[(size_t)v * a.x_ld + m] = __float2bfloat16(y * inv);
  }
  if (a.x)
    for (int m = a.nmeas + lane; m < a.x_ld; m += 32)
      a.x[(size_t)v * a.x_ld + m] = __float2bfloat16(0.0f);
}

#ifdef CDM_MLP_HEAD
// Network targets from parameters (plugin hook MLP_Encode).
CDM_KERNEL0 cdm_mlp_encode_kernel(const double* __restrict__ params, int n,
                                      float* __restrict__ t) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    double P[kNP];
#pragma unroll
    for (int p = 0; p < kNP; p++) P[p] = params[(size_t)v * kNP + p];
    float out[CDM_MLP_NMU];
    MLP_Encode<double>(P, out);
#pragma unroll
    for (int j = 0; j < CDM_MLP_NMU; j++) t[(size_t)v * CDM_MLP_NMU + j] = out[j];
  }
}

// Parameters and MCMC proposal widths from network outputs (plugin hook
// MLP_Decode); outputs are [n][ld] float, means then log-stds.
CDM_KERNEL0 cdm_mlp_decode_kernel(const float* __restrict__ out, int ld, int n,
                                      double* __restrict__ params, double* __restrict__ prop_sd) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    float mu[CDM_MLP_NMU], ls[CDM_MLP_NSIG];
#pragma unroll
    for (int j = 0; j < CDM_MLP_NMU; j++) mu[j] = out[(size_t)v * ld + j];
#pragma unroll
    for (int j = 0; j < CDM_MLP_NSIG; j++) ls[j] = out[(size_t)v * ld + CDM_MLP_NMU + j];
    double P[kNP], sd[kNP];
    MLP_Decode<double>(mu, ls, P, sd);
#pragma unroll
    for (int p = 0; p < kNP; p++) {
      params[(size_t)v * kNP + p] = P[p];
      if (prop_sd) prop_sd[(size_t)v * kNP + p] = sd[p];
    }
  }
}
#endif
