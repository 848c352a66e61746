// cdm_postfit.cuh - predicted signal, BIC/AIC, and the layout kernels.
#pragma once
#include "cdm_common.cuh"

// Mean of a voxel's samples as CUDIMOT forms it (getPredictedSignal.cu:
// 63-79, BIC_AIC.cu:160-188): a plain sum divided by nsamples, or the
// single sample when nsamples == 1. Every lane of the group computes it.
__device__ __forceinline__ void cdm_sample_mean(const double* __restrict__ s, int nsamples,
                                                fp32* P) {
#pragma unroll
  for (int i = 0; i < kNPS; i++) P[i] = fp32(0.0f);
#pragma unroll
  for (int p = 0; p < kNP; p++) {
    double acc = 0.0;
    for (int k = 0; k < nsamples; k++) acc += s[(size_t)p * nsamples + k];
    P[p] = fp32((float)(nsamples > 1 ? acc / nsamples : acc));
  }
}

struct cdm_post_args {
  int nvox, nmeas, nmeas_pad, nsamples, fixp_tsize;
  uint32_t proto_bytes;
  const float* proto;
  const double* meas;     // [nvox][nmeas] (BIC/AIC)
  const double* samples;  // [nvox][NPARAMS][nsamples]
  const double* tau;      // [nvox][nsamples] or null
  const double* fixp;
  double* pred;           // [nvox][nmeas]
  double* bic;
  double* aic;
  int rician;
  int* err;
};

// getPredictedSignal_kernel (getPredictedSignal.cu:22-92): S(mean sample)
// for every measurement; a warp per voxel, lanes stride the measurements.
__global__ void __launch_bounds__(CDM_NT) cdm_predicted_kernel(const __grid_constant__ cdm_post_args a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int lane = threadIdx.x & 31;
  fp32 P[kNPS], FixP[kNFIX];
  cdm_sample_mean(a.samples + (size_t)v * kNP * a.nsamples, a.nsamples, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_update_derived(P, FixP);
  int m = lane;
#ifdef CDM_SIGNAL_PAIR
  // measurements m and m + 32 through the paired hook, the function the
  // fitting kernels' cost loops evaluate
  for (; m + 32 < a.nmeas; m += 64) {
    fp32 ca[kNCOLS], cb[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, ca);
    cdm_load_cfp(sproto, a.nmeas_pad, m + 32, cb);
    float2 ab[kNCOLS];
#pragma unroll
    for (int k = 0; k < kNCOLS; k++) ab[k] = make_float2(ca[k].v, cb[k].v);
    const float2 s = Predicted_Signal_Pair(P, ab, FixP);
    a.pred[(size_t)v * a.nmeas + m] = (double)s.x;
    a.pred[(size_t)v * a.nmeas + m + 32] = (double)s.y;
  }
#endif
  for (; m < a.nmeas; m += 32) {
    fp32 cf[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
    a.pred[(size_t)v * a.nmeas + m] = (double)(float)Predicted_Signal(NPARAMS, P, cf, FixP);
  }
}

// bic_aic_kernel (BIC_AIC.cu:112-201): Gaussian log-likelihood
// -(n/2) log(SSE/2), or the Rician one with tau averaged over its samples;
// BIC = -2 logL + np log n, AIC = -2 logL + 2 np (np + 1 with tau).
__global__ void __launch_bounds__(CDM_NT) cdm_bic_aic_kernel(const __grid_constant__ cdm_post_args a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int lane = threadIdx.x & 31;
  fp32 P[kNPS], FixP[kNFIX];
  cdm_sample_mean(a.samples + (size_t)v * kNP * a.nsamples, a.nsamples, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_update_derived(P, FixP);
  double tau = 0.0;
  if (a.rician) {
    double acc = 0.0;
    for (int k = 0; k < a.nsamples; k++) acc += a.tau[(size_t)v * a.nsamples + k];
    tau = a.nsamples > 1 ? acc / a.nsamples : acc;
  }
  const float tauf = (float)tau;
  float acc = 0.0f;
  for (int m = lane; m < a.nmeas; m += 32) {
    fp32 cf[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
    const float s = (float)Predicted_Signal(NPARAMS, P, cf, FixP);
    const float y = (float)a.meas[(size_t)v * a.nmeas + m];
    if (a.rician)
      acc += logf(y) + (-0.5f * tauf * (y * y + s * s) + cdm_log_i0(tauf * s * y));
    else
      acc = fmaf(s - y, s - y, acc);
  }
  const double tot = cdm_group_sum<32>((double)acc, 0xFFFFFFFFu);
  if (lane != 0) return;
  const double n = (double)a.nmeas;
  int np = kNP;
  double b;
  if (a.rician) {
    np++;
    b = n * log(tau) + tot;
  } else {
    b = -(n / 2.0) * log(tot / 2.0);
  }
  a.aic[v] = -2.0 * b + np * 2.0;
  a.bic[v] = -2.0 * b + np * log(n);
}

// Cost of given parameters, as the LM and grid search score them: sum of
// squared residuals (FP32 model, FP64 warp sum); a warp per voxel.
__global__ void __launch_bounds__(CDM_NT) cdm_cost_kernel(const __grid_constant__ cdm_post_args a,
                                                          const double* __restrict__ params,
                                                          double* __restrict__ cost) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int lane = threadIdx.x & 31;
  fp32 P[kNPS], FixP[kNFIX];
  cdm_load_params(params + (size_t)v * kNP, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_update_derived(P, FixP);
  float acc = 0.0f;
  for (int m = lane; m < a.nmeas; m += 32) {
    fp32 cf[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
    const float r = (float)Predicted_Signal(NPARAMS, P, cf, FixP) - (float)a.meas[(size_t)v * a.nmeas + m];
    acc = fmaf(r, r, acc);
  }
  const double tot = cdm_group_sum<32>((double)acc, 0xFFFFFFFFu);
  if (lane == 0) cost[v] = tot;
}

// Row helpers of the learned initialiser's fallback (voxels whose cost
// exceeds a reference cost by more than a margin are refit).
__global__ void cdm_select_worse_kernel(int n, const double* __restrict__ cost,
                                        const double* __restrict__ ref, double margin,
                                        int* __restrict__ idx, int* __restrict__ count) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    if (cost[v] > ref[v] * (1.0 + margin)) idx[atomicAdd(count, 1)] = v;
}

// dst[k][:] = src[idx[k]][:] (gather) or dst[idx[k]][:] = src[k][:] (scatter),
// or dst[idx[k]][:] = value (src null).
__global__ void cdm_rows_kernel(int nsel, const int* __restrict__ idx, int ncols,
                                const double* __restrict__ src, double* __restrict__ dst,
                                int scatter, double value) {
  const size_t total = (size_t)nsel * ncols;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / ncols), c = (int)(i % ncols);
    const size_t r = (size_t)idx[k];
    if (!src)
      dst[r * ncols + c] = value;
    else if (scatter)
      dst[r * ncols + c] = src[(size_t)k * ncols + c];
    else
      dst[(size_t)k * ncols + c] = src[r * ncols + c];
  }
}

// ---------------------------------------------------------------------------
// Layout kernels.
// Protocol: CUDIMOT's CFP [nmeas][CFP_Tsize] (double) plus the plugin's
// derived values -> FP32 [nmeas_pad][NCOLS4] (padding rows repeat
// measurement 0, padding columns are 0) and FP64 [nmeas][NCOLS] for the
// grid-search re-check.
__global__ void cdm_prep_protocol_kernel(const double* __restrict__ cfp, int nmeas, int nmeas_pad,
                                         float* __restrict__ p32, double* __restrict__ p64) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nmeas_pad; m += gridDim.x * blockDim.x) {
    const int src = m < nmeas ? m : 0;
    double row[kNCOLS];
#pragma unroll
    for (int k = 0; k < CDM_CFP_TSIZE; k++) row[k] = cfp[(size_t)src * CDM_CFP_TSIZE + k];
#ifdef CDM_DERIVED_CFP
    Derived_CFP<double>(row, row + CDM_CFP_TSIZE);
#endif
#pragma unroll
    for (int k = 0; k < kNCOLS4; k++) p32[(size_t)m * kNCOLS4 + k] = k < kNCOLS ? (float)row[k] : 0.0f;
#pragma unroll
    for (int k = 0; k < kNCOLS; k++)
      if (m < nmeas && p64) p64[(size_t)m * kNCOLS + k] = row[k];
  }
}

// Signals: [nvox][nmeas] double -> [nchunk][nvox][Gw] float, so that the Gw
// lanes of consecutive groups read one contiguous line per chunk.
template <int Gw>
__global__ void cdm_pack_signals_kernel(const double* __restrict__ meas, int nvox, int nmeas,
                                        int nchunk, float* __restrict__ out) {
  const size_t total = (size_t)nchunk * nvox * Gw;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % Gw);
    const size_t rest = i / Gw;
    const int v = (int)(rest % nvox);
    const int c = (int)(rest / nvox);
    const int m = c * Gw + j;
    out[i] = m < nmeas ? (float)meas[(size_t)v * nmeas + m] : 0.0f;
  }
}

// nsamples = 1 output when MCMC does not run: the fitted parameters are
// the single sample (Parameters.cu copyParams2Samples).
__global__ void cdm_params_to_samples_kernel(const double* __restrict__ params, int nvox,
                                             double* __restrict__ samples) {
  const size_t n = (size_t)nvox * kNP;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    samples[i] = params[i];
}
