// cdm_postfit.cuh - predicted signal, BIC/AIC, and the layout kernels.
#pragma once
#include "cdm_common.cuh"

// Mean of a voxel's samples as CUDIMOT forms it (getPredictedSignal.cu:
// 63-79, BIC_AIC.cu:160-188): a plain sum divided by nsamples, or the
// single sample when nsamples == 1. Every lane of the group computes it.
__device__ __forceinline__ void cdm_sample_mean(const double* __restrict__ s, int nsamples,
                                                cdm_real* P) {
#pragma unroll
  for (int i = 0; i < kNPS; i++) P[i] = cdm_real(0.0f);
#pragma unroll
  for (int p = 0; p < kNP; p++) {
    double acc = 0.0;
    for (int k = 0; k < nsamples; k++) acc += s[(size_t)p * nsamples + k];
    P[p] = cdm_real((float)(nsamples > 1 ? acc / nsamples : acc));
  }
}


// getPredictedSignal_kernel (getPredictedSignal.cu:22-92): S(mean sample)
// for every measurement; a warp per voxel, lanes stride the measurements.
CDM_KERNEL(CDM_NT) cdm_predicted_kernel(CDM_KARG(cdm_post_args) a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int lane = threadIdx.x & 31;
  cdm_real P[kNPS], FixP[kNFIX];
  cdm_sample_mean(a.samples + (size_t)v * kNP * a.nsamples, a.nsamples, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_update_derived(P, FixP);
  int m = lane;
#if CDM_PAIRED
  // measurements m and m + 32 through the paired hook, the function the
  // fitting kernels' cost loops evaluate
  for (; m + 32 < a.nmeas; m += 64) {
    cdm_real ca[kNCOLS], cb[kNCOLS];
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
    cdm_real cf[kNCOLS];
    cdm_load_cfp(sproto, a.nmeas_pad, m, cf);
    a.pred[(size_t)v * a.nmeas + m] = (double)(float)Predicted_Signal(NPARAMS, P, cf, FixP);
  }
}

// bic_aic_kernel (BIC_AIC.cu:112-201): Gaussian log-likelihood
// -(n/2) log(SSE/2), or the Rician one with tau averaged over its samples;
// BIC = -2 logL + np log n, AIC = -2 logL + 2 np (np + 1 with tau).
CDM_KERNEL(CDM_NT) cdm_bic_aic_kernel(CDM_KARG(cdm_post_args) a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int lane = threadIdx.x & 31;
  cdm_real P[kNPS], FixP[kNFIX];
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
    cdm_real cf[kNCOLS];
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


// Row helpers of the learned initialiser's fallback (voxels whose cost
// exceeds a reference cost by more than a margin are refit).
CDM_KERNEL0 cdm_select_worse_kernel(int n, const double* __restrict__ cost,
                                        const double* __restrict__ ref, double margin,
                                        int* __restrict__ idx, int* __restrict__ count) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    if (cost[v] > ref[v] * (1.0 + margin)) idx[atomicAdd(count, 1)] = v;
}

// dst[k][:] = src[idx[k]][:] (gather) or dst[idx[k]][:] = src[k][:] (scatter),
// or dst[idx[k]][:] = value (src null).
CDM_KERNEL0 cdm_rows_kernel(int nsel, const int* __restrict__ idx, int ncols,
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
CDM_KERNEL0 cdm_prep_protocol_kernel(const double* __restrict__ cfp, int nmeas, int nmeas_pad,
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

// Signals: [nvox][nmeas] double -> float, tile-major (cdm_tile_index): row
// c of a tile holds chunk c (measurement c * Gw + lane) of its voxels, so
// the Gw lanes of consecutive groups read one contiguous line per chunk.
template <int Gw>
CDM_KERNEL0 cdm_pack_signals_kernel(const double* __restrict__ meas, int nvox, int nmeas,
                                        int nchunk, float* __restrict__ out) {
  const size_t total = (size_t)nchunk * nvox * Gw;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % Gw);
    const size_t rest = i / Gw;
    const int v = (int)(rest % nvox);
    const int c = (int)(rest / nvox);
    const int m = c * Gw + j;
    out[cdm_tile_index(v, c, j, nchunk, Gw)] = m < nmeas ? (float)meas[(size_t)v * nmeas + m] : 0.0f;
  }
}

// nsamples = 1 output when MCMC does not run: the fitted parameters are
// the single sample (Parameters.cu copyParams2Samples).
CDM_KERNEL0 cdm_params_to_samples_kernel(const double* __restrict__ params, int nvox,
                                             double* __restrict__ samples) {
  const size_t n = (size_t)nvox * kNP;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    samples[i] = params[i];
}

// dMRI_Data::remove_NonPositive_entries (dMRI_Data.cu:15-30), which CUDIMOT
// applies to every voxel's signals when --rician is set (dMRI_Data.cu:133),
// so that log(S) in the Rician likelihood stays finite. If the smallest
// value is non-positive and the largest positive (both read as float, as
// the reference's MinS/MaxS), every entry that is non-positive as a float
// takes the smallest remaining value, min(smallest positive entry,
// float(largest)), rounded to float. One warp per voxel.
CDM_KERNEL0 cdm_clean_signals_kernel(int nvox, int nmeas, double* __restrict__ meas) {
  const int v = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = (int)(threadIdx.x & 31);
  if (v >= nvox) return;
  double* row = meas + (size_t)v * nmeas;
  double mn = CUDART_INF, mx = -CUDART_INF, mpos = CUDART_INF;
  for (int m = lane; m < nmeas; m += 32) {
    const double x = row[m];
    mn = fmin(mn, x);
    mx = fmax(mx, x);
    if ((float)x > 0.0f) mpos = fmin(mpos, x);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
    mpos = fmin(mpos, __shfl_xor_sync(0xFFFFFFFFu, mpos, o));
  }
  if (!((float)mn <= 0.0f && (float)mx > 0.0f)) return;
  const double rep = (double)(float)fmin(mpos, (double)(float)mx);
  for (int m = lane; m < nmeas; m += 32)
    if ((float)row[m] <= 0.0f) row[m] = rep;
}

// Self-test of the bounded waits: the CTA initialises an mbarrier that
// expects one arrival nobody makes and waits on it; the wait must give up
// after limit_ns and record CDM_DEVERR_STAGE_TIMEOUT (no copy is in flight,
// so the CTA can simply return).
CDM_KERNEL0 cdm_wait_selftest_kernel(uint64_t limit_ns, int* err) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t sbar = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sbar), "r"(1) : "memory");
  __syncthreads();
  cdm_mbar_wait_phase0(sbar, limit_ns, threadIdx.x == 0 ? err : nullptr);
}

#if CDM_SHELLS
// Shell table of the per-shell series (see cdm_prepare_tables): one CTA.
// Thread 0 assigns every measurement its shell (equal values of protocol
// column CDM_SHELL_KEY; in order of first appearance, at most kShellMax)
// and its rank in the shell, and lays the shells out one after another,
// each padded to whole pairs of Gw-lane chunks; the table is marked invalid
// (the kernels then take the per-measurement path) when there are more
// shells or the padding would add more than nmeas / 8 positions. All
// threads then fill perm (padded position -> measurement, -1 for padding)
// and the pair entries. shell_rank: int scratch [nmeas].
template <int Gw>
CDM_KERNEL0 cdm_prep_shells_kernel(const double* __restrict__ cfp, int nmeas, int nmeas_pad,
                                   float* __restrict__ table, int* __restrict__ perm,
                                   int* __restrict__ shell_rank) {
  int* hdr = reinterpret_cast<int*>(table);
  __shared__ int s_valid, s_nshell, s_npos, s_start[kShellMax + 1];
  if (threadIdx.x == 0) {
    double key[kShellMax];
    int count[kShellMax], rep[kShellMax];
    int nshell = 0;
    bool ok = true;
    for (int m = 0; m < nmeas && ok; m++) {
      const double b = cfp[(size_t)m * CDM_CFP_TSIZE + CDM_SHELL_KEY];
      int s = 0;
      while (s < nshell && key[s] != b) s++;
      if (s == nshell) {
        if (nshell == kShellMax) {
          ok = false;
          break;
        }
        key[s] = b;
        count[s] = 0;
        rep[s] = m;
        nshell++;
      }
      shell_rank[m] = (s << 24) | count[s]++;
    }
    int npos = 0;
    for (int s = 0; ok && s < nshell; s++) {
      s_start[s] = npos;
      const int padded = (count[s] + 2 * Gw - 1) / (2 * Gw) * (2 * Gw);
      hdr[4 + 3 * s] = rep[s];
      hdr[5 + 3 * s] = padded / (2 * Gw);
      hdr[6 + 3 * s] = npos / (2 * Gw);
      npos += padded;
    }
    ok = ok && nmeas < (1 << 24) && npos <= nmeas + nmeas / 8 && npos <= cdm_shell_max_pos(nmeas, Gw);
    s_valid = ok ? 1 : 0;
    s_nshell = ok ? nshell : 0;
    s_npos = ok ? npos : 0;
    hdr[0] = s_valid;
    hdr[1] = s_nshell;
    hdr[2] = s_npos;
  }
  __syncthreads();
  if (!s_valid) return;
  const int npos = s_npos;
  float* ent = table + kShellHeader;
  for (int p = threadIdx.x; p < npos; p += blockDim.x) perm[p] = -1;
  for (int p = threadIdx.x; p < npos; p += blockDim.x) {
    const int c = p / Gw, l = p % Gw;
    float* e = ent + ((size_t)(c / 2) * Gw + l) * 8 + (c & 1);
    e[0] = e[2] = e[4] = e[6] = 0.0f;
  }
  __syncthreads();
  for (int m = threadIdx.x; m < nmeas; m += blockDim.x) {
    const int sr = shell_rank[m];
    const int p = s_start[sr >> 24] + (sr & 0xFFFFFF);
    perm[p] = m;
    const int c = p / Gw, l = p % Gw;
    float* e = ent + ((size_t)(c / 2) * Gw + l) * 8 + (c & 1);
#pragma unroll
    for (int k = 0; k < CDM_SHELL_MCOLS; k++) e[2 * k] = (float)cfp[(size_t)m * CDM_CFP_TSIZE + k];
    e[6] = 1.0f;
  }
}

// Signals in the shell order of the table, pair-interleaved and tile-major
// ([nvox/T][npos / (2 Gw)][T][Gw][2]: a lane's positions of chunks 2k and
// 2k + 1 side by side, 0 on padding), or in measurement order as
// cdm_pack_signals_kernel when the table is invalid.
template <int Gw>
CDM_KERNEL0 cdm_pack_shell_signals_kernel(const double* __restrict__ meas, int nvox, int nmeas,
                                          int nchunk, const float* __restrict__ table,
                                          const int* __restrict__ perm, float* __restrict__ out) {
  const int* hdr = reinterpret_cast<const int*>(table);
  const bool shells = hdr[0] != 0;
  if (shells) {
    // pair-interleaved, tile-major (cdm_tile_index): element (pair k,
    // voxel v, lane j) holds the lane's positions of chunks 2k and 2k + 1
    const int npairs = hdr[2] / (2 * Gw);
    const size_t total = (size_t)npairs * nvox * Gw;
    float2* out2 = reinterpret_cast<float2*>(out);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
      const int j = (int)(i % Gw);
      const size_t rest = i / Gw;
      const int v = (int)(rest % nvox);
      const int k = (int)(rest / nvox);
      const int m0 = perm[(2 * k) * Gw + j], m1 = perm[(2 * k + 1) * Gw + j];
      const double* row = meas + (size_t)v * nmeas;
      out2[cdm_tile_index(v, k, j, npairs, Gw)] = make_float2(m0 >= 0 ? (float)row[m0] : 0.0f, m1 >= 0 ? (float)row[m1] : 0.0f);
    }
    return;
  }
  const size_t total = (size_t)nchunk * nvox * Gw;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(i % Gw);
    const size_t rest = i / Gw;
    const int v = (int)(rest % nvox);
    const int c = (int)(rest / nvox);
    const int p = c * Gw + j;
    out[cdm_tile_index(v, c, j, nchunk, Gw)] = p < nmeas ? (float)meas[(size_t)v * nmeas + p] : 0.0f;
  }
}
#endif
