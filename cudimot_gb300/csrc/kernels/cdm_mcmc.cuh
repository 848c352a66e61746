// cdm_mcmc.cuh - Metropolis-within-Gibbs sampler, one voxel per lane group.
//
// Semantics follow CUDIMOT's mcmc_kernel (MCMC.cu:327-683) launched twice by
// MCMC<T>::run (MCMC.cu:799-847): a burn-in of max(bi,1) iterations that
// always adapts the proposal widths, then a recording run of nj iterations
// that keeps every se-th state. Here both runs are one launch with the chain
// state kept in registers between them.
//  * proposal widths start at P/10 (MCMC.cu:428) and are scaled by
//    sqrt((accepted+1)/(rejected+1)) every se iterations, capped at 1e10
//    (MCMC.cu:630-646);
//  * parameters are clamped into bounds and priors initialised at the start
//    of each run (MCMC.cu:97-139);
//  * per iteration: the Rician precision tau (if enabled), then every
//    parameter in order: propose, reject outside bounds or
//    ConstraintsMCMC, otherwise accept if exp(E_old - E_new) > U
//    (MCMC.cu:498-613);
//  * Gaussian likelihood (n/2) log(SSE/2); Rician -n log(tau) - sum(...)
//    (MCMC.cu:254-307).
// Differences: draws come from Philox (philox.h), keyed by the seed and
// counted by (voxel, iteration, parameter, part); fixed parameters skip the
// likelihood evaluation CUDIMOT spends re-proposing them at their own value
// (always accepted there too). Energies are kept in FP64; the SSE is summed
// in FP32 per lane and in FP64 across lanes.
#pragma once
#include "cdm_common.cuh"


__device__ __forceinline__ float cdm_prior(const cdm_limits& lim, int p, cdm_real* P, int nmeas,
                                           cdm_real* cfp_all, cdm_real* FixP) {
  cdm_real xv = P[0];
#pragma unroll
  for (int k = 1; k < kNP; k++) xv = (k == p) ? P[k] : xv;
  const float x = (float)xv;
  switch (lim.ptype[p]) {
    case GAUSSPRIOR: {
      const float d = x - lim.pa[p];
      return d * d / (2.0f * lim.pb[p] * lim.pb[p]);
    }
    case GAMMAPRIOR:
      return __fmaf_rn(lim.pb[p], x, __fmul_rn(1.0f - lim.pa[p], logf(x)));
    case ARDPRIOR:
      return lim.pa[p] * logf(x);
    case SINPRIOR:
      return -logf(fabsf(sinf(x) * 0.5f));
    case CUSTOM:
      return (float)custom_priors(p, P, nmeas, cfp_all, FixP);
    default:
      return 0.0f;
  }
}

__device__ __forceinline__ bool cdm_in_bounds(const cdm_limits& lim, int p, cdm_real* P) {
  if (!ConstraintsMCMC(NPARAMS, P)) return false;
  cdm_real xv = P[0];
#pragma unroll
  for (int k = 1; k < kNP; k++) xv = (k == p) ? P[k] : xv;
  const float x = (float)xv;
  if (lim.btype[p] == BMIN) return !(x < lim.bmin[p]);
  if (lim.btype[p] == BMAX) return !(x > lim.bmax[p]);
  if (lim.btype[p] == BMINMAX) return !(x < lim.bmin[p]) && !(x > lim.bmax[p]);
  return true;
}

// Register arrays indexed by a runtime parameter id: the proposal loop over
// parameters is kept rolled (one copy of the inlined likelihood in the
// instruction cache instead of NPARAMS), and these unrolled selects keep
// the arrays in registers.
// Only the first kNP entries are ever selected (the model parameters).
template <class Tv>
__device__ __forceinline__ Tv cdm_get(const Tv* a, int i) {
  Tv v = a[0];
#pragma unroll
  for (int k = 1; k < kNP; k++) v = (k == i) ? a[k] : v;
  return v;
}
template <class Tv>
__device__ __forceinline__ void cdm_set(Tv* a, int i, Tv x) {
#pragma unroll
  for (int k = 0; k < kNP; k++) a[k] = (k == i) ? x : a[k];
}

// Rician energy of the current state: -n log(tau) - sum log-likelihood
// terms (FP64 group sum). Written with explicitly rounded operations, so
// that whether a multiply and an add are fused is fixed by the source, not
// by the compiler's view of the surrounding code: the chain is the same in
// every kernel this code is compiled into (model library, multi-model
// kernel).
template <int Gw>
__device__ __forceinline__ double cdm_rician_energy(const cdm_voxel_io& io, const float* sproto,
                                                    cdm_real* P, cdm_real* FixP, float tau,
                                                    unsigned gmask) {
  const double s = cdm_group_rician<Gw>(io, sproto, P, FixP, tau, gmask);
  return __fma_rn(-(double)io.nmeas, (double)logf(tau), -s);
}

// Gaussian energy difference of a proposal. The energy is prior +
// (n/2) log(SSE/2) (MCMC.cu:206-219); the acceptance needs only
// E_old - E_new = (prior_old - prior_new) + (n/2) log(SSE_old / SSE_new).
// The SSE sums are FP64 (group sum); their ratio is near 1 and is taken,
// with its logarithm, in FP32: the difference is then good to about
// n/2 x 2e-7 (3e-5 for 288 measurements) with no FP64 operation beyond the
// sum, where the absolute energies (~1e3) would need FP64 logarithms.
__device__ __forceinline__ float cdm_gauss_delta(double sse_old, double sse_new, float tp_old,
                                                 float tp_new, float halfn) {
  const float r = __fdividef((float)sse_old, (float)sse_new);
  return __fmaf_rn(halfn, logf(r), __fsub_rn(tp_old, tp_new));
}

// Records sample s of a sample row (element index row0 + s of dst, a row
// of nsamples doubles). Samples are recorded every sampleevery iterations,
// one double per row each time; written straight to global memory, each
// would leave its 32-byte DRAM sector partly written for a long time, and a
// partly written sector costs a read of the sector when it is evicted (the
// read excess of the sampler's DRAM traffic). So the value is kept in the
// row's shared-memory slot until the sector is complete - element index
// = 3 mod 4, assuming dst 32-byte aligned (cudaMalloc and torch
// allocations are 256-byte aligned) - or the row ends, and the sector's
// elements of this row are then written back to back.
__device__ __forceinline__ void cdm_record_sample(double (&buf)[4], double* dst, size_t row0,
                                                  int s, int nsamples, double x) {
  const size_t e = row0 + (size_t)s;
  const int slot = (int)(e & 3);
  buf[slot] = x;
  if (slot == 3 || s == nsamples - 1) {
    const int first = slot < s ? 0 : slot - s;  // elements of this row in the sector
    for (int k = first; k <= slot; k++) dst[e - slot + k] = buf[k];
  }
}

// Minimum resident CTAs per SM requested from the register allocator.
#ifndef CDM_MCMC_MIN_BLOCKS
#define CDM_MCMC_MIN_BLOCKS 4
#endif

template <int Gw, bool RICIAN>
CDM_KERNEL(CDM_NT, CDM_MCMC_MIN_BLOCKS) cdm_mcmc_kernel(CDM_KARG(cdm_mcmc_args) a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int* shdr;
  const float* ptab = cdm_prepare_tables<Gw>(sproto, a.nmeas_pad, a.nchunk, a.shells_staged != 0, &shdr);
  if (a.cfp_all_off >= 0) {  // the protocol as custom priors see it
    cdm_real* dst = reinterpret_cast<cdm_real*>(sproto + a.cfp_all_off);
    for (int i = (int)threadIdx.x; i < a.nmeas * CDM_CFP_TSIZE; i += CDM_NT)
      dst[i] = cdm_real(sproto[(size_t)(i / CDM_CFP_TSIZE) * kNCOLS4 + i % CDM_CFP_TSIZE]);
    __syncthreads();
  }
  // recorded samples wait here until their 32-byte DRAM sector is complete
#ifdef CDM_HETERO
  double(*sbuf)[kNP + 1][4] = reinterpret_cast<double(*)[kNP + 1][4]>(cdm_scratch);
#else
  __shared__ double sbuf[CDM_NT / Gw][kNP + 1][4];
#endif
  const int vloc = (int)threadIdx.x / Gw;
  const int v = (int)CDM_BLOCK_IDX * (CDM_NT / Gw) + vloc;
  if (v >= a.nvox) return;
  const unsigned gm = cdm_group_mask<Gw>();
  const int lane = (int)threadIdx.x % Gw;
  const cdm_limits& lim = a.lim;

  cdm_voxel_io io;
  io.sig = a.sig + cdm_tile_index(v, 0, lane, a.nchunk, Gw);
  io.sig2 = shdr ? reinterpret_cast<const float2*>(a.sig) +
                       cdm_tile_index(v, 0, lane, shdr[2] / (2 * Gw), Gw)
                 : nullptr;
  io.chunk_stride = CDM_NT;
  io.nchunk = a.nchunk;
  io.nmeas = a.nmeas;
  io.nmeas_pad = a.nmeas_pad;
  io.lane = lane;
  io.pairs = ptab + (size_t)lane * kNCOLSP * 2;
  io.shells = shdr;
  io.stab = ptab + (size_t)lane * 8;

  cdm_real P[kNPS], FixP[kNFIX];
  cdm_load_params(a.params + (size_t)v * kNP, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  float propSD[kNP], prior[kNP];
  int acc[kNP], rej[kNP];
#pragma unroll
  for (int p = 0; p < kNP; p++)
    propSD[p] = (a.prop_sd && a.prop_sd[(size_t)v * kNP + p] > 0.0)
                    ? (float)a.prop_sd[(size_t)v * kNP + p]
                    : (float)P[p] / 10.0f;
  float tau = 0.0f, tauSD = 0.0f;
  int tacc = 0, trej = 0;
  const uint32_t vid = a.voxel_offset + (uint32_t)v;
  const int nburn = a.nburn < 1 ? 1 : a.nburn;
  // custom priors receive the whole CFP array, [nmeas][CFP_Tsize], as in
  // CUDIMOT (MCMC.cu custom_priors); the copy is built by the CTA below
  cdm_real* cf0 = a.cfp_all_off >= 0 ? reinterpret_cast<cdm_real*>(sproto + a.cfp_all_off) : nullptr;

  double energy = 0.0;  // Rician: the current energy
  double sse_c = 1.0;   // Gaussian: the current SSE and prior total
  float tp_c = 0.0f;
  const float halfn = 0.5f * (float)a.nmeas;
  bool stale = false;  // derived values of P out of date (after a rejection)
  for (int phase = 0; phase < 2; phase++) {
    const bool recording = phase == 1;
    const int niters = recording ? a.njumps : nburn;
#pragma unroll
    for (int p = 0; p < kNP; p++) {
      acc[p] = 0;
      rej[p] = 0;
      float x = (float)P[p];
      if (lim.btype[p] == BMIN) {
        if (x < lim.bmin[p]) x = lim.bmin[p];
      } else if (lim.btype[p] == BMAX) {
        if (x > lim.bmax[p]) x = lim.bmax[p];
      } else if (lim.btype[p] == BMINMAX) {
        if (x < lim.bmin[p]) x = lim.bmin[p];
        else if (x > lim.bmax[p]) x = lim.bmax[p];
      }
      P[p] = cdm_real(x);
    }
    cdm_update_derived(P, FixP);
    stale = false;
    float total_prior = 0.0f;
#pragma unroll
    for (int p = 0; p < kNP; p++) {
      prior[p] = cdm_prior(lim, p, P, a.nmeas, cf0, FixP);
      total_prior += prior[p];
    }
    tacc = trej = 0;
    if (RICIAN && !recording) {
      // Initialise_TauRician (MCMC.cu:193-251): tau = 1 / variance of residuals.
      float s1 = 0.0f;
      for (int c = 0; c < io.nchunk; c++) {
        const int m = c * Gw + lane;
        cdm_real cf[kNCOLS];
        cdm_load_cfp(sproto, io.nmeas_pad, m < io.nmeas ? m : 0, cf);
        const float r = (float)Predicted_Signal(NPARAMS, P, cf, FixP) - io.sig[(size_t)c * io.chunk_stride];
        s1 = (m < io.nmeas) ? s1 + r : s1;
      }
      const float mean = (float)(cdm_group_sum<Gw>((double)s1, gm) / io.nmeas);
      float s2 = 0.0f;
      for (int c = 0; c < io.nchunk; c++) {
        const int m = c * Gw + lane;
        cdm_real cf[kNCOLS];
        cdm_load_cfp(sproto, io.nmeas_pad, m < io.nmeas ? m : 0, cf);
        const float r = mean - ((float)Predicted_Signal(NPARAMS, P, cf, FixP) - io.sig[(size_t)c * io.chunk_stride]);
        s2 = (m < io.nmeas) ? fmaf(r, r, s2) : s2;
      }
      tau = (float)((double)io.nmeas / cdm_group_sum<Gw>((double)s2, gm));
      tauSD = tau * 0.5f;
    }
    if constexpr (RICIAN) {
      energy = __dadd_rn((double)total_prior, cdm_rician_energy<Gw>(io, sproto, P, FixP, tau, gm));
    } else {
      sse_c = cdm_group_sse<Gw>(io, sproto, P, FixP, gm);
      tp_c = total_prior;
    }

    for (int it = 0; it < niters; it++) {
      const uint32_t git = (uint32_t)(recording ? nburn + it : it);
      if constexpr (RICIAN) {
        const cdm_draw d = cdm_mcmc_draw(a.seed, vid, git, CDM_RNG_SLOT_TAU, a.stream);
        const float old = tau;
        tau = __fmaf_rn(d.normal, tauSD, tau);
        if (tau > 0.0f) {
          if (stale) cdm_update_derived(P, FixP);
          stale = false;
          float tp = 0.0f;
#pragma unroll
          for (int p = 0; p < kNP; p++) tp += prior[p];
          const double ne = __dadd_rn((double)tp, cdm_rician_energy<Gw>(io, sproto, P, FixP, tau, gm));
          if (expf((float)__dsub_rn(energy, ne)) > d.uniform) {
            tacc++;
            energy = ne;
          } else {
            trej++;
            tau = old;
          }
        } else {
          trej++;
          tau = old;
        }
      }
#pragma unroll 1
      for (int p = 0; p < kNP; p++) {
        if (lim.fixed[p]) {
          cdm_set(acc, p, cdm_get(acc, p) + 1);
          continue;
        }
        const cdm_draw d = cdm_mcmc_draw(a.seed, vid, git, (uint32_t)p, a.stream);
        const cdm_real old = cdm_get(P, p);
        cdm_set(P, p, cdm_real(__fmaf_rn(d.normal, cdm_get(propSD, p), (float)old)));
        bool accepted = false;
        bool derived = false;
        if (cdm_in_bounds(lim, p, P)) {
          cdm_update_derived(P, FixP);
          derived = true;
          stale = false;
          const float np_ = cdm_prior(lim, p, P, a.nmeas, cf0, FixP);
          float tp = 0.0f;
#pragma unroll
          for (int q = 0; q < kNP; q++) tp += (q == p) ? np_ : prior[q];
          if constexpr (RICIAN) {
            const double ne = __dadd_rn((double)tp, cdm_rician_energy<Gw>(io, sproto, P, FixP, tau, gm));
            if (expf((float)__dsub_rn(energy, ne)) > d.uniform) {
              accepted = true;
              energy = ne;
              cdm_set(prior, p, np_);
            }
          } else {
            const double sse_n = cdm_group_sse<Gw>(io, sproto, P, FixP, gm);
            if (expf(cdm_gauss_delta(sse_c, sse_n, tp_c, tp, halfn)) > d.uniform) {
              accepted = true;
              sse_c = sse_n;
              tp_c = tp;
              cdm_set(prior, p, np_);
            }
          }
        }
        if (accepted) {
          cdm_set(acc, p, cdm_get(acc, p) + 1);
        } else {
          cdm_set(rej, p, cdm_get(rej, p) + 1);
          cdm_set(P, p, old);
          // The derived values now belong to the rejected point. Derived_P
          // is a function of P, and the next likelihood (the next proposal,
          // or the tau proposal) derives first, so they are not recomputed
          // here (3 % of the MCMC time on NODDI-Watson).
          stale = stale || derived;  // out of bounds: P and its derived values unchanged
        }
      }
      if (recording && (it % a.sampleevery) == 0) {
        const int s = it / a.sampleevery;
        if (s < a.nsamples && lane == 0) {
#pragma unroll
          for (int p = 0; p < kNP; p++)  // fixed parameters: their input value, in double
            cdm_record_sample(sbuf[vloc][p], a.samples, ((size_t)v * kNP + p) * a.nsamples, s,
                              a.nsamples,
                              lim.fixed[p] ? a.params[(size_t)v * kNP + p] : (double)(float)P[p]);
          if (RICIAN && a.tau_samples)
            cdm_record_sample(sbuf[vloc][kNP], a.tau_samples, (size_t)v * a.nsamples, s,
                              a.nsamples, (double)tau);
        }
      }
      if ((!recording || a.update_proposal) && it > 0 && (it % a.sampleevery) == 0) {
#pragma unroll
        for (int p = 0; p < kNP; p++) {
          propSD[p] *= sqrtf(((float)acc[p] + 1.0f) / ((float)rej[p] + 1.0f));
          propSD[p] = fminf(propSD[p], 1e10f);
          acc[p] = 0;
          rej[p] = 0;
        }
        if (RICIAN) {
          tauSD *= sqrtf(((float)tacc + 1.0f) / ((float)trej + 1.0f));
          tauSD = fminf(tauSD, 1e10f);
          tacc = 0;
          trej = 0;
        }
      }
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int p = 0; p < kNP; p++)
      if (!lim.fixed[p]) a.params[(size_t)v * kNP + p] = (double)(float)P[p];
  }
}
