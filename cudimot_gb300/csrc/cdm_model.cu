// cdm_model.cu - one translation unit per model plugin: the fitting kernels
// instantiated for the plugin, and the C ABI of include/cudimot_gb300.h.
//
// Include order is CUDIMOT's (GridSearch.cu:7-11): math prelude, the
// plugin's modelparameters.h, macro_numerical.h, the plugin's
// modelfunctions.h; then this library's plugin tail and kernels.
//
// System and library headers come first: a plugin's object-like macros
// (CUDIMOT's NODDI_Watson defines H, MPI, NMAX, A1-A3; its Legendre header
// MN) stay in force for everything included after it, so only the kernels,
// written with prefixed or multi-letter names, follow the plugin.
#include <math_constants.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "cdm_host.h"
#include "cudimot_gb300.h"

#include "functions_gpu.h"
#include "modelparameters.h"
#include "macro_numerical.h"
#include "modelfunctions.h"
#include "cdm_plugin_tail.h"
#include "cdm_model_sizes.h"

#include "cdm_common.cuh"
#include "cdm_gridsearch.cuh"
#include "cdm_levmar.cuh"
#include "cdm_mcmc.cuh"
#include "cdm_postfit.cuh"
#include "cdm_synth.cuh"

#ifndef CDM_MODEL_NAME
#define CDM_MODEL_NAME "model"
#endif

static_assert(NPARAMS <= CDM_MAX_PARAMS, "NPARAMS exceeds CDM_MAX_PARAMS");

namespace {

constexpr float kGsBand = 2e-5f;  // FP32 grid-search near-tie band (relative)

#define CDM_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      cdm_fail(CDM_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
      return CDM_CUDA_ERROR;                                                  \
    }                                                                         \
  } while (0)

#define CDM_TRY(expr)                   \
  do {                                  \
    cdm_status s_ = (expr);             \
    if (s_ != CDM_OK) return s_;        \
  } while (0)

template <class T>
cdm_status dev_alloc(T** p, size_t* cap, size_t n) {
  if (n <= *cap && *p) return CDM_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  if (n == 0) return CDM_OK;
  CDM_CUDA(cudaMalloc((void**)p, n * sizeof(T)));
  *cap = n;
  return CDM_OK;
}

int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

struct cdm_ctx {
  cdm_model_cfg cfg;
  std::vector<double> grid_host;
  cdm_limits lim;
  int gpos[kNP];
  int device = 0;
  int num_sms = 0;
  // scratch (owned)
  double* grid_dev = nullptr;
  size_t grid_cap = 0;
  float* proto32 = nullptr;
  size_t proto32_cap = 0;
  double* proto64 = nullptr;
  size_t proto64_cap = 0;
  float* sig = nullptr;
  size_t sig_cap = 0;
  int* gs_flags = nullptr;
  size_t gs_flags_cap = 0;
  int* gs_cand = nullptr;
  size_t gs_cand_cap = 0;
  int* gs_best = nullptr;
  size_t gs_best_cap = 0;
  int* err = nullptr;
  unsigned long long* counters = nullptr;  // [0] lm passes [1] lm successes [2] gs rechecks
  const double* prop_sd = nullptr;          // initial MCMC proposal widths of the next run_mcmc
  // host-buffer path
  double* h_meas = nullptr; size_t h_meas_cap = 0;
  double* h_params = nullptr; size_t h_params_cap = 0;
  double* h_cfp = nullptr; size_t h_cfp_cap = 0;
  double* h_fixp = nullptr; size_t h_fixp_cap = 0;
  double* h_samples = nullptr; size_t h_samples_cap = 0;
  double* h_tau = nullptr; size_t h_tau_cap = 0;
  double* h_pred = nullptr; size_t h_pred_cap = 0;
  double* h_bic = nullptr; size_t h_bic_cap = 0;
  double* h_aic = nullptr; size_t h_aic_cap = 0;
  cudaStream_t own_stream = nullptr;
  // captured fit
  cudaGraphExec_t graph = nullptr;
  std::vector<uintptr_t> graph_key;
  // current protocol / packed signal state
  int nmeas_pad = 0;
};

namespace {

cdm_status ensure_base(cdm_ctx* c) {
  if (!c->err) {
    CDM_CUDA(cudaMalloc((void**)&c->err, sizeof(int)));
    CDM_CUDA(cudaMemset(c->err, 0, sizeof(int)));
    CDM_CUDA(cudaMalloc((void**)&c->counters, 4 * sizeof(unsigned long long)));
    CDM_CUDA(cudaMemset(c->counters, 0, 4 * sizeof(unsigned long long)));
  }
  return CDM_OK;
}

size_t proto_bytes(int nmeas_pad) { return (size_t)kNCOLS4 * nmeas_pad * sizeof(float); }
// Dynamic shared memory of the kernels with the paired cost loop (grid
// search, LM, MCMC): the staged protocol and, with the paired signal hook,
// its pair table of the same size.
size_t fit_smem(int nmeas_pad) { return proto_bytes(nmeas_pad) * (1 + kPairTables); }

cdm_status check_common(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size) {
  if (!c) return cdm_fail(CDM_BAD_ARG, "null context");
  if (nvox < 0 || nmeas <= 0) return cdm_fail(CDM_BAD_ARG, "nvox must be >= 0 and nmeas > 0");
  if (CFP_size != CDM_CFP_TSIZE)
    return cdm_fail(CDM_BAD_ARG, "CFP_size " + std::to_string(CFP_size) + " != model CFP_Tsize " +
                                     std::to_string(CDM_CFP_TSIZE));
  if (FixP_size != CDM_FIXP_TSIZE)
    return cdm_fail(CDM_BAD_ARG, "FixP_size " + std::to_string(FixP_size) +
                                     " != model FixP_Tsize " + std::to_string(CDM_FIXP_TSIZE));
  const int pad = round_up(nmeas, 32);
  if (fit_smem(pad) > 200 * 1024)
    return cdm_fail(CDM_BAD_ARG, "protocol too large for shared memory staging");
  return CDM_OK;
}

// Protocol tables from CUDIMOT's CFP array (device pointer).
cdm_status prep_protocol(cdm_ctx* c, int nmeas, const double* CFP, cudaStream_t st) {
  const int pad = round_up(nmeas, 32);
  CDM_TRY(dev_alloc(&c->proto32, &c->proto32_cap, (size_t)kNCOLS4 * pad));
  CDM_TRY(dev_alloc(&c->proto64, &c->proto64_cap, (size_t)kNCOLS * nmeas));
  c->nmeas_pad = pad;
  cdm_prep_protocol_kernel<<<(pad + 127) / 128, 128, 0, st>>>(CFP, nmeas, pad, c->proto32, c->proto64);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

template <int Gw>
cdm_status pack_signals_g(cdm_ctx* c, int nvox, int nmeas, const double* meas, cudaStream_t st) {
  const int nchunk = (nmeas + Gw - 1) / Gw;
  CDM_TRY(dev_alloc(&c->sig, &c->sig_cap, (size_t)nchunk * std::max(nvox, 1) * Gw));
  if (nvox == 0) return CDM_OK;
  const size_t total = (size_t)nchunk * nvox * Gw;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)c->num_sms * 32);
  cdm_pack_signals_kernel<Gw><<<blocks, 256, 0, st>>>(meas, nvox, nmeas, nchunk, c->sig);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status pack_signals(cdm_ctx* c, int Gw, int nvox, int nmeas, const double* meas, cudaStream_t st) {
  switch (Gw) {
    case 1: return pack_signals_g<1>(c, nvox, nmeas, meas, st);
    case 2: return pack_signals_g<2>(c, nvox, nmeas, meas, st);
    case 4: return pack_signals_g<4>(c, nvox, nmeas, meas, st);
    case 8: return pack_signals_g<8>(c, nvox, nmeas, meas, st);
    case 16: return pack_signals_g<16>(c, nvox, nmeas, meas, st);
    case 32: return pack_signals_g<32>(c, nvox, nmeas, meas, st);
  }
  return cdm_fail(CDM_BAD_ARG, "lanes per voxel must be 1, 2, 4, 8, 16 or 32");
}

template <class Kfn>
cdm_status set_smem(Kfn kernel, size_t bytes) {
  if (bytes > 48 * 1024) CDM_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return CDM_OK;
}

// Lanes per voxel: explicit choice, else a per-stage floor measured on
// GB300 for a 200k-voxel, 288-measurement NODDI-Watson fit (grid search 2,
// LM 4, MCMC 2). Each lane repeats the parameter-only work and takes part
// in the group reductions, so few lanes are best while there are enough
// voxels to fill the GPU; with fewer voxels than about four waves of
// resident threads the group is widened.
int pick_lanes(const cdm_ctx* c, int requested, int base, int nvox) {
  if (requested == 1 || requested == 2 || requested == 4 || requested == 8 || requested == 16 ||
      requested == 32)
    return requested;
  const long resident = (long)std::max(c->num_sms, 1) * 512;
  int g = base;
  while (g < 32 && (long)nvox * g < 4 * resident) g *= 2;
  return g;
}

template <class Args>
void fill_common(cdm_ctx* c, Args& a, int nvox, int nmeas, int Gw) {
  a.nvox = nvox;
  a.nmeas = nmeas;
  a.nmeas_pad = c->nmeas_pad;
  a.nchunk = (nmeas + Gw - 1) / Gw;
  a.fixp_tsize = CDM_FIXP_TSIZE;
  a.proto_bytes = (uint32_t)proto_bytes(c->nmeas_pad);
  a.proto = c->proto32;
  a.sig = c->sig;
  a.err = c->err;
  a.lim = c->lim;
}

int blocks_for(int nvox, int Gw) { return (nvox + (CDM_NT / Gw) - 1) / (CDM_NT / Gw); }

// ------------------------------------------------------------------ stages
template <int Gw>
cdm_status launch_gs(cdm_ctx* c, int nvox, int nmeas, double* params, const double* FixP,
                     cudaStream_t st) {
  cdm_gs_args a;
  fill_common(c, a, nvox, nmeas, Gw);
  a.params = params;
  a.fixp = FixP;
  a.grid = c->grid_dev;
  a.ngp = c->cfg.n_grid_params;
  a.combs = c->cfg.grid_combs;
  for (int p = 0; p < kNP; p++) a.gpos[p] = c->gpos[p];
  a.band = kGsBand;
  a.flags = c->gs_flags;
  a.cand = c->gs_cand;
  a.best = c->gs_best;
  const size_t sm = fit_smem(c->nmeas_pad);
  CDM_TRY(set_smem(cdm_gridsearch_kernel<Gw>, sm));
  cdm_gridsearch_kernel<Gw><<<blocks_for(nvox, Gw), CDM_NT, sm, st>>>(a);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status run_gridsearch(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                          const double* CFP, const double* FixP, cudaStream_t st) {
  if (c->cfg.grid_combs <= 0 || c->cfg.n_grid_params <= 0) return CDM_OK;
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  // narrowest groups first: measured on NODDI-Watson, 200k voxels x 288
  // measurements, 968 combinations: 2 lanes 91 ms, 4 lanes 100 ms, 8 lanes
  // 150 ms (1 lane 164 ms)
  const int Gw = pick_lanes(c, c->cfg.lanes_gridsearch, 2, nvox);
  CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  const size_t n = (size_t)std::max(nvox, 1);
  CDM_TRY(dev_alloc(&c->gs_flags, &c->gs_flags_cap, n));
  CDM_TRY(dev_alloc(&c->gs_cand, &c->gs_cand_cap, n * kGsTop));
  CDM_TRY(dev_alloc(&c->gs_best, &c->gs_best_cap, n));
  if (nvox == 0) return CDM_OK;
  switch (Gw) {
    case 1: CDM_TRY(launch_gs<1>(c, nvox, nmeas, params, FixP, st)); break;
    case 2: CDM_TRY(launch_gs<2>(c, nvox, nmeas, params, FixP, st)); break;
    case 4: CDM_TRY(launch_gs<4>(c, nvox, nmeas, params, FixP, st)); break;
    case 8: CDM_TRY(launch_gs<8>(c, nvox, nmeas, params, FixP, st)); break;
    case 16: CDM_TRY(launch_gs<16>(c, nvox, nmeas, params, FixP, st)); break;
    case 32: CDM_TRY(launch_gs<32>(c, nvox, nmeas, params, FixP, st)); break;
    default: return cdm_fail(CDM_BAD_ARG, "bad lane count");
  }
  cdm_gs_recheck_args r;
  r.nvox = nvox;
  r.nmeas = nmeas;
  r.fixp_tsize = CDM_FIXP_TSIZE;
  r.proto64 = c->proto64;
  r.meas = meas;
  r.params = params;
  r.fixp = FixP;
  r.grid = c->grid_dev;
  r.ngp = c->cfg.n_grid_params;
  r.combs = c->cfg.grid_combs;
  for (int p = 0; p < kNP; p++) r.gpos[p] = c->gpos[p];
  r.flags = c->gs_flags;
  r.cand = c->gs_cand;
  r.best = c->gs_best;
  r.rechecked = c->counters + 2;
  r.lim = c->lim;
  cdm_gs_recheck_kernel<<<blocks_for(nvox, 32), CDM_NT, 0, st>>>(r);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

template <int Gw>
cdm_status launch_lm(cdm_ctx* c, int nvox, int nmeas, double* params, const double* FixP,
                     cudaStream_t st) {
  cdm_lm_args a;
  fill_common(c, a, nvox, nmeas, Gw);
  a.params = params;
  a.fixp = FixP;
  a.max_iters = c->cfg.iter_levmar;
  a.marquardt = c->cfg.marquardt;
  a.iter_count = c->counters + 0;
  a.succ_count = c->counters + 1;
  const size_t sm = fit_smem(c->nmeas_pad);
  CDM_TRY(set_smem(cdm_levmar_kernel<Gw>, sm));
  cdm_levmar_kernel<Gw><<<blocks_for(nvox, Gw), CDM_NT, sm, st>>>(a);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status run_levmar(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                      const double* CFP, const double* FixP, cudaStream_t st) {
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  const int Gw = pick_lanes(c, c->cfg.lanes_levmar, 4, nvox);
  CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  if (nvox == 0) return CDM_OK;
  switch (Gw) {
    case 1: return launch_lm<1>(c, nvox, nmeas, params, FixP, st);
    case 2: return launch_lm<2>(c, nvox, nmeas, params, FixP, st);
    case 4: return launch_lm<4>(c, nvox, nmeas, params, FixP, st);
    case 8: return launch_lm<8>(c, nvox, nmeas, params, FixP, st);
    case 16: return launch_lm<16>(c, nvox, nmeas, params, FixP, st);
    case 32: return launch_lm<32>(c, nvox, nmeas, params, FixP, st);
    default: return cdm_fail(CDM_BAD_ARG, "bad lane count");
  }
}

template <int Gw, bool RICIAN>
cdm_status launch_mcmc(cdm_ctx* c, int nvox, int nmeas, double* params, const double* FixP,
                       double* samples, double* tau, uint32_t voxel_offset, cudaStream_t st) {
  cdm_mcmc_args a;
  fill_common(c, a, nvox, nmeas, Gw);
  a.params = params;
  a.fixp = FixP;
  a.samples = samples;
  a.tau_samples = tau;
  a.nburn = c->cfg.nburn;
  a.njumps = c->cfg.njumps;
  a.sampleevery = c->cfg.sampleevery;
  a.nsamples = c->cfg.njumps / c->cfg.sampleevery;
  a.update_proposal = c->cfg.update_proposal;
  a.seed = c->cfg.seed;
  a.stream = (uint32_t)c->cfg.id_part;
  a.voxel_offset = voxel_offset;
  a.prop_sd = c->prop_sd;
  const size_t sm = fit_smem(c->nmeas_pad);
  CDM_TRY(set_smem(cdm_mcmc_kernel<Gw, RICIAN>, sm));
  cdm_mcmc_kernel<Gw, RICIAN><<<blocks_for(nvox, Gw), CDM_NT, sm, st>>>(a);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status run_mcmc(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                    const double* CFP, const double* FixP, double* samples, double* tau,
                    uint32_t voxel_offset, cudaStream_t st) {
  if (c->cfg.sampleevery <= 0 || c->cfg.njumps < c->cfg.sampleevery)
    return cdm_fail(CDM_BAD_ARG,
                    "MCMC must record at least one sample: --nj must be >= --se (MCMC.cu:707-710)");
  if (!samples && nvox > 0) return cdm_fail(CDM_BAD_ARG, "samples is null");
  if (c->cfg.rician && !tau && nvox > 0) return cdm_fail(CDM_BAD_ARG, "rician MCMC needs tau_samples");
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  // measured on NODDI-Watson, 200k voxels, 500 + 500 jumps: 2 lanes 420 ms,
  // 1 lane 443 ms, 4 lanes 469 ms: fewer lanes per voxel repeat the
  // per-proposal work in fewer threads
  const int Gw = pick_lanes(c, c->cfg.lanes_mcmc, 2, nvox);
  CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  if (nvox == 0) return CDM_OK;
  const bool ric = c->cfg.rician != 0;
#define CDM_MCMC_CASE(Gw2)                                                                     \
  case Gw2:                                                                                    \
    return ric ? launch_mcmc<Gw2, true>(c, nvox, nmeas, params, FixP, samples, tau, voxel_offset, st) \
               : launch_mcmc<Gw2, false>(c, nvox, nmeas, params, FixP, samples, tau, voxel_offset, st);
  switch (Gw) {
    CDM_MCMC_CASE(1)
    CDM_MCMC_CASE(2)
    CDM_MCMC_CASE(4)
    CDM_MCMC_CASE(8)
    CDM_MCMC_CASE(16)
    CDM_MCMC_CASE(32)
  }
#undef CDM_MCMC_CASE
  return cdm_fail(CDM_BAD_ARG, "bad lane count");
}

cdm_status run_post(cdm_ctx* c, bool bic, int nvox, int nmeas, int nsamples, const double* meas,
                    const double* samples, const double* CFP, const double* FixP, double* pred,
                    double* BIC, double* AIC, const double* tau, bool rician, cudaStream_t st) {
  if (nsamples <= 0) return cdm_fail(CDM_BAD_ARG, "nsamples must be > 0");
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  if (nvox == 0) return CDM_OK;
  cdm_post_args a;
  a.nvox = nvox;
  a.nmeas = nmeas;
  a.nmeas_pad = c->nmeas_pad;
  a.nsamples = nsamples;
  a.fixp_tsize = CDM_FIXP_TSIZE;
  a.proto_bytes = (uint32_t)proto_bytes(c->nmeas_pad);
  a.proto = c->proto32;
  a.meas = meas;
  a.samples = samples;
  a.tau = tau;
  a.fixp = FixP;
  a.pred = pred;
  a.bic = BIC;
  a.aic = AIC;
  a.rician = rician ? 1 : 0;
  a.err = c->err;
  const size_t sm = proto_bytes(c->nmeas_pad);
  if (bic) {
    CDM_TRY(set_smem(cdm_bic_aic_kernel, sm));
    cdm_bic_aic_kernel<<<blocks_for(nvox, 32), CDM_NT, sm, st>>>(a);
  } else {
    CDM_TRY(set_smem(cdm_predicted_kernel, sm));
    cdm_predicted_kernel<<<blocks_for(nvox, 32), CDM_NT, sm, st>>>(a);
  }
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status fit_sequence(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                        const double* CFP, const double* FixP, double* samples, double* tau,
                        double* pred, double* BIC, double* AIC, uint32_t voxel_offset,
                        cudaStream_t st) {
  const cdm_model_cfg& o = c->cfg;
  if (o.run_gridsearch) CDM_TRY(run_gridsearch(c, nvox, nmeas, meas, params, CFP, FixP, st));
  if (o.run_levmar) CDM_TRY(run_levmar(c, nvox, nmeas, meas, params, CFP, FixP, st));
  int nsamples = 1;
  if (o.run_mcmc) {
    CDM_TRY(run_mcmc(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau, voxel_offset, st));
    nsamples = o.njumps / o.sampleevery;
  } else if (nvox > 0) {
    cdm_params_to_samples_kernel<<<std::max(1, std::min(c->num_sms * 4, (nvox * kNP + 255) / 256)), 256, 0,
                                   st>>>(params, nvox, samples);
    CDM_CUDA(cudaGetLastError());
  }
  const bool rician = o.rician && o.run_mcmc;
  if (o.get_predicted && pred)
    CDM_TRY(run_post(c, false, nvox, nmeas, nsamples, meas, samples, CFP, FixP, pred, nullptr,
                     nullptr, tau, rician, st));
  if (o.bic_aic && BIC && AIC)
    CDM_TRY(run_post(c, true, nvox, nmeas, nsamples, meas, samples, CFP, FixP, nullptr, BIC, AIC,
                     tau, rician, st));
  return CDM_OK;
}

// Allocate every scratch buffer a fit of this shape needs, so that the
// captured graph contains no allocation.
cdm_status reserve_fit(cdm_ctx* c, int nvox, int nmeas) {
  const int pad = round_up(nmeas, 32);
  CDM_TRY(dev_alloc(&c->proto32, &c->proto32_cap, (size_t)kNCOLS4 * pad));
  CDM_TRY(dev_alloc(&c->proto64, &c->proto64_cap, (size_t)kNCOLS * nmeas));
  size_t sig = 0;
  for (int Gw : {1, 2, 4, 8, 16, 32}) sig = std::max(sig, (size_t)((nmeas + Gw - 1) / Gw) * std::max(nvox, 1) * Gw);
  CDM_TRY(dev_alloc(&c->sig, &c->sig_cap, sig));
  const size_t n = (size_t)std::max(nvox, 1);
  CDM_TRY(dev_alloc(&c->gs_flags, &c->gs_flags_cap, n));
  CDM_TRY(dev_alloc(&c->gs_cand, &c->gs_cand_cap, n * kGsTop));
  CDM_TRY(dev_alloc(&c->gs_best, &c->gs_best_cap, n));
  // kernel attributes are set outside capture too
  const size_t sm = fit_smem(pad);
  CDM_TRY(set_smem(cdm_gridsearch_kernel<1>, sm)); CDM_TRY(set_smem(cdm_gridsearch_kernel<2>, sm));
  CDM_TRY(set_smem(cdm_gridsearch_kernel<4>, sm)); CDM_TRY(set_smem(cdm_gridsearch_kernel<8>, sm));
  CDM_TRY(set_smem(cdm_gridsearch_kernel<16>, sm)); CDM_TRY(set_smem(cdm_gridsearch_kernel<32>, sm));
  return CDM_OK;
}

// dMRI_Data::remove_NonPositive_entries (dMRI_Data.cu:15-30), which CUDIMOT
// applies to every voxel's signals when --rician is set (dMRI_Data.cu:133),
// so that log(S) in the Rician likelihood stays finite. If the smallest
// value is non-positive and the largest positive (both read as float, as
// the reference's MinS/MaxS), every entry that is non-positive as a float
// takes the smallest remaining value, min(smallest positive entry,
// float(largest)), rounded to float. One warp per voxel.
__global__ void cdm_clean_signals_kernel(int nvox, int nmeas, double* __restrict__ meas) {
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
__global__ void cdm_wait_selftest_kernel(uint64_t limit_ns, int* err) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t sbar = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sbar), "r"(1) : "memory");
  __syncthreads();
  cdm_mbar_wait_phase0(sbar, limit_ns, threadIdx.x == 0 ? err : nullptr);
}

}  // namespace

// cdm_selftest_wait_timeout without a context: the no-allocation error word
// (defined with that word, at the end of this file).
static cdm_status noalloc_selftest(int limit_ms, cudaStream_t st);

// =================================================================== C ABI
extern "C" {

cdm_status cdm_get_model_info(cdm_model_info* info) {
  if (!info) return cdm_fail(CDM_BAD_ARG, "null info");
  std::memset(info, 0, sizeof(*info));
  std::snprintf(info->name, sizeof(info->name), "%s", CDM_MODEL_NAME);
  info->nparams = NPARAMS;
  info->ncfp = NCFP;
  info->nfixp = NFIXP;
  for (int i = 0; i < NCFP && i < CDM_MAX_BLOCKS; i++) info->cfp_size[i] = MODEL::CFP_size[i];
  for (int i = 0; i < NFIXP && i < CDM_MAX_BLOCKS; i++) info->fixp_size[i] = MODEL::FixP_size[i];
  info->cfp_tsize = CDM_CFP_TSIZE;
  info->fixp_tsize = CDM_FIXP_TSIZE;
  info->derived_cfp = CDM_NDCFP;
  info->derived_p = CDM_NDP;
  return CDM_OK;
}

cdm_status cdm_default_cfg(cdm_model_cfg* cfg) {
  if (!cfg) return cdm_fail(CDM_BAD_ARG, "null cfg");
  cdm_fill_default_cfg(cfg, NPARAMS);
  return CDM_OK;
}

cdm_status cdm_parse_priors(const char* path, cdm_model_cfg* cfg, double* p_init, int* p_init_given) {
  return cdm_parse_priors_impl(path, NPARAMS, cfg, p_init, p_init_given);
}

cdm_status cdm_parse_grid(const char* path, int* n_grid_params, int* grid_params, int* grid_combs,
                          double* grid, int64_t grid_capacity) {
  return cdm_parse_grid_impl(path, NPARAMS, n_grid_params, grid_params, grid_combs, grid,
                             grid_capacity);
}

cdm_status cdm_parse_fixed(const char* list, int* fixed) {
  return cdm_parse_fixed_impl(list, NPARAMS, fixed);
}

cdm_status cdm_read_cfp_list(const char* path, int nmeas, double* cfp) {
  std::vector<int> sizes(MODEL::CFP_size, MODEL::CFP_size + NCFP);
  return cdm_read_cfp_list_impl(path, nmeas, sizes, cfp);
}

cdm_status cdm_create(const cdm_model_cfg* cfg, cdm_ctx** out) {
  if (!cfg || !out) return cdm_fail(CDM_BAD_ARG, "null argument");
  *out = nullptr;
  if (cfg->nparams != NPARAMS)
    return cdm_fail(CDM_BAD_ARG, "cfg.nparams " + std::to_string(cfg->nparams) +
                                     " != model NPARAMS " + std::to_string(NPARAMS));
  CDM_TRY(cdm_validate_cfg(cfg, NPARAMS));
  cdm_ctx* c = new cdm_ctx();
  c->cfg = *cfg;
  c->cfg.grid = nullptr;
  for (int p = 0; p < kNP; p++) {
    c->lim.btype[p] = cfg->bound_types[p];
    c->lim.bmin[p] = (float)cfg->bounds_min[p];
    c->lim.bmax[p] = (float)cfg->bounds_max[p];
    c->lim.ptype[p] = cfg->prior_types[p];
    c->lim.pa[p] = (float)cfg->priors_a[p];
    c->lim.pb[p] = (float)cfg->priors_b[p];
    c->lim.fixed[p] = cfg->fixed[p];
    c->gpos[p] = -1;
  }
  if (cfg->run_gridsearch && cfg->grid_combs > 0 && cfg->n_grid_params > 0) {
    const size_t n = (size_t)cfg->grid_combs * cfg->n_grid_params;
    c->grid_host.assign(cfg->grid, cfg->grid + n);
    for (int i = 0; i < cfg->n_grid_params; i++) c->gpos[cfg->grid_params[i]] = i;
  } else {
    c->cfg.run_gridsearch = 0;
  }
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (e != cudaSuccess) {
    delete c;
    return cdm_fail(CDM_CUDA_ERROR, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
  }
  cdm_status s = ensure_base(c);
  if (s == CDM_OK && !c->grid_host.empty()) {
    s = dev_alloc(&c->grid_dev, &c->grid_cap, c->grid_host.size());
    if (s == CDM_OK) {
      e = cudaMemcpy(c->grid_dev, c->grid_host.data(), c->grid_host.size() * sizeof(double),
                     cudaMemcpyHostToDevice);
      if (e != cudaSuccess) s = cdm_fail(CDM_CUDA_ERROR, cudaGetErrorString(e));
    }
  }
  if (s != CDM_OK) {
    cdm_destroy(c);
    return s;
  }
  *out = c;
  return CDM_OK;
}

cdm_status cdm_destroy(cdm_ctx* c) {
  if (!c) return CDM_OK;
  if (c->graph) cudaGraphExecDestroy(c->graph);
  void* bufs[] = {c->grid_dev, c->proto32, c->proto64, c->sig, c->gs_flags, c->gs_cand,
                  c->gs_best, c->err, c->counters, c->h_meas, c->h_params, c->h_cfp, c->h_fixp,
                  c->h_samples, c->h_tau, c->h_pred, c->h_bic, c->h_aic};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return CDM_OK;
}

cdm_status cdm_gridsearch(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size,
                          const double* meas, double* params, const double* CFP, const double* FixP,
                          void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  if (!c->cfg.run_gridsearch) return cdm_fail(CDM_BAD_ARG, "context has no grid");
  return run_gridsearch(c, nvox, nmeas, meas, params, CFP, FixP, (cudaStream_t)stream);
}

cdm_status cdm_levmar(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size,
                      const double* meas, double* params, const double* CFP, const double* FixP,
                      void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  return run_levmar(c, nvox, nmeas, meas, params, CFP, FixP, (cudaStream_t)stream);
}

cdm_status cdm_mcmc(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size,
                    const double* meas, double* params, const double* CFP, const double* FixP,
                    double* samples, double* tau_samples, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  return run_mcmc(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau_samples, 0,
                  (cudaStream_t)stream);
}

cdm_status cdm_mcmc_seeded(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size,
                           const double* meas, double* params, const double* CFP,
                           const double* FixP, double* samples, double* tau_samples,
                           const double* prop_sd, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  c->prop_sd = prop_sd;
  const cdm_status s = run_mcmc(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau_samples, 0,
                                (cudaStream_t)stream);
  c->prop_sd = nullptr;
  return s;
}

cdm_status cdm_synth_signals(cdm_ctx* c, int nvox, int nmeas, const double* CFP,
                             const double* params, const double* FixP, double snr_lo,
                             double snr_hi, uint64_t seed, int b_col, double* meas,
                             double* s0_est, void* x, int x_ld, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!CFP || !params || (CDM_FIXP_TSIZE > 0 && !FixP)) return cdm_fail(CDM_BAD_ARG, "null array");
  if (b_col >= kNCOLS) return cdm_fail(CDM_BAD_ARG, "b_col beyond the protocol columns");
  if (x && x_ld < nmeas) return cdm_fail(CDM_BAD_ARG, "x_ld < nmeas");
  if (!(snr_lo > 0.0) || snr_hi < snr_lo) return cdm_fail(CDM_BAD_ARG, "bad SNR range");
  cudaStream_t st = (cudaStream_t)stream;
  CDM_TRY(reserve_fit(c, std::max(nvox, 1), nmeas));
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  if (nvox == 0) return CDM_OK;
  cdm_synth_args a;
  a.nvox = nvox;
  a.nmeas = nmeas;
  a.nmeas_pad = c->nmeas_pad;
  a.fixp_tsize = CDM_FIXP_TSIZE;
  a.b_col = b_col;
  a.x_ld = x_ld;
  a.proto_bytes = (uint32_t)proto_bytes(c->nmeas_pad);
  a.proto = c->proto32;
  a.params = params;
  a.fixp = FixP;
  a.snr_lo = (float)snr_lo;
  a.snr_hi = (float)snr_hi;
  a.seed = seed;
  a.meas = meas;
  a.s0_est = s0_est;
  a.x = (__nv_bfloat16*)x;
  a.err = c->err;
  const size_t sm = proto_bytes(c->nmeas_pad);
  CDM_TRY(set_smem(cdm_synth_kernel, sm));
  cdm_synth_kernel<<<(nvox + CDM_NT / 32 - 1) / (CDM_NT / 32), CDM_NT, sm, st>>>(a);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_cost(cdm_ctx* c, int nvox, int nmeas, const double* meas, const double* params,
                    const double* CFP, const double* FixP, double* cost, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!meas || !params || !CFP || !cost || (CDM_FIXP_TSIZE > 0 && !FixP))
    return cdm_fail(CDM_BAD_ARG, "null array");
  cudaStream_t st = (cudaStream_t)stream;
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  if (nvox == 0) return CDM_OK;
  cdm_post_args a;
  std::memset(&a, 0, sizeof(a));
  a.nvox = nvox;
  a.nmeas = nmeas;
  a.nmeas_pad = c->nmeas_pad;
  a.nsamples = 1;
  a.fixp_tsize = CDM_FIXP_TSIZE;
  a.proto_bytes = (uint32_t)proto_bytes(c->nmeas_pad);
  a.proto = c->proto32;
  a.meas = meas;
  a.fixp = FixP;
  a.err = c->err;
  const size_t sm = proto_bytes(c->nmeas_pad);
  CDM_TRY(set_smem(cdm_cost_kernel, sm));
  cdm_cost_kernel<<<blocks_for(nvox, 32), CDM_NT, sm, st>>>(a, params, cost);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_select_worse(int n, const double* cost, const double* ref, double margin, int* idx,
                            int* count, void* stream) {
  if (n < 0 || !cost || !ref || !idx || !count) return cdm_fail(CDM_BAD_ARG, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  CDM_CUDA(cudaMemsetAsync(count, 0, sizeof(int), st));
  if (n == 0) return CDM_OK;
  cdm_select_worse_kernel<<<std::min((n + 255) / 256, 152 * 8), 256, 0, st>>>(n, cost, ref, margin,
                                                                             idx, count);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_rows(int nsel, const int* idx, int ncols, const double* src, double* dst, int mode,
                    double value, void* stream) {
  if (nsel < 0 || ncols <= 0 || !idx || !dst || mode < 0 || mode > 2 || (mode < 2 && !src))
    return cdm_fail(CDM_BAD_ARG, "bad argument");
  if (nsel == 0) return CDM_OK;
  const size_t total = (size_t)nsel * ncols;
  cdm_rows_kernel<<<(int)std::min<size_t>((total + 255) / 256, 152 * 8), 256, 0,
                    (cudaStream_t)stream>>>(nsel, idx, ncols, mode == 2 ? nullptr : src, dst,
                                            mode == 1, value);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_mlp_head_info(int* n_mu, int* n_sig, int* group) {
#ifdef CDM_MLP_HEAD
  const int g[CDM_MLP_NMU] = CDM_MLP_GROUPS;
  if (n_mu) *n_mu = CDM_MLP_NMU;
  if (n_sig) *n_sig = CDM_MLP_NSIG;
  if (group)
    for (int j = 0; j < CDM_MLP_NMU; j++) group[j] = g[j];
  return CDM_OK;
#else
  (void)n_mu; (void)n_sig; (void)group;
  return cdm_fail(CDM_NOT_SUPPORTED, "this plugin defines no learned-initialiser head");
#endif
}

cdm_status cdm_mlp_targets(cdm_ctx* c, int n, const double* params, float* targets, void* stream) {
#ifdef CDM_MLP_HEAD
  if (!c || n < 0 || !params || !targets) return cdm_fail(CDM_BAD_ARG, "bad argument");
  if (n == 0) return CDM_OK;
  cdm_mlp_encode_kernel<<<std::min((n + 255) / 256, 152 * 8), 256, 0, (cudaStream_t)stream>>>(
      params, n, targets);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
#else
  (void)c; (void)n; (void)params; (void)targets; (void)stream;
  return cdm_fail(CDM_NOT_SUPPORTED, "this plugin defines no learned-initialiser head");
#endif
}

cdm_status cdm_mlp_decode(cdm_ctx* c, int n, const float* out, int ld, double* params,
                          double* prop_sd, void* stream) {
#ifdef CDM_MLP_HEAD
  if (!c || n < 0 || !out || !params || ld < CDM_MLP_NMU + CDM_MLP_NSIG)
    return cdm_fail(CDM_BAD_ARG, "bad argument");
  if (n == 0) return CDM_OK;
  cdm_mlp_decode_kernel<<<std::min((n + 255) / 256, 152 * 8), 256, 0, (cudaStream_t)stream>>>(
      out, ld, n, params, prop_sd);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
#else
  (void)c; (void)n; (void)out; (void)ld; (void)params; (void)prop_sd; (void)stream;
  return cdm_fail(CDM_NOT_SUPPORTED, "this plugin defines no learned-initialiser head");
#endif
}

cdm_status cdm_bic_aic(cdm_ctx* c, int nvox, int nmeas, int nsamples, int CFP_size, int FixP_size,
                       const double* meas, const double* samples, const double* CFP,
                       const double* FixP, double* BIC, double* AIC, const double* tau_samples,
                       void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  // Rician BIC only after a Rician MCMC (BIC_AIC.cu:208).
  const bool rician = c->cfg.rician && c->cfg.run_mcmc && tau_samples;
  return run_post(c, true, nvox, nmeas, nsamples, meas, samples, CFP, FixP, nullptr, BIC, AIC,
                  tau_samples, rician, (cudaStream_t)stream);
}

cdm_status cdm_predicted_signal(cdm_ctx* c, int nvox, int nmeas, int nsamples, int CFP_size,
                                int FixP_size, const double* samples, const double* CFP,
                                const double* FixP, double* pred, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  return run_post(c, false, nvox, nmeas, nsamples, nullptr, samples, CFP, FixP, pred, nullptr,
                  nullptr, nullptr, false, (cudaStream_t)stream);
}

cdm_status cdm_fit(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                   const double* CFP, const double* FixP, double* samples, double* tau,
                   double* pred, double* BIC, double* AIC, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!samples && nvox > 0) return cdm_fail(CDM_BAD_ARG, "samples is null");
  if (c->cfg.run_mcmc && (c->cfg.sampleevery <= 0 || c->cfg.njumps < c->cfg.sampleevery))
    return cdm_fail(CDM_BAD_ARG, "MCMC must record at least one sample: --nj must be >= --se");
  if (c->cfg.run_mcmc && c->cfg.rician && !tau && nvox > 0) return cdm_fail(CDM_BAD_ARG, "rician needs tau");
  cudaStream_t st = (cudaStream_t)stream;
  if (nvox == 0) return CDM_OK;
  CDM_TRY(reserve_fit(c, nvox, nmeas));
  const std::vector<uintptr_t> key = {(uintptr_t)nvox, (uintptr_t)nmeas, (uintptr_t)meas,
                                      (uintptr_t)params, (uintptr_t)CFP, (uintptr_t)FixP,
                                      (uintptr_t)samples, (uintptr_t)tau, (uintptr_t)pred,
                                      (uintptr_t)BIC, (uintptr_t)AIC, (uintptr_t)st};
  if (!c->graph || key != c->graph_key) {
    if (c->graph) {
      cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
    }
    // The legacy default stream cannot be captured; record on a private one.
    cudaStream_t cap = st;
    if (cap == nullptr || cap == cudaStreamLegacy || cap == cudaStreamPerThread) {
      if (!c->own_stream) CDM_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
      cap = c->own_stream;
    }
    CDM_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    cdm_status s = fit_sequence(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau, pred, BIC,
                                AIC, 0, cap);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    if (s != CDM_OK) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    if (e != cudaSuccess) return cdm_fail(CDM_CUDA_ERROR, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      c->graph = nullptr;
      return cdm_fail(CDM_CUDA_ERROR, std::string("instantiate: ") + cudaGetErrorString(e));
    }
    c->graph_key = key;
  }
  CDM_CUDA(cudaMemsetAsync(c->counters, 0, 4 * sizeof(unsigned long long), st));
  CDM_CUDA(cudaGraphLaunch(c->graph, st));
  return CDM_OK;
}

cdm_status cdm_fit_reserve(cdm_ctx* c, int nvox, int nmeas) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  return reserve_fit(c, nvox, nmeas);
}

cdm_status cdm_fit_enqueue(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                           const double* CFP, const double* FixP, double* samples, double* tau,
                           double* pred, double* BIC, double* AIC, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!samples && nvox > 0) return cdm_fail(CDM_BAD_ARG, "samples is null");
  if (c->cfg.run_mcmc && (c->cfg.sampleevery <= 0 || c->cfg.njumps < c->cfg.sampleevery))
    return cdm_fail(CDM_BAD_ARG, "MCMC must record at least one sample: --nj must be >= --se");
  if (c->cfg.run_mcmc && c->cfg.rician && !tau && nvox > 0) return cdm_fail(CDM_BAD_ARG, "rician needs tau");
  if (nvox == 0) return CDM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CDM_CUDA(cudaStreamIsCapturing(st, &cs));
  if (cs == cudaStreamCaptureStatusActive) {
    // no allocation may happen under capture: the shape must be reserved
    const int pad = round_up(nmeas, 32);
    size_t sig = 0;
    for (int Gw : {1, 2, 4, 8, 16, 32})
      sig = std::max(sig, (size_t)((nmeas + Gw - 1) / Gw) * std::max(nvox, 1) * Gw);
    if (c->proto32_cap < (size_t)kNCOLS4 * pad || c->sig_cap < sig ||
        c->gs_flags_cap < (size_t)std::max(nvox, 1))
      return cdm_fail(CDM_BAD_ARG, "cdm_fit_enqueue under stream capture needs cdm_fit_reserve "
                                   "for this shape first");
  } else {
    CDM_TRY(reserve_fit(c, nvox, nmeas));
  }
  CDM_CUDA(cudaMemsetAsync(c->counters, 0, 4 * sizeof(unsigned long long), st));
  return fit_sequence(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau, pred, BIC, AIC, 0,
                      st);
}

cdm_status cdm_synchronize(cdm_ctx* c, void* stream, int64_t timeout_ms) {
  if (!c) return cdm_fail(CDM_BAD_ARG, "null context");
  cudaStream_t st = (cudaStream_t)stream;
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(st);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return cdm_fail(CDM_CUDA_ERROR, cudaGetErrorString(e));
    if (timeout_ms >= 0 &&
        std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0)
                .count() > timeout_ms)
      return cdm_fail(CDM_TIMEOUT, "stream did not finish within the time limit");
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  int err = 0;
  CDM_CUDA(cudaMemcpy(&err, c->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    const cudaError_t ce = cudaMemset(c->err, 0, sizeof(int));
    if (ce != cudaSuccess)
      return cdm_fail(CDM_CUDA_ERROR, std::string("clearing the device error word: ") +
                                          cudaGetErrorString(ce));
    return cdm_fail(CDM_TIMEOUT, "a bounded device wait ran out (code " + std::to_string(err) + ")");
  }
  return CDM_OK;
}

cdm_status cdm_get_stats(cdm_ctx* c, cdm_stats* s) {
  if (!c || !s) return cdm_fail(CDM_BAD_ARG, "null argument");
  unsigned long long h[4] = {0, 0, 0, 0};
  CDM_CUDA(cudaMemcpy(h, c->counters, sizeof(h), cudaMemcpyDeviceToHost));
  s->lm_iterations = (int64_t)h[0];
  s->lm_successes = (int64_t)h[1];
  s->gs_recheck_voxels = (int64_t)h[2];
  int err = 0;
  CDM_CUDA(cudaMemcpy(&err, c->err, sizeof(int), cudaMemcpyDeviceToHost));
  s->device_errors = err;
  return CDM_OK;
}

cdm_status cdm_selftest_wait_timeout(cdm_ctx* c, int limit_ms, void* stream) {
  if (limit_ms < 1 || limit_ms > 2000) return cdm_fail(CDM_BAD_ARG, "limit_ms must be in 1..2000");
  if (!c) return noalloc_selftest(limit_ms, (cudaStream_t)stream);
  CDM_TRY(ensure_base(c));
  cdm_wait_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((uint64_t)limit_ms * 1000000ull, c->err);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_clean_signals(int nvox, int nmeas, double* meas, void* stream) {
  if (nvox < 0 || nmeas <= 0 || (nvox > 0 && !meas)) return cdm_fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  const size_t threads = (size_t)nvox * 32;
  cdm_clean_signals_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      nvox, nmeas, meas);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_fit_host(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                        const double* CFP, const double* FixP, double* samples, double* tau,
                        double* pred, double* BIC, double* AIC, int part_size, int64_t timeout_ms) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!meas || !params || !CFP || !samples || (CDM_FIXP_TSIZE > 0 && !FixP))
    return cdm_fail(CDM_BAD_ARG, "null array");
  (void)part_size;  // CUDIMOT's SIZE_PART parts (dMRI_Data.cu:66-79): one part here
  const cdm_model_cfg& o = c->cfg;
  const int ns = o.run_mcmc ? o.njumps / std::max(o.sampleevery, 1) : 1;
  const size_t nv = (size_t)nvox;
  CDM_TRY(dev_alloc(&c->h_meas, &c->h_meas_cap, nv * nmeas));
  CDM_TRY(dev_alloc(&c->h_params, &c->h_params_cap, nv * kNP));
  CDM_TRY(dev_alloc(&c->h_cfp, &c->h_cfp_cap, (size_t)nmeas * CDM_CFP_TSIZE));
  CDM_TRY(dev_alloc(&c->h_fixp, &c->h_fixp_cap, std::max<size_t>(1, nv * CDM_FIXP_TSIZE)));
  CDM_TRY(dev_alloc(&c->h_samples, &c->h_samples_cap, nv * kNP * ns));
  const bool want_tau = o.run_mcmc && o.rician && tau;
  const bool want_pred = o.get_predicted && pred;
  const bool want_bic = o.bic_aic && BIC && AIC;
  if (want_tau) CDM_TRY(dev_alloc(&c->h_tau, &c->h_tau_cap, nv * ns));
  if (want_pred) CDM_TRY(dev_alloc(&c->h_pred, &c->h_pred_cap, nv * nmeas));
  if (want_bic) {
    CDM_TRY(dev_alloc(&c->h_bic, &c->h_bic_cap, nv));
    CDM_TRY(dev_alloc(&c->h_aic, &c->h_aic_cap, nv));
  }
  if (!c->own_stream) CDM_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
  cudaStream_t st = c->own_stream;
  CDM_CUDA(cudaMemcpyAsync(c->h_meas, meas, nv * nmeas * sizeof(double), cudaMemcpyHostToDevice, st));
  CDM_CUDA(cudaMemcpyAsync(c->h_params, params, nv * kNP * sizeof(double), cudaMemcpyHostToDevice, st));
  CDM_CUDA(cudaMemcpyAsync(c->h_cfp, CFP, (size_t)nmeas * CDM_CFP_TSIZE * sizeof(double),
                           cudaMemcpyHostToDevice, st));
  if (CDM_FIXP_TSIZE > 0)
    CDM_CUDA(cudaMemcpyAsync(c->h_fixp, FixP, nv * CDM_FIXP_TSIZE * sizeof(double),
                             cudaMemcpyHostToDevice, st));
  if (o.rician) CDM_TRY(cdm_clean_signals(nvox, nmeas, c->h_meas, st));  // dMRI_Data.cu:133
  CDM_TRY(cdm_fit(c, nvox, nmeas, c->h_meas, c->h_params, c->h_cfp, c->h_fixp, c->h_samples,
                  want_tau ? c->h_tau : nullptr, want_pred ? c->h_pred : nullptr,
                  want_bic ? c->h_bic : nullptr, want_bic ? c->h_aic : nullptr, st));
  CDM_CUDA(cudaMemcpyAsync(params, c->h_params, nv * kNP * sizeof(double), cudaMemcpyDeviceToHost, st));
  CDM_CUDA(cudaMemcpyAsync(samples, c->h_samples, nv * kNP * ns * sizeof(double),
                           cudaMemcpyDeviceToHost, st));
  if (want_tau)
    CDM_CUDA(cudaMemcpyAsync(tau, c->h_tau, nv * ns * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (want_pred)
    CDM_CUDA(cudaMemcpyAsync(pred, c->h_pred, nv * nmeas * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (want_bic) {
    CDM_CUDA(cudaMemcpyAsync(BIC, c->h_bic, nv * sizeof(double), cudaMemcpyDeviceToHost, st));
    CDM_CUDA(cudaMemcpyAsync(AIC, c->h_aic, nv * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  return cdm_synchronize(c, st, timeout_ms);
}

}  // extern "C"

// ============================================================ no-allocation
// Levenberg-Marquardt for callers that may not allocate device memory.
//
// Some hosts cannot let a library call cudaMalloc: a real-time acquisition
// or reconstruction pipeline that has reserved its whole device memory
// budget up front, or a framework that owns all device memory through its
// own pool and hands this library only its input and output buffers.
// cudaMalloc/cudaFree can also synchronise the whole device, which such
// hosts must avoid in the middle of a pipeline. cdm_levmar_noalloc takes
// no context (cdm_create allocates) and keeps its working memory - the
// staged protocol table, the lane-packed signals and the device error word
// - in the fixed array below, which every GPU that loads this library holds
// until the process exits.
namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB
constexpr size_t kNoAllocHeader = 256;               // device error word

static __device__ __align__(256) unsigned char cdm_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mutex;

// Device address of the scratch array for the current device. The first
// call on a device resolves it with cudaGetSymbolAddress while that device
// is current and clears the error word (a synchronous cudaMemset, which
// allocates nothing); later calls reuse the cached address. After that the
// error word is cleared only by cdm_noalloc_status, so a wait that ran out
// in any call stays visible until the caller asks.
cdm_status noalloc_scratch(unsigned char** out) {
  int dev = 0;
  CDM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return cdm_fail(CDM_NOT_SUPPORTED, "device index beyond the no-allocation table");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    CDM_CUDA(cudaGetSymbolAddress(&p, cdm_noalloc_scratch));
    CDM_CUDA(cudaMemset(p, 0, kNoAllocHeader));
    g_noalloc_ptr[dev] = (unsigned char*)p;
  }
  *out = g_noalloc_ptr[dev];
  return CDM_OK;
}

template <int Gw>
cdm_status noalloc_lm_launch(const cdm_model_cfg* cfg, unsigned char* scratch, int sms, int nvox,
                             int nmeas, const double* meas, double* params, const double* CFP,
                             const double* FixP, cudaStream_t st) {
  const int pad = round_up(nmeas, 32);
  const int nchunk = (nmeas + Gw - 1) / Gw;
  const size_t pbytes = proto_bytes(pad);
  const size_t sbytes = (size_t)nchunk * nvox * Gw * sizeof(float);
  const size_t soff = kNoAllocHeader + (pbytes + 255) / 256 * 256;
  if (soff + sbytes > kNoAllocScratchBytes)
    return cdm_fail(CDM_BAD_ARG,
                    "cdm_levmar_noalloc: " + std::to_string(nvox) + " voxels x " +
                        std::to_string(nmeas) + " measurements need " +
                        std::to_string(soff + sbytes) + " bytes of scratch; the fixed scratch holds " +
                        std::to_string(kNoAllocScratchBytes) + " bytes (split the voxels into parts)");
  int* err = (int*)scratch;
  float* proto = (float*)(scratch + kNoAllocHeader);
  float* sig = (float*)(scratch + soff);
  // The error word accumulates with atomicOr across calls (cleared at
  // set-up and by cdm_noalloc_status); the protocol table and the signals
  // are fully rewritten by every call.
  cdm_prep_protocol_kernel<<<(pad + 127) / 128, 128, 0, st>>>(CFP, nmeas, pad, proto, nullptr);
  CDM_CUDA(cudaGetLastError());
  if (nvox == 0) return CDM_OK;
  const size_t total = (size_t)nchunk * nvox * Gw;
  cdm_pack_signals_kernel<Gw><<<(int)std::min<size_t>((total + 255) / 256, (size_t)std::max(sms, 1) * 32),
                               256, 0, st>>>(meas, nvox, nmeas, nchunk, sig);
  CDM_CUDA(cudaGetLastError());
  cdm_lm_args a;
  a.nvox = nvox;
  a.nmeas = nmeas;
  a.nmeas_pad = pad;
  a.nchunk = nchunk;
  a.fixp_tsize = CDM_FIXP_TSIZE;
  a.proto_bytes = (uint32_t)pbytes;
  a.proto = proto;
  a.sig = sig;
  a.params = params;
  a.fixp = FixP;
  a.max_iters = cfg->iter_levmar;
  a.marquardt = cfg->marquardt;
  a.err = err;
  a.iter_count = nullptr;
  a.succ_count = nullptr;
  for (int p = 0; p < kNP; p++) {
    a.lim.btype[p] = cfg->bound_types[p];
    a.lim.bmin[p] = (float)cfg->bounds_min[p];
    a.lim.bmax[p] = (float)cfg->bounds_max[p];
    a.lim.ptype[p] = cfg->prior_types[p];
    a.lim.pa[p] = (float)cfg->priors_a[p];
    a.lim.pb[p] = (float)cfg->priors_b[p];
    a.lim.fixed[p] = cfg->fixed[p];
  }
  CDM_TRY(set_smem(cdm_levmar_kernel<Gw>, fit_smem(pad)));
  cdm_levmar_kernel<Gw><<<blocks_for(nvox, Gw), CDM_NT, fit_smem(pad), st>>>(a);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}

}  // namespace

extern "C" cdm_status cdm_levmar_noalloc(const cdm_model_cfg* cfg, int nvox, int nmeas,
                                         int CFP_size, int FixP_size, const double* meas,
                                         double* params, const double* CFP, const double* FixP,
                                         void* stream) {
  if (!cfg) return cdm_fail(CDM_BAD_ARG, "null cfg");
  if (cfg->nparams != NPARAMS) return cdm_fail(CDM_BAD_ARG, "cfg.nparams != model NPARAMS");
  CDM_TRY(cdm_validate_cfg(cfg, NPARAMS));
  if (nvox < 0 || nmeas <= 0) return cdm_fail(CDM_BAD_ARG, "nvox must be >= 0 and nmeas > 0");
  if (CFP_size != CDM_CFP_TSIZE || FixP_size != CDM_FIXP_TSIZE)
    return cdm_fail(CDM_BAD_ARG, "CFP_size/FixP_size do not match the model");
  // the shared-memory bound of every other entry point (check_common)
  if (fit_smem(round_up(nmeas, 32)) > 200 * 1024)
    return cdm_fail(CDM_BAD_ARG, "protocol too large for shared memory staging");
  unsigned char* scratch = nullptr;
  CDM_TRY(noalloc_scratch(&scratch));
  int dev = 0, sms = 0;
  CDM_CUDA(cudaGetDevice(&dev));
  CDM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // lanes per voxel: cdm_levmar's rule (pick_lanes), on this device's SM count
  int Gw = cfg->lanes_levmar;
  if (Gw == 0) {
    const long resident = (long)std::max(sms, 1) * 512;
    Gw = 4;
    while (Gw < 32 && (long)nvox * Gw < 4 * resident) Gw *= 2;
  }
  cudaStream_t st = (cudaStream_t)stream;
  switch (Gw) {
    case 1: return noalloc_lm_launch<1>(cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP, st);
    case 2: return noalloc_lm_launch<2>(cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP, st);
    case 4: return noalloc_lm_launch<4>(cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP, st);
    case 8: return noalloc_lm_launch<8>(cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP, st);
    case 16: return noalloc_lm_launch<16>(cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP, st);
    case 32: return noalloc_lm_launch<32>(cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP, st);
  }
  return cdm_fail(CDM_BAD_ARG, "lanes_levmar must be 0, 1, 2, 4, 8, 16 or 32");
}

// Reads and clears the no-allocation error word of the current device after
// the caller's stream has finished: CDM_TIMEOUT if a bounded wait of any
// cdm_levmar_noalloc call (or of cdm_selftest_wait_timeout with no context)
// ran out since the last check. Waiting, the 4-byte read and the clear
// allocate nothing.
extern "C" cdm_status cdm_noalloc_status(void* stream) {
  unsigned char* scratch = nullptr;
  CDM_TRY(noalloc_scratch(&scratch));
  CDM_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  int err = 0;
  CDM_CUDA(cudaMemcpy(&err, scratch, sizeof(int), cudaMemcpyDeviceToHost));
  if (!err) return CDM_OK;
  CDM_CUDA(cudaMemset(scratch, 0, sizeof(int)));
  return cdm_fail(CDM_TIMEOUT, "a bounded device wait of a no-allocation call ran out (code " +
                                   std::to_string(err) + ")");
}

// cdm_selftest_wait_timeout with a null context records into the
// no-allocation error word.
static cdm_status noalloc_selftest(int limit_ms, cudaStream_t st) {
  unsigned char* scratch = nullptr;
  CDM_TRY(noalloc_scratch(&scratch));
  cdm_wait_selftest_kernel<<<1, 32, 0, st>>>((uint64_t)limit_ms * 1000000ull, (int*)scratch);
  CDM_CUDA(cudaGetLastError());
  return CDM_OK;
}
