// oracle_capi.cpp - extern "C" entry points of the CPU oracle, built once
// per model plugin (oracle/build_oracle.py). TEST INFRASTRUCTURE ONLY: the
// tests, smoke() and bench.py's CPU baseline load it through ctypes to
// check and time the GPU library.
//
// Arguments use CUDIMOT's layouts (see include/cudimot_gb300.h). `prec`
// selects the evaluation type: 0 = double (the FP64 oracle), 1 = fp32 (the
// single-precision type the GPU kernels use), for measuring FP32 error on
// the host. Voxels are independent and are spread over OpenMP threads.
#include "host_prelude.h"
#include "modelparameters.h"
#include "macro_numerical.h"
#include "modelfunctions.h"
#include "cdm_plugin_tail.h"
#include "modelparameters.cc"
#include "cudimot_oracle.hpp"

#include <omp.h>
#include <cstdio>
#include <cstring>

#ifndef CDM_MODEL_NAME
#define CDM_MODEL_NAME "model"
#endif

namespace {

int cfp_tsize() {
  int t = 0;
  for (int i = 0; i < NCFP; i++) t += MODEL::CFP_size[i];
  return t;
}
int fixp_tsize() {
  int t = 0;
  for (int i = 0; i < NFIXP; i++) t += MODEL::FixP_size[i];
  return t;
}
void set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

template <typename T>
int signal_impl(int nvox, int nmeas, const double* params, const double* cfp, const double* fixp,
                double* S, double* J) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const int ft = fixp_tsize();
#pragma omp parallel
  {
    orc::Voxel<T> v;
    std::vector<double> zero(nmeas, 0.0);
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, zero.data(), fixp + (size_t)i * ft, ft);
      T P[orc::NPS];
      for (int k = 0; k < orc::NPS; k++) P[k] = (k < NPARAMS) ? (T)params[(size_t)i * NPARAMS + k] : (T)0.0;
      cdm_update_derived(P, v.fixp);
      for (int m = 0; m < nmeas; m++) {
        T* cf = &v.cfp[(size_t)m * v.stride];
        S[(size_t)i * nmeas + m] = (double)Predicted_Signal(NPARAMS, P, cf, v.fixp);
        if (J) {
          T d[NPARAMS];
          Partial_Derivatives(NPARAMS, P, cf, v.fixp, d);
          for (int p = 0; p < NPARAMS; p++) J[((size_t)i * nmeas + m) * NPARAMS + p] = (double)d[p];
        }
      }
    }
  }
  return 0;
}

template <typename T>
int cost_impl(int nvox, int nmeas, const double* meas, const double* params, const double* cfp,
              const double* fixp, double* out) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const int ft = fixp_tsize();
#pragma omp parallel
  {
    orc::Voxel<T> v;
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, meas + (size_t)i * nmeas, fixp + (size_t)i * ft, ft);
      T P[orc::NPS];
      for (int k = 0; k < orc::NPS; k++) P[k] = (k < NPARAMS) ? (T)params[(size_t)i * NPARAMS + k] : (T)0.0;
      cdm_update_derived(P, v.fixp);
      out[i] = orc::cost(v, P);
    }
  }
  return 0;
}

template <typename T>
int gs_impl(const cdm_model_cfg* cfg, int nvox, int nmeas, const double* meas, double* params,
            const double* cfp, const double* fixp, int* best_index, double* best_cost) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const orc::Limits L = orc::make_limits(*cfg);
  const int ft = fixp_tsize();
#pragma omp parallel
  {
    orc::Voxel<T> v;
#pragma omp for schedule(dynamic, 4)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, meas + (size_t)i * nmeas, fixp + (size_t)i * ft, ft);
      double bc = 0.0;
      const int b = orc::gridsearch_voxel(L, cfg->n_grid_params, cfg->grid_params, cfg->grid_combs,
                                          cfg->grid, v, params + (size_t)i * NPARAMS, &bc);
      if (best_index) best_index[i] = b;
      if (best_cost) best_cost[i] = bc;
    }
  }
  return 0;
}

template <typename T>
int lm_impl(const cdm_model_cfg* cfg, int nvox, int nmeas, const double* meas, double* params,
            const double* cfp, const double* fixp, int* iters, int* succ, double* costs) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const orc::Limits L = orc::make_limits(*cfg);
  const int ft = fixp_tsize();
#pragma omp parallel
  {
    orc::Voxel<T> v;
#pragma omp for schedule(dynamic, 4)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, meas + (size_t)i * nmeas, fixp + (size_t)i * ft, ft);
      const orc::LMResult r = orc::levmar_voxel(L, cfg->iter_levmar, cfg->marquardt != 0, v,
                                                params + (size_t)i * NPARAMS);
      if (iters) iters[i] = r.iterations;
      if (succ) succ[i] = r.successes;
      if (costs) costs[i] = r.cost;
    }
  }
  return 0;
}

template <typename T>
int mcmc_impl(const cdm_model_cfg* cfg, int nvox, int nmeas, const double* meas, double* params,
              const double* cfp, const double* fixp, double* samples, double* tau,
              uint32_t voxel_offset) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const orc::Limits L = orc::make_limits(*cfg);
  const int ft = fixp_tsize();
  orc::MCMCOpts o;
  o.nburn = cfg->nburn;
  o.njumps = cfg->njumps;
  o.sampleevery = cfg->sampleevery;
  o.update_proposal = cfg->update_proposal;
  o.rician = cfg->rician;
  o.seed = cfg->seed;
  o.stream = (uint32_t)cfg->id_part;
  const int ns = cfg->njumps / cfg->sampleevery;
#pragma omp parallel
  {
    orc::Voxel<T> v;
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, meas + (size_t)i * nmeas, fixp + (size_t)i * ft, ft);
      orc::mcmc_voxel(L, o, voxel_offset + (uint32_t)i, v, params + (size_t)i * NPARAMS,
                      samples + (size_t)i * NPARAMS * ns, tau ? tau + (size_t)i * ns : nullptr, ns);
    }
  }
  return 0;
}

template <typename T>
int bic_impl(int rician, int nvox, int nmeas, int nsamples, const double* meas,
             const double* samples, const double* cfp, const double* fixp, const double* tau,
             double* bic, double* aic) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const int ft = fixp_tsize();
#pragma omp parallel
  {
    orc::Voxel<T> v;
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, meas + (size_t)i * nmeas, fixp + (size_t)i * ft, ft);
      orc::bic_aic_voxel(v, samples + (size_t)i * NPARAMS * nsamples, nsamples, rician != 0,
                         tau ? tau + (size_t)i * nsamples : nullptr, bic + i, aic + i);
    }
  }
  return 0;
}

template <typename T>
int pred_impl(int nvox, int nmeas, int nsamples, const double* samples, const double* cfp,
              const double* fixp, double* pred) {
  const orc::Protocol pr = orc::make_protocol(nmeas, cfp_tsize(), cfp);
  const int ft = fixp_tsize();
#pragma omp parallel
  {
    orc::Voxel<T> v;
    std::vector<double> zero(nmeas, 0.0);
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < nvox; i++) {
      orc::load_voxel(v, pr, zero.data(), fixp + (size_t)i * ft, ft);
      orc::predicted_voxel(v, samples + (size_t)i * NPARAMS * nsamples, nsamples,
                           pred + (size_t)i * nmeas);
    }
  }
  return 0;
}

}  // namespace

#define ORC_DISPATCH(prec, CALL) ((prec) == 1 ? CALL<fp32> : CALL<double>)

extern "C" {

int orc_model_info(cdm_model_info* info) {
  std::memset(info, 0, sizeof(*info));
  std::snprintf(info->name, sizeof(info->name), "%s", CDM_MODEL_NAME);
  info->nparams = NPARAMS;
  info->ncfp = NCFP;
  info->nfixp = NFIXP;
  for (int i = 0; i < NCFP; i++) info->cfp_size[i] = MODEL::CFP_size[i];
  for (int i = 0; i < NFIXP; i++) info->fixp_size[i] = MODEL::FixP_size[i];
  info->cfp_tsize = cfp_tsize();
  info->fixp_tsize = fixp_tsize();
  info->derived_cfp = CDM_NDCFP;
  info->derived_p = CDM_NDP;
  return 0;
}

int orc_signal(int prec, int nvox, int nmeas, const double* params, const double* cfp,
               const double* fixp, double* S, double* J, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, signal_impl)(nvox, nmeas, params, cfp, fixp, S, J);
}

int orc_cost(int prec, int nvox, int nmeas, const double* meas, const double* params,
             const double* cfp, const double* fixp, double* cost, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, cost_impl)(nvox, nmeas, meas, params, cfp, fixp, cost);
}

int orc_gridsearch(int prec, const cdm_model_cfg* cfg, int nvox, int nmeas, const double* meas,
                   double* params, const double* cfp, const double* fixp, int* best_index,
                   double* best_cost, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, gs_impl)(cfg, nvox, nmeas, meas, params, cfp, fixp, best_index,
                                     best_cost);
}

int orc_levmar(int prec, const cdm_model_cfg* cfg, int nvox, int nmeas, const double* meas,
               double* params, const double* cfp, const double* fixp, int* iters, int* succ,
               double* costs, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, lm_impl)(cfg, nvox, nmeas, meas, params, cfp, fixp, iters, succ,
                                     costs);
}

int orc_mcmc(int prec, const cdm_model_cfg* cfg, int nvox, int nmeas, const double* meas,
             double* params, const double* cfp, const double* fixp, double* samples, double* tau,
             uint32_t voxel_offset, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, mcmc_impl)(cfg, nvox, nmeas, meas, params, cfp, fixp, samples, tau,
                                       voxel_offset);
}

int orc_bic_aic(int prec, int rician, int nvox, int nmeas, int nsamples, const double* meas,
                const double* samples, const double* cfp, const double* fixp, const double* tau,
                double* bic, double* aic, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, bic_impl)(rician, nvox, nmeas, nsamples, meas, samples, cfp, fixp,
                                      tau, bic, aic);
}

int orc_predicted(int prec, int nvox, int nmeas, int nsamples, const double* samples,
                  const double* cfp, const double* fixp, double* pred, int nthreads) {
  set_threads(nthreads);
  return ORC_DISPATCH(prec, pred_impl)(nvox, nmeas, nsamples, samples, cfp, fixp, pred);
}

int orc_max_threads(void) { return omp_get_max_threads(); }

// Philox4x32-10 block (known-answer tests) and the MCMC draw built on it.
void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  cdm_u32x4 c = {ctr[0], ctr[1], ctr[2], ctr[3]};
  const cdm_u32x4 r = cdm_philox4x32_10(c, key[0], key[1]);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

void orc_mcmc_draws(uint64_t seed, uint32_t voxel, uint32_t n, float* normal, float* uniform) {
  for (uint32_t i = 0; i < n; i++) {
    const cdm_draw d = cdm_mcmc_draw(seed, voxel, i, 0, 0);
    normal[i] = d.normal;
    uniform[i] = d.uniform;
  }
}

}  // extern "C"
