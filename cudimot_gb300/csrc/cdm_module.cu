// cdm_module.cu - the device half of a split model library.
//
// Compiled with nvcc -cubin against a model plugin (same include order and
// headers as cdm_model.cu), it holds every kernel of the library as an
// extern "C" kernel with a fixed name (cdm_kernels.h), plus the
// no-allocation scratch array. The host half (cdm_model.cu built with
// CDM_MODULE_HOST) is compiled without the plugin, from the generated model
// description, and looks these kernels up by name. A split build lets the
// device code be compiled where the plugin's sources are while the host
// library is compiled on the machine that runs it.
#define CDM_DEVICE_MODULE 1

#include <math_constants.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

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
#include "cdm_noalloc_scratch.h"

// The scratch of cdm_levmar_noalloc; external linkage so that the host half
// can find it with cudaLibraryGetGlobal.
extern "C" __device__ __align__(256) unsigned char cdm_noalloc_scratch[kNoAllocScratchBytes];

// Every lane count, or only CDM_CHECK_LANES (a compile check of a plugin,
// which then takes a sixth of the time).
#ifdef CDM_CHECK_LANES
#define CDM_LANES(X, ...) X(CDM_CHECK_LANES, __VA_ARGS__)
#else
#define CDM_LANES(X, ...) X(1, __VA_ARGS__) X(2, __VA_ARGS__) X(4, __VA_ARGS__) \
  X(8, __VA_ARGS__) X(16, __VA_ARGS__) X(32, __VA_ARGS__)
#endif

#define CDM_W_BLOCK(Gw, fam, Args, body, ...)                                          \
  extern "C" __global__ void __launch_bounds__(__VA_ARGS__)                            \
      cdm_k_##fam##_##Gw(const __grid_constant__ Args a) { body; }

#define CDM_W_GS(Gw, _) CDM_W_BLOCK(Gw, gridsearch, cdm_gs_args, cdm_gridsearch_kernel<Gw>(a), CDM_NT)
#define CDM_W_LM(Gw, _) CDM_W_BLOCK(Gw, levmar, cdm_lm_args, cdm_levmar_kernel<Gw>(a), CDM_NT)
#define CDM_W_MC(Gw, _)                                                                       \
  CDM_W_BLOCK(Gw, mcmc, cdm_mcmc_args, (cdm_mcmc_kernel<Gw, false>(a)), CDM_NT, CDM_MCMC_MIN_BLOCKS)
#define CDM_W_MCR(Gw, _)                                                                      \
  CDM_W_BLOCK(Gw, mcmc_rician, cdm_mcmc_args, (cdm_mcmc_kernel<Gw, true>(a)), CDM_NT,         \
              CDM_MCMC_MIN_BLOCKS)
#define CDM_W_PACK(Gw, _)                                                                     \
  extern "C" __global__ void cdm_k_pack_signals_##Gw(const double* __restrict__ meas, int nvox, \
                                                     int nmeas, int nchunk,                   \
                                                     float* __restrict__ out) {               \
    cdm_pack_signals_kernel<Gw>(meas, nvox, nmeas, nchunk, out);                              \
  }

#if CDM_SHELLS
#define CDM_W_PREP_SHELLS(Gw, _)                                                              \
  extern "C" __global__ void cdm_k_prep_shells_##Gw(const double* __restrict__ cfp, int nmeas,  \
                                                    int nmeas_pad, float* __restrict__ table,  \
                                                    int* __restrict__ perm,                    \
                                                    int* __restrict__ shell_rank) {            \
    cdm_prep_shells_kernel<Gw>(cfp, nmeas, nmeas_pad, table, perm, shell_rank);                \
  }
#define CDM_W_PACK_SHELLS(Gw, _)                                                              \
  extern "C" __global__ void cdm_k_pack_shell_signals_##Gw(                                   \
      const double* __restrict__ meas, int nvox, int nmeas, int nchunk,                       \
      const float* __restrict__ table, const int* __restrict__ perm, float* __restrict__ out) { \
    cdm_pack_shell_signals_kernel<Gw>(meas, nvox, nmeas, nchunk, table, perm, out);           \
  }
CDM_LANES(CDM_W_PREP_SHELLS, 0)
CDM_LANES(CDM_W_PACK_SHELLS, 0)
#endif

CDM_LANES(CDM_W_GS, 0)
CDM_LANES(CDM_W_LM, 0)
CDM_LANES(CDM_W_MC, 0)
CDM_LANES(CDM_W_MCR, 0)
CDM_LANES(CDM_W_PACK, 0)

extern "C" __global__ void __launch_bounds__(CDM_NT)
    cdm_k_gs_recheck(const __grid_constant__ cdm_gs_recheck_args a) { cdm_gs_recheck_kernel(a); }
extern "C" __global__ void __launch_bounds__(CDM_NT)
    cdm_k_predicted(const __grid_constant__ cdm_post_args a) { cdm_predicted_kernel(a); }
extern "C" __global__ void __launch_bounds__(CDM_NT)
    cdm_k_bic_aic(const __grid_constant__ cdm_post_args a) { cdm_bic_aic_kernel(a); }
extern "C" __global__ void __launch_bounds__(CDM_NT)
    cdm_k_synth(const __grid_constant__ cdm_synth_args a) { cdm_synth_kernel(a); }
extern "C" __global__ void cdm_k_select_worse(int n, const double* __restrict__ cost,
                                              const double* __restrict__ ref, double margin,
                                              int* __restrict__ idx, int* __restrict__ count) {
  cdm_select_worse_kernel(n, cost, ref, margin, idx, count);
}
extern "C" __global__ void cdm_k_rows(int nsel, const int* __restrict__ idx, int ncols,
                                      const double* __restrict__ src, double* __restrict__ dst,
                                      int scatter, double value) {
  cdm_rows_kernel(nsel, idx, ncols, src, dst, scatter, value);
}
extern "C" __global__ void cdm_k_prep_protocol(const double* __restrict__ cfp, int nmeas,
                                               int nmeas_pad, float* __restrict__ p32,
                                               double* __restrict__ p64) {
  cdm_prep_protocol_kernel(cfp, nmeas, nmeas_pad, p32, p64);
}
extern "C" __global__ void cdm_k_params_to_samples(const double* __restrict__ params, int nvox,
                                                   double* __restrict__ samples) {
  cdm_params_to_samples_kernel(params, nvox, samples);
}
#ifdef CDM_MLP_HEAD
extern "C" __global__ void cdm_k_mlp_encode(const double* __restrict__ params, int n,
                                            float* __restrict__ t) {
  cdm_mlp_encode_kernel(params, n, t);
}
extern "C" __global__ void cdm_k_mlp_decode(const float* __restrict__ out, int ld, int n,
                                            double* __restrict__ params,
                                            double* __restrict__ prop_sd) {
  cdm_mlp_decode_kernel(out, ld, n, params, prop_sd);
}
#endif
extern "C" __global__ void cdm_k_clean_signals(int nvox, int nmeas, double* __restrict__ meas) {
  cdm_clean_signals_kernel(nvox, nmeas, meas);
}
extern "C" __global__ void cdm_k_wait_selftest(uint64_t limit_ns, int* err) {
  cdm_wait_selftest_kernel(limit_ns, err);
}
