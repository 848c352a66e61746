// cdm_hetero_part.cu - one model's part of the persistent multi-model kernel.
//
// Compiled once per model (nvcc -rdc, with that model's plugin directory
// and generated sizes on the include path, CDM_HX_ID = the model's index in
// the set) and device-linked with cdm_hetero_kernel.cu into one module.
// The plugin and the kernel code are included inside an unnamed namespace:
// every function, table and template instance of the model gets internal
// linkage, so the models' identically named functions (Predicted_Signal,
// cdm_mcmc_kernel<2, false>, ...) stay apart at device link. What is
// exported is one extern "C" device function per lane count and
// likelihood, cdm_hx_<id>_mcmc_<lanes>_<rician>(tile, scratch), which runs
// the MCMC of one tile (the CTA that blockIdx.x would have been) with the
// argument block the model's own library prepared (cdm_mcmc_prepare),
// found in the entry's slot of a constant-memory table.
#define CDM_DEVICE_MODULE 1
#define CDM_HETERO 1

// Everything the plugin and the kernels include from the system, first and
// at global scope; included again inside the namespace, their guards make
// them empty.
#include <math_constants.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <cmath>
#include <type_traits>

namespace {
#include "functions_gpu.h"
#include "modelparameters.h"
#include "macro_numerical.h"
#include "modelfunctions.h"
#include "cdm_plugin_tail.h"
#include "cdm_model_sizes.h"
#include "cdm_common.cuh"
#include "cdm_mcmc.cuh"
}  // namespace

#ifndef CDM_HX_ID
#error "CDM_HX_ID (the model's index in the set) is required"
#endif

// generated with the set: CDM_HX_ENTRIES, CDM_HX_ARGS_BLOCK, CDM_HX_NLANES
// and CDM_HX_LANES(X) = X(lanes, lane index) for every lane count
#include "cdm_hx_entries.h"

// The argument slots (cdm_hetero_kernel.cu): slot (model, lane index,
// likelihood) holds the argument block of the fit that runs on that entry.
// Each entry indexes its own slot with a constant, so the chain code reads
// its arguments from the constant bank, as the model library's kernel reads
// its parameters.
extern "C" __constant__ unsigned char cdm_hx_args[CDM_HX_ENTRIES][CDM_HX_ARGS_BLOCK];

#define CDM_HX_SLOT(li, r) ((CDM_HX_ID * CDM_HX_NLANES + (li)) * 2 + (r))
#define CDM_HX_CAT2(a, b, c, d) cdm_hx_##a##_mcmc_##b##_##c##d
#define CDM_HX_CAT(a, b, c, d) CDM_HX_CAT2(a, b, c, d)
#define CDM_HX_ENTRY(Gw, li)                                                                   \
  extern "C" __device__ void CDM_HX_CAT(CDM_HX_ID, Gw, 0, )(int tile, unsigned char* scratch) { \
    cdm_mcmc_kernel<Gw, false>(                                                                 \
        tile, scratch, *reinterpret_cast<const cdm_mcmc_args*>(cdm_hx_args[CDM_HX_SLOT(li, 0)])); \
  }                                                                                             \
  extern "C" __device__ void CDM_HX_CAT(CDM_HX_ID, Gw, 1, )(int tile, unsigned char* scratch) { \
    cdm_mcmc_kernel<Gw, true>(                                                                  \
        tile, scratch, *reinterpret_cast<const cdm_mcmc_args*>(cdm_hx_args[CDM_HX_SLOT(li, 1)])); \
  }

static_assert(sizeof(cdm_mcmc_args) <= CDM_HX_ARGS_BLOCK,
              "the model's MCMC argument block does not fit a slot of the persistent kernel");

// the argument block size, read by the host half to check an item against
// the model's build
#define CDM_HX_SIZE2(a) cdm_hx_##a##_args_bytes
#define CDM_HX_SIZE(a) CDM_HX_SIZE2(a)
extern "C" __device__ const unsigned CDM_HX_SIZE(CDM_HX_ID) = sizeof(cdm_mcmc_args);

CDM_HX_LANES(CDM_HX_ENTRY)
