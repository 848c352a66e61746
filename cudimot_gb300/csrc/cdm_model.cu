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
#include <type_traits>
#include <vector>

#include "cdm_host.h"
#include "cudimot_gb300.h"
#include "cdm_hetero.h"

#include "cdm_kernels.h"
#include "cdm_noalloc_scratch.h"

#ifdef CDM_MODULE_HOST
// Host half of a split build: the model's sizes and hooks come from the
// description generated from the plugin; the kernels come from the device
// module (cdm_module.cu) embedded in this library.
#include "cdm_model_desc.h"
#include "cdm_args.h"
constexpr int kNH = kNP * (kNP + 1) / 2;
#else
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
#endif

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

// Block sizes of the plugin's CFP and FixP arrays (MODEL::CFP_size /
// FixP_size of modelparameters.cc), padded so that a model without blocks
// still has an array.
#ifdef CDM_MODULE_HOST
const int kCfpBlocks[] = CDM_CFP_SIZES;
const int kFixpBlocks[] = CDM_FIXP_SIZES;
#else
const int* const kCfpBlocks = MODEL::CFP_size;
const int* const kFixpBlocks = MODEL::FixP_size;
#endif

// ------------------------------------------------------------------ kernels
// Every launch goes through cudaLaunchKernel with the kernel's address
// (normal build) or its handle in the embedded device module (split build).
#ifdef CDM_MODULE_HOST
extern "C" const unsigned char cdm_module_image[];

struct module_state {
  std::once_flag once;
  cudaError_t err = cudaSuccess;
  cudaLibrary_t lib = nullptr;
  std::mutex mu;
  const void* fn[CDM_K_COUNT][6] = {};
};
module_state g_module;

cudaError_t module_library(cudaLibrary_t* lib) {
  std::call_once(g_module.once, [] {
    g_module.err = cudaLibraryLoadData(&g_module.lib, cdm_module_image, nullptr, nullptr, 0,
                                       nullptr, nullptr, 0);
  });
  *lib = g_module.lib;
  return g_module.err;
}

const void* kfn(int fam, int lanes) {
  const bool laned = fam < CDM_K_NLANE_FAMILIES;
  const int li = laned ? cdm_lane_index(lanes) : 0;
  if (fam < 0 || fam >= CDM_K_COUNT || li < 0) return nullptr;
  cudaLibrary_t lib = nullptr;
  if (module_library(&lib) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(g_module.mu);
  if (!g_module.fn[fam][li]) {
    char name[64];
    if (laned)
      std::snprintf(name, sizeof(name), "cdm_k_%s_%d", cdm_kfam_name(fam), lanes);
    else
      std::snprintf(name, sizeof(name), "cdm_k_%s", cdm_kfam_name(fam));
    cudaKernel_t k = nullptr;
    if (cudaLibraryGetKernel(&k, lib, name) == cudaSuccess) g_module.fn[fam][li] = (const void*)k;
  }
  return g_module.fn[fam][li];
}
#else
template <int Gw>
const void* kfn_lanes(int fam) {
  switch (fam) {
    case CDM_K_GRIDSEARCH: return (const void*)cdm_gridsearch_kernel<Gw>;
    case CDM_K_LEVMAR: return (const void*)cdm_levmar_kernel<Gw>;
    case CDM_K_MCMC: return (const void*)cdm_mcmc_kernel<Gw, false>;
    case CDM_K_MCMC_RICIAN: return (const void*)cdm_mcmc_kernel<Gw, true>;
    case CDM_K_PACK_SIGNALS: return (const void*)cdm_pack_signals_kernel<Gw>;
#if CDM_SHELLS
    case CDM_K_PREP_SHELLS: return (const void*)cdm_prep_shells_kernel<Gw>;
    case CDM_K_PACK_SHELL_SIGNALS: return (const void*)cdm_pack_shell_signals_kernel<Gw>;
#endif
  }
  return nullptr;
}

const void* kfn(int fam, int lanes) {
  if (fam < CDM_K_NLANE_FAMILIES) {
    switch (lanes) {
      case 1: return kfn_lanes<1>(fam);
      case 2: return kfn_lanes<2>(fam);
      case 4: return kfn_lanes<4>(fam);
      case 8: return kfn_lanes<8>(fam);
      case 16: return kfn_lanes<16>(fam);
      case 32: return kfn_lanes<32>(fam);
    }
    return nullptr;
  }
  switch (fam) {
    case CDM_K_GS_RECHECK: return (const void*)cdm_gs_recheck_kernel;
    case CDM_K_PREDICTED: return (const void*)cdm_predicted_kernel;
    case CDM_K_BIC_AIC: return (const void*)cdm_bic_aic_kernel;
    case CDM_K_SELECT_WORSE: return (const void*)cdm_select_worse_kernel;
    case CDM_K_ROWS: return (const void*)cdm_rows_kernel;
    case CDM_K_PREP_PROTOCOL: return (const void*)cdm_prep_protocol_kernel;
    case CDM_K_PARAMS_TO_SAMPLES: return (const void*)cdm_params_to_samples_kernel;
    case CDM_K_SYNTH: return (const void*)cdm_synth_kernel;
#ifdef CDM_MLP_HEAD
    case CDM_K_MLP_ENCODE: return (const void*)cdm_mlp_encode_kernel;
    case CDM_K_MLP_DECODE: return (const void*)cdm_mlp_decode_kernel;
#endif
    case CDM_K_CLEAN_SIGNALS: return (const void*)cdm_clean_signals_kernel;
    case CDM_K_WAIT_SELFTEST: return (const void*)cdm_wait_selftest_kernel;
  }
  return nullptr;
}
#endif

cdm_status launch_argv(int fam, int lanes, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       void** args) {
  const void* fn = kfn(fam, lanes);
  if (!fn)
    return cdm_fail(CDM_CUDA_ERROR, std::string("kernel ") + cdm_kfam_name(fam) + " (" +
                                        std::to_string(lanes) + " lanes) is not available");
  CDM_CUDA(cudaLaunchKernel(fn, grid, block, args, smem, st));
  return CDM_OK;
}

// One launch; every argument is passed by address, so each must already
// have the exact type of the kernel's parameter (the typed wrappers below).
template <class... A>
cdm_status launch(int fam, int lanes, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                  A... args) {
  void* argv[] = {(void*)&args...};
  return launch_argv(fam, lanes, grid, block, smem, st, argv);
}

// The dynamic shared memory a launch may use without opting in is 48 KB
// less the kernel's static shared memory (the MCMC kernel's sample staging
// is 4-37 KB, by lane count and parameter count), so the opt-in depends on
// both; the static size is read once per kernel. The opt-in only ever
// grows: lowering it while an earlier launch of the same kernel with more
// shared memory is still queued is not safe.
cdm_status set_smem(int fam, int lanes, size_t bytes) {
  if (bytes == 0) return CDM_OK;
  const void* fn = kfn(fam, lanes);
  if (!fn) return cdm_fail(CDM_CUDA_ERROR, std::string("kernel ") + cdm_kfam_name(fam) + " is not available");
  static std::mutex mu;
  static long static_bytes[CDM_K_COUNT][6];
  static long opted[CDM_K_COUNT][6];
  static bool known[CDM_K_COUNT][6];
  const int li = fam < CDM_K_NLANE_FAMILIES ? cdm_lane_index(lanes) : 0;
  if (fam < 0 || fam >= CDM_K_COUNT || li < 0) return cdm_fail(CDM_BAD_ARG, "kernel family or lanes");
  std::lock_guard<std::mutex> lock(mu);
  if (!known[fam][li]) {
    cudaFuncAttributes fa;
    CDM_CUDA(cudaFuncGetAttributes(&fa, fn));
    static_bytes[fam][li] = (long)fa.sharedSizeBytes;
    known[fam][li] = true;
  }
  if ((long)bytes + static_bytes[fam][li] <= 48 * 1024 || (long)bytes <= opted[fam][li]) return CDM_OK;
  CDM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  opted[fam][li] = (long)bytes;
  return CDM_OK;
}

// Typed launches: the parameters are those of the kernels (cdm_postfit.cuh,
// cdm_synth.cuh), so the argument blocks match them exactly.
cdm_status k_prep_protocol(cudaStream_t st, const double* cfp, int nmeas, int nmeas_pad, float* p32,
                           double* p64) {
  return launch(CDM_K_PREP_PROTOCOL, 0, (nmeas_pad + 127) / 128, 128, 0, st, cfp, nmeas, nmeas_pad,
                p32, p64);
}
cdm_status k_pack_signals(int lanes, int blocks, cudaStream_t st, const double* meas, int nvox,
                          int nmeas, int nchunk, float* out) {
  return launch(CDM_K_PACK_SIGNALS, lanes, blocks, 256, 0, st, meas, nvox, nmeas, nchunk, out);
}
cdm_status k_params_to_samples(int blocks, cudaStream_t st, const double* params, int nvox,
                               double* samples) {
  return launch(CDM_K_PARAMS_TO_SAMPLES, 0, blocks, 256, 0, st, params, nvox, samples);
}
cdm_status k_prep_shells(int lanes, cudaStream_t st, const double* cfp, int nmeas, int nmeas_pad,
                         float* table, int* perm, int* shell_rank) {
  return launch(CDM_K_PREP_SHELLS, lanes, 1, 256, 0, st, cfp, nmeas, nmeas_pad, table, perm,
                shell_rank);
}
cdm_status k_pack_shell_signals(int lanes, int blocks, cudaStream_t st, const double* meas, int nvox,
                                int nmeas, int nchunk, const float* table, const int* perm,
                                float* out) {
  return launch(CDM_K_PACK_SHELL_SIGNALS, lanes, blocks, 256, 0, st, meas, nvox, nmeas, nchunk,
                table, perm, out);
}
cdm_status k_select_worse(int blocks, cudaStream_t st, int n, const double* cost, const double* ref,
                          double margin, int* idx, int* count) {
  return launch(CDM_K_SELECT_WORSE, 0, blocks, 256, 0, st, n, cost, ref, margin, idx, count);
}
cdm_status k_rows(int blocks, cudaStream_t st, int nsel, const int* idx, int ncols,
                  const double* src, double* dst, int scatter, double value) {
  return launch(CDM_K_ROWS, 0, blocks, 256, 0, st, nsel, idx, ncols, src, dst, scatter, value);
}
cdm_status k_mlp_encode(int blocks, cudaStream_t st, const double* params, int n, float* t) {
  return launch(CDM_K_MLP_ENCODE, 0, blocks, 256, 0, st, params, n, t);
}
cdm_status k_mlp_decode(int blocks, cudaStream_t st, const float* out, int ld, int n,
                        double* params, double* prop_sd) {
  return launch(CDM_K_MLP_DECODE, 0, blocks, 256, 0, st, out, ld, n, params, prop_sd);
}
cdm_status k_clean_signals(int blocks, cudaStream_t st, int nvox, int nmeas, double* meas) {
  return launch(CDM_K_CLEAN_SIGNALS, 0, blocks, 256, 0, st, nvox, nmeas, meas);
}
cdm_status k_wait_selftest(cudaStream_t st, uint64_t limit_ns, int* err) {
  return launch(CDM_K_WAIT_SELFTEST, 0, 1, 32, 0, st, limit_ns, err);
}

#ifndef CDM_MODULE_HOST
// The typed launches above must match the kernels' parameter lists.
template <class F, class G>
constexpr bool cdm_same_sig = std::is_same<F, G>::value;
static_assert(cdm_same_sig<decltype(&cdm_prep_protocol_kernel),
                           void (*)(const double*, int, int, float*, double*)>, "prep_protocol");
static_assert(cdm_same_sig<decltype(&cdm_pack_signals_kernel<1>),
                           void (*)(const double*, int, int, int, float*)>, "pack_signals");
static_assert(cdm_same_sig<decltype(&cdm_params_to_samples_kernel),
                           void (*)(const double*, int, double*)>, "params_to_samples");
#if CDM_SHELLS
static_assert(cdm_same_sig<decltype(&cdm_prep_shells_kernel<1>),
                           void (*)(const double*, int, int, float*, int*, int*)>, "prep_shells");
static_assert(cdm_same_sig<decltype(&cdm_pack_shell_signals_kernel<1>),
                           void (*)(const double*, int, int, int, const float*, const int*, float*)>,
              "pack_shell_signals");
#endif
static_assert(cdm_same_sig<decltype(&cdm_select_worse_kernel),
                           void (*)(int, const double*, const double*, double, int*, int*)>,
              "select_worse");
static_assert(cdm_same_sig<decltype(&cdm_rows_kernel),
                           void (*)(int, const int*, int, const double*, double*, int, double)>,
              "rows");
static_assert(cdm_same_sig<decltype(&cdm_clean_signals_kernel), void (*)(int, int, double*)>,
              "clean_signals");
static_assert(cdm_same_sig<decltype(&cdm_wait_selftest_kernel), void (*)(uint64_t, int*)>,
              "wait_selftest");
#ifdef CDM_MLP_HEAD
static_assert(cdm_same_sig<decltype(&cdm_mlp_encode_kernel), void (*)(const double*, int, float*)>,
              "mlp_encode");
static_assert(cdm_same_sig<decltype(&cdm_mlp_decode_kernel),
                           void (*)(const float*, int, int, double*, double*)>, "mlp_decode");
#endif
#endif

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
  float* grid32 = nullptr;     // the grid rounded to float, as the kernel evaluates it
  size_t grid32_cap = 0;
  uint32_t* grid_ok = nullptr; // bit c: combination c's grid values are within the bounds
  size_t grid_ok_cap = 0;
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
  int* shell_perm = nullptr;   // per-shell series: padded position -> measurement
  size_t shell_perm_cap = 0;
  int* shell_rank = nullptr;   // per-shell series: scratch of the shell prep kernel
  size_t shell_rank_cap = 0;
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
  // cdm_mcmc_prepare: the MCMC launch is described here instead of made
  cdm_tile_work* export_to = nullptr;
  // cdm_fit_host on large calls: the pieces' contexts (own streams, own
  // buffers) and the configuration they were made for
  static constexpr int kMaxPieces = 4;
  cdm_ctx* piece[kMaxPieces] = {};
  cdm_model_cfg piece_cfg[kMaxPieces];
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
// With the per-shell series (grid search and Gaussian MCMC of plugins with
// the hook) the shell table is staged after the protocol; the pair table is
// built over it when the protocol has no usable shells, so the region
// holds the larger of the two.
size_t shell_bytes(int nmeas, int Gw) { return (size_t)cdm_shell_table_floats(nmeas, Gw) * sizeof(float); }
size_t fit_smem_shells(int nmeas_pad, int nmeas, int Gw) {
  return proto_bytes(nmeas_pad) +
         std::max(proto_bytes(nmeas_pad) * kPairTables, shell_bytes(nmeas, Gw));
}
// Float count of the protocol buffer: the table, then room for a shell table.
size_t proto32_floats(int nmeas_pad, int nmeas) {
  return (size_t)kNCOLS4 * nmeas_pad + (size_t)cdm_shell_table_floats(nmeas, 32);
}

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
  const size_t cap = std::min<size_t>(200 * 1024, 227 * 1024 - kMcmcStaticSmem - 1024);
  if (std::max(fit_smem(pad), fit_smem_shells(pad, nmeas, 32)) > cap)
    return cdm_fail(CDM_BAD_ARG, "protocol too large for shared memory staging");
  return CDM_OK;
}

// Protocol tables from CUDIMOT's CFP array (device pointer).
cdm_status prep_protocol(cdm_ctx* c, int nmeas, const double* CFP, cudaStream_t st) {
  const int pad = round_up(nmeas, 32);
  CDM_TRY(dev_alloc(&c->proto32, &c->proto32_cap, proto32_floats(pad, nmeas)));
  CDM_TRY(dev_alloc(&c->proto64, &c->proto64_cap, (size_t)kNCOLS * nmeas));
  c->nmeas_pad = pad;
  return k_prep_protocol(st, CFP, nmeas, pad, c->proto32, c->proto64);
}

// The grid search and the Gaussian MCMC of plugins with the per-shell
// series: the shell table after the protocol rows (valid or marked invalid
// on the device) and the signals in its order.
constexpr bool kShells = CDM_SHELLS != 0;

size_t shell_sig_floats(int nvox, int nmeas, int Gw) {
  // the per-shell layout (float2 pair rows), or the measurement-order
  // layout when the table turns out invalid
  return std::max(2 * cdm_tile_elems(nvox, cdm_shell_sig_rows(nmeas, Gw), Gw),
                  cdm_tile_elems(nvox, (nmeas + Gw - 1) / Gw, Gw));
}

cdm_status prep_shells_and_pack(cdm_ctx* c, int Gw, int nvox, int nmeas, const double* CFP,
                                const double* meas, cudaStream_t st) {
  const int maxpos = cdm_shell_max_pos(nmeas, Gw);
  CDM_TRY(dev_alloc(&c->shell_perm, &c->shell_perm_cap, (size_t)maxpos));
  CDM_TRY(dev_alloc(&c->shell_rank, &c->shell_rank_cap, (size_t)nmeas));
  CDM_TRY(dev_alloc(&c->sig, &c->sig_cap, shell_sig_floats(nvox, nmeas, Gw)));
  float* table = c->proto32 + (size_t)kNCOLS4 * c->nmeas_pad;
  CDM_TRY(k_prep_shells(Gw, st, CFP, nmeas, c->nmeas_pad, table, c->shell_perm, c->shell_rank));
  if (nvox == 0) return CDM_OK;
  const int nchunk = (nmeas + Gw - 1) / Gw;
  const size_t total = (size_t)((maxpos + Gw - 1) / Gw) * nvox * Gw;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)c->num_sms * 32);
  return k_pack_shell_signals(Gw, blocks, st, meas, nvox, nmeas, nchunk, table, c->shell_perm, c->sig);
}

cdm_status pack_signals(cdm_ctx* c, int Gw, int nvox, int nmeas, const double* meas, cudaStream_t st) {
  if (cdm_lane_index(Gw) < 0) return cdm_fail(CDM_BAD_ARG, "lanes per voxel must be 1, 2, 4, 8, 16 or 32");
  const int nchunk = (nmeas + Gw - 1) / Gw;
  CDM_TRY(dev_alloc(&c->sig, &c->sig_cap, cdm_tile_elems(nvox, nchunk, Gw)));
  if (nvox == 0) return CDM_OK;
  const size_t total = (size_t)nchunk * nvox * Gw;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)c->num_sms * 32);
  return k_pack_signals(Gw, blocks, st, meas, nvox, nmeas, nchunk, c->sig);
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

uint32_t first_voxel(const cdm_ctx* c) { return (uint32_t)c->cfg.first_voxel; }

int blocks_for(int nvox, int Gw) { return (nvox + (CDM_NT / Gw) - 1) / (CDM_NT / Gw); }

// ------------------------------------------------------------------ stages
// The staged bytes and shared memory of a grid-search launch (with the
// shell table when the plugin has the per-shell series).
cdm_status launch_gs_args(cdm_ctx* c, cdm_gs_args& a, int Gw, int nvox, int nmeas, cudaStream_t st) {
  a.shells_staged = kShells ? 1 : 0;
  size_t sm = fit_smem(c->nmeas_pad);
  if (kShells) {
    a.proto_bytes = (uint32_t)(proto_bytes(c->nmeas_pad) + shell_bytes(nmeas, Gw));
    sm = fit_smem_shells(c->nmeas_pad, nmeas, Gw);
  }
  CDM_TRY(set_smem(CDM_K_GRIDSEARCH, Gw, sm));
  return launch(CDM_K_GRIDSEARCH, Gw, blocks_for(nvox, Gw), CDM_NT, sm, st, a);
}

cdm_status launch_gs(cdm_ctx* c, int Gw, int nvox, int nmeas, double* params, const double* FixP,
                     cudaStream_t st) {
  cdm_gs_args a;
  fill_common(c, a, nvox, nmeas, Gw);
  a.params = params;
  a.fixp = FixP;
  a.grid = c->grid32;
  a.grid64 = c->grid_dev;
  a.grid_ok = c->grid_ok;
  a.ngp = c->cfg.n_grid_params;
  a.combs = c->cfg.grid_combs;
  for (int p = 0; p < kNP; p++) a.gpos[p] = c->gpos[p];
  a.band = kGsBand;
  a.flags = c->gs_flags;
  a.cand = c->gs_cand;
  a.best = c->gs_best;
  a.cost_out = nullptr;
  a.cost_only = 0;
  return launch_gs_args(c, a, Gw, nvox, nmeas, st);
}

cdm_status run_gridsearch(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                          const double* CFP, const double* FixP, cudaStream_t st) {
  if (c->cfg.grid_combs <= 0 || c->cfg.n_grid_params <= 0) return CDM_OK;
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  // narrowest groups first: measured on NODDI-Watson, 200k voxels x 288
  // measurements, 968 combinations: 2 lanes 49.8 ms, 4 lanes 55.1 ms, 1 lane
  // 84.9 ms
  const int Gw = pick_lanes(c, c->cfg.lanes_gridsearch, 2, nvox);
  if (kShells)
    CDM_TRY(prep_shells_and_pack(c, Gw, nvox, nmeas, CFP, meas, st));
  else
    CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  const size_t n = (size_t)std::max(nvox, 1);
  CDM_TRY(dev_alloc(&c->gs_flags, &c->gs_flags_cap, n));
  CDM_TRY(dev_alloc(&c->gs_cand, &c->gs_cand_cap, n * kGsTop));
  CDM_TRY(dev_alloc(&c->gs_best, &c->gs_best_cap, n));
  if (nvox == 0) return CDM_OK;
  CDM_TRY(launch_gs(c, Gw, nvox, nmeas, params, FixP, st));
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
  return launch(CDM_K_GS_RECHECK, 0, blocks_for(nvox, 32), CDM_NT, 0, st, r);
}

cdm_status launch_lm(cdm_ctx* c, int Gw, int nvox, int nmeas, double* params, const double* FixP,
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
  CDM_TRY(set_smem(CDM_K_LEVMAR, Gw, sm));
  return launch(CDM_K_LEVMAR, Gw, blocks_for(nvox, Gw), CDM_NT, sm, st, a);
}

cdm_status run_levmar(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                      const double* CFP, const double* FixP, cudaStream_t st) {
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  // NODDI-Watson, 200k voxels x 288 measurements: 4 lanes 37.6 ms, 2 lanes
  // 40.4 ms, 1 lane 41.0 ms, 8 lanes 42.5 ms
  const int Gw = pick_lanes(c, c->cfg.lanes_levmar, 4, nvox);
  CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  if (nvox == 0) return CDM_OK;
  return launch_lm(c, Gw, nvox, nmeas, params, FixP, st);
}

cdm_status launch_mcmc(cdm_ctx* c, int Gw, bool rician, int nvox, int nmeas, double* params,
                       const double* FixP, double* samples, double* tau, uint32_t voxel_offset,
                       cudaStream_t st) {
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
  const int fam = rician ? CDM_K_MCMC_RICIAN : CDM_K_MCMC;
  size_t sm = fit_smem(c->nmeas_pad);
  a.shells_staged = 0;
  if (kShells && !rician) {
    a.shells_staged = 1;
    a.proto_bytes = (uint32_t)(proto_bytes(c->nmeas_pad) + shell_bytes(nmeas, Gw));
    sm = fit_smem_shells(c->nmeas_pad, nmeas, Gw);
  }
  // custom priors: a [nmeas][CFP_Tsize] copy of the protocol after the tables
  a.cfp_all_off = -1;
  for (int p = 0; p < kNP; p++)
    if (c->lim.ptype[p] == kCustomPrior) a.cfp_all_off = (int)((sm + 7) / 8 * 2);
  if (a.cfp_all_off >= 0) {
    sm = (size_t)a.cfp_all_off * 4 + (size_t)nmeas * CDM_CFP_TSIZE * kRealBytes;
    if (sm > 227 * 1024 - (size_t)kMcmcStaticSmem - 1024)
      return cdm_fail(CDM_BAD_ARG, "protocol too large for the custom priors' copy of it");
  }
  CDM_TRY(set_smem(fam, Gw, sm));
  if (c->export_to) {
    static_assert(sizeof(cdm_mcmc_args) <= CDM_TILE_ARGS_MAX, "MCMC argument block");
    cdm_tile_work* w = c->export_to;
    std::snprintf(w->model, sizeof(w->model), "%s", CDM_MODEL_NAME);
    w->eval_double = kRealBytes == 8 ? 1 : 0;
    w->threads = CDM_NT;
    w->lanes = Gw;
    w->rician = rician ? 1 : 0;
    w->ntiles = blocks_for(nvox, Gw);
    w->smem_bytes = (uint32_t)sm;
    w->scratch_bytes = (uint32_t)((CDM_NT / Gw) * (kNP + 1) * 4 * sizeof(double));
    w->args_bytes = (uint32_t)sizeof(cdm_mcmc_args);
    w->err = c->err;
    std::memcpy(w->args, &a, sizeof(cdm_mcmc_args));
    return CDM_OK;
  }
  return launch(fam, Gw, blocks_for(nvox, Gw), CDM_NT, sm, st, a);
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
  if (kShells && !c->cfg.rician)
    CDM_TRY(prep_shells_and_pack(c, Gw, nvox, nmeas, CFP, meas, st));
  else
    CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  if (nvox == 0) return CDM_OK;
  return launch_mcmc(c, Gw, c->cfg.rician != 0, nvox, nmeas, params, FixP, samples, tau,
                     voxel_offset, st);
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
  const int fam = bic ? CDM_K_BIC_AIC : CDM_K_PREDICTED;
  CDM_TRY(set_smem(fam, 0, sm));
  return launch(fam, 0, blocks_for(nvox, 32), CDM_NT, sm, st, a);
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
    CDM_TRY(k_params_to_samples(std::max(1, std::min(c->num_sms * 4, (nvox * kNP + 255) / 256)), st,
                                params, nvox, samples));
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
// Signal floats a fit of this shape may pack: every lane count in
// measurement order, and the shell order of the grid search and MCMC.
size_t fit_sig_floats(const cdm_ctx* c, int nvox, int nmeas) {
  size_t sig = 0;
  for (int Gw : {1, 2, 4, 8, 16, 32})
    sig = std::max(sig, cdm_tile_elems(nvox, (nmeas + Gw - 1) / Gw, Gw));
  if (kShells)
    for (int Gw : {pick_lanes(c, c->cfg.lanes_gridsearch, 2, nvox), pick_lanes(c, c->cfg.lanes_mcmc, 2, nvox)})
      sig = std::max(sig, shell_sig_floats(nvox, nmeas, Gw));
  return sig;
}

cdm_status reserve_fit(cdm_ctx* c, int nvox, int nmeas) {
  const int pad = round_up(nmeas, 32);
  CDM_TRY(dev_alloc(&c->proto32, &c->proto32_cap, proto32_floats(pad, nmeas)));
  CDM_TRY(dev_alloc(&c->proto64, &c->proto64_cap, (size_t)kNCOLS * nmeas));
  CDM_TRY(dev_alloc(&c->sig, &c->sig_cap, fit_sig_floats(c, nvox, nmeas)));
  if (kShells) {
    CDM_TRY(dev_alloc(&c->shell_perm, &c->shell_perm_cap, (size_t)cdm_shell_max_pos(nmeas, 32)));
    CDM_TRY(dev_alloc(&c->shell_rank, &c->shell_rank_cap, (size_t)nmeas));
  }
  const size_t n = (size_t)std::max(nvox, 1);
  CDM_TRY(dev_alloc(&c->gs_flags, &c->gs_flags_cap, n));
  CDM_TRY(dev_alloc(&c->gs_cand, &c->gs_cand_cap, n * kGsTop));
  CDM_TRY(dev_alloc(&c->gs_best, &c->gs_best_cap, n));
  // kernel attributes are set outside capture too
  for (int Gw : {1, 2, 4, 8, 16, 32})
    CDM_TRY(set_smem(CDM_K_GRIDSEARCH, Gw,
                     kShells ? fit_smem_shells(pad, nmeas, Gw) : fit_smem(pad)));
  return CDM_OK;
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
  for (int i = 0; i < NCFP && i < CDM_MAX_BLOCKS; i++) info->cfp_size[i] = kCfpBlocks[i];
  for (int i = 0; i < NFIXP && i < CDM_MAX_BLOCKS; i++) info->fixp_size[i] = kFixpBlocks[i];
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
  std::vector<int> sizes(kCfpBlocks, kCfpBlocks + NCFP);
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
    // the grid as the FP32 ranking pass reads it: each value rounded to
    // float, and per combination whether its grid values pass the bounds
    // test (the same double-against-float-bound comparisons as the FP64
    // re-check, so both passes skip the same combinations)
    const int ngp = cfg->n_grid_params, combs = cfg->grid_combs;
    std::vector<float> g32(c->grid_host.size());
    std::vector<uint32_t> ok(((size_t)combs + 31) / 32, 0u);
    for (size_t i = 0; i < g32.size(); i++) g32[i] = (float)c->grid_host[i];
    for (int k = 0; k < combs; k++) {
      bool in = true;
      for (int p = 0; p < kNP; p++)
        if (c->gpos[p] >= 0)
          in = in && cdm_in_bounds1(c->lim, p, c->grid_host[(size_t)k * ngp + c->gpos[p]]);
      if (in) ok[k / 32] |= 1u << (k % 32);
    }
    s = dev_alloc(&c->grid_dev, &c->grid_cap, c->grid_host.size());
    if (s == CDM_OK) s = dev_alloc(&c->grid32, &c->grid32_cap, g32.size());
    if (s == CDM_OK) s = dev_alloc(&c->grid_ok, &c->grid_ok_cap, ok.size());
    if (s == CDM_OK) {
      e = cudaMemcpy(c->grid_dev, c->grid_host.data(), c->grid_host.size() * sizeof(double),
                     cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(c->grid32, g32.data(), g32.size() * sizeof(float), cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(c->grid_ok, ok.data(), ok.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
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
  for (cdm_ctx* p : c->piece) cdm_destroy(p);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  void* bufs[] = {c->grid_dev, c->grid32, c->grid_ok, c->proto32, c->proto64, c->sig, c->gs_flags, c->gs_cand,
                  c->gs_best, c->shell_perm, c->shell_rank, c->err, c->counters, c->h_meas, c->h_params, c->h_cfp, c->h_fixp,
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
  return run_mcmc(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau_samples, first_voxel(c),
                  (cudaStream_t)stream);
}

cdm_status cdm_mcmc_prepare(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size,
                            const double* meas, double* params, const double* CFP,
                            const double* FixP, double* samples, double* tau_samples,
                            void* stream, cdm_tile_work* out) {
  if (!out) return cdm_fail(CDM_BAD_ARG, "null cdm_tile_work");
  std::memset(out, 0, sizeof(*out));
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  c->export_to = out;
  const cdm_status s = run_mcmc(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau_samples,
                                first_voxel(c), (cudaStream_t)stream);
  c->export_to = nullptr;
  if (s == CDM_OK && nvox == 0) {  // run_mcmc returns before the launch
    std::snprintf(out->model, sizeof(out->model), "%s", CDM_MODEL_NAME);
    out->eval_double = kRealBytes == 8 ? 1 : 0;
    out->threads = CDM_NT;
    out->err = c->err;
  }
  return s;
}

cdm_status cdm_mcmc_seeded(cdm_ctx* c, int nvox, int nmeas, int CFP_size, int FixP_size,
                           const double* meas, double* params, const double* CFP,
                           const double* FixP, double* samples, double* tau_samples,
                           const double* prop_sd, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CFP_size, FixP_size));
  c->prop_sd = prop_sd;
  const cdm_status s = run_mcmc(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau_samples, first_voxel(c),
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
  CDM_TRY(set_smem(CDM_K_SYNTH, 0, sm));
  return launch(CDM_K_SYNTH, 0, (nvox + CDM_NT / 32 - 1) / (CDM_NT / 32), CDM_NT, sm, st, a);
}

cdm_status cdm_cost(cdm_ctx* c, int nvox, int nmeas, const double* meas, const double* params,
                    const double* CFP, const double* FixP, double* cost, void* stream) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!meas || !params || !CFP || !cost || (CDM_FIXP_TSIZE > 0 && !FixP))
    return cdm_fail(CDM_BAD_ARG, "null array");
  cudaStream_t st = (cudaStream_t)stream;
  CDM_TRY(prep_protocol(c, nmeas, CFP, st));
  // the grid-search kernel with one "combination", the voxel's own
  // parameters: the cost exactly as grid search and MCMC score it
  const int Gw = pick_lanes(c, c->cfg.lanes_gridsearch, 2, nvox);
  if (kShells)
    CDM_TRY(prep_shells_and_pack(c, Gw, nvox, nmeas, CFP, meas, st));
  else
    CDM_TRY(pack_signals(c, Gw, nvox, nmeas, meas, st));
  if (nvox == 0) return CDM_OK;
  cdm_gs_args a;
  std::memset(&a, 0, sizeof(a));
  fill_common(c, a, nvox, nmeas, Gw);
  a.params = const_cast<double*>(params);  // read only when cost_only is set
  a.fixp = FixP;
  a.grid = nullptr;
  a.ngp = 0;
  a.combs = 1;
  for (int p = 0; p < kNP; p++) a.gpos[p] = -1;
  a.band = kGsBand;
  a.cost_out = cost;
  a.cost_only = 1;
  return launch_gs_args(c, a, Gw, nvox, nmeas, st);
}

cdm_status cdm_select_worse(int n, const double* cost, const double* ref, double margin, int* idx,
                            int* count, void* stream) {
  if (n < 0 || !cost || !ref || !idx || !count) return cdm_fail(CDM_BAD_ARG, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  CDM_CUDA(cudaMemsetAsync(count, 0, sizeof(int), st));
  if (n == 0) return CDM_OK;
  return k_select_worse(std::min((n + 255) / 256, 152 * 8), st, n, cost, ref, margin, idx, count);
}

cdm_status cdm_rows(int nsel, const int* idx, int ncols, const double* src, double* dst, int mode,
                    double value, void* stream) {
  if (nsel < 0 || ncols <= 0 || !idx || !dst || mode < 0 || mode > 2 || (mode < 2 && !src))
    return cdm_fail(CDM_BAD_ARG, "bad argument");
  if (nsel == 0) return CDM_OK;
  const size_t total = (size_t)nsel * ncols;
  return k_rows((int)std::min<size_t>((total + 255) / 256, 152 * 8), (cudaStream_t)stream, nsel, idx,
                ncols, mode == 2 ? nullptr : src, dst, mode == 1 ? 1 : 0, value);
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
  return k_mlp_encode(std::min((n + 255) / 256, 152 * 8), (cudaStream_t)stream, params, n, targets);
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
  return k_mlp_decode(std::min((n + 255) / 256, 152 * 8), (cudaStream_t)stream, out, ld, n, params,
                      prop_sd);
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
                                AIC, first_voxel(c), cap);
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
    if (c->proto32_cap < proto32_floats(pad, nmeas) || c->sig_cap < fit_sig_floats(c, nvox, nmeas) ||
        c->gs_flags_cap < (size_t)std::max(nvox, 1) ||
        (kShells && c->shell_perm_cap < (size_t)cdm_shell_max_pos(nmeas, 32)))
      return cdm_fail(CDM_BAD_ARG, "cdm_fit_enqueue under stream capture needs cdm_fit_reserve "
                                   "for this shape first");
  } else {
    CDM_TRY(reserve_fit(c, nvox, nmeas));
  }
  CDM_CUDA(cudaMemsetAsync(c->counters, 0, 4 * sizeof(unsigned long long), st));
  return fit_sequence(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau, pred, BIC, AIC,
                      first_voxel(c), st);
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
  return k_wait_selftest((cudaStream_t)stream, (uint64_t)limit_ms * 1000000ull, c->err);
}

cdm_status cdm_clean_signals(int nvox, int nmeas, double* meas, void* stream) {
  if (nvox < 0 || nmeas <= 0 || (nvox > 0 && !meas)) return cdm_fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  const size_t threads = (size_t)nvox * 32;
  return k_clean_signals((int)((threads + 255) / 256), (cudaStream_t)stream, nvox, nmeas, meas);
}

}  // extern "C"

namespace {

// cdm_fit_host's stream work for one context: host->device copies, the fit
// (cdm_fit, one captured graph), device->host copies; no synchronisation.
cdm_status fit_host_enqueue(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                            const double* CFP, const double* FixP, double* samples, double* tau,
                            double* pred, double* BIC, double* AIC, cudaStream_t st) {
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
  return CDM_OK;
}

// Pieces of a large cdm_fit_host call: 50,000 voxels or more per piece, at
// most kMaxPieces.
int fit_host_npieces(int nvox) {
  return std::max(1, std::min(cdm_ctx::kMaxPieces, nvox / 50000));
}

// A large cdm_fit_host call as consecutive voxel ranges, each fitted by a
// context of its own on its own stream (copies in, fit, copies out), all
// in flight at once: the copies of one range overlap the fits of the
// others, and the ranges' kernels share the GPU. Each range's context has
// first_voxel = its start and the lane counts the whole call would have, so
// every voxel gets the result of one call over all of them (the MCMC draws
// are keyed by the global voxel index). On the GB300 a single 460 MB copy
// issued right after the GPU had been busy took 26-45 ms instead of 2.2 ms;
// in pieces, behind other pieces' fits, that time is hidden.
cdm_status fit_host_pieces(cdm_ctx* c, int npieces, int nvox, int nmeas, const double* meas,
                           double* params, const double* CFP, const double* FixP, double* samples,
                           double* tau, double* pred, double* BIC, double* AIC, int64_t timeout_ms) {
  const cdm_model_cfg& o = c->cfg;
  const int ns = o.run_mcmc ? o.njumps / std::max(o.sampleevery, 1) : 1;
  const int lanes_gs = pick_lanes(c, o.lanes_gridsearch, 2, nvox);
  const int lanes_lm = pick_lanes(c, o.lanes_levmar, 4, nvox);
  const int lanes_mc = pick_lanes(c, o.lanes_mcmc, 2, nvox);
  for (int k = 0; k < npieces; k++) {
    const int v0 = (int)((int64_t)nvox * k / npieces), v1 = (int)((int64_t)nvox * (k + 1) / npieces);
    cdm_model_cfg pc;
    std::memcpy(&pc, &o, sizeof(pc));  // byte for byte, padding included (compared below)
    pc.first_voxel = o.first_voxel + v0;
    pc.lanes_gridsearch = lanes_gs;
    pc.lanes_levmar = lanes_lm;
    pc.lanes_mcmc = lanes_mc;
    pc.grid = c->grid_host.empty() ? nullptr : c->grid_host.data();
    if (c->grid_host.empty()) pc.run_gridsearch = 0;
    if (c->piece[k] && std::memcmp(&c->piece_cfg[k], &pc, sizeof(pc)) != 0) {
      cdm_destroy(c->piece[k]);
      c->piece[k] = nullptr;
    }
    if (!c->piece[k]) {
      CDM_TRY(cdm_create(&pc, &c->piece[k]));
      c->piece_cfg[k] = pc;
    }
    cdm_ctx* p = c->piece[k];
    if (!p->own_stream) CDM_CUDA(cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking));
    const size_t a = (size_t)v0;
    CDM_TRY(fit_host_enqueue(p, v1 - v0, nmeas, meas + a * nmeas, params + a * kNP, CFP,
                             FixP ? FixP + a * CDM_FIXP_TSIZE : nullptr, samples + a * kNP * ns,
                             tau ? tau + a * ns : nullptr, pred ? pred + a * nmeas : nullptr,
                             BIC ? BIC + a : nullptr, AIC ? AIC + a : nullptr, p->own_stream));
  }
  // wait for every piece; this context's counters become the pieces' sums
  // (the statistics of this fit, as cdm_fit leaves them)
  cdm_status first = CDM_OK;
  std::string msg;
  unsigned long long sum[4] = {0, 0, 0, 0};
  for (int k = 0; k < npieces; k++) {
    cdm_ctx* p = c->piece[k];
    const cdm_status st = cdm_synchronize(p, p->own_stream, timeout_ms);
    if (st != CDM_OK && first == CDM_OK) {
      first = st;
      msg = cdm_last_error();
    }
    unsigned long long h[4];
    CDM_CUDA(cudaMemcpy(h, p->counters, sizeof(h), cudaMemcpyDeviceToHost));
    CDM_CUDA(cudaMemset(p->counters, 0, sizeof(h)));
    for (int i = 0; i < 4; i++) sum[i] += h[i];
  }
  CDM_TRY(ensure_base(c));
  CDM_CUDA(cudaMemcpy(c->counters, sum, sizeof(sum), cudaMemcpyHostToDevice));
  if (first != CDM_OK) return cdm_fail(first, msg);
  return CDM_OK;
}

}  // namespace

extern "C" {

cdm_status cdm_fit_host(cdm_ctx* c, int nvox, int nmeas, const double* meas, double* params,
                        const double* CFP, const double* FixP, double* samples, double* tau,
                        double* pred, double* BIC, double* AIC, int part_size, int64_t timeout_ms) {
  CDM_TRY(check_common(c, nvox, nmeas, CDM_CFP_TSIZE, CDM_FIXP_TSIZE));
  if (!meas || !params || !CFP || !samples || (CDM_FIXP_TSIZE > 0 && !FixP))
    return cdm_fail(CDM_BAD_ARG, "null array");
  (void)part_size;  // CUDIMOT's SIZE_PART parts (dMRI_Data.cu:66-79): see fit_host_pieces
  const int npieces = fit_host_npieces(nvox);
  if (npieces <= 1) {
    if (!c->own_stream) CDM_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    CDM_TRY(fit_host_enqueue(c, nvox, nmeas, meas, params, CFP, FixP, samples, tau, pred, BIC, AIC,
                             c->own_stream));
    return cdm_synchronize(c, c->own_stream, timeout_ms);
  }
  return fit_host_pieces(c, npieces, nvox, nmeas, meas, params, CFP, FixP, samples, tau, pred, BIC,
                         AIC, timeout_ms);
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

#ifndef CDM_MODULE_HOST
static __device__ __align__(256) unsigned char cdm_noalloc_scratch[kNoAllocScratchBytes];
#endif

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
#ifdef CDM_MODULE_HOST
    // split build: the array lives in the embedded device module
    cudaLibrary_t lib = nullptr;
    CDM_CUDA(module_library(&lib));
    size_t bytes = 0;
    CDM_CUDA(cudaLibraryGetGlobal(&p, &bytes, lib, "cdm_noalloc_scratch"));
    if (bytes < kNoAllocScratchBytes)
      return cdm_fail(CDM_CUDA_ERROR, "the device module's no-allocation array is too small");
#else
    CDM_CUDA(cudaGetSymbolAddress(&p, cdm_noalloc_scratch));
#endif
    CDM_CUDA(cudaMemset(p, 0, kNoAllocHeader));
    g_noalloc_ptr[dev] = (unsigned char*)p;
  }
  *out = g_noalloc_ptr[dev];
  return CDM_OK;
}

cdm_status noalloc_lm_launch(int Gw, const cdm_model_cfg* cfg, unsigned char* scratch, int sms, int nvox,
                             int nmeas, const double* meas, double* params, const double* CFP,
                             const double* FixP, cudaStream_t st) {
  const int pad = round_up(nmeas, 32);
  const int nchunk = (nmeas + Gw - 1) / Gw;
  const size_t pbytes = proto_bytes(pad);
  const size_t sbytes = cdm_tile_elems(nvox, nchunk, Gw) * sizeof(float);
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
  CDM_TRY(k_prep_protocol(st, CFP, nmeas, pad, proto, nullptr));
  if (nvox == 0) return CDM_OK;
  const size_t total = (size_t)nchunk * nvox * Gw;
  CDM_TRY(k_pack_signals(Gw, (int)std::min<size_t>((total + 255) / 256, (size_t)std::max(sms, 1) * 32),
                         st, meas, nvox, nmeas, nchunk, sig));
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
  CDM_TRY(set_smem(CDM_K_LEVMAR, Gw, fit_smem(pad)));
  return launch(CDM_K_LEVMAR, Gw, blocks_for(nvox, Gw), CDM_NT, fit_smem(pad), st, a);
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
  if (fit_smem(round_up(nmeas, 32)) > std::min<size_t>(200 * 1024, 227 * 1024 - kMcmcStaticSmem - 1024))
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
  if (cdm_lane_index(Gw) < 0) return cdm_fail(CDM_BAD_ARG, "lanes_levmar must be 0, 1, 2, 4, 8, 16 or 32");
  return noalloc_lm_launch(Gw, cfg, scratch, sms, nvox, nmeas, meas, params, CFP, FixP,
                           (cudaStream_t)stream);
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
  return k_wait_selftest(st, (uint64_t)limit_ms * 1000000ull, (int*)scratch);
}
