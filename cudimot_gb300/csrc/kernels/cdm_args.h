// cdm_args.h - the compile-time sizes and the launch arguments of the
// fitting kernels, shared by the kernels and the host code that fills them.
//
// Needs only the model's sizes: NPARAMS, CDM_PSTORE, CDM_CFP_TSIZE,
// CDM_FIXP_TSIZE, CDM_NDCFP and, for plugins with the paired signal hook,
// CDM_SIGNAL_PAIR. A normal build takes them from the plugin (through
// cdm_plugin_tail.h and the generated cdm_model_sizes.h); the host half of a
// split build (device code compiled separately into a module) takes them
// from the generated model description, without the plugin.
#pragma once
#include <stdint.h>
#include <cuda_bf16.h>

#ifndef CDM_NT
#define CDM_NT 128  // threads per CTA
#endif

// The paired (two-measurement) cost loop: plugins with the paired signal
// hook, evaluated in single precision.
#if defined(CDM_SIGNAL_PAIR) && !defined(CDM_EVAL_DOUBLE)
#define CDM_PAIRED 1
#else
#define CDM_PAIRED 0
#endif

constexpr int kNP = NPARAMS;
constexpr int kNPS = CDM_PSTORE;
constexpr int kNCOLS = CDM_CFP_TSIZE + CDM_NDCFP;
constexpr int kNCOLS4 = (kNCOLS + 3) / 4 * 4;  // protocol row stride (floats)
constexpr int kNFIX = CDM_FIXP_TSIZE > 0 ? CDM_FIXP_TSIZE : 1;
constexpr int kNCOLSP = (kNCOLS + 1) / 2 * 2;  // pair-table entry stride (column pairs, even)
#if CDM_PAIRED
constexpr int kPairTables = 1;  // shared-memory protocol copies of the paired-loop kernels
#else
constexpr int kPairTables = 0;
#endif

constexpr int kGsTop = 4;
constexpr int kCustomPrior = 5;  // prior type CUSTOM (cudimot.h)
#ifdef CDM_EVAL_DOUBLE
constexpr int kRealBytes = 8;    // bytes of the plugin's evaluation type
#else
constexpr int kRealBytes = 4;
#endif
// Static shared memory of the MCMC kernel at one lane per voxel (its sample
// staging buffer, cdm_record_sample) plus its barrier: the dynamic shared
// memory the host allows leaves room for it.
constexpr int kMcmcStaticSmem = CDM_NT * (kNP + 1) * 4 * 8 + 64;

// Per-shell series (plugins with the hook CDM_SHELL_SERIES, evaluated in
// single precision): grid search and the Gaussian MCMC sum the signals of
// each b-shell with per-shell coefficients (Shell_Coeffs /
// Predicted_Signal_Shell_Pair). A prep kernel groups the measurements by
// shell on the device; protocols with more than kShellMax shells, or whose
// per-shell padding would add more than 1/8 of the measurements, keep the
// per-measurement path (the shell table is then marked invalid).
#if defined(CDM_SHELL_SERIES) && CDM_PAIRED
#define CDM_SHELLS 1
#else
#define CDM_SHELLS 0
#endif
constexpr int kShellMax = 8;
constexpr int kShellHeader = 32;  // ints: valid, nshell, npos, then per shell rep, pairs, first
#ifndef CDM_SHELL_MCOLS
#define CDM_SHELL_MCOLS 3
#endif
// Padded positions of a shell-ordered protocol of nmeas measurements at
// most, with Gw lanes per voxel (each shell padded to whole pairs of lane
// chunks).
__host__ __device__ constexpr int cdm_shell_max_pos(int nmeas, int Gw) {
  return nmeas + kShellMax * (2 * Gw - 1);
}
// Packed signals are tile-major: the voxels of one CTA (a tile, CDM_NT / Gw
// of them) keep all their rows in one contiguous block, [tile][row][voxel in
// tile][lane], so the signals that the resident CTAs re-read on every pass
// or proposal form one contiguous stretch of memory (with each row spanning
// all voxels instead, the rows lay megabytes apart and the MCMC's L2 misses
// varied 3x with the buffer's placement). A row is one lane chunk (one
// float per lane) in measurement order, or in the per-shell path one pair of
// chunks (a float2 per lane, one 8-byte load). Within a tile the next row
// of a lane is CDM_NT elements on.
__host__ __device__ constexpr size_t cdm_tile_index(int v, int row, int j, int rows, int Gw) {
  return (((size_t)(v / (CDM_NT / Gw)) * rows + row) * (CDM_NT / Gw) + v % (CDM_NT / Gw)) * Gw + j;
}
// Elements of the packed signals of nvox voxels with `rows` rows (whole tiles).
__host__ __device__ constexpr size_t cdm_tile_elems(int nvox, int rows, int Gw) {
  return ((size_t)(nvox > 1 ? nvox : 1) + CDM_NT / Gw - 1) / (CDM_NT / Gw) * rows * CDM_NT;
}
// Pair rows the per-shell layout may need.
__host__ __device__ constexpr int cdm_shell_sig_rows(int nmeas, int Gw) {
  return (cdm_shell_max_pos(nmeas, Gw) + 2 * Gw - 1) / (2 * Gw);
}
// Floats of the shell table that follows the staged protocol: the header,
// then 4 floats (gx, gy, gz, weight) per padded position.
__host__ __device__ constexpr int cdm_shell_table_floats(int nmeas, int Gw) {
  return CDM_SHELLS ? kShellHeader + 4 * cdm_shell_max_pos(nmeas, Gw) : 0;
}

// Bounds, priors and fixed flags as the kernels use them. Bounds and prior
// arguments are floats, as in CUDIMOT's __constant__ copies.
struct cdm_limits {
  int btype[kNP];
  float bmin[kNP];
  float bmax[kNP];
  int ptype[kNP];
  float pa[kNP];
  float pb[kNP];
  int fixed[kNP];
};

// One parameter value against its bounds, in double against the float
// bounds, as grid search tests a combination (btype: CUDIMOT's enum bound,
// 0 none, 1 min, 2 max, 3 both).
__host__ __device__ inline bool cdm_in_bounds1(const cdm_limits& lim, int p, double x) {
  const int t = lim.btype[p];
  if ((t == 1 || t == 3) && x < (double)lim.bmin[p]) return false;
  if ((t == 2 || t == 3) && x > (double)lim.bmax[p]) return false;
  return true;
}

struct cdm_gs_args {
  int nvox, nmeas, nmeas_pad, nchunk, fixp_tsize;
  uint32_t proto_bytes;
  const float* proto;
  const float* sig;
  double* params;
  const double* fixp;
  const float* grid;   // [combs][ngp], rounded to float
  const double* grid64;  // [combs][ngp], the winner's values are written from here
  const uint32_t* grid_ok;  // bit c: combination c's grid values pass the bounds test
  int ngp;
  int combs;
  int gpos[kNP];       // column of parameter p in the grid, or -1
  float band;
  int shells_staged;   // a shell table follows the protocol in the staged bytes
  int* flags;          // [nvox]: 0 decided, 1 recheck candidates, 2 recheck all
  int* cand;           // [nvox][kGsTop]
  int* best;           // [nvox] winning combination (or -1)
  double* cost_out;    // cost_only: [nvox] the cost (FP32 terms, FP64 sum)
  int cost_only;       // evaluate the cost at the voxel's own parameters (no grid)
  int* err;
  cdm_limits lim;
};

struct cdm_gs_recheck_args {
  int nvox, nmeas, fixp_tsize;
  const double* proto64;  // [nmeas][NCOLS]
  const double* meas;     // [nvox][nmeas]
  double* params;
  const double* fixp;
  const double* grid;
  int ngp, combs;
  int gpos[kNP];
  const int* flags;
  const int* cand;
  int* best;
  unsigned long long* rechecked;
  cdm_limits lim;
};

struct cdm_lm_args {
  int nvox, nmeas, nmeas_pad, nchunk, fixp_tsize;
  uint32_t proto_bytes;
  const float* proto;
  const float* sig;
  double* params;
  const double* fixp;
  int max_iters;
  int marquardt;
  int* err;
  unsigned long long* iter_count;  // sum of loop passes, may be null
  unsigned long long* succ_count;  // sum of accepted steps, may be null
  cdm_limits lim;
};

struct cdm_mcmc_args {
  int nvox, nmeas, nmeas_pad, nchunk, fixp_tsize;
  uint32_t proto_bytes;
  const float* proto;
  const float* sig;
  double* params;
  const double* fixp;
  double* samples;
  double* tau_samples;
  int nburn, njumps, sampleevery, nsamples, update_proposal;
  uint64_t seed;
  uint32_t stream;
  uint32_t voxel_offset;
  const double* prop_sd;  // [nvox][NPARAMS] initial proposal widths; null or <= 0: P/10 as CUDIMOT
  int shells_staged;      // a shell table follows the protocol in the staged bytes (Gaussian only)
  int cfp_all_off;        // float offset in shared memory of the [nmeas][CFP_Tsize] copy of
                          // the protocol that custom priors receive, or -1 (no custom prior)
  int* err;
  cdm_limits lim;
};

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

struct cdm_synth_args {
  int nvox, nmeas, nmeas_pad, fixp_tsize, b_col, x_ld;
  uint32_t proto_bytes;
  const float* proto;
  const double* params;     // [nvox][NPARAMS]
  const double* fixp;       // [nvox][fixp_tsize] (true values)
  float snr_lo, snr_hi;
  uint64_t seed;
  double* meas;             // [nvox][nmeas] (optional)
  double* s0_est;           // [nvox] mean of the noisy b = 0 signals (optional)
  __nv_bfloat16* x;         // [nvox][x_ld] noisy / s0_est (optional)
  int* err;
};
