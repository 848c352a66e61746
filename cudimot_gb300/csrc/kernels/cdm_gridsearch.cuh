// cdm_gridsearch.cuh - exhaustive grid search, one voxel per lane group.
//
// Semantics follow CUDIMOT's gridSearch_kernel (GridSearch.cu:97-248): the
// grid parameters of each combination replace the voxel's parameters,
// combinations outside the bounds are skipped (checkBounds, :25-47), and the
// first combination with the lowest sum of squares wins (strict '<',
// :216). Combination order is Model.cu's set_grid order.
//
// GB300 structure: costs are evaluated in FP32 (each lane sums its own
// measurements, the group total too) and ranked in FP32; the grid is read
// as floats, and which combinations pass the bounds test is decided once
// per grid on the host (grid_ok), so the loop over combinations runs no FP64
// instruction (the FP64 pipe is 1/64 of the FP32 rate on this GPU). Each
// group tracks its four best combinations. If the runner-up lies within `band` (relative) of the best,
// the FP32 ranking is not trusted: the voxel is flagged and
// cdm_gs_recheck_kernel re-evaluates the candidates (or, when more than
// three are within the band, every combination) in FP64 with CUDIMOT's
// summation order and keeps the first minimum. `band` is chosen well above
// the measured FP32 cost error (~1e-6 relative), so the argmin equals the
// FP64 argmin.
#pragma once
#include "cdm_common.cuh"



__device__ __forceinline__ bool cdm_gs_in_bounds(const cdm_limits& lim, const double* x) {
  bool in = true;
#pragma unroll
  for (int p = 0; p < kNP; p++) in = in && cdm_in_bounds1(lim, p, x[p]);
  return in;
}

template <int Gw>
CDM_KERNEL(CDM_NT) cdm_gridsearch_kernel(CDM_KARG(cdm_gs_args) a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const int* shdr;
  const float* ptab = cdm_prepare_tables<Gw>(sproto, a.nmeas_pad, a.nchunk, a.shells_staged != 0, &shdr);
  const int v = (int)CDM_BLOCK_IDX * (CDM_NT / Gw) + (int)threadIdx.x / Gw;
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

  double base[kNP];
#pragma unroll
  for (int p = 0; p < kNP; p++) base[p] = a.params[(size_t)v * kNP + p];
  cdm_real FixP[kNFIX];
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_real P[kNPS];
#pragma unroll
  for (int i = 0; i < kNPS; i++) P[i] = cdm_real(0.0f);
#pragma unroll
  for (int p = 0; p < kNP; p++) P[p] = cdm_real((float)base[p]);

  if (a.cost_only) {  // the cost at the voxel's own parameters, FP64 group sum
    cdm_update_derived(P, FixP);
    const double cost = cdm_group_sse<Gw>(io, sproto, P, FixP, gm);
    if (lane == 0) a.cost_out[v] = cost;
    return;
  }
  // the voxel's own values of the parameters outside the grid are the same
  // in every combination: tested once
  bool base_in = true;
#pragma unroll
  for (int p = 0; p < kNP; p++) base_in = base_in && (a.gpos[p] >= 0 || cdm_in_bounds1(lim, p, base[p]));

  float bcost[kGsTop];
  int bcomb[kGsTop];
#pragma unroll
  for (int k = 0; k < kGsTop; k++) {
    bcost[k] = 9e20f;  // CUDIMOT's initial best cost (GridSearch.cu:178)
    bcomb[k] = -1;
  }
  for (int c = 0; base_in && c < a.combs; c++) {
    if (!((__ldg(a.grid_ok + (c >> 5)) >> (c & 31)) & 1u)) continue;
#pragma unroll
    for (int p = 0; p < kNP; p++)
      if (a.gpos[p] >= 0) P[p] = cdm_real(__ldg(a.grid + (size_t)c * a.ngp + a.gpos[p]));
    cdm_update_derived(P, FixP);
    const float cost = cdm_group_sse<Gw, float>(io, sproto, P, FixP, gm);
    // Sorted insertion with constant indices (register arrays): entries
    // strictly worse than `cost` move down one place, equal costs keep the
    // earlier combination first (CUDIMOT's strict '<').
#pragma unroll
    for (int j = kGsTop - 1; j >= 0; j--) {
      const bool above = (j > 0) && (cost < bcost[j > 0 ? j - 1 : 0]);
      const bool here = cost < bcost[j];
      if (above) {
        bcost[j] = bcost[j - 1 >= 0 ? j - 1 : 0];
        bcomb[j] = bcomb[j - 1 >= 0 ? j - 1 : 0];
      } else if (here) {
        bcost[j] = cost;
        bcomb[j] = c;
      }
    }
  }
  if (lane != 0) return;
  a.best[v] = bcomb[0];
  if (bcomb[0] < 0) {
    a.flags[v] = 0;
    return;
  }
  const double band_cost = (double)bcost[0] * (1.0 + (double)a.band);
  int nin = 0;
#pragma unroll
  for (int k = 0; k < kGsTop; k++) nin += (bcomb[k] >= 0 && bcost[k] <= band_cost) ? 1 : 0;
  a.flags[v] = nin <= 1 ? 0 : (nin < kGsTop ? 1 : 2);
#pragma unroll
  for (int k = 0; k < kGsTop; k++) a.cand[(size_t)v * kGsTop + k] = bcomb[k];
#pragma unroll
  for (int p = 0; p < kNP; p++)
    if (a.gpos[p] >= 0) a.params[(size_t)v * kNP + p] = a.grid64[(size_t)bcomb[0] * a.ngp + a.gpos[p]];
}

// ----------------------------------------------------------------------------
// FP64 re-check of flagged voxels: one warp per voxel, lane l sums
// measurements l, l+32, ... and the warp folds with the 16/8/4/2/1 shuffle
// tree, CUDIMOT's summation order (GridSearch.cu:49-95).

__device__ __forceinline__ double cdm_warp_cost64(const cdm_gs_recheck_args& a, int v, double* P,
                                                  double* FixP) {
  const int lane = threadIdx.x & 31;
  double acc = 0.0;
  for (int m = lane; m < a.nmeas; m += 32) {
    double cf[kNCOLS];
#pragma unroll
    for (int k = 0; k < kNCOLS; k++) cf[k] = a.proto64[(size_t)m * kNCOLS + k];
    const double e = Predicted_Signal(NPARAMS, P, cf, FixP) - a.meas[(size_t)v * a.nmeas + m];
    acc += e * e;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
  return __shfl_sync(0xFFFFFFFFu, acc, 0);
}

CDM_KERNEL(CDM_NT) cdm_gs_recheck_kernel(CDM_KARG(cdm_gs_recheck_args) a) {
  const int v = blockIdx.x * (CDM_NT / 32) + (int)threadIdx.x / 32;
  if (v >= a.nvox) return;
  const int flag = a.flags[v];
  if (flag == 0) return;
  const int lane = threadIdx.x & 31;
  double base[kNP];
#pragma unroll
  for (int p = 0; p < kNP; p++) base[p] = a.params[(size_t)v * kNP + p];
  double FixP[kNFIX];
#pragma unroll
  for (int k = 0; k < kNFIX; k++) FixP[k] = k < a.fixp_tsize ? a.fixp[(size_t)v * a.fixp_tsize + k] : 0.0;
  const int ntry = flag == 1 ? kGsTop : a.combs;
  double best = 9e20;
  int bestc = -1;
  for (int t = 0; t < ntry; t++) {
    const int c = flag == 1 ? a.cand[(size_t)v * kGsTop + t] : t;
    if (c < 0) continue;
    double P[kNPS];
#pragma unroll
    for (int i = 0; i < kNPS; i++) P[i] = 0.0;
#pragma unroll
    for (int p = 0; p < kNP; p++)
      P[p] = a.gpos[p] >= 0 ? a.grid[(size_t)c * a.ngp + a.gpos[p]] : base[p];
    if (!cdm_gs_in_bounds(a.lim, P)) continue;
    cdm_update_derived(P, FixP);
    const double cost = cdm_warp_cost64(a, v, P, FixP);
    // strict '<' in combination order; candidates arrive cost-sorted, so ties
    // are broken towards the lower combination index explicitly.
    if (cost < best || (cost == best && c < bestc)) {
      best = cost;
      bestc = c;
    }
  }
  if (lane == 0 && bestc >= 0) {
    a.best[v] = bestc;
#pragma unroll
    for (int p = 0; p < kNP; p++)
      if (a.gpos[p] >= 0) a.params[(size_t)v * kNP + p] = a.grid[(size_t)bestc * a.ngp + a.gpos[p]];
    if (a.rechecked) atomicAdd(a.rechecked, 1ull);
  }
}
