// cdm_levmar.cuh - bounded Levenberg-Marquardt, one voxel per lane group.
//
// Semantics follow CUDIMOT's levenberg_kernel (Levenberg_Marquardt.cu:
// 409-623): parameters are optimised in a transformed space (log for
// one-sided bounds, tan for two-sided bounds, with CUDIMOT's 1e-4 nudges and
// speed factor 10; :37-118); the loop runs while
// !(success && iter++ >= max_iters) so only accepted steps count; damping
// is Marquardt's (1+lambda) diagonal scaling (or Levenberg's +lambda);
// lambda starts at 0.1, is divided by 10 on success and multiplied by 10 on
// failure; the fit ends when 2|dc| <= tol (|c|+|c'|+2e-16) after a success
// or when lambda exceeds 1e20; FixConstraintsLM runs at the end. Two
// departures, both for single-precision costs: tol is CDM_LM_CFTOL (1e-6)
// instead of 1e-8, and a rejected step that changed no parameter ends the
// fit (every later trial would be the same point).
//
// GB300 structure: one pass over the measurements per accepted step forms
// the residual and the Jacobian once and accumulates J^T r and the upper
// triangle of J^T J in FP32 registers (CUDIMOT evaluates S and dS twice, once
// for the gradient and once for the Hessian, with a warp reduction per
// element and 32-measurement chunk). The lane partials are summed across the
// group in FP64 and the damped normal equations are solved in FP64 registers
// by symmetric elimination in the pivot order of CUDIMOT's unpivoted LUsolver
// (:334-407). Undamped sums are kept, and damping is applied to a fresh copy
// each iteration, which equals CUDIMOT's cumulative rescaling.
#pragma once
#include "cdm_common.cuh"


constexpr float kTwoDivPIf = 0.636619772367581f;
constexpr float kAvoidf = 1e-4f;
constexpr float kSpeedf = 10.0f;

__device__ __forceinline__ float cdm_minmax_inv(float x, float lo, float hi) {
  float t = x - (lo + hi) * 0.5f;
  t *= 2.0f / ((hi - lo) * kTwoDivPIf);
  return tanf(t) * kSpeedf;
}

// invtransformAll (Levenberg_Marquardt.cu:90-103).
__device__ __forceinline__ void cdm_lm_inv_transform(const cdm_limits& lim, cdm_real* P, float* Pt) {
#pragma unroll
  for (int p = 0; p < kNP; p++) {
    const float lo = lim.bmin[p], hi = lim.bmax[p];
    float x = (float)P[p];
    if (lim.fixed[p]) {  // a fixed parameter never moves: no round trip through the transform
      Pt[p] = x;
      continue;
    }
    if (lim.btype[p] == BMIN) {
      Pt[p] = logf(x - lo);
    } else if (lim.btype[p] == BMAX) {
      Pt[p] = logf(hi - x);
    } else if (lim.btype[p] == BMINMAX) {
      if (x <= lo + kAvoidf) x += kAvoidf;
      if (x >= hi - kAvoidf) x -= kAvoidf;
      P[p] = cdm_real(x);
      Pt[p] = cdm_minmax_inv(x, lo, hi);
    } else {
      Pt[p] = x;
    }
  }
}

// transformAll (Levenberg_Marquardt.cu:105-118); may nudge Pt.
__device__ __forceinline__ void cdm_lm_transform(const cdm_limits& lim, cdm_real* P, float* Pt) {
#pragma unroll
  for (int p = 0; p < kNP; p++) {
    const float lo = lim.bmin[p], hi = lim.bmax[p];
    if (lim.fixed[p]) continue;
    if (lim.btype[p] == BMIN) {
      P[p] = cdm_real(expf(Pt[p]) + lo);
    } else if (lim.btype[p] == BMAX) {
      P[p] = cdm_real(hi - expf(Pt[p]));
    } else if (lim.btype[p] == BMINMAX) {
      float x = (hi - lo) * 0.5f * atanf(Pt[p] / kSpeedf) * kTwoDivPIf + (lo + hi) * 0.5f;
      if (x <= lo + kAvoidf) {
        x += kAvoidf;
        Pt[p] = cdm_minmax_inv(x, lo, hi);
      }
      if (x >= hi - kAvoidf) {
        x -= kAvoidf;
        Pt[p] = cdm_minmax_inv(x, lo, hi);
      }
      P[p] = cdm_real(x);
    } else {
      P[p] = cdm_real(Pt[p]);
    }
  }
}

// d theta / d theta_t per parameter (derivative_transf, :120-135).
__device__ __forceinline__ void cdm_lm_chain(const cdm_limits& lim, const float* Pt, float* f) {
#pragma unroll
  for (int p = 0; p < kNP; p++) {
    if (lim.btype[p] == BMIN)
      f[p] = expf(Pt[p]);
    else if (lim.btype[p] == BMAX)
      f[p] = -expf(Pt[p]);
    else if (lim.btype[p] == BMINMAX)
      f[p] = (lim.bmax[p] - lim.bmin[p]) * 0.5f * kTwoDivPIf * (kSpeedf / (kSpeedf * kSpeedf + Pt[p] * Pt[p]));
    else
      f[p] = 1.0f;
  }
}

constexpr int kNH = kNP * (kNP + 1) / 2;

// Index of (i, q), i <= q, in the packed upper triangle (row-major).
__host__ __device__ constexpr int cdm_hidx(int i, int q) { return i * kNP - i * (i - 1) / 2 + (q - i); }

// Convergence tolerance on the relative cost change of an accepted step.
// CUDIMOT's is 1e-8 (Levenberg_Marquardt.cu:21,34), below the resolution of
// a cost built from single-precision residuals (relative noise ~1e-7), so
// an FP32 fit would only stop on lambda > 1e20 or the iteration limit after
// dozens of noise-driven steps. 1e-6 stops where the FP32 cost stops
// carrying information; the final cost then differs from a fully converged
// FP64 fit by a few 1e-6 relative.
#ifndef CDM_LM_CFTOL
#define CDM_LM_CFTOL 1.0e-6
#endif

// Damped normal equations (hess + damping) x = g in FP64, all in registers:
// symmetric Gaussian elimination on the packed upper triangle (no pivoting,
// the pivot order of CUDIMOT's Gauss-Jordan LUsolver,
// Levenberg_Marquardt.cu:334-407), then back substitution. ~n^3/6
// multiply-adds instead of Gauss-Jordan's ~n^3/2.
__device__ __forceinline__ void cdm_lm_solve(const double (&hess)[kNH], const double (&g)[kNP],
                                             double lambda, bool marquardt, double (&x)[kNP]) {
  double amat[kNH], b[kNP];
#pragma unroll
  for (int i = 0; i < kNP; i++) {
    b[i] = g[i];
#pragma unroll
    for (int q = i; q < kNP; q++) {
      const double h = hess[cdm_hidx(i, q)];
      amat[cdm_hidx(i, q)] = i == q ? (marquardt ? (1.0 + lambda) * h : h + lambda) : h;
    }
  }
  double dinv[kNP];
#pragma unroll
  for (int j = 0; j < kNP; j++) {
    dinv[j] = 1.0 / amat[cdm_hidx(j, j)];
#pragma unroll
    for (int i = j + 1; i < kNP; i++) {
      const double f = amat[cdm_hidx(j, i)] * dinv[j];
#pragma unroll
      for (int q = i; q < kNP; q++) amat[cdm_hidx(i, q)] -= f * amat[cdm_hidx(j, q)];
      b[i] -= f * b[j];
    }
  }
#pragma unroll
  for (int i = kNP - 1; i >= 0; i--) {
    double acc = b[i];
#pragma unroll
    for (int q = i + 1; q < kNP; q++) acc -= amat[cdm_hidx(i, q)] * x[q];
    x[i] = acc * dinv[i];
  }
}

template <int Gw>
CDM_KERNEL(CDM_NT) cdm_levmar_kernel(CDM_KARG(cdm_lm_args) a) {
  extern __shared__ __align__(16) float sproto[];
  if (!cdm_stage_protocol(a.proto, sproto, a.proto_bytes, a.err)) return;
  const float* ptab = cdm_build_pair_table<Gw>(sproto, a.nmeas_pad, a.nchunk);
  const int v = (int)CDM_BLOCK_IDX * (CDM_NT / Gw) + (int)threadIdx.x / Gw;
  if (v >= a.nvox) return;
  const unsigned gm = cdm_group_mask<Gw>();
  const int lane = (int)threadIdx.x % Gw;
  const cdm_limits& lim = a.lim;

  cdm_voxel_io io;
  io.sig = a.sig + cdm_tile_index(v, 0, lane, a.nchunk, Gw);
  io.chunk_stride = CDM_NT;
  io.nchunk = a.nchunk;
  io.nmeas = a.nmeas;
  io.nmeas_pad = a.nmeas_pad;
  io.lane = lane;
  io.pairs = ptab + (size_t)lane * kNCOLSP * 2;
  io.shells = nullptr;
  io.stab = nullptr;
  io.sig2 = nullptr;

  cdm_real P[kNPS], FixP[kNFIX];
  float Pt[kNP];
  cdm_load_params(a.params + (size_t)v * kNP, P);
  cdm_load_fixp(a.fixp + (size_t)v * a.fixp_tsize, a.fixp_tsize, FixP);
  cdm_lm_inv_transform(lim, P, Pt);
  cdm_update_derived(P, FixP);
  double pcf = cdm_group_sse<Gw>(io, sproto, P, FixP, gm);

  double hess[kNH], g[kNP];
#pragma unroll
  for (int i = 0; i < kNH; i++) hess[i] = 0.0;
#pragma unroll
  for (int i = 0; i < kNP; i++) g[i] = 0.0;
  double lambda = 0.1;
  bool success = true, end = false;
  int iter = 0, passes = 0, nsucc = 0;
  while (!(success && iter++ >= a.max_iters)) {
    passes++;
    if (success) {
      float chain[kNP];
      cdm_lm_chain(lim, Pt, chain);
      float gl[kNP], hl[kNH];
#pragma unroll
      for (int i = 0; i < kNP; i++) gl[i] = 0.0f;
#pragma unroll
      for (int i = 0; i < kNH; i++) hl[i] = 0.0f;
      for (int c = 0; c < io.nchunk; c++) {
        const int m = c * Gw + lane;
        const bool valid = m < io.nmeas;
        cdm_real cf[kNCOLS];
        cdm_load_cfp(sproto, io.nmeas_pad, valid ? m : 0, cf);
        const float y = io.sig[(size_t)c * io.chunk_stride];
        const float r = valid ? (float)Predicted_Signal(NPARAMS, P, cf, FixP) - y : 0.0f;
        cdm_real d[kNP];
        Partial_Derivatives(NPARAMS, P, cf, FixP, d);
        float j[kNP];
#pragma unroll
        for (int i = 0; i < kNP; i++) j[i] = valid ? (float)d[i] * chain[i] : 0.0f;
#pragma unroll
        for (int i = 0; i < kNP; i++) gl[i] = fmaf(r, j[i], gl[i]);
        int k = 0;
#pragma unroll
        for (int i = 0; i < kNP; i++)
#pragma unroll
          for (int q = i; q < kNP; q++) {
            hl[k] = fmaf(j[i], j[q], hl[k]);
            k++;
          }
      }
      // Group sums in FP64; factor 2 of CUDIMOT's gradient/Hessian (:240, :308).
#pragma unroll
      for (int i = 0; i < kNP; i++) g[i] = lim.fixed[i] ? 0.0 : 2.0 * cdm_group_sum<Gw>((double)gl[i], gm);
      int k = 0;
#pragma unroll
      for (int i = 0; i < kNP; i++)
#pragma unroll
        for (int q = i; q < kNP; q++) {
          const double s = 2.0 * cdm_group_sum<Gw>((double)hl[k], gm);
          hess[k++] = (lim.fixed[i] || lim.fixed[q]) ? (i == q ? 1.0 : 0.0) : s;
        }
    }
    double x[kNP];
    cdm_lm_solve(hess, g, lambda, a.marquardt != 0, x);

    float step[kNP];
#pragma unroll
    for (int i = 0; i < kNP; i++) step[i] = Pt[i] - (float)x[i];
    cdm_real Pn[kNPS];
#pragma unroll
    for (int i = 0; i < kNPS; i++) Pn[i] = P[i];
    cdm_lm_transform(lim, Pn, step);
    cdm_update_derived(Pn, FixP);
    const double ncf = cdm_group_sse<Gw>(io, sproto, Pn, FixP, gm);
    success = ncf < pcf;
    if (success) {
      nsucc++;
#pragma unroll
      for (int i = 0; i < kNP; i++) Pt[i] = step[i];
#pragma unroll
      for (int i = 0; i < kNPS; i++) P[i] = Pn[i];
      lambda *= 0.1;
      if (2.0 * fabs(pcf - ncf) <= CDM_LM_CFTOL * (fabs(pcf) + fabs(ncf) + 2.0e-16)) end = true;
      pcf = ncf;
    } else {
      // amat rejected step that moved no parameter at all: larger damping only
      // shrinks the step further, so every later trial is the same point.
      bool moved = false;
#pragma unroll
      for (int i = 0; i < kNP; i++) moved |= (float)Pn[i] != (float)P[i];
      lambda *= 10.0;
      if (lambda > 1.0e20 || !moved) end = true;
      // CUDIMOT re-derives P from Pt after a rejected step (:593), which can
      // nudge Pt at a two-sided bound.
      cdm_lm_transform(lim, P, Pt);
      cdm_update_derived(P, FixP);
    }
    if (end) break;
  }
  FixConstraintsLM(NPARAMS, P);
  if (lane == 0) {
#pragma unroll
    for (int p = 0; p < kNP; p++) {
      // a fixed parameter that FixConstraintsLM left alone keeps its input
      // value in full double precision
      const double in = a.params[(size_t)v * kNP + p];
      a.params[(size_t)v * kNP + p] =
          (lim.fixed[p] && (float)P[p] == (float)in) ? in : (double)(float)P[p];
    }
    if (a.iter_count) atomicAdd(a.iter_count, (unsigned long long)passes);
    if (a.succ_count) atomicAdd(a.succ_count, (unsigned long long)nsucc);
  }
}
