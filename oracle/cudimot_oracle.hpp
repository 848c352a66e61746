// cudimot_oracle.hpp - CPU restatement of CUDIMOT's voxelwise fitting
// kernels. TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke()
// and the CPU baseline of bench.py to check and time the GPU library; the
// library itself never links or calls it.
//
// Included by oracle_capi.cpp after a model plugin (host_prelude.h ->
// modelparameters.h -> macro_numerical.h -> modelfunctions.h ->
// cdm_plugin_tail.h). Templated on the evaluation type T (double for the
// FP64 oracle; fp32 to measure single-precision error on the host).
//
// Each voxel is processed exactly as one warp of the CUDIMOT kernel would:
// sums over measurements are formed as 32 lane-strided partial sums folded
// by the 16/8/4/2/1 shuffle tree (e.g. GridSearch.cu:49-95), so costs are
// rounded in CUDIMOT's order.
//
// Parity pinning: CUDIMOT ships no tests, golden vectors or fixtures. The
// model functions are pinned by building CUDIMOT's own plugins with this
// oracle (oracle/build_oracle.py --reference) and committing their outputs
// under tests/golden/. The fitting loops below are a line-by-line
// restatement (file:line cited per function); MCMC draws come from Philox
// instead of cuRAND's XORWOW, so MCMC is compared statistically.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "cudimot_gb300.h"
#include "philox.h"

namespace orc {

constexpr int kLanes = 32;        // THREADS_VOXEL in every CUDIMOT kernel
constexpr int NP = NPARAMS;
constexpr int NPS = CDM_PSTORE;   // parameters + parameter-derived values

struct Protocol {
  int nmeas = 0;
  int tsize = 0;    // CFP_Tsize
  int stride = 0;   // CFP_Tsize + derived values per measurement
  std::vector<double> cfp;  // [nmeas][stride]
};

inline Protocol make_protocol(int nmeas, int tsize, const double* cfp) {
  Protocol p;
  p.nmeas = nmeas;
  p.tsize = tsize;
  p.stride = tsize + CDM_NDCFP;
  p.cfp.assign((size_t)nmeas * p.stride, 0.0);
  for (int m = 0; m < nmeas; m++) {
    for (int k = 0; k < tsize; k++) p.cfp[(size_t)m * p.stride + k] = cfp[(size_t)m * tsize + k];
#ifdef CDM_DERIVED_CFP
    Derived_CFP<double>(&p.cfp[(size_t)m * p.stride], &p.cfp[(size_t)m * p.stride + tsize]);
#endif
  }
  return p;
}

// Bounds and priors as CUDIMOT's kernels see them: float copies
// (GridSearch.cu:20-23, Levenberg_Marquardt.cu:28-31, MCMC.cu:24-30).
struct Limits {
  int btype[NP];
  float bmin[NP], bmax[NP];
  int ptype[NP];
  float pa[NP], pb[NP];
  int fixed[NP];
};

inline Limits make_limits(const cdm_model_cfg& c) {
  Limits L;
  for (int p = 0; p < NP; p++) {
    L.btype[p] = c.bound_types[p];
    L.bmin[p] = (float)c.bounds_min[p];
    L.bmax[p] = (float)c.bounds_max[p];
    L.ptype[p] = c.prior_types[p];
    L.pa[p] = (float)c.priors_a[p];
    L.pb[p] = (float)c.priors_b[p];
    L.fixed[p] = c.fixed[p];
  }
  return L;
}

// One voxel's view of the inputs, converted to the evaluation type.
template <typename T>
struct Voxel {
  const Protocol* proto;
  std::vector<T> cfp;   // [nmeas][stride]
  std::vector<T> meas;  // [nmeas]
  T fixp[CDM_MAX_BLOCKS * 8 + 1];
  int nmeas;
  int stride;
};

template <typename T>
inline void load_voxel(Voxel<T>& v, const Protocol& pr, const double* meas, const double* fixp,
                       int fixp_tsize) {
  v.proto = &pr;
  v.nmeas = pr.nmeas;
  v.stride = pr.stride;
  if ((int)v.cfp.size() != pr.nmeas * pr.stride) {
    v.cfp.resize((size_t)pr.nmeas * pr.stride);
    for (size_t i = 0; i < v.cfp.size(); i++) v.cfp[i] = (T)pr.cfp[i];
  }
  v.meas.resize(pr.nmeas);
  for (int m = 0; m < pr.nmeas; m++) v.meas[m] = (T)meas[m];
  for (int k = 0; k < fixp_tsize; k++) v.fixp[k] = (T)fixp[k];
}

// 32 lane-strided partial sums folded by the shuffle tree.
template <typename A>
inline A tree_fold(A* part) {
  for (int off = kLanes / 2; off > 0; off >>= 1)
    for (int i = 0; i < off; i++) part[i] += part[i + off];
  return part[0];
}

// Cost_Function (GridSearch.cu:49-95, Levenberg_Marquardt.cu:137-184).
template <typename T>
inline double cost(Voxel<T>& v, T* P) {
  T part[kLanes];
  for (int l = 0; l < kLanes; l++) part[l] = (T)0.0;
  for (int m = 0; m < v.nmeas; m++) {
    T e = Predicted_Signal(NPARAMS, P, &v.cfp[(size_t)m * v.stride], v.fixp);
    e = e - v.meas[m];
    part[m % kLanes] += e * e;
  }
  return (double)tree_fold(part);
}

// ---------------------------------------------------------------- GridSearch
// checkBounds (GridSearch.cu:25-47).
template <typename T>
inline bool gs_check_bounds(const Limits& L, const T* P) {
  for (int p = 0; p < NP; p++) {
    if (L.btype[p] == BMIN) {
      if (P[p] < L.bmin[p]) return false;
    } else if (L.btype[p] == BMAX) {
      if (P[p] > L.bmax[p]) return false;
    } else if (L.btype[p] == BMINMAX) {
      if (P[p] < L.bmin[p]) return false;
      if (P[p] > L.bmax[p]) return false;
    }
  }
  return true;
}

// gridSearch_kernel (GridSearch.cu:97-248): strict '<' keeps the first
// minimum in combination order. Returns the winning combination (-1 if no
// combination was within bounds) and its cost in *best_cost.
template <typename T>
inline int gridsearch_voxel(const Limits& L, int ngp, const int* gparams, int combs,
                            const double* grid, Voxel<T>& v, double* params, double* best_cost) {
  T base[NPS];
  for (int i = 0; i < NP; i++) base[i] = (T)params[i];
  double pcf = 9e20;
  int best = -1;
  T bestP[NPS];
  for (int i = 0; i < NPS; i++) bestP[i] = (i < NP) ? base[i] : (T)0.0;
  // one parameter array across the combinations: its derived slots start at
  // zero (Derived_P's caches count as empty) and then always belong to the
  // previous combination, as the plugin's caches expect
  T trial[NPS];
  for (int i = 0; i < NPS; i++) trial[i] = (i < NP) ? base[i] : (T)0.0;
  for (int c = 0; c < combs; c++) {
    for (int i = 0; i < NP; i++) trial[i] = base[i];
    for (int i = 0; i < ngp; i++) trial[gparams[i]] = (T)grid[(size_t)c * ngp + i];
    if (!gs_check_bounds(L, trial)) continue;
    cdm_update_derived(trial, v.fixp);
    const double ncf = cost(v, trial);
    if (ncf < pcf) {
      pcf = ncf;
      best = c;
      for (int i = 0; i < NP; i++) bestP[i] = trial[i];
    }
  }
  // CUDIMOT keeps the winning combination in T precision.
  for (int i = 0; i < NP; i++) params[i] = (double)bestP[i];
  if (best >= 0) {
    for (int i = 0; i < ngp; i++) params[gparams[i]] = grid[(size_t)best * ngp + i];
  }
  *best_cost = pcf;
  return best;
}

// ------------------------------------------------------ Levenberg-Marquardt
constexpr double kCFTOL = 1.0e-8, kLTOL = 1.0e20, kEPS = 2.0e-16;
constexpr double kTwoDivPI = 0.636619772367581;
constexpr double kAvoid = 1e-4;
constexpr double kSpeed = 10.0;

// MinMaxInvTransform / MinInvTransform / MaxInvTransform and invtransformAll
// (Levenberg_Marquardt.cu:37-103).
template <typename T>
inline void lm_inv_transform(const Limits& L, T* P, T* Pt) {
  for (int p = 0; p < NP; p++) {
    const T lo = (T)L.bmin[p], hi = (T)L.bmax[p];
    if (L.btype[p] == BMIN) {
      Pt[p] = log_gpu(P[p] - lo);
    } else if (L.btype[p] == BMAX) {
      Pt[p] = log_gpu(hi - P[p]);
    } else if (L.btype[p] == BMINMAX) {
      if (P[p] <= lo + (T)kAvoid) P[p] += (T)kAvoid;
      if (P[p] >= hi - (T)kAvoid) P[p] -= (T)kAvoid;
      T t = P[p] - (lo + hi) / (T)2.0;
      t *= ((T)2.0 / ((hi - lo) * (T)kTwoDivPI));
      Pt[p] = (T)tan_gpu(t) * (T)kSpeed;
    } else {
      Pt[p] = P[p];
    }
  }
}

// MinMaxTransform / MinTransform / MaxTransform and transformAll
// (Levenberg_Marquardt.cu:49-118). May nudge Pt for parameters that land
// within 1e-4 of a two-sided bound.
template <typename T>
inline void lm_transform(const Limits& L, T* P, T* Pt) {
  for (int p = 0; p < NP; p++) {
    const T lo = (T)L.bmin[p], hi = (T)L.bmax[p];
    if (L.btype[p] == BMIN) {
      P[p] = exp_gpu(Pt[p]) + lo;
    } else if (L.btype[p] == BMAX) {
      P[p] = hi - exp_gpu(Pt[p]);
    } else if (L.btype[p] == BMINMAX) {
      P[p] = (hi - lo) / (T)2.0;
      P[p] *= atan_gpu(Pt[p] / (T)kSpeed);
      P[p] *= (T)kTwoDivPI;
      P[p] += (lo + hi) / (T)2.0;
      if (P[p] <= lo + (T)kAvoid) {
        P[p] += (T)kAvoid;
        T t = P[p] - (lo + hi) / (T)2.0;
        t *= ((T)2.0 / ((hi - lo) * (T)kTwoDivPI));
        Pt[p] = (T)tan_gpu(t) * (T)kSpeed;
      }
      if (P[p] >= hi - (T)kAvoid) {
        P[p] -= (T)kAvoid;
        T t = P[p] - (lo + hi) / (T)2.0;
        t *= ((T)2.0 / ((hi - lo) * (T)kTwoDivPI));
        Pt[p] = (T)tan_gpu(t) * (T)kSpeed;
      }
    } else {
      P[p] = Pt[p];
    }
  }
}

// derivative_transf (Levenberg_Marquardt.cu:120-135). The bound span is a
// float difference, as in CUDIMOT (both operands are float constants).
template <typename T>
inline void lm_derivative_transf(const Limits& L, const T* Pt, T* d) {
  for (int p = 0; p < NP; p++) {
    if (L.btype[p] == BMIN) {
      d[p] = d[p] * exp_gpu(Pt[p]);
    } else if (L.btype[p] == BMAX) {
      d[p] = d[p] * (-exp_gpu(Pt[p]));
    } else if (L.btype[p] == BMINMAX) {
      const float span = L.bmax[p] - L.bmin[p];
      d[p] = d[p] * ((T)span / (T)2.0) * (T)kTwoDivPI;
      d[p] = d[p] * ((T)kSpeed / ((T)kSpeed * (T)kSpeed + Pt[p] * Pt[p]));
    }
  }
}

// Calculate_Gradient and Calculate_Hessian (Levenberg_Marquardt.cu:186-332):
// per 32-measurement chunk, each entry is folded over the lanes and added
// to the running sum; fixed parameters get zero gradient and identity rows.
template <typename T>
inline void lm_gradient_hessian(const Limits& L, Voxel<T>& v, T* P, const T* Pt, T* grad,
                                T* hess) {
  const int chunks = (v.nmeas + kLanes - 1) / kLanes;
  for (int p = 0; p < NP; p++) grad[p] = (T)0.0;
  for (int i = 0; i < NP * NP; i++) hess[i] = (T)0.0;
  std::vector<T> r(kLanes), J((size_t)kLanes * NP);
  for (int c = 0; c < chunks; c++) {
    for (int l = 0; l < kLanes; l++) {
      const int m = c * kLanes + l;
      r[l] = (T)0.0;
      for (int p = 0; p < NP; p++) J[(size_t)l * NP + p] = (T)0.0;
      if (m < v.nmeas) {
        T* cf = &v.cfp[(size_t)m * v.stride];
        T e = Predicted_Signal(NPARAMS, P, cf, v.fixp);
        r[l] = e - v.meas[m];
        Partial_Derivatives(NPARAMS, P, cf, v.fixp, &J[(size_t)l * NP]);
        lm_derivative_transf(L, Pt, &J[(size_t)l * NP]);
      }
    }
    T part[kLanes];
    for (int p = 0; p < NP; p++) {
      for (int l = 0; l < kLanes; l++) part[l] = (T)2.0 * r[l] * J[(size_t)l * NP + p];
      grad[p] += tree_fold(part);
      if (L.fixed[p]) grad[p] = (T)0.0;
    }
    for (int p = 0; p < NP; p++)
      for (int q = 0; q < NP; q++) {
        for (int l = 0; l < kLanes; l++)
          part[l] = (T)2.0 * J[(size_t)l * NP + p] * J[(size_t)l * NP + q];
        hess[p * NP + q] += tree_fold(part);
      }
  }
  for (int p = 0; p < NP; p++)
    for (int q = 0; q < NP; q++)
      if (L.fixed[p] || L.fixed[q]) hess[p * NP + q] = (p == q) ? (T)1.0 : (T)0.0;
}

// LUsolver (Levenberg_Marquardt.cu:334-407): Gauss-Jordan on [H | g]
// without pivoting; lane j of the warp holds column j.
template <typename T>
inline void lm_solve(const T* hess, const T* grad, T* x) {
  T M[NP][NP + 1];
  for (int p = 0; p < NP; p++) {
    for (int q = 0; q < NP; q++) M[p][q] = hess[p * NP + q];
    M[p][NP] = grad[p];
  }
  for (int col = 0; col < NP; col++) {
    const T piv = M[col][col];
    for (int j = 0; j <= NP; j++) M[col][j] = M[col][j] / piv;
    for (int row = col + 1; row < NP; row++) {
      const T f = M[row][col];
      for (int j = 0; j <= NP; j++) M[row][j] -= f * M[col][j];
    }
  }
  for (int col = NP - 1; col > 0; col--)
    for (int row = 0; row < col; row++) {
      const T f = M[row][col];
      for (int j = 0; j <= NP; j++) M[row][j] -= f * M[col][j];
    }
  for (int p = 0; p < NP; p++) x[p] = M[p][NP];
}

struct LMResult {
  int iterations = 0;  // loop passes
  int successes = 0;
  double cost = 0.0;
};

// levenberg_kernel (Levenberg_Marquardt.cu:409-623).
template <typename T>
inline LMResult levmar_voxel(const Limits& L, int max_iters, bool marquardt, Voxel<T>& v,
                             double* params) {
  LMResult res;
  T P[NPS], Pt[NP], grad[NP], hess[NP * NP], step[NP];
  for (int i = 0; i < NPS; i++) P[i] = (i < NP) ? (T)params[i] : (T)0.0;
  double lambda = 0.1, olambda = 0.0;
  bool success = true, end = false;
  lm_inv_transform(L, P, Pt);
  cdm_update_derived(P, v.fixp);
  double pcf = cost(v, P);
  int iter = 0;
  while (!(success && iter++ >= max_iters)) {
    res.iterations++;
    if (success) lm_gradient_hessian(L, v, P, Pt, grad, hess);
    for (int i = 0; i < NP; i++) {
      if (marquardt)
        hess[i * NP + i] = (T)((1 + lambda) / (1 + olambda)) * hess[i * NP + i];
      else
        hess[i * NP + i] += (T)(lambda - olambda);
    }
    lm_solve(hess, grad, step);
    for (int p = 0; p < NP; p++) step[p] = Pt[p] - step[p];
    lm_transform(L, P, step);
    cdm_update_derived(P, v.fixp);
    const double ncf = cost(v, P);
    if ((success = (ncf < pcf))) {
      res.successes++;
      olambda = 0.0;
      for (int p = 0; p < NP; p++) Pt[p] = step[p];
      lambda = lambda / 10.0;
      if (2.0 * std::fabs(pcf - ncf) <= kCFTOL * (std::fabs(pcf) + std::fabs(ncf) + kEPS))
        end = true;
      pcf = ncf;
    } else {
      olambda = lambda;
      lambda = lambda * 10.0;
      if (lambda > kLTOL) end = true;
      lm_transform(L, P, Pt);
      cdm_update_derived(P, v.fixp);
    }
    if (end) break;
  }
  FixConstraintsLM(NPARAMS, P);
  for (int i = 0; i < NP; i++) params[i] = (double)P[i];
  res.cost = pcf;
  return res;
}

// --------------------------------------------------------------------- MCMC
// logIo (MCMC.cu:32-68): log of the modified Bessel function I0 with the
// polynomial approximations of Abramowitz & Stegun 9.8.1/9.8.2.
template <typename T>
inline T log_bessel_i0(T x) {
  const T b = fabs_gpu(x);
  if (b < (T)3.75) {
    T a = x / (T)3.75;
    a *= a;
    const T y = (T)1.0 + a * ((T)3.5156229 + a * ((T)3.0899424 + a * ((T)1.2067492 +
                a * ((T)0.2659732 + a * ((T)0.0360768 + a * (T)0.0045813)))));
    return log_gpu(y);
  }
  const T a = (T)3.75 / b;
  return b + log_gpu(((T)0.39894228 + a * ((T)0.01328592 + a * ((T)0.00225319 +
             a * ((T)-0.00157565 + a * ((T)0.00916281 + a * ((T)-0.02057706 +
             a * ((T)0.02635537 + a * ((T)-0.01647633 + a * (T)0.00392377)))))))) /
             (T)sqrt_gpu(b));
}

// Compute_prior for one parameter (MCMC.cu:162-191).
template <typename T>
inline T mcmc_prior(const Limits& L, int p, T* P, int nmeas, T* cfp_all, T* fixp) {
  switch (L.ptype[p]) {
    case GAUSSPRIOR: {
      const T s2 = (T)L.pb[p] * (T)L.pb[p];
      return (P[p] - (T)L.pa[p]) * (P[p] - (T)L.pa[p]) / ((T)2 * s2);
    }
    case GAMMAPRIOR:
      return ((T)1.0 - (T)L.pa[p]) * log_gpu(P[p]) + (T)L.pb[p] * P[p];
    case ARDPRIOR:
      return (T)L.pa[p] * log_gpu(P[p]);
    case SINPRIOR:
      return -log_gpu(fabs_gpu(sin_gpu(P[p]) / (T)2.0));
    case CUSTOM:
      return custom_priors(p, P, nmeas, cfp_all, fixp);
    default:
      return (T)0.0;
  }
}

// Check_bounds_constraints (MCMC.cu:141-160).
template <typename T>
inline bool mcmc_in_bounds(const Limits& L, int p, T* P) {
  if (!ConstraintsMCMC(NPARAMS, P)) return false;
  if (L.btype[p] == BMIN) return !(P[p] < L.bmin[p]);
  if (L.btype[p] == BMAX) return !(P[p] > L.bmax[p]);
  if (L.btype[p] == BMINMAX) return !(P[p] < L.bmin[p]) && !(P[p] > L.bmax[p]);
  return true;
}

// Compute_Likelihood (MCMC.cu:254-307).
template <typename T>
inline T mcmc_likelihood(Voxel<T>& v, T* P, bool rician, T tau) {
  T part[kLanes];
  for (int l = 0; l < kLanes; l++) part[l] = (T)0.0;
  for (int m = 0; m < v.nmeas; m++) {
    T s = Predicted_Signal(NPARAMS, P, &v.cfp[(size_t)m * v.stride], v.fixp);
    if (rician) {
      const T y = v.meas[m];
      part[m % kLanes] += log_gpu(y) + (-(T)0.5 * tau * (y * y + s * s) + log_bessel_i0(tau * s * y));
    } else {
      s = s - v.meas[m];
      part[m % kLanes] += s * s;
    }
  }
  const T acc = tree_fold(part);
  if (rician) return -(T)v.nmeas * log_gpu(tau) - acc;
  return ((T)v.nmeas / (T)2.0) * log_gpu(acc / (T)2.0);
}

struct MCMCOpts {
  int nburn, njumps, sampleevery, update_proposal, rician;
  uint64_t seed;
  uint32_t stream;
};

// mcmc_kernel burn-in launch followed by the recording launch
// (MCMC.cu:327-683, launches :799-847), one voxel. Draws: Philox with
// counter (voxel, global iteration, parameter slot, stream).
template <typename T>
inline void mcmc_voxel(const Limits& L, const MCMCOpts& o, uint32_t voxel_id, Voxel<T>& v,
                       double* params, double* samples, double* tau_out, int nsamples) {
  T P[NPS], prior[NP], propSD[NP];
  int acc[NP], rej[NP];
  T tau = (T)0.0, tauSD = (T)0.0;
  int tacc = 0, trej = 0;
  for (int i = 0; i < NPS; i++) P[i] = (i < NP) ? (T)params[i] : (T)0.0;
  for (int p = 0; p < NP; p++) propSD[p] = P[p] / (T)10.0;  // MCMC.cu:428
  const int nburn = o.nburn < 1 ? 1 : o.nburn;                 // MCMC.cu:702-703
  T* cfp_all = v.cfp.data();
  for (int phase = 0; phase < 2; phase++) {
    const bool recording = (phase == 1);
    const int niters = recording ? o.njumps : nburn;
    // Initialize_priors_params (MCMC.cu:97-139) and Compute_TotalPrior.
    for (int p = 0; p < NP; p++) {
      acc[p] = rej[p] = 0;
      if (L.btype[p] == BMIN) {
        if (P[p] < L.bmin[p]) P[p] = (T)L.bmin[p];
      } else if (L.btype[p] == BMAX) {
        if (P[p] > L.bmax[p]) P[p] = (T)L.bmax[p];
      } else if (L.btype[p] == BMINMAX) {
        if (P[p] < L.bmin[p]) P[p] = (T)L.bmin[p];
        else if (P[p] > L.bmax[p]) P[p] = (T)L.bmax[p];
      }
    }
    cdm_update_derived(P, v.fixp);
    for (int p = 0; p < NP; p++) prior[p] = mcmc_prior(L, p, P, v.nmeas, cfp_all, v.fixp);
    tacc = trej = 0;
    if (o.rician && !recording) {
      // Initialise_TauRician (MCMC.cu:193-251): 1 / variance of residuals.
      T part[kLanes];
      for (int l = 0; l < kLanes; l++) part[l] = (T)0.0;
      for (int m = 0; m < v.nmeas; m++) {
        T e = Predicted_Signal(NPARAMS, P, &v.cfp[(size_t)m * v.stride], v.fixp);
        part[m % kLanes] += e - v.meas[m];
      }
      const T mean = tree_fold(part) / (T)v.nmeas;
      for (int l = 0; l < kLanes; l++) part[l] = (T)0.0;
      for (int m = 0; m < v.nmeas; m++) {
        T e = Predicted_Signal(NPARAMS, P, &v.cfp[(size_t)m * v.stride], v.fixp);
        e = mean - (e - v.meas[m]);
        part[m % kLanes] += e * e;
      }
      tau = (T)1.0 / (tree_fold(part) / (T)v.nmeas);
      tauSD = tau / (T)2.0;
    }
    T total_prior = (T)0.0;
    for (int p = 0; p < NP; p++) total_prior += prior[p];
    T like = mcmc_likelihood(v, P, o.rician != 0, tau);
    T energy = total_prior + like;
    for (int it = 0; it < niters; it++) {
      const uint32_t git = (uint32_t)(recording ? nburn + it : it);
      if (o.rician) {
        const cdm_draw d = cdm_mcmc_draw(o.seed, voxel_id, git, CDM_RNG_SLOT_TAU, o.stream);
        const T old = tau;
        tau = tau + (T)d.normal * tauSD;
        if (tau > (T)0.0) {
          const T nl = mcmc_likelihood(v, P, true, tau);
          total_prior = (T)0.0;
          for (int p = 0; p < NP; p++) total_prior += prior[p];
          const T ne = total_prior + nl;
          const T old_e = energy;
          if ((T)exp_gpu(old_e - ne) > (T)d.uniform) {
            tacc++;
            energy = ne;
          } else {
            trej++;
            tau = old;
            energy = old_e;
          }
        } else {
          trej++;
          tau = old;
        }
      }
      for (int p = 0; p < NP; p++) {
        if (L.fixed[p]) {
          // A fixed parameter is re-proposed at its own value: same energy,
          // accepted with probability 1 (MCMC.cu:72-76); no draw is needed.
          acc[p]++;
          continue;
        }
        const cdm_draw d = cdm_mcmc_draw(o.seed, voxel_id, git, (uint32_t)p, o.stream);
        const T old = P[p];
        T saved[NPS];
        for (int i = 0; i < NPS; i++) saved[i] = P[i];
        P[p] = P[p] + (T)d.normal * propSD[p];
        if (mcmc_in_bounds(L, p, P)) {
          cdm_update_derived(P, v.fixp);
          const T nl = mcmc_likelihood(v, P, o.rician != 0, tau);
          const T old_prior = prior[p];
          prior[p] = mcmc_prior(L, p, P, v.nmeas, cfp_all, v.fixp);
          total_prior = (T)0.0;
          for (int q = 0; q < NP; q++) total_prior += prior[q];
          const T ne = total_prior + nl;
          const T old_e = energy;
          if ((T)exp_gpu(old_e - ne) > (T)d.uniform) {
            acc[p]++;
            energy = ne;
          } else {
            rej[p]++;
            for (int i = 0; i < NPS; i++) P[i] = saved[i];
            prior[p] = old_prior;
            energy = old_e;
          }
        } else {
          rej[p]++;
          P[p] = old;
        }
      }
      if (recording && (it % o.sampleevery) == 0) {
        const int s = it / o.sampleevery;
        if (s < nsamples) {
          for (int p = 0; p < NP; p++) samples[(size_t)p * nsamples + s] = (double)P[p];
          if (o.rician && tau_out) tau_out[s] = (double)tau;
        }
      }
      if (!recording || o.update_proposal) {
        if (it > 0 && (it % o.sampleevery) == 0) {  // updateproposalevery = se (MCMC.cu:711)
          for (int p = 0; p < NP; p++) {
            propSD[p] *= (T)sqrt_gpu(((T)acc[p] + (T)1.0) / ((T)rej[p] + (T)1.0));
            propSD[p] = min_gpu(propSD[p], (T)1e10);
            acc[p] = rej[p] = 0;
          }
          if (o.rician) {
            tauSD *= (T)sqrt_gpu(((T)tacc + (T)1.0) / ((T)trej + (T)1.0));
            tauSD = min_gpu(tauSD, (T)1e10);
            tacc = trej = 0;
          }
        }
      }
    }
  }
  for (int p = 0; p < NP; p++) params[p] = (double)P[p];
}

// ------------------------------------------------- BIC/AIC, PredictedSignal
// Mean of the samples as the leader lane forms it (BIC_AIC.cu:160-188,
// getPredictedSignal.cu:63-79).
template <typename T>
inline void sample_mean(const double* s, int nsamples, T* P) {
  for (int p = 0; p < NP; p++) {
    if (nsamples > 1) {
      T acc = (T)0.0;
      for (int k = 0; k < nsamples; k++) acc += (T)s[(size_t)p * nsamples + k];
      P[p] = acc / (T)nsamples;
    } else {
      P[p] = (T)s[p];
    }
  }
}

// Compute_BIC_AIC (BIC_AIC.cu:61-110).
template <typename T>
inline void bic_aic_voxel(Voxel<T>& v, const double* s, int nsamples, bool rician,
                          const double* tau_s, double* bic, double* aic) {
  T P[NPS];
  for (int i = 0; i < NPS; i++) P[i] = (T)0.0;
  sample_mean(s, nsamples, P);
  T tau = (T)0.0;
  if (rician) {
    if (nsamples > 1) {
      T acc = (T)0.0;
      for (int k = 0; k < nsamples; k++) acc += (T)tau_s[k];
      tau = acc / (T)nsamples;
    } else {
      tau = (T)tau_s[0];
    }
  }
  cdm_update_derived(P, v.fixp);
  T part[kLanes];
  for (int l = 0; l < kLanes; l++) part[l] = (T)0.0;
  for (int m = 0; m < v.nmeas; m++) {
    T e = Predicted_Signal(NPARAMS, P, &v.cfp[(size_t)m * v.stride], v.fixp);
    if (rician) {
      const T y = v.meas[m];
      part[m % kLanes] += log_gpu(y) + (-(T)0.5 * tau * (y * y + e * e) + log_bessel_i0(tau * e * y));
    } else {
      e = e - v.meas[m];
      part[m % kLanes] += e * e;
    }
  }
  const T acc = tree_fold(part);
  int np = NPARAMS;
  T b;
  if (rician) {
    np++;
    b = (T)v.nmeas * log_gpu(tau) + acc;
  } else {
    b = -((T)v.nmeas / (T)2.0) * log_gpu(acc / (T)2.0);
  }
  *aic = (double)((T)-2.0 * b + (T)np * (T)2.0);
  *bic = (double)((T)-2.0 * b + (T)np * log_gpu((T)v.nmeas));
}

// getPredictedSignal_kernel (getPredictedSignal.cu:22-92).
template <typename T>
inline void predicted_voxel(Voxel<T>& v, const double* s, int nsamples, double* pred) {
  T P[NPS];
  for (int i = 0; i < NPS; i++) P[i] = (T)0.0;
  sample_mean(s, nsamples, P);
  cdm_update_derived(P, v.fixp);
  for (int m = 0; m < v.nmeas; m++)
    pred[m] = (double)Predicted_Signal(NPARAMS, P, &v.cfp[(size_t)m * v.stride], v.fixp);
}

}  // namespace orc
