// cdm_plugin_tail.h - included right after a plugin's modelfunctions.h.
//
// Defines the numerical derivative and the uniform access to the two
// optional plugin hooks:
//   CDM_DERIVED_CFP n + Derived_CFP(const double* cfp, double* d):
//       n protocol-only values per measurement, computed once per protocol
//       in double and appended after the plugin's CFP values;
//   CDM_DERIVED_P n + Derived_P(T* P, T* FixP):
//       n parameter-only values, recomputed after every parameter change
//       and stored in P[NPARAMS .. NPARAMS+n-1].
// Plugins written for CUDIMOT define neither and behave exactly as there.
#pragma once

#ifdef CDM_DERIVED_CFP
#define CDM_NDCFP CDM_DERIVED_CFP
#else
#define CDM_NDCFP 0
#endif
#ifdef CDM_DERIVED_P
#define CDM_NDP CDM_DERIVED_P
#else
#define CDM_NDP 0
#endif
// Length of the parameter array the kernels hand to the plugin.
#define CDM_PSTORE (NPARAMS + CDM_NDP)

template <typename T>
__device__ inline void cdm_update_derived(T* P, T* FixP) {
#ifdef CDM_DERIVED_P
  Derived_P(P, FixP);
#endif
}

// Step rule for the central difference. For T = double (and float) it is
// CUDIMOT's (macro_numerical.h:15-32): h = clamp(TINY*|p|, MINSTEP, MAXSTEP).
// That rule is tuned for double: in single precision a 1e-5 relative step
// leaves 2-3 significant digits in S(p+h/2) - S(p-h/2). For the fp32
// evaluation type the relative step is eps^(1/3) ~ 5e-3 (the usual optimum
// of a central difference) with a floor of 1e-4, which keeps the
// derivative error near 1e-5 relative.
template <typename T> struct cdm_step_rule {
  static constexpr double tiny = TINY, minstep = MINSTEP, maxstep = MAXSTEP;
};
template <> struct cdm_step_rule<fp32> {
  static constexpr double tiny = 4.8828125e-3, minstep = 1e-4, maxstep = MAXSTEP;
};

// dS/dp = (S(p+h/2) - S(p-h/2)) / h. The divisor is the difference of the
// two evaluation points as actually rounded (equal to h in double for
// CUDIMOT's steps). With Derived_P the derived values are refreshed for each
// perturbed point and restored afterwards.
MACRO T numerical(int idpar, T* P, T* CFP, T* FixP) {
  T h = fabs_gpu(P[idpar]) * (T)cdm_step_rule<T>::tiny;
  h = min_gpu(max_gpu(h, (T)cdm_step_rule<T>::minstep), (T)cdm_step_rule<T>::maxstep);
  const T p0 = P[idpar];
  const T half = h * (T)0.5;
#if CDM_NDP > 0
  T saved[CDM_NDP];
#pragma unroll
  for (int k = 0; k < CDM_NDP; k++) saved[k] = P[NPARAMS + k];
#endif
  const T pu = p0 + half;
  const T pd = pu - (half + half);
  P[idpar] = pu;
  cdm_update_derived(P, FixP);
  const T up = Predicted_Signal(NPARAMS, P, CFP, FixP);
  P[idpar] = pd;
  cdm_update_derived(P, FixP);
  const T down = Predicted_Signal(NPARAMS, P, CFP, FixP);
  P[idpar] = p0;
#if CDM_NDP > 0
#pragma unroll
  for (int k = 0; k < CDM_NDP; k++) P[NPARAMS + k] = saved[k];
#endif
  return (up - down) / (pu - pd);
}
