// macro_numerical.h - numerical partial derivatives for model plugins,
// used as `derivatives[i] = NUMERICAL(i);`.
//
// Keeps the macro names CUDIMOT plugins rely on (macro_numerical.h:1-6 in
// CUDIMOT: MACRO, NUMERICAL, TINY, MAXSTEP, MINSTEP, nonzerosign); some
// plugins reuse TINY/MINSTEP/MAXSTEP in their own step helpers, so the
// values are kept too. `numerical` is only declared here; its definition is
// in cdm_plugin_tail.h, included after the plugin, because it must know
// whether the plugin provides the optional Derived_P hook.
#pragma once

#define MACRO template <typename T> __device__ inline
#define NUMERICAL(idpar) numerical(idpar, P, CFP, FixP);
#define TINY 1e-5
#define MAXSTEP 0.2
#define MINSTEP 1e-6
#define nonzerosign(a) ((a) < 0 ? -1 : 1)

MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP);
MACRO T numerical(int idpar, T* P, T* CFP, T* FixP);
