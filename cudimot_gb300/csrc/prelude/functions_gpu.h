// functions_gpu.h - math prelude seen by CUDIMOT model plugins.
//
// Plugins call `*_gpu` wrappers (functions_gpu.h:4-40 in CUDIMOT) and the
// warp helpers `shfl`/`shfl_down` (functions_gpu.h:45-99). This header keeps
// every one of those names and signatures so an unchanged plugin compiles.
// Differences from CUDIMOT, all deliberate:
//  * float arguments give float results for sqrt/tan/atan2/acos/pow; CUDIMOT
//    promotes those five to double even in float builds, which would put
//    FP64 work on GB300's narrow FP64 pipe.
//  * overloads for `fp32` (fp32.h), the type the GPU kernels instantiate
//    plugins with, run the float versions.
//  * mixed-type calls (e.g. pow_gpu(x, 2)) resolve through templates
//    instead of failing on ambiguity.
// The same header builds for the host (oracle/host_prelude.h defines
// __device__ away first), where the double overloads give the FP64 oracle.
#pragma once

#include <cmath>
#include "cudimot.h"
#include "fp32.h"

#ifndef FUNC
#define FUNC __device__ inline
#endif

#if !defined(__CUDACC__)
#include <algorithm>
using std::sqrt; using std::exp; using std::log; using std::sin; using std::cos;
using std::tan; using std::atan; using std::atan2; using std::acos; using std::pow;
using std::fabs; using std::fmin; using std::fmax; using std::erf;
#endif

#define CDM_UNARY(NAME, FF, DF)                                   \
  FUNC float NAME(float x) { return FF(x); }                      \
  FUNC double NAME(double x) { return DF(x); }                    \
  FUNC fp32 NAME(fp32 x) { return fp32(FF(x.v)); }

CDM_UNARY(log_gpu, logf, log)
// Build option CDM_FAST_EXP: fp32 exp through the hardware ex2 approximation
// (__expf, a few ulp more error) instead of the correctly rounded-ish expf.
#if defined(CDM_FAST_EXP) && defined(__CUDA_ARCH__)
FUNC float exp_gpu(float x) { return expf(x); }
FUNC double exp_gpu(double x) { return exp(x); }
FUNC fp32 exp_gpu(fp32 x) { return fp32(__expf(x.v)); }
#else
CDM_UNARY(exp_gpu, expf, exp)
#endif
CDM_UNARY(fabs_gpu, fabsf, fabs)
CDM_UNARY(sin_gpu, sinf, sin)
CDM_UNARY(cos_gpu, cosf, cos)
CDM_UNARY(atan_gpu, atanf, atan)
CDM_UNARY(tan_gpu, tanf, tan)
CDM_UNARY(sqrt_gpu, sqrtf, sqrt)
CDM_UNARY(acos_gpu, acosf, acos)
#undef CDM_UNARY

// rcp_gpu(x) = 1/x for the inner steps of iterative solvers in plugins: in
// single precision the hardware reciprocal approximation (__fdividef, 2 ulp)
// instead of the IEEE-rounded division sequence; exact 1/x in double.
#if defined(__CUDA_ARCH__)
FUNC float rcp_gpu(float x) { return __fdividef(1.0f, x); }
FUNC fp32 rcp_gpu(fp32 x) { return fp32(__fdividef(1.0f, x.v)); }
#else
FUNC float rcp_gpu(float x) { return 1.0f / x; }
FUNC fp32 rcp_gpu(fp32 x) { return fp32(1.0f / x.v); }
#endif
FUNC double rcp_gpu(double x) { return 1.0 / x; }

// Integer arguments (e.g. sqrt_gpu(3)) follow C's promotion to double.
template <class I, class = typename std::enable_if<std::is_integral<I>::value>::type>
FUNC double sqrt_gpu(I x) { return sqrt((double)x); }

// Two-argument wrappers: the result type follows cdm_math_result (fp32 wins,
// otherwise the ordinary arithmetic type of the two arguments).
template <class R> struct cdm_bin;
template <> struct cdm_bin<float> {
  static FUNC float mn(float a, float b) { return fminf(a, b); }
  static FUNC float mx(float a, float b) { return fmaxf(a, b); }
  static FUNC float at2(float a, float b) { return atan2f(a, b); }
  static FUNC float pw(float a, float b) { return powf(a, b); }
};
template <> struct cdm_bin<double> {
  static FUNC double mn(double a, double b) { return fmin(a, b); }
  static FUNC double mx(double a, double b) { return fmax(a, b); }
  static FUNC double at2(double a, double b) { return atan2(a, b); }
  static FUNC double pw(double a, double b) { return pow(a, b); }
};
template <> struct cdm_bin<fp32> {
  static FUNC fp32 mn(fp32 a, fp32 b) { return fp32(fminf(a.v, b.v)); }
  static FUNC fp32 mx(fp32 a, fp32 b) { return fp32(fmaxf(a.v, b.v)); }
  static FUNC fp32 at2(fp32 a, fp32 b) { return fp32(atan2f(a.v, b.v)); }
  static FUNC fp32 pw(fp32 a, fp32 b) { return fp32(powf(a.v, b.v)); }
};
template <> struct cdm_bin<int> : cdm_bin<double> {};
template <> struct cdm_bin<long> : cdm_bin<double> {};

template <class A, class B>
FUNC typename cdm_math_result<A, B>::type min_gpu(A a, B b) {
  typedef typename cdm_math_result<A, B>::type R;
  return cdm_bin<R>::mn(R(a), R(b));
}
template <class A, class B>
FUNC typename cdm_math_result<A, B>::type max_gpu(A a, B b) {
  typedef typename cdm_math_result<A, B>::type R;
  return cdm_bin<R>::mx(R(a), R(b));
}
template <class A, class B>
FUNC typename cdm_math_result<A, B>::type atan2_gpu(A a, B b) {
  typedef typename cdm_math_result<A, B>::type R;
  return cdm_bin<R>::at2(R(a), R(b));
}
template <class A, class B>
FUNC typename cdm_math_result<A, B>::type pow_gpu(A a, B b) {
  typedef typename cdm_math_result<A, B>::type R;
  return cdm_bin<R>::pw(R(a), R(b));
}

// Warp helpers some plugins may call. Full-warp masks, as in CUDIMOT.
#if defined(__CUDACC__)
FUNC double shfl_down(double x, unsigned s) { return __shfl_down_sync(0xFFFFFFFFu, x, s); }
FUNC float shfl_down(float x, unsigned s) { return __shfl_down_sync(0xFFFFFFFFu, x, s); }
FUNC fp32 shfl_down(fp32 x, unsigned s) { return fp32(__shfl_down_sync(0xFFFFFFFFu, x.v, s)); }
FUNC double shfl(double x, int s) { return __shfl_sync(0xFFFFFFFFu, x, s); }
FUNC float shfl(float x, unsigned s) { return __shfl_sync(0xFFFFFFFFu, x, s); }
FUNC fp32 shfl(fp32 x, int s) { return fp32(__shfl_sync(0xFFFFFFFFu, x.v, s)); }
FUNC int shfl(int x, int s) { return __shfl_sync(0xFFFFFFFFu, x, s); }
#endif
