// cdm_flops.cpp - operation counts of a model plugin, for the roofline.
//
// The plugin is compiled for the host with a counting number type: every
// +, -, *, / on it adds one to `flops`, every *_gpu math call adds one to
// `mufu` (transcendental or square root). Counting Derived_P separately from
// Predicted_Signal gives the work done once per parameter change and the
// work done per measurement. Built per model by cudimot_gb300/build.py.
#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <algorithm>
using std::max;
using std::min;
#include "functions_gpu.h"

namespace {
thread_local int64_t g_flops = 0, g_mufu = 0;
}

struct cnt {
  double v;
  cnt() = default;
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
  cnt(U x) : v((double)x) {}
  cnt(fp32 x) : v((double)x.v) {}
  operator double() const { return v; }
  cnt& operator+=(cnt o) { g_flops++; v += o.v; return *this; }
  cnt& operator-=(cnt o) { g_flops++; v -= o.v; return *this; }
  cnt& operator*=(cnt o) { g_flops++; v *= o.v; return *this; }
  cnt& operator/=(cnt o) { g_flops++; v /= o.v; return *this; }
};
inline cnt operator-(cnt a) { return cnt(-a.v); }
#define CNT_BIN(OP)                                                                      \
  inline cnt operator OP(cnt a, cnt b) { g_flops++; return cnt(a.v OP b.v); }            \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  inline cnt operator OP(cnt a, U b) { g_flops++; return cnt(a.v OP (double)b); }        \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  inline cnt operator OP(U a, cnt b) { g_flops++; return cnt((double)a OP b.v); }
CNT_BIN(+) CNT_BIN(-) CNT_BIN(*) CNT_BIN(/)
#define CNT_CMP(OP)                                                                      \
  inline bool operator OP(cnt a, cnt b) { return a.v OP b.v; }                           \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  inline bool operator OP(cnt a, U b) { return a.v OP (double)b; }                       \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  inline bool operator OP(U a, cnt b) { return (double)a OP b.v; }
CNT_CMP(<) CNT_CMP(>) CNT_CMP(<=) CNT_CMP(>=) CNT_CMP(==) CNT_CMP(!=)
#define CNT_MUFU(NAME, F) \
  inline cnt NAME(cnt x) { g_mufu++; return cnt(F(x.v)); }
CNT_MUFU(log_gpu, std::log) CNT_MUFU(exp_gpu, std::exp) CNT_MUFU(sin_gpu, std::sin)
CNT_MUFU(cos_gpu, std::cos) CNT_MUFU(atan_gpu, std::atan) CNT_MUFU(tan_gpu, std::tan)
CNT_MUFU(sqrt_gpu, std::sqrt) CNT_MUFU(acos_gpu, std::acos)
inline cnt fabs_gpu(cnt x) { return cnt(std::fabs(x.v)); }
inline cnt rcp_gpu(cnt x) { g_mufu++; return cnt(1.0 / x.v); }
template <> struct cdm_bin<cnt> {
  static cnt mn(cnt a, cnt b) { return cnt(std::fmin(a.v, b.v)); }
  static cnt mx(cnt a, cnt b) { return cnt(std::fmax(a.v, b.v)); }
  static cnt at2(cnt a, cnt b) { g_mufu++; return cnt(std::atan2(a.v, b.v)); }
  static cnt pw(cnt a, cnt b) { g_mufu++; return cnt(std::pow(a.v, b.v)); }
};
template <class B> struct cdm_math_result<cnt, B> { typedef cnt type; };
template <class A> struct cdm_math_result<A, cnt> { typedef cnt type; };
template <> struct cdm_math_result<cnt, cnt> { typedef cnt type; };

#include "modelparameters.h"
#include "macro_numerical.h"
#include "modelfunctions.h"
#include "cdm_plugin_tail.h"
#include "cdm_model_sizes.h"

constexpr int kNCOLS = CDM_CFP_TSIZE + CDM_NDCFP;

// out[0] = FLOPs of Derived_P from scratch, out[1] = FLOPs of
// Predicted_Signal per measurement, out[2] = FLOPs of Partial_Derivatives per
// measurement; out[3..5] the same for transcendental/sqrt calls; out[6]/[7]
// FLOPs/transcendentals of Derived_P after a change of one parameter (the
// sampler's case; plugins may reuse cached parameter-only blocks), averaged
// over the parameters. Averaged over the nvox parameter vectors and nmeas
// measurements given.
extern "C" int cdm_count_ops(int nvox, const double* params, int nmeas, const double* cfp,
                             const double* fixp, double* out) {
  int64_t fd = 0, fs = 0, fj = 0, md = 0, ms = 0, mj = 0, fw = 0, mw = 0;
  for (int v = 0; v < nvox; v++) {
    cnt P[CDM_PSTORE], F[CDM_FIXP_TSIZE + 1], d[NPARAMS];
    for (int i = 0; i < CDM_PSTORE; i++) P[i] = i < NPARAMS ? params[(size_t)v * NPARAMS + i] : 0.0;
    for (int k = 0; k < CDM_FIXP_TSIZE; k++) F[k] = fixp[(size_t)v * CDM_FIXP_TSIZE + k];
    g_flops = g_mufu = 0;
    cdm_update_derived(P, F);
    fd += g_flops;
    md += g_mufu;
    for (int p = 0; p < NPARAMS; p++) {
      const cnt keep = P[p];
      P[p] = P[p].v * (1.0 + 1e-3) + 1e-6;
      g_flops = g_mufu = 0;
      cdm_update_derived(P, F);
      fw += g_flops;
      mw += g_mufu;
      P[p] = keep;
      cdm_update_derived(P, F);
    }
    for (int m = 0; m < nmeas; m++) {
      double raw[kNCOLS];
      for (int k = 0; k < CDM_CFP_TSIZE; k++) raw[k] = cfp[(size_t)m * CDM_CFP_TSIZE + k];
#ifdef CDM_DERIVED_CFP
      Derived_CFP<double>(raw, raw + CDM_CFP_TSIZE);
#endif
      cnt c[kNCOLS];
      for (int k = 0; k < kNCOLS; k++) c[k] = raw[k];
      g_flops = g_mufu = 0;
      (void)Predicted_Signal(NPARAMS, P, c, F);
      fs += g_flops;
      ms += g_mufu;
      g_flops = g_mufu = 0;
      Partial_Derivatives(NPARAMS, P, c, F, d);
      fj += g_flops;
      mj += g_mufu;
    }
  }
  const double nv = nvox > 0 ? nvox : 1, nm = (double)nvox * nmeas > 0 ? (double)nvox * nmeas : 1;
  out[0] = fd / nv;
  out[1] = fs / nm;
  out[2] = fj / nm;
  out[3] = md / nv;
  out[4] = ms / nm;
  out[5] = mj / nm;
  out[6] = fw / (nv * NPARAMS);
  out[7] = mw / (nv * NPARAMS);
  return 0;
}

// The model description of a split build (the header the host half of the
// library is compiled with instead of the plugin): the plugin's sizes and
// which optional hooks it defines. Writes at most cap bytes of text into
// buf; returns the length, or -1 if it did not fit. The CFP/FixP block
// sizes are appended by the build from modelparameters.cc.
#define CDM_DESC_STR2(...) #__VA_ARGS__
#define CDM_DESC_STR(...) CDM_DESC_STR2(__VA_ARGS__)
extern "C" int cdm_describe(char* buf, int cap) {
  std::string s;
  auto def = [&s](const char* name, long v) {
    s += "#define ";
    s += name;
    s += " ";
    s += std::to_string(v);
    s += "\n";
  };
  def("NPARAMS", NPARAMS);
  def("NCFP", NCFP);
  def("NFIXP", NFIXP);
  def("CDM_CFP_TSIZE", CDM_CFP_TSIZE);
  def("CDM_FIXP_TSIZE", CDM_FIXP_TSIZE);
  def("CDM_NDCFP", CDM_NDCFP);
  def("CDM_NDP", CDM_NDP);
  def("CDM_PSTORE", CDM_PSTORE);
#ifdef CDM_SIGNAL_PAIR
  def("CDM_SIGNAL_PAIR", 1);
#endif
#ifdef CDM_SHELL_SERIES
  def("CDM_SHELL_SERIES", 1);
  def("CDM_SHELL_KEY", CDM_SHELL_KEY);
  def("CDM_SHELL_NCOEF", CDM_SHELL_NCOEF);
  def("CDM_SHELL_MCOLS", CDM_SHELL_MCOLS);
#endif
#ifdef CDM_MLP_HEAD
  def("CDM_MLP_HEAD", 1);
  def("CDM_MLP_NMU", CDM_MLP_NMU);
  def("CDM_MLP_NSIG", CDM_MLP_NSIG);
  s += "#define CDM_MLP_GROUPS " CDM_DESC_STR(CDM_MLP_GROUPS) "\n";
#endif
  if ((int)s.size() + 1 > cap) return -1;
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return (int)s.size();
}
