// fp32.h - single-precision number type used to instantiate model plugins.
//
// A CUDIMOT model plugin is a set of function templates over a number type
// T (Predicted_Signal, Partial_Derivatives, ...). Plugins written for
// T = double mix T with double literals and double-valued macros
// (e.g. `-CFP[3]*Diso` with `#define Diso 0.003`). Instantiated with plain
// `float`, every such expression is promoted to double by the usual C++
// arithmetic conversions and lands on the FP64 pipe, which on GB300 runs at
// about 1/64 of the FP32 rate.
//
// `fp32` wraps a float and defines every arithmetic operator, comparison and
// compound assignment against all arithmetic types so that mixed
// expressions stay single precision: fp32 (op) double -> fp32. Plugins
// compile unchanged and evaluate entirely on the FP32 pipe. Code that
// deliberately declares `double` variables still gets double, through the
// implicit conversion to float followed by the standard float->double
// promotion.
#pragma once

#include <type_traits>

#if defined(__CUDACC__)
#define CDM_HD __host__ __device__ __forceinline__
#else
#define CDM_HD inline
#endif

struct fp32 {
  float v;

  fp32() = default;
  CDM_HD constexpr fp32(float x) : v(x) {}
  CDM_HD constexpr fp32(double x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(long double x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(int x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(unsigned x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(long x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(unsigned long x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(long long x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(unsigned long long x) : v(static_cast<float>(x)) {}
  CDM_HD constexpr fp32(bool x) : v(x ? 1.0f : 0.0f) {}

  CDM_HD constexpr operator float() const { return v; }

  CDM_HD fp32 &operator+=(fp32 o) { v += o.v; return *this; }
  CDM_HD fp32 &operator-=(fp32 o) { v -= o.v; return *this; }
  CDM_HD fp32 &operator*=(fp32 o) { v *= o.v; return *this; }
  CDM_HD fp32 &operator/=(fp32 o) { v /= o.v; return *this; }
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
  CDM_HD fp32 &operator+=(U o) { v += static_cast<float>(o); return *this; }
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
  CDM_HD fp32 &operator-=(U o) { v -= static_cast<float>(o); return *this; }
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
  CDM_HD fp32 &operator*=(U o) { v *= static_cast<float>(o); return *this; }
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type>
  CDM_HD fp32 &operator/=(U o) { v /= static_cast<float>(o); return *this; }

  CDM_HD fp32 &operator++() { v += 1.0f; return *this; }
  CDM_HD fp32 &operator--() { v -= 1.0f; return *this; }
  CDM_HD fp32 operator++(int) { fp32 t = *this; v += 1.0f; return t; }
  CDM_HD fp32 operator--(int) { fp32 t = *this; v -= 1.0f; return t; }
};

CDM_HD fp32 operator-(fp32 a) { return fp32(-a.v); }
CDM_HD fp32 operator+(fp32 a) { return a; }

#define CDM_FP32_BINOP(OP)                                                       \
  CDM_HD fp32 operator OP(fp32 a, fp32 b) { return fp32(a.v OP b.v); }           \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  CDM_HD fp32 operator OP(fp32 a, U b) { return fp32(a.v OP static_cast<float>(b)); } \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  CDM_HD fp32 operator OP(U a, fp32 b) { return fp32(static_cast<float>(a) OP b.v); }
CDM_FP32_BINOP(+)
CDM_FP32_BINOP(-)
CDM_FP32_BINOP(*)
CDM_FP32_BINOP(/)
#undef CDM_FP32_BINOP

#define CDM_FP32_CMP(OP)                                                         \
  CDM_HD bool operator OP(fp32 a, fp32 b) { return a.v OP b.v; }                 \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  CDM_HD bool operator OP(fp32 a, U b) { return a.v OP static_cast<float>(b); }  \
  template <class U, class = typename std::enable_if<std::is_arithmetic<U>::value>::type> \
  CDM_HD bool operator OP(U a, fp32 b) { return static_cast<float>(a) OP b.v; }
CDM_FP32_CMP(<)
CDM_FP32_CMP(>)
CDM_FP32_CMP(<=)
CDM_FP32_CMP(>=)
CDM_FP32_CMP(==)
CDM_FP32_CMP(!=)
#undef CDM_FP32_CMP

// Result type of a binary math wrapper: fp32 if either argument is fp32,
// otherwise the usual arithmetic result type.
template <class A, class B>
struct cdm_math_result {
  typedef typename std::conditional<
      std::is_same<A, fp32>::value || std::is_same<B, fp32>::value, fp32,
      decltype(A() + B())>::type type;
};
