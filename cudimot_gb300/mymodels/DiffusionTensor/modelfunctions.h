// Diffusion tensor model (Basser et al., 1994):
//   S = S0 exp(-b g^T D g)
// with D symmetric, P = {S0, Dxx, Dxy, Dxz, Dyy, Dyz, Dzz};
// CFP = {gx, gy, gz, b}; no FixP. Same model and parameter order as
// CUDIMOT's mymodels/DiffusionTensor/modelfunctions.h:20-104; derivatives
// analytic.
//
// The six products of the protocol that multiply the tensor entries,
//   q = (b gx^2, 2b gx gy, 2b gx gz, b gy^2, 2b gy gz, b gz^2),
// depend on the measurement only: they are computed once per protocol in
// double (Derived_CFP) and sit after the four CFP values, so a signal is
// six FMAs and one exp. Products and sums keep CUDIMOT's order, so the FP64
// signal and Jacobian are CUDIMOT's bit for bit, including one quirk kept
// on purpose: CUDIMOT's signal squares gz through powf (single precision,
// modelfunctions.h:27) while its derivatives square it in double. q[5] is
// the signal's single-precision square, q[6] the derivatives' double one.

#define CDM_DERIVED_CFP 7

template <typename T>
__host__ __device__ inline void Derived_CFP(const T* cfp, T* d) {
  const T gx = cfp[0], gy = cfp[1], gz = cfp[2], b = cfp[3];
  d[0] = b * (gx * gx);
  d[1] = 2.0 * b * gx * gy;
  d[2] = 2.0 * b * gx * gz;
  d[3] = b * (gy * gy);
  d[4] = 2.0 * b * gy * gz;
  d[5] = b * (T)powf((float)gz, 2.0f);
  d[6] = b * (gz * gz);
}

// -b g^T D g from the derived protocol products (CFP[4..10]); zz is the
// column of q used for the D_zz term.
MACRO T dt_exponent(T* P, T* CFP, int zz) {
  return -CFP[4] * P[1] - CFP[7] * P[4] - CFP[zz] * P[6] - CFP[5] * P[2] - CFP[6] * P[3] -
         CFP[8] * P[5];
}

MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP) {
  return P[0] * exp_gpu(dt_exponent(P, CFP, 9));
}

// Two measurements per call on the paired FP32 instructions (optional hook
// CDM_SIGNAL_PAIR; ab[k] = column k of both measurements): the same six
// products and exponential, with the exponential in base 2 -- the factor
// -log2(e) rides on the (per-proposal) tensor entries -- on the hardware
// ex2.approx.ftz (relative error ~2^-22).
#if defined(__CUDACC__) && !defined(CDM_NO_SIGNAL_PAIR)
#define CDM_SIGNAL_PAIR 1
__device__ __forceinline__ float2 dt_bc(float x) { return make_float2(x, x); }
__device__ __forceinline__ float dt_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float2 Predicted_Signal_Pair(const fp32* P, const float2* ab,
                                                        const fp32* FixP) {
  const float k = -1.4426950408889634f;
  float2 z = __fmul2_rn(ab[4], dt_bc(P[1].v * k));
  z = __ffma2_rn(ab[7], dt_bc(P[4].v * k), z);
  z = __ffma2_rn(ab[9], dt_bc(P[6].v * k), z);
  z = __ffma2_rn(ab[5], dt_bc(P[2].v * k), z);
  z = __ffma2_rn(ab[6], dt_bc(P[3].v * k), z);
  z = __ffma2_rn(ab[8], dt_bc(P[5].v * k), z);
  return __fmul2_rn(dt_bc(P[0].v), make_float2(dt_ex2(z.x), dt_ex2(z.y)));
}
#endif

MACRO bool ConstraintsMCMC(int npar, T* P) { return true; }

MACRO void Partial_Derivatives(int npar, T* P, T* CFP, T* FixP, T* derivatives) {
  const T e = exp_gpu(dt_exponent(P, CFP, 10));
  const T s = P[0] * e;
  derivatives[0] = e;
  derivatives[1] = s * -CFP[4];
  derivatives[2] = s * -CFP[5];
  derivatives[3] = s * -CFP[6];
  derivatives[4] = s * -CFP[7];
  derivatives[5] = s * -CFP[8];
  derivatives[6] = s * -CFP[10];
}

MACRO void FixConstraintsLM(int npar, T* P) {}

MACRO T custom_priors(int id_p, T* P, int nmeas, T* CFP, T* FixP) { return (T)0.0; }
