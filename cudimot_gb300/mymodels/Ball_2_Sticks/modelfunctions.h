// Ball & 2 Sticks diffusion model (Behrens et al., NeuroImage 2007):
//   S = S0 [ (1-f1-f2) exp(-b d) + f1 exp(-b d (g.v1)^2) + f2 exp(-b d (g.v2)^2) ]
// with v_k = (sin th_k cos ph_k, sin th_k sin ph_k, cos th_k).
// P = {S0, d, f1, th1, ph1, f2, th2, ph2}; CFP = {gx, gy, gz, b}; no FixP.
// Same model, parameter order, MCMC constraint (f1 >= f2) and LM fix-up
// (swap the sticks when f1 < f2) as CUDIMOT's
// mymodels/Ball_2_Sticks/modelfunctions.h:7-158; derivatives analytic.
//
// The sines and cosines of the two stick angles depend on the parameters
// only: Derived_P keeps them after P[7] (P[8..11] = sin th1, cos th1,
// sin ph1, cos ph1; P[12..15] the same for stick 2), so a signal evaluation
// is two dot products and three exps; it recomputes a stick's block only
// when that stick's angles changed. Products are formed in CUDIMOT's
// order, so the FP64 signal and Jacobian are CUDIMOT's bit for bit.
//
// dS/dph2: CUDIMOT's plugin (modelfunctions.h:125-129) computes the
// phi-derivative of g.v2 into a variable it then does not use, so its
// column 7 is d(g.v2)/dth2 in place of d(g.v2)/dph2. The LM fits (and
// nothing else) depend on it. This plugin reproduces that column so that
// fits match CUDIMOT's; building with -DCDM_B2S_EXACT_PH2_DERIVATIVE gives
// the true derivative (on the 48-voxel golden case LM then ends at 0.2-1.0x
// CUDIMOT's cost, never above it).

#define CDM_DERIVED_P 13

// P[16..19] hold the angles the sines and cosines were computed for and
// P[20] is 1 once they are valid (callers zero the derived slots): a
// sampler changes one parameter per proposal, so only the stick whose angle
// changed is recomputed.
MACRO void Derived_P(T* P, T* FixP) {
  const bool valid = P[20] != (T)0.0;
  if (!valid || P[3] != P[16] || P[4] != P[17]) {
    P[8] = sin_gpu(P[3]);
    P[9] = cos_gpu(P[3]);
    P[10] = sin_gpu(P[4]);
    P[11] = cos_gpu(P[4]);
    P[16] = P[3];
    P[17] = P[4];
  }
  if (!valid || P[6] != P[18] || P[7] != P[19]) {
    P[12] = sin_gpu(P[6]);
    P[13] = cos_gpu(P[6]);
    P[14] = sin_gpu(P[7]);
    P[15] = cos_gpu(P[7]);
    P[18] = P[6];
    P[19] = P[7];
  }
  P[20] = (T)1.0;
}

// g.v for the stick whose sin/cos block starts at P[k].
MACRO T b2s_dot(T* P, int k, T* CFP) {
  return CFP[0] * P[k] * P[k + 3] + CFP[1] * P[k] * P[k + 2] + CFP[2] * P[k + 1];
}

MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP) {
  const T bd = -P[1] * CFP[3];
  const T x1 = b2s_dot(P, 8, CFP);
  const T x2 = b2s_dot(P, 12, CFP);
  return P[0] * (((T)1.0 - P[2] - P[5]) * exp_gpu(bd) + P[2] * exp_gpu(bd * x1 * x1) +
                 P[5] * exp_gpu(bd * x2 * x2));
}

// Two measurements per call on the paired FP32 instructions (optional hook
// CDM_SIGNAL_PAIR; ab[k] = column k of both measurements):
//   S = k0 2^(u) + k1 2^(u x1^2) + k2 2^(u x2^2),  u = -log2(e) d b,
// with k0 = S0 (1 - f1 - f2), k1 = S0 f1, k2 = S0 f2 and the stick
// directions formed once per proposal; the powers of two on the hardware
// ex2.approx.ftz (relative error ~2^-22).
#if defined(__CUDACC__) && !defined(CDM_NO_SIGNAL_PAIR)
#define CDM_SIGNAL_PAIR 1
__device__ __forceinline__ float2 b2s_bc(float x) { return make_float2(x, x); }
__device__ __forceinline__ float b2s_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float2 Predicted_Signal_Pair(const fp32* P, const float2* ab,
                                                        const fp32* FixP) {
  const float s0 = P[0].v, f1 = P[2].v, f2 = P[5].v;
  const float k0 = s0 * (1.0f - f1 - f2), k1 = s0 * f1, k2 = s0 * f2;
  float2 x1 = __fmul2_rn(ab[0], b2s_bc(P[8].v * P[11].v));
  x1 = __ffma2_rn(ab[1], b2s_bc(P[8].v * P[10].v), x1);
  x1 = __ffma2_rn(ab[2], b2s_bc(P[9].v), x1);
  float2 x2 = __fmul2_rn(ab[0], b2s_bc(P[12].v * P[15].v));
  x2 = __ffma2_rn(ab[1], b2s_bc(P[12].v * P[14].v), x2);
  x2 = __ffma2_rn(ab[2], b2s_bc(P[13].v), x2);
  const float2 u = __fmul2_rn(ab[3], b2s_bc(-1.4426950408889634f * P[1].v));
  const float2 u1 = __fmul2_rn(u, __fmul2_rn(x1, x1));
  const float2 u2 = __fmul2_rn(u, __fmul2_rn(x2, x2));
  float2 s = __fmul2_rn(b2s_bc(k0), make_float2(b2s_ex2(u.x), b2s_ex2(u.y)));
  s = __ffma2_rn(b2s_bc(k1), make_float2(b2s_ex2(u1.x), b2s_ex2(u1.y)), s);
  return __ffma2_rn(b2s_bc(k2), make_float2(b2s_ex2(u2.x), b2s_ex2(u2.y)), s);
}
#endif

MACRO bool ConstraintsMCMC(int npar, T* P) { return !(P[2] < P[5]); }

MACRO void Partial_Derivatives(int npar, T* P, T* CFP, T* FixP, T* derivatives) {
  const T bd = -P[1] * CFP[3];
  const T x1 = b2s_dot(P, 8, CFP);
  const T x2 = b2s_dot(P, 12, CFP);
  const T iso = exp_gpu(bd);
  const T a1 = exp_gpu(bd * x1 * x1);
  const T a2 = exp_gpu(bd * x2 * x2);
  const T fiso = (T)1.0 - P[2] - P[5];
  derivatives[0] = fiso * iso + P[2] * a1 + P[5] * a2;
  derivatives[1] = -(P[0] * CFP[3]) * (fiso * iso + P[2] * x1 * x1 * a1 + P[5] * x2 * x2 * a2);
  derivatives[2] = P[0] * (a1 - iso);
  derivatives[5] = P[0] * (a2 - iso);
  // d(g.v)/dth and d(g.v)/dph of each stick
  const T t1 = P[9] * (P[11] * CFP[0] + P[10] * CFP[1]) - P[8] * CFP[2];
  const T f1 = P[8] * (P[11] * CFP[1] - P[10] * CFP[0]);
  const T t2 = P[13] * (P[15] * CFP[0] + P[14] * CFP[1]) - P[12] * CFP[2];
  const T k1 = -(T)2.0 * P[0] * P[1] * P[2] * CFP[3];
  const T k2 = -(T)2.0 * P[0] * P[1] * P[5] * CFP[3];
  derivatives[3] = k1 * t1 * x1 * a1;
  derivatives[4] = k1 * f1 * x1 * a1;
  derivatives[6] = k2 * t2 * x2 * a2;
#ifdef CDM_B2S_EXACT_PH2_DERIVATIVE
  const T f2 = P[12] * (P[15] * CFP[1] - P[14] * CFP[0]);
  derivatives[7] = k2 * f2 * x2 * a2;
#else
  derivatives[7] = k2 * t2 * x2 * a2;
#endif
}

// After LM: keep the larger fraction in stick 1.
MACRO void FixConstraintsLM(int npar, T* P) {
  if (P[2] < P[5]) {
    T t = P[2]; P[2] = P[5]; P[5] = t;
    t = P[3]; P[3] = P[6]; P[6] = t;
    t = P[4]; P[4] = P[7]; P[7] = t;
  }
}

MACRO T custom_priors(int id_p, T* P, int nmeas, T* CFP, T* FixP) { return (T)0.0; }
