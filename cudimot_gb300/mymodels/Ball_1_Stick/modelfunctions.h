// Ball & 1 Stick diffusion model (Behrens et al., MRM 2003):
//   S = S0 * [ (1-f) exp(-b d) + f exp(-b d (g.v)^2) ]
// with the stick direction v = (sin th cos ph, sin th sin ph, cos th).
// P = {S0, d, f, th, ph}; CFP = {gx, gy, gz, b}; no FixP.
// Same model, parameter order and derivative set as CUDIMOT's
// mymodels/Ball_1_Stick/modelfunctions.h:11-94; all derivatives analytic.

MACRO T b1s_dot(T* P, T* CFP) {
  const T st = sin_gpu(P[3]);
  return CFP[0] * st * cos_gpu(P[4]) + CFP[1] * st * sin_gpu(P[4]) + CFP[2] * cos_gpu(P[3]);
}

MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP) {
  const T bd = -P[1] * CFP[3];
  const T gv = b1s_dot(P, CFP);
  const T ball = exp_gpu(bd);
  const T stick = exp_gpu(bd * gv * gv);
  return P[0] * (((T)1.0 - P[2]) * ball + P[2] * stick);
}

MACRO bool ConstraintsMCMC(int npar, T* P) { return true; }

MACRO void Partial_Derivatives(int npar, T* P, T* CFP, T* FixP, T* derivatives) {
  const T st = sin_gpu(P[3]), ct = cos_gpu(P[3]);
  const T sp = sin_gpu(P[4]), cp = cos_gpu(P[4]);
  const T bd = -P[1] * CFP[3];
  const T gv = CFP[0] * st * cp + CFP[1] * st * sp + CFP[2] * ct;
  const T ball = exp_gpu(bd);
  const T stick = exp_gpu(bd * gv * gv);
  // d gv / d th and d gv / d ph
  const T gv_th = ct * (cp * CFP[0] + sp * CFP[1]) - st * CFP[2];
  const T gv_ph = st * (cp * CFP[1] - sp * CFP[0]);
  const T k = -(T)2.0 * P[0] * P[1] * P[2] * CFP[3] * gv * stick;
  derivatives[0] = ((T)1.0 - P[2]) * ball + P[2] * stick;
  derivatives[1] = -(P[0] * CFP[3]) * (((T)1.0 - P[2]) * ball + P[2] * gv * gv * stick);
  derivatives[2] = P[0] * (stick - ball);
  derivatives[3] = k * gv_th;
  derivatives[4] = k * gv_ph;
}

MACRO void FixConstraintsLM(int npar, T* P) {}

MACRO T custom_priors(int id_p, T* P, int nmeas, T* CFP, T* FixP) { return (T)0.0; }
