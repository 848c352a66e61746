// Test plugin for custom priors: S = S0 exp(-b D), P = {S0, D},
// CFP = {gx, gy, gz, b} (the direction is unused), no FixP.
//
// The prior on D is Gaussian around c = 0.5 / mean(b), the mean taken over
// EVERY measurement of the protocol: custom_priors receives the whole
// [nmeas][CFP_Tsize] CFP array, as in CUDIMOT's MCMC kernel (MCMC.cu:134,
// :186 with the copy of :382-384). A kernel that handed it one measurement,
// or the wrong stride, would centre the prior elsewhere (measurement 0 has
// b = 0).

MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP) {
  return P[0] * exp_gpu(-P[1] * CFP[3]);
}

MACRO bool ConstraintsMCMC(int npar, T* P) { return true; }

MACRO void Partial_Derivatives(int npar, T* P, T* CFP, T* FixP, T* derivatives) {
  const T e = exp_gpu(-P[1] * CFP[3]);
  derivatives[0] = e;
  derivatives[1] = -P[0] * CFP[3] * e;
}

MACRO void FixConstraintsLM(int npar, T* P) {}

MACRO T custom_priors(int id_p, T* P, int nmeas, T* CFP, T* FixP) {
  if (id_p != 1) return (T)0.0;
  T sum_b = (T)0.0;
  for (int i = 0; i < nmeas; i++) sum_b += CFP[i * 4 + 3];
  const T c = (T)0.5 * (T)nmeas / sum_b;
  const T z = (P[1] - c) / ((T)0.2 * c);
  return (T)0.5 * z * z;
}
