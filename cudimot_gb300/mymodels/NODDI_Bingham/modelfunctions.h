// NODDI-Bingham (Tariq et al., NeuroImage 2016): NODDI with a Bingham
// distribution of fibre orientations.
//   S = S0 [ (1-fiso) ((1-fintra) E + fintra I) + fiso exp(-b Diso) ]
// P = {fiso, fintra, kappa, beta, theta, phi, psi}; CFP = {gx, gy, gz, b};
// FixP = {S0}. Same model, parameterisation, constraints and derivative set
// as CUDIMOT's mymodels/NODDI_Bingham (modelfunctions.h:20-230,
// hyp_Sapprox_doublePrecision.h, eigenValues.h, diffusivities.h).
//
// In the fibre frame (n = fibre, f = fanning direction, h = f x n) a
// gradient has coordinates w = (g.h, g.f, g.n). With c = -b Dpar:
//   I = H(eig(diag(0, beta, kappa) + c w w^T)) / H(0, beta, kappa),
//   E = exp(-b (dPar xv^2 + sin^2(th_g) (dPerp1 sin^2(ph_g) + dPerp2 cos^2(ph_g)))),
// H = the saddlepoint approximation of 1F1(1/2; 3/2; X) (Kume & Wood 2005),
// dPar and dPerp1 from d log H / d kappa and d log H / d beta.
//
// Restated for single precision (CUDIMOT evaluates H in double and takes
// the two derivatives by central differences with step 5e-5):
//  * every H is evaluated relative to its largest eigenvalue x_max:
//    log H = x_max + s - log K2 / 2 - (sum log u_i) / 2 + T2 + const with
//    u_i = (x_max - x_i) + s and s in [1/2, 3/2] solving sum 1/(2 u_i) = 1,
//    so the ratio I never forms exp(kappa) ~ 1e28 and the common kappa
//    cancels before any rounding;
//  * the largest eigenvalue of the shifted matrix diag(0,beta,kappa) -
//    max(0,beta,kappa) + c w w^T is the largest root of its characteristic
//    cubic, found by monotone Newton steps from 0 (it lies in [c, 0]); the
//    two gaps to the other eigenvalues enter only through their sum and
//    product (trace and the cubic's derivative at the root), which stay
//    accurate when the gaps are nearly equal;
//  * d log H / dx_j is analytic (implicit derivative of the saddlepoint).
// Derived_P keeps the frame vectors and the denominator (log H and the
// hindered diffusivities) after P[6].

#define BINGHAM_DISO 0.003
#define BINGHAM_DPAR 0.0017

#define CDM_DERIVED_CFP 2  // CFP[4] = exp(-b Diso), CFP[5] = -b Dpar
#define CDM_DERIVED_P 17   // P[7..23], see Derived_P

template <typename T>
__host__ __device__ inline void Derived_CFP(const T* cfp, T* d) {
  const double b = (double)cfp[3];
  d[0] = (T)exp(-b * BINGHAM_DISO);
  d[1] = (T)(-b * BINGHAM_DPAR);
}

// Convergence test of the Newton iterations: a step below the working
// precision of the iterate (relative 1e-7 in single, 1e-15 in double).
MACRO bool bingham_done(T step, T x) {
  return fabs_gpu(step) <= (T)(sizeof(T) == sizeof(double) ? 1e-15 : 1e-7) * fabs_gpu(x);
}

// Saddle point s in [1/2, 3/2]: root of h(s) = 1/(2s) + (A + 2s) / (2 q) - 1,
// q = B + A s + s^2 (u1 + u2 = A + 2s, u1 u2 = q). h decreases and is
// convex, so Newton from s = 1/2 rises monotonically onto the root.
MACRO T bingham_saddle(T A, T B) {
  T s = (T)0.5;
#pragma unroll 1
  for (int it = 0; it < 12; it++) {
    const T q = B + A * s + s * s;
    const T ps = A + (T)2.0 * s;
    const T is = rcp_gpu(s), iq = rcp_gpu(q);
    const T h = (T)0.5 * is + (T)0.5 * ps * iq - (T)1.0;
    const T dh = -(T)0.5 * is * is + (T)0.5 * ((T)2.0 * q - ps * ps) * iq * iq;
    const T step = h * rcp_gpu(dh);
    s = min_gpu(max_gpu(s - step, (T)0.5), (T)1.5);
    if (bingham_done(step, s)) break;
  }
  return s;
}

// Saddlepoint terms for eigenvalues x_max (gap 0) and two more with gap sum
// A = e1 + e2 >= 0 and gap product B = e1 e2 >= 0:
// returns F = s - log K2 / 2 - (log u_0 + log u_1 + log u_2) / 2 + T2,
// so that log H = const + x_max + F.
MACRO T bingham_F(T A, T B) {
  const T s = bingham_saddle(A, B);
  const T q = B + A * s + s * s;
  const T ps = A + (T)2.0 * s;
  const T iq = (T)1.0 / q, is = (T)1.0 / s;
  // sums over the pair (u1, u2) from their sum ps and product q
  const T s2 = (ps * ps - (T)2.0 * q) * iq * iq;                          // 1/u1^2 + 1/u2^2
  const T s3 = (ps * ps * ps - (T)3.0 * q * ps) * iq * iq * iq;           // 1/u1^3 + 1/u2^3
  const T p2 = ps * ps - (T)2.0 * q;                                        // u1^2 + u2^2
  const T s4 = (p2 * p2 - (T)2.0 * q * q) * iq * iq * iq * iq;             // 1/u1^4 + 1/u2^4
  const T K2 = (T)0.5 * (is * is + s2);
  const T K3 = is * is * is + s3;
  const T K4 = (T)3.0 * (is * is * is * is + s4);
  const T iK2 = (T)1.0 / K2;
  const T T2 = (T)0.125 * K4 * iK2 * iK2 - (T)(5.0 / 24.0) * K3 * K3 * iK2 * iK2 * iK2;
  return s - (T)0.5 * log_gpu(K2) - (T)0.5 * log_gpu(s * q) + T2;
}

// Largest eigenvalue of D + c w w^T with D = diag(d) <= 0 (max 0) and
// c <= 0: the largest root of p(x) = det(x I - D - c w w^T) =
// prod(x - d_i) - c sum_i w_i^2 prod_{j != i}(x - d_j). It lies in
// [c |w|^2, 0] and p is increasing and convex right of it, so Newton from
// x = 0 descends monotonically onto it (stopping when a step no longer
// moves it). Also returns p'(root) = product of the two gaps below it.
MACRO T bingham_top_eig(const T* d, const T* w2, T c, T& dp_root) {
  // start: the lowest Gershgorin upper bound that is still >= the root
  // (the rows' centre + radius; never above 0)
  const T aw0 = sqrt_gpu(w2[0]), aw1 = sqrt_gpu(w2[1]), aw2 = sqrt_gpu(w2[2]);
  const T g0 = d[0] + c * w2[0] - c * aw0 * (aw1 + aw2);
  const T g1 = d[1] + c * w2[1] - c * aw1 * (aw0 + aw2);
  const T g2 = d[2] + c * w2[2] - c * aw2 * (aw0 + aw1);
  T x = min_gpu(max_gpu(max_gpu(g0, g1), g2), (T)0.0), dp = (T)1.0;
#pragma unroll 1
  for (int it = 0; it < 24; it++) {
    const T l0 = x - d[0], l1 = x - d[1], l2 = x - d[2];
    const T p = l0 * l1 * l2 - c * (w2[0] * l1 * l2 + w2[1] * l0 * l2 + w2[2] * l0 * l1);
    dp = l1 * l2 + l0 * l2 + l0 * l1 - c * (w2[0] * (l1 + l2) + w2[1] * (l0 + l2) + w2[2] * (l0 + l1));
    if (!(dp > (T)0.0)) break;
    const T step = p * rcp_gpu(dp);
    if (!(step > (T)0.0)) break;
    x = x - step;
    if (bingham_done(step, fabs_gpu(x) + fabs_gpu(c))) break;
  }
  const T l0 = x - d[0], l1 = x - d[1], l2 = x - d[2];
  dp_root = l1 * l2 + l0 * l2 + l0 * l1 - c * (w2[0] * (l1 + l2) + w2[1] * (l0 + l2) + w2[2] * (l0 + l1));
  return x;
}

// log H(eig(D + c w w^T)) - const - max(0, beta, kappa) for
// D = diag(0, beta, kappa), c <= 0 (the shift is the denominator's too, so
// it is never added: in single precision adding and subtracting kappa ~ 64
// would cost 4e-6 of the ratio).
MACRO T bingham_logH(T beta, T kappa, T c, T wx, T wy, T wz) {
  const T sh = max_gpu(max_gpu(kappa, beta), (T)0.0);
  const T d[3] = {-sh, beta - sh, kappa - sh};
  const T w2[3] = {wx * wx, wy * wy, wz * wz};
  T B;
  const T lam = bingham_top_eig(d, w2, c, B);
  // gaps of the two other eigenvalues below lam: their sum from the trace,
  // their product = p'(lam)
  const T tr = d[0] + d[1] + d[2] + c * (w2[0] + w2[1] + w2[2]);
  const T A = max_gpu((T)3.0 * lam - tr, (T)0.0);
  return lam + bingham_F(A, max_gpu(B, (T)0.0));
}

// Denominator H(0, beta, kappa): log H - const and its derivatives in kappa
// and beta (implicit differentiation of the saddlepoint:
// d log H / dx_j = 1/(2 u_j) - dK2/(2 K2) + dT2, dt/dx_j = -u_j^-2 / (2 K2)).
MACRO void bingham_denominator(T beta, T kappa, T& L, T& dk, T& db) {
  const T x[3] = {(T)0.0, beta, kappa};
  const T xm = max_gpu(max_gpu(kappa, beta), (T)0.0);
  const T e0 = xm - x[0], e1 = xm - x[1], e2 = xm - x[2];
  // one gap is 0; the other two give A, B
  const T A = e0 + e1 + e2;
  const T B = e0 * e1 + e0 * e2 + e1 * e2;
  L = bingham_F(A, B);  // log H - const - max(0, beta, kappa)
  const T s = bingham_saddle(A, B);
  const T u[3] = {e0 + s, e1 + s, e2 + s};
  T K2 = (T)0.0, K3 = (T)0.0, K4 = (T)0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const T r = (T)1.0 / u[i];
    K2 += (T)0.5 * r * r;
    K3 += r * r * r;
    K4 += (T)3.0 * r * r * r * r;
  }
  T out[2];
#pragma unroll
  for (int jj = 0; jj < 2; jj++) {
    const int j = jj == 0 ? 2 : 1;  // kappa, beta
    const T uj = u[j];
    const T dt = -((T)1.0 / (uj * uj)) / ((T)2.0 * K2);
    T dK2 = (T)0.0, dK3 = (T)0.0, dK4 = (T)0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const T du = (i == j ? -(T)1.0 : (T)0.0) - dt;
      const T r = (T)1.0 / u[i];
      dK2 += -r * r * r * du;
      dK3 += -(T)3.0 * r * r * r * r * du;
      dK4 += -(T)12.0 * r * r * r * r * r * du;
    }
    const T dT2 = dK4 / ((T)8.0 * K2 * K2) - K4 * dK2 / ((T)4.0 * K2 * K2 * K2) -
                  (T)5.0 * K3 * dK3 / ((T)12.0 * K2 * K2 * K2) +
                  (T)5.0 * K3 * K3 * dK2 / ((T)8.0 * K2 * K2 * K2 * K2);
    out[jj] = (T)0.5 / uj - dK2 / ((T)2.0 * K2) + dT2;
  }
  dk = out[0];
  db = out[1];
}

// Derived_P layout: P[7..9] fibre n, P[10..12] fanning f, P[13..15] h = f x n,
// P[16] log H(0, beta, kappa) - const - max(0, beta, kappa), P[17] dPar, P[18] dPerp1,
// P[19] dPerp2, P[20..22] memo (kappa, beta, fintra of P[16..19]), P[23] 1
// once the memo holds values (callers zero the derived slots).
MACRO void Derived_P(T* P, T* FixP) {
  const T st = sin_gpu(P[4]), ct = cos_gpu(P[4]);
  const T sp = sin_gpu(P[5]), cp = cos_gpu(P[5]);
  const T ss = sin_gpu(P[6]), cs = cos_gpu(P[6]);
  const T n0 = st * cp, n1 = st * sp, n2 = ct;
  const T f0 = -cs * sp - ct * cp * ss, f1 = cp * cs - ct * sp * ss, f2 = st * ss;
  P[7] = n0; P[8] = n1; P[9] = n2;
  P[10] = f0; P[11] = f1; P[12] = f2;
  P[13] = f1 * n2 - f2 * n1;
  P[14] = f2 * n0 - f0 * n2;
  P[15] = f0 * n1 - f1 * n0;
  if (!(P[23] != (T)0.0 && P[20] == P[2] && P[21] == P[3] && P[22] == P[1])) {
    T L, dk, db;
    bingham_denominator(P[3], P[2], L, dk, db);
    const T dperp = (T)BINGHAM_DPAR * ((T)1.0 - P[1]);
    const T gap = (T)BINGHAM_DPAR - dperp;
    P[16] = L;
    P[17] = dperp + gap * dk;
    P[18] = dperp + gap * db;
    P[19] = (T)BINGHAM_DPAR + (T)2.0 * dperp - P[17] - P[18];
    P[20] = P[2];
    P[21] = P[3];
    P[22] = P[1];
    P[23] = (T)1.0;
  }
}

MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP) {
  const T wz = CFP[0] * P[7] + CFP[1] * P[8] + CFP[2] * P[9];    // g.n
  const T wy = CFP[0] * P[10] + CFP[1] * P[11] + CFP[2] * P[12]; // g.f
  const T wx = CFP[0] * P[13] + CFP[1] * P[14] + CFP[2] * P[15]; // g.(f x n)
  // hindered compartment; sin^2(th_g) cos^2(ph_g) with cos(atan2(wy, wx))
  const T cos2 = wz * wz;
  const T sin2 = (T)1.0 - cos2;
  const T r2 = wx * wx + wy * wy;
  const T cph2 = r2 > (T)0.0 ? wx * wx / r2 : (T)1.0;
  const T extra = exp_gpu(-CFP[3] * (P[17] * cos2 + sin2 * (P[18] * ((T)1.0 - cph2) + P[19] * cph2)));
  // restricted compartment
  const T intra = exp_gpu(bingham_logH(P[3], P[2], CFP[5], wx, wy, wz) - P[16]);
  const T aniso = ((T)1.0 - P[1]) * extra + P[1] * intra;
  return FixP[0] * (((T)1.0 - P[0]) * aniso + P[0] * CFP[4]);
}

// MCMC rejects kappa - 0.05 < beta (modelfunctions.h:177-186).
MACRO bool ConstraintsMCMC(int npar, T* P) { return !((P[2] - (T)0.05) < P[3]); }

MACRO void Partial_Derivatives(int npar, T* P, T* CFP, T* FixP, T* derivatives) {
  const T wz = CFP[0] * P[7] + CFP[1] * P[8] + CFP[2] * P[9];
  const T wy = CFP[0] * P[10] + CFP[1] * P[11] + CFP[2] * P[12];
  const T wx = CFP[0] * P[13] + CFP[1] * P[14] + CFP[2] * P[15];
  const T cos2 = wz * wz;
  const T sin2 = (T)1.0 - cos2;
  const T r2 = wx * wx + wy * wy;
  const T cph2 = r2 > (T)0.0 ? wx * wx / r2 : (T)1.0;
  const T extra = exp_gpu(-CFP[3] * (P[17] * cos2 + sin2 * (P[18] * ((T)1.0 - cph2) + P[19] * cph2)));
  const T intra = exp_gpu(bingham_logH(P[3], P[2], CFP[5], wx, wy, wz) - P[16]);
  const T aniso = ((T)1.0 - P[1]) * extra + P[1] * intra;
  derivatives[0] = FixP[0] * (CFP[4] - aniso);
  derivatives[1] = FixP[0] * ((T)1.0 - P[0]) * (intra - extra);
  derivatives[2] = NUMERICAL(2);
  derivatives[3] = NUMERICAL(3);
  derivatives[4] = NUMERICAL(4);
  derivatives[5] = NUMERICAL(5);
  derivatives[6] = NUMERICAL(6);
}

// After LM: if kappa < beta then beta = kappa - 0.05 (modelfunctions.h:212-219).
MACRO void FixConstraintsLM(int npar, T* P) {
  if (P[2] < P[3]) P[3] = P[2] - (T)0.05;
}

MACRO T custom_priors(int id_p, T* P, int nmeas, T* CFP, T* FixP) { return (T)0.0; }
