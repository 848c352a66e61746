// NODDI-Watson (Zhang et al., NeuroImage 61:1000-1016, 2012) in CUDIMOT's
// parameterisation (mymodels/NODDI_Watson/modelfunctions.h:88-108):
//
//   S = S0 [ (1-fiso) ((1-fin) E + fin I) + fiso exp(-b Diso) ]
//
// P = {fiso, fintra, kappa, th, ph}; FixP = {S0}; CFP = {gx, gy, gz, b}.
// E: hindered extra-cellular signal with the Watson-averaged tensor
//    (WatsonFunctions.h:53-89); I: Watson-dispersed sticks expanded in
//    even spherical harmonics up to order 12 (modelfunctions.h:45-86).
//
// The model, its branch points (kappa <= 0.4 series, kappa > 30 fits,
// kappa < 1e-5 hindered-diffusion series, b*Dpar <= 0.05 integral series)
// and its numerical derivatives for kappa, th, ph are CUDIMOT's. The
// evaluation is reorganised so that it is accurate in single precision:
//  * the seven Legendre-Gaussian integrals and exp(-b Diso) depend on b
//    only; they are computed once per protocol in double (Derived_CFP) and
//    appended to each measurement's CFP values;
//  * everything that depends on the parameters only (orientation vector,
//    equivalent diffusivities, SH coefficients of the Watson density) is
//    computed once per parameter change (Derived_P) and appended to P;
//  * for 0.4 < kappa <= 30 the SH coefficients are 2 sqrt(pi) sqrt(4l+1)
//    <P_2l>_kappa with the Watson moments <P_2l> from a backward (Miller)
//    three-term recurrence in the Legendre basis. The closed forms used by
//    CUDIMOT (WatsonFunctions.h:112-172) cancel terms of size ~1e10 and
//    are only usable in double; the recurrence is stable in float.
//  * the seven even Legendre polynomials P_0..P_12 come from one pass of a
//    recurrence in x^2 instead of seven separate recurrences.

#define WATSON_DISO 0.003
#define WATSON_DPAR 0.0017

// ---------------------------------------------------------------------------
// Protocol-derived values (double, once per protocol).
//   d[0]   = exp(-b Diso)
//   d[1+l] = 0.5 sqrt((4l+1)/(4 pi)) * LGI_l(b Dpar),  l = 1..6,
//   d[1]   = 0.5 sqrt(1/(4 pi)) * LGI_0(b Dpar) * c_0 (c_0 = 2 sqrt(pi), the
//            l = 0 SH coefficient, which does not depend on kappa)
// with LGI_l(x) = int_{-1}^{1} P_2l(t) exp(-x t^2) dt.
#define CDM_DERIVED_CFP 8

__host__ __device__ inline void watson_lgi(double x, double* L) {
  if (x > 0.05) {
    // I_n = int_{-1}^{1} t^2n exp(-x t^2) dt by upward recurrence from
    // I_0 = sqrt(pi) erf(sqrt x)/sqrt x. CUDIMOT takes erf in single
    // precision here (LegendreFunctions.h:12); the recurrence and the
    // Legendre combinations below amplify its 1e-7 error, and single-
    // precision erf differs between math libraries (host vs device), so the
    // double erf is used: these values are computed once per protocol.
    double I[7];
    const double sx = sqrt(x);
    I[0] = 1.7724538509055160273 * erf(sx) / sx;
    const double emx = -exp(-x);
    for (int n = 1; n < 7; n++) I[n] = (emx + (n - 0.5) * I[n - 1]) / x;
    // Coefficients of P_2l(t) in powers of t^2 (Legendre polynomials).
    L[0] = I[0];
    L[1] = (-I[0] + 3.0 * I[1]) / 2.0;
    L[2] = (3.0 * I[0] - 30.0 * I[1] + 35.0 * I[2]) / 8.0;
    L[3] = (-5.0 * I[0] + 105.0 * I[1] - 315.0 * I[2] + 231.0 * I[3]) / 16.0;
    L[4] = (35.0 * I[0] - 1260.0 * I[1] + 6930.0 * I[2] - 12012.0 * I[3] + 6435.0 * I[4]) / 128.0;
    L[5] = (-63.0 * I[0] + 3465.0 * I[1] - 30030.0 * I[2] + 90090.0 * I[3] - 109395.0 * I[4] +
            46189.0 * I[5]) / 256.0;
    L[6] = (231.0 * I[0] - 18018.0 * I[1] + 225225.0 * I[2] - 1021020.0 * I[3] +
            2078505.0 * I[4] - 1939938.0 * I[5] + 676039.0 * I[6]) / 1024.0;
  } else {
    // Taylor series in x (LegendreFunctions.h:231-253).
    const double x2 = x * x, x3 = x2 * x, x4 = x3 * x, x5 = x4 * x, x6 = x5 * x;
    L[0] = 2.0 - 2.0 * x / 3.0 + x2 / 5.0 - x3 / 21.0 + x4 / 108.0;
    L[1] = -4.0 * x / 15.0 + 4.0 * x2 / 35.0 - 2.0 * x3 / 63.0 + 2.0 * x4 / 297.0;
    L[2] = 8.0 * x2 / 315.0 - 8.0 * x3 / 693.0 + 4.0 * x4 / 1287.0;
    L[3] = -16.0 * x3 / 9009.0 + 16.0 * x4 / 19305.0;
    L[4] = 32.0 * x4 / 328185.0;
    L[5] = -64.0 * x5 / 14549535.0;
    L[6] = 128.0 * x6 / 760543875.0;
  }
}

template <typename T>
__host__ __device__ inline void Derived_CFP(const T* cfp, T* d) {
  const double b = (double)cfp[3];
  d[0] = (T)exp(-b * WATSON_DISO);
  double L[7];
  watson_lgi(b * WATSON_DPAR, L);
  for (int l = 0; l < 7; l++) d[1 + l] = (T)(0.14104739588693907 * sqrt(4.0 * l + 1.0) * L[l]);
  d[1] = (T)(0.14104739588693907 * 3.5449077018110318 * L[0]);
}

// ---------------------------------------------------------------------------
// Parameter-derived values (once per parameter change), stored after the
// NPARAMS model parameters:
//   P[5..7]   orientation vector (sin th cos ph, sin th sin ph, cos th)
//   P[8]      perpendicular equivalent diffusivity dPerp_eq
//   P[9]      dPar_eq - dPerp_eq
//   P[10..15] SH coefficients c_1..c_6 of the Watson density times h_1..h_6
//             (c_0 = 2 sqrt pi; h_l: scale of the rescaled Legendre
//             recurrence below)
//   P[16..18] cos th cos ph, cos th sin ph, sin th (orientation derivatives)
//   P[19]     d<P_2>/dkappa
//   P[20..25] h_1 dc_1/dkappa .. h_6 dc_6/dkappa
//   P[26]     <P_2>
//   P[27..29] kappa, th, ph the cached blocks were computed for
//   P[30]     1 once the caches hold values (callers zero the derived slots)
// A sampler changes one parameter per proposal; the kappa block (Miller
// recurrence) and the trigonometric block are only recomputed when their
// own inputs changed.
#define CDM_DERIVED_P 26

// Dawson's integral by Rybicki's sampling-theorem method (Numerical
// Recipes 6.10; WatsonFunctions.h:13-51): h = 0.4, six terms, series for
// |x| < 0.2. Only used for kappa > 30, where the results do not cancel.
MACRO T watson_dawson(T x) {
  const T ax = fabs_gpu(x);
  if (ax < (T)0.2) {
    const T x2 = x * x;
    return x * ((T)1.0 - (T)(2.0 / 3.0) * x2 * ((T)1.0 - (T)0.4 * x2 * ((T)1.0 - (T)(2.0 / 7.0) * x2)));
  }
  // exp(-((2i+1) h)^2), i = 0..5
  const double cw[6] = {0.8521437889662113, 0.23692775868212165, 0.01831563888873418,
                        0.0003936690406550776, 2.352575200009771e-06, 3.90893843426485e-09};
  const int n0 = 2 * (int)((T)0.5 * ax / (T)0.4 + (T)0.5);
  const T xp = ax - (T)n0 * (T)0.4;
  T e1 = exp_gpu((T)0.8 * xp);
  const T e2 = e1 * e1;
  T d1 = (T)(n0 + 1);
  T d2 = d1 - (T)2.0;
  T sum = (T)0.0;
  for (int i = 0; i < 6; i++) {
    sum += (T)cw[i] * (e1 / d1 + (T)1.0 / (d2 * e1));
    d1 += (T)2.0;
    d2 -= (T)2.0;
    e1 *= e2;
  }
  const T r = (T)0.56418958354775628695 * exp_gpu(-xp * xp) * sum;
  return x < (T)0.0 ? -r : r;
}

// Watson moments <P_2l>_kappa, l = 1..7, for the density exp(kappa t^2):
// Lambda_n = int P_n(t) exp(kappa t^2) dt obeys (integration by parts with
// (2n+1) P_n = P'_{n+1} - P'_{n-1})
//   Lambda_{n-2} = (A_n/(2 kappa) - B_n) Lambda_n + C_n Lambda_{n+2},
//   A_n = (2n-1)(2n+1)/(n-1), B_n = (2n+1)/((n-1)(2n+3)),
//   C_n = (2n-1)(n+2)/((n-1)(2n+3)).
// Lambda_n is the minimal solution, so the recurrence is run downwards from
// Lambda_{N+2} = 0 (Miller's algorithm) and normalised by Lambda_0. N is
// large enough that <P_N> is below 1e-9 for the kappa range it is used in.
template <int N, typename T>
__device__ inline void watson_miller(T kappa, T* mom) {
  const T inv2k = (T)0.5 / kappa;
  T hi = (T)0.0, cur = (T)1e-30;
#pragma unroll
  for (int n = N; n >= 2; n -= 2) {
    if (n <= 14) mom[n / 2] = cur;
    const double A = (double)((2 * n - 1) * (2 * n + 1)) / (double)(n - 1);
    const double B = (double)(2 * n + 1) / (double)((n - 1) * (2 * n + 3));
    const double C = (double)((2 * n - 1) * (n + 2)) / (double)((n - 1) * (2 * n + 3));
    const T lo = ((T)A * inv2k - (T)B) * cur + (T)C * hi;
    hi = cur;
    cur = lo;
  }
  const T inv0 = (T)1.0 / cur;
  mom[0] = (T)1.0;
#pragma unroll
  for (int l = 1; l <= 7; l++) mom[l] *= inv0;
}

// d<P_n>/dkappa = <t^2 P_n> - <t^2><P_n> with
// t^2 P_n = a_n P_{n+2} + b_n P_n + g_n P_{n-2} (two uses of the Legendre
// recurrence t P_n = ((n+1) P_{n+1} + n P_{n-1})/(2n+1)).
MACRO T watson_dmoment(int l, const T* mom, T t2) {
  const double n = 2.0 * l;
  const double a = (n + 1) * (n + 2) / ((2 * n + 1) * (2 * n + 3));
  const double b = (n + 1) * (n + 1) / ((2 * n + 1) * (2 * n + 3)) + n * n / ((2 * n + 1) * (2 * n - 1));
  const double g = n * (n - 1) / ((2 * n + 1) * (2 * n - 1));
  return (T)a * mom[l + 1] + ((T)b - t2) * mom[l] + (T)g * mom[l - 1];
}

// SH coefficients c_1..c_6 (c[1..6]), <P_2> for the hindered tensor, and
// their kappa derivatives (dc[1..6], dp2).
MACRO void watson_kappa_terms(T k, T* c, T& p2, T* dc, T& dp2) {
  // 2 sqrt(pi) sqrt(4l+1)
  const double norm[7] = {3.5449077018110318, 7.926654595212022, 10.634723105433096,
                          12.781346485666884, 14.616028887632437, 16.244807875181,
                          17.724538509055158};
  if (k > (T)30.0) {
    // Large-kappa fits in ln(kappa/30) (WatsonFunctions.h:97-111).
    const double fit[6][7] = {
        {7.52308, 0.411538, -0.214588, 0.0784091, -0.023981, 0.00731537, -0.0026467},
        {8.93718, 1.62147, -0.733421, 0.191568, -0.0202906, -0.00779095, 0.00574847},
        {8.87905, 3.35689, -1.15935, 0.0673053, 0.121857, -0.066642, 0.0180215},
        {7.84352, 5.03178, -1.0193, -0.426362, 0.328816, -0.0688176, -0.0229398},
        {6.30113, 6.09914, -0.16088, -1.05578, 0.338069, 0.0937157, -0.106935},
        {4.65678, 6.30069, 1.13754, -1.38393, -0.0134758, 0.331686, -0.105954}};
    const T L = log_gpu(k) - log_gpu((T)30.0);
    const T ik = (T)1.0 / k;
#pragma unroll
    for (int i = 0; i < 6; i++) {
      T acc = (T)fit[i][6], dacc = (T)(6.0 * fit[i][6]);
#pragma unroll
      for (int j = 5; j >= 0; j--) {
        acc = acc * L + (T)fit[i][j];
        if (j >= 1) dacc = dacc * L + (T)(j * fit[i][j]);
      }
      c[i + 1] = acc;
      dc[i + 1] = dacc * ik;
    }
    // <t^2> = R1 = (s/D(s) - 1) / (2k), s = sqrt(k), with D' = 1 - 2 s D.
    const T sk = sqrt_gpu(k);
    const T D = watson_dawson(sk);
    const T q = sk / D;
    const T r1 = (q - (T)1.0) * (T)0.5 * ik;
    const T dq = (D - sk + (T)2.0 * k * D) / ((T)2.0 * sk * D * D);
    const T dr1 = (dq * (T)2.0 * k - (T)2.0 * (q - (T)1.0)) * (T)0.25 * ik * ik;
    p2 = ((T)3.0 * r1 - (T)1.0) * (T)0.5;
    dp2 = (T)1.5 * dr1;
    return;
  }
  T mom[8];
  if (k >= (T)1e-5) {
    if (k > (T)12.0) {
      watson_miller<52>(k, mom);
    } else if (k > (T)4.0) {
      watson_miller<36>(k, mom);
    } else if (k > (T)1.0) {
      watson_miller<24>(k, mom);
    } else {
      watson_miller<16>(k, mom);
    }
    const T t2 = ((T)1.0 + (T)2.0 * mom[1]) * (T)(1.0 / 3.0);
    p2 = mom[1];
    dp2 = watson_dmoment(1, mom, t2);
    if (k > (T)0.4) {
#pragma unroll
      for (int l = 1; l <= 6; l++) {
        c[l] = (T)norm[l] * mom[l];
        dc[l] = (T)norm[l] * watson_dmoment(l, mom, t2);
      }
      return;
    }
  } else {
    // Second-order series (WatsonFunctions.h:62-73).
    p2 = (T)(2.0 / 15.0) * k + (T)(4.0 / 315.0) * k * k;
    dp2 = (T)(2.0 / 15.0) + (T)(8.0 / 315.0) * k;
  }
  // Small-kappa series (WatsonFunctions.h:173-193) and their derivatives.
  const T k2 = k * k, k3 = k2 * k, k4 = k3 * k, k5 = k4 * k, k6 = k5 * k;
  const T r5 = (T)0.79266545952120224, r1 = (T)0.35449077018110318;   // sqrt(pi/5), 0.2 sqrt(pi)
  const T r13 = (T)0.49159078480905764, r17 = (T)0.42988741044466255; // sqrt(pi/13), sqrt(pi/17)
  const T c5k = (T)(64.0 * 0.38678062186808244 / 692835.0);           // 64 sqrt(pi/21)/692835
  const T c6k = (T)(128.0 * 1.7724538509055160273 / 152108775.0);
  c[1] = ((T)(4.0 / 3.0) * k + (T)(8.0 / 63.0) * k2) * r5;
  c[2] = ((T)(8.0 / 21.0) * k2 + (T)(32.0 / 693.0) * k3) * r1;
  c[3] = ((T)(16.0 / 693.0) * k3 + (T)(32.0 / 10395.0) * k4) * r13;
  c[4] = (T)(32.0 / 19305.0) * k4 * r17;
  c[5] = c5k * k5;
  c[6] = c6k * k6;
  dc[1] = ((T)(4.0 / 3.0) + (T)(16.0 / 63.0) * k) * r5;
  dc[2] = ((T)(16.0 / 21.0) * k + (T)(96.0 / 693.0) * k2) * r1;
  dc[3] = ((T)(48.0 / 693.0) * k2 + (T)(128.0 / 10395.0) * k3) * r13;
  dc[4] = (T)(128.0 / 19305.0) * k3 * r17;
  dc[5] = (T)5.0 * c5k * k4;
  dc[6] = (T)6.0 * c6k * k5;
}

// Even Legendre polynomials by the recurrence in y = x^2 obtained from two
// uses of t P_n = ((n+1) P_{n+1} + n P_{n-1})/(2n+1):
//   P_{n+2} = (a_n y - b_n) P_n - g_n P_{n-2},  n = 0, 2, ..., 10,
// a_n = 1/alpha, b_n = beta/alpha, g_n = gamma/alpha with
// alpha = (n+1)(n+2)/((2n+1)(2n+3)),
// beta = (n+1)^2/((2n+1)(2n+3)) + n^2/((2n+1)(2n-1)),
// gamma = n(n-1)/((2n+1)(2n-1)).
__host__ __device__ constexpr double watson_leg_a(int l) {
  return l == 0 ? 1.5 : l == 1 ? 2.9166666666666665 : l == 2 ? 3.2999999999999998
       : l == 3 ? 3.4821428571428572 : l == 4 ? 3.588888888888889 : 3.6590909090909087;
}
__host__ __device__ constexpr double watson_leg_b(int l) {
  return l == 0 ? 0.5 : l == 1 ? 1.5277777777777775 : l == 2 ? 1.6714285714285715
       : l == 3 ? 1.7516233766233769 : l == 4 ? 1.8007407407407408 : 1.8337320574162681;
}
__host__ __device__ constexpr double watson_leg_g(int l) {
  return l == 0 ? 0.0 : l == 1 ? 0.3888888888888889 : l == 2 ? 0.62857142857142856
       : l == 3 ? 0.73051948051948057 : l == 4 ? 0.78814814814814815 : 0.82535885167464107;
}

// The recurrence rescaled so that its last term has no coefficient (one
// multiply fewer per degree): with q_l = P_2l / h_l, h_0 = h_1 = 1 and
// h_(l+1) = g_l h_(l-1),
//   q_1 = a_0 y - b_0,  q_(l+1) = (qa_l y - qb_l) q_l - q_(l-1)  (l >= 1),
//   qa_l = a_l h_l / h_(l+1),  qb_l = b_l h_l / h_(l+1),
// and the factors h_l are carried by the cached coefficients P[10..15] and
// P[20..25]. The derivative follows as dq_(l+1) = 2 qa_l x q_l +
// (qa_l y - qb_l) dq_l - dq_(l-1).
// h_l, qa_l and qb_l evaluated (literals, so that they fold into immediates):
__host__ __device__ constexpr double watson_h(int l) {
  return l <= 1 ? 1.0 : l == 2 ? 0.3888888888888889 : l == 3 ? 0.6285714285714286
       : l == 4 ? 0.2840909090909091 : l == 5 ? 0.4954074074074074 : 0.23447694649847758;
}
__host__ __device__ constexpr double watson_qa(int l) {
  return l == 0 ? 1.5 : l == 1 ? 7.499999999999999 : l == 2 ? 2.0416666666666665
       : l == 3 ? 7.704489795918367 : l == 4 ? 2.058044938016529 : 7.730997728395061;
}
__host__ __device__ constexpr double watson_qb(int l) {
  return l == 0 ? 0.5 : l == 1 ? 3.9285714285714275 : l == 2 ? 1.0340909090909092
       : l == 3 ? 3.8755918367346944 : l == 4 ? 1.0326330741626795 : 3.874344399355878;
}

MACRO void Derived_P(T* P, T* FixP) {
  const bool valid = P[30] != (T)0.0;
  if (!valid || P[2] != P[27]) {
    T c[7], dc[7];
    T p2, dp2;
    watson_kappa_terms(P[2], c, p2, dc, dp2);
#pragma unroll
    for (int l = 1; l <= 6; l++) {
      P[9 + l] = c[l] * (T)watson_h(l);
      P[19 + l] = dc[l] * (T)watson_h(l);
    }
    P[19] = dp2;
    P[26] = p2;
    P[27] = P[2];
  }
  if (!valid || P[3] != P[28] || P[4] != P[29]) {
    const T st = sin_gpu(P[3]), ct = cos_gpu(P[3]);
    const T sp = sin_gpu(P[4]), cp = cos_gpu(P[4]);
    P[5] = st * cp;
    P[6] = st * sp;
    P[7] = ct;
    P[16] = ct * cp;
    P[17] = ct * sp;
    P[18] = st;
    P[28] = P[3];
    P[29] = P[4];
  }
  const T dperp = (T)WATSON_DPAR * ((T)1.0 - P[1]);
  const T dgap = (T)WATSON_DPAR - dperp;
  P[8] = dperp + dgap * ((T)1.0 - P[26]) * (T)(1.0 / 3.0);
  P[9] = dgap * P[26];
  P[30] = (T)1.0;
}

// ---------------------------------------------------------------------------
MACRO T Predicted_Signal(int npar, T* P, T* CFP, T* FixP) {
  const T xv = CFP[0] * P[5] + CFP[1] * P[6] + CFP[2] * P[7];
  const T extra = exp_gpu(-CFP[3] * (P[9] * xv * xv + P[8]));
  // Dispersed-stick SH sum over P_0..P_12 at the clamped cosine.
  const T y = min_gpu(xv * xv, (T)1.0);  // x^2 at the cosine clamped to [-1, 1]
  T qm = (T)1.0, qc = (T)watson_leg_a(0) * y - (T)watson_leg_b(0);
  T intra = CFP[5] + CFP[6] * P[10] * qc;
#pragma unroll
  for (int l = 1; l < 6; l++) {
    const T qn = ((T)watson_qa(l) * y - (T)watson_qb(l)) * qc - qm;
    qm = qc;
    qc = qn;
    intra += CFP[6 + l] * P[10 + l] * qc;
  }
  if (intra < (T)0.0) intra = (T)0.5e-3;
  const T aniso = ((T)1.0 - P[1]) * extra + P[1] * intra;
  return FixP[0] * (((T)1.0 - P[0]) * aniso + P[0] * CFP[4]);
}

// Two measurements per call on Blackwell's paired FP32 instructions
// (FFMA2/FMUL2/FADD2 on float2): the arithmetic of Predicted_Signal for
// measurements a and b, with every multiply and add issued once for both.
// ab[k] = (column k of a, column k of b). The extra-cellular exponential is
// the hardware exp2 approximation of its base-2 form: its error is about
// (2 + |x| log2(e)) ulp of e^x, and because |x| is large only where e^x is
// small, at most 2e-7 S0 of the signal. Used by the kernels' cost loops
// (optional hook CDM_SIGNAL_PAIR).
#if defined(__CUDACC__) && !defined(CDM_NO_SIGNAL_PAIR)
#define CDM_SIGNAL_PAIR 1
__device__ __forceinline__ float2 watson_bc(float x) { return make_float2(x, x); }
__device__ __forceinline__ float watson_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float2 Predicted_Signal_Pair(const fp32* P, const float2* ab,
                                                        const fp32* FixP) {
  // S = k1 extra + k2 intra + k3 CFP4: the compartment weights folded
  const float k3 = FixP[0].v * P[0].v;
  const float k0 = FixP[0].v * (1.0f - P[0].v);
  const float k1 = k0 * (1.0f - P[1].v), k2 = k0 * P[1].v;
  float2 xv = __fmul2_rn(ab[0], watson_bc(P[5].v));
  xv = __ffma2_rn(ab[1], watson_bc(P[6].v), xv);
  xv = __ffma2_rn(ab[2], watson_bc(P[7].v), xv);
  // extra = exp(-b q) = 2^(b * (-log2(e) q)): the factor -log2(e) rides on
  // the (per-proposal) diffusivities, and the power of two is the hardware
  // ex2.approx.ftz (relative error ~2^-22; results below 2^-126, where the
  // term no longer counts, flush to zero)
  const float nl2e = -1.4426950408889634f;
  const float2 q = __ffma2_rn(__fmul2_rn(watson_bc(P[9].v * nl2e), xv), xv, watson_bc(P[8].v * nl2e));
  const float2 z = __fmul2_rn(ab[3], q);
  const float2 extra = make_float2(watson_ex2(z.x), watson_ex2(z.y));
  // x^2 at the cosine clamped to [-1, 1]: a saturated multiply per half
  const float2 y = make_float2(__saturatef(xv.x * xv.x), __saturatef(xv.y * xv.y));
  // intra = sum_l a_l q_l (a_0 = ab[5], a_l = ab[5+l] P[9+l]) by Clenshaw's
  // backward recurrence on the rescaled one: b_l = a_l + u_l b_(l+1) -
  // b_(l+2) for l = 6..1, intra = a_0 + u_0 b_1 - b_2 (three operations per
  // degree instead of four)
  float2 b2 = make_float2(0.0f, 0.0f);
  float2 b1 = __fmul2_rn(ab[11], watson_bc(P[15].v));
#pragma unroll
  for (int l = 5; l >= 1; l--) {
    const float2 u = __ffma2_rn(watson_bc((float)watson_qa(l)), y, watson_bc(-(float)watson_qb(l)));
    const float2 t = __ffma2_rn(ab[5 + l], watson_bc(P[9 + l].v), make_float2(-b2.x, -b2.y));
    const float2 bn = __ffma2_rn(u, b1, t);
    b2 = b1;
    b1 = bn;
  }
  const float2 u0 = __ffma2_rn(watson_bc((float)watson_qa(0)), y, watson_bc(-(float)watson_qb(0)));
  float2 intra = __ffma2_rn(u0, b1, __fadd2_rn(ab[5], make_float2(-b2.x, -b2.y)));
  if (intra.x < 0.0f) intra.x = 0.5e-3f;
  if (intra.y < 0.0f) intra.y = 0.5e-3f;
  return __ffma2_rn(watson_bc(k3), ab[4],
                    __ffma2_rn(watson_bc(k1), extra, __fmul2_rn(watson_bc(k2), intra)));
}

// Per-shell series (optional hook CDM_SHELL_SERIES). Within one b-shell the
// dispersed-stick sum is a degree-6 polynomial in y = x^2 whose
// coefficients depend on the parameters only: intra(y) = sum_j alpha_j
// q_j(y), alpha_0 = a_0(b), alpha_j = a_j(b) P[9+j] (the Legendre-Gaussian
// columns of the shell times the Watson coefficients). Written in the
// Chebyshev basis of t = 2y - 1 (q_j(y) = sum_k WATSON_CHEB[j][k] T_k(t),
// entries <= 1.41, so single precision keeps ~1e-7 of S0) and then, per
// shell, in powers of t (T_k's integer coefficients, at most 48): the pair
// evaluation is Horner's rule, one fused multiply-add per degree on a
// chain of six. In FP32 this is as accurate as Clenshaw's recurrence on the
// Chebyshev coefficients for these functions (emulated over kappa 0.5-64
// and b 1000-3000: both within 2.1e-7 of the largest intra value; the
// power-basis coefficients add up to no more than that value, so nothing
// cancels). The compartment weights and the isotropic term are folded into
// the coefficients. Shell_Coeffs forms them once per shell and parameter
// set from the shell's protocol row (columns: gx, gy, gz, b, exp(-b Diso),
// a_0..a_6):
//   coef[0..1]  exponent of the extra-cellular term as c0 + c1 x^2, base 2
//   coef[2..8]  k2 intra + k3 exp(-b Diso) = sum_i p_i t^i, as p_6 .. p_0
//   coef[9..10] intra < 0 (the truncated series) becomes 0.5e-3 as in
//               Predicted_Signal: below coef[9] the sum is replaced by coef[10]
//   coef[11]    k1, the extra-cellular weight
// The protocol columns the pair needs per measurement are gx, gy, gz.
#define CDM_SHELL_SERIES 1
#define CDM_SHELL_KEY 3      // measurements with equal b form a shell
#define CDM_SHELL_NCOEF 12
#define CDM_SHELL_MCOLS 3

__device__ constexpr float WATSON_CHEB[7][7] = {
    {1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f},
    {0.25f, 0.75f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f},
    {0.36160714285714257f, 0.8035714285714288f, 1.4062499999999998f, 0.0f, 0.0f, 0.0f, 0.0f},
    {0.15536221590909216f, 0.3262606534090914f, 0.39151278409090917f, 0.7177734374999999f, 0.0f,
     0.0f, 0.0f},
    {0.26318359375001155f, 0.5414062500000156f, 0.5955468750000072f, 0.7373437500000009f,
     1.3825195312499998f, 0.0f, 0.0f},
    {0.12224713010651644f, 0.24902193169846143f, 0.2642681724146847f, 0.29730169396652073f,
     0.3743799109207968f, 0.7113218307495117f, 0.0f},
    {0.2170320620332813f, 0.43970132048254484f, 0.4580222088360886f, 0.49437317779102763f,
     0.5635854226817418f, 0.7172905379585632f, 1.3748068644205729f}};

__device__ __forceinline__ void Shell_Coeffs(const fp32* P, const float* row, const fp32* FixP,
                                             float* coef) {
  const float k3 = FixP[0].v * P[0].v;
  const float k0 = FixP[0].v * (1.0f - P[0].v);
  const float k1 = k0 * (1.0f - P[1].v), k2 = k0 * P[1].v;
  const float nb = -1.4426950408889634f * row[3];
  coef[0] = nb * P[8].v;
  coef[1] = nb * P[9].v;
  float al[7];
  al[0] = row[5];
#pragma unroll
  for (int j = 1; j < 7; j++) al[j] = row[5 + j] * P[9 + j].v;
  float e[7];
#pragma unroll
  for (int k = 0; k < 7; k++) {
    float acc = 0.0f;
#pragma unroll
    for (int j = k; j < 7; j++) acc = fmaf(al[j], WATSON_CHEB[j][k], acc);
    e[k] = acc;
  }
  // powers of t: T_0..T_6 = 1, t, 2t^2-1, 4t^3-3t, 8t^4-8t^2+1,
  // 16t^5-20t^3+5t, 32t^6-48t^4+18t^2-1
  const float iso = k3 * row[4];
  coef[2] = k2 * (32.0f * e[6]);
  coef[3] = k2 * (16.0f * e[5]);
  coef[4] = k2 * fmaf(-48.0f, e[6], 8.0f * e[4]);
  coef[5] = k2 * fmaf(-20.0f, e[5], 4.0f * e[3]);
  coef[6] = k2 * fmaf(18.0f, e[6], fmaf(-8.0f, e[4], 2.0f * e[2]));
  coef[7] = k2 * fmaf(5.0f, e[5], fmaf(-3.0f, e[3], e[1]));
  coef[8] = fmaf(k2, (e[0] - e[2]) + (e[4] - e[6]), iso);
  coef[9] = iso;
  coef[10] = fmaf(k2, 0.5e-3f, iso);
  coef[11] = k1;
}

// The signal of two measurements of one shell: g[c] = column c (gx, gy,
// gz) of both.
__device__ __forceinline__ float2 Predicted_Signal_Shell_Pair(const fp32* P, const float* coef,
                                                              const float2* g) {
  float2 xv = __fmul2_rn(g[0], watson_bc(P[5].v));
  xv = __ffma2_rn(g[1], watson_bc(P[6].v), xv);
  xv = __ffma2_rn(g[2], watson_bc(P[7].v), xv);
  const float2 x2 = __fmul2_rn(xv, xv);
  const float2 z = __ffma2_rn(watson_bc(coef[1]), x2, watson_bc(coef[0]));
  const float2 extra = make_float2(watson_ex2(z.x), watson_ex2(z.y));
  // t = 2y - 1 (a cosine rounded past 1 moves t by an ulp: harmless here)
  const float2 t = __ffma2_rn(watson_bc(2.0f), x2, watson_bc(-1.0f));
  float2 f = __ffma2_rn(watson_bc(coef[2]), t, watson_bc(coef[3]));
  f = __ffma2_rn(f, t, watson_bc(coef[4]));
  f = __ffma2_rn(f, t, watson_bc(coef[5]));
  f = __ffma2_rn(f, t, watson_bc(coef[6]));
  f = __ffma2_rn(f, t, watson_bc(coef[7]));
  f = __ffma2_rn(f, t, watson_bc(coef[8]));
  if (f.x < coef[9]) f.x = coef[10];
  if (f.y < coef[9]) f.y = coef[10];
  return __ffma2_rn(watson_bc(coef[11]), extra, f);
}
#endif

MACRO bool ConstraintsMCMC(int npar, T* P) { return true; }

// Analytic derivatives (CUDIMOT takes kappa, th, ph numerically,
// modelfunctions.h:145-155; single-precision central differences are too
// coarse for LM, so all five are analytic here).
MACRO void Partial_Derivatives(int npar, T* P, T* CFP, T* FixP, T* derivatives) {
  const T xv = CFP[0] * P[5] + CFP[1] * P[6] + CFP[2] * P[7];
  const T extra = exp_gpu(-CFP[3] * (P[9] * xv * xv + P[8]));
  const T x = min_gpu(max_gpu(xv, (T)-1.0), (T)1.0);
  const bool inside = (xv > (T)-1.0) && (xv < (T)1.0);
  const T y = x * x;
  // q_l = P_2l / h_l and dq_l/dx by the rescaled recurrence and its
  // derivative (see watson_h)
  T qm = (T)1.0, qc = (T)watson_leg_a(0) * y - (T)watson_leg_b(0);
  T dqm = (T)0.0, dqc = (T)2.0 * (T)watson_leg_a(0) * x;
  T intra = CFP[5] + CFP[6] * P[10] * qc;
  T dintra_x = CFP[6] * P[10] * dqc, dintra_k = CFP[6] * P[20] * qc;
#pragma unroll
  for (int l = 1; l < 6; l++) {
    const T a = (T)watson_qa(l);
    const T f = a * y - (T)watson_qb(l);
    const T qn = f * qc - qm;
    const T dqn = (T)2.0 * a * x * qc + f * dqc - dqm;
    qm = qc;
    qc = qn;
    dqm = dqc;
    dqc = dqn;
    intra += CFP[6 + l] * P[10 + l] * qc;
    dintra_x += CFP[6 + l] * P[10 + l] * dqc;
    dintra_k += CFP[6 + l] * P[20 + l] * qc;
  }
  if (intra < (T)0.0) {
    intra = (T)0.5e-3;
    dintra_x = (T)0.0;
    dintra_k = (T)0.0;
  }
  if (!inside) dintra_x = (T)0.0;
  const T aniso = ((T)1.0 - P[1]) * extra + P[1] * intra;
  const T s0w = FixP[0] * ((T)1.0 - P[0]);
  // dE/dxv and dE/dkappa (dPerp_eq' = -dgap/3 dp2, (dPar_eq-dPerp_eq)' = dgap dp2).
  const T dgap = (T)WATSON_DPAR * P[1];
  const T dextra_x = extra * (-CFP[3]) * (T)2.0 * P[9] * xv;
  const T dextra_k = extra * (-CFP[3]) * dgap * P[19] * (xv * xv - (T)(1.0 / 3.0));
  const T dS_dx = s0w * (((T)1.0 - P[1]) * dextra_x + P[1] * dintra_x);
  derivatives[0] = FixP[0] * (CFP[4] - aniso);
  derivatives[1] = s0w * (intra - extra);
  derivatives[2] = s0w * (((T)1.0 - P[1]) * dextra_k + P[1] * dintra_k);
  derivatives[3] = dS_dx * (CFP[0] * P[16] + CFP[1] * P[17] - CFP[2] * P[18]);
  derivatives[4] = dS_dx * (CFP[1] * P[5] - CFP[0] * P[6]);
}

MACRO void FixConstraintsLM(int npar, T* P) {}

MACRO T custom_priors(int id_p, T* P, int nmeas, T* CFP, T* FixP) { return (T)0.0; }

// ---------------------------------------------------------------------------
// Optional hooks of the learned initialiser (no counterpart in CUDIMOT).
// Network head: 8 means = (fiso, fintra, log kappa, and the five independent
// entries vx^2, vy^2, vx vy, vx vz, vy vz of the fibre dyad v v^T, which is
// sign-free: v and -v are the same fibre), 4 log-stds: one per scalar and
// one shared by the dyad entries.
#define CDM_MLP_HEAD 1
#define CDM_MLP_NMU 8
#define CDM_MLP_NSIG 4
#define CDM_MLP_GROUPS {0, 1, 2, 3, 3, 3, 3, 3}

template <typename T>
__host__ __device__ inline void MLP_Encode(const T* P, float* t) {
  const double st = sin((double)P[3]), ct = cos((double)P[3]);
  const double vx = st * cos((double)P[4]), vy = st * sin((double)P[4]), vz = ct;
  t[0] = (float)P[0];
  t[1] = (float)P[1];
  t[2] = (float)log(fmax((double)P[2], 1e-3));
  t[3] = (float)(vx * vx);
  t[4] = (float)(vy * vy);
  t[5] = (float)(vx * vy);
  t[6] = (float)(vx * vz);
  t[7] = (float)(vy * vz);
}

// Parameters inside the bounds and MCMC proposal widths from the network's
// outputs. The fibre is the principal eigenvector of the predicted dyad
// (power iteration on dyad + I, which keeps the top eigenvalue on top even
// when the prediction is slightly indefinite).
template <typename T>
__host__ __device__ inline void MLP_Decode(const float* mu, const float* ls, T* P, T* sd) {
  const double lo = 1e-3, hi = 1.0 - 1e-3;
  P[0] = (T)fmin(fmax((double)mu[0], lo), hi);
  P[1] = (T)fmin(fmax((double)mu[1], lo), hi);
  const double kappa = fmin(fmax(exp((double)mu[2]), 0.05), 63.0);
  P[2] = (T)kappa;
  const double a = mu[3], b = mu[4], c = mu[5], d = mu[6], e = mu[7];
  const double M[3][3] = {{a + 1.0, c, d}, {c, b + 1.0, e}, {d, e, 2.0 - a - b}};
  double v[3] = {0.0, 0.0, 0.0};
  const double dg[3] = {a, b, 1.0 - a - b};
  v[dg[0] >= dg[1] && dg[0] >= dg[2] ? 0 : (dg[1] >= dg[2] ? 1 : 2)] = 1.0;
  for (int it = 0; it < 32; it++) {
    double w[3];
    for (int i = 0; i < 3; i++) w[i] = M[i][0] * v[0] + M[i][1] * v[1] + M[i][2] * v[2];
    const double n = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (!(n > 0.0)) break;
    for (int i = 0; i < 3; i++) v[i] = w[i] / n;
  }
  const double th = acos(fmin(fmax(v[2], -1.0), 1.0));
  P[3] = (T)th;
  P[4] = (T)atan2(v[1], v[0]);
  const double sang = fmin(fmax(exp((double)ls[3]), 1e-3), 0.5);
  sd[0] = (T)fmin(fmax(exp((double)ls[0]), 1e-4), 0.5);
  sd[1] = (T)fmin(fmax(exp((double)ls[1]), 1e-4), 0.5);
  sd[2] = (T)fmin(fmax(kappa * exp((double)ls[2]), 1e-3), 16.0);
  sd[3] = (T)sang;
  sd[4] = (T)fmin(sang / fmax(sin(th), 0.1), 1.0);
}
