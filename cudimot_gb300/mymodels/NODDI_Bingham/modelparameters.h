// NODDI-Bingham: compile-time sizes in the CUDIMOT plugin layout
// (mymodels/<name>/modelparameters.h).
#ifndef MODEL_H_INCLUDED
#define MODEL_H_INCLUDED
typedef double MyType;
#define NPARAMS 7  // fiso, fintra, kappa, beta, theta, phi, psi
#define NCFP 2     // gradient direction (3 rows), b-value (1 row)
#define NFIXP 1    // S0
struct MODEL {
  static int CFP_size[NCFP];
  static int FixP_size[NFIXP];
};
#endif
