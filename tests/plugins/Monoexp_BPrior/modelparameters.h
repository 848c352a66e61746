// Mono-exponential decay with a custom prior on D (test plugin): compile-time
// sizes in the CUDIMOT plugin layout.
#ifndef MODEL_H_INCLUDED
#define MODEL_H_INCLUDED
typedef double MyType;
#define NPARAMS 2  // S0, D
#define NCFP 2     // gradient direction (3 rows, unused), b-value (1 row)
#define NFIXP 0
struct MODEL {
  static int CFP_size[NCFP];
  static int FixP_size[NFIXP];
};
#endif
