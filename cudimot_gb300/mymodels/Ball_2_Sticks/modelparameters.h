// Ball & 2 Sticks: compile-time sizes in the CUDIMOT plugin layout
// (mymodels/<name>/modelparameters.h).
#ifndef MODEL_H_INCLUDED
#define MODEL_H_INCLUDED
typedef double MyType;
#define NPARAMS 8  // S0, d, f1, th1, ph1, f2, th2, ph2
#define NCFP 2     // gradient direction (3 rows), b-value (1 row)
#define NFIXP 0
struct MODEL {
  static int CFP_size[NCFP];
  static int FixP_size[NFIXP];
};
#endif
