// Ball & 1 Stick: compile-time sizes in the CUDIMOT plugin layout
// (mymodels/<name>/modelparameters.h): parameter count, number of common
// fixed parameter blocks (CFP) and per-voxel fixed parameter blocks (FixP).
#ifndef MODEL_H_INCLUDED
#define MODEL_H_INCLUDED
typedef double MyType;
#define NPARAMS 5  // S0, d, f, theta, phi
#define NCFP 2     // gradient direction (3 rows), b-value (1 row)
#define NFIXP 0
struct MODEL {
  static int CFP_size[NCFP];
  static int FixP_size[NFIXP];
};
#endif
