#include "modelparameters.h"
// Rows of each CFP block: bvecs (3), bvals (1). One per-voxel fixed value: S0.
int MODEL::CFP_size[] = {3, 1};
int MODEL::FixP_size[] = {1};
