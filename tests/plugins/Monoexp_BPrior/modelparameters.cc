#include "modelparameters.h"
// Rows of each CFP block: bvecs (3), bvals (1). No per-voxel fixed blocks.
int MODEL::CFP_size[] = {3, 1};
int MODEL::FixP_size[] = {};
