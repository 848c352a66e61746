// host_prelude.h - lets CUDIMOT model plugins compile as plain host C++ for
// the CPU oracle. TEST INFRASTRUCTURE: the oracle checks the GPU library and
// is never part of it.
//
// Plugins are CUDA device templates (`#define MACRO template <typename T>
// __device__ inline`); on the host the CUDA qualifiers expand to nothing and
// the *_gpu wrappers of the library prelude resolve to <cmath>.
#pragma once
#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#include <cmath>
#include <math.h>
#include "functions_gpu.h"
// CUDA device code has global min/max overloads for float and double; some
// plugins (the Bingham family's hyp_Sapprox_doublePrecision.h) call them.
#include <algorithm>
using std::max;
using std::min;
