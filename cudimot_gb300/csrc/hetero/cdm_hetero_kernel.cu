// cdm_hetero_kernel.cu - the persistent multi-model MCMC kernel.
//
// One launch of SMs x resident CTAs. Each CTA repeatedly takes the next
// tile from a device counter (tiles of all fits numbered consecutively,
// fit after fit), finds its fit, copies the fit's argument block into
// shared memory and calls that model's MCMC code for the tile
// (cdm_hetero_part.cu: the same code as the model library's own MCMC
// kernel, with the tile in place of blockIdx.x). Dynamic shared memory is
// laid out as [the largest fit's protocol tables | argument block |
// scratch]. A fit whose error word is set (a bounded wait ran out) makes
// the CTA that ran it stop taking tiles; there is no other wait.
#include <stdint.h>

#include "cdm_hetero_desc.h"
#include "cdm_hx_dispatch.h"  // generated: the entries of the linked models

#ifndef CDM_NT
#define CDM_NT 128
#endif
#ifndef CDM_MCMC_MIN_BLOCKS
#define CDM_MCMC_MIN_BLOCKS 4
#endif

extern "C" __global__ void __launch_bounds__(CDM_NT, CDM_MCMC_MIN_BLOCKS)
    cdm_hx_mcmc(const __grid_constant__ cdm_hx_launch L) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ int s_tile, s_item;
  int prev = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      int t = L.ntiles;
      if (prev < 0 || *(volatile const int*)L.items[prev].err == 0) t = atomicAdd(L.counter, 1);
      int i = 0;
      if (t < L.ntiles)
        while (i + 1 < L.nitems && t >= L.items[i + 1].tile0) ++i;
      s_tile = t;
      s_item = i;
    }
    __syncthreads();
    const int t = s_tile, i = s_item;
    if (t >= L.ntiles) break;
    const cdm_hx_item it = L.items[i];
    uint32_t* dst = reinterpret_cast<uint32_t*>(dsm + L.args_off);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(it.args);
    for (uint32_t k = threadIdx.x; k < it.args_words; k += CDM_NT) dst[k] = src[k];
    __syncthreads();
    cdm_hx_dispatch(it.fn, t - it.tile0, dsm + L.scratch_off, dsm + L.args_off);
    __syncthreads();
    prev = i;
  }
}
