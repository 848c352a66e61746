// cdm_hetero_kernel.cu - the persistent multi-model MCMC kernel.
//
// One launch of SMs x resident CTAs. Each CTA repeatedly takes the next
// tile from a device counter (tiles of all fits numbered consecutively,
// fit after fit), finds its fit and calls that model's MCMC code for the
// tile (cdm_hetero_part.cu: the same code as the model library's own MCMC
// kernel, with the tile in place of blockIdx.x). The fits' argument blocks
// are in cdm_hx_args, one constant-memory slot per entry of the dispatch
// table, written by the host before the launch in stream order; each entry
// reads its own slot, so the chain code takes its arguments from the
// constant bank as the model library's kernel does. Dynamic shared memory
// is laid out as [the largest fit's protocol tables | scratch]. A fit whose
// error word is set (a bounded wait ran out) makes the CTA that ran it stop
// taking tiles; there is no other wait.
#include <stdint.h>

#include "cdm_hetero_desc.h"
#include "cdm_hx_dispatch.h"  // generated: the entries of the linked models

#ifndef CDM_NT
#define CDM_NT 128
#endif
#ifndef CDM_MCMC_MIN_BLOCKS
#define CDM_MCMC_MIN_BLOCKS 4
#endif

extern "C" {
__constant__ __align__(16) unsigned char cdm_hx_args[CDM_HX_ENTRIES][CDM_HX_ARGS_BLOCK];
}

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
    cdm_hx_dispatch(it.fn, t - it.tile0, dsm + L.scratch_off);
    __syncthreads();
    prev = i;
  }
}
