// cdm_hetero_desc.h - descriptors the host half of the multi-model library
// passes to the persistent kernel (cdm_hetero_kernel.cu).
#ifndef CDM_HETERO_DESC_H
#define CDM_HETERO_DESC_H
#include <stdint.h>

#include "cdm_hx_entries.h"  // generated: CDM_HX_ENTRIES, CDM_HX_ARGS_BLOCK

// One prepared fit (device memory).
struct cdm_hx_item {
  int* err;    // its context's error word
  int fn;      // its entry in the dispatch table: (model * nlanes + lane index) * 2 + rician
  int tile0;   // its first tile in the launch's numbering
  int ntiles;
  int pad;
};

// The launch (kernel parameters). The fits' argument blocks are in the
// constant-memory slot table cdm_hx_args, one slot per entry, so at most
// one fit per entry in one launch.
struct cdm_hx_launch {
  const cdm_hx_item* items;  // sorted by tile0
  int nitems;
  int ntiles;                // sum over the items
  int* counter;              // next tile (zeroed before the launch)
  uint32_t scratch_off;      // byte offset of the kernel's scratch in dynamic shared memory
  uint32_t pad;
};
#endif
