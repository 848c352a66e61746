// cdm_hetero_desc.h - descriptors the host half of the multi-model library
// uploads for the persistent kernel (cdm_hetero_kernel.cu).
#ifndef CDM_HETERO_DESC_H
#define CDM_HETERO_DESC_H
#include <stdint.h>

// One prepared fit.
struct cdm_hx_item {
  const unsigned char* args;  // its argument block (device copy)
  int* err;                   // its context's error word
  int fn;                     // entry in the dispatch table: (model * nlanes + lane index) * 2 + rician
  int tile0;                  // its first tile in the launch's numbering
  int ntiles;
  uint32_t args_words;        // 4-byte words of the argument block
};

// The launch.
struct cdm_hx_launch {
  const cdm_hx_item* items;  // sorted by tile0
  int nitems;
  int ntiles;                // sum over the items
  int* counter;              // next tile (zeroed before the launch)
  uint32_t args_off;         // byte offset of the argument block copy in dynamic shared memory
  uint32_t scratch_off;      // byte offset of the kernel's scratch
};
#endif
