// cdm_noalloc_scratch.h - size and layout of the fixed device array that
// cdm_levmar_noalloc works in (no counterpart in CUDIMOT).
#pragma once
#include <stddef.h>

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB per GPU
constexpr size_t kNoAllocHeader = 256;               // device error word, then the protocol
