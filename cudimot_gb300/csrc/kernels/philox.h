// philox.h - Philox4x32-10 counter-based random numbers (Salmon, Moraes,
// Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3", SC'11).
//
// MCMC draws are a pure function of (seed, voxel, iteration, parameter): the
// counter is (voxel, iteration, slot, stream) and the key is the 64-bit
// seed. Every lane that cooperates on a voxel computes the same draw, so no
// lane has to broadcast proposals or accept/reject decisions, and no
// generator state is stored between launches.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define CDM_RNG_HD __host__ __device__ __forceinline__
#else
#define CDM_RNG_HD inline
#endif

struct cdm_u32x4 {
  uint32_t x, y, z, w;
};

CDM_RNG_HD void cdm_mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umulhi(a, b);
#else
  const uint64_t p = (uint64_t)a * (uint64_t)b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

// Ten rounds of the Philox S-box; round multipliers and Weyl key increments
// are the ones published with the generator.
CDM_RNG_HD cdm_u32x4 cdm_philox4x32_10(cdm_u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
  const uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    cdm_mulhilo32(kPhiloxM0, c.x, hi0, lo0);
    cdm_mulhilo32(kPhiloxM1, c.z, hi1, lo1);
    cdm_u32x4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return c;
}

// Uniform in (0, 1] from the top 24 bits (exactly representable in float).
CDM_RNG_HD float cdm_u01_open0(uint32_t v) { return (float)((v >> 8) + 1u) * (1.0f / 16777216.0f); }
// Uniform in [0, 1) from the top 24 bits.
CDM_RNG_HD float cdm_u01_open1(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }

// Slots of the counter's third word.
#define CDM_RNG_SLOT_TAU 31u   // Rician tau proposal (parameter slots are 0..30)

// One proposal's randomness: a standard normal (Box-Muller on x, y) and an
// acceptance uniform in (0, 1] (from z).
struct cdm_draw {
  float normal;
  float uniform;
};

CDM_RNG_HD cdm_draw cdm_mcmc_draw(uint64_t seed, uint32_t voxel, uint32_t iter, uint32_t slot,
                                  uint32_t stream) {
  cdm_u32x4 c = {voxel, iter, slot, stream};
  const cdm_u32x4 r = cdm_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float u1 = cdm_u01_open0(r.x);
  const float u2 = cdm_u01_open1(r.y);
  cdm_draw d;
#if defined(__CUDA_ARCH__)
  d.normal = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
#else
  d.normal = (float)(std::sqrt(-2.0 * std::log((double)u1)) * std::cos(6.283185307179586 * (double)u2));
#endif
  d.uniform = cdm_u01_open0(r.z);
  return d;
}
