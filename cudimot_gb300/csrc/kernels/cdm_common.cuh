// cdm_common.cuh - shared device pieces of the fitting kernels.
//
// Included after the model plugin (functions_gpu.h -> modelparameters.h ->
// macro_numerical.h -> modelfunctions.h -> cdm_plugin_tail.h) and after
// cdm_model_sizes.h, which the build generates from modelparameters.cc
// (CDM_CFP_TSIZE, CDM_FIXP_TSIZE).
//
// Work decomposition: a voxel is processed by a group of Gw consecutive lanes
// of one warp (Gw in {1, 2, 4, 8, 16, 32}); lane j of the group takes measurements
// j, j+Gw, j+2G, ... Group sums are butterfly (xor) shuffles, which leave the
// identical value in every lane, so every lane of a group takes the same
// decisions without a broadcast. Several groups share a warp when Gw < 32.
//
// HBM layouts the kernels read (built by cdm_pack_* kernels):
//   protocol  float [nmeas_pad][NCOLS4]  NCOLS = CFP_Tsize + derived CFP,
//                                        rows padded to NCOLS4 (16 bytes)
//   signals   float [nvox/T][nchunk][T][Gw]  tile-major (cdm_tile_index, T =
//                                        CDM_NT / Gw voxels per CTA); row c
//                                        holds measurements cG..cG+Gw-1
// so a warp's signal load is one contiguous 128-byte line and a CTA's
// signals are one contiguous block.
// With the paired signal hook (Predicted_Signal_Pair) the kernels that take
// the paired cost loop also keep, after the staged protocol in shared
// memory, a pair table float2 [nchunk/2][Gw][NCOLSP] (NCOLS rounded up to
// even, the pad column zero): entry (j, l, k) holds column k of
// measurements 2jG+l and (2j+1)Gw+l, the two a lane evaluates together, so a
// 16-byte load gives two columns already paired.
#pragma once

#include <stdint.h>
#include "cdm_args.h"
#include "philox.h"

#ifndef CDM_SSE_UNROLL
#define CDM_SSE_UNROLL 2  // measurement-loop unroll of the cost sums
#endif

constexpr int kSseUnroll = CDM_SSE_UNROLL;
// Unroll of the paired (two-measurement) cost loops: how many pairs' signal
// loads are in flight per lane. In the per-shell series a pair is short
// (one multiply-add per degree) and the loads from L2 become the wait:
// 4 pairs there (NODDI-Watson, grid search + MCMC: 115 ms against 124 ms at
// 2); 2 in the per-measurement loop.
#ifndef CDM_PAIR_UNROLL
#define CDM_PAIR_UNROLL 2
#endif
#ifndef CDM_SHELL_UNROLL
#define CDM_SHELL_UNROLL 4
#endif
constexpr int kPairUnroll = CDM_PAIR_UNROLL;
constexpr int kShellUnroll = CDM_SHELL_UNROLL;

// Number type the plugin is evaluated in: fp32 (fp32.h), or double with
// CDM_EVAL_DOUBLE for plugins whose closed forms need it (CUDIMOT's
// NODDI-Watson cancels terms of ~1e10). Chain state, residuals and their
// per-lane sums stay single precision either way; group sums, energies and
// the LM solve are double either way.
#ifdef CDM_EVAL_DOUBLE
typedef double cdm_real;
#else
typedef fp32 cdm_real;
#endif

// Kernel definitions. A normal build makes each one a __global__ function.
// The device half of a split build (CDM_DEVICE_MODULE) makes them inline
// device functions taking their argument block by reference; the module
// defines extern "C" kernels with fixed names that call them, so that a
// host library compiled without the plugin can look them up by name.
//
// A part of the persistent multi-model kernel (CDM_HETERO) also makes them
// device functions, with two more leading arguments: the tile the CTA
// works on in place of blockIdx.x, and shared-memory scratch for what the
// kernel would otherwise keep in static shared memory (the static shared
// memory of every model linked into the one kernel would add up).
#if defined(CDM_HETERO)
#define CDM_KERNEL(...) __device__ __forceinline__ void
#define CDM_KERNEL0 __device__ __forceinline__ void
// The argument block is in memory the kernel never writes: __restrict__
// lets the compiler keep what it has loaded from it across the kernel's
// own stores (a kernel parameter is known read-only; a reference is not).
#define CDM_KARG(T) int cdm_tile, unsigned char* __restrict__ cdm_scratch, const T& __restrict__
#define CDM_BLOCK_IDX cdm_tile
#elif defined(CDM_DEVICE_MODULE)
#define CDM_KERNEL(...) __device__ __forceinline__ void
#define CDM_KERNEL0 __device__ __forceinline__ void
#define CDM_KARG(T) const T&
#define CDM_BLOCK_IDX blockIdx.x
#else
#define CDM_KERNEL(...) __global__ void __launch_bounds__(__VA_ARGS__)
#define CDM_KERNEL0 __global__ void
#define CDM_KARG(T) const __grid_constant__ T
#define CDM_BLOCK_IDX blockIdx.x
#endif

static_assert(CUSTOM == kCustomPrior, "prior type CUSTOM");
static_assert(sizeof(cdm_real) == kRealBytes, "evaluation type size");

// Error codes written to the device error word.
#define CDM_DEVERR_STAGE_TIMEOUT 1


template <int Gw>
__device__ __forceinline__ unsigned cdm_group_mask() {
  if (Gw == 32) return 0xFFFFFFFFu;
  if (Gw == 1) return 1u << (threadIdx.x & 31u);
  const unsigned lane = threadIdx.x & 31u;
  return ((1u << Gw) - 1u) << (lane & ~(unsigned)(Gw - 1));
}

template <int Gw, class Tv>
__device__ __forceinline__ Tv cdm_group_sum(Tv v, unsigned mask) {
#pragma unroll
  for (int o = Gw / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// Wait for phase 0 of the mbarrier at shared address sbar, at most limit_ns
// of %globaltimer; on expiry record CDM_DEVERR_STAGE_TIMEOUT in *err (may
// be null) and return false instead of spinning forever.
__device__ __forceinline__ bool cdm_mbar_wait_phase0(uint32_t sbar, uint64_t limit_ns, int* err) {
  uint64_t t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(sbar)
        : "memory");
    if (done) return true;
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > limit_ns) {
      if (err) atomicOr(err, CDM_DEVERR_STAGE_TIMEOUT);
      return false;
    }
  }
}

// ---------------------------------------------------------------------------
// Protocol staging: one elected thread issues a bulk asynchronous copy
// (cp.async.bulk, the TMA engine's 1-D form) of the whole protocol table from
// HBM into shared memory; the CTA waits on an mbarrier. The wait is bounded
// by the global timer: after 2 s the CTA records CDM_DEVERR_STAGE_TIMEOUT
// and returns false instead of spinning forever.
__device__ __forceinline__ bool cdm_stage_protocol(const float* __restrict__ gsrc, float* sdst,
                                                   uint32_t bytes, int* err) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t sbar = (uint32_t)__cvta_generic_to_shared(&bar);
  const uint32_t sdst_a = (uint32_t)__cvta_generic_to_shared(sdst);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
#ifdef CDM_HETERO
  // the previous tile wrote this shared memory with ordinary stores; order
  // them before the bulk copy (async proxy) that overwrites it
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
#endif
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            sdst_a),
        "l"(gsrc), "r"(bytes), "r"(sbar)
        : "memory");
  }
  const bool done = cdm_mbar_wait_phase0(sbar, 2000000000ull, err);
#ifdef CDM_HETERO
  // the whole CTA leaves together (the persistent kernel's barriers follow),
  // and the next tile initialises the barrier again
  const bool all = __syncthreads_and(done) != 0;
  if (threadIdx.x == 0 && all) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(sbar) : "memory");
  return all;
#else
  __syncthreads();
  return done;
#endif
}

// Load one measurement's protocol values (raw CFP then derived) from the
// staged table into a register array the plugin can index: one 16-byte
// shared-memory load per four values. The Gw lanes of a group read Gw
// consecutive rows (distinct banks for 48-byte rows); other groups of the
// warp read the same rows (broadcast).
__device__ __forceinline__ void cdm_load_cfp(const float* sproto, int nmeas_pad, int m, cdm_real* cf) {
  const float4* row = reinterpret_cast<const float4*>(sproto + (size_t)m * kNCOLS4);
#pragma unroll
  for (int q = 0; q < kNCOLS4 / 4; q++) {
    const float4 v = row[q];
    if (4 * q + 0 < kNCOLS) cf[4 * q + 0] = cdm_real(v.x);
    if (4 * q + 1 < kNCOLS) cf[4 * q + 1] = cdm_real(v.y);
    if (4 * q + 2 < kNCOLS) cf[4 * q + 2] = cdm_real(v.z);
    if (4 * q + 3 < kNCOLS) cf[4 * q + 3] = cdm_real(v.w);
  }
}

// Per-voxel view handed to the group cost routines.
struct cdm_voxel_io {
  const float* sig;  // this lane's first signal value (chunk 0, tile-major: cdm_tile_index)
  size_t chunk_stride;  // to the lane's next chunk: CDM_NT floats
  int nchunk;
  int nmeas;
  int nmeas_pad;
  int lane;
  const float* pairs;  // this lane's first pair-table entry (paired hook only)
  const int* shells;   // shell-table header in shared memory, or null (per-measurement path)
  const float* stab;   // this lane's first shell pair entry
  const float2* sig2;  // shell order: this lane's first pair of signals (pair-interleaved,
                       // tile-major: cdm_tile_index; pairs CDM_NT float2 apart)
};

// Build the pair table (see the layout notes above) after the staged
// protocol, with every thread of the CTA; returns its start. Call before
// any thread leaves the kernel.
template <int Gw>
__device__ __forceinline__ const float* cdm_build_pair_table(float* sproto, int nmeas_pad,
                                                             int nchunk) {
  float2* ptab = reinterpret_cast<float2*>(sproto + (size_t)nmeas_pad * kNCOLS4);
#if CDM_PAIRED
  const int total = (nchunk / 2) * Gw * kNCOLSP;
  for (int i = (int)threadIdx.x; i < total; i += (int)blockDim.x) {
    const int k = i % kNCOLSP, l = (i / kNCOLSP) % Gw, j = i / (kNCOLSP * Gw);
    ptab[i] = k < kNCOLS ? make_float2(sproto[(size_t)(2 * j * Gw + l) * kNCOLS4 + k],
                                       sproto[(size_t)((2 * j + 1) * Gw + l) * kNCOLS4 + k])
                         : make_float2(0.0f, 0.0f);
  }
  __syncthreads();
#endif
  return reinterpret_cast<const float*>(ptab);
}

// Shell table (CDM_SHELLS; built by cdm_prep_shells_kernel right after the
// protocol rows, staged with them): an int header - valid, nshell, npos,
// then per shell its representative protocol row, its pairs per lane and
// its first pair index - followed by one 8-float entry per (pair, lane):
// (gx_a, gx_b, gy_a, gy_b, gz_a, gz_b, w_a, w_b) for the lane's two
// measurements of the pair, w = 0 on padding positions. Measurements are
// ordered shell by shell, each shell padded to whole pairs of lane chunks,
// so the signals (packed in the same order) are walked chunk by chunk as
// in the per-measurement path.
// Prepare the shared-memory tables after staging: the shell table when the
// host staged one and it is valid, else the pair table of the paired hook.
template <int Gw>
__device__ __forceinline__ const float* cdm_prepare_tables(float* sproto, int nmeas_pad, int nchunk,
                                                           bool shells_staged, const int** hdr) {
  *hdr = nullptr;
#if CDM_SHELLS
  if (shells_staged) {
    const int* h = reinterpret_cast<const int*>(sproto + (size_t)nmeas_pad * kNCOLS4);
    if (h[0]) {
      *hdr = h;
      return sproto + (size_t)nmeas_pad * kNCOLS4 + kShellHeader;
    }
    __syncthreads();  // every thread has read the flag before the table is overwritten
  }
#endif
  return cdm_build_pair_table<Gw>(sproto, nmeas_pad, nchunk);
}

// One pair-table entry: the NCOLS column pairs of a lane's two measurements
// (16-byte loads: entries are a whole number of 16-byte units).
__device__ __forceinline__ void cdm_load_pairs(const float* q, float2* ab) {
  const float4* q4 = reinterpret_cast<const float4*>(q);
#pragma unroll
  for (int k = 0; k < kNCOLSP / 2; k++) {
    const float4 v = q4[k];
    ab[2 * k] = make_float2(v.x, v.y);
    if (2 * k + 1 < kNCOLS) ab[2 * k + 1] = make_float2(v.z, v.w);
  }
}

// Sum of squared residuals over the voxel's measurements: each lane sums its
// own measurements in FP32, the group total is formed in FP64. The loop walks
// a protocol-row pointer and a signal pointer; chunks where every lane has a
// measurement need no bounds test, only the last chunk may be partial.
#if CDM_SHELLS
static_assert(CDM_SHELL_MCOLS == 3, "shell pair entries hold three protocol columns and a weight");
// Sum of squared residuals through the per-shell series: per shell, the
// plugin forms its coefficients once (Shell_Coeffs, from the shell's
// protocol row), then the lane's pairs of that shell are evaluated
// (Predicted_Signal_Shell_Pair); padding positions have weight 0 and
// signal 0, so r = w S - y vanishes there.
template <int Gw, typename Ts>
__device__ __forceinline__ Ts cdm_group_sse_shells(const cdm_voxel_io& io, const float* sproto,
                                                   cdm_real* P, cdm_real* FixP, unsigned gmask) {
  const int* hdr = io.shells;
  const int nshell = hdr[1];
  float2 acc2 = make_float2(0.0f, 0.0f);
  const float2* sig = io.sig2;
  for (int s = 0; s < nshell; s++) {
    float coef[CDM_SHELL_NCOEF];
    Shell_Coeffs(P, sproto + (size_t)hdr[4 + 3 * s] * kNCOLS4, FixP, coef);
    const int npairs = hdr[5 + 3 * s];
    const float4* q = reinterpret_cast<const float4*>(io.stab) + (size_t)hdr[6 + 3 * s] * Gw * 2;
#pragma unroll kShellUnroll
    for (int j = 0; j < npairs; j++) {
      const float4 c01 = q[0], c2w = q[1];
      const float2 g[3] = {make_float2(c01.x, c01.y), make_float2(c01.z, c01.w),
                           make_float2(c2w.x, c2w.y)};
      const float2 s2 = Predicted_Signal_Shell_Pair(P, coef, g);
      const float2 y = *sig;
      const float2 r = __ffma2_rn(make_float2(c2w.z, c2w.w), s2, make_float2(-y.x, -y.y));
      acc2 = __ffma2_rn(r, r, acc2);
      q += 2 * Gw;
      sig += CDM_NT;
    }
  }
  return cdm_group_sum<Gw>((Ts)(acc2.x + acc2.y), gmask);
}
#endif

// The group total is formed in Ts: double for the chain energies and the
// reported costs, float for the grid search's ranking pass (whose near ties
// are settled in FP64).
template <int Gw, typename Ts = double>
__device__ __forceinline__ Ts cdm_group_sse(const cdm_voxel_io& io, const float* sproto,
                                            cdm_real* P, cdm_real* FixP, unsigned gmask) {
#if CDM_SHELLS
  if (io.shells) return cdm_group_sse_shells<Gw, Ts>(io, sproto, P, FixP, gmask);
#endif
  float acc = 0.0f;
  const int full = io.nmeas / Gw;
  const float* row = sproto + (size_t)io.lane * kNCOLS4;
  const float* sig = io.sig;
#if CDM_PAIRED
  // two chunks per step on the paired FP32 instructions (plugin hook
  // Predicted_Signal_Pair) with the protocol from the pair table; two
  // interleaved partial sums
  float2 acc2 = make_float2(0.0f, 0.0f);
  int c = 0;
  const float* q = io.pairs;
#pragma unroll kPairUnroll
  for (; c + 1 < full; c += 2) {
    float2 ab[kNCOLS];
    cdm_load_pairs(q, ab);
    const float2 s2 = Predicted_Signal_Pair(P, ab, FixP);
    const float2 r = __fadd2_rn(s2, make_float2(-sig[0], -sig[io.chunk_stride]));
    acc2 = __ffma2_rn(r, r, acc2);
    q += 2 * Gw * kNCOLSP;
    sig += 2 * io.chunk_stride;
  }
  acc = acc2.x + acc2.y;
  row += (size_t)c * Gw * kNCOLS4;
  if (c < full) {
    cdm_real cf[kNCOLS];
    cdm_load_cfp(row, 0, 0, cf);
    const float r = (float)Predicted_Signal(NPARAMS, P, cf, FixP) - *sig;
    acc = fmaf(r, r, acc);
    row += Gw * kNCOLS4;
    sig += io.chunk_stride;
  }
#else
#pragma unroll kSseUnroll
  for (int c = 0; c < full; c++) {
    cdm_real cf[kNCOLS];
    cdm_load_cfp(row, 0, 0, cf);
    const float r = (float)Predicted_Signal(NPARAMS, P, cf, FixP) - *sig;
    acc = fmaf(r, r, acc);
    row += Gw * kNCOLS4;
    sig += io.chunk_stride;
  }
#endif
  if (full < io.nchunk) {
    const bool valid = full * Gw + io.lane < io.nmeas;
    cdm_real cf[kNCOLS];
    cdm_load_cfp(valid ? row : sproto, 0, 0, cf);
    const float r = (float)Predicted_Signal(NPARAMS, P, cf, FixP) - *sig;
    acc = valid ? fmaf(r, r, acc) : acc;
  }
  return cdm_group_sum<Gw>((Ts)acc, gmask);
}

// log I0(x) with the polynomial approximations of Abramowitz & Stegun
// 9.8.1/9.8.2, as CUDIMOT's logIo (MCMC.cu:32-49).
__device__ __forceinline__ float cdm_log_i0(float x) {
  const float b = fabsf(x);
  if (b < 3.75f) {
    float a = x / 3.75f;
    a *= a;
    return logf(1.0f + a * (3.5156229f + a * (3.0899424f + a * (1.2067492f + a * (0.2659732f +
                        a * (0.0360768f + a * 0.0045813f))))));
  }
  const float a = 3.75f / b;
  return b + logf((0.39894228f + a * (0.01328592f + a * (0.00225319f + a * (-0.00157565f +
                  a * (0.00916281f + a * (-0.02057706f + a * (0.02635537f + a * (-0.01647633f +
                  a * 0.00392377f)))))))) * rsqrtf(b));
}

// log I0 for the MCMC energies: the same polynomials with the hardware
// reciprocal and logarithm approximations (absolute error ~2e-7 per term,
// far below the energy differences the Metropolis test compares); BIC/AIC
// keep cdm_log_i0.
__device__ __forceinline__ float cdm_log_i0_fast(float x) {
  const float b = fabsf(x);
  if (b < 3.75f) {
    float a = x * (1.0f / 3.75f);
    a *= a;
    return __logf(1.0f + a * (3.5156229f + a * (3.0899424f + a * (1.2067492f + a * (0.2659732f +
                          a * (0.0360768f + a * 0.0045813f))))));
  }
  const float a = __fdividef(3.75f, b);
  return b + __logf((0.39894228f + a * (0.01328592f + a * (0.00225319f + a * (-0.00157565f +
                    a * (0.00916281f + a * (-0.02057706f + a * (0.02635537f + a * (-0.01647633f +
                    a * 0.00392377f)))))))) * rsqrtf(b));
}

#if CDM_PAIRED
// cdm_log_i0_fast on both halves of a pair without branches: the two
// polynomial pieces are evaluated on the paired FP32 instructions (the same
// Horner steps, so each half gets cdm_log_i0_fast's value) and the piece
// that applies is selected per half. Lanes of a warp hold different voxels
// and measurements, so the branchy form runs both pieces in most warps
// anyway, one half at a time. The piece not selected may be inf or NaN
// (|x| = 0 in the reciprocal and rsqrt); a select does not propagate it.
__device__ __forceinline__ float2 cdm_log_i0_fast2(float2 x) {
  const float2 b = make_float2(fabsf(x.x), fabsf(x.y));
  float2 a = __fmul2_rn(x, make_float2(1.0f / 3.75f, 1.0f / 3.75f));
  a = __fmul2_rn(a, a);
  float2 ps = make_float2(0.0045813f, 0.0045813f);
  ps = __ffma2_rn(a, ps, make_float2(0.0360768f, 0.0360768f));
  ps = __ffma2_rn(a, ps, make_float2(0.2659732f, 0.2659732f));
  ps = __ffma2_rn(a, ps, make_float2(1.2067492f, 1.2067492f));
  ps = __ffma2_rn(a, ps, make_float2(3.0899424f, 3.0899424f));
  ps = __ffma2_rn(a, ps, make_float2(3.5156229f, 3.5156229f));
  ps = __ffma2_rn(a, ps, make_float2(1.0f, 1.0f));
  const float2 al = make_float2(__fdividef(3.75f, b.x), __fdividef(3.75f, b.y));
  float2 pl = make_float2(0.00392377f, 0.00392377f);
  pl = __ffma2_rn(al, pl, make_float2(-0.01647633f, -0.01647633f));
  pl = __ffma2_rn(al, pl, make_float2(0.02635537f, 0.02635537f));
  pl = __ffma2_rn(al, pl, make_float2(-0.02057706f, -0.02057706f));
  pl = __ffma2_rn(al, pl, make_float2(0.00916281f, 0.00916281f));
  pl = __ffma2_rn(al, pl, make_float2(-0.00157565f, -0.00157565f));
  pl = __ffma2_rn(al, pl, make_float2(0.00225319f, 0.00225319f));
  pl = __ffma2_rn(al, pl, make_float2(0.01328592f, 0.01328592f));
  pl = __ffma2_rn(al, pl, make_float2(0.39894228f, 0.39894228f));
  pl = __fmul2_rn(pl, make_float2(rsqrtf(b.x), rsqrtf(b.y)));
  const bool sx = b.x < 3.75f, sy = b.y < 3.75f;
  const float lx = __logf(sx ? ps.x : pl.x), ly = __logf(sy ? ps.y : pl.y);
  return make_float2(sx ? lx : b.x + lx, sy ? ly : b.y + ly);
}
#endif

// Rician log-likelihood sum without the voxel-constant sum of log(y)
// (which cancels in every Metropolis ratio): sum of
// -tau/2 (y^2 + S^2) + log I0(tau S y).
template <int Gw>
__device__ __forceinline__ double cdm_group_rician(const cdm_voxel_io& io, const float* sproto,
                                                   cdm_real* P, cdm_real* FixP, float tau, unsigned gmask) {
  float acc = 0.0f;
  int c0 = 0;
#if CDM_PAIRED
  // full chunk pairs through the paired signal hook (the pair table), the
  // log I0 term per measurement
  {
    const int full = io.nmeas / Gw;
    const float* q = io.pairs;
    const float* sig = io.sig;
    float2 acc2 = make_float2(0.0f, 0.0f);
    const float2 nht = make_float2(-0.5f * tau, -0.5f * tau);
    const float2 tau2 = make_float2(tau, tau);
#pragma unroll kPairUnroll
    for (; c0 + 1 < full; c0 += 2) {
      float2 ab[kNCOLS];
      cdm_load_pairs(q, ab);
      const float2 s2 = Predicted_Signal_Pair(P, ab, FixP);
      const float2 y2 = make_float2(sig[0], sig[io.chunk_stride]);
      const float2 e = __ffma2_rn(y2, y2, __fmul2_rn(s2, s2));
      acc2 = __ffma2_rn(nht, e, acc2);
      acc2 = __fadd2_rn(acc2, cdm_log_i0_fast2(__fmul2_rn(__fmul2_rn(tau2, s2), y2)));
      q += 2 * Gw * kNCOLSP;
      sig += 2 * io.chunk_stride;
    }
    acc = acc2.x + acc2.y;
  }
#endif
  for (int c = c0; c < io.nchunk; c++) {
    const int m = c * Gw + io.lane;
    const bool valid = m < io.nmeas;
    cdm_real cf[kNCOLS];
    cdm_load_cfp(sproto, io.nmeas_pad, valid ? m : 0, cf);
    const float y = io.sig[(size_t)c * io.chunk_stride];
    const float s = (float)Predicted_Signal(NPARAMS, P, cf, FixP);
    const float t = -0.5f * tau * (y * y + s * s) + cdm_log_i0_fast(tau * s * y);
    acc = valid ? acc + t : acc;
  }
  return cdm_group_sum<Gw>((double)acc, gmask);
}

// Sum of log(y) over the voxel (for BIC/AIC, which need the full Rician
// likelihood).
template <int Gw>
__device__ __forceinline__ double cdm_group_sum_log_meas(const cdm_voxel_io& io, unsigned gmask) {
  float acc = 0.0f;
  for (int c = 0; c < io.nchunk; c++) {
    const int m = c * Gw + io.lane;
    const float y = io.sig[(size_t)c * io.chunk_stride];
    acc = (m < io.nmeas) ? acc + logf(y) : acc;
  }
  return cdm_group_sum<Gw>((double)acc, gmask);
}

__device__ __forceinline__ void cdm_load_params(const double* __restrict__ src, cdm_real* P) {
#pragma unroll
  for (int i = 0; i < kNPS; i++) P[i] = cdm_real(0.0f);
#pragma unroll
  for (int i = 0; i < kNP; i++) P[i] = cdm_real((float)src[i]);
}

__device__ __forceinline__ void cdm_load_fixp(const double* __restrict__ src, int fixp_tsize,
                                              cdm_real* fixv) {
#pragma unroll
  for (int k = 0; k < kNFIX; k++) fixv[k] = cdm_real(k < fixp_tsize ? (float)src[k] : 0.0f);
}
