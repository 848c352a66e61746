// cdm_umma.cuh - BF16 GEMM on the 5th-generation tensor cores (tcgen05).
//
//   D[M x N] = A[M x K] * B[N x K]^T (+ epilogue),  A, B bf16 row-major with
//   K contiguous (both K-major), FP32 accumulation in tensor memory.
//
// One CTA computes a 128 x BN tile (BN <= 256, a multiple of 16) with 128
// threads:
//   * warp 0, lane 0 - TMA producer: 128x64 (A) and BNx64 (B) bf16 boxes of
//     the tensor maps, 128-byte swizzle, into a ring of shared-memory
//     stages, each completing a "full" mbarrier with its transaction bytes;
//   * warp 1, lane 0 - MMA issuer: per stage four tcgen05.mma
//     (kind::f16, M=128, N=BN, K=16) reading both operands through shared
//     memory descriptors, accumulating into BN TMEM columns;
//     tcgen05.commit frees the stage ("empty" mbarrier) and, after the last
//     stage, signals the epilogue;
//   * all four warps - epilogue: warp w owns TMEM lanes 32w..32w+31 (= tile
//     rows), reads 32 columns at a time with tcgen05.ld, applies the fused
//     epilogue and stores to global memory.
// Every mbarrier wait is bounded (%globaltimer, 2 s): on expiry the CTA
// writes kErrTimeout to the error word and skips to the TMEM release, so no
// wait can hang the GPU.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace cdm_mma {

constexpr int kBM = 128;     // tile rows (TMEM lanes)
constexpr int kBK = 64;      // bf16 elements per 128-byte swizzle row
// Ring depth: two stages for 256-wide tiles (two CTAs fit on an SM, so one
// CTA's epilogue overlaps the other's loads and MMAs), more for narrower.
__host__ __device__ constexpr int stages_for(int bn) { return bn >= 256 ? 2 : bn >= 144 ? 3 : 4; }
constexpr int kThreads = 128;
constexpr int kErrTimeout = 0x4D4D41;  // "MMA"
constexpr unsigned long long kWaitNs = 2000000000ull;

enum Epilogue : int {
  EPI_F32 = 0,        // out_f32[row][col] = acc
  EPI_BIAS_F32 = 1,   // out_f32 = acc + bias[col]
  EPI_BIAS_GELU = 2,  // z = acc + bias; out_bf16 = gelu(z); aux_bf16 = z; out_t (if set) = gelu(z)^T
  EPI_DGELU = 3       // out_bf16 = acc * gelu'(aux_bf16[row][col]); out_t (if set) = same^T
};

struct gemm_args {
  int M, N, K;             // valid sizes (rows of A, rows of B, reduction length)
  float* out_f32;          // [M][ld_out]
  __nv_bfloat16* out_bf16; // [M][ld_out]
  __nv_bfloat16* aux_bf16; // [M][ld_out] (pre-activation: written by BIAS_GELU, read by DGELU)
  __nv_bfloat16* out_t;    // [N][ld_t] transposed copy (optional)
  const float* bias;       // [N]
  int ld_out, ld_t;
  int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = gtime();
  while (!mbar_try(bar, parity)) {
    if (gtime() - t0 > kWaitNs) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor, K-major operand in 128-byte swizzle
// atoms of 8 rows x 128 bytes: start address >> 4 (bits 0-13), leading
// byte offset (unused for swizzled K-major, 16 B), stride byte offset 1024 B
// between 8-row groups (bits 32-45), descriptor version 1 (bits 46-47),
// layout SWIZZLE_128B = 2 (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor for kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, bits 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// GELU in its tanh form, 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))),
// with the hardware tanh approximation (tanh.approx.f32, relative error
// ~2^-11, below the bf16 rounding the activations get): five FP32
// operations and one MUFU instead of an erf. The network is defined with
// this form (training and inference), and the CPU oracle restates it.
constexpr float kGeluC0 = 0.7978845608028654f;               // sqrt(2/pi)
constexpr float kGeluC1 = 0.7978845608028654f * 0.044715f;

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float gelu(float z) {
  const float t = tanh_approx(z * fmaf(kGeluC1, z * z, kGeluC0));
  const float hz = 0.5f * z;
  return fmaf(hz, t, hz);
}

__device__ __forceinline__ float gelu_grad(float z) {
  const float z2 = z * z;
  const float t = tanh_approx(z * fmaf(kGeluC1, z2, kGeluC0));
  // d/dz: 0.5 (1 + t) + 0.5 z (1 - t^2) (c0 + 3 c1 z^2)
  const float du = fmaf(3.0f * kGeluC1, z2, kGeluC0);
  return fmaf(0.5f * z * fmaf(-t, t, 1.0f), du, 0.5f * (1.0f + t));
}

// TMEM columns to allocate for BN accumulator columns (power of two >= 32).
__host__ __device__ constexpr uint32_t tmem_cols(int bn) {
  return bn <= 32 ? 32u : bn <= 64 ? 64u : bn <= 128 ? 128u : 256u;
}

template <int BN>
struct smem_layout {
  static constexpr int kStages = stages_for(BN);
  static constexpr int kABytes = kBM * kBK * 2;  // 16 KB
  static constexpr int kBBytes = BN * kBK * 2;
  static constexpr int kStageBytes = kABytes + kBBytes;
  // stages (1024-aligned), then barriers; the bf16 output tile of the
  // epilogue ([128][BN + 8], padded rows) reuses the stage memory
  static constexpr int kOutLd = BN + 8;
  static constexpr int kBarOffset = kStages * kStageBytes;
  static constexpr int kBytes = kBarOffset + (2 * kStages + 1) * 8 + 16;
  static constexpr int kAlloc = kBytes + 1024;  // slack for 1024-byte alignment
  static_assert(kBM * kOutLd * 2 <= kBarOffset, "output tile must fit in the stage memory");
};

template <int BN, int EPI>
__global__ void __launch_bounds__(kThreads, 1)
    umma_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const __grid_constant__ gemm_args a) {
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "UMMA N for M=128");
  using L = smem_layout<BN>;
  constexpr int kStages = L::kStages;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + L::kBarOffset);
  uint64_t* empty = full + kStages;
  uint64_t* done = empty + kStages;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  __shared__ int abort_flag;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const int nk = (a.K + kBK - 1) / kBK;

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(tmem_cols(BN)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (kt >= kStages && !mbar_wait(&empty[s], ((kt / kStages) - 1) & 1)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      if (abort_flag) break;
      unsigned char* st = smem + s * L::kStageBytes;
      mbar_expect_tx(&full[s], L::kStageBytes);
      tma_load_2d(st, &tmA, &full[s], kt * kBK, m0);
      tma_load_2d(st + L::kABytes, &tmB, &full[s], kt * kBK, n0);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = instr_desc_bf16(kBM, BN);
    bool ok = true;
    for (int kt = 0; kt < nk && ok; kt++) {
      const int s = kt % kStages;
      if (!mbar_wait(&full[s], (kt / kStages) & 1)) {
        atomicExch(&abort_flag, 1);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = smem_u32(smem + s * L::kStageBytes);
      const uint32_t sb = sa + L::kABytes;
#pragma unroll
      for (int k = 0; k < kBK / 16; k++) {
        // advance K by 16 bf16 = 32 bytes inside the 128-byte swizzle row
        mma_bf16(tmem, smem_desc(sa + k * 32), smem_desc(sb + k * 32), idesc,
                 (kt > 0 || k > 0) ? 1u : 0u);
      }
      mma_commit(&empty[s]);
    }
    if (ok) mma_commit(done);
  }

  // Epilogue: every thread waits for the accumulator; the decision to read
  // it is made for the whole CTA (the staged path below has CTA barriers).
  bool ready = mbar_wait(done, 0);
  ready = __syncthreads_and(ready) != 0;
  if (!ready && threadIdx.x == 0) atomicExch(&abort_flag, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ready) {
    const int rloc = warp * 32 + lane;  // tile row (TMEM lane) of this thread
    const int row = m0 + rloc;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    if constexpr (EPI == EPI_F32 || EPI == EPI_BIAS_F32) {
      // fp32 rows straight from registers (128 contiguous bytes per chunk)
      const bool vec = (a.ld_out % 4) == 0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(lane_base + (uint32_t)c0, v);
        if (row >= a.M) continue;
        float* dst = a.out_f32 + (size_t)row * a.ld_out + n0 + c0;
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
          const int col = n0 + c0 + j;
          float4 q;
          q.x = v[j] + (EPI == EPI_BIAS_F32 && col + 0 < a.N ? a.bias[col + 0] : 0.0f);
          q.y = v[j + 1] + (EPI == EPI_BIAS_F32 && col + 1 < a.N ? a.bias[col + 1] : 0.0f);
          q.z = v[j + 2] + (EPI == EPI_BIAS_F32 && col + 2 < a.N ? a.bias[col + 2] : 0.0f);
          q.w = v[j + 3] + (EPI == EPI_BIAS_F32 && col + 3 < a.N ? a.bias[col + 3] : 0.0f);
          if (vec && c0 + j + 3 < BN && col + 3 < a.N) {
            *reinterpret_cast<float4*>(dst + j) = q;
          } else {
            const float e[4] = {q.x, q.y, q.z, q.w};
            for (int t = 0; t < 4; t++)
              if (c0 + j + t < BN && col + t < a.N) dst[j + t] = e[t];
          }
        }
      }
    } else {
      // bf16 outputs: each thread converts its row into a padded shared
      // tile, then the CTA writes whole rows with coalesced 16-byte stores.
      // BIAS_GELU with an aux output takes a second pass for z.
      constexpr int LD = L::kOutLd;
      __nv_bfloat16* stile = reinterpret_cast<__nv_bfloat16*>(smem);
      const int ncols = min(BN, a.N - n0);  // valid columns of this tile (a multiple of 8)
      const int passes = (EPI == EPI_BIAS_GELU && a.aux_bf16) ? 2 : 1;
      for (int pass = 0; pass < passes; pass++) {
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
          float v[32];
          tmem_ld32(lane_base + (uint32_t)c0, v);
          float zin[32];
          if constexpr (EPI == EPI_DGELU) {
#pragma unroll
            for (int j = 0; j < 32; j++) zin[j] = 0.0f;
            if (row < a.M && c0 < ncols) {
              const __nv_bfloat16* zr = a.aux_bf16 + (size_t)row * a.ld_out + n0 + c0;
#pragma unroll
              for (int q = 0; q < 4; q++)
                if (c0 + 8 * q < ncols) {
                  const uint4 raw = *reinterpret_cast<const uint4*>(zr + 8 * q);
                  const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&raw);
#pragma unroll
                  for (int t = 0; t < 8; t++) zin[8 * q + t] = __bfloat162float(h[t]);
                }
            }
          }
          __align__(16) __nv_bfloat16 o[32];
#pragma unroll
          for (int j = 0; j < 32; j++) {
            const int col = n0 + c0 + j;
            const bool ok = c0 + j < ncols;
            float val;
            if constexpr (EPI == EPI_BIAS_GELU) {
              const float z = __bfloat162float(__float2bfloat16(v[j] + (ok ? a.bias[col] : 0.0f)));
              val = pass == 0 ? gelu(z) : z;
            } else {
              val = v[j] * gelu_grad(zin[j]);
            }
            o[j] = __float2bfloat16(val);
            if (pass == 0 && a.out_t && ok && row < a.M) a.out_t[(size_t)col * a.ld_t + row] = o[j];
          }
          if (c0 < BN) {
#pragma unroll
            for (int q = 0; q < 4; q++)
              if (c0 + 8 * q < BN)
                *reinterpret_cast<uint4*>(stile + rloc * LD + c0 + 8 * q) =
                    *reinterpret_cast<const uint4*>(o + 8 * q);
          }
        }
        __syncthreads();
        __nv_bfloat16* gout = pass == 0 ? a.out_bf16 : a.aux_bf16;
        const int vpr = ncols / 8;  // 16-byte vectors per row
        for (int i = threadIdx.x; i < kBM * vpr; i += kThreads) {
          const int r = i / vpr, q = i % vpr;
          if (m0 + r < a.M)
            *reinterpret_cast<uint4*>(gout + (size_t)(m0 + r) * a.ld_out + n0 + 8 * q) =
                *reinterpret_cast<const uint4*>(stile + r * LD + 8 * q);
        }
        __syncthreads();
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (abort_flag && threadIdx.x == 0 && a.err) atomicExch(a.err, kErrTimeout);
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(tmem_cols(BN)));
  }
}

// ---------------------------------------------------------------------------
// Persistent hidden layer for inference: out_bf16 = bf16(gelu(bf16(A B^T +
// bias))) with N <= 256 (one 256-wide tile column), any M. One CTA per SM
// loops over the 128-row tiles (tile blockIdx.x, then every gridDim.x-th):
//   * warp 0, lane 0 - TMA producer over a 4-stage ring (A 128x64 and B
//     256x64 boxes), across tile boundaries;
//   * warp 1, lane 0 - MMA issuer; it accumulates tile j in one of two TMEM
//     accumulators (columns 256 (j & 1) .. +255 of a 512-column allocation),
//     so the MMAs of tile j+1 run while the epilogue drains tile j;
//   * warps 2..9 - epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (its
//     32 rows) and columns 128 ((w - 2) / 4) .. +127 of the accumulator, 32
//     at a time; bias (staged in shared memory), GELU, bf16; each 32 x 32
//     block goes through a per-warp shared-memory buffer so that the global
//     stores are whole 16-byte pieces, 64 contiguous bytes per row; then the
//     warp releases the accumulator (acc_empty, 8 arrivals).
// Every wait is bounded (2 s): on expiry the CTA stops its loops, records
// kErrTimeout and still releases its tensor memory.
namespace pers {
constexpr int kBN = 256;
constexpr int kStages = 3;
// 16 epilogue warps: four per SM sub-partition, so that one warp's TMEM
// load, shared-memory round trip and stores overlap three others' GELU
constexpr int kEpiWarps = 16;
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr int kColsPerWarp = kBN / (kEpiWarps / 4);  // 64: each TMEM lane quarter has 4 warps
constexpr int kABytes = kBM * kBK * 2;            // 16 KB
constexpr int kBBytes = kBN * kBK * 2;            // 32 KB
constexpr int kStageBytes = kABytes + kBBytes;    // 48 KB
// per epilogue warp: 32 rows x 32 bf16 (64 B per row, no padding); the
// 16-byte piece j of row r sits at slot j ^ ((r >> 1) & 3), so that both the
// row-per-lane writes and the four-pieces-per-row reads of a quarter warp
// touch eight different 16-byte bank groups
constexpr int kOutBytes = 32 * 64;
constexpr int kOffOut = kStages * kStageBytes;
constexpr int kOffBias = kOffOut + kEpiWarps * kOutBytes;
constexpr int kOffBar = kOffBias + kBN * 4;
constexpr int kBytes = kOffBar + (2 * kStages + 4) * 8 + 16;
constexpr int kAlloc = kBytes + 1024;  // slack for the 1024-byte alignment of the stages
// (the kernel's static shared memory, up to 1 KB with its alignment, comes on top)
static_assert(kAlloc + 1024 <= 227 * 1024, "shared memory of the persistent GEMM");
}  // namespace pers

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(pers::kThreads, 1)
    umma_gelu_persistent_kernel(const __grid_constant__ CUtensorMap tmA,
                                const __grid_constant__ CUtensorMap tmB,
                                const __grid_constant__ gemm_args a) {
  using namespace pers;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + kOffBar);
  uint64_t* empty = full + kStages;
  uint64_t* acc_full = empty + kStages;
  uint64_t* acc_empty = acc_full + 2;
  uint32_t* tmem_slot = (uint32_t*)(acc_empty + 2);
  float* sbias = (float*)(smem + kOffBias);
  __shared__ int abort_flag;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int ntiles = (a.M + kBM - 1) / kBM;
  const int nk = (a.K + kBK - 1) / kBK;
  const int ncols = min(kBN, a.N);

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kEpiWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  for (int i = threadIdx.x; i < kBN; i += blockDim.x) sbias[i] = i < a.N ? a.bias[i] : 0.0f;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t g = 0;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        for (int kt = 0; kt < nk; kt++, g++) {
          const uint32_t s = g % kStages;
          if (g >= (uint32_t)kStages && !mbar_wait(&empty[s], ((g / kStages) - 1) & 1)) {
            atomicExch(&abort_flag, 1);
            t = ntiles;
            break;
          }
          if (*(volatile int*)&abort_flag) {
            t = ntiles;
            break;
          }
          unsigned char* st = smem + s * kStageBytes;
          mbar_expect_tx(&full[s], kStageBytes);
          tma_load_2d(st, &tmA, &full[s], kt * kBK, t * kBM);
          tma_load_2d(st + kABytes, &tmB, &full[s], kt * kBK, 0);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = instr_desc_bf16(kBM, kBN);
      uint32_t g = 0;
      int j = 0;
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x, j++) {
        const int b = j & 1;
        if (j >= 2 && !mbar_wait(&acc_empty[b], ((j >> 1) - 1) & 1)) {
          atomicExch(&abort_flag, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + (uint32_t)(b * kBN);
        bool ok = true;
        for (int kt = 0; kt < nk; kt++, g++) {
          const uint32_t s = g % kStages;
          if (!mbar_wait(&full[s], (g / kStages) & 1)) {
            atomicExch(&abort_flag, 1);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(smem + s * kStageBytes);
          const uint32_t sb = sa + kABytes;
#pragma unroll
          for (int k = 0; k < kBK / 16; k++)
            mma_bf16(acc, smem_desc(sa + k * 32), smem_desc(sb + k * 32), idesc,
                     (kt > 0 || k > 0) ? 1u : 0u);
          mma_commit(&empty[s]);
        }
        if (!ok) break;
        mma_commit(&acc_full[b]);
      }
    }
  } else {
    const int q = warp % 4;             // TMEM lane quarter this warp may read
    const int h = (warp - 2) / 4;       // column quarter of the accumulator
    unsigned char* stage = smem + kOffOut + (warp - 2) * kOutBytes;
    int j = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, j++) {
      const int b = j & 1;
      if (!mbar_wait(&acc_full[b], (j >> 1) & 1)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int r0 = t * kBM + 32 * q;  // first global row of this warp
      const uint32_t base = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * kBN);
#pragma unroll 1
      for (int c = 0; c < kColsPerWarp / 32; c++) {
        const int c0 = h * kColsPerWarp + 32 * c;
        float v[32];
        tmem_ld32(base + (uint32_t)c0, v);
        uint32_t o[16];  // bf16 pairs
        const float4* b4 = reinterpret_cast<const float4*>(sbias + c0);  // broadcast loads
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const float4 b = b4[i];
          const float z0 = __bfloat162float(__float2bfloat16(v[4 * i] + b.x));
          const float z1 = __bfloat162float(__float2bfloat16(v[4 * i + 1] + b.y));
          const float z2 = __bfloat162float(__float2bfloat16(v[4 * i + 2] + b.z));
          const float z3 = __bfloat162float(__float2bfloat16(v[4 * i + 3] + b.w));
          const __nv_bfloat162 g01 = __floats2bfloat162_rn(gelu(z0), gelu(z1));
          const __nv_bfloat162 g23 = __floats2bfloat162_rn(gelu(z2), gelu(z3));
          o[2 * i] = *reinterpret_cast<const uint32_t*>(&g01);
          o[2 * i + 1] = *reinterpret_cast<const uint32_t*>(&g23);
        }
        const int sw = (lane >> 1) & 3;
#pragma unroll
        for (int p = 0; p < 4; p++)
          *reinterpret_cast<uint4*>(stage + lane * 64 + ((p ^ sw) << 4)) =
              make_uint4(o[4 * p], o[4 * p + 1], o[4 * p + 2], o[4 * p + 3]);
        __syncwarp();
#pragma unroll
        for (int p = lane; p < 128; p += 32) {
          const int r = p >> 2, j = p & 3, col = c0 + 8 * j;
          if (r0 + r < a.M && col < ncols)
            *reinterpret_cast<uint4*>(a.out_bf16 + (size_t)(r0 + r) * a.ld_out + col) =
                *reinterpret_cast<const uint4*>(stage + r * 64 + ((j ^ ((r >> 1) & 3)) << 4));
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (abort_flag && threadIdx.x == 0 && a.err) atomicExch(a.err, kErrTimeout);
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

}  // namespace cdm_mma
