// cdm_mlp.cu - the learned initialiser: an MLP trained and run on the GPU
// with hand-written BF16 tensor-core kernels (cdm_umma.cuh).
//
// Network: n_in -> H -> H -> H -> n_out, GELU, BF16 weights and activations,
// FP32 accumulation, FP32 master weights with Adam. Output = n_mu means and
// n_sig log-standard-deviations; mean j is scored against sigma group
// group[j] with the Gaussian negative log-likelihood
//   L = 1/B sum_b sum_j [ 0.5 (t_j - mu_j)^2 exp(-2 s_g(j)) + s_g(j) ].
//
// A training step (forward, loss, backward, Adam) is a fixed sequence of
// launches on one stream, captured once into a CUDA graph per input buffer.
// The GEMMs are all "TN": both operands K-major; the transposed activations
// and gradients the weight gradients need are written by the producing
// GEMM's epilogue, and W^T for the input gradients by the Adam kernel.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "cdm_mlp.h"
#include "cdm_umma.cuh"

using namespace cdm_mma;

namespace {

thread_local std::string g_err;

cdm_status fail(cdm_status s, const std::string& m) {
  g_err = m;
  return s;
}

#define MLP_CUDA(x)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) return fail(CDM_CUDA_ERROR, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)
#define MLP_TRY(x)                 \
  do {                             \
    cdm_status s_ = (x);           \
    if (s_ != CDM_OK) return s_;   \
  } while (0)

// ------------------------------------------------------------ tensor maps
typedef CUresult (*encode_fn_t)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

encode_fn_t encoder() {
  static encode_fn_t fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (encode_fn_t)p;
  });
  return fn;
}

// 2-D bf16 map over a row-major [rows][ld] array, box [box_rows][64],
// 128-byte swizzle; out-of-range elements read as zero.
cdm_status make_map(CUtensorMap* m, const void* base, int rows, int cols, int ld, int box_rows) {
  encode_fn_t enc = encoder();
  if (!enc) return fail(CDM_CUDA_ERROR, "cuTensorMapEncodeTiled is not available");
  if (((uintptr_t)base & 15) || (ld * 2) % 16)
    return fail(CDM_BAD_ARG, "tensor map base must be 16-byte aligned and rows a multiple of 16 bytes");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(CDM_CUDA_ERROR, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return CDM_OK;
}

template <int BN, int EPI>
cdm_status launch_bn(const CUtensorMap& ta, const CUtensorMap& tb, const gemm_args& a,
                     cudaStream_t st) {
  auto k = umma_gemm_kernel<BN, EPI>;
  const int smem = smem_layout<BN>::kAlloc;
  static bool attr = false;  // set once per instantiation (outside any capture)
  if (!attr) {
    MLP_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr = true;
  }
  dim3 grid((a.M + kBM - 1) / kBM, (a.N + BN - 1) / BN);
  k<<<grid, kThreads, smem, st>>>(ta, tb, a);
  MLP_CUDA(cudaGetLastError());
  return CDM_OK;
}

// The persistent hidden-layer kernel (inference: bias + GELU, bf16 out,
// N <= 256): one CTA per SM.
cdm_status launch_persistent(const CUtensorMap& ta, const CUtensorMap& tb, const gemm_args& a,
                             cudaStream_t st) {
  static int sms = 0;
  static bool attr = false;
  if (!attr) {
    int dev = 0;
    MLP_CUDA(cudaGetDevice(&dev));
    MLP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MLP_CUDA(cudaFuncSetAttribute(umma_gelu_persistent_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, pers::kAlloc));
    attr = true;
  }
  const int tiles = (a.M + kBM - 1) / kBM;
  umma_gelu_persistent_kernel<<<std::max(1, std::min(tiles, sms)), pers::kThreads, pers::kAlloc,
                                st>>>(ta, tb, a);
  MLP_CUDA(cudaGetLastError());
  return CDM_OK;
}

template <int EPI>
cdm_status launch_epi(int bn, const CUtensorMap& ta, const CUtensorMap& tb, const gemm_args& a,
                      cudaStream_t st) {
  switch (bn) {
    case 16: return launch_bn<16, EPI>(ta, tb, a, st);
    case 144: return launch_bn<144, EPI>(ta, tb, a, st);
    case 256: return launch_bn<256, EPI>(ta, tb, a, st);
    default: return fail(CDM_BAD_ARG, "unsupported GEMM tile width");
  }
}

// Tile width for N output columns: one tile when N <= 256 (rounded up to a
// multiple of 16), 144 for N = 288.
int pick_bn(int N) {
  if (N <= 16) return 16;
  if (N <= 256) return 256;
  if (N % 144 == 0) return 144;
  return 256;
}

// A GEMM with its tensor maps.
struct gemm {
  CUtensorMap ta, tb;
  gemm_args a;
  int bn = 256, epi = EPI_F32;
};

cdm_status make_gemm(gemm* g, const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                     int epi, int* err) {
  g->bn = pick_bn(N);
  if (N <= 256 && g->bn == 256 && N <= 16) g->bn = 16;
  MLP_TRY(make_map(&g->ta, A, M, K, lda, kBM));
  MLP_TRY(make_map(&g->tb, B, N, K, ldb, g->bn));
  std::memset(&g->a, 0, sizeof(g->a));
  g->a.M = M;
  g->a.N = N;
  g->a.K = K;
  g->a.err = err;
  g->epi = epi;
  return CDM_OK;
}

cdm_status run_gemm(const gemm& g, cudaStream_t st) {
  if (g.epi == EPI_BIAS_GELU || g.epi == EPI_DGELU) {
    // the staged epilogue writes 16-byte row pieces
    const void* ptrs[3] = {g.a.out_bf16, g.a.aux_bf16, nullptr};
    for (const void* p : ptrs)
      if (p && ((uintptr_t)p & 15)) return fail(CDM_BAD_ARG, "bf16 GEMM outputs must be 16-byte aligned");
    if (g.a.ld_out % 8 || g.a.N % 8 || (g.epi == EPI_DGELU && !g.a.aux_bf16) || !g.a.out_bf16)
      return fail(CDM_BAD_ARG, "bf16 GEMM outputs need ld_out and N multiples of 8");
    if (g.bn < 256 && g.a.N > g.bn && (g.a.N % g.bn) % 8)
      return fail(CDM_BAD_ARG, "bf16 GEMM tile remainder must be a multiple of 8");
  }
  // inference hidden layers (no pre-activation or transposed copy) on the
  // persistent kernel
  if (g.epi == EPI_BIAS_GELU && !g.a.aux_bf16 && !g.a.out_t && g.a.N <= 256 && g.bn == 256)
    return launch_persistent(g.ta, g.tb, g.a, st);
  switch (g.epi) {
    case EPI_F32: return launch_epi<EPI_F32>(g.bn, g.ta, g.tb, g.a, st);
    case EPI_BIAS_F32: return launch_epi<EPI_BIAS_F32>(g.bn, g.ta, g.tb, g.a, st);
    case EPI_BIAS_GELU: return launch_epi<EPI_BIAS_GELU>(g.bn, g.ta, g.tb, g.a, st);
    case EPI_DGELU: return launch_epi<EPI_DGELU>(g.bn, g.ta, g.tb, g.a, st);
    default: return fail(CDM_BAD_ARG, "unknown epilogue");
  }
}

// ------------------------------------------------------------ small kernels

// Gaussian NLL head: out [B][ld_out] fp32 (n_mu means then n_sig
// log-stds), targets [B][n_mu]; writes d(loss)/d(out) as bf16 [B][ld_g]
// (zero beyond n_mu + n_sig), its transpose [ld_g][ldt] and per-row losses.
__global__ void nll_head_kernel(const float* __restrict__ out, int ld_out,
                                const float* __restrict__ tgt, int B, int n_mu, int n_sig,
                                const int* __restrict__ group, float smin, float smax,
                                __nv_bfloat16* __restrict__ g, int ld_g,
                                __nv_bfloat16* __restrict__ gt, int ldt,
                                float* __restrict__ row_loss) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float* o = out + (size_t)b * ld_out;
  float ds[16];
  float s[16];
  for (int k = 0; k < n_sig; k++) {
    s[k] = fminf(fmaxf(o[n_mu + k], smin), smax);
    ds[k] = 0.0f;
  }
  float loss = 0.0f;
  const float invB = 1.0f / (float)B;
  for (int j = 0; j < ld_g; j++) {
    float gj = 0.0f;
    if (j < n_mu) {
      const int k = group[j];
      const float w = __expf(-2.0f * s[k]);
      const float r = o[j] - tgt[(size_t)b * n_mu + j];
      loss += 0.5f * r * r * w + s[k];
      gj = r * w * invB;
      ds[k] += 1.0f - r * r * w;
    }
    if (j < ld_g) {
      g[(size_t)b * ld_g + j] = __float2bfloat16(gj);
    }
  }
  for (int k = 0; k < n_sig; k++) {
    const float raw = o[n_mu + k];
    const float gk = (raw > smin && raw < smax) ? ds[k] * invB : 0.0f;
    g[(size_t)b * ld_g + n_mu + k] = __float2bfloat16(gk);
  }
  for (int j = 0; j < ld_g; j++) gt[(size_t)j * ldt + b] = g[(size_t)b * ld_g + j];
  row_loss[b] = loss;
}

// Column sums of a bf16 [B][ld] matrix (bias gradients), FP32; one block
// per 32 columns, threads stride the rows.
__global__ void colsum_kernel(const __nv_bfloat16* __restrict__ x, int B, int n, int ld,
                              float* __restrict__ out) {
  __shared__ float part[8][33];
  const int c = blockIdx.x * 32 + (threadIdx.x & 31);
  const int r0 = threadIdx.x >> 5;
  float acc = 0.0f;
  if (c < n)
    for (int r = r0; r < B; r += 8) acc += __bfloat162float(x[(size_t)r * ld + c]);
  part[r0][threadIdx.x & 31] = acc;
  __syncthreads();
  if (r0 == 0 && c < n) {
    float t = 0.0f;
    for (int k = 0; k < 8; k++) t += part[k][threadIdx.x & 31];
    out[c] = t;
  }
}

// Sum of per-row losses / B into loss[0] (single block).
__global__ void loss_sum_kernel(const float* __restrict__ row_loss, int B, float* __restrict__ loss) {
  __shared__ float sh[256];
  float acc = 0.0f;
  for (int i = threadIdx.x; i < B; i += blockDim.x) acc += row_loss[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[0] = sh[0] / (float)B;
}

// Adam on one layer (weights [rows][cols] and bias [rows]) from FP32
// gradients; refreshes the bf16 copy W [rows_pad][cols] and its transpose
// WT [cols][rows_pad] used by the forward and input-gradient GEMMs.
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ grad, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2, int rows, int cols, int wt_ld,
                            __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) {
      const int r = i / cols, c = i % cols;
      const __nv_bfloat16 q = __float2bfloat16(wi);
      wb[i] = q;
      if (wt) wt[(size_t)c * wt_ld + r] = q;
    }
  }
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ x, int n, int rows, int cols,
                                   int wt_ld, __nv_bfloat16* __restrict__ y,
                                   __nv_bfloat16* __restrict__ yt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const __nv_bfloat16 q = __float2bfloat16(x[i]);
    y[i] = q;
    if (yt) yt[(size_t)(i % cols) * wt_ld + i / cols] = q;
  }
}

// signals [n][nmeas] (double) / S0 [n] -> bf16 [n][ld] (zero padded)
__global__ void prep_input_kernel(const double* __restrict__ meas, const double* __restrict__ s0,
                                  int s0_ld, int n, int nmeas, int ld,
                                  __nv_bfloat16* __restrict__ x) {
  const size_t total = (size_t)n * ld;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / ld), c = (int)(i % ld);
    float v = 0.0f;
    if (c < nmeas) {
      const double d = s0 ? s0[(size_t)r * s0_ld] : 1.0;
      v = (float)(meas[(size_t)r * nmeas + c] / (d > 0.0 ? d : 1.0));
    }
    x[i] = __float2bfloat16(v);
  }
}

int blocks_for(size_t n, int t = 256) { return (int)std::min<size_t>((n + t - 1) / t, 152 * 16); }

}  // namespace

// ================================================================ MLP object
struct cdm_mlp {
  cdm_mlp_cfg cfg;
  int dims[5];           // n_in, H, H, H, n_out
  int pad_out;           // n_out rounded up to 16
  int B = 0;             // training batch the buffers are sized for
  // parameters (fp32 master), Adam state, gradients
  float *w[4] = {}, *bias[4] = {}, *mw[4] = {}, *vw[4] = {}, *mb[4] = {}, *vb[4] = {};
  float *gw[4] = {}, *gb[4] = {};
  __nv_bfloat16 *wb[4] = {}, *wt[4] = {};   // bf16 W [rows_pad][in], W^T [in][rows_pad]
  // activations for batch B
  __nv_bfloat16 *z[3] = {}, *act[3] = {}, *actT[3] = {}, *dz[3] = {}, *dzT[3] = {};
  __nv_bfloat16 *xT = nullptr, *gout = nullptr, *goutT = nullptr;
  float *out = nullptr, *row_loss = nullptr, *loss = nullptr;
  int* group = nullptr;
  int* err = nullptr;
  int step = 0;
  // inference buffers
  int inf_cap = 0;
  __nv_bfloat16 *iz = nullptr, *ia[2] = {};
  // captured training step
  cudaGraphExec_t graph = nullptr;
  const void* graph_x = nullptr;
  const void* graph_t = nullptr;
  cudaStream_t graph_st = nullptr;
  cudaStream_t own = nullptr;
  std::vector<void*> allocs;
};

namespace {

template <class T>
cdm_status alloc(cdm_mlp* m, T** p, size_t n) {
  void* q = nullptr;
  MLP_CUDA(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
  MLP_CUDA(cudaMemset(q, 0, std::max<size_t>(n, 1) * sizeof(T)));
  m->allocs.push_back(q);
  *p = (T*)q;
  return CDM_OK;
}

int rows_pad(const cdm_mlp* m, int l) { return l == 3 ? m->pad_out : m->dims[l + 1]; }

cdm_status ensure_batch(cdm_mlp* m, int B) {
  if (m->B >= B) return CDM_OK;
  if (m->B) return fail(CDM_BAD_ARG, "the training batch size cannot grow after the first step");
  const int H = m->cfg.hidden, nin = m->dims[0];
  for (int l = 0; l < 3; l++) {
    MLP_TRY(alloc(m, &m->z[l], (size_t)B * H));
    MLP_TRY(alloc(m, &m->act[l], (size_t)B * H));
    MLP_TRY(alloc(m, &m->actT[l], (size_t)B * H));
    MLP_TRY(alloc(m, &m->dz[l], (size_t)B * H));
    MLP_TRY(alloc(m, &m->dzT[l], (size_t)B * H));
  }
  MLP_TRY(alloc(m, &m->xT, (size_t)nin * B));
  MLP_TRY(alloc(m, &m->gout, (size_t)B * m->pad_out));
  MLP_TRY(alloc(m, &m->goutT, (size_t)m->pad_out * B));
  MLP_TRY(alloc(m, &m->out, (size_t)B * m->pad_out));
  MLP_TRY(alloc(m, &m->row_loss, (size_t)B));
  m->B = B;
  return CDM_OK;
}

// x [B][n_in] bf16 -> x^T [n_in][B]
__global__ void transpose_bf16_kernel(const __nv_bfloat16* __restrict__ x, int rows, int cols,
                                      __nv_bfloat16* __restrict__ y) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[i][threadIdx.x] = x[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) y[(size_t)c * rows + r] = t[threadIdx.x][i];
  }
}

// Forward of the hidden layers and the output layer for `n` rows of x.
// Writes fp32 outputs [n][pad_out]. With `train`, the batch buffers
// (z, act, actT) are used; otherwise the inference ping-pong buffers.
cdm_status forward(cdm_mlp* m, const __nv_bfloat16* x, int n, float* out, bool train,
                   cudaStream_t st) {
  const int H = m->cfg.hidden;
  const __nv_bfloat16* in = x;
  int ld_in = m->dims[0];
  for (int l = 0; l < 3; l++) {
    gemm g;
    MLP_TRY(make_gemm(&g, in, ld_in, m->wb[l], m->dims[l], n, H, m->dims[l], EPI_BIAS_GELU, m->err));
    g.a.bias = m->bias[l];
    g.a.ld_out = H;
    if (train) {
      g.a.aux_bf16 = m->z[l];
      g.a.out_bf16 = m->act[l];
      g.a.out_t = m->actT[l];
      g.a.ld_t = n;
    } else {
      g.a.aux_bf16 = nullptr;  // the pre-activation is only needed for training
      g.a.out_bf16 = m->ia[l & 1];
    }
    MLP_TRY(run_gemm(g, st));
    in = g.a.out_bf16;
    ld_in = H;
  }
  gemm g;
  MLP_TRY(make_gemm(&g, in, H, m->wb[3], H, n, m->dims[4], H, EPI_BIAS_F32, m->err));
  g.a.bias = m->bias[3];
  g.a.out_f32 = out;
  g.a.ld_out = m->pad_out;
  return run_gemm(g, st);
}

// Loss, backward and (optionally) Adam for the batch in m's buffers.
cdm_status backward(cdm_mlp* m, const __nv_bfloat16* x, const float* tgt, bool update,
                    cudaStream_t st) {
  const int B = m->B, H = m->cfg.hidden, n_mu = m->cfg.n_mu, n_sig = m->cfg.n_sig;
  nll_head_kernel<<<(B + 127) / 128, 128, 0, st>>>(m->out, m->pad_out, tgt, B, n_mu, n_sig,
                                                   m->group, m->cfg.logstd_min, m->cfg.logstd_max,
                                                   m->gout, m->pad_out, m->goutT, B, m->row_loss);
  MLP_CUDA(cudaGetLastError());
  loss_sum_kernel<<<1, 256, 0, st>>>(m->row_loss, B, m->loss);
  MLP_CUDA(cudaGetLastError());
  {
    dim3 tb(32, 8), gr((m->dims[0] + 31) / 32, (B + 31) / 32);
    transpose_bf16_kernel<<<gr, tb, 0, st>>>(x, B, m->dims[0], m->xT);
    MLP_CUDA(cudaGetLastError());
  }
  // layer 4 (output): dW4 = gout^T x act3, db4 = colsum(gout), d act3 = gout x W4
  const __nv_bfloat16* gT = m->goutT;  // [rows of this layer][B]
  const __nv_bfloat16* gN = m->gout;   // [B][rows]
  int g_rows = m->pad_out, g_ld = m->pad_out;
  for (int l = 3; l >= 0; l--) {
    const int nin = m->dims[l];
    const __nv_bfloat16* inT = l == 0 ? m->xT : m->actT[l - 1];
    {  // weight gradient [rows][nin] = g^T (rows x B) . in^T (nin x B)^T
      gemm g;
      MLP_TRY(make_gemm(&g, gT, B, inT, B, m->dims[l + 1], nin, B, EPI_F32, m->err));
      g.a.out_f32 = m->gw[l];
      g.a.ld_out = nin;
      MLP_TRY(run_gemm(g, st));
    }
    colsum_kernel<<<(m->dims[l + 1] + 31) / 32, 256, 0, st>>>(gN, B, m->dims[l + 1], g_ld, m->gb[l]);
    MLP_CUDA(cudaGetLastError());
    if (l > 0) {  // input gradient through GELU: dz[l-1] = (g . W) * gelu'(z[l-1])
      gemm g;
      MLP_TRY(make_gemm(&g, gN, g_ld, m->wt[l], rows_pad(m, l), B, nin, g_rows, EPI_DGELU, m->err));
      g.a.aux_bf16 = m->z[l - 1];
      g.a.out_bf16 = m->dz[l - 1];
      g.a.out_t = m->dzT[l - 1];
      g.a.ld_out = H;
      g.a.ld_t = B;
      MLP_TRY(run_gemm(g, st));
      gN = m->dz[l - 1];
      gT = m->dzT[l - 1];
      g_rows = H;
      g_ld = H;
    }
  }
  if (update) {
    m->step++;
    const float b1 = m->cfg.beta1, b2 = m->cfg.beta2;
    const float c1 = 1.0f - powf(b1, (float)m->step), c2 = 1.0f - powf(b2, (float)m->step);
    for (int l = 0; l < 4; l++) {
      const int rows = m->dims[l + 1], cols = m->dims[l];
      const int n = rows * cols;
      adam_kernel<<<blocks_for(n), 256, 0, st>>>(m->w[l], m->mw[l], m->vw[l], m->gw[l], n,
                                                  m->cfg.lr, b1, b2, m->cfg.eps, c1, c2, rows,
                                                  cols, rows_pad(m, l), m->wb[l], m->wt[l]);
      MLP_CUDA(cudaGetLastError());
      adam_kernel<<<1, 256, 0, st>>>(m->bias[l], m->mb[l], m->vb[l], m->gb[l], rows, m->cfg.lr,
                                     b1, b2, m->cfg.eps, c1, c2, rows, 1, 0, nullptr, nullptr);
      MLP_CUDA(cudaGetLastError());
    }
  }
  return CDM_OK;
}

cdm_status refresh_bf16(cdm_mlp* m, cudaStream_t st) {
  for (int l = 0; l < 4; l++) {
    const int rows = m->dims[l + 1], cols = m->dims[l];
    f32_to_bf16_kernel<<<blocks_for((size_t)rows * cols), 256, 0, st>>>(
        m->w[l], rows * cols, rows, cols, rows_pad(m, l), m->wb[l], m->wt[l]);
    MLP_CUDA(cudaGetLastError());
  }
  return CDM_OK;
}

}  // namespace

extern "C" {

const char* cdm_mlp_last_error(void) { return g_err.c_str(); }

void cdm_mlp_default_cfg(cdm_mlp_cfg* c) {
  std::memset(c, 0, sizeof(*c));
  c->n_in = 288;
  c->hidden = 256;
  c->n_mu = 8;
  c->n_sig = 4;
  const int grp[8] = {0, 1, 2, 3, 3, 3, 3, 3};
  for (int i = 0; i < 8; i++) c->group[i] = grp[i];
  c->lr = 1e-3f;
  c->beta1 = 0.9f;
  c->beta2 = 0.999f;
  c->eps = 1e-8f;
  c->logstd_min = -7.0f;
  c->logstd_max = 3.0f;
}

cdm_status cdm_mlp_create(const cdm_mlp_cfg* cfg, cdm_mlp** out) {
  if (!cfg || !out) return fail(CDM_BAD_ARG, "null argument");
  const int nout = cfg->n_mu + cfg->n_sig;
  if (cfg->n_in <= 0 || cfg->n_in % 8 || cfg->hidden <= 0 || cfg->hidden % 16 || cfg->hidden > 256 ||
      cfg->n_mu <= 0 || cfg->n_sig <= 0 || cfg->n_sig > 16 || nout > 16 || cfg->n_mu > CDM_MLP_MAX_MU)
    return fail(CDM_BAD_ARG, "unsupported network shape (n_in multiple of 8, hidden multiple of 16 "
                             "and <= 256, n_mu + n_sig <= 16)");
  if (cfg->n_in > 256 && cfg->n_in % 144 && cfg->n_in % 256)
    return fail(CDM_BAD_ARG, "n_in above 256 must be a multiple of 144 or 256");
  for (int j = 0; j < cfg->n_mu; j++)
    if (cfg->group[j] < 0 || cfg->group[j] >= cfg->n_sig) return fail(CDM_BAD_ARG, "bad sigma group");
  cdm_mlp* m = new cdm_mlp();
  m->cfg = *cfg;
  m->dims[0] = cfg->n_in;
  m->dims[1] = m->dims[2] = m->dims[3] = cfg->hidden;
  m->dims[4] = nout;
  m->pad_out = 16;
  cdm_status s = CDM_OK;
  for (int l = 0; l < 4 && s == CDM_OK; l++) {
    const size_t rows = m->dims[l + 1], cols = m->dims[l], rp = rows_pad(m, l);
    s = alloc(m, &m->w[l], rows * cols);
    if (s == CDM_OK) s = alloc(m, &m->bias[l], rows);
    if (s == CDM_OK) s = alloc(m, &m->mw[l], rows * cols);
    if (s == CDM_OK) s = alloc(m, &m->vw[l], rows * cols);
    if (s == CDM_OK) s = alloc(m, &m->mb[l], rows);
    if (s == CDM_OK) s = alloc(m, &m->vb[l], rows);
    if (s == CDM_OK) s = alloc(m, &m->gw[l], rows * cols);
    if (s == CDM_OK) s = alloc(m, &m->gb[l], rows);
    if (s == CDM_OK) s = alloc(m, &m->wb[l], rp * cols);
    if (s == CDM_OK) s = alloc(m, &m->wt[l], cols * rp);
  }
  if (s == CDM_OK) s = alloc(m, &m->group, 16);
  if (s == CDM_OK) s = alloc(m, &m->loss, 1);
  if (s == CDM_OK) s = alloc(m, &m->err, 1);
  if (s == CDM_OK && cudaMemcpy(m->group, cfg->group, sizeof(int) * cfg->n_mu, cudaMemcpyHostToDevice) != cudaSuccess)
    s = fail(CDM_CUDA_ERROR, "copy of sigma groups failed");
  if (s != CDM_OK) {
    cdm_mlp_destroy(m);
    return s;
  }
  *out = m;
  return CDM_OK;
}

cdm_status cdm_mlp_destroy(cdm_mlp* m) {
  if (!m) return CDM_OK;
  if (m->graph) cudaGraphExecDestroy(m->graph);
  if (m->own) cudaStreamDestroy(m->own);
  for (void* p : m->allocs) cudaFree(p);
  delete m;
  return CDM_OK;
}

cdm_status cdm_mlp_set_params(cdm_mlp* m, int layer, const float* w, const float* b) {
  if (!m || layer < 0 || layer > 3 || !w || !b) return fail(CDM_BAD_ARG, "bad argument");
  const size_t rows = m->dims[layer + 1], cols = m->dims[layer];
  MLP_CUDA(cudaMemcpy(m->w[layer], w, rows * cols * sizeof(float), cudaMemcpyDefault));
  MLP_CUDA(cudaMemcpy(m->bias[layer], b, rows * sizeof(float), cudaMemcpyDefault));
  MLP_CUDA(cudaMemset(m->mw[layer], 0, rows * cols * sizeof(float)));
  MLP_CUDA(cudaMemset(m->vw[layer], 0, rows * cols * sizeof(float)));
  MLP_CUDA(cudaMemset(m->mb[layer], 0, rows * sizeof(float)));
  MLP_CUDA(cudaMemset(m->vb[layer], 0, rows * sizeof(float)));
  m->step = 0;
  MLP_TRY(refresh_bf16(m, nullptr));
  MLP_CUDA(cudaDeviceSynchronize());
  return CDM_OK;
}

cdm_status cdm_mlp_get_params(cdm_mlp* m, int layer, float* w, float* b, float* gw, float* gb) {
  if (!m || layer < 0 || layer > 3) return fail(CDM_BAD_ARG, "bad argument");
  const size_t rows = m->dims[layer + 1], cols = m->dims[layer];
  MLP_CUDA(cudaDeviceSynchronize());
  if (w) MLP_CUDA(cudaMemcpy(w, m->w[layer], rows * cols * sizeof(float), cudaMemcpyDefault));
  if (b) MLP_CUDA(cudaMemcpy(b, m->bias[layer], rows * sizeof(float), cudaMemcpyDefault));
  if (gw) MLP_CUDA(cudaMemcpy(gw, m->gw[layer], rows * cols * sizeof(float), cudaMemcpyDefault));
  if (gb) MLP_CUDA(cudaMemcpy(gb, m->gb[layer], rows * sizeof(float), cudaMemcpyDefault));
  return CDM_OK;
}

cdm_status cdm_mlp_gradients(cdm_mlp* m, const void* x, const float* targets, int batch,
                             float* loss, void* stream) {
  if (!m || !x || !targets || batch <= 0) return fail(CDM_BAD_ARG, "bad argument");
  MLP_TRY(ensure_batch(m, batch));
  if (batch != m->B) return fail(CDM_BAD_ARG, "batch differs from the buffers' batch size");
  cudaStream_t st = (cudaStream_t)stream;
  MLP_TRY(forward(m, (const __nv_bfloat16*)x, batch, m->out, true, st));
  MLP_TRY(backward(m, (const __nv_bfloat16*)x, targets, false, st));
  if (loss) MLP_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDefault, st));
  return CDM_OK;
}

cdm_status cdm_mlp_train_step(cdm_mlp* m, const void* x, const float* targets, int batch,
                              float* loss, void* stream) {
  if (!m || !x || !targets || batch <= 0) return fail(CDM_BAD_ARG, "bad argument");
  MLP_TRY(ensure_batch(m, batch));
  if (batch != m->B) return fail(CDM_BAD_ARG, "batch differs from the buffers' batch size");
  cudaStream_t st = (cudaStream_t)stream;
  // Adam's bias corrections change every step and are kernel arguments, so
  // the step is launched directly (about 25 launches); the GEMMs dominate.
  MLP_TRY(forward(m, (const __nv_bfloat16*)x, batch, m->out, true, st));
  MLP_TRY(backward(m, (const __nv_bfloat16*)x, targets, true, st));
  if (loss) MLP_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDefault, st));
  return CDM_OK;
}

cdm_status cdm_mlp_forward(cdm_mlp* m, const void* x, int n, float* out, void* stream) {
  if (!m || !x || !out || n < 0) return fail(CDM_BAD_ARG, "bad argument");
  if (n == 0) return CDM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int chunk = 1 << 18;
  if (m->inf_cap < std::min(n, chunk)) {
    const int cap = std::min(n, chunk);
    MLP_TRY(alloc(m, &m->iz, (size_t)cap * m->cfg.hidden));
    MLP_TRY(alloc(m, &m->ia[0], (size_t)cap * m->cfg.hidden));
    MLP_TRY(alloc(m, &m->ia[1], (size_t)cap * m->cfg.hidden));
    m->inf_cap = cap;
  }
  for (int r0 = 0; r0 < n; r0 += chunk) {
    const int rows = std::min(chunk, n - r0);
    MLP_TRY(forward(m, (const __nv_bfloat16*)x + (size_t)r0 * m->dims[0], rows,
                    out + (size_t)r0 * m->pad_out, false, st));
  }
  return CDM_OK;
}

cdm_status cdm_mlp_hidden_layer(cdm_mlp* m, int layer, const void* x, int ld_x, int n, void* out,
                                int ld_out, void* stream) {
  if (!m || !x || !out || n < 0 || layer < 0 || layer > 2) return fail(CDM_BAD_ARG, "bad argument");
  if (ld_x < m->dims[layer] || ld_out < m->cfg.hidden) return fail(CDM_BAD_ARG, "bad leading dimension");
  if (n == 0) return CDM_OK;
  gemm g;
  MLP_TRY(make_gemm(&g, x, ld_x, m->wb[layer], m->dims[layer], n, m->cfg.hidden, m->dims[layer],
                    EPI_BIAS_GELU, m->err));
  g.a.bias = m->bias[layer];
  g.a.ld_out = ld_out;
  g.a.out_bf16 = (__nv_bfloat16*)out;
  return run_gemm(g, (cudaStream_t)stream);
}

cdm_status cdm_mlp_prep_input(const double* meas, const double* s0, int s0_ld, int n, int nmeas,
                              int ld, void* x, void* stream) {
  if (!meas || !x || n < 0 || nmeas <= 0 || ld < nmeas || ld % 8) return fail(CDM_BAD_ARG, "bad argument");
  if (n == 0) return CDM_OK;
  prep_input_kernel<<<blocks_for((size_t)n * ld), 256, 0, (cudaStream_t)stream>>>(
      meas, s0, s0_ld, n, nmeas, ld, (__nv_bfloat16*)x);
  MLP_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_mlp_gemm_bf16(const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                             float* out, int ld_out, void* stream) {
  if (!A || !B || !out || M <= 0 || N <= 0 || K <= 0) return fail(CDM_BAD_ARG, "bad argument");
  if (N > 256 && N % 144 && N % 256) return fail(CDM_BAD_ARG, "N above 256 must be a multiple of 144 or 256");
  static int* err = nullptr;
  if (!err) MLP_CUDA(cudaMalloc(&err, sizeof(int)));
  gemm g;
  MLP_TRY(make_gemm(&g, A, lda, B, ldb, M, N, K, EPI_F32, err));
  g.a.out_f32 = out;
  g.a.ld_out = ld_out;
  return run_gemm(g, (cudaStream_t)stream);
}

cdm_status cdm_mlp_check(cdm_mlp* m) {
  if (!m) return fail(CDM_BAD_ARG, "null");
  int e = 0;
  MLP_CUDA(cudaMemcpy(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    MLP_CUDA(cudaMemset(m->err, 0, sizeof(int)));
    return fail(CDM_TIMEOUT, "a bounded tensor-core pipeline wait ran out");
  }
  return CDM_OK;
}

}  // extern "C"
