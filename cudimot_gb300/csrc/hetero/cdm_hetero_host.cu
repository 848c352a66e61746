// cdm_hetero_host.cu - host half of the multi-model library (cdm_hetero.h).
//
// The device module (every model part device-linked with the persistent
// kernel) is embedded as cdm_hetero_image and loaded with the CUDA runtime's
// library API; cdm_hx_set.h (generated with it) names the models, their
// evaluation types and the lane counts compiled.
#include "cdm_hetero.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cdm_hetero_desc.h"
#include "cdm_hx_set.h"

extern "C" const unsigned char cdm_hetero_image[];

namespace {

thread_local std::string g_err;

cdm_status fail(cdm_status s, const std::string& m) {
  g_err = m;
  return s;
}

#define HX_CUDA(x)                                                                           \
  do {                                                                                       \
    cudaError_t e_ = (x);                                                                    \
    if (e_ != cudaSuccess) return fail(CDM_CUDA_ERROR, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

size_t round16(size_t x) { return (x + 15) & ~(size_t)15; }

}  // namespace

struct cdm_hetero {
  int device = 0;
  int num_sms = 0;
  cudaLibrary_t lib = nullptr;
  const void* kernel = nullptr;
  size_t static_smem = 0;
  unsigned args_bytes[kHxNumModels] = {};
  cdm_hx_item* d_items = nullptr;
  unsigned char* d_args = nullptr;
  int* d_counter = nullptr;
  int cap = 0;
  int last_grid = 0;
  std::vector<cdm_hx_item> items;
  std::vector<unsigned char> args;
};

namespace {

cdm_status grow(cdm_hetero* h, int n) {
  if (n <= h->cap) return CDM_OK;
  const int cap = std::max(n, 2 * h->cap);
  cdm_hx_item* it = nullptr;
  unsigned char* ar = nullptr;
  HX_CUDA(cudaMalloc(&it, sizeof(cdm_hx_item) * cap));
  if (cudaMalloc(&ar, (size_t)CDM_TILE_ARGS_MAX * cap) != cudaSuccess) {
    cudaFree(it);
    return fail(CDM_CUDA_ERROR, "cudaMalloc of the argument blocks failed");
  }
  cudaFree(h->d_items);
  cudaFree(h->d_args);
  h->d_items = it;
  h->d_args = ar;
  h->cap = cap;
  return CDM_OK;
}

// index of the item's model in this library, or -1
int model_index(const cdm_tile_work& w) {
  for (int m = 0; m < kHxNumModels; m++)
    if (std::strncmp(w.model, kHxModels[m], sizeof(w.model)) == 0 && w.eval_double == kHxEvalDouble[m])
      return m;
  return -1;
}

int lane_index(int lanes) {
  for (int l = 0; l < kHxNumLanes; l++)
    if (kHxLanes[l] == lanes) return l;
  return -1;
}

}  // namespace

extern "C" {

const char* cdm_hetero_last_error(void) { return g_err.c_str(); }

size_t cdm_hetero_models(char* buf, size_t cap) {
  std::string s;
  for (int m = 0; m < kHxNumModels; m++) {
    if (m) s += ",";
    s += std::string(kHxModels[m]) + (kHxEvalDouble[m] ? "/f64/" : "/f32/");
    for (int l = 0; l < kHxNumLanes; l++) s += (l ? ":" : "") + std::to_string(kHxLanes[l]);
  }
  if (buf && cap > s.size()) std::memcpy(buf, s.c_str(), s.size() + 1);
  return s.size();
}

cdm_status cdm_hetero_create(cdm_hetero** out) {
  if (!out) return fail(CDM_BAD_ARG, "null output");
  *out = nullptr;
  cdm_hetero* h = new cdm_hetero();
  auto bail = [&](cdm_status s) {
    cdm_hetero_destroy(h);
    return s;
  };
  if (cudaGetDevice(&h->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess)
    return bail(fail(CDM_CUDA_ERROR, "no CUDA device"));
  cudaError_t e = cudaLibraryLoadData(&h->lib, cdm_hetero_image, nullptr, nullptr, 0, nullptr,
                                      nullptr, 0);
  if (e != cudaSuccess)
    return bail(fail(CDM_CUDA_ERROR, std::string("loading the multi-model module: ") + cudaGetErrorString(e)));
  cudaKernel_t k = nullptr;
  e = cudaLibraryGetKernel(&k, h->lib, "cdm_hx_mcmc");
  if (e != cudaSuccess)
    return bail(fail(CDM_CUDA_ERROR, std::string("cdm_hx_mcmc: ") + cudaGetErrorString(e)));
  h->kernel = (const void*)k;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, h->kernel);
  if (e != cudaSuccess)
    return bail(fail(CDM_CUDA_ERROR, std::string("cdm_hx_mcmc attributes: ") + cudaGetErrorString(e)));
  h->static_smem = fa.sharedSizeBytes;
  for (int m = 0; m < kHxNumModels; m++) {
    char name[64];
    std::snprintf(name, sizeof(name), "cdm_hx_%d_args_bytes", m);
    void* p = nullptr;
    size_t bytes = 0;
    e = cudaLibraryGetGlobal(&p, &bytes, h->lib, name);
    if (e == cudaSuccess && bytes == sizeof(unsigned))
      e = cudaMemcpy(&h->args_bytes[m], p, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
      return bail(fail(CDM_CUDA_ERROR, std::string(name) + ": " + cudaGetErrorString(e)));
  }
  if (cudaMalloc(&h->d_counter, sizeof(int)) != cudaSuccess)
    return bail(fail(CDM_CUDA_ERROR, "cudaMalloc of the tile counter failed"));
  const cdm_status s = grow(h, 16);
  if (s != CDM_OK) return bail(s);
  *out = h;
  return CDM_OK;
}

cdm_status cdm_hetero_destroy(cdm_hetero* h) {
  if (!h) return CDM_OK;
  if (h->d_items) cudaFree(h->d_items);
  if (h->d_args) cudaFree(h->d_args);
  if (h->d_counter) cudaFree(h->d_counter);
  if (h->lib) cudaLibraryUnload(h->lib);
  delete h;
  return CDM_OK;
}

int cdm_hetero_last_grid(const cdm_hetero* h) { return h ? h->last_grid : 0; }

cdm_status cdm_hetero_mcmc(cdm_hetero* h, int n, const cdm_tile_work* items, void* stream) {
  if (!h) return fail(CDM_BAD_ARG, "null cdm_hetero");
  if (n < 0 || (n > 0 && !items)) return fail(CDM_BAD_ARG, "bad item list");
  h->items.clear();
  h->args.assign((size_t)std::max(n, 1) * CDM_TILE_ARGS_MAX, 0);
  size_t max_sm = 0, max_args = 0, max_scratch = 0;
  long tiles = 0;
  for (int k = 0; k < n; k++) {
    const cdm_tile_work& w = items[k];
    const int m = model_index(w);
    if (m < 0)
      return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": model " +
                                   std::string(w.model, strnlen(w.model, sizeof(w.model))) +
                                   (w.eval_double ? " (double)" : " (float)") +
                                   " is not linked into this library");
    const int l = lane_index(w.lanes);
    if (l < 0)
      return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": " + std::to_string(w.lanes) +
                                   " lanes per voxel are not compiled into this library");
    if (w.threads != kHxThreads)
      return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": built for " +
                                   std::to_string(w.threads) + " threads per CTA, this library for " +
                                   std::to_string(kHxThreads));
    if (w.args_bytes != h->args_bytes[m] || w.args_bytes % 4 || w.args_bytes > CDM_TILE_ARGS_MAX)
      return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": argument block of " +
                                   std::to_string(w.args_bytes) + " bytes, the linked model's is " +
                                   std::to_string(h->args_bytes[m]));
    if (w.ntiles < 0 || !w.err) return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": not prepared");
    if (w.ntiles == 0) continue;
    cdm_hx_item it;
    it.args = nullptr;  // set after the upload buffer is known
    it.err = static_cast<int*>(w.err);
    it.fn = (m * kHxNumLanes + l) * 2 + (w.rician ? 1 : 0);
    it.tile0 = (int)tiles;
    it.ntiles = w.ntiles;
    it.args_words = w.args_bytes / 4;
    std::memcpy(h->args.data() + h->items.size() * CDM_TILE_ARGS_MAX, w.args, w.args_bytes);
    h->items.push_back(it);
    tiles += w.ntiles;
    max_sm = std::max(max_sm, (size_t)w.smem_bytes);
    max_args = std::max(max_args, (size_t)w.args_bytes);
    max_scratch = std::max(max_scratch, (size_t)w.scratch_bytes);
  }
  h->last_grid = 0;
  if (h->items.empty()) return CDM_OK;
  if (tiles > 0x7fffffffL) return fail(CDM_BAD_ARG, "too many tiles");
  const int ni = (int)h->items.size();
  const cdm_status gs = grow(h, ni);
  if (gs != CDM_OK) return gs;
  for (int k = 0; k < ni; k++) h->items[k].args = h->d_args + (size_t)k * CDM_TILE_ARGS_MAX;
  cdm_hx_launch L;
  L.items = h->d_items;
  L.nitems = ni;
  L.ntiles = (int)tiles;
  L.counter = h->d_counter;
  L.args_off = (uint32_t)round16(max_sm);
  L.scratch_off = (uint32_t)round16(L.args_off + max_args);
  const size_t smem = L.scratch_off + max_scratch;
  if (smem + h->static_smem > 227 * 1024)
    return fail(CDM_BAD_ARG, "the fits need " + std::to_string(smem + h->static_smem) +
                                 " bytes of shared memory per CTA, more than 227 KB");
  cudaStream_t st = (cudaStream_t)stream;
  HX_CUDA(cudaMemcpyAsync(h->d_items, h->items.data(), sizeof(cdm_hx_item) * ni,
                          cudaMemcpyHostToDevice, st));
  HX_CUDA(cudaMemcpyAsync(h->d_args, h->args.data(), (size_t)CDM_TILE_ARGS_MAX * ni,
                          cudaMemcpyHostToDevice, st));
  HX_CUDA(cudaMemsetAsync(h->d_counter, 0, sizeof(int), st));
  HX_CUDA(cudaFuncSetAttribute(h->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->kernel, kHxThreads, smem));
  if (per_sm < 1) return fail(CDM_BAD_ARG, "the persistent kernel does not fit on an SM");
  const int grid = (int)std::min<long>(tiles, (long)h->num_sms * per_sm);
  void* argv[] = {&L};
  HX_CUDA(cudaLaunchKernel(h->kernel, dim3(grid), dim3(kHxThreads), argv, smem, st));
  h->last_grid = grid;
  return CDM_OK;
}

}  // extern "C"
