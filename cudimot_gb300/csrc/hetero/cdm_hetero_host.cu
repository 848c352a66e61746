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
  long opted_smem = 0;  // dynamic shared memory the kernel is opted in for
  unsigned args_bytes[kHxNumModels] = {};
  cdm_hx_item* d_items = nullptr;
  int* d_counter = nullptr;  // one per launch of a call
  int cap = 0;
  int counters = 0;
  int last_grid = 0;
  int last_launches = 0;
  unsigned char* d_args = nullptr;  // the constant slot table cdm_hx_args
  std::vector<cdm_hx_item> items;
  std::vector<unsigned char> slots;  // host image of the slot table, per launch
};

namespace {

cdm_status grow(cdm_hetero* h, int n, int launches) {
  if (n > h->cap) {
    const int cap = std::max(n, 2 * h->cap);
    cdm_hx_item* it = nullptr;
    HX_CUDA(cudaMalloc(&it, sizeof(cdm_hx_item) * cap));
    cudaFree(h->d_items);
    h->d_items = it;
    h->cap = cap;
  }
  if (launches > h->counters) {
    int* c = nullptr;
    HX_CUDA(cudaMalloc(&c, sizeof(int) * launches));
    cudaFree(h->d_counter);
    h->d_counter = c;
    h->counters = launches;
  }
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
  {
    void* p = nullptr;
    size_t bytes = 0;
    e = cudaLibraryGetGlobal(&p, &bytes, h->lib, "cdm_hx_args");
    if (e != cudaSuccess || bytes != sizeof(unsigned char) * CDM_HX_ENTRIES * CDM_HX_ARGS_BLOCK)
      return bail(fail(CDM_CUDA_ERROR, std::string("cdm_hx_args: ") + cudaGetErrorString(e)));
    h->d_args = static_cast<unsigned char*>(p);
  }
  const cdm_status s = grow(h, 16, 4);
  if (s != CDM_OK) return bail(s);
  *out = h;
  return CDM_OK;
}

cdm_status cdm_hetero_destroy(cdm_hetero* h) {
  if (!h) return CDM_OK;
  if (h->d_items) cudaFree(h->d_items);
  if (h->d_counter) cudaFree(h->d_counter);
  if (h->lib) cudaLibraryUnload(h->lib);
  delete h;
  return CDM_OK;
}

int cdm_hetero_last_grid(const cdm_hetero* h) { return h ? h->last_grid : 0; }

cdm_status cdm_hetero_mcmc(cdm_hetero* h, int n, const cdm_tile_work* items, void* stream) {
  if (!h) return fail(CDM_BAD_ARG, "null cdm_hetero");
  if (n < 0 || (n > 0 && !items)) return fail(CDM_BAD_ARG, "bad item list");
  // check every item first: nothing is launched for a bad list
  std::vector<int> fn(n, -1);
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
    if (w.args_bytes != h->args_bytes[m] || w.args_bytes > CDM_HX_ARGS_BLOCK)
      return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": argument block of " +
                                   std::to_string(w.args_bytes) + " bytes, the linked model's is " +
                                   std::to_string(h->args_bytes[m]));
    if (w.ntiles < 0 || !w.err) return fail(CDM_BAD_ARG, "item " + std::to_string(k) + ": not prepared");
    if (w.ntiles > 0) fn[k] = (m * kHxNumLanes + l) * 2 + (w.rician ? 1 : 0);
  }
  // launches: each fit's argument block has the slot of its entry, so fits
  // that share an entry (same model, lanes and likelihood) go to successive
  // launches, in order
  std::vector<std::vector<int>> groups;
  for (int k = 0; k < n; k++) {
    if (fn[k] < 0) continue;
    size_t g = 0;
    while (g < groups.size() &&
           std::any_of(groups[g].begin(), groups[g].end(), [&](int j) { return fn[j] == fn[k]; }))
      g++;
    if (g == groups.size()) groups.emplace_back();
    groups[g].push_back(k);
  }
  h->last_grid = 0;
  if (groups.empty()) return CDM_OK;
  const cdm_status gs = grow(h, n, (int)groups.size());
  if (gs != CDM_OK) return gs;
  cudaStream_t st = (cudaStream_t)stream;
  HX_CUDA(cudaMemsetAsync(h->d_counter, 0, sizeof(int) * groups.size(), st));
  h->items.clear();
  const size_t table = (size_t)CDM_HX_ENTRIES * CDM_HX_ARGS_BLOCK;
  h->slots.assign(table * groups.size(), 0);
  for (size_t g = 0; g < groups.size(); g++) {
    cdm_hx_launch L;
    std::memset(&L, 0, sizeof(L));
    unsigned char* slots = h->slots.data() + g * table;
    size_t max_sm = 0, max_scratch = 0;
    long tiles = 0;
    const size_t first = h->items.size();
    for (int k : groups[g]) {
      const cdm_tile_work& w = items[k];
      cdm_hx_item it;
      it.err = static_cast<int*>(w.err);
      it.fn = fn[k];
      it.tile0 = (int)tiles;
      it.ntiles = w.ntiles;
      it.pad = 0;
      h->items.push_back(it);
      std::memcpy(slots + (size_t)fn[k] * CDM_HX_ARGS_BLOCK, w.args, w.args_bytes);
      tiles += w.ntiles;
      max_sm = std::max(max_sm, (size_t)w.smem_bytes);
      max_scratch = std::max(max_scratch, (size_t)w.scratch_bytes);
    }
    if (tiles > 0x7fffffffL) return fail(CDM_BAD_ARG, "too many tiles");
    L.items = h->d_items + first;
    L.nitems = (int)(h->items.size() - first);
    L.ntiles = (int)tiles;
    L.counter = h->d_counter + g;
    L.scratch_off = (uint32_t)round16(max_sm);
    const size_t smem = L.scratch_off + max_scratch;
    if (smem + h->static_smem > 227 * 1024)
      return fail(CDM_BAD_ARG, "the fits need " + std::to_string(smem + h->static_smem) +
                                   " bytes of shared memory per CTA, more than 227 KB");
    // descriptors and argument slots of this launch, in stream order: a
    // later launch of the same call rewrites the slots only after this
    // launch has run
    HX_CUDA(cudaMemcpyAsync(h->d_items + first, h->items.data() + first,
                            sizeof(cdm_hx_item) * L.nitems, cudaMemcpyHostToDevice, st));
    HX_CUDA(cudaMemcpyAsync(h->d_args, slots, table, cudaMemcpyHostToDevice, st));
    // the opt-in only grows: an earlier launch of this call (or of an
    // earlier call) with more shared memory may still be queued
    if ((long)smem > h->opted_smem) {
      HX_CUDA(cudaFuncSetAttribute(h->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      h->opted_smem = (long)smem;
    }
    int per_sm = 0;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->kernel, kHxThreads, smem));
    if (per_sm < 1) return fail(CDM_BAD_ARG, "the persistent kernel does not fit on an SM");
    const int grid = (int)std::min<long>(tiles, (long)h->num_sms * per_sm);
    void* argv[] = {&L};
    HX_CUDA(cudaLaunchKernel(h->kernel, dim3(grid), dim3(kHxThreads), argv, smem, st));
    h->last_grid = std::max(h->last_grid, grid);
  }
  h->last_launches = (int)groups.size();
  return CDM_OK;
}

int cdm_hetero_last_launches(const cdm_hetero* h) { return h ? h->last_launches : 0; }

}  // extern "C"
