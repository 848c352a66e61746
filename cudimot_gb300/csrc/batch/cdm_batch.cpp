// cdm_batch.cpp - one CUDA graph over several model contexts (cdm_batch.h).
#include "cdm_batch.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

cdm_status fail(cdm_status s, const std::string& m) {
  g_err = m;
  return s;
}

#define BATCH_CUDA(x)                                                              \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) return fail(CDM_CUDA_ERROR, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

struct item {
  cdm_reserve_fn reserve;
  cdm_enqueue_fn enqueue;
  cdm_ctx* ctx;
  int nvox, nmeas;
  const double* meas;
  double* params;
  const double* CFP;
  const double* FixP;
  double *samples, *tau, *pred, *BIC, *AIC;
  double work;
};

}  // namespace

struct cdm_batch {
  std::vector<item> items;
  std::vector<cudaStream_t> branches;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaStream_t own = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t captured_on = nullptr;
};

extern "C" {

const char* cdm_batch_last_error(void) { return g_err.c_str(); }

cdm_status cdm_batch_create(cdm_batch** out) {
  if (!out) return fail(CDM_BAD_ARG, "null output");
  *out = new cdm_batch();
  return CDM_OK;
}

cdm_status cdm_batch_destroy(cdm_batch* b) {
  if (!b) return CDM_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (auto s : b->branches) cudaStreamDestroy(s);
  for (auto e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
  return CDM_OK;
}

cdm_status cdm_batch_add(cdm_batch* b, cdm_reserve_fn reserve, cdm_enqueue_fn enqueue,
                         cdm_ctx* ctx, int nvox, int nmeas, const double* meas, double* params,
                         const double* CFP, const double* FixP, double* samples, double* tau,
                         double* pred, double* BIC, double* AIC, double work) {
  if (!b || !reserve || !enqueue || !ctx) return fail(CDM_BAD_ARG, "null argument");
  if (nvox < 0 || nmeas <= 0) return fail(CDM_BAD_ARG, "bad nvox/nmeas");
  item it{reserve, enqueue, ctx, nvox, nmeas, meas, params, CFP, FixP,
          samples, tau, pred, BIC, AIC, work > 0 ? work : (double)nvox * nmeas};
  b->items.push_back(it);
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return CDM_OK;
}

cdm_status cdm_batch_run(cdm_batch* b, void* stream) {
  if (!b) return fail(CDM_BAD_ARG, "null batch");
  cudaStream_t st = (cudaStream_t)stream;
  if (b->items.empty()) return CDM_OK;
  if (!b->exec || b->captured_on != st) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    // every allocation before the capture
    for (auto& it : b->items) {
      cdm_status s = it.reserve(it.ctx, it.nvox, it.nmeas);
      if (s != CDM_OK) return fail(s, "cdm_fit_reserve failed for a batch item");
    }
    while (b->branches.size() < b->items.size()) {
      cudaStream_t s;
      cudaEvent_t e;
      BATCH_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      BATCH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      b->branches.push_back(s);
      b->joins.push_back(e);
    }
    if (!b->fork) BATCH_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    cudaStream_t cap = st;
    if (cap == nullptr || cap == cudaStreamLegacy || cap == cudaStreamPerThread) {
      if (!b->own) BATCH_CUDA(cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking));
      cap = b->own;
    }
    std::vector<size_t> order(b->items.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t x, size_t y) { return b->items[x].work > b->items[y].work; });
    BATCH_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    cdm_status s = CDM_OK;
    cudaError_t e = cudaEventRecord(b->fork, cap);
    for (size_t k = 0; k < order.size() && s == CDM_OK && e == cudaSuccess; k++) {
      const item& it = b->items[order[k]];
      e = cudaStreamWaitEvent(b->branches[k], b->fork, 0);
      if (e != cudaSuccess) break;
      s = it.enqueue(it.ctx, it.nvox, it.nmeas, it.meas, it.params, it.CFP, it.FixP, it.samples,
                     it.tau, it.pred, it.BIC, it.AIC, b->branches[k]);
      if (s != CDM_OK) break;
      e = cudaEventRecord(b->joins[k], b->branches[k]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(cap, b->joins[k], 0);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cap, &g);
    if (s != CDM_OK || e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (s != CDM_OK) return fail(s, "cdm_fit_enqueue failed for a batch item");
      return fail(CDM_CUDA_ERROR, std::string("batch capture: ") +
                                      cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      b->exec = nullptr;
      return fail(CDM_CUDA_ERROR, std::string("instantiate: ") + cudaGetErrorString(e));
    }
    b->captured_on = st;
  }
  BATCH_CUDA(cudaGraphLaunch(b->exec, st));
  return CDM_OK;
}

}  // extern "C"
