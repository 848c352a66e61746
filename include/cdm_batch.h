/* cdm_batch.h - several fits (models, protocols, volumes) in one CUDA graph.
 *
 * No counterpart in CUDIMOT, which fits one model on one volume per
 * process (cudimot.cc:57-125). Each item is a context of some model library
 * (libcudimot_<Model>.so) with its arrays, as for cdm_fit; the batch records
 * every item's stage sequence (cdm_fit_enqueue) on its own branch of one
 * graph - fork from the launch stream, one branch per item, join - so a
 * single graph launch runs all of them and their kernels share the GPU: the
 * hardware block scheduler fills SMs left idle by one model's kernels with
 * another's. The graph is captured on the first cdm_batch_run and reused
 * while the items are unchanged. Items are enqueued in decreasing order of
 * their estimated work (voxels x measurements x iterations).
 */
#ifndef CDM_BATCH_H
#define CDM_BATCH_H

#include "cudimot_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cdm_batch cdm_batch;  /* cdm_ctx comes from cudimot_gb300.h */

/* cdm_fit_reserve / cdm_fit_enqueue of the item's model library */
typedef cdm_status (*cdm_reserve_fn)(cdm_ctx*, int nvox, int nmeas);
typedef cdm_status (*cdm_enqueue_fn)(cdm_ctx*, int nvox, int nmeas, const double* meas,
                                     double* params, const double* CFP, const double* FixP,
                                     double* samples, double* tau, double* pred, double* BIC,
                                     double* AIC, void* stream);

cdm_status cdm_batch_create(cdm_batch** out);
cdm_status cdm_batch_destroy(cdm_batch* b);

/* Add one fit; arrays are DEVICE pointers as for cdm_fit. `work` orders
 * the branches (<= 0: nvox * nmeas). Invalidates a captured graph. */
cdm_status cdm_batch_add(cdm_batch* b, cdm_reserve_fn reserve, cdm_enqueue_fn enqueue,
                         cdm_ctx* ctx, int nvox, int nmeas, const double* meas, double* params,
                         const double* CFP, const double* FixP, double* samples, double* tau,
                         double* pred, double* BIC, double* AIC, double work);

/* Launch every item on `stream` (captured into one graph on first use). */
cdm_status cdm_batch_run(cdm_batch* b, void* stream);

/* Message of the last failure on this thread. */
const char* cdm_batch_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
