/* cdm_hetero.h - one persistent kernel over the MCMC tiles of several fits.
 *
 * No counterpart in CUDIMOT, which fits one model on one volume per process
 * (cudimot.cc:57-125). Each fit (a context of some model library,
 * libcudimot_<Model>.so, with its arrays) is first PREPARED by its own
 * library: cdm_mcmc_prepare does everything cdm_mcmc does before the MCMC
 * launch (protocol tables, signal packing, on the given stream) and, in
 * place of the launch, returns the kernel's argument block and launch
 * shape. A multi-model library (libcdm_hetero_<set>.so, built from several
 * plugins: each model's device code compiled in a translation unit of its
 * own, device-linked into one module) then runs every prepared fit in ONE
 * launch of a persistent kernel: each CTA takes the next tile (CDM_NT
 * threads' worth of voxels of one fit) from a device counter, stages that
 * fit's protocol and runs that model's MCMC chain code on it, until no tile
 * is left. Its chains are those of cdm_mcmc on the same context (the same
 * code on the same counter-based draws); the chain code is compiled apart
 * from the model library, so a chain can part from its library twin where
 * the two compilations round an operation differently and a borderline
 * accept/reject goes the other way (under 1 % of voxels in the tests).
 */
#ifndef CDM_HETERO_H
#define CDM_HETERO_H

#include <stddef.h>
#include <stdint.h>

#include "cudimot_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CDM_TILE_ARGS_MAX 1024

/* One prepared MCMC launch (filled by cdm_mcmc_prepare). */
typedef struct cdm_tile_work {
  char model[64];          /* model name of the library that prepared it */
  int eval_double;         /* the plugin is evaluated in double (an --eval double build) */
  int threads;             /* threads per CTA the library was built with (CDM_NT) */
  int lanes;               /* lanes per voxel */
  int rician;              /* Rician likelihood (tau sampled) */
  int ntiles;              /* CTAs the launch would have had */
  uint32_t smem_bytes;     /* dynamic shared memory of the launch */
  uint32_t scratch_bytes;  /* shared memory the kernel otherwise keeps statically */
  uint32_t args_bytes;     /* bytes of args used */
  void* err;               /* the context's device error word */
  unsigned char args[CDM_TILE_ARGS_MAX]; /* the kernel's argument block */
} cdm_tile_work;

/* Model library (libcudimot_<Model>.so): cdm_mcmc with the launch left to
 * the caller. Same arguments, checks and stream work as cdm_mcmc; the
 * context's scratch holds the packed signals and tables until the MCMC
 * that uses them has run, so the context must not fit anything else in
 * between. nvox = 0 gives ntiles = 0. */
cdm_status cdm_mcmc_prepare(cdm_ctx* ctx, int nvox, int nmeas, int CFP_size, int FixP_size,
                            const double* meas, double* params, const double* CFP,
                            const double* FixP, double* samples, double* tau_samples,
                            void* stream, cdm_tile_work* out);

/* Multi-model library (libcdm_hetero_<set>.so). */
typedef struct cdm_hetero cdm_hetero;

/* Load the persistent kernel on the current device and allocate its
 * descriptor buffers (the only allocations: a failed run allocates
 * nothing more). */
cdm_status cdm_hetero_create(cdm_hetero** out);
cdm_status cdm_hetero_destroy(cdm_hetero* h);

/* Comma-separated "model/eval/lanes" entries this library can run, e.g.
 * "NODDI_Watson/f32/1:2:4". Returns the length written (without the NUL),
 * or the length needed when cap is too small. */
size_t cdm_hetero_models(char* buf, size_t cap);

/* Run the MCMC of n prepared fits in one persistent launch on `stream`
 * (the stream the fits were prepared on, or one ordered after it). Every
 * item's model, evaluation type, lane count and CTA size must be one this
 * library was built with (CDM_BAD_ARG otherwise, before any launch). The
 * fits' argument blocks travel as the kernel's parameters, one slot per
 * (model, lanes, likelihood): fits that share all three run in successive
 * launches of the same kernel. A bounded wait that runs out inside a tile
 * sets that context's error word (read by cdm_synchronize / cdm_get_stats
 * of its library) and stops the CTA. Calls on one cdm_hetero must be
 * ordered on the GPU (one stream, or streams ordered by the caller): they
 * share its descriptor buffers. Not capturable into a CUDA graph (the
 * descriptors are uploaded from host memory on each call). */
cdm_status cdm_hetero_mcmc(cdm_hetero* h, int n, const cdm_tile_work* items, void* stream);

/* CTAs of the largest launch of the last cdm_hetero_mcmc call (SMs x
 * resident CTAs, or fewer when there are fewer tiles), and the number of
 * launches it made (1 unless two fits shared model, lanes and likelihood). */
int cdm_hetero_last_grid(const cdm_hetero* h);
int cdm_hetero_last_launches(const cdm_hetero* h);

/* Message of the last failure on this thread. */
const char* cdm_hetero_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
