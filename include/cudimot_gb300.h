/*
 * cudimot_gb300.h - C ABI of the GB300 voxelwise fitting library.
 *
 * One shared library is built per model plugin (libcudimot_<Model>.so), in
 * the same way CUDIMOT compiles one binary per mymodels/<Model> directory;
 * every library exports the symbols below. Host code (C, C++, or any FFI)
 * binds them with plain pointers and sizes; no C++ or torch types appear.
 *
 * Data layouts are CUDIMOT's, accepted as they are (all arrays of double,
 * the MyType of every shipped plugin):
 *   meas      [nvox][nmeas]                 dMRI_Data.cu:82-88
 *   params    [nvox][NPARAMS]               Parameters.cu:72,251
 *   CFP       [nmeas][CFP_Tsize]            Parameters.cu:119
 *   FixP      [nvox][FixP_Tsize]            Parameters.cu:186
 *   samples   [nvox][NPARAMS][nsamples]     MCMC.cu:392,621
 *   tau       [nvox][nsamples]              MCMC.cu:624
 * Pointers passed to the per-stage calls are DEVICE pointers (as in
 * CUDIMOT's run() methods); cdm_fit_host takes host pointers.
 *
 * Every call returns a cdm_status; nothing calls exit(). Calls on one
 * context are not thread safe; use one context per host thread.
 */
#ifndef CUDIMOT_GB300_H
#define CUDIMOT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CDM_MAX_PARAMS 32
#define CDM_MAX_BLOCKS 16

typedef enum {
  CDM_OK = 0,
  CDM_BAD_ARG = 1,       /* invalid argument or configuration              */
  CDM_CUDA_ERROR = 2,    /* a CUDA runtime call failed                     */
  CDM_TIMEOUT = 3,       /* a bounded wait (host or device) ran out        */
  CDM_NOT_SUPPORTED = 4, /* feature not available for this model/build    */
  CDM_IO_ERROR = 5       /* a file could not be opened or parsed           */
} cdm_status;

/* bound / prior kinds, numbered as CUDIMOT's cudimot.h:16-17 */
enum { CDM_NOBOUNDS = 0, CDM_BMIN = 1, CDM_BMAX = 2, CDM_BMINMAX = 3 };
enum { CDM_NOPRIOR = 0, CDM_GAUSSPRIOR = 1, CDM_GAMMAPRIOR = 2, CDM_ARDPRIOR = 3,
       CDM_SINPRIOR = 4, CDM_CUSTOM = 5 };

/* Compile-time facts of the model plugin the library was built from
 * (modelparameters.h / modelparameters.cc of the plugin). */
typedef struct {
  char name[64];
  int nparams;                    /* NPARAMS                               */
  int ncfp;                       /* NCFP                                  */
  int nfixp;                      /* NFIXP                                 */
  int cfp_size[CDM_MAX_BLOCKS];   /* MODEL::CFP_size[]                     */
  int fixp_size[CDM_MAX_BLOCKS];  /* MODEL::FixP_size[]                    */
  int cfp_tsize;                  /* sum of cfp_size                       */
  int fixp_tsize;                 /* sum of fixp_size                      */
  int derived_cfp;                /* protocol-derived values per measurement */
  int derived_p;                  /* parameter-derived values               */
} cdm_model_info;

/* Everything CUDIMOT's method constructors read from the model priors, the
 * grid file and the command-line options (GridSearch.h:89,
 * Levenberg_Marquardt.h:81, MCMC.h:150-171, cudimotoptions.h:78-168).
 * cdm_default_cfg fills the option defaults of cudimotoptions.h. */
typedef struct {
  int nparams;                           /* must equal the model's NPARAMS */
  /* bounds and priors (Model.cu:16-299); bounds and prior arguments are
   * rounded to float before use, as CUDIMOT's __constant__ copies are. */
  int bound_types[CDM_MAX_PARAMS];
  double bounds_min[CDM_MAX_PARAMS];
  double bounds_max[CDM_MAX_PARAMS];
  int prior_types[CDM_MAX_PARAMS];
  double priors_a[CDM_MAX_PARAMS];
  double priors_b[CDM_MAX_PARAMS];
  int fixed[CDM_MAX_PARAMS];             /* --fixed                         */
  /* grid search (Model.cu:302-393); grid is a host pointer to
   * grid_combs * n_grid_params values, copied by cdm_create.              */
  int n_grid_params;
  int grid_params[CDM_MAX_PARAMS];
  int grid_combs;
  const double* grid;
  /* options */
  int run_gridsearch;    /* --gridSearch given                        */
  int run_levmar;        /* !--no_LevMar                              */
  int run_mcmc;          /* --runMCMC                                 */
  int iter_levmar;       /* --iterLevMar (200)                        */
  int marquardt;         /* !--no_Marquardt                           */
  int nburn;             /* --bi (1000)                               */
  int njumps;            /* --nj (1250)                               */
  int sampleevery;       /* --se (25)                                 */
  int update_proposal;   /* !--no_updateproposal                      */
  int rician;            /* --rician                                  */
  int get_predicted;     /* --getPredictedSignal                      */
  int bic_aic;           /* --BIC_AIC                                 */
  uint64_t seed;         /* --seed (8219)                             */
  int id_part;           /* --idPart (0)                              */
  /* GB300 launch shape: lanes cooperating on one voxel per stage
   * (0 = chosen by the built-in tuner; otherwise one of 1, 2, 4, 8, 16, 32). */
  int lanes_gridsearch;
  int lanes_levmar;
  int lanes_mcmc;
  /* Index of this call's first voxel in the whole volume (0). MCMC draws
   * are keyed by (seed, id_part, global voxel index, iteration), so a
   * volume fitted in contiguous shards - each call with first_voxel = its
   * range start, the same seed, id_part and lane counts - gives exactly the
   * fit of one call over the whole volume (split_parts.cc:80-94 ranges). */
  int64_t first_voxel;
} cdm_model_cfg;

/* Per-context counters filled by the last fit. */
typedef struct {
  int64_t gs_recheck_voxels;    /* grid-search near ties re-evaluated in FP64 */
  int64_t lm_iterations;        /* LM iterations summed over voxels           */
  int64_t lm_successes;         /* accepted LM steps summed over voxels        */
  int64_t device_errors;        /* bounded device waits that ran out           */
} cdm_stats;

typedef struct cdm_ctx cdm_ctx;

cdm_status cdm_get_model_info(cdm_model_info* info);
cdm_status cdm_default_cfg(cdm_model_cfg* cfg);
const char* cdm_status_string(cdm_status s);
/* Message of the last failure on this thread. */
const char* cdm_last_error(void);

/* modelpriors reader (Model.cu:16-299). Keeps CUDIMOT's parsing rules:
 * lines containing "//" anywhere are skipped; "prior[i]=" is recognised but
 * "priors[i]=" is not; Gaussian(a,b) takes b as the standard deviation.
 * p_init receives P_init[...] when present (*p_init_given set to 1). */
cdm_status cdm_parse_priors(const char* path, cdm_model_cfg* cfg, double* p_init,
                            int* p_init_given);
/* Grid file reader (Model.cu:302-393): search[i]=(v1,...,vn) lines.
 * Combinations are enumerated with the lowest parameter id outermost.
 * Call with grid == NULL to get *n_grid_params and *grid_combs; then with a
 * buffer of (*grid_combs) * (*n_grid_params) doubles. */
cdm_status cdm_parse_grid(const char* path, int* n_grid_params, int* grid_params,
                          int* grid_combs, double* grid, int64_t grid_capacity);
/* --fixed=i,j list (Model.cu:279-298). */
cdm_status cdm_parse_fixed(const char* list, int* fixed);
/* CFP list file (Parameters.cu:93-149): one ASCII matrix path per line,
 * rows = that block's CFP size, columns = nmeas. Writes CFP[nmeas][Tsize]. */
cdm_status cdm_read_cfp_list(const char* path, int nmeas, double* cfp);

/* Context: copies the configuration (and grid) and allocates nothing else
 * until the first call needs it. Replaces CUDIMOT's GridSearch,
 * Levenberg_Marquardt, MCMC, BIC_AIC and getPredictedSignal constructors
 * (GridSearch.cu:252-289, Levenberg_Marquardt.cu:627-663, MCMC.cu:691-768,
 * BIC_AIC.cu:203-210, getPredictedSignal.cu:96-97). */
cdm_status cdm_create(const cdm_model_cfg* cfg, cdm_ctx** ctx);
cdm_status cdm_destroy(cdm_ctx* ctx);

/* Stage calls; device pointers, asynchronous on `stream` (cudaStream_t,
 * 0 = legacy default stream). Argument meaning follows CUDIMOT's run():
 * CFP_size / FixP_size are the total sizes CFP_Tsize / FixP_Tsize.
 * nvox = 0 is valid: the call returns CDM_OK and touches no per-voxel array,
 * which may then be null (CFP must still hold nmeas rows). */
/* GridSearch<T>::run, GridSearch.cu:291-317 */
cdm_status cdm_gridsearch(cdm_ctx* ctx, int nvox, int nmeas, int CFP_size, int FixP_size,
                          const double* meas, double* params, const double* CFP,
                          const double* FixP, void* stream);
/* Levenberg_Marquardt<T>::run, Levenberg_Marquardt.cu:665-704 */
cdm_status cdm_levmar(cdm_ctx* ctx, int nvox, int nmeas, int CFP_size, int FixP_size,
                      const double* meas, double* params, const double* CFP,
                      const double* FixP, void* stream);
/* MCMC<T>::run, MCMC.cu:770-848 (burn-in and recording in one launch).
 * samples: [nvox][NPARAMS][njumps/sampleevery]; tau_samples only read or
 * written when the context was created with rician = 1 (may be NULL). */
cdm_status cdm_mcmc(cdm_ctx* ctx, int nvox, int nmeas, int CFP_size, int FixP_size,
                    const double* meas, double* params, const double* CFP, const double* FixP,
                    double* samples, double* tau_samples, void* stream);
/* BIC_AIC<T>::run, BIC_AIC.cu:212-243 */
cdm_status cdm_bic_aic(cdm_ctx* ctx, int nvox, int nmeas, int nsamples, int CFP_size,
                       int FixP_size, const double* meas, const double* samples,
                       const double* CFP, const double* FixP, double* BIC, double* AIC,
                       const double* tau_samples, void* stream);
/* getPredictedSignal<T>::run, getPredictedSignal.cu:100-117 */
cdm_status cdm_predicted_signal(cdm_ctx* ctx, int nvox, int nmeas, int nsamples,
                                int CFP_size, int FixP_size, const double* samples,
                                const double* CFP, const double* FixP, double* pred,
                                void* stream);

/* The per-part sequence of cudimot.cc:80-125 (GridSearch -> LM -> MCMC ->
 * predicted signal / BIC-AIC, as enabled in the context's cfg), on device
 * pointers, recorded once per shape into a CUDA graph and replayed.
 * samples must hold nvox*NPARAMS*nsamples values, nsamples =
 * njumps/sampleevery with MCMC and 1 without (the fitted parameters, as in
 * Parameters.cu copyParams2Samples). pred/BIC/AIC/tau may be NULL when the
 * corresponding option is off. */
cdm_status cdm_fit(cdm_ctx* ctx, int nvox, int nmeas, const double* meas, double* params,
                   const double* CFP, const double* FixP, double* samples, double* tau,
                   double* pred, double* BIC, double* AIC, void* stream);

/* As cdm_fit, with HOST arrays: copies in, fits, copies out, and waits for
 * completion (at most timeout_ms, < 0 = no limit). The signals go through
 * cdm_clean_signals first when the cfg has rician, as CUDIMOT's data loader
 * does. part_size stands for CUDIMOT's SIZE_PART and is ignored: the
 * voxels are fitted as one part when fewer than 100,000, else as 2-4
 * consecutive ranges in flight at once, each on a context and stream of its
 * own (created on first use and kept by ctx), so that the copies of one
 * range overlap the fits of the others; with first_voxel set per range and
 * the lane counts of the whole call, every result equals one cdm_fit over
 * all the voxels, and cdm_get_stats reports the call's sums. */
cdm_status cdm_fit_host(cdm_ctx* ctx, int nvox, int nmeas, const double* meas,
                        double* params, const double* CFP, const double* FixP,
                        double* samples, double* tau, double* pred, double* BIC, double* AIC,
                        int part_size, int64_t timeout_ms);

/* Self-test of the bounded device waits (no CUDIMOT counterpart; CUDIMOT's
 * kernels have no waits that can run out): launches a kernel whose mbarrier
 * wait can never complete. The wait gives up after limit_ms (1..2000) and
 * records a device error, which the next cdm_synchronize on this context
 * reports as CDM_TIMEOUT and clears; the context stays usable. Every wait in
 * the fitting kernels takes the same path with a 2 s limit. With ctx NULL
 * the error goes to the no-allocation error word of the current device
 * (reported by cdm_noalloc_status). */
cdm_status cdm_selftest_wait_timeout(cdm_ctx* ctx, int limit_ms, void* stream);

/* dMRI_Data::remove_NonPositive_entries (dMRI_Data.cu:15-30), applied by
 * CUDIMOT to every voxel when --rician is set (dMRI_Data.cu:133): in each
 * voxel of meas [nvox][nmeas] (device, in place) whose smallest value is
 * non-positive and largest positive, the non-positive entries take the
 * smallest positive value. The stage entry points and cdm_fit use meas as
 * given, like the reference's method classes. */
cdm_status cdm_clean_signals(int nvox, int nmeas, double* meas, void* stream);

/* The stage sequence of cdm_fit recorded as plain launches on `stream`
 * (no graph of its own), so that a caller can capture several contexts -
 * other models, protocols or volumes - into one CUDA graph (cdm_batch.h).
 * Same arguments and results as cdm_fit. Under stream capture it makes no
 * allocation and returns CDM_BAD_ARG unless cdm_fit_reserve was called for
 * this (nvox, nmeas) before the capture. Replaces, like cdm_fit, the
 * per-part stage sequence of cudimot.cc:80-125. */
cdm_status cdm_fit_reserve(cdm_ctx* ctx, int nvox, int nmeas);
cdm_status cdm_fit_enqueue(cdm_ctx* ctx, int nvox, int nmeas, const double* meas,
                           double* params, const double* CFP, const double* FixP,
                           double* samples, double* tau, double* pred, double* BIC,
                           double* AIC, void* stream);

/* As cdm_mcmc, with each voxel's initial proposal widths prop_sd
 * [nvox][NPARAMS] (CUDIMOT starts from P/10, MCMC.cu:474-476; a null array
 * or an entry <= 0 gives that). Used by the learned initialiser to seed
 * the proposal scales. */
cdm_status cdm_mcmc_seeded(cdm_ctx* ctx, int nvox, int nmeas, int CFP_size, int FixP_size,
                           const double* meas, double* params, const double* CFP,
                           const double* FixP, double* samples, double* tau_samples,
                           const double* prop_sd, void* stream);

/* Synthetic acquisitions from the model itself (training data of the
 * learned initialiser; no CUDIMOT counterpart): for each voxel the
 * plugin's Predicted_Signal at params [nvox][NPARAMS] / FixP (true values),
 * Rician noise with sigma = mean clean b = 0 signal / SNR, SNR uniform in
 * [snr_lo, snr_hi] per voxel, Philox-keyed by (seed, voxel, measurement).
 * b_col: the CFP column holding b (-1: none; then sigma uses the largest
 * clean signal). Outputs (each optional): meas [nvox][nmeas], s0_est [nvox]
 * = mean noisy b = 0 signal, x bf16 [nvox][x_ld] = meas / s0_est. */
cdm_status cdm_synth_signals(cdm_ctx* ctx, int nvox, int nmeas, const double* CFP,
                             const double* params, const double* FixP, double snr_lo,
                             double snr_hi, uint64_t seed, int b_col, double* meas,
                             double* s0_est, void* x, int x_ld, void* stream);

/* Per-voxel cost (sum of squared residuals, the LM/grid-search score,
 * GridSearch.cu:25-73) of params [nvox][NPARAMS] -> cost [nvox]. */
cdm_status cdm_cost(cdm_ctx* ctx, int nvox, int nmeas, const double* meas, const double* params,
                    const double* CFP, const double* FixP, double* cost, void* stream);

/* Row helpers of the learned initialiser's fallback (no CUDIMOT
 * counterpart). cdm_select_worse: idx[0 .. *count) = the voxels with
 * cost > ref * (1 + margin), in no particular order (count is a device int).
 * cdm_rows, mode 0: dst[k] = src[idx[k]]; mode 1: dst[idx[k]] = src[k];
 * mode 2: dst[idx[k]] = value; rows of ncols doubles. */
cdm_status cdm_select_worse(int n, const double* cost, const double* ref, double margin, int* idx,
                            int* count, void* stream);
cdm_status cdm_rows(int nsel, const int* idx, int ncols, const double* src, double* dst, int mode,
                    double value, void* stream);

/* The plugin's learned-initialiser head (optional hooks MLP_Encode /
 * MLP_Decode; CDM_NOT_SUPPORTED without them): number of means, of
 * log-stds, and the log-std group of each mean; network targets (float
 * [n][n_mu]) from parameters; parameters and MCMC proposal widths
 * [n][NPARAMS] from network outputs (float [n][ld], means then log-stds). */
cdm_status cdm_mlp_head_info(int* n_mu, int* n_sig, int* group);
cdm_status cdm_mlp_targets(cdm_ctx* ctx, int n, const double* params, float* targets,
                           void* stream);
cdm_status cdm_mlp_decode(cdm_ctx* ctx, int n, const float* out, int ld, double* params,
                          double* prop_sd, void* stream);

/* Wait for all work of the context on `stream`, polling at most timeout_ms
 * (< 0 = no limit); CDM_TIMEOUT if it did not finish. */
cdm_status cdm_synchronize(cdm_ctx* ctx, void* stream, int64_t timeout_ms);
cdm_status cdm_get_stats(cdm_ctx* ctx, cdm_stats* stats);

/* Levenberg-Marquardt that allocates no device memory. No counterpart in
 * CUDIMOT: it serves hosts that may not call cudaMalloc from inside this
 * library (a pipeline that reserved its device memory up front, or a
 * framework that owns all device memory through its own pool), since
 * allocation can fail under such budgets and can synchronise the device.
 * Same arguments and results as cdm_levmar, but no context: the fit
 * options come from cfg (lanes_levmar = 0 picks the lane count by
 * cdm_levmar's rule), and the working memory (protocol table, packed
 * signals, error word) is a fixed 16 MiB array in the library that every
 * GPU loading it holds until exit. Calls needing more than 16 MiB
 * (about nvox * nmeas * 4 bytes plus the protocol) return CDM_BAD_ARG;
 * split the voxels into parts. The protocol limit is cdm_levmar's (its
 * staged table must fit in shared memory). The first call on a device
 * looks up the array's device address and clears its error word (make it
 * before any stream capture). All calls share the array: calls that
 * overlap on the GPU (different streams, or different host threads) race
 * and must be serialised by the caller.
 * A bounded device wait that runs out (2 s) leaves that call's params at
 * their start values and sets the device's error word; the call itself
 * has already returned CDM_OK, so check cdm_noalloc_status. */
cdm_status cdm_levmar_noalloc(const cdm_model_cfg* cfg, int nvox, int nmeas, int CFP_size,
                              int FixP_size, const double* meas, double* params,
                              const double* CFP, const double* FixP, void* stream);

/* Error word of cdm_levmar_noalloc on the current device (no CUDIMOT
 * counterpart). Waits for `stream`, then returns CDM_TIMEOUT if a bounded
 * device wait of any no-allocation call ran out since the last check (and
 * clears the word), CDM_OK otherwise. Allocates nothing. The word is shared
 * by all callers on the device: a check races with calls still running on
 * other streams. */
cdm_status cdm_noalloc_status(void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CUDIMOT_GB300_H */
