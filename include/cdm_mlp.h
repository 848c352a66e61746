/* cdm_mlp.h - learned initialiser for the fitting path (libcdm_mlp.so).
 *
 * No counterpart in CUDIMOT, which initialises LM from a grid search
 * (GridSearch.cu) or from user-supplied volumes (--init_params). An MLP
 * maps a voxel's S0-normalised signal to parameter means and log standard
 * deviations; the means seed LM (replacing the grid search) and the
 * standard deviations seed the MCMC proposal widths.
 *
 * Network: n_in -> hidden -> hidden -> hidden -> n_mu + n_sig, GELU (tanh
 * form), BF16 weights and activations, FP32 accumulation on the tensor cores
 * (tcgen05.mma, TMA-fed), FP32 master weights, Adam. Loss: Gaussian
 * negative log-likelihood, mean j against log-std group[j].
 *
 * All arrays are DEVICE pointers; `x` rows are bf16 [n][n_in] (see
 * cdm_mlp_prep_input), outputs fp32 [n][16] (means, then log-stds, then
 * zero padding), targets fp32 [batch][n_mu].
 */
#ifndef CDM_MLP_H
#define CDM_MLP_H

#include "cudimot_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CDM_MLP_MAX_MU 16

typedef struct cdm_mlp cdm_mlp;

typedef struct {
  int n_in;                    /* inputs per row (multiple of 8)                 */
  int hidden;                  /* hidden width (multiple of 16, <= 256)          */
  int n_mu, n_sig;             /* means and log-std outputs (sum <= 16)          */
  int group[CDM_MLP_MAX_MU];   /* log-std index of each mean                     */
  float lr, beta1, beta2, eps; /* Adam                                           */
  float logstd_min, logstd_max;/* log-std clamp in the loss                      */
} cdm_mlp_cfg;

void cdm_mlp_default_cfg(cdm_mlp_cfg* cfg);
cdm_status cdm_mlp_create(const cdm_mlp_cfg* cfg, cdm_mlp** out);
cdm_status cdm_mlp_destroy(cdm_mlp* m);

/* Layer l in 0..3: w [rows][cols] (rows = outputs), b [rows], host or
 * device memory. set resets Adam's moments; get also returns the last
 * gradients (gw, gb may be null). */
cdm_status cdm_mlp_set_params(cdm_mlp* m, int layer, const float* w, const float* b);
cdm_status cdm_mlp_get_params(cdm_mlp* m, int layer, float* w, float* b, float* gw, float* gb);

/* One Adam step on a batch (forward, loss, backward, update). The first
 * call fixes the batch size. *loss (device, may be null) gets the mean NLL. */
cdm_status cdm_mlp_train_step(cdm_mlp* m, const void* x, const float* targets, int batch,
                              float* loss, void* stream);
/* Forward + backward without the update (gradient checks). */
cdm_status cdm_mlp_gradients(cdm_mlp* m, const void* x, const float* targets, int batch,
                             float* loss, void* stream);
/* Inference on n rows. */
cdm_status cdm_mlp_forward(cdm_mlp* m, const void* x, int n, float* out, void* stream);

/* One hidden layer (0..2) of inference alone, for tests and timing:
 * out bf16 [n][ld_out] = bf16(gelu(bf16(x W_l^T + b_l))), x bf16 [n][ld_x]
 * with the layer's input width; the kernel cdm_mlp_forward runs for it. */
cdm_status cdm_mlp_hidden_layer(cdm_mlp* m, int layer, const void* x, int ld_x, int n, void* out,
                                int ld_out, void* stream);
/* x[r][c] = meas[r][c] / s0[r * s0_ld] (s0 null: 1) as bf16 [n][ld],
 * columns nmeas..ld-1 zero. */
cdm_status cdm_mlp_prep_input(const double* meas, const double* s0, int s0_ld, int n, int nmeas,
                              int ld, void* x, void* stream);

/* out[M][ld_out] = A[M][K] * B[N][K]^T, bf16 in, fp32 out: the tensor-core
 * GEMM alone (tests). */
cdm_status cdm_mlp_gemm_bf16(const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                             float* out, int ld_out, void* stream);

/* CDM_TIMEOUT if a bounded wait inside a tensor-core kernel ran out. */
cdm_status cdm_mlp_check(cdm_mlp* m);
const char* cdm_mlp_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
