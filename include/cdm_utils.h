/* cdm_utils.h - the steps either side of the fitting path (libcdm_utils.so).
 *
 *  - cdm_dti_fit: log-linear diffusion-tensor fit on the GPU, the
 *    initialiser every CUDIMOT pipeline runs first (FSL dtifit +
 *    utils/cart2spherical.cc + utils/initialise_Psi.cc, e.g.
 *    Pipeline_NODDI_Watson.sh:195-196, Pipeline_Ball_2_Sticks.sh:150-158);
 *  - cdm_sample_stats, cdm_dyads, cdm_od_from_kappa: the *_finish.sh
 *    post-processing (fslmaths -Tmean, make_dyadic_vectors,
 *    OD = 2/pi atan(1/kappa), NODDI_Watson_finish.sh:22-35) on the GPU;
 *  - cdm_part_*: CUDIMOT's binary part files (split_parts.cc:19-34,
 *    Parameters.cu:44-70 and 405-420, dMRI_Data.cu:37-62): a header
 *    int32 nvox, int32 nrows, int64 nbytes, then nrows x nvox doubles,
 *    row-major (row = measurement, sample or value; column = voxel).
 *
 * GPU arrays are DEVICE pointers; the part-file calls take host arrays
 * in the library's voxel-major layout ([nvox][ncols]) and transpose.
 */
#ifndef CDM_UTILS_H
#define CDM_UTILS_H

#include <stdint.h>

#include "cudimot_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Output columns of cdm_dti_fit, per voxel. */
enum {
  CDM_DTI_S0 = 0, CDM_DTI_L1, CDM_DTI_L2, CDM_DTI_L3,
  CDM_DTI_V1X, CDM_DTI_V1Y, CDM_DTI_V1Z, CDM_DTI_V2X, CDM_DTI_V2Y, CDM_DTI_V2Z,
  CDM_DTI_FA, CDM_DTI_MD, CDM_DTI_TH1, CDM_DTI_PH1, CDM_DTI_TH2, CDM_DTI_PH2, CDM_DTI_PSI,
  CDM_DTI_NOUT
};

/* Ordinary least squares on log(max(S, 1e-3)) with the design
 * (1, -b gx^2, -b gy^2, -b gz^2, -2b gx gy, -2b gx gz, -2b gy gz); eigen-
 * decomposition of the tensor (descending eigenvalues); theta/phi of V1
 * and V2 (cart2spherical); psi = angle of V2 in the plane orthogonal to
 * V1 from the fanning direction at psi = 0 (NODDI-Bingham's
 * parameterisation, as initialise_Psi.cc). meas [nvox][nmeas] and
 * out [nvox][CDM_DTI_NOUT] on the device; bvecs [nmeas][3] and bvals
 * [nmeas] in host or device memory (at most 512 measurements). */
cdm_status cdm_dti_fit(int nvox, int nmeas, const double* meas, const double* bvecs,
                       const double* bvals, double* out, void* stream);

/* Mean and standard deviation (n-1) over the samples of each parameter:
 * samples [nvox][nparams][nsamples] -> mean, sd [nvox][nparams] (sd may
 * be null). */
cdm_status cdm_sample_stats(int nvox, int nparams, int nsamples, const double* samples,
                            double* mean, double* sd, void* stream);

/* make_dyadic_vectors: principal eigenvector of the mean dyadic tensor of
 * the orientation samples (theta = parameter ith, phi = iph) and its
 * dispersion 1 - largest eigenvalue -> dyads [nvox][4] (x, y, z, disp). */
cdm_status cdm_dyads(int nvox, int nparams, int nsamples, const double* samples, int ith,
                     int iph, double* dyads, void* stream);

/* OD = 2/pi atan(1/kappa) for kappa = src[v * stride] -> od [nvox]. */
cdm_status cdm_od_from_kappa(int nvox, const double* src, int stride, double* od, void* stream);

/* out[v * out_ld] = mean of meas[v][idx[k]], k < nidx (idx on the device):
 * the S0 of the pipelines (mean of the b <= 50 volumes,
 * Pipeline_NODDI_Watson.sh:155-170). */
cdm_status cdm_mean_columns(int nvox, int nmeas, const double* meas, const int* idx, int nidx,
                            double* out, int out_ld, void* stream);
/* dst[v][dst_col + c] = scale * src[v][src_col + c] for c < ncols, or
 * = scale when src is null: parameter columns between pipeline steps. */
cdm_status cdm_copy_columns(int nvox, const double* src, int src_ld, int src_col, double* dst,
                            int dst_ld, int dst_col, int ncols, double scale, void* stream);

/* "<partsdir>/part_<id_part>/<name>" into buf (CDM_BAD_ARG if too long). */
cdm_status cdm_part_path(const char* partsdir, int id_part, const char* name, char* buf,
                         int buflen);
/* Write data [nvox][ncols] as a part file ([ncols][nvox] on disk). */
cdm_status cdm_part_write(const char* path, int nvox, int ncols, const double* data);
/* Read a part file into data [nvox][ncols]; with data null only the sizes
 * are returned. CDM_IO_ERROR for a missing, short or inconsistent file,
 * CDM_BAD_ARG if capacity (doubles) is too small. */
cdm_status cdm_part_read(const char* path, int* nvox, int* ncols, double* data, int64_t capacity);
/* split_parts: voxels 0..nvox-1 into nparts parts of nvox/nparts voxels
 * (the last takes the remainder), written as <name> into
 * <partsdir>/part_<i>/ (directories created). */
cdm_status cdm_split_parts(const char* partsdir, int nparts, const char* name, int nvox, int ncols,
                           const double* data);
/* merge_parts: parts 0..nparts-1 of <name> concatenated along voxels. */
cdm_status cdm_merge_parts(const char* partsdir, int nparts, const char* name, int* nvox,
                           int* ncols, double* data, int64_t capacity);

const char* cdm_utils_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
