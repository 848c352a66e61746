/* cdm_volumes.h - NIfTI volumes in and out of the fitting path
 * (libcdm_utils.so, host code).
 *
 * CUDIMOT's own tools read and write the image volumes through FSL's
 * newimage library: split_parts.cc:41-53 reads the 4-D data and the mask and
 * takes the voxels inside the mask (volume4D::matrix(mask)), :104-196 splits
 * the --init_params list of 3-D volumes into ParamInit_<i> part files,
 * :198-277 the --FixP list into FixParam_<i>, and merge_parts.cc:21-59
 * joins the part files of one output and writes it back on the mask's grid
 * (volume4D::setmatrix). These entry points do the same without FSL:
 *
 *  - cdm_nifti_*: single-file NIfTI-1 images (".nii", and ".nii.gz" when the
 *    library was built with zlib; cdm_nifti_gzip() says which), any byte
 *    order on input, integer and floating-point voxel types, scl_slope /
 *    scl_inter applied on input; outputs copy the geometry (pixdim, qform,
 *    sform, units) of a template header;
 *  - cdm_mask_*: voxels with a positive mask value, in file order (x fastest,
 *    then y, then z), to and from the library's voxel-major arrays;
 *  - cdm_split_volumes / cdm_merge_volumes: split_parts and merge_parts with
 *    their checks and part-file names.
 *
 * Volumes in memory are double [nt][nz][ny][nx] (the file's order); voxel
 * arrays are double [nvox][nt], the layout of meas, params and FixP.
 */
#ifndef CDM_VOLUMES_H
#define CDM_VOLUMES_H

#include <stdint.h>

#include "cudimot_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A NIfTI-1 header as read (native byte order). */
typedef struct {
  int32_t dim[8];        /* dim[0] = number of dimensions, dim[1..7] sizes (>= 1) */
  float pixdim[8];
  int32_t datatype;      /* NIfTI DT_* code of the stored voxels */
  int32_t bitpix;
  float scl_slope, scl_inter;
  float cal_min, cal_max;
  int64_t vox_offset;
  unsigned char raw[348];/* the header in native byte order: the geometry and
                            text fields outputs inherit */
} cdm_nifti_hdr;

/* NIfTI voxel types accepted on input (DT_UINT8 ... DT_UINT64); outputs are
 * CDM_NIFTI_FLOAT32 or CDM_NIFTI_FLOAT64. */
enum {
  CDM_NIFTI_UINT8 = 2, CDM_NIFTI_INT16 = 4, CDM_NIFTI_INT32 = 8, CDM_NIFTI_FLOAT32 = 16,
  CDM_NIFTI_FLOAT64 = 64, CDM_NIFTI_INT8 = 256, CDM_NIFTI_UINT16 = 512, CDM_NIFTI_UINT32 = 768,
  CDM_NIFTI_INT64 = 1024, CDM_NIFTI_UINT64 = 1280
};

/* 1 if ".nii.gz" files can be read and written (built with zlib). */
int cdm_nifti_gzip(void);

/* Read a NIfTI-1 file: the header, and with data non-null the voxels as
 * double [nt][nz][ny][nx] (all dimensions past the third folded into nt),
 * scaled by scl_slope/scl_inter when scl_slope is neither 0 nor 1 with
 * inter 0. CDM_IO_ERROR for a missing, short, NIfTI-2, two-file or
 * unsupported-type image; CDM_BAD_ARG if capacity (doubles) is too small. */
cdm_status cdm_nifti_read(const char* path, cdm_nifti_hdr* hdr, double* data, int64_t capacity);
/* Number of voxels (nx*ny*nz) and volumes (nt) of a header. */
cdm_status cdm_nifti_shape(const cdm_nifti_hdr* hdr, int64_t* nxyz, int* nt);

/* Write nt volumes of like's spatial grid (data double [nt][nz][ny][nx]) as
 * datatype (CDM_NIFTI_FLOAT32 or CDM_NIFTI_FLOAT64). The header is like's
 * with dim[0] = 3 or 4, dim[4] = nt, scl_slope 1, scl_inter 0, cal_min /
 * cal_max = the data's range, vox_offset 352. ".gz" paths are compressed. */
cdm_status cdm_nifti_write(const char* path, const cdm_nifti_hdr* like, int nt, const double* data,
                           int datatype);

/* Voxels of mask (nxyz values) that are positive. */
cdm_status cdm_mask_count(int64_t nxyz, const double* mask, int* nvox);
/* out[v][t] = vol[t][voxel v of the mask] for t < nt: volume4D::matrix(mask)
 * transposed to the library's voxel-major layout. */
cdm_status cdm_mask_gather(int64_t nxyz, int nt, const double* vol, const double* mask, double* out);
/* vol[t][voxel v of the mask] = in[v][t]; 0 outside the mask. */
cdm_status cdm_mask_scatter(int64_t nxyz, int nt, const double* in, const double* mask, double* vol);

/* split_parts (split_parts.cc:41-277): the voxels of data_path inside
 * mask_path -> <partsdir>/part_<i>/data for i < nparts (nvox/nparts voxels
 * each, the last takes the remainder). init_list (may be null): a text file
 * of at most nparams lines, one per parameter, each the path of a 3-D
 * volume on the mask's grid or empty; empty lines take init_values[p] (or 0
 * with init_values null), and the number of lines must be nparams ->
 * ParamInit_<p>. fixp_list: nfixp non-empty lines, volume i with
 * fixp_sizes[i] volumes -> FixParam_<i>; required when nfixp > 0, refused
 * when nfixp == 0. *nvox (may be null) gets the voxels in the mask. Errors
 * as CDM_BAD_ARG / CDM_IO_ERROR with cdm_volumes_last_error(). */
cdm_status cdm_split_volumes(const char* partsdir, int nparts, const char* data_path,
                             const char* mask_path, const char* init_list, int nparams,
                             const double* init_values, const char* fixp_list, int nfixp,
                             const int* fixp_sizes, int* nvox);

/* merge_parts' join_Parts (merge_parts.cc:21-59): parts 0..nparts-1 of
 * <name> concatenated along voxels, written as a NIfTI of nrows volumes
 * (nrows = -1: taken from the first part) on mask_path's grid, double
 * voxels, zero outside the mask, cal_min/cal_max = its range. A part with
 * another row count is an error (CDM_IO_ERROR). */
cdm_status cdm_merge_volumes(const char* partsdir, int nparts, const char* name, int nrows,
                             const char* mask_path, const char* out_path);

const char* cdm_volumes_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
