// cdm_utils.cu - DTI initialiser, post-processing and part files
// (include/cdm_utils.h).
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cdm_utils.h"

namespace {

thread_local std::string g_err;

cdm_status fail(cdm_status s, const std::string& m) {
  g_err = m;
  return s;
}

#define U_CUDA(x)                                                                           \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess) return fail(CDM_CUDA_ERROR, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kDtiMaxMeas = 512;

// The pseudo-inverse of the design matrix travels as a kernel argument
// (7 x 512 doubles fit the 32 KB parameter space), so the fit needs no
// device allocation.
struct dti_args {
  int nvox, nmeas;
  const double* meas;
  double* out;
  double pinv[7 * kDtiMaxMeas];  // [7][nmeas]
};

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (double):
// eigenvalues w, eigenvectors as columns of V.
__host__ __device__ inline void sym3_eig(double A[3][3], double w[3], double V[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 16; sweep++) {
    const double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    const double scale = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
    if (off <= 1e-17 * scale || off == 0.0) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {  // A = J^T A J
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; k++) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; i++) w[i] = A[i][i];
}

// Indices of w in descending order.
__host__ __device__ inline void order3(const double w[3], int o[3]) {
  o[0] = 0; o[1] = 1; o[2] = 2;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2 - i; j++)
      if (w[o[j]] < w[o[j + 1]]) {
        const int t = o[j]; o[j] = o[j + 1]; o[j + 1] = t;
      }
}

// One warp per voxel: log-signal projections on the pseudo-inverse rows,
// warp sums, then lane 0 decomposes the tensor.
__global__ void dti_kernel(const __grid_constant__ dti_args a) {
  const int v = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (v >= a.nvox) return;
  double c[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int m = lane; m < a.nmeas; m += 32) {
    const double y = log(fmax(a.meas[(size_t)v * a.nmeas + m], 1e-3));
#pragma unroll
    for (int j = 0; j < 7; j++) c[j] += a.pinv[j * a.nmeas + m] * y;
  }
#pragma unroll
  for (int j = 0; j < 7; j++)
    for (int o = 16; o > 0; o >>= 1) c[j] += __shfl_xor_sync(0xFFFFFFFFu, c[j], o);
  if (lane != 0) return;
  // c = (log S0, Dxx, Dyy, Dzz, Dxy, Dxz, Dyz)
  double D[3][3] = {{c[1], c[4], c[5]}, {c[4], c[2], c[6]}, {c[5], c[6], c[3]}};
  double w[3], V[3][3];
  sym3_eig(D, w, V);
  int o[3];
  order3(w, o);
  double* out = a.out + (size_t)v * CDM_DTI_NOUT;
  out[CDM_DTI_S0] = exp(c[0]);
  const double l1 = w[o[0]], l2 = w[o[1]], l3 = w[o[2]];
  out[CDM_DTI_L1] = l1;
  out[CDM_DTI_L2] = l2;
  out[CDM_DTI_L3] = l3;
  double v1[3], v2[3];
  for (int k = 0; k < 3; k++) {
    v1[k] = V[k][o[0]];
    v2[k] = V[k][o[1]];
  }
  for (int k = 0; k < 3; k++) {
    out[CDM_DTI_V1X + k] = v1[k];
    out[CDM_DTI_V2X + k] = v2[k];
  }
  const double md = (l1 + l2 + l3) / 3.0;
  const double num = (l1 - md) * (l1 - md) + (l2 - md) * (l2 - md) + (l3 - md) * (l3 - md);
  const double den = l1 * l1 + l2 * l2 + l3 * l3;
  out[CDM_DTI_FA] = den > 0.0 ? sqrt(1.5 * num / den) : 0.0;
  out[CDM_DTI_MD] = md;
  const double th1 = acos(fmin(fmax(v1[2], -1.0), 1.0)), ph1 = atan2(v1[1], v1[0]);
  out[CDM_DTI_TH1] = th1;
  out[CDM_DTI_PH1] = ph1;
  out[CDM_DTI_TH2] = acos(fmin(fmax(v2[2], -1.0), 1.0));
  out[CDM_DTI_PH2] = atan2(v2[1], v2[0]);
  // psi: V2 in the plane orthogonal to V1, from the psi = 0 fanning direction
  const double f0[3] = {-sin(ph1), cos(ph1), 0.0};
  const double h0[3] = {cos(th1) * cos(ph1), cos(th1) * sin(ph1), -sin(th1)};
  out[CDM_DTI_PSI] = atan2(-(v2[0] * h0[0] + v2[1] * h0[1] + v2[2] * h0[2]),
                           v2[0] * f0[0] + v2[1] * f0[1] + v2[2] * f0[2]);
}

__global__ void stats_kernel(int nvox, int np, int ns, const double* __restrict__ s,
                             double* __restrict__ mean, double* __restrict__ sd) {
  const size_t n = (size_t)nvox * np;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double* x = s + i * ns;
    double acc = 0.0;
    for (int k = 0; k < ns; k++) acc += x[k];
    const double m = acc / ns;
    mean[i] = m;
    if (sd) {
      double q = 0.0;
      for (int k = 0; k < ns; k++) q += (x[k] - m) * (x[k] - m);
      sd[i] = ns > 1 ? sqrt(q / (ns - 1)) : 0.0;
    }
  }
}

__global__ void dyads_kernel(int nvox, int np, int ns, const double* __restrict__ s, int ith,
                             int iph, double* __restrict__ dy) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += gridDim.x * blockDim.x) {
    const double* th = s + ((size_t)v * np + ith) * ns;
    const double* ph = s + ((size_t)v * np + iph) * ns;
    double T[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int k = 0; k < ns; k++) {
      const double x[3] = {sin(th[k]) * cos(ph[k]), sin(th[k]) * sin(ph[k]), cos(th[k])};
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) T[i][j] += x[i] * x[j] / ns;
    }
    double w[3], V[3][3];
    sym3_eig(T, w, V);
    int o[3];
    order3(w, o);
    double* out = dy + (size_t)v * 4;
    for (int k = 0; k < 3; k++) out[k] = V[k][o[0]];
    out[3] = 1.0 - w[o[0]];
  }
}

__global__ void od_kernel(int n, const double* __restrict__ k, int stride, double* __restrict__ od) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    od[v] = 0.63661977236758134 * atan(1.0 / k[(size_t)v * stride]);
}

__global__ void mean_cols_kernel(int nvox, int nmeas, const double* __restrict__ meas,
                                 const int* __restrict__ idx, int nidx, double* __restrict__ out,
                                 int out_ld) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < nidx; k++) acc += meas[(size_t)v * nmeas + idx[k]];
    out[(size_t)v * out_ld] = acc / nidx;
  }
}

__global__ void copy_cols_kernel(int nvox, const double* __restrict__ src, int src_ld, int src_col,
                                 double* __restrict__ dst, int dst_ld, int dst_col, int ncols,
                                 double scale, int fill, double value) {
  const size_t n = (size_t)nvox * ncols;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t v = i / ncols, c = i % ncols;
    dst[v * dst_ld + dst_col + c] = fill ? value : scale * src[v * src_ld + src_col + c];
  }
}

int grid_for(size_t n, int t = 256) { return (int)std::min<size_t>((n + t - 1) / t, 152 * 8); }

// 7x7 Gauss-Jordan inverse with partial pivoting (host, double).
bool inv7(double A[7][7], double B[7][7]) {
  for (int i = 0; i < 7; i++)
    for (int j = 0; j < 7; j++) B[i][j] = i == j ? 1.0 : 0.0;
  for (int c = 0; c < 7; c++) {
    int p = c;
    for (int r = c + 1; r < 7; r++)
      if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
    if (fabs(A[p][c]) < 1e-300) return false;
    for (int j = 0; j < 7; j++) {
      std::swap(A[c][j], A[p][j]);
      std::swap(B[c][j], B[p][j]);
    }
    const double d = 1.0 / A[c][c];
    for (int j = 0; j < 7; j++) {
      A[c][j] *= d;
      B[c][j] *= d;
    }
    for (int r = 0; r < 7; r++)
      if (r != c && A[r][c] != 0.0) {
        const double f = A[r][c];
        for (int j = 0; j < 7; j++) {
          A[r][j] -= f * A[c][j];
          B[r][j] -= f * B[c][j];
        }
      }
  }
  return true;
}

}  // namespace

extern "C" {

const char* cdm_utils_last_error(void) { return g_err.c_str(); }

cdm_status cdm_dti_fit(int nvox, int nmeas, const double* meas, const double* bvecs,
                       const double* bvals, double* out, void* stream) {
  if (nvox < 0 || nmeas < 7 || !meas || !bvecs || !bvals || !out)
    return fail(CDM_BAD_ARG, "bad argument (the tensor fit needs at least 7 measurements)");
  if (nmeas > kDtiMaxMeas)
    return fail(CDM_BAD_ARG, "cdm_dti_fit supports at most 512 measurements");
  // the gradient table may be in host or device memory; the design matrix
  // is formed on the host
  std::vector<double> hg((size_t)nmeas * 3), hb((size_t)nmeas);
  for (int k = 0; k < 2; k++) {
    const void* src = k == 0 ? (const void*)bvecs : (const void*)bvals;
    void* dst = k == 0 ? (void*)hg.data() : (void*)hb.data();
    const size_t bytes = (k == 0 ? 3 : 1) * (size_t)nmeas * sizeof(double);
    cudaPointerAttributes attr;
    const cudaError_t e = cudaPointerGetAttributes(&attr, src);
    if (e == cudaSuccess && attr.type == cudaMemoryTypeDevice) {
      U_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    } else {
      cudaGetLastError();  // an unregistered host pointer is not an error here
      std::memcpy(dst, src, bytes);
    }
  }
  dti_args* a = new dti_args();
  a->nvox = nvox;
  a->nmeas = nmeas;
  a->meas = meas;
  a->out = out;
  std::vector<double> X((size_t)nmeas * 7);
  for (int m = 0; m < nmeas; m++) {
    const double gx = hg[3 * m], gy = hg[3 * m + 1], gz = hg[3 * m + 2], b = hb[m];
    const double r[7] = {1.0, -b * gx * gx, -b * gy * gy, -b * gz * gz, -2 * b * gx * gy,
                         -2 * b * gx * gz, -2 * b * gy * gz};
    for (int j = 0; j < 7; j++) X[(size_t)m * 7 + j] = r[j];
  }
  double XtX[7][7], Inv[7][7];
  for (int i = 0; i < 7; i++)
    for (int j = 0; j < 7; j++) {
      double s = 0.0;
      for (int m = 0; m < nmeas; m++) s += X[(size_t)m * 7 + i] * X[(size_t)m * 7 + j];
      XtX[i][j] = s;
    }
  if (!inv7(XtX, Inv)) {
    delete a;
    return fail(CDM_BAD_ARG, "the gradient table does not determine a tensor (singular design)");
  }
  for (int j = 0; j < 7; j++)
    for (int m = 0; m < nmeas; m++) {
      double s = 0.0;
      for (int k = 0; k < 7; k++) s += Inv[j][k] * X[(size_t)m * 7 + k];
      a->pinv[j * nmeas + m] = s;
    }
  cdm_status st = CDM_OK;
  if (nvox > 0) {
    dti_kernel<<<(nvox + 3) / 4, 128, 0, (cudaStream_t)stream>>>(*a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = fail(CDM_CUDA_ERROR, std::string("dti_kernel: ") + cudaGetErrorString(e));
  }
  delete a;
  return st;
}

cdm_status cdm_sample_stats(int nvox, int nparams, int nsamples, const double* samples,
                            double* mean, double* sd, void* stream) {
  if (nvox < 0 || nparams <= 0 || nsamples <= 0 || !samples || !mean) return fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  stats_kernel<<<grid_for((size_t)nvox * nparams), 256, 0, (cudaStream_t)stream>>>(
      nvox, nparams, nsamples, samples, mean, sd);
  U_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_dyads(int nvox, int nparams, int nsamples, const double* samples, int ith, int iph,
                     double* dyads, void* stream) {
  if (nvox < 0 || nsamples <= 0 || !samples || !dyads || ith < 0 || iph < 0 || ith >= nparams ||
      iph >= nparams)
    return fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  dyads_kernel<<<grid_for(nvox), 256, 0, (cudaStream_t)stream>>>(nvox, nparams, nsamples, samples,
                                                                 ith, iph, dyads);
  U_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_od_from_kappa(int nvox, const double* src, int stride, double* od, void* stream) {
  if (nvox < 0 || !src || !od || stride <= 0) return fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  od_kernel<<<grid_for(nvox), 256, 0, (cudaStream_t)stream>>>(nvox, src, stride, od);
  U_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_mean_columns(int nvox, int nmeas, const double* meas, const int* idx, int nidx,
                            double* out, int out_ld, void* stream) {
  if (nvox < 0 || nmeas <= 0 || !meas || !idx || nidx <= 0 || !out || out_ld <= 0)
    return fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  mean_cols_kernel<<<grid_for(nvox), 256, 0, (cudaStream_t)stream>>>(nvox, nmeas, meas, idx, nidx,
                                                                     out, out_ld);
  U_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_copy_columns(int nvox, const double* src, int src_ld, int src_col, double* dst,
                            int dst_ld, int dst_col, int ncols, double scale, void* stream) {
  if (nvox < 0 || !dst || ncols <= 0 || dst_ld < dst_col + ncols || dst_col < 0 ||
      (src && (src_ld < src_col + ncols || src_col < 0)))
    return fail(CDM_BAD_ARG, "bad argument");
  if (nvox == 0) return CDM_OK;
  copy_cols_kernel<<<grid_for((size_t)nvox * ncols), 256, 0, (cudaStream_t)stream>>>(
      nvox, src, src_ld, src_col, dst, dst_ld, dst_col, ncols, src ? scale : 0.0, src ? 0 : 1,
      scale);
  U_CUDA(cudaGetLastError());
  return CDM_OK;
}

cdm_status cdm_part_path(const char* partsdir, int id_part, const char* name, char* buf, int buflen) {
  if (!partsdir || !name || !buf || buflen <= 0 || id_part < 0) return fail(CDM_BAD_ARG, "bad argument");
  const std::string p = std::string(partsdir) + "/part_" + std::to_string(id_part) + "/" + name;
  if ((int)p.size() + 1 > buflen) return fail(CDM_BAD_ARG, "path buffer too small");
  std::memcpy(buf, p.c_str(), p.size() + 1);
  return CDM_OK;
}

cdm_status cdm_part_write(const char* path, int nvox, int ncols, const double* data) {
  if (!path || nvox < 0 || ncols <= 0 || (nvox > 0 && !data)) return fail(CDM_BAD_ARG, "bad argument");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(CDM_IO_ERROR, std::string("cannot create ") + path + ": " + std::strerror(errno));
  const int32_t hdr[2] = {nvox, ncols};
  const int64_t nbytes = (int64_t)nvox * ncols * (int64_t)sizeof(double);
  bool ok = std::fwrite(hdr, sizeof(int32_t), 2, f) == 2 && std::fwrite(&nbytes, 8, 1, f) == 1;
  std::vector<double> row((size_t)nvox);
  for (int c = 0; c < ncols && ok; c++) {
    for (int v = 0; v < nvox; v++) row[v] = data[(size_t)v * ncols + c];
    ok = std::fwrite(row.data(), sizeof(double), (size_t)nvox, f) == (size_t)nvox;
  }
  if (std::fclose(f) != 0) ok = false;
  return ok ? CDM_OK : fail(CDM_IO_ERROR, std::string("write failed: ") + path);
}

cdm_status cdm_part_read(const char* path, int* nvox, int* ncols, double* data, int64_t capacity) {
  if (!path || !nvox || !ncols) return fail(CDM_BAD_ARG, "bad argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(CDM_IO_ERROR, std::string("cannot open ") + path + ": " + std::strerror(errno));
  int32_t hdr[2];
  int64_t nbytes = 0;
  if (std::fread(hdr, sizeof(int32_t), 2, f) != 2 || std::fread(&nbytes, 8, 1, f) != 1) {
    std::fclose(f);
    return fail(CDM_IO_ERROR, std::string("short header: ") + path);
  }
  if (hdr[0] < 0 || hdr[1] <= 0 || nbytes != (int64_t)hdr[0] * hdr[1] * (int64_t)sizeof(double)) {
    std::fclose(f);
    return fail(CDM_IO_ERROR, std::string("inconsistent header: ") + path);
  }
  *nvox = hdr[0];
  *ncols = hdr[1];
  if (!data) {
    std::fclose(f);
    return CDM_OK;
  }
  if (capacity < (int64_t)hdr[0] * hdr[1]) {
    std::fclose(f);
    return fail(CDM_BAD_ARG, "output capacity too small");
  }
  std::vector<double> row((size_t)hdr[0]);
  for (int c = 0; c < hdr[1]; c++) {
    if (std::fread(row.data(), sizeof(double), (size_t)hdr[0], f) != (size_t)hdr[0]) {
      std::fclose(f);
      return fail(CDM_IO_ERROR, std::string("short data: ") + path);
    }
    for (int v = 0; v < hdr[0]; v++) data[(size_t)v * hdr[1] + c] = row[v];
  }
  std::fclose(f);
  return CDM_OK;
}

cdm_status cdm_split_parts(const char* partsdir, int nparts, const char* name, int nvox, int ncols,
                           const double* data) {
  if (!partsdir || !name || nparts <= 0 || nvox <= 0 || ncols <= 0 || !data)
    return fail(CDM_BAD_ARG, "bad argument");
  if (nvox < nparts) return fail(CDM_BAD_ARG, "more parts than voxels");
  ::mkdir(partsdir, 0755);
  const int size = nvox / nparts;
  char path[4096];
  for (int i = 0; i < nparts; i++) {
    const std::string dir = std::string(partsdir) + "/part_" + std::to_string(i);
    if (::mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST)
      return fail(CDM_IO_ERROR, "cannot create " + dir + ": " + std::strerror(errno));
    const int v0 = i * size, n = i == nparts - 1 ? nvox - v0 : size;
    cdm_status s = cdm_part_path(partsdir, i, name, path, sizeof(path));
    if (s != CDM_OK) return s;
    s = cdm_part_write(path, n, ncols, data + (size_t)v0 * ncols);
    if (s != CDM_OK) return s;
  }
  return CDM_OK;
}

cdm_status cdm_merge_parts(const char* partsdir, int nparts, const char* name, int* nvox, int* ncols,
                           double* data, int64_t capacity) {
  if (!partsdir || !name || nparts <= 0 || !nvox || !ncols) return fail(CDM_BAD_ARG, "bad argument");
  char path[4096];
  int total = 0, nc = -1;
  for (int i = 0; i < nparts; i++) {
    int n, c;
    cdm_status s = cdm_part_path(partsdir, i, name, path, sizeof(path));
    if (s == CDM_OK) s = cdm_part_read(path, &n, &c, nullptr, 0);
    if (s != CDM_OK) return s;
    if (nc >= 0 && c != nc) return fail(CDM_IO_ERROR, "parts disagree on the number of rows");
    nc = c;
    if (data) {
      if (capacity < (int64_t)(total + n) * c) return fail(CDM_BAD_ARG, "output capacity too small");
      s = cdm_part_read(path, &n, &c, data + (size_t)total * c, capacity - (int64_t)total * c);
      if (s != CDM_OK) return s;
    }
    total += n;
  }
  *nvox = total;
  *ncols = nc;
  return CDM_OK;
}

}  // extern "C"
