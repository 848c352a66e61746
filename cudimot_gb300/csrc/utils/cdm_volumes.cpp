// cdm_volumes.cpp - NIfTI-1 volumes, masks, split_parts / merge_parts on
// volumes (include/cdm_volumes.h). Host code of libcdm_utils.so.
#include "cdm_volumes.h"

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <string>
#include <vector>

#include "cdm_utils.h"

#ifdef CDM_HAVE_ZLIB
#include <zlib.h>
#endif

namespace {

thread_local std::string g_err;

cdm_status fail(cdm_status s, const std::string& m) {
  g_err = m;
  return s;
}

// Byte offsets of the NIfTI-1 header fields this file reads or writes.
enum : int {
  kSizeofHdr = 0, kDim = 40, kDatatype = 70, kBitpix = 72, kPixdim = 76, kVoxOffset = 108,
  kSclSlope = 112, kSclInter = 116, kCalMax = 124, kCalMin = 128, kMagic = 344, kHdrBytes = 348
};

// Every numeric field of the header as (offset, element bytes, count): what
// a byte-order swap touches.
struct field {
  int off, size, count;
};
constexpr field kNumeric[] = {
    {0, 4, 1},   {32, 4, 1},  {36, 2, 1},  {40, 2, 8},   {56, 4, 3},   {68, 2, 1},  {70, 2, 1},
    {72, 2, 1},  {74, 2, 1},  {76, 4, 8},  {108, 4, 1},  {112, 4, 1},  {116, 4, 1}, {120, 2, 1},
    {124, 4, 1}, {128, 4, 1}, {132, 4, 1}, {136, 4, 1},  {140, 4, 1},  {144, 4, 1}, {252, 2, 1},
    {254, 2, 1}, {256, 4, 6}, {280, 4, 12}};

void swap_bytes(unsigned char* p, int size) {
  for (int i = 0; i < size / 2; i++) {
    const unsigned char t = p[i];
    p[i] = p[size - 1 - i];
    p[size - 1 - i] = t;
  }
}

template <typename T>
T get(const unsigned char* raw, int off) {
  T v;
  std::memcpy(&v, raw + off, sizeof(T));
  return v;
}

template <typename T>
void put(unsigned char* raw, int off, T v) {
  std::memcpy(raw + off, &v, sizeof(T));
}

int type_bytes(int dt) {
  switch (dt) {
    case CDM_NIFTI_UINT8: case CDM_NIFTI_INT8: return 1;
    case CDM_NIFTI_INT16: case CDM_NIFTI_UINT16: return 2;
    case CDM_NIFTI_INT32: case CDM_NIFTI_UINT32: case CDM_NIFTI_FLOAT32: return 4;
    case CDM_NIFTI_FLOAT64: case CDM_NIFTI_INT64: case CDM_NIFTI_UINT64: return 8;
    default: return 0;
  }
}

double to_double(const unsigned char* p, int dt) {
  switch (dt) {
    case CDM_NIFTI_UINT8: return (double)get<uint8_t>(p, 0);
    case CDM_NIFTI_INT8: return (double)get<int8_t>(p, 0);
    case CDM_NIFTI_INT16: return (double)get<int16_t>(p, 0);
    case CDM_NIFTI_UINT16: return (double)get<uint16_t>(p, 0);
    case CDM_NIFTI_INT32: return (double)get<int32_t>(p, 0);
    case CDM_NIFTI_UINT32: return (double)get<uint32_t>(p, 0);
    case CDM_NIFTI_FLOAT32: return (double)get<float>(p, 0);
    case CDM_NIFTI_FLOAT64: return get<double>(p, 0);
    case CDM_NIFTI_INT64: return (double)get<int64_t>(p, 0);
    case CDM_NIFTI_UINT64: return (double)get<uint64_t>(p, 0);
    default: return 0.0;
  }
}

bool ends_with(const std::string& s, const char* suffix) {
  const size_t n = std::strlen(suffix);
  return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

// A file read sequentially, plain or gzip-compressed (zlib's reader passes
// plain files through unchanged).
class in_file {
 public:
  explicit in_file(const char* path) {
#ifdef CDM_HAVE_ZLIB
    gz_ = gzopen(path, "rb");
    ok_ = gz_ != nullptr;
#else
    f_ = std::fopen(path, "rb");
    ok_ = f_ != nullptr;
    if (ok_) {
      unsigned char m[2] = {0, 0};
      const size_t n = std::fread(m, 1, 2, f_);
      gzipped_ = n == 2 && m[0] == 0x1f && m[1] == 0x8b;
      std::rewind(f_);
    }
#endif
    if (!ok_) err_ = std::strerror(errno);
  }
  ~in_file() {
#ifdef CDM_HAVE_ZLIB
    if (gz_) gzclose(gz_);
#else
    if (f_) std::fclose(f_);
#endif
  }
  bool ok() const { return ok_; }
  bool gzipped() const { return gzipped_; }
  const std::string& err() const { return err_; }
  bool read(void* p, size_t n) {
#ifdef CDM_HAVE_ZLIB
    unsigned char* q = (unsigned char*)p;
    while (n > 0) {  // gzread takes an unsigned count
      const unsigned chunk = n > (1u << 30) ? (1u << 30) : (unsigned)n;
      const int got = gzread(gz_, q, chunk);
      if (got != (int)chunk) return false;
      q += chunk;
      n -= chunk;
    }
    return true;
#else
    return std::fread(p, 1, n, f_) == n;
#endif
  }
  bool skip(int64_t n) {
    std::vector<unsigned char> tmp(4096);
    while (n > 0) {
      const size_t k = n > 4096 ? 4096 : (size_t)n;
      if (!read(tmp.data(), k)) return false;
      n -= (int64_t)k;
    }
    return true;
  }

 private:
  std::string err_;
  bool ok_ = false, gzipped_ = false;
#ifdef CDM_HAVE_ZLIB
  gzFile gz_ = nullptr;
#else
  FILE* f_ = nullptr;
#endif
};

cdm_status parse_header(const unsigned char* file_hdr, const std::string& path, cdm_nifti_hdr* h,
                        bool* swapped) {
  unsigned char raw[kHdrBytes];
  std::memcpy(raw, file_hdr, kHdrBytes);
  int32_t sz = get<int32_t>(raw, kSizeofHdr);
  bool swap = false;
  if (sz != kHdrBytes) {
    unsigned char t[4];
    std::memcpy(t, raw, 4);
    swap_bytes(t, 4);
    int32_t s2;
    std::memcpy(&s2, t, 4);
    if (sz == 540 || s2 == 540) return fail(CDM_IO_ERROR, "NIfTI-2 images are not supported: " + path);
    if (s2 != kHdrBytes) return fail(CDM_IO_ERROR, "not a NIfTI-1 image: " + path);
    swap = true;
  }
  if (swap)
    for (const field& f : kNumeric)
      for (int i = 0; i < f.count; i++) swap_bytes(raw + f.off + i * f.size, f.size);
  if (std::memcmp(raw + kMagic, "ni1", 4) == 0)
    return fail(CDM_IO_ERROR, "two-file (.hdr/.img) NIfTI images are not supported: " + path);
  if (std::memcmp(raw + kMagic, "n+1", 4) != 0)
    return fail(CDM_IO_ERROR, "not a single-file NIfTI-1 image (magic n+1): " + path);
  std::memset(h, 0, sizeof(*h));
  const int nd = get<int16_t>(raw, kDim);
  if (nd < 1 || nd > 7) return fail(CDM_IO_ERROR, "bad dim[0] in " + path);
  h->dim[0] = nd;
  for (int i = 1; i < 8; i++) {
    const int d = get<int16_t>(raw, kDim + 2 * i);
    if (i <= nd && d < 1) return fail(CDM_IO_ERROR, "bad dimension in " + path);
    h->dim[i] = i <= nd ? d : 1;
  }
  for (int i = 0; i < 8; i++) h->pixdim[i] = get<float>(raw, kPixdim + 4 * i);
  h->datatype = get<int16_t>(raw, kDatatype);
  h->bitpix = get<int16_t>(raw, kBitpix);
  if (type_bytes(h->datatype) == 0)
    return fail(CDM_IO_ERROR, "unsupported NIfTI datatype " + std::to_string(h->datatype) + " in " + path);
  h->scl_slope = get<float>(raw, kSclSlope);
  h->scl_inter = get<float>(raw, kSclInter);
  h->cal_min = get<float>(raw, kCalMin);
  h->cal_max = get<float>(raw, kCalMax);
  const float vo = get<float>(raw, kVoxOffset);
  h->vox_offset = vo < (float)kHdrBytes ? kHdrBytes : (int64_t)vo;
  std::memcpy(h->raw, raw, kHdrBytes);
  *swapped = swap;
  return CDM_OK;
}

void shape_of(const cdm_nifti_hdr* h, int64_t* nxyz, int64_t* nt) {
  *nxyz = (int64_t)h->dim[1] * h->dim[2] * h->dim[3];
  int64_t t = 1;
  for (int i = 4; i < 8; i++) t *= h->dim[i];
  *nt = t;
}

bool same_grid(const cdm_nifti_hdr& a, const cdm_nifti_hdr& b) {
  return a.dim[1] == b.dim[1] && a.dim[2] == b.dim[2] && a.dim[3] == b.dim[3];
}

// One image read whole: header and double voxels [nt][nxyz].
cdm_status read_image(const std::string& path, cdm_nifti_hdr* h, std::vector<double>* data) {
  cdm_status s = cdm_nifti_read(path.c_str(), h, nullptr, 0);
  if (s != CDM_OK) return s;
  int64_t nxyz, nt;
  shape_of(h, &nxyz, &nt);
  data->assign((size_t)(nxyz * nt), 0.0);
  return cdm_nifti_read(path.c_str(), h, data->data(), (int64_t)data->size());
}

std::string dir_part(const char* partsdir, int i) {
  return std::string(partsdir) + "/part_" + std::to_string(i);
}

// Voxel-major [nvox][ncols] into the parts of `name` (cdm_split_parts),
// carrying its error message over.
cdm_status split_into(const char* partsdir, int nparts, const std::string& name, int nvox, int ncols,
                      const double* data) {
  const cdm_status s = cdm_split_parts(partsdir, nparts, name.c_str(), nvox, ncols, data);
  return s == CDM_OK ? s : fail(s, std::string("writing ") + name + ": " + cdm_utils_last_error());
}

std::string trim_right(std::string s) {
  while (!s.empty() && (s.back() == '\r' || s.back() == ' ' || s.back() == '\t')) s.pop_back();
  return s;
}

}  // namespace

extern "C" {

const char* cdm_volumes_last_error(void) { return g_err.c_str(); }

int cdm_nifti_gzip(void) {
#ifdef CDM_HAVE_ZLIB
  return 1;
#else
  return 0;
#endif
}

cdm_status cdm_nifti_shape(const cdm_nifti_hdr* hdr, int64_t* nxyz, int* nt) {
  if (!hdr || !nxyz || !nt) return fail(CDM_BAD_ARG, "bad argument");
  int64_t t;
  shape_of(hdr, nxyz, &t);
  if (t > std::numeric_limits<int>::max()) return fail(CDM_BAD_ARG, "too many volumes");
  *nt = (int)t;
  return CDM_OK;
}

cdm_status cdm_nifti_read(const char* path, cdm_nifti_hdr* hdr, double* data, int64_t capacity) {
  if (!path || !hdr) return fail(CDM_BAD_ARG, "bad argument");
  in_file in(path);
  if (!in.ok()) return fail(CDM_IO_ERROR, std::string("cannot open ") + path + ": " + in.err());
  if (in.gzipped())
    return fail(CDM_IO_ERROR, std::string("gzip-compressed image and the library was built without zlib: ") + path);
  unsigned char raw[kHdrBytes];
  if (!in.read(raw, kHdrBytes)) return fail(CDM_IO_ERROR, std::string("short header: ") + path);
  bool swap = false;
  cdm_status s = parse_header(raw, path, hdr, &swap);
  if (s != CDM_OK || !data) return s;
  int64_t nxyz, nt;
  shape_of(hdr, &nxyz, &nt);
  const int64_t n = nxyz * nt;
  if (capacity < n) return fail(CDM_BAD_ARG, "output capacity too small");
  if (!in.skip(hdr->vox_offset - kHdrBytes)) return fail(CDM_IO_ERROR, std::string("short file: ") + path);
  const int tb = type_bytes(hdr->datatype);
  const bool scale = hdr->scl_slope != 0.0f && std::isfinite(hdr->scl_slope) &&
                     !(hdr->scl_slope == 1.0f && hdr->scl_inter == 0.0f);
  const double slope = hdr->scl_slope, inter = hdr->scl_inter;
  std::vector<unsigned char> buf((size_t)1 << 20);
  const int64_t per = (int64_t)buf.size() / tb;
  for (int64_t i0 = 0; i0 < n; i0 += per) {
    const int64_t k = n - i0 < per ? n - i0 : per;
    if (!in.read(buf.data(), (size_t)(k * tb))) return fail(CDM_IO_ERROR, std::string("short data: ") + path);
    for (int64_t i = 0; i < k; i++) {
      unsigned char* p = buf.data() + i * tb;
      if (swap) swap_bytes(p, tb);
      const double v = to_double(p, hdr->datatype);
      data[i0 + i] = scale ? v * slope + inter : v;
    }
  }
  return CDM_OK;
}

cdm_status cdm_nifti_write(const char* path, const cdm_nifti_hdr* like, int nt, const double* data,
                           int datatype) {
  if (!path || !like || nt <= 0 || !data) return fail(CDM_BAD_ARG, "bad argument");
  if (datatype != CDM_NIFTI_FLOAT32 && datatype != CDM_NIFTI_FLOAT64)
    return fail(CDM_BAD_ARG, "output datatype must be float32 or float64");
  if (nt > 32767) return fail(CDM_BAD_ARG, "more volumes than a NIfTI-1 dimension holds");
  unsigned char raw[kHdrBytes];
  std::memcpy(raw, like->raw, kHdrBytes);
  put<int32_t>(raw, kSizeofHdr, kHdrBytes);
  int16_t dim[8];
  dim[0] = nt > 1 ? 4 : 3;
  for (int i = 1; i <= 3; i++) dim[i] = (int16_t)(like->dim[i] > 0 ? like->dim[i] : 1);
  dim[4] = (int16_t)nt;
  dim[5] = dim[6] = dim[7] = 1;
  for (int i = 0; i < 8; i++) put<int16_t>(raw, kDim + 2 * i, dim[i]);
  put<int16_t>(raw, kDatatype, (int16_t)datatype);
  put<int16_t>(raw, kBitpix, (int16_t)(8 * type_bytes(datatype)));
  put<float>(raw, kVoxOffset, 352.0f);
  put<float>(raw, kSclSlope, 1.0f);
  put<float>(raw, kSclInter, 0.0f);
  const int64_t nxyz = (int64_t)dim[1] * dim[2] * dim[3], n = nxyz * nt;
  double lo = std::numeric_limits<double>::infinity(), hi = -lo;
  for (int64_t i = 0; i < n; i++) {
    if (data[i] < lo) lo = data[i];
    if (data[i] > hi) hi = data[i];
  }
  put<float>(raw, kCalMin, n ? (float)lo : 0.0f);
  put<float>(raw, kCalMax, n ? (float)hi : 0.0f);
  std::memcpy(raw + kMagic, "n+1", 4);
  const unsigned char ext[4] = {0, 0, 0, 0};
  const int tb = type_bytes(datatype);
  std::vector<unsigned char> body;
  body.reserve((size_t)(n * tb));
  for (int64_t i = 0; i < n; i++) {
    unsigned char b[8];
    if (datatype == CDM_NIFTI_FLOAT32) {
      const float f = (float)data[i];
      std::memcpy(b, &f, 4);
    } else {
      std::memcpy(b, &data[i], 8);
    }
    body.insert(body.end(), b, b + tb);
  }
  const std::string p(path);
  if (ends_with(p, ".gz")) {
#ifdef CDM_HAVE_ZLIB
    gzFile g = gzopen(path, "wb6");
    if (!g) return fail(CDM_IO_ERROR, "cannot create " + p + ": " + std::strerror(errno));
    bool ok = gzwrite(g, raw, kHdrBytes) == kHdrBytes && gzwrite(g, ext, 4) == 4;
    for (size_t off = 0; ok && off < body.size(); off += (size_t)1 << 30) {
      const unsigned k = (unsigned)std::min(body.size() - off, (size_t)1 << 30);
      ok = gzwrite(g, body.data() + off, k) == (int)k;
    }
    if (gzclose(g) != Z_OK) ok = false;
    return ok ? CDM_OK : fail(CDM_IO_ERROR, "write failed: " + p);
#else
    return fail(CDM_IO_ERROR, "the library was built without zlib: cannot write " + p);
#endif
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(CDM_IO_ERROR, "cannot create " + p + ": " + std::strerror(errno));
  bool ok = std::fwrite(raw, 1, kHdrBytes, f) == (size_t)kHdrBytes && std::fwrite(ext, 1, 4, f) == 4 &&
            std::fwrite(body.data(), 1, body.size(), f) == body.size();
  if (std::fclose(f) != 0) ok = false;
  return ok ? CDM_OK : fail(CDM_IO_ERROR, "write failed: " + p);
}

cdm_status cdm_mask_count(int64_t nxyz, const double* mask, int* nvox) {
  if (nxyz < 0 || !mask || !nvox) return fail(CDM_BAD_ARG, "bad argument");
  int64_t n = 0;
  for (int64_t i = 0; i < nxyz; i++) n += mask[i] > 0.0;
  if (n > std::numeric_limits<int>::max()) return fail(CDM_BAD_ARG, "too many voxels");
  *nvox = (int)n;
  return CDM_OK;
}

cdm_status cdm_mask_gather(int64_t nxyz, int nt, const double* vol, const double* mask, double* out) {
  if (nxyz < 0 || nt <= 0 || !vol || !mask || !out) return fail(CDM_BAD_ARG, "bad argument");
  int64_t v = 0;
  for (int64_t i = 0; i < nxyz; i++) {
    if (!(mask[i] > 0.0)) continue;
    for (int t = 0; t < nt; t++) out[v * nt + t] = vol[(int64_t)t * nxyz + i];
    v++;
  }
  return CDM_OK;
}

cdm_status cdm_mask_scatter(int64_t nxyz, int nt, const double* in, const double* mask, double* vol) {
  if (nxyz < 0 || nt <= 0 || !in || !mask || !vol) return fail(CDM_BAD_ARG, "bad argument");
  int64_t v = 0;
  for (int64_t i = 0; i < nxyz; i++) {
    const bool m = mask[i] > 0.0;
    for (int t = 0; t < nt; t++) vol[(int64_t)t * nxyz + i] = m ? in[v * nt + t] : 0.0;
    v += m;
  }
  return CDM_OK;
}

cdm_status cdm_split_volumes(const char* partsdir, int nparts, const char* data_path,
                             const char* mask_path, const char* init_list, int nparams,
                             const double* init_values, const char* fixp_list, int nfixp,
                             const int* fixp_sizes, int* nvox_out) {
  if (!partsdir || nparts <= 0 || !data_path || !mask_path || nparams <= 0 || nfixp < 0 ||
      (nfixp > 0 && !fixp_sizes))
    return fail(CDM_BAD_ARG, "bad argument");
  cdm_nifti_hdr mh, dh;
  std::vector<double> mask, vol;
  cdm_status s = read_image(mask_path, &mh, &mask);
  if (s != CDM_OK) return s;
  s = read_image(data_path, &dh, &vol);
  if (s != CDM_OK) return s;
  if (!same_grid(mh, dh)) return fail(CDM_BAD_ARG, "the data and the mask have different grids");
  int64_t nxyz, nmeas;
  shape_of(&dh, &nxyz, &nmeas);
  int nvox = 0;
  if ((s = cdm_mask_count(nxyz, mask.data(), &nvox)) != CDM_OK) return s;
  if (nvox <= 0) return fail(CDM_BAD_ARG, "The number of voxels must be greater than 0");
  if (nvox < nparts) return fail(CDM_BAD_ARG, "The number of parts/jobs must be lower than number of voxels");
  // checks of the lists before anything is written
  if (nfixp > 0 && !fixp_list)
    return fail(CDM_BAD_ARG, "Expected a list with " + std::to_string(nfixp) +
                                 " NIfTI files for specifying the Fixed Parameters of the model");
  if (nfixp == 0 && fixp_list)
    return fail(CDM_BAD_ARG, "This model does not need any Fixed Parameter, however a Fixed Parameter file was given");

  std::vector<double> vox((size_t)nvox * (size_t)nmeas);
  cdm_mask_gather(nxyz, (int)nmeas, vol.data(), mask.data(), vox.data());
  vol.clear();
  vol.shrink_to_fit();
  if ((s = split_into(partsdir, nparts, "data", nvox, (int)nmeas, vox.data())) != CDM_OK) return s;

  std::vector<double> col((size_t)nvox);
  if (init_list) {
    std::ifstream file(init_list);
    if (!file.is_open()) return fail(CDM_IO_ERROR, std::string("Unable to open Initialization Parameter file: ") + init_list);
    std::string line;
    int id = -1;
    while (std::getline(file, line)) {
      id++;
      if (id >= nparams)
        return fail(CDM_BAD_ARG, std::string("Too many lines for specifying the initialization of the parameters in the file: ") +
                                     init_list + ". The number of lines must match the number of parameters in this model: " +
                                     std::to_string(nparams));
      line = trim_right(line);
      if (!line.empty()) {
        cdm_nifti_hdr ph;
        std::vector<double> pv;
        if ((s = read_image(line, &ph, &pv)) != CDM_OK) return s;
        if (!same_grid(mh, ph))
          return fail(CDM_BAD_ARG, "The size of the mask and the volume used for initializing the parameters: " + line +
                                       " does not match");
        int64_t pxyz, pt;
        shape_of(&ph, &pxyz, &pt);
        if (pt != 1) return fail(CDM_BAD_ARG, "The volume used to initialize the parameters: " + line + " must be a 3D volume");
        cdm_mask_gather(pxyz, 1, pv.data(), mask.data(), col.data());
      } else {
        const double c = init_values ? init_values[id] : 0.0;
        for (double& x : col) x = c;
      }
      if ((s = split_into(partsdir, nparts, "ParamInit_" + std::to_string(id), nvox, 1, col.data())) != CDM_OK)
        return s;
    }
    if (id != nparams - 1)
      return fail(CDM_BAD_ARG, std::string("The number of volumes (lines) provided for initializing the parameters in: ") +
                                   init_list + " does not match the number of parameters of this model: " +
                                   std::to_string(nparams) + ". If a parameter does not need initialization, its line can be empty.");
  }

  if (nfixp > 0) {
    std::ifstream file(fixp_list);
    if (!file.is_open()) return fail(CDM_IO_ERROR, std::string("Unable to open Fixed Parameter file: ") + fixp_list);
    std::string line;
    int id = -1;
    while (id < nfixp - 1 && std::getline(file, line)) {
      id++;
      line = trim_right(line);
      if (line.empty())
        return fail(CDM_BAD_ARG, std::string("Please remove the empty lines in the file used for specifying the Fixed Parameters: ") +
                                     fixp_list);
      cdm_nifti_hdr fh;
      std::vector<double> fv;
      if ((s = read_image(line, &fh, &fv)) != CDM_OK) return s;
      if (!same_grid(mh, fh))
        return fail(CDM_BAD_ARG, "The size of the mask and the volume used for specifying the Fixed Parameters: " + line +
                                     " does not match");
      int64_t fxyz, ft;
      shape_of(&fh, &fxyz, &ft);
      if (ft != fixp_sizes[id])
        return fail(CDM_BAD_ARG, "The NIfTI file used for specifying the Fixed Parameters: " + line + " must have " +
                                     std::to_string(fixp_sizes[id]) + " volumes");
      std::vector<double> fp((size_t)nvox * (size_t)ft);
      cdm_mask_gather(fxyz, (int)ft, fv.data(), mask.data(), fp.data());
      if ((s = split_into(partsdir, nparts, "FixParam_" + std::to_string(id), nvox, (int)ft, fp.data())) != CDM_OK)
        return s;
    }
    if (id != nfixp - 1)
      return fail(CDM_BAD_ARG, std::string("The number of NIfTI files (lines) provided in the file for specifying the Fixed Parameters: ") +
                                   fixp_list + " does not match the number of parameters of this model: " + std::to_string(nfixp));
  }
  if (nvox_out) *nvox_out = nvox;
  return CDM_OK;
}

cdm_status cdm_merge_volumes(const char* partsdir, int nparts, const char* name, int nrows,
                             const char* mask_path, const char* out_path) {
  if (!partsdir || nparts <= 0 || !name || !mask_path || !out_path || nrows == 0 || nrows < -1)
    return fail(CDM_BAD_ARG, "bad argument");
  cdm_nifti_hdr mh;
  std::vector<double> mask;
  cdm_status s = read_image(mask_path, &mh, &mask);
  if (s != CDM_OK) return s;
  int64_t nxyz, mt;
  shape_of(&mh, &nxyz, &mt);
  int nvox = 0, total = 0, ncols = 0;
  cdm_mask_count(nxyz, mask.data(), &nvox);
  // every part must carry nrows rows (the first part's count with nrows -1)
  char path[4096];
  for (int i = 0; i < nparts; i++) {
    int n, c;
    if ((s = cdm_part_path(partsdir, i, name, path, sizeof(path))) != CDM_OK ||
        (s = cdm_part_read(path, &n, &c, nullptr, 0)) != CDM_OK)
      return fail(s, cdm_utils_last_error());
    if (nrows == -1) nrows = c;
    if (n <= 0 || c != nrows)
      return fail(CDM_IO_ERROR, std::string("The amount of data in the intermediate output file: ") + path +
                                    " is not correct.");
    total += n;
  }
  if (total != nvox)
    return fail(CDM_IO_ERROR, "the parts of " + std::string(name) + " hold " + std::to_string(total) +
                                  " voxels and the mask " + std::to_string(nvox));
  std::vector<double> vox((size_t)nvox * (size_t)nrows);
  if ((s = cdm_merge_parts(partsdir, nparts, name, &total, &ncols, vox.data(), (int64_t)vox.size())) != CDM_OK)
    return fail(s, cdm_utils_last_error());
  std::vector<double> vol((size_t)(nxyz * nrows));
  cdm_mask_scatter(nxyz, nrows, vox.data(), mask.data(), vol.data());
  return cdm_nifti_write(out_path, &mh, nrows, vol.data(), CDM_NIFTI_FLOAT64);
}

}  // extern "C"
