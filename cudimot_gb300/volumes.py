"""ctypes mirror of include/cdm_volumes.h: NIfTI-1 volumes, masks, and
CUDIMOT's split_parts / merge_parts on volumes (libcdm_utils.so).

Volumes are numpy float64 arrays [nt][nz][ny][nx] (the file's order, x
fastest); voxel arrays are [nvox][nt], the library's layout."""
import ctypes as C

import numpy as np

from . import utils
from .capi import STATUS, CdmError

FLOAT32, FLOAT64 = 16, 64


class NiftiHdr(C.Structure):
    _fields_ = [("dim", C.c_int32 * 8), ("pixdim", C.c_float * 8), ("datatype", C.c_int32),
                ("bitpix", C.c_int32), ("scl_slope", C.c_float), ("scl_inter", C.c_float),
                ("cal_min", C.c_float), ("cal_max", C.c_float), ("vox_offset", C.c_int64),
                ("raw", C.c_ubyte * 348)]

    @property
    def shape(self):
        """(nt, nz, ny, nx) of the voxel array cdm_nifti_read returns."""
        nt = 1
        for i in range(4, 8):
            nt *= self.dim[i]
        return (nt, self.dim[3], self.dim[2], self.dim[1])


_READY = False


def lib():
    global _READY
    L = utils.lib()
    if not _READY:
        vp, i, i64, cp = C.c_void_p, C.c_int, C.c_int64, C.c_char_p
        hp = C.POINTER(NiftiHdr)
        sig = {
            "cdm_nifti_read": [cp, hp, vp, i64],
            "cdm_nifti_shape": [hp, C.POINTER(i64), C.POINTER(i)],
            "cdm_nifti_write": [cp, hp, i, vp, i],
            "cdm_mask_count": [i64, vp, C.POINTER(i)],
            "cdm_mask_gather": [i64, i, vp, vp, vp],
            "cdm_mask_scatter": [i64, i, vp, vp, vp],
            "cdm_split_volumes": [cp, i, cp, cp, cp, i, vp, cp, i, vp, C.POINTER(i)],
            "cdm_merge_volumes": [cp, i, cp, i, cp, cp],
        }
        for n, a in sig.items():
            f = getattr(L, n)
            f.argtypes = a
            f.restype = C.c_int
        L.cdm_nifti_gzip.restype = C.c_int
        L.cdm_volumes_last_error.restype = C.c_char_p
        _READY = True
    return L


def _check(status, what):
    if status != 0:
        raise CdmError(f"{what}: {STATUS.get(status, status)}: "
                       f"{lib().cdm_volumes_last_error().decode(errors='replace')}")


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _s(x):
    return None if x is None else str(x).encode()


def gzip_supported():
    return bool(lib().cdm_nifti_gzip())


def read_header(path):
    h = NiftiHdr()
    _check(lib().cdm_nifti_read(_s(path), C.byref(h), None, 0), "nifti_read")
    return h


def read(path):
    """(header, float64 array [nt][nz][ny][nx])."""
    h = read_header(path)
    out = np.empty(h.shape)
    _check(lib().cdm_nifti_read(_s(path), C.byref(h), _p(out), out.size), "nifti_read")
    return h, out


def write(path, like, data, datatype=FLOAT64):
    """Write data [nt][nz][ny][nx] (or [nz][ny][nx]) on like's grid."""
    data = np.ascontiguousarray(data, dtype=np.float64)
    nt = 1 if data.ndim == 3 else data.shape[0]
    if data.size != nt * like.dim[1] * like.dim[2] * like.dim[3]:
        raise CdmError("write: data does not match the template's grid")
    _check(lib().cdm_nifti_write(_s(path), C.byref(like), nt, _p(data), datatype), "nifti_write")


def mask_count(mask):
    mask = np.ascontiguousarray(mask, dtype=np.float64)
    n = C.c_int()
    _check(lib().cdm_mask_count(mask.size, _p(mask), C.byref(n)), "mask_count")
    return n.value


def mask_gather(vol, mask):
    """[nt][...] volume -> [nvox][nt] voxels inside the mask."""
    mask = np.ascontiguousarray(mask, dtype=np.float64)
    vol = np.ascontiguousarray(vol, dtype=np.float64)
    nt = vol.size // mask.size
    out = np.empty((mask_count(mask), nt))
    _check(lib().cdm_mask_gather(mask.size, nt, _p(vol), _p(mask), _p(out)), "mask_gather")
    return out


def mask_scatter(vox, mask):
    """[nvox][nt] voxels -> [nt][*mask.shape] volume, zero outside the mask."""
    mask = np.ascontiguousarray(mask, dtype=np.float64)
    vox = np.ascontiguousarray(vox, dtype=np.float64)
    if vox.ndim == 1:
        vox = vox[:, None]
    nt = vox.shape[1]
    out = np.empty((nt,) + mask.shape)
    _check(lib().cdm_mask_scatter(mask.size, nt, _p(vox), _p(mask), _p(out)), "mask_scatter")
    return out


def split_volumes(partsdir, nparts, data_path, mask_path, nparams, init_list=None, init_values=None,
                  fixp_list=None, fixp_sizes=()):
    """split_parts: data, ParamInit_<p> and FixParam_<i> part files; returns
    the number of voxels in the mask."""
    iv = None if init_values is None else np.ascontiguousarray(init_values, dtype=np.float64)
    fs = np.ascontiguousarray(fixp_sizes, dtype=np.int32) if len(fixp_sizes) else None
    n = C.c_int()
    _check(lib().cdm_split_volumes(_s(partsdir), nparts, _s(data_path), _s(mask_path), _s(init_list),
                                   nparams, _p(iv), _s(fixp_list), len(fixp_sizes), _p(fs),
                                   C.byref(n)), "split_volumes")
    return n.value


def merge_volumes(partsdir, nparts, name, mask_path, out_path, nrows=-1):
    """merge_parts' join_Parts: the parts of <name> as a NIfTI on the mask's grid."""
    _check(lib().cdm_merge_volumes(_s(partsdir), nparts, _s(name), nrows, _s(mask_path), _s(out_path)),
           "merge_volumes")
