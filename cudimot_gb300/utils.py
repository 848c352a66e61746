"""ctypes mirror of include/cdm_utils.h: DTI initialiser, *_finish
post-processing and CUDIMOT's binary part files."""
import ctypes as C
import os

import numpy as np

from .capi import LIBDIR, STATUS, CdmError

DTI_COLS = ("S0", "L1", "L2", "L3", "V1X", "V1Y", "V1Z", "V2X", "V2Y", "V2Z", "FA", "MD", "TH1",
            "PH1", "TH2", "PH2", "PSI")
_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(LIBDIR, "libcdm_utils.so")
        if not os.path.exists(path):
            raise CdmError(f"{path} is not built (python -m cudimot_gb300.build)")
        L = C.CDLL(path)
        vp, i, i64, cp = C.c_void_p, C.c_int, C.c_int64, C.c_char_p
        sig = {
            "cdm_dti_fit": [i, i, vp, vp, vp, vp, vp],
            "cdm_sample_stats": [i, i, i, vp, vp, vp, vp],
            "cdm_dyads": [i, i, i, vp, i, i, vp, vp],
            "cdm_od_from_kappa": [i, vp, i, vp, vp],
            "cdm_mean_columns": [i, i, vp, vp, i, vp, i, vp],
            "cdm_copy_columns": [i, vp, i, i, vp, i, i, i, C.c_double, vp],
            "cdm_part_path": [cp, i, cp, C.c_char_p, i],
            "cdm_part_write": [cp, i, i, vp],
            "cdm_part_read": [cp, C.POINTER(i), C.POINTER(i), vp, i64],
            "cdm_split_parts": [cp, i, cp, i, i, vp],
            "cdm_merge_parts": [cp, i, cp, C.POINTER(i), C.POINTER(i), vp, i64],
        }
        for n, a in sig.items():
            f = getattr(L, n)
            f.argtypes = a
            f.restype = C.c_int
        L.cdm_utils_last_error.restype = C.c_char_p
        _LIB = L
    return _LIB


def _check(status, what):
    if status != 0:
        raise CdmError(f"{what}: {STATUS.get(status, status)}: "
                       f"{lib().cdm_utils_last_error().decode(errors='replace')}")


def _d(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _hd(x):
    """Pointer of a CUDA tensor or a numpy array (host)."""
    if isinstance(x, np.ndarray):
        return x.ctypes.data_as(C.c_void_p)
    return C.c_void_p(x.contiguous().data_ptr())


def dti_fit(meas, bvecs, bvals, out=None):
    """meas [n][nmeas] (CUDA float64), bvecs [nmeas][3], bvals [nmeas]
    (numpy or CUDA) -> [n][17] (columns DTI_COLS)."""
    import torch
    n, nm = meas.shape
    if out is None:
        out = torch.empty(n, len(DTI_COLS), dtype=torch.float64, device=meas.device)
    keep = (bvecs, bvals)
    bv = np.ascontiguousarray(bvecs, dtype=np.float64) if isinstance(bvecs, np.ndarray) else bvecs.contiguous()
    bb = np.ascontiguousarray(bvals, dtype=np.float64) if isinstance(bvals, np.ndarray) else bvals.contiguous()
    _check(lib().cdm_dti_fit(n, nm, _d(meas), _hd(bv), _hd(bb), _d(out), _stream()), "dti_fit")
    del keep
    return out


def sample_stats(samples):
    import torch
    n, p, s = samples.shape
    mean = torch.empty(n, p, dtype=torch.float64, device=samples.device)
    sd = torch.empty_like(mean)
    sample_stats_into(samples, mean, sd)
    return mean, sd


def sample_stats_into(samples, mean, sd=None):
    n, p, s = samples.shape
    _check(lib().cdm_sample_stats(n, p, s, _d(samples), _d(mean), _d(sd), _stream()), "sample_stats")


def dyads(samples, ith, iph):
    import torch
    out = torch.empty(samples.shape[0], 4, dtype=torch.float64, device=samples.device)
    dyads_into(samples, ith, iph, out)
    return out


def dyads_into(samples, ith, iph, out):
    n, p, s = samples.shape
    _check(lib().cdm_dyads(n, p, s, _d(samples), ith, iph, _d(out), _stream()), "dyads")


def od_from_kappa(kappa_col, out=None):
    """kappa_col: CUDA float64 tensor [n] or a column view (any stride)."""
    import torch
    n = kappa_col.shape[0]
    if out is None:
        out = torch.empty(n, dtype=torch.float64, device=kappa_col.device)
    _check(lib().cdm_od_from_kappa(n, C.c_void_p(kappa_col.data_ptr()), kappa_col.stride(0), _d(out),
                                   _stream()), "od")
    return out


def mean_columns(meas, idx, out, out_ld=None):
    """out[v * out_ld] = mean(meas[v, idx]); idx an int32 CUDA tensor."""
    n, nm = meas.shape
    _check(lib().cdm_mean_columns(n, nm, _d(meas), C.c_void_p(idx.data_ptr()), idx.shape[0], _d(out),
                                  out_ld or out.stride(0), _stream()), "mean_columns")


def copy_columns(src, src_col, dst, dst_col, ncols, scale=1.0):
    """dst[:, dst_col:dst_col+ncols] = scale * src[:, src_col:...] (src None:
    fill with scale)."""
    n = dst.shape[0]
    _check(lib().cdm_copy_columns(n, _d(src), 0 if src is None else src.stride(0), src_col, _d(dst),
                                  dst.stride(0), dst_col, ncols, float(scale), _stream()),
           "copy_columns")


def part_path(partsdir, id_part, name):
    buf = C.create_string_buffer(4096)
    _check(lib().cdm_part_path(partsdir.encode(), id_part, name.encode(), buf, 4096), "part_path")
    return buf.value.decode()


def part_write(path, data):
    data = np.ascontiguousarray(data, dtype=np.float64)
    if data.ndim == 1:
        data = data[:, None]
    _check(lib().cdm_part_write(path.encode(), data.shape[0], data.shape[1],
                                data.ctypes.data_as(C.c_void_p)), "part_write")


def part_read(path):
    n, c = C.c_int(), C.c_int()
    _check(lib().cdm_part_read(path.encode(), C.byref(n), C.byref(c), None, 0), "part_read")
    out = np.empty((n.value, c.value))
    _check(lib().cdm_part_read(path.encode(), C.byref(n), C.byref(c), out.ctypes.data_as(C.c_void_p),
                               out.size), "part_read")
    return out


def split_parts(partsdir, nparts, name, data):
    data = np.ascontiguousarray(data, dtype=np.float64)
    if data.ndim == 1:
        data = data[:, None]
    _check(lib().cdm_split_parts(partsdir.encode(), nparts, name.encode(), data.shape[0],
                                 data.shape[1], data.ctypes.data_as(C.c_void_p)), "split_parts")


def merge_parts(partsdir, nparts, name):
    n, c = C.c_int(), C.c_int()
    _check(lib().cdm_merge_parts(partsdir.encode(), nparts, name.encode(), C.byref(n), C.byref(c),
                                 None, 0), "merge_parts")
    out = np.empty((n.value, c.value))
    _check(lib().cdm_merge_parts(partsdir.encode(), nparts, name.encode(), C.byref(n), C.byref(c),
                                 out.ctypes.data_as(C.c_void_p), out.size), "merge_parts")
    return out
