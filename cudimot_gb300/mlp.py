"""ctypes mirror of include/cdm_mlp.h (the learned initialiser library),
on torch CUDA tensors."""
import ctypes as C
import os

import numpy as np

from .capi import LIBDIR, STATUS, CdmError

MAX_MU = 16


class MlpCfg(C.Structure):
    _fields_ = [("n_in", C.c_int), ("hidden", C.c_int), ("n_mu", C.c_int), ("n_sig", C.c_int),
                ("group", C.c_int * MAX_MU), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("logstd_min", C.c_float),
                ("logstd_max", C.c_float)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(LIBDIR, "libcdm_mlp.so")
        if not os.path.exists(path):
            raise CdmError(f"{path} is not built (python -m cudimot_gb300.build)")
        L = C.CDLL(path)
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        sig = {
            "cdm_mlp_create": [C.POINTER(MlpCfg), C.POINTER(vp)],
            "cdm_mlp_destroy": [vp],
            "cdm_mlp_set_params": [vp, i, vp, vp],
            "cdm_mlp_get_params": [vp, i, vp, vp, vp, vp],
            "cdm_mlp_train_step": [vp, vp, vp, i, vp, vp],
            "cdm_mlp_gradients": [vp, vp, vp, i, vp, vp],
            "cdm_mlp_forward": [vp, vp, i, vp, vp],
            "cdm_mlp_prep_input": [vp, vp, i, i, i, i, vp, vp],
            "cdm_mlp_gemm_bf16": [vp, i, vp, i, i, i, i, vp, i, vp],
            "cdm_mlp_hidden_layer": [vp, i, vp, i, i, vp, i, vp],
            "cdm_mlp_check": [vp],
        }
        for n, a in sig.items():
            fn = getattr(L, n)
            fn.argtypes = a
            fn.restype = C.c_int
        L.cdm_mlp_default_cfg.argtypes = [C.POINTER(MlpCfg)]
        L.cdm_mlp_default_cfg.restype = None
        L.cdm_mlp_last_error.restype = C.c_char_p
        _LIB = L
    return _LIB


def _check(status, what):
    if status != 0:
        raise CdmError(f"{what}: {STATUS.get(status, status)}: "
                       f"{lib().cdm_mlp_last_error().decode(errors='replace')}")


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def default_cfg(**kw) -> MlpCfg:
    c = MlpCfg()
    lib().cdm_mlp_default_cfg(C.byref(c))
    for k, v in kw.items():
        if k == "group":
            for j, g in enumerate(v):
                c.group[j] = g
        else:
            setattr(c, k, v)
    return c


def gemm_bf16(A, B):
    """A [M][K], B [N][K] bf16 CUDA tensors -> fp32 [M][N] = A B^T on the
    tensor cores."""
    import torch
    M, K = A.shape
    N = B.shape[0]
    out = torch.zeros(M, N, dtype=torch.float32, device=A.device)
    _check(lib().cdm_mlp_gemm_bf16(_p(A), A.stride(0), _p(B), B.stride(0), M, N, K, _p(out), N,
                                   _stream()), "gemm")
    return out


def prep_input(meas, s0, ld=None):
    """meas [n][nmeas] float64, s0 [n][k] float64 (column 0 used) -> bf16 [n][ld]."""
    import torch
    n, nm = meas.shape
    ld = ld or (nm + 7) // 8 * 8
    x = torch.empty(n, ld, dtype=torch.bfloat16, device=meas.device)
    _check(lib().cdm_mlp_prep_input(_p(meas), _p(s0), s0.stride(0) if s0 is not None else 0, n, nm,
                                    ld, _p(x), _stream()), "prep_input")
    return x


class Mlp:
    def __init__(self, cfg: MlpCfg):
        self.cfg = cfg
        h = C.c_void_p()
        _check(lib().cdm_mlp_create(C.byref(cfg), C.byref(h)), "create")
        self.h = h
        self.n_out = cfg.n_mu + cfg.n_sig

    def close(self):
        if getattr(self, "h", None):
            lib().cdm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dims(self):
        c = self.cfg
        return [c.n_in, c.hidden, c.hidden, c.hidden, self.n_out]

    def set_params(self, W, b):
        for l in range(4):
            w = np.ascontiguousarray(W[l], dtype=np.float32)
            bb = np.ascontiguousarray(b[l], dtype=np.float32)
            _check(lib().cdm_mlp_set_params(self.h, l, w.ctypes.data_as(C.c_void_p),
                                            bb.ctypes.data_as(C.c_void_p)), "set_params")

    def get_params(self, grads=False):
        d = self.dims()
        W, b, gW, gb = [], [], [], []
        for l in range(4):
            w = np.zeros((d[l + 1], d[l]), np.float32)
            bb = np.zeros(d[l + 1], np.float32)
            gw = np.zeros_like(w)
            gbb = np.zeros_like(bb)
            q = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
            _check(lib().cdm_mlp_get_params(self.h, l, q(w), q(bb), q(gw), q(gbb)), "get_params")
            W.append(w)
            b.append(bb)
            gW.append(gw)
            gb.append(gbb)
        return (W, b, gW, gb) if grads else (W, b)

    def train_step(self, x, t, loss=None):
        _check(lib().cdm_mlp_train_step(self.h, _p(x), _p(t), x.shape[0], _p(loss), _stream()),
               "train_step")

    def gradients(self, x, t, loss=None):
        _check(lib().cdm_mlp_gradients(self.h, _p(x), _p(t), x.shape[0], _p(loss), _stream()),
               "gradients")

    def forward(self, x, out=None):
        import torch
        n = x.shape[0]
        if out is None:
            out = torch.zeros(n, 16, dtype=torch.float32, device=x.device)
        _check(lib().cdm_mlp_forward(self.h, _p(x), n, _p(out), _stream()), "forward")
        return out

    def hidden_layer(self, layer, x, out):
        """One hidden layer of inference alone: out = bf16(gelu(x W^T + b))
        (bf16 CUDA tensors [n][width])."""
        _check(lib().cdm_mlp_hidden_layer(self.h, layer, _p(x), x.stride(0), x.shape[0], _p(out),
                                          out.stride(0), _stream()), "hidden_layer")

    def check(self):
        _check(lib().cdm_mlp_check(self.h), "device check")
