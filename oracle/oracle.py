"""ctypes bindings of the CPU oracle (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, to check and to time the GPU library; the library never does.

    o = Oracle("NODDI_Watson")                  # oracle/_build/liboracle_*.so
    r = Oracle("NODDI_Watson", reference=True)  # CUDIMOT's own plugin (here only)
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from cudimot_gb300.capi import CfgStruct, ModelInfo, make_cfg  # noqa: E402

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _arr(x, dtype=np.float64):
    return np.ascontiguousarray(x, dtype=dtype)


def _ptr(x):
    return None if x is None else x.ctypes.data_as(C.c_void_p)


class Oracle:
    def __init__(self, model: str, reference: bool = False, build: bool = True):
        if reference:
            path = os.path.join(HERE, "_ref", f"libref_{model}.so")
        else:
            path = os.path.join(HERE, "_build", f"liboracle_{model}.so")
        if build and not os.path.exists(path):
            from oracle import build_oracle  # noqa
            if reference:
                raise FileNotFoundError(path)
            errs = build_oracle.build([model])
            if errs:
                raise RuntimeError(str(errs))
        self.lib = C.CDLL(path)
        self.model = model
        info = ModelInfo()
        self.lib.orc_model_info(C.byref(info))
        self.info = info
        self.nparams = info.nparams
        self.cfp_tsize = info.cfp_tsize
        self.fixp_tsize = info.fixp_tsize
        for name in ("orc_signal", "orc_cost", "orc_gridsearch", "orc_levmar", "orc_mcmc",
                     "orc_bic_aic", "orc_predicted"):
            getattr(self.lib, name).restype = C.c_int
        self.lib.orc_max_threads.restype = C.c_int

    def max_threads(self):
        return self.lib.orc_max_threads()

    def _fix(self, fixp, nvox):
        if fixp is None:
            fixp = np.zeros((nvox, self.fixp_tsize))
        return _arr(fixp).reshape(nvox, self.fixp_tsize)

    def signal(self, params, cfp, fixp=None, jac=False, prec=0, threads=0):
        params = _arr(params)
        nvox = params.shape[0]
        cfp = _arr(cfp)
        nmeas = cfp.shape[0]
        fixp = self._fix(fixp, nvox)
        S = np.zeros((nvox, nmeas))
        J = np.zeros((nvox, nmeas, self.nparams)) if jac else None
        self.lib.orc_signal(prec, nvox, nmeas, _ptr(params), _ptr(cfp), _ptr(fixp), _ptr(S),
                            _ptr(J), threads)
        return (S, J) if jac else S

    def cost(self, meas, params, cfp, fixp=None, prec=0, threads=0):
        meas = _arr(meas)
        params = _arr(params)
        cfp = _arr(cfp)
        nvox, nmeas = meas.shape
        fixp = self._fix(fixp, nvox)
        out = np.zeros(nvox)
        self.lib.orc_cost(prec, nvox, nmeas, _ptr(meas), _ptr(params), _ptr(cfp), _ptr(fixp),
                          _ptr(out), threads)
        return out

    def gridsearch(self, cfg, meas, params, cfp, fixp=None, prec=0, threads=0):
        meas = _arr(meas)
        params = _arr(params).copy()
        cfp = _arr(cfp)
        nvox, nmeas = meas.shape
        fixp = self._fix(fixp, nvox)
        best = np.zeros(nvox, dtype=np.int32)
        bc = np.zeros(nvox)
        c = cfg.struct if hasattr(cfg, "struct") else cfg
        self.lib.orc_gridsearch(prec, C.byref(c), nvox, nmeas, _ptr(meas), _ptr(params), _ptr(cfp),
                                _ptr(fixp), _ptr(best), _ptr(bc), threads)
        return params, best, bc

    def levmar(self, cfg, meas, params, cfp, fixp=None, prec=0, threads=0):
        meas = _arr(meas)
        params = _arr(params).copy()
        cfp = _arr(cfp)
        nvox, nmeas = meas.shape
        fixp = self._fix(fixp, nvox)
        it = np.zeros(nvox, dtype=np.int32)
        su = np.zeros(nvox, dtype=np.int32)
        co = np.zeros(nvox)
        c = cfg.struct if hasattr(cfg, "struct") else cfg
        self.lib.orc_levmar(prec, C.byref(c), nvox, nmeas, _ptr(meas), _ptr(params), _ptr(cfp),
                            _ptr(fixp), _ptr(it), _ptr(su), _ptr(co), threads)
        return params, it, su, co

    def mcmc(self, cfg, meas, params, cfp, fixp=None, prec=0, threads=0, voxel_offset=0):
        meas = _arr(meas)
        params = _arr(params).copy()
        cfp = _arr(cfp)
        nvox, nmeas = meas.shape
        fixp = self._fix(fixp, nvox)
        c = cfg.struct if hasattr(cfg, "struct") else cfg
        ns = c.njumps // c.sampleevery
        samples = np.zeros((nvox, self.nparams, ns))
        tau = np.zeros((nvox, ns)) if c.rician else None
        self.lib.orc_mcmc(prec, C.byref(c), nvox, nmeas, _ptr(meas), _ptr(params), _ptr(cfp),
                          _ptr(fixp), _ptr(samples), _ptr(tau), C.c_uint32(voxel_offset), threads)
        return params, samples, tau

    def bic_aic(self, meas, samples, cfp, fixp=None, tau=None, rician=False, prec=0, threads=0):
        meas = _arr(meas)
        samples = _arr(samples)
        cfp = _arr(cfp)
        nvox, nmeas = meas.shape
        ns = samples.shape[-1] if samples.ndim == 3 else 1
        fixp = self._fix(fixp, nvox)
        bic = np.zeros(nvox)
        aic = np.zeros(nvox)
        tau = None if tau is None else _arr(tau)
        self.lib.orc_bic_aic(prec, int(rician), nvox, nmeas, ns, _ptr(meas), _ptr(samples),
                             _ptr(cfp), _ptr(fixp), _ptr(tau), _ptr(bic), _ptr(aic), threads)
        return bic, aic

    def predicted(self, samples, cfp, fixp=None, prec=0, threads=0):
        samples = _arr(samples)
        cfp = _arr(cfp)
        nvox = samples.shape[0]
        ns = samples.shape[-1] if samples.ndim == 3 else 1
        nmeas = cfp.shape[0]
        fixp = self._fix(fixp, nvox)
        pred = np.zeros((nvox, nmeas))
        self.lib.orc_predicted(prec, nvox, nmeas, ns, _ptr(samples), _ptr(cfp), _ptr(fixp),
                               _ptr(pred), threads)
        return pred
