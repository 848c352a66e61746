"""ctypes wrapper of refharness.cpp: CUDIMOT's own kernels on torch CUDA
tensors (test infrastructure; CUDIMOT's layouts). T = double (the MyType the
plugins ship with) by default; RefKernels(..., real=torch.float32) runs
CUDIMOT's float instantiations, and every array passed is then float32."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "_ref")
_LIB = None
_LOADED = None


def available(model):
    from oracle.refkernels.build_ref_kernels import available as av
    return av(model)


def _lib():
    global _LIB
    if _LIB is None:
        from oracle.refkernels.build_ref_kernels import build_harness
        err = build_harness()
        if err:
            raise RuntimeError(err)
        _LIB = C.CDLL(os.path.join(REF, "librefharness.so"))
        _LIB.ref_last_error.restype = C.c_char_p
    return _LIB


def _p(t):
    return C.c_uint64(0 if t is None else t.data_ptr())


def _arr(v, ct):
    return (ct * len(v))(*v)


class RefKernels:
    def __init__(self, model, nparams, real=None):
        global _LOADED
        import torch
        self.lib = _lib()
        self.np = nparams
        self.real = torch.float64 if real is None else real
        if self.real not in (torch.float64, torch.float32):
            raise ValueError("real must be torch.float64 or torch.float32")
        if _LOADED != model:
            rc = self.lib.ref_load(os.path.join(REF, model).encode())
            if rc:
                raise RuntimeError(self.lib.ref_last_error().decode())
            _LOADED = model

    def _use(self, *arrays):
        """Select T in the harness and check that every array is a T array."""
        for a in arrays:
            if a is not None and a.dtype != self.real:
                raise TypeError(f"expected {self.real} arrays, got {a.dtype}")
        self.lib.ref_set_real(8 if self.real.itemsize == 8 else 4)

    def _check(self, rc, what):
        if rc:
            raise RuntimeError(f"{what}: {rc} {self.lib.ref_last_error().decode()}")

    def _lim(self, cfg):
        s = cfg.struct
        n = self.np
        return (_arr(list(s.bound_types)[:n], C.c_int), _arr(list(s.bounds_min)[:n], C.c_float),
                _arr(list(s.bounds_max)[:n], C.c_float))

    def gridsearch(self, cfg, meas, params, cfp, fixp, grid):
        self._use(meas, params, cfp, fixp, grid)
        bt, bmin, bmax = self._lim(cfg)
        s = cfg.struct
        nv, nm = meas.shape
        rc = self.lib.ref_gridsearch(self.np, nv, nm, cfp.shape[1], fixp.shape[1] if fixp is not None else 0,
                                     _p(meas), _p(params), _p(cfp), _p(fixp), s.n_grid_params,
                                     _arr(list(s.grid_params)[:self.np], C.c_int), s.grid_combs, _p(grid),
                                     bt, bmin, bmax)
        self._check(rc, "ref_gridsearch")

    def levmar(self, cfg, meas, params, cfp, fixp):
        self._use(meas, params, cfp, fixp)
        bt, bmin, bmax = self._lim(cfg)
        s = cfg.struct
        nv, nm = meas.shape
        rc = self.lib.ref_levmar(self.np, nv, nm, cfp.shape[1], fixp.shape[1] if fixp is not None else 0,
                                 _p(meas), _p(params), _p(cfp), _p(fixp), s.iter_levmar, s.marquardt,
                                 bt, bmin, bmax, _arr(list(s.fixed)[:self.np], C.c_int))
        self._check(rc, "ref_levmar")

    def mcmc(self, cfg, meas, params, cfp, fixp, samples, tau=None):
        self._use(meas, params, cfp, fixp, samples, tau)
        bt, bmin, bmax = self._lim(cfg)
        s = cfg.struct
        n = self.np
        nv, nm = meas.shape
        rc = self.lib.ref_mcmc(n, nv, nm, cfp.shape[1], fixp.shape[1] if fixp is not None else 0,
                               _p(meas), _p(params), _p(cfp), _p(fixp), _p(samples), _p(tau),
                               s.nburn, s.njumps, s.sampleevery, s.update_proposal, s.rician,
                               int(s.seed), s.id_part, bt, bmin, bmax,
                               _arr(list(s.prior_types)[:n], C.c_int), _arr(list(s.priors_a)[:n], C.c_float),
                               _arr(list(s.priors_b)[:n], C.c_float), _arr(list(s.fixed)[:n], C.c_int))
        self._check(rc, "ref_mcmc")

    def bic_aic(self, meas, samples, cfp, fixp, bic, aic, tau=None, rician=False):
        self._use(meas, samples, cfp, fixp, bic, aic, tau)
        nv, nm = meas.shape
        ns = samples.shape[-1] if samples.dim() == 3 else 1
        rc = self.lib.ref_bic_aic(self.np, nv, nm, ns, cfp.shape[1], fixp.shape[1] if fixp is not None else 0,
                                  _p(meas), _p(samples), _p(cfp), _p(fixp), _p(bic), _p(aic), _p(tau),
                                  int(rician))
        self._check(rc, "ref_bic_aic")

    def predicted(self, samples, cfp, fixp, pred):
        self._use(samples, cfp, fixp, pred)
        nv, nm = pred.shape
        ns = samples.shape[-1] if samples.dim() == 3 else 1
        rc = self.lib.ref_predicted(self.np, nv, nm, ns, cfp.shape[1], fixp.shape[1] if fixp is not None else 0,
                                    _p(samples), _p(cfp), _p(fixp), _p(pred))
        self._check(rc, "ref_predicted")
