"""ctypes mirror of include/cudimot_gb300.h and a thin Python host layer.

`Cudimot(model)` loads libcudimot_<model>.so (built in-tree by
cudimot_gb300/build.py) and exposes the same operations as CUDIMOT's method
classes (GridSearch, Levenberg_Marquardt, MCMC, BIC_AIC,
getPredictedSignal) on torch CUDA tensors, plus the fused fit. Torch only
provides device memory and streams; all work runs in the library's kernels.
There is no CPU fallback: without a GPU or without the library the calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "_lib")

CDM_MAX_PARAMS = 32
CDM_MAX_BLOCKS = 16

NOBOUNDS, BMIN, BMAX, BMINMAX = 0, 1, 2, 3
NOPRIOR, GAUSSPRIOR, GAMMAPRIOR, ARDPRIOR, SINPRIOR, CUSTOM = 0, 1, 2, 3, 4, 5

STATUS = {0: "OK", 1: "BAD_ARG", 2: "CUDA_ERROR", 3: "TIMEOUT", 4: "NOT_SUPPORTED",
          5: "IO_ERROR"}


class ModelInfo(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("nparams", C.c_int), ("ncfp", C.c_int),
                ("nfixp", C.c_int), ("cfp_size", C.c_int * CDM_MAX_BLOCKS),
                ("fixp_size", C.c_int * CDM_MAX_BLOCKS), ("cfp_tsize", C.c_int),
                ("fixp_tsize", C.c_int), ("derived_cfp", C.c_int), ("derived_p", C.c_int)]


class CfgStruct(C.Structure):
    _fields_ = [
        ("nparams", C.c_int),
        ("bound_types", C.c_int * CDM_MAX_PARAMS),
        ("bounds_min", C.c_double * CDM_MAX_PARAMS),
        ("bounds_max", C.c_double * CDM_MAX_PARAMS),
        ("prior_types", C.c_int * CDM_MAX_PARAMS),
        ("priors_a", C.c_double * CDM_MAX_PARAMS),
        ("priors_b", C.c_double * CDM_MAX_PARAMS),
        ("fixed", C.c_int * CDM_MAX_PARAMS),
        ("n_grid_params", C.c_int),
        ("grid_params", C.c_int * CDM_MAX_PARAMS),
        ("grid_combs", C.c_int),
        ("grid", C.POINTER(C.c_double)),
        ("run_gridsearch", C.c_int),
        ("run_levmar", C.c_int),
        ("run_mcmc", C.c_int),
        ("iter_levmar", C.c_int),
        ("marquardt", C.c_int),
        ("nburn", C.c_int),
        ("njumps", C.c_int),
        ("sampleevery", C.c_int),
        ("update_proposal", C.c_int),
        ("rician", C.c_int),
        ("get_predicted", C.c_int),
        ("bic_aic", C.c_int),
        ("seed", C.c_uint64),
        ("id_part", C.c_int),
        ("lanes_gridsearch", C.c_int),
        ("lanes_levmar", C.c_int),
        ("lanes_mcmc", C.c_int),
        ("first_voxel", C.c_int64),
    ]


class Cfg:
    """Python view of cdm_model_cfg that keeps the grid buffer alive."""

    def __init__(self, nparams: int):
        s = CfgStruct()
        s.nparams = nparams
        s.iter_levmar = 200
        s.marquardt = 1
        s.nburn = 1000
        s.njumps = 1250
        s.sampleevery = 25
        s.update_proposal = 1
        s.seed = 8219
        s.run_levmar = 1
        self.struct = s
        self._grid = None

    def __getattr__(self, k):
        return getattr(self.__dict__["struct"], k)

    def __setattr__(self, k, v):
        if k in ("struct", "_grid"):
            object.__setattr__(self, k, v)
        else:
            setattr(self.struct, k, v)

    def set_bounds(self, bounds: dict):
        """bounds: {i: (min or None, max or None)}"""
        for i, (lo, hi) in bounds.items():
            if lo is not None and hi is not None:
                t = BMINMAX
            elif lo is not None:
                t = BMIN
            elif hi is not None:
                t = BMAX
            else:
                t = NOBOUNDS
            self.struct.bound_types[i] = t
            self.struct.bounds_min[i] = 0.0 if lo is None else lo
            self.struct.bounds_max[i] = 0.0 if hi is None else hi

    def set_prior(self, i, kind, a=0.0, b=0.0):
        self.struct.prior_types[i] = kind
        self.struct.priors_a[i] = a
        self.struct.priors_b[i] = b

    def set_grid(self, values: dict):
        """values: {param index: sequence}; lowest index outermost
        (CUDIMOT's set_grid, Model.cu:371-393)."""
        ids = sorted(k for k, v in values.items() if len(v))
        axes = [np.asarray(values[i], dtype=np.float64) for i in ids]
        if not ids:
            self.struct.n_grid_params = 0
            self.struct.grid_combs = 0
            self.struct.run_gridsearch = 0
            return
        mesh = np.meshgrid(*axes, indexing="ij")
        grid = np.ascontiguousarray(np.stack([m.reshape(-1) for m in mesh], axis=1))
        self._grid = grid
        self.struct.n_grid_params = len(ids)
        for k, i in enumerate(ids):
            self.struct.grid_params[k] = i
        self.struct.grid_combs = grid.shape[0]
        self.struct.grid = grid.ctypes.data_as(C.POINTER(C.c_double))
        self.struct.run_gridsearch = 1

    @property
    def grid_array(self):
        return self._grid


def make_cfg(nparams, bounds=None, priors=None, fixed=(), grid=None, **opts) -> Cfg:
    c = Cfg(nparams)
    if bounds:
        c.set_bounds(bounds)
    for i, pr in (priors or {}).items():
        c.set_prior(i, *pr)
    for i in fixed:
        c.struct.fixed[i] = 1
    if grid:
        c.set_grid(grid)
    for k, v in opts.items():
        setattr(c.struct, k, v)
    return c


# Bounds and priors of the shipped plugins' modelpriors files.
MODEL_LIMITS = {
    "Ball_1_Stick": dict(bounds={0: (1e-9, None), 1: (1e-9, 0.01), 2: (0.01, 1.0),
                                 3: (-100.0, 100.0), 4: (-100.0, 100.0)},
                         priors={3: (SINPRIOR,)}),
    "NODDI_Watson": dict(bounds={0: (0.0, 1.0), 1: (0.0, 1.0), 2: (0.0, 64.0),
                                 3: (-100.0, 100.0), 4: (-100.0, 100.0)},
                         priors={3: (SINPRIOR,)}),
    "DiffusionTensor": dict(bounds={0: (0.1, 10000.0), 1: (0.0, 0.01), 2: (None, None),
                                    3: (None, None), 4: (0.0, 0.01), 5: (None, None),
                                    6: (0.0, 0.01)},
                            priors={}),
    "Ball_2_Sticks": dict(bounds={0: (0.0, 10000.0), 1: (0.0, 0.01), 2: (0.0, 1.0),
                                  3: (-100.0, 100.0), 4: (-100.0, 100.0), 5: (0.0, 1.0),
                                  6: (-100.0, 100.0), 7: (-100.0, 100.0)},
                          priors={3: (SINPRIOR,), 5: (ARDPRIOR, 1.0), 6: (SINPRIOR,)}),
    # CUDIMOT's modelpriors writes "priors[4]=sin()", which its parser ignores
    "NODDI_Bingham": dict(bounds={0: (0.0, 1.0), 1: (0.0, 1.0), 2: (0.1, 64.0), 3: (0.01, 32.0),
                                  4: (-10000.0, 10000.0), 5: (-10000.0, 10000.0),
                                  6: (-100.0, 100.0)},
                          priors={}),
    # two of CUDIMOT's plugins used unchanged (no copy in mymodels/)
    "toymodel": dict(bounds={0: (None, None), 1: (None, None)}, priors={}),
    "Ball_2_Sticks_1Shell_SSFP": dict(
        bounds={0: (1e-9, 0.01), 1: (0.0, 1.0), 2: (-100.0, 100.0), 3: (-100.0, 100.0),
                4: (0.0, 1.0), 5: (-100.0, 100.0), 6: (-100.0, 100.0), 7: (0.0, None)},
        priors={2: (SINPRIOR,), 4: (ARDPRIOR, 1.0), 5: (SINPRIOR,)}),
}


def model_cfg(model: str, **opts) -> Cfg:
    lim = MODEL_LIMITS[model]
    nparams = len(lim["bounds"])
    return make_cfg(nparams, bounds=lim["bounds"], priors=lim["priors"], **opts)


class CdmError(RuntimeError):
    pass


class Stats(C.Structure):
    _fields_ = [("gs_recheck_voxels", C.c_int64), ("lm_iterations", C.c_int64),
                ("lm_successes", C.c_int64), ("device_errors", C.c_int64)]


_vp = C.c_void_p


def _declare(lib):
    i, i64 = C.c_int, C.c_int64
    sigs = {
        "cdm_get_model_info": [C.POINTER(ModelInfo)],
        "cdm_default_cfg": [C.POINTER(CfgStruct)],
        "cdm_parse_priors": [C.c_char_p, C.POINTER(CfgStruct), _vp, C.POINTER(i)],
        "cdm_parse_grid": [C.c_char_p, C.POINTER(i), _vp, C.POINTER(i), _vp, i64],
        "cdm_parse_fixed": [C.c_char_p, _vp],
        "cdm_read_cfp_list": [C.c_char_p, i, _vp],
        "cdm_create": [C.POINTER(CfgStruct), C.POINTER(_vp)],
        "cdm_destroy": [_vp],
        "cdm_gridsearch": [_vp, i, i, i, i, _vp, _vp, _vp, _vp, _vp],
        "cdm_levmar": [_vp, i, i, i, i, _vp, _vp, _vp, _vp, _vp],
        "cdm_mcmc": [_vp, i, i, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_bic_aic": [_vp, i, i, i, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_predicted_signal": [_vp, i, i, i, i, i, _vp, _vp, _vp, _vp, _vp],
        "cdm_fit": [_vp, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_fit_host": [_vp, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, i, i64],
        "cdm_clean_signals": [i, i, _vp, _vp],
        "cdm_selftest_wait_timeout": [_vp, i, _vp],
        "cdm_fit_reserve": [_vp, i, i],
        "cdm_mcmc_seeded": [_vp, i, i, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_mcmc_prepare": [_vp, i, i, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_synth_signals": [_vp, i, i, _vp, _vp, _vp, C.c_double, C.c_double, C.c_uint64, i,
                              _vp, _vp, _vp, i, _vp],
        "cdm_mlp_head_info": [C.POINTER(i), C.POINTER(i), _vp],
        "cdm_cost": [_vp, i, i, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_select_worse": [i, _vp, _vp, C.c_double, _vp, _vp, _vp],
        "cdm_rows": [i, _vp, i, _vp, _vp, i, C.c_double, _vp],
        "cdm_mlp_targets": [_vp, i, _vp, _vp, _vp],
        "cdm_mlp_decode": [_vp, i, _vp, i, _vp, _vp, _vp],
        "cdm_fit_enqueue": [_vp, i, i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "cdm_synchronize": [_vp, _vp, i64],
        "cdm_get_stats": [_vp, C.POINTER(Stats)],
        "cdm_levmar_noalloc": [C.POINTER(CfgStruct), i, i, i, i, _vp, _vp, _vp, _vp, _vp],
        "cdm_noalloc_status": [_vp],
    }
    for name, args in sigs.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    lib.cdm_last_error.restype = C.c_char_p
    lib.cdm_last_error.argtypes = []
    lib.cdm_status_string.restype = C.c_char_p
    lib.cdm_status_string.argtypes = [C.c_int]


EXPORTED = ("cdm_get_model_info", "cdm_default_cfg", "cdm_status_string", "cdm_last_error",
            "cdm_parse_priors", "cdm_parse_grid", "cdm_parse_fixed", "cdm_read_cfp_list",
            "cdm_create", "cdm_destroy", "cdm_gridsearch", "cdm_levmar", "cdm_mcmc",
            "cdm_bic_aic", "cdm_predicted_signal", "cdm_fit", "cdm_fit_host",
            "cdm_fit_reserve", "cdm_fit_enqueue", "cdm_synchronize", "cdm_get_stats",
            "cdm_mcmc_seeded", "cdm_synth_signals", "cdm_mlp_head_info", "cdm_mlp_targets",
            "cdm_mlp_decode", "cdm_cost", "cdm_select_worse", "cdm_rows", "cdm_clean_signals",
            "cdm_selftest_wait_timeout", "cdm_levmar_noalloc", "cdm_noalloc_status")


def lib_path(model: str) -> str:
    return os.path.join(LIBDIR, f"libcudimot_{model}.so")


def load_library(model: str, path: str = None):
    """Load libcudimot_<model>.so (or the library at path); raises if it has
    not been built."""
    path = path or lib_path(model)
    if not os.path.exists(path):
        raise CdmError(f"{path} is not built (python -m cudimot_gb300.build)")
    lib = C.CDLL(path)
    _declare(lib)
    return lib


def _check(lib, status, what):
    if status != 0:
        msg = lib.cdm_last_error().decode(errors="replace")
        raise CdmError(f"{what}: {STATUS.get(status, status)}: {msg}")


def _dptr(t):
    """Device pointer of a torch CUDA tensor (float64, contiguous) or None."""
    if t is None:
        return None
    import torch
    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise CdmError("expected a contiguous float64 CUDA tensor")
    return C.c_void_p(t.data_ptr())


class Cudimot:
    """A fitting context for one model (CUDIMOT's method objects in one).

    Stage calls take torch CUDA float64 tensors in CUDIMOT's layouts and run
    asynchronously on the current torch stream."""

    def __init__(self, model: str, cfg: Cfg, path: str = None):
        self.model = model
        self.lib = load_library(model, path)
        self.info = ModelInfo()
        _check(self.lib, self.lib.cdm_get_model_info(C.byref(self.info)), "model info")
        self.cfg = cfg
        ctx = C.c_void_p()
        _check(self.lib, self.lib.cdm_create(C.byref(cfg.struct), C.byref(ctx)), "cdm_create")
        self.ctx = ctx

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.cdm_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nparams(self):
        return self.info.nparams

    def _stream(self):
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _sizes(self, meas):
        return meas.shape[0], meas.shape[1], self.info.cfp_tsize, self.info.fixp_tsize

    def gridsearch(self, meas, params, cfp, fixp):
        nv, nm, ct, ft = self._sizes(meas)
        _check(self.lib, self.lib.cdm_gridsearch(self.ctx, nv, nm, ct, ft, _dptr(meas), _dptr(params),
                                                 _dptr(cfp), _dptr(fixp), self._stream()), "gridsearch")

    def levmar(self, meas, params, cfp, fixp):
        nv, nm, ct, ft = self._sizes(meas)
        _check(self.lib, self.lib.cdm_levmar(self.ctx, nv, nm, ct, ft, _dptr(meas), _dptr(params),
                                             _dptr(cfp), _dptr(fixp), self._stream()), "levmar")

    def mcmc(self, meas, params, cfp, fixp, samples, tau=None):
        nv, nm, ct, ft = self._sizes(meas)
        _check(self.lib, self.lib.cdm_mcmc(self.ctx, nv, nm, ct, ft, _dptr(meas), _dptr(params),
                                           _dptr(cfp), _dptr(fixp), _dptr(samples), _dptr(tau),
                                           self._stream()), "mcmc")

    def bic_aic(self, meas, samples, cfp, fixp, bic, aic, tau=None):
        nv, nm, ct, ft = self._sizes(meas)
        ns = samples.shape[-1] if samples.dim() == 3 else 1
        _check(self.lib, self.lib.cdm_bic_aic(self.ctx, nv, nm, ns, ct, ft, _dptr(meas), _dptr(samples),
                                              _dptr(cfp), _dptr(fixp), _dptr(bic), _dptr(aic),
                                              _dptr(tau), self._stream()), "bic_aic")

    def predicted_signal(self, samples, cfp, fixp, pred):
        nv, nm = pred.shape
        ns = samples.shape[-1] if samples.dim() == 3 else 1
        _check(self.lib, self.lib.cdm_predicted_signal(
            self.ctx, nv, nm, ns, self.info.cfp_tsize, self.info.fixp_tsize, _dptr(samples),
            _dptr(cfp), _dptr(fixp), _dptr(pred), self._stream()), "predicted_signal")

    def fit(self, meas, params, cfp, fixp, samples, tau=None, pred=None, bic=None, aic=None):
        nv, nm = meas.shape
        _check(self.lib, self.lib.cdm_fit(self.ctx, nv, nm, _dptr(meas), _dptr(params), _dptr(cfp),
                                          _dptr(fixp), _dptr(samples), _dptr(tau), _dptr(pred),
                                          _dptr(bic), _dptr(aic), self._stream()), "fit")

    def fit_host(self, meas, params, cfp, fixp, samples, tau=None, pred=None, bic=None, aic=None,
                 part_size=0, timeout_ms=-1):
        """numpy float64 arrays (params/samples/... written in place)."""
        def p(a):
            return None if a is None else a.ctypes.data_as(C.c_void_p)
        nv, nm = meas.shape
        _check(self.lib, self.lib.cdm_fit_host(self.ctx, nv, nm, p(meas), p(params), p(cfp), p(fixp),
                                               p(samples), p(tau), p(pred), p(bic), p(aic),
                                               part_size, timeout_ms), "fit_host")

    def selftest_wait_timeout(self, limit_ms=50):
        """cdm_selftest_wait_timeout on the current torch stream."""
        _check(self.lib, self.lib.cdm_selftest_wait_timeout(self.ctx, limit_ms, self._stream()),
               "selftest_wait_timeout")

    def clean_signals(self, meas):
        """cdm_clean_signals in place on a CUDA float64 [nvox][nmeas] tensor."""
        nv, nm = meas.shape
        _check(self.lib, self.lib.cdm_clean_signals(nv, nm, _dptr(meas), self._stream()),
               "clean_signals")

    def mcmc_seeded(self, meas, params, cfp, fixp, samples, prop_sd, tau=None):
        nv, nm, ct, ft = self._sizes(meas)
        _check(self.lib, self.lib.cdm_mcmc_seeded(self.ctx, nv, nm, ct, ft, _dptr(meas), _dptr(params),
                                                  _dptr(cfp), _dptr(fixp), _dptr(samples), _dptr(tau),
                                                  _dptr(prop_sd), self._stream()), "mcmc_seeded")

    def synth(self, cfp, params, fixp, snr=(20.0, 20.0), seed=1, b_col=3, meas=None, s0=None,
              x=None):
        """Synthetic noisy signals from the plugin (see cdm_synth_signals);
        x is a bf16 CUDA tensor [nvox][x_ld]."""
        nv = params.shape[0]
        nm = cfp.shape[0]
        xp = None if x is None else C.c_void_p(x.data_ptr())
        _check(self.lib, self.lib.cdm_synth_signals(
            self.ctx, nv, nm, _dptr(cfp), _dptr(params), _dptr(fixp), float(snr[0]), float(snr[1]),
            int(seed), b_col, _dptr(meas), _dptr(s0), xp, 0 if x is None else x.shape[1],
            self._stream()), "synth_signals")

    def cost(self, meas, params, cfp, fixp, out):
        nv, nm = meas.shape
        _check(self.lib, self.lib.cdm_cost(self.ctx, nv, nm, _dptr(meas), _dptr(params), _dptr(cfp),
                                           _dptr(fixp), _dptr(out), self._stream()), "cost")

    def select_worse(self, cost, ref, margin, idx, count):
        """idx, count: int32 CUDA tensors ([n], [1])."""
        _check(self.lib, self.lib.cdm_select_worse(cost.shape[0], _dptr(cost), _dptr(ref), float(margin),
                                                   C.c_void_p(idx.data_ptr()),
                                                   C.c_void_p(count.data_ptr()), self._stream()),
               "select_worse")

    def rows(self, nsel, idx, src, dst, mode, value=0.0):
        ncols = dst.shape[1]
        _check(self.lib, self.lib.cdm_rows(nsel, C.c_void_p(idx.data_ptr()), ncols, _dptr(src),
                                           _dptr(dst), mode, float(value), self._stream()), "rows")

    def mlp_head(self):
        n_mu, n_sig = C.c_int(), C.c_int()
        g = (C.c_int * 16)()
        _check(self.lib, self.lib.cdm_mlp_head_info(C.byref(n_mu), C.byref(n_sig),
                                                    C.cast(g, C.c_void_p)), "mlp_head_info")
        return n_mu.value, n_sig.value, list(g)[:n_mu.value]

    def mlp_targets(self, params, targets):
        _check(self.lib, self.lib.cdm_mlp_targets(self.ctx, params.shape[0], _dptr(params),
                                                  C.c_void_p(targets.data_ptr()), self._stream()),
               "mlp_targets")

    def mlp_decode(self, out, params, prop_sd=None):
        _check(self.lib, self.lib.cdm_mlp_decode(self.ctx, out.shape[0], C.c_void_p(out.data_ptr()),
                                                 out.shape[1], _dptr(params), _dptr(prop_sd),
                                                 self._stream()), "mlp_decode")

    def fit_reserve(self, nvox, nmeas):
        """Allocate the scratch buffers of a fit of this shape now."""
        _check(self.lib, self.lib.cdm_fit_reserve(self.ctx, nvox, nmeas), "fit_reserve")

    def fit_enqueue(self, meas, params, cfp, fixp, samples, tau=None, pred=None, bic=None, aic=None):
        """The stage sequence as plain launches on the current stream."""
        nv, nm = meas.shape
        _check(self.lib, self.lib.cdm_fit_enqueue(self.ctx, nv, nm, _dptr(meas), _dptr(params),
                                                  _dptr(cfp), _dptr(fixp), _dptr(samples),
                                                  _dptr(tau), _dptr(pred), _dptr(bic), _dptr(aic),
                                                  self._stream()), "fit_enqueue")

    def synchronize(self, timeout_ms=-1):
        _check(self.lib, self.lib.cdm_synchronize(self.ctx, self._stream(), timeout_ms), "synchronize")

    def stats(self):
        s = Stats()
        _check(self.lib, self.lib.cdm_get_stats(self.ctx, C.byref(s)), "stats")
        return s


def parse_priors(model: str, path: str, nparams: int):
    """modelpriors file -> (Cfg, p_init or None) through the library's parser."""
    lib = load_library(model)
    cfg = Cfg(nparams)
    _check(lib, lib.cdm_default_cfg(C.byref(cfg.struct)), "default cfg")
    p_init = (C.c_double * CDM_MAX_PARAMS)()
    given = C.c_int(0)
    _check(lib, lib.cdm_parse_priors(path.encode(), C.byref(cfg.struct), C.cast(p_init, C.c_void_p),
                                     C.byref(given)), "parse_priors")
    return cfg, (list(p_init)[:nparams] if given.value else None)


class Batch:
    """Several fits - any mix of models, protocols and volumes - recorded as
    parallel branches of one CUDA graph (include/cdm_batch.h) and launched
    together on the current torch stream."""

    def __init__(self):
        path = os.path.join(LIBDIR, "libcdm_batch.so")
        if not os.path.exists(path):
            raise CdmError(f"{path} is not built (python -m cudimot_gb300.build)")
        self.lib = C.CDLL(path)
        vp, i = C.c_void_p, C.c_int
        self.lib.cdm_batch_create.argtypes = [C.POINTER(vp)]
        self.lib.cdm_batch_destroy.argtypes = [vp]
        self.lib.cdm_batch_add.argtypes = [vp, vp, vp, vp, i, i] + [vp] * 9 + [C.c_double]
        self.lib.cdm_batch_run.argtypes = [vp, vp]
        self.lib.cdm_batch_last_error.restype = C.c_char_p
        for f in ("cdm_batch_create", "cdm_batch_destroy", "cdm_batch_add", "cdm_batch_run"):
            getattr(self.lib, f).restype = C.c_int
        h = C.c_void_p()
        self._check(self.lib.cdm_batch_create(C.byref(h)), "create")
        self.h = h
        self._keep = []

    def _check(self, status, what):
        if status != 0:
            raise CdmError(f"batch {what}: {STATUS.get(status, status)}: "
                           f"{self.lib.cdm_batch_last_error().decode(errors='replace')}")

    def add(self, fit: Cudimot, meas, params, cfp, fixp, samples, tau=None, pred=None, bic=None,
            aic=None, work=0.0):
        nv, nm = meas.shape
        self._keep.append((fit, meas, params, cfp, fixp, samples, tau, pred, bic, aic))
        reserve = C.cast(fit.lib.cdm_fit_reserve, C.c_void_p)
        enqueue = C.cast(fit.lib.cdm_fit_enqueue, C.c_void_p)
        self._check(self.lib.cdm_batch_add(self.h, reserve, enqueue, fit.ctx, nv, nm, _dptr(meas),
                                           _dptr(params), _dptr(cfp), _dptr(fixp), _dptr(samples),
                                           _dptr(tau), _dptr(pred), _dptr(bic), _dptr(aic),
                                           float(work)), "add")

    def run(self):
        import torch
        self._check(self.lib.cdm_batch_run(self.h, C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                    "run")

    def close(self):
        if getattr(self, "h", None):
            self.lib.cdm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
