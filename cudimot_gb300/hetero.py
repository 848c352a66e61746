"""Several fits' MCMC in one persistent launch (include/cdm_hetero.h).

    h = Hetero()                                   # libcdm_hetero_default.so
    works = [h.prepare(ctx, meas, params, cfp, fixp, samples) for ctx, ... in fits]
    h.mcmc(works)                                  # one launch for all of them

`prepare` runs a fit's own library up to its MCMC launch
(cdm_mcmc_prepare); `mcmc` runs every prepared fit's tiles in one launch of
the multi-model kernel, whose CTAs take tiles from a device counter across
fits, models and protocols. No counterpart in CUDIMOT, which fits one model
per process (cudimot.cc:57-125).
"""
from __future__ import annotations

import ctypes as C
import os

from . import build, capi


class TileWork(C.Structure):
    """cdm_tile_work (include/cdm_hetero.h)."""
    _fields_ = [("model", C.c_char * 64), ("eval_double", C.c_int), ("threads", C.c_int),
                ("lanes", C.c_int), ("rician", C.c_int), ("ntiles", C.c_int),
                ("smem_bytes", C.c_uint32), ("scratch_bytes", C.c_uint32),
                ("args_bytes", C.c_uint32), ("err", C.c_void_p), ("args", C.c_ubyte * 1024)]


EXPORTED = ("cdm_hetero_create", "cdm_hetero_destroy", "cdm_hetero_models", "cdm_hetero_mcmc",
            "cdm_hetero_last_grid", "cdm_hetero_last_launches", "cdm_hetero_last_error")


def load(tag: str = "default", path: str = None):
    path = path or build.hetero_lib_path(tag)
    if not os.path.exists(path):
        raise capi.CdmError(f"{path} is not built (cudimot_gb300.build.build_hetero)")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.cdm_hetero_create.argtypes = [C.POINTER(vp)]
    lib.cdm_hetero_destroy.argtypes = [vp]
    lib.cdm_hetero_models.argtypes = [C.c_char_p, C.c_size_t]
    lib.cdm_hetero_models.restype = C.c_size_t
    lib.cdm_hetero_mcmc.argtypes = [vp, C.c_int, C.POINTER(TileWork), vp]
    lib.cdm_hetero_last_grid.argtypes = [vp]
    lib.cdm_hetero_last_launches.argtypes = [vp]
    lib.cdm_hetero_last_error.restype = C.c_char_p
    for n in ("cdm_hetero_create", "cdm_hetero_destroy", "cdm_hetero_mcmc", "cdm_hetero_last_grid",
              "cdm_hetero_last_launches"):
        getattr(lib, n).restype = C.c_int
    return lib


class Hetero:
    def __init__(self, tag: str = "default", path: str = None):
        self.lib = load(tag, path)
        h = C.c_void_p()
        st = self.lib.cdm_hetero_create(C.byref(h))
        if st != 0:
            raise capi.CdmError(f"cdm_hetero_create: {capi.STATUS.get(st, st)}: "
                                f"{self.lib.cdm_hetero_last_error().decode(errors='replace')}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.cdm_hetero_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def models(self) -> str:
        n = self.lib.cdm_hetero_models(None, 0)
        buf = C.create_string_buffer(n + 1)
        self.lib.cdm_hetero_models(buf, n + 1)
        return buf.value.decode()

    @staticmethod
    def prepare(ctx: "capi.Cudimot", meas, params, cfp, fixp, samples, tau=None) -> TileWork:
        """The fit's MCMC up to its launch, on the current torch stream."""
        w = TileWork()
        nv, nm, ct, ft = ctx._sizes(meas)
        capi._check(ctx.lib, ctx.lib.cdm_mcmc_prepare(
            ctx.ctx, nv, nm, ct, ft, capi._dptr(meas), capi._dptr(params), capi._dptr(cfp),
            capi._dptr(fixp), capi._dptr(samples), capi._dptr(tau), ctx._stream(), C.byref(w)),
            "mcmc_prepare")
        return w

    def mcmc(self, works):
        """One persistent launch over every prepared fit, on the current
        torch stream."""
        import torch
        arr = (TileWork * max(len(works), 1))(*works)
        st = self.lib.cdm_hetero_mcmc(self.h, len(works), arr,
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st != 0:
            raise capi.CdmError(f"cdm_hetero_mcmc: {capi.STATUS.get(st, st)}: "
                                f"{self.lib.cdm_hetero_last_error().decode(errors='replace')}")

    @property
    def last_grid(self) -> int:
        return self.lib.cdm_hetero_last_grid(self.h)

    @property
    def last_launches(self) -> int:
        return self.lib.cdm_hetero_last_launches(self.h)
