"""cdm_levmar_noalloc: the LM entry point for hosts that may not allocate
device memory from inside the library (fixed pipeline memory budgets, or a
framework that owns all device memory). It must give the same fits as
cdm_levmar, call after call, while its working memory is one fixed array
that the calls share.

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from tests.helpers import angle_deg, oracle, watson

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.cdm_levmar_noalloc
    f.argtypes = [C.POINTER(capi.CfgStruct), C.c_int, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 5
    f.restype = C.c_int
    return f


def _agree(o, wl, sl, a, b):
    """The LM parity tolerance of the other tests: cost within 1e-4
    relative, fibre orientation within 0.5 degrees."""
    ca = o.cost(wl.meas[sl], a, wl.cfp, wl.fixp[sl])
    cb = o.cost(wl.meas[sl], b, wl.cfp, wl.fixp[sl])
    rel = np.abs(ca - cb) / ca
    ang = angle_deg(a[:, 3], a[:, 4], b[:, 3], b[:, 4])
    return np.all(rel <= 1e-4) and np.all(ang <= 0.5)


def test_levmar_noalloc_matches_levmar_twice(built, cuda):
    wl = watson(3000, seed=5)
    o = oracle("NODDI_Watson")
    cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid, lanes_levmar=8)
    start, _, _ = o.gridsearch(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    ctx = capi.Cudimot("NODDI_Watson", cfg)
    fn = _noalloc(ctx.lib)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=cuda)  # noqa
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = lambda x: C.c_void_p(x.data_ptr())  # noqa
    # two calls in a row on different voxel sets (the second reuses the
    # scratch the first left behind)
    for sl in (slice(0, 3000), slice(700, 2100)):
        meas, cfp, fixp = t(wl.meas[sl]), t(wl.cfp), t(wl.fixp[sl])
        ref = t(start[sl])
        ctx.levmar(meas, ref, cfp, fixp)
        got = t(start[sl])
        st = fn(C.byref(cfg.struct), got.shape[0], wl.nmeas, 4, 1, ptr(meas), ptr(got), ptr(cfp),
                ptr(fixp), stream)
        assert st == 0, ctx.lib.cdm_last_error()
        torch.cuda.synchronize()
        assert _agree(o, wl, sl, ref.cpu().numpy(), got.cpu().numpy())


def test_levmar_noalloc_rejects_oversize(built, cuda):
    cfg = capi.model_cfg("NODDI_Watson")
    lib = capi.load_library("NODDI_Watson")
    fn = _noalloc(lib)
    # 100k voxels x 288 measurements need ~115 MB > the 16 MiB scratch;
    # rejected before any pointer is used.
    st = fn(C.byref(cfg.struct), 100_000, 288, 4, 1, None, None, None, None, None)
    assert st == 1  # CDM_BAD_ARG
    assert b"16777216" in lib.cdm_last_error()
