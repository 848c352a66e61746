"""cdm_levmar_noalloc: the LM entry point for hosts that may not allocate
device memory from inside the library (fixed pipeline memory budgets, or a
framework that owns all device memory). It must give the same fits as
cdm_levmar, call after call, while its working memory is one fixed array
that the calls share; and a bounded wait that runs out inside it must be
visible to the caller through cdm_noalloc_status.

Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from tests.helpers import angle_deg, oracle, watson

pytestmark = pytest.mark.gpu

CDM_OK, CDM_BAD_ARG, CDM_TIMEOUT = 0, 1, 3


def _agree(o, wl, sl, a, b):
    """The LM parity tolerance of the other tests: cost within 1e-4
    relative, fibre orientation within 0.5 degrees."""
    ca = o.cost(wl.meas[sl], a, wl.cfp, wl.fixp[sl])
    cb = o.cost(wl.meas[sl], b, wl.cfp, wl.fixp[sl])
    rel = np.abs(ca - cb) / ca
    ang = angle_deg(a[:, 3], a[:, 4], b[:, 3], b[:, 4])
    return np.all(rel <= 1e-4) and np.all(ang <= 0.5)


def _t(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)


def _ptr(x):
    return C.c_void_p(None if x is None else x.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _call(lib, cfg, meas, params, cfp, fixp, nmeas):
    return lib.cdm_levmar_noalloc(C.byref(cfg.struct), params.shape[0], nmeas, 4, 1, _ptr(meas),
                                  _ptr(params), _ptr(cfp), _ptr(fixp), _stream())


@pytest.mark.parametrize("lanes", [8, 0])
def test_levmar_noalloc_matches_levmar_twice(built, cuda, lanes):
    """Two calls in a row on different voxel sets (the second reuses the
    scratch the first left behind), with an explicit lane count and with
    the default rule (lanes_levmar = 0): the same kernel on the same inputs
    as cdm_levmar, so the fits are identical."""
    wl = watson(3000, seed=5)
    o = oracle("NODDI_Watson")
    cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid, lanes_levmar=lanes)
    start, _, _ = o.gridsearch(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    ctx = capi.Cudimot("NODDI_Watson", cfg)
    for sl in (slice(0, 3000), slice(700, 2100)):
        meas, cfp, fixp = _t(wl.meas[sl], cuda), _t(wl.cfp, cuda), _t(wl.fixp[sl], cuda)
        ref = _t(start[sl], cuda)
        ctx.levmar(meas, ref, cfp, fixp)
        got = _t(start[sl], cuda)
        st = _call(ctx.lib, cfg, meas, got, cfp, fixp, wl.nmeas)
        assert st == CDM_OK, ctx.lib.cdm_last_error()
        assert ctx.lib.cdm_noalloc_status(_stream()) == CDM_OK
        assert torch.equal(ref, got)
        assert _agree(o, wl, sl, ref.cpu().numpy(), got.cpu().numpy())


def test_levmar_noalloc_empty_and_oversize(built, cuda):
    lib = capi.load_library("NODDI_Watson")
    cfg = capi.model_cfg("NODDI_Watson")
    wl = watson(4, seed=2)
    # nvox = 0: the protocol is staged, nothing else runs, params untouched
    params = _t(wl.init, cuda)
    before = params.clone()
    cfp = _t(wl.cfp, cuda)
    st = lib.cdm_levmar_noalloc(C.byref(cfg.struct), 0, wl.nmeas, 4, 1, None, _ptr(params),
                                _ptr(cfp), None, _stream())
    assert st == CDM_OK, lib.cdm_last_error()
    assert lib.cdm_noalloc_status(_stream()) == CDM_OK
    assert torch.equal(params, before)
    # 100k voxels x 288 measurements need ~115 MB > the 16 MiB scratch;
    # rejected before any pointer is used.
    st = lib.cdm_levmar_noalloc(C.byref(cfg.struct), 100_000, 288, 4, 1, None, None, None, None,
                                None)
    assert st == CDM_BAD_ARG
    assert b"16777216" in lib.cdm_last_error()


def test_levmar_noalloc_allocates_nothing_and_reports_waits(built, cuda):
    """Device free memory is the same before and after repeated calls (after
    one warm-up call has loaded the kernels), and a bounded wait that runs
    out on the no-allocation error word is reported once by
    cdm_noalloc_status, after which the same entry point fits again."""
    wl = watson(2000, seed=9)
    o = oracle("NODDI_Watson")
    cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid)
    start, _, _ = o.gridsearch(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    lib = capi.load_library("NODDI_Watson")
    meas, cfp, fixp = _t(wl.meas, cuda), _t(wl.cfp, cuda), _t(wl.fixp, cuda)
    fits = [_t(start, cuda) for _ in range(4)]
    assert _call(lib, cfg, meas, fits[0], cfp, fixp, wl.nmeas) == CDM_OK, lib.cdm_last_error()
    assert lib.cdm_noalloc_status(_stream()) == CDM_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for k in (1, 2):
        assert _call(lib, cfg, meas, fits[k], cfp, fixp, wl.nmeas) == CDM_OK, lib.cdm_last_error()
    assert lib.cdm_noalloc_status(_stream()) == CDM_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.equal(fits[0], fits[1]) and torch.equal(fits[1], fits[2])
    # a wait that runs out (50 ms, nothing in flight) on the shared word
    assert lib.cdm_selftest_wait_timeout(None, 50, _stream()) == CDM_OK
    assert lib.cdm_noalloc_status(_stream()) == CDM_TIMEOUT
    assert b"ran out" in lib.cdm_last_error()
    assert lib.cdm_noalloc_status(_stream()) == CDM_OK  # reported once, then cleared
    assert _call(lib, cfg, meas, fits[3], cfp, fixp, wl.nmeas) == CDM_OK, lib.cdm_last_error()
    assert lib.cdm_noalloc_status(_stream()) == CDM_OK
    assert torch.equal(fits[3], fits[0])
    # and the fits improved on their grid-search start
    c_fit = o.cost(wl.meas, fits[3].cpu().numpy(), wl.cfp, wl.fixp)
    c_start = o.cost(wl.meas, start, wl.cfp, wl.fixp)
    assert c_fit.sum() < c_start.sum()
