"""Failure detection of the bounded device waits, without a GPU fault.

Every mbarrier wait in the fitting kernels gives up after a time limit,
records a device error and lets its CTA return. cdm_selftest_wait_timeout
launches a kernel whose wait can never complete (an mbarrier that expects
an arrival nobody makes; no copy is in flight), so the limit runs out. The
next cdm_synchronize must report CDM_TIMEOUT and clear the error, and the
same context must then fit normally.
"""
import time

import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from tests.helpers import b1s, oracle

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def test_wait_runs_out_then_context_usable(built, cuda):
    cfg = capi.model_cfg("Ball_1_Stick")
    lib = capi.Cudimot("Ball_1_Stick", cfg)
    t0 = time.perf_counter()
    lib.selftest_wait_timeout(50)
    with pytest.raises(capi.CdmError, match="TIMEOUT"):
        lib.synchronize(timeout_ms=5000)
    took = time.perf_counter() - t0
    assert 0.04 <= took < 5.0, took
    # the error word was cleared: a second synchronize is clean
    lib.synchronize(timeout_ms=5000)
    assert lib.stats().device_errors == 0

    wl = b1s(2000)
    params = T(wl.init, cuda)
    lib.levmar(T(wl.meas, cuda), params, T(wl.cfp, cuda), T(wl.fixp, cuda))
    lib.synchronize(timeout_ms=60000)
    got = params.cpu().numpy()
    o = oracle("Ball_1_Stick")
    ref, _, _, _ = o.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    c_got = o.cost(wl.meas, got, wl.cfp, wl.fixp)
    c_ref = o.cost(wl.meas, ref, wl.cfp, wl.fixp)
    assert np.mean((c_got - c_ref) / c_ref <= 1e-4) >= 0.995


def test_selftest_rejects_bad_limit(built, cuda):
    lib = capi.Cudimot("Ball_1_Stick", capi.model_cfg("Ball_1_Stick"))
    for bad in (0, 2001):
        with pytest.raises(capi.CdmError, match="BAD_ARG"):
            lib.selftest_wait_timeout(bad)
