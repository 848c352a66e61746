"""Numerics of the shipped plugins on the host: single-precision error of the
model as the kernels evaluate it (the fp32 number type), the analytic
Watson Jacobian against finite differences of the FP64 model, and the FP32
step rule of the generic numerical derivative."""
import numpy as np
import pytest

from cudimot_gb300 import synth
from tests.helpers import oracle


def watson_draws(n, seed):
    rng = np.random.default_rng(seed)
    cfp = synth.protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], rng)
    k = np.exp(rng.uniform(np.log(1e-4), np.log(64), n))
    P = np.stack([rng.uniform(0, 1, n), rng.uniform(0, 1, n), k, rng.uniform(-3, 3, n),
                  rng.uniform(-3, 3, n)], 1)
    S0 = rng.uniform(500, 1500, (n, 1))
    return P, cfp, S0


def test_watson_fp32_signal_error(built):
    P, cfp, S0 = watson_draws(600, 1)
    o = oracle("NODDI_Watson")
    s64 = o.signal(P, cfp, S0)
    s32 = o.signal(P, cfp, S0, prec=1)
    assert np.max(np.abs(s32 - s64) / S0) < 1e-6


def test_watson_fp32_jacobian_error(built):
    P, cfp, S0 = watson_draws(300, 2)
    o = oracle("NODDI_Watson")
    _, j64 = o.signal(P, cfp, S0, jac=True)
    _, j32 = o.signal(P, cfp, S0, jac=True, prec=1)
    scale = np.abs(j64).max(axis=1, keepdims=True) + 1e-30
    err = np.abs(j32 - j64) / scale
    assert np.median(err) < 1e-6
    assert np.quantile(err, 0.999) < 1e-4


@pytest.mark.parametrize("col", [2, 3, 4])
def test_watson_analytic_derivatives(built, col):
    """kappa, theta, phi columns (numerical in CUDIMOT, analytic here)."""
    P, cfp, S0 = watson_draws(300, 3)
    keep = (np.abs(P[:, 2] - 0.4) > 1e-3) & (np.abs(P[:, 2] - 30) > 1e-2) & (P[:, 2] > 2e-5)
    P, S0 = P[keep], S0[keep]
    o = oracle("NODDI_Watson")
    _, J = o.signal(P, cfp, S0, jac=True)
    h = 1e-6 * np.maximum(np.abs(P[:, col]), 1e-3)
    Pp, Pm = P.copy(), P.copy()
    Pp[:, col] += h
    Pm[:, col] -= h
    fd = (o.signal(Pp, cfp, S0) - o.signal(Pm, cfp, S0)) / (2 * h[:, None])
    err = np.abs(fd - J[..., col]) / S0
    assert np.max(err) < 1e-4 * np.max(np.abs(J[..., col]) / S0) + 1e-7


def test_ball_1_stick_fp32(built):
    wl = synth.ball_1_stick(500)
    o = oracle("Ball_1_Stick")
    s64 = o.signal(wl.truth, wl.cfp)
    s32 = o.signal(wl.truth, wl.cfp, prec=1)
    assert np.max(np.abs(s32 - s64) / wl.truth[:, :1]) < 1e-6
