"""Edge cases of the fitting entry points against the FP64 oracle.

* empty input (nvox = 0) on every stage and on cdm_fit: CDM_OK, nothing
  written;
* voxel counts below one CTA and not a multiple of its voxels (1, 3, 65);
* ragged protocols: measurement counts that are odd, below one lane group,
  or leave a partial pair and a partial chunk (1, 3, 7, 33, 67, 129);
* the largest protocol whose tables fit the shared-memory staging
  (NODDI-Watson: 2,112 measurements) and the first size that does not
  (rejected with CDM_BAD_ARG before any launch).

Tolerances are those of the main parity tests: predicted signal within
2e-5 |S| + 2e-6 S0, grid-search winners bit-exact (with 1 or 3
measurements: the same FP64 cost up to FP32 rounding), LM final cost
within 1e-4 relative of the oracle's fit from the same start.
"""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from tests.helpers import b1s, oracle, watson

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def _empty(shape, dev):
    return torch.zeros(shape, dtype=torch.float64, device=dev)


def test_empty_input_every_stage(built, cuda):
    wl = watson(4)
    cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid, run_mcmc=1, nburn=10, njumps=10,
                         sampleevery=5, get_predicted=1, bic_aic=1)
    lib = capi.Cudimot("NODDI_Watson", cfg)
    nm = wl.nmeas
    meas, params = _empty((0, nm), cuda), _empty((0, 5), cuda)
    fixp, cfp = _empty((0, 1), cuda), T(wl.cfp, cuda)
    samples, pred = _empty((0, 5, 2), cuda), _empty((0, nm), cuda)
    bic, aic = _empty((0,), cuda), _empty((0,), cuda)
    lib.gridsearch(meas, params, cfp, fixp)
    lib.levmar(meas, params, cfp, fixp)
    lib.mcmc(meas, params, cfp, fixp, samples)
    lib.predicted_signal(samples, cfp, fixp, pred)
    lib.bic_aic(meas, samples, cfp, fixp, bic, aic)
    lib.fit(meas, params, cfp, fixp, samples, pred=pred, bic=bic, aic=aic)
    lib.synchronize(timeout_ms=10000)
    # the context still fits a real voxel afterwards
    p = T(wl.init, cuda)
    lib.levmar(T(wl.meas, cuda), p, cfp, T(wl.fixp, cuda))
    lib.synchronize(timeout_ms=10000)
    assert np.all(np.isfinite(p.cpu().numpy()))


@pytest.mark.parametrize("nvox", [1, 3, 65])
def test_few_voxels(built, cuda, nvox):
    wl = watson(nvox, seed=100 + nvox)
    o = oracle("NODDI_Watson")
    cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid)
    lib = capi.Cudimot("NODDI_Watson", cfg)
    params = T(wl.init, cuda)
    lib.gridsearch(T(wl.meas, cuda), params, T(wl.cfp, cuda), T(wl.fixp, cuda))
    lib.synchronize(timeout_ms=30000)
    ref_p, _, _ = o.gridsearch(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    got = params.cpu().numpy()
    assert np.array_equal(got, ref_p), np.argwhere(got != ref_p)[:5]

    wb = b1s(nvox, seed=200 + nvox)
    ob = oracle("Ball_1_Stick")
    cb = capi.model_cfg("Ball_1_Stick")
    lb = capi.Cudimot("Ball_1_Stick", cb)
    pb = T(wb.init, cuda)
    lb.levmar(T(wb.meas, cuda), pb, T(wb.cfp, cuda), T(wb.fixp, cuda))
    lb.synchronize(timeout_ms=30000)
    ref, _, _, _ = ob.levmar(cb, wb.meas, wb.init, wb.cfp, wb.fixp)
    c_got = ob.cost(wb.meas, pb.cpu().numpy(), wb.cfp, wb.fixp)
    c_ref = ob.cost(wb.meas, ref, wb.cfp, wb.fixp)
    # as the main LM parity test: a rare voxel may settle in another minimum
    ok = (c_got - c_ref) / c_ref <= 1e-4
    assert ok.all() if nvox < 10 else np.mean(ok) >= 0.95, (c_got, c_ref)


def _subset(wl, nm, seed):
    """The first b=0 row plus nm - 1 diffusion-weighted rows chosen at random
    (sorted), so that every subset constrains the fit."""
    rng = np.random.default_rng(seed)
    b0 = np.flatnonzero(wl.cfp[:, 3] == 0)
    dw = np.flatnonzero(wl.cfp[:, 3] > 0)
    rows = np.sort(np.concatenate([b0[:1], rng.choice(dw, nm - 1, replace=False)]))
    return wl.cfp[rows].copy(), wl.meas[:, rows].copy()


@pytest.mark.parametrize("nm", [1, 3, 7, 33, 67, 129])
def test_ragged_protocols(built, cuda, nm):
    wl = watson(300, seed=31)
    o = oracle("NODDI_Watson")
    if nm == 1:
        rows = np.flatnonzero(wl.cfp[:, 3] > 0)[:1]
        cfp, meas = wl.cfp[rows].copy(), wl.meas[:, rows].copy()
    else:
        cfp, meas = _subset(wl, nm, seed=nm)
    for lanes in (2, 8):
        cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid, lanes_gridsearch=lanes)
        lib = capi.Cudimot("NODDI_Watson", cfg)
        # predicted signal (paired hook on whole pairs, Predicted_Signal on the rest)
        pred = _empty((wl.nvox, nm), cuda)
        lib.predicted_signal(T(wl.truth, cuda), T(cfp, cuda), T(wl.fixp, cuda), pred)
        lib.synchronize(timeout_ms=30000)
        ref = o.signal(wl.truth, cfp, wl.fixp)
        got = pred.cpu().numpy()
        assert np.all(np.abs(got - ref) <= 2e-5 * np.abs(ref) + 2e-6 * wl.fixp)
        # grid search: the same winner as the oracle for every voxel
        params = T(wl.init, cuda)
        lib.gridsearch(T(meas, cuda), params, T(cfp, cuda), T(wl.fixp, cuda))
        lib.synchronize(timeout_ms=30000)
        ref_p, _, _ = o.gridsearch(cfg, meas, wl.init, cfp, wl.fixp)
        got = params.cpu().numpy()
        if nm >= 7:
            assert np.array_equal(got, ref_p), (lanes, np.argwhere(got != ref_p)[:5])
        else:
            # With 1 or 3 measurements a near-zero residual makes the FP32
            # cost's relative error larger than the FP64 re-check window, so
            # the winner may differ by FP32 rounding: its FP64 cost must
            # then be within that rounding of the oracle's best.
            c_got = o.cost(meas, got, cfp, wl.fixp)
            c_ref = o.cost(meas, ref_p, cfp, wl.fixp)
            s0 = wl.fixp[:, 0]
            tol = 1e-5 * c_ref + 4e-6 * s0 * np.sqrt(nm * c_ref) + (1e-6 * s0) ** 2 * nm
            assert np.all(c_got - c_ref <= tol), (lanes, np.max((c_got - c_ref) / tol))
            assert np.mean(np.all(got == ref_p, axis=1)) >= 0.9
        # BIC/AIC on the truth (the SSE sums the ragged tail)
        bic, aic = _empty((wl.nvox,), cuda), _empty((wl.nvox,), cuda)
        lib.bic_aic(T(meas, cuda), T(wl.truth[:, :, None], cuda), T(cfp, cuda), T(wl.fixp, cuda),
                    bic, aic)
        lib.synchronize(timeout_ms=30000)
        rb, ra = o.bic_aic(meas, wl.truth[:, :, None], cfp, wl.fixp)
        # BIC/AIC = n ln(SSE / 2) + const: an FP32 signal error dS moves the
        # SSE by up to 2 dS sum|r| + n dS^2, i.e. n (2 dS sqrt(n SSE) + n
        # dS^2) / SSE in BIC -- large only when a few small residuals make
        # up the SSE (1 measurement)
        sse = o.cost(meas, wl.truth, cfp, wl.fixp)
        dS = 2e-6 * wl.fixp[:, 0]
        tol = 5e-6 * np.abs(rb) + nm * (2 * dS * np.sqrt(nm * sse) + nm * dS ** 2) / sse
        assert np.all(np.abs(bic.cpu().numpy() - rb) <= tol)
        assert np.all(np.abs(aic.cpu().numpy() - ra) <= tol)


# NODDI-Watson stages 12 protocol columns per measurement (4 of CFP + 8
# derived), padded to 32 measurements, and a pair table of the same size:
# 96 B per padded measurement against the 200 KiB staging limit.
WATSON_MAX_NMEAS = 2112


def test_largest_protocol(built, cuda):
    wl = watson(48, seed=41)
    o = oracle("NODDI_Watson")
    rng = np.random.default_rng(5)
    reps = -(-WATSON_MAX_NMEAS // wl.nmeas)
    cfp = np.tile(wl.cfp, (reps, 1))[:WATSON_MAX_NMEAS].copy()
    clean = o.signal(wl.truth, cfp, wl.fixp)
    sigma = wl.fixp / 20.0
    meas = np.hypot(clean + sigma * rng.standard_normal(clean.shape),
                    sigma * rng.standard_normal(clean.shape))
    cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid)
    lib = capi.Cudimot("NODDI_Watson", cfg)
    pred = _empty((wl.nvox, WATSON_MAX_NMEAS), cuda)
    lib.predicted_signal(T(wl.truth, cuda), T(cfp, cuda), T(wl.fixp, cuda), pred)
    params = T(wl.init, cuda)
    lib.gridsearch(T(meas, cuda), params, T(cfp, cuda), T(wl.fixp, cuda))
    lib.synchronize(timeout_ms=60000)
    got_pred = pred.cpu().numpy()
    assert np.all(np.abs(got_pred - clean) <= 2e-5 * np.abs(clean) + 2e-6 * wl.fixp)
    ref_p, _, _ = o.gridsearch(cfg, meas, wl.init, cfp, wl.fixp)
    got = params.cpu().numpy()
    assert np.array_equal(got, ref_p), np.argwhere(got != ref_p)[:5]
    start = got.copy()
    lib.levmar(T(meas, cuda), params, T(cfp, cuda), T(wl.fixp, cuda))
    lib.synchronize(timeout_ms=60000)
    ref, _, _, _ = o.levmar(cfg, meas, start, cfp, wl.fixp)
    c_got = o.cost(meas, params.cpu().numpy(), cfp, wl.fixp)
    c_ref = o.cost(meas, ref, cfp, wl.fixp)
    assert np.mean((c_got - c_ref) / c_ref <= 1e-4) >= 0.95, np.quantile((c_got - c_ref) / c_ref, [0.5, 1])

    # one padded chunk more does not fit: every stage refuses before launching
    nm = WATSON_MAX_NMEAS + 1
    cfp2 = np.tile(wl.cfp, (reps + 1, 1))[:nm].copy()
    meas2 = _empty((wl.nvox, nm), cuda)
    for call in (lambda: lib.gridsearch(meas2, params, T(cfp2, cuda), T(wl.fixp, cuda)),
                 lambda: lib.levmar(meas2, params, T(cfp2, cuda), T(wl.fixp, cuda))):
        with pytest.raises(capi.CdmError, match="BAD_ARG"):
            call()
    lib.synchronize(timeout_ms=10000)


@pytest.mark.parametrize("model", ["Ball_1_Stick", "DiffusionTensor", "Ball_2_Sticks",
                                   "NODDI_Watson", "NODDI_Bingham"])
def test_mcmc_every_lane_count(built, cuda, model):
    """MCMC runs at every lane count, Gaussian and Rician: the kernel's
    static shared memory (sample staging, up to 37 KB at one lane for the
    8-parameter model) plus the staged protocol may pass 48 KB, which needs
    the opt-in even when the protocol alone does not."""
    from tests import helpers
    wl = {"Ball_1_Stick": helpers.b1s, "DiffusionTensor": helpers.dt, "Ball_2_Sticks": helpers.b2s,
          "NODDI_Watson": helpers.watson, "NODDI_Bingham": helpers.bingham}[model](70, seed=44)
    npar = wl.init.shape[1]
    for rician in (0, 1):
        for lanes in (1, 2, 4, 8, 16, 32):
            cfg = capi.model_cfg(model, run_mcmc=1, nburn=10, njumps=20, sampleevery=10,
                                 lanes_mcmc=lanes, rician=rician)
            lib = capi.Cudimot(model, cfg)
            s = torch.zeros(70, npar, 2, dtype=torch.float64, device=cuda)
            tau = torch.zeros(70, 2, dtype=torch.float64, device=cuda) if rician else None
            lib.mcmc(T(wl.meas, cuda), T(wl.init, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda), s,
                     tau=tau)
            lib.synchronize(timeout_ms=60000)
            got = s.cpu().numpy()
            assert np.all(np.isfinite(got)) and np.any(got != 0.0), (model, lanes, rician)
