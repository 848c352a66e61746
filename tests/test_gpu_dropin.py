"""CUDIMOT's own model plugins, unchanged, fitted by this library on the GPU.

The libraries are split builds from the plugin directories of CUDIMOT's
tree (oracle/build_dropin.py): the device half is compiled where the tree
is, the host half here. They are checked against the FP64 oracle run with
the same unchanged plugins (fixtures in tests/golden/, made by
make_golden.py and make_dropin_golden.py) and, for grid search, against
CUDIMOT's own kernels with the same plugin on the same GPU.

Bounds, voxel by voxel:
  * predicted signal: float evaluation |dS| <= 2e-5 |S| + 2e-6 S0 (S0 = the
    largest signal of the voxel), double evaluation |dS| <= 2e-6 |S| + 1e-7
    S0 (the parameters are single-precision state either way). CUDIMOT's
    NODDI-Watson is the exception: its closed forms cancel terms of ~1e10
    and take single-precision erff, so the same FP64 code gives different
    values on the GPU and on the host wherever it is far from the exact
    model; there the bound adds twice the host's distance from the exact
    model (quadrature, in the fixture);
  * grid search: the winning combination equals the oracle's, bit for bit;
  * LM: on every voxel either the cost agrees within 1e-4 relative and the
    fibre orientation within 0.5 degrees, or the library's cost is lower;
    for NODDI-Bingham a few voxels may end at another stationary point,
    bounded in number and excess (see assert_lm_voxelwise); Ball_2_Sticks
    (CUDIMOT's phi2 derivative is not the derivative of its signal, so LM
    paths part easily) is held to the distribution bounds of its own test;
  * MCMC (the SSFP plugin has no derivatives, so no LM): posterior means
    within Monte Carlo error of the oracle's chain.
"""
import os

import numpy as np
import pytest
import torch

from cudimot_gb300 import capi, synth
from oracle import build_dropin
from tests.helpers import angle_deg, assert_lm_voxelwise

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# model, evaluation type, start of LM in the fixture, orientation columns
LM_CASES = [("Ball_1_Stick", "float", "init", (3, 4)),
            ("NODDI_Watson", "double", "gs", (3, 4)),
            ("DiffusionTensor", "float", "init", None),
            ("Ball_2_Sticks", "float", "init", (3, 4)),
            ("NODDI_Bingham", "double", "gs", (4, 5)),
            ("toymodel", "float", "init", None)]
GRIDS = {"NODDI_Watson": synth.WATSON_GRID, "NODDI_Bingham": synth.BINGHAM_GRID}


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)


def dropin(model, ev, cfg):
    if not build_dropin.available(model, ev):
        pytest.skip(f"no device module for {model} ({ev}): CUDIMOT's tree was absent at build time")
    errs = build_dropin.build_all()
    assert not errs, errs
    return capi.Cudimot(model, cfg, path=build_dropin.lib_path(model, ev))


def gpu_cost(lib, meas, params, cfp, fixp, dev):
    out = torch.empty(meas.shape[0], dtype=torch.float64, device=dev)
    lib.cost(T(meas, dev), T(params, dev), T(cfp, dev), T(fixp, dev), out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def signal_fixture(model):
    name = "plugin" if os.path.exists(os.path.join(GOLDEN, f"plugin_{model}.npz")) else "fit"
    d = np.load(os.path.join(GOLDEN, f"{name}_{model}.npz"))
    return d["params"], d["cfp"], d["fixp"], d["signal"], d.get("signal_exact")


@pytest.mark.parametrize("model,ev", [(m, e) for m, e, _, _ in LM_CASES] +
                         [("Ball_2_Sticks_1Shell_SSFP", "double")])
def test_dropin_predicted_signal(built, cuda, model, ev):
    lib = dropin(model, ev, capi.model_cfg(model))
    P, cfp, F, S, exact = signal_fixture(model)
    pred = torch.zeros(S.shape, dtype=torch.float64, device=cuda)
    lib.predicted_signal(T(P[:, :, None], cuda), T(cfp, cuda), T(F, cuda), pred)
    torch.cuda.synchronize()
    got = pred.cpu().numpy()
    s0 = np.abs(S).max(1, keepdims=True)
    tol = 2e-6 * np.abs(S) + 1e-7 * s0 if ev == "double" else 2e-5 * np.abs(S) + 2e-6 * s0
    if exact is not None:
        tol = tol + 2.0 * np.abs(S - exact)
    err = np.abs(got - S)
    assert np.all(err <= tol), (model, float((err / np.maximum(tol, 1e-300)).max()))


@pytest.mark.parametrize("model,ev,start,orient", LM_CASES)
def test_dropin_gridsearch_and_levmar(built, cuda, model, ev, start, orient):
    fx = np.load(os.path.join(GOLDEN, f"fit_{model}.npz"))
    cfg = capi.model_cfg(model, grid=GRIDS.get(model))
    lib = dropin(model, ev, cfg)
    meas, cfp, fixp = fx["meas"], fx["cfp"], fx["fixp"]
    if start == "gs":
        p = T(fx["init"], cuda)
        lib.gridsearch(T(meas, cuda), p, T(cfp, cuda), T(fixp, cuda))
        torch.cuda.synchronize()
        got = p.cpu().numpy()
        assert np.array_equal(got, fx["gs"]), (model, np.argwhere(got != fx["gs"])[:5])
    p = T(fx[start], cuda)
    lib.levmar(T(meas, cuda), p, T(cfp, cuda), T(fixp, cuda))
    torch.cuda.synchronize()
    got = p.cpu().numpy()
    ref = fx["lm"]
    c_got = gpu_cost(lib, meas, got, cfp, fixp, cuda)
    c_ref = gpu_cost(lib, meas, ref, cfp, fixp, cuda)
    rel = (c_got - c_ref) / c_ref
    if model == "Ball_2_Sticks":
        # the distribution bounds of test_gpu_models.test_levmar_ball_2_sticks
        assert abs(np.median(rel)) <= 1e-5, np.quantile(rel, [0.1, 0.5, 0.9])
        assert np.mean(rel <= 1e-4) >= 0.75, np.mean(rel <= 1e-4)
        return
    ang = None
    if orient:
        i, j = orient
        ang = angle_deg(got[:, i], got[:, j], ref[:, i], ref[:, j])
    if model == "NODDI_Bingham":
        assert_lm_voxelwise(c_got, c_ref, ang, max_frac=0.05, max_excess=0.025)
    else:
        assert_lm_voxelwise(c_got, c_ref, ang)


def test_dropin_watson_gridsearch_matches_cudimot_kernels(built, cuda):
    """Grid search winners of the unchanged NODDI-Watson plugin: this
    library (double evaluation) against CUDIMOT's own grid-search kernel
    (T = double) on the same 2,000 voxels."""
    from oracle.refkernels.refkernels import RefKernels, available
    if not available("NODDI_Watson"):
        pytest.skip("CUDIMOT's kernels were not compiled (tree absent at build time)")
    cfg = capi.model_cfg("NODDI_Watson", grid=synth.WATSON_GRID)
    lib = dropin("NODDI_Watson", "double", cfg)

    def signal(truth, cfp, s0):
        out = torch.zeros(truth.shape[0], cfp.shape[0], dtype=torch.float64, device=cuda)
        lib.predicted_signal(T(truth[:, :, None], cuda), T(cfp, cuda), T(s0[:, None], cuda), out)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    wl = synth.noddi_watson(2000, seed=31, signal_fn=signal)
    m, c, f = T(wl.meas, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda)
    ours = T(wl.init, cuda)
    lib.gridsearch(m, ours, c, f)
    theirs = T(wl.init, cuda)
    RefKernels("NODDI_Watson", 5).gridsearch(cfg, m, theirs, c, f, T(cfg.grid_array, cuda))
    torch.cuda.synchronize()
    a, b = ours.cpu().numpy(), theirs.cpu().numpy()
    assert np.array_equal(a, b), np.argwhere(np.any(a != b, axis=1))[:5].ravel()


def test_dropin_ssfp_mcmc_matches_oracle(built, cuda):
    """Ball_2_Sticks_1Shell_SSFP (empty Partial_Derivatives: an MCMC-only
    model) in double evaluation: posterior means of d, f1 and S0 against
    the FP64 oracle's chain from the same start (independent seeds)."""
    model = "Ball_2_Sticks_1Shell_SSFP"
    fx = np.load(os.path.join(GOLDEN, f"fit_{model}.npz"))
    cfg = capi.model_cfg(model, run_mcmc=1, nburn=500, njumps=1000, sampleevery=10)
    lib = dropin(model, "double", cfg)
    n = fx["meas"].shape[0]
    samples = torch.zeros(n, 8, 100, dtype=torch.float64, device=cuda)
    lib.mcmc(T(fx["meas"], cuda), T(fx["init"], cuda), T(fx["cfp"], cuda), T(fx["fixp"], cuda),
             samples)
    torch.cuda.synchronize()
    g, r = samples.cpu().numpy(), fx["samples"].astype(np.float64)

    def se(x):  # batch means, 10 batches of 10 thinned samples
        b = x.reshape(x.shape[0], 10, -1).mean(2)
        return b.std(1, ddof=1) / np.sqrt(10)

    for p in (0, 1, 7):
        mg, mr = g[:, p].mean(1), r[:, p].mean(1)
        z = (mg - mr) / np.sqrt(se(g[:, p]) ** 2 + se(r[:, p]) ** 2 + 1e-30)
        assert abs(np.median(z)) < 0.6, (p, float(np.median(z)))
        assert np.mean(np.abs(z) < 4) > 0.9, (p, float(np.mean(np.abs(z) < 4)))
