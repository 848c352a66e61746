"""Pipelines restating CUDIMOT's Pipeline_<Model>.sh on the GPU:
  * NODDI-Watson (S0 from the b=0 volumes, tensor fit, grid search with the
    orientation fixed, fractions with kappa and orientation fixed, full
    fit, finish) replayed from one captured CUDA graph equals the same
    steps run eagerly, bit for bit, and twice in a row;
  * the steps do what the scripts do: the grid search leaves theta/phi at
    the tensor fit's V1, FitFractions leaves kappa at the grid value, and
    the final fit's cost is no worse than the grid search's; and each stage
    matches the FP64 oracle's run of the same stage from the same input;
  * Ball_1_Stick's and Ball_2_Sticks' one-step pipelines from the tensor
    fit match LM from the same initial values;
  * NODDI-Bingham's pipeline (grid search + LM with the orientation fixed,
    then all but fiso) replays its graph exactly and passes fiso through
    the last step unchanged."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from cudimot_gb300.pipeline import Pipeline
from tests.helpers import angle_deg, assert_lm_voxelwise, b1s, oracle, watson

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def test_watson_pipeline_graph_equals_eager(built, cuda):
    wl = watson(2048, seed=31)
    m = T(wl.meas, cuda)
    eager = Pipeline("NODDI_Watson", m, wl.cfp[:, :3], wl.cfp[:, 3], run_mcmc=True, nburn=100,
                     njumps=100, sampleevery=10)
    eager.run(graph=False)
    torch.cuda.synchronize()
    g = Pipeline("NODDI_Watson", m, wl.cfp[:, :3], wl.cfp[:, 3], run_mcmc=True, nburn=100,
                 njumps=100, sampleevery=10)
    g.run()
    torch.cuda.synchronize()
    first = g.samples.clone()
    g.run()
    torch.cuda.synchronize()
    assert torch.equal(g.samples, first)
    assert torch.equal(g.samples, eager.samples)
    assert torch.equal(g.fixp, eager.fixp)
    assert torch.equal(g.od, eager.od) and torch.equal(g.dyads, eager.dyads)
    s0 = wl.meas[:, wl.cfp[:, 3] <= 50].mean(1)
    np.testing.assert_allclose(g.fixp.cpu().numpy()[:, 0], s0, rtol=1e-12)


def test_watson_pipeline_steps(built, cuda):
    """Pipeline_NODDI_Watson.sh's staged --fixed sequence, stage by stage,
    against the FP64 oracle run from the same input as each GPU stage: the
    b=0 mean (S0, FixP), the grid search with the orientation fixed (winners
    bit for bit), FitFractions (LM with kappa and orientation fixed) and
    the full fit (LM), both held to the LM parity bounds of the library's
    own NODDI-Watson test."""
    wl = watson(1024, seed=32)
    m = T(wl.meas, cuda)
    pl = Pipeline("NODDI_Watson", m, wl.cfp[:, :3], wl.cfp[:, 3])
    o = oracle("NODDI_Watson")
    # step by step, inspecting the shared parameter array
    from cudimot_gb300 import utils
    utils.mean_columns(m, pl.b0, pl.fixp)
    utils.dti_fit(m, pl.bvecs, pl.bvals, out=pl.dti)
    for p, col, scale in pl.spec["init"]:
        if col is None:
            utils.copy_columns(None, 0, pl.params, p, 1, scale)
        else:
            utils.copy_columns(pl.dti, utils.DTI_COLS.index(col), pl.params, p, 1, scale)
    torch.cuda.synchronize()
    f = pl.fixp.cpu().numpy()
    b0 = wl.cfp[:, 3] <= 50.0
    np.testing.assert_allclose(f[:, 0], wl.meas[:, b0].mean(1), rtol=1e-13)
    start = pl.params.cpu().numpy().copy()
    st, lib, samples = pl.ctx[0]
    lib.fit_enqueue(m, pl.params, pl.cfp, pl.fixp, samples)
    torch.cuda.synchronize()
    after_gs = pl.params.cpu().numpy().copy()
    np.testing.assert_array_equal(after_gs[:, 3:5], pl.dti.cpu().numpy()[:, 12:14])
    ref_gs, _, _ = o.gridsearch(lib.cfg, wl.meas, start, wl.cfp, f)
    np.testing.assert_array_equal(after_gs, ref_gs)
    st, lib, samples = pl.ctx[1]
    lib.fit_enqueue(m, pl.params, pl.cfp, pl.fixp, samples)
    torch.cuda.synchronize()
    after_ff = pl.params.cpu().numpy().copy()
    np.testing.assert_array_equal(after_ff[:, 2:5], after_gs[:, 2:5])
    ref_ff = o.levmar(lib.cfg, wl.meas, after_gs, wl.cfp, f)[0]
    # the oracle, like CUDIMOT, carries fixed parameters through the bounds
    # transform and back (a few ulp); the library leaves them untouched
    np.testing.assert_allclose(ref_ff[:, 2:5], after_gs[:, 2:5], rtol=1e-13, atol=1e-13)
    assert_lm_voxelwise(o.cost(wl.meas, after_ff, wl.cfp, f), o.cost(wl.meas, ref_ff, wl.cfp, f),
                        max_frac=0.0075, max_excess=0.01)
    st, lib, samples = pl.ctx[2]
    lib.fit_enqueue(m, pl.params, pl.cfp, pl.fixp, samples)
    torch.cuda.synchronize()
    final = pl.params.cpu().numpy()
    ref_fin = o.levmar(lib.cfg, wl.meas, after_ff, wl.cfp, f)[0]
    ang = angle_deg(final[:, 3], final[:, 4], ref_fin[:, 3], ref_fin[:, 4])
    c_fin = o.cost(wl.meas, final, wl.cfp, f)
    assert_lm_voxelwise(c_fin, o.cost(wl.meas, ref_fin, wl.cfp, f), ang, max_frac=0.0075,
                        max_excess=0.01)
    c_gs = o.cost(wl.meas, after_gs, wl.cfp, f)
    assert np.mean(c_fin <= c_gs * (1 + 1e-6)) >= 0.99


def test_ball_1_stick_pipeline(built, cuda):
    wl = b1s(2048, seed=33)
    m = T(wl.meas, cuda)
    pl = Pipeline("Ball_1_Stick", m, wl.cfp[:, :3], wl.cfp[:, 3])
    pl.run()
    torch.cuda.synchronize()
    d = pl.dti.cpu().numpy()
    init = np.stack([d[:, 0], d[:, 1], d[:, 10], d[:, 12], d[:, 13]], 1)
    lib = capi.Cudimot("Ball_1_Stick", capi.model_cfg("Ball_1_Stick"))
    q = T(init, cuda)
    lib.levmar(m, q, T(wl.cfp, cuda), T(wl.fixp, cuda))
    torch.cuda.synchronize()
    assert torch.equal(pl.params, q)


def test_ball_2_sticks_pipeline(built, cuda):
    """Pipeline_Ball_2_Sticks.sh: one fit from S0, L1, FA, V1, FA/4, V2 of the
    tensor fit, as LM from those values."""
    from tests.helpers import b2s
    wl = b2s(2048, seed=34)
    m = T(wl.meas, cuda)
    pl = Pipeline("Ball_2_Sticks", m, wl.cfp[:, :3], wl.cfp[:, 3])
    pl.run()
    torch.cuda.synchronize()
    d = pl.dti.cpu().numpy()
    init = np.stack([d[:, 0], d[:, 1], d[:, 10], d[:, 12], d[:, 13], 0.25 * d[:, 10], d[:, 14],
                     d[:, 15]], 1)
    lib = capi.Cudimot("Ball_2_Sticks", capi.model_cfg("Ball_2_Sticks"))
    q = T(init, cuda)
    lib.levmar(m, q, T(wl.cfp, cuda), T(wl.fixp, cuda))
    torch.cuda.synchronize()
    assert torch.equal(pl.params, q)


def test_bingham_pipeline_graph_equals_eager(built, cuda):
    """Pipeline_NODDI_Bingham.sh: grid search + LM with the orientation
    fixed (psi from the tensor fit), then all but fiso; the graph replay
    equals the eager run, fiso passes the second step unchanged, and the
    finish step gives finite dyads and OD."""
    from tests.helpers import bingham
    wl = bingham(512, seed=35)
    m = T(wl.meas, cuda)
    eager = Pipeline("NODDI_Bingham", m, wl.cfp[:, :3], wl.cfp[:, 3], run_mcmc=True, nburn=40,
                     njumps=40, sampleevery=10)
    eager.run(graph=False)
    torch.cuda.synchronize()
    g = Pipeline("NODDI_Bingham", m, wl.cfp[:, :3], wl.cfp[:, 3], run_mcmc=True, nburn=40,
                 njumps=40, sampleevery=10)
    g.run()
    torch.cuda.synchronize()
    assert torch.equal(g.samples, eager.samples)
    s = g.samples.cpu().numpy()
    # fiso is fixed in the last step: every sample equals the grid/LM value
    assert np.all(s[:, 0, :] == s[:, 0, :1])
    np.testing.assert_array_equal(s[:, 0, 0], g.params.cpu().numpy()[:, 0])
    assert np.all(np.isfinite(g.dyads.cpu().numpy())) and np.all(np.isfinite(g.od.cpu().numpy()))
