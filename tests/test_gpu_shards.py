"""Voxel shards through the library: fitting a volume as contiguous ranges
(CUDIMOT's split_parts.cc:80-94 rule, parts.shard_range), each call with
first_voxel = its range start, gives bit for bit the fit of one call over
the whole volume - grid search, LM, MCMC samples and the final parameters.
This is what makes splitting the voxels across GPUs (or parts) exact."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi, parts
from tests.helpers import watson

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)


@pytest.mark.parametrize("nshards", [2, 3])
def test_shards_equal_one_call(built, cuda, nshards):
    wl = watson(1001, seed=17)  # odd size: the last range takes the remainder
    ns = 20

    def fit(lo, hi):
        # explicit lane counts: the automatic choice widens groups for small calls
        cfg = capi.model_cfg("NODDI_Watson", grid=wl.grid, run_mcmc=1, nburn=100, njumps=200,
                             sampleevery=10, lanes_gridsearch=2, lanes_levmar=4, lanes_mcmc=2,
                             first_voxel=lo)
        lib = capi.Cudimot("NODDI_Watson", cfg)
        p = T(wl.init[lo:hi], cuda)
        s = torch.zeros(hi - lo, 5, ns, dtype=torch.float64, device=cuda)
        lib.fit(T(wl.meas[lo:hi], cuda), p, T(wl.cfp, cuda), T(wl.fixp[lo:hi], cuda), s)
        torch.cuda.synchronize()
        return p.cpu().numpy(), s.cpu().numpy()

    p1, s1 = fit(0, wl.nvox)
    got_p, got_s = [], []
    for r in range(nshards):
        a, b = parts.shard_range(wl.nvox, nshards, r)
        p, s = fit(a, b)
        got_p.append(p)
        got_s.append(s)
    assert np.array_equal(np.concatenate(got_p), p1)
    assert np.array_equal(np.concatenate(got_s), s1)


def test_first_voxel_changes_the_draws(built, cuda):
    """The draws do depend on the global index: the same voxels fitted with
    another first_voxel give other samples (same posterior)."""
    wl = watson(64, seed=3)
    out = []
    for fv in (0, 5000):
        cfg = capi.model_cfg("NODDI_Watson", run_mcmc=1, nburn=50, njumps=100, sampleevery=10,
                             run_levmar=0, first_voxel=fv)
        lib = capi.Cudimot("NODDI_Watson", cfg)
        s = torch.zeros(64, 5, 10, dtype=torch.float64, device=cuda)
        lib.mcmc(T(wl.meas, cuda), T(wl.init, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda), s)
        torch.cuda.synchronize()
        out.append(s.cpu().numpy())
    assert not np.array_equal(out[0], out[1])


def test_fit_host_pieces_equal_one_fit(built, cuda):
    """cdm_fit_host on 150,001 voxels runs as 3 voxel ranges in flight at
    once (each on a context and stream of its own, copies overlapping the
    other ranges' fits); parameters, samples, BIC/AIC and the LM counters
    equal those of cdm_fit over the whole volume on the device."""
    from cudimot_gb300 import synth
    wl = synth.ball_1_stick(150_001, seed=23)
    cfg = capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=20, njumps=40, sampleevery=10,
                         bic_aic=1)
    dev_lib = capi.Cudimot("Ball_1_Stick", cfg)
    p = T(wl.init, cuda)
    s = torch.zeros(wl.nvox, 5, 4, dtype=torch.float64, device=cuda)
    bic = torch.zeros(wl.nvox, dtype=torch.float64, device=cuda)
    aic = torch.zeros_like(bic)
    dev_lib.fit(T(wl.meas, cuda), p, T(wl.cfp, cuda), T(wl.fixp, cuda), s, bic=bic, aic=aic)
    torch.cuda.synchronize()
    ref_stats = dev_lib.stats()
    host_lib = capi.Cudimot("Ball_1_Stick", cfg)
    hp = np.ascontiguousarray(wl.init.copy())
    hs = np.zeros((wl.nvox, 5, 4))
    hb, ha = np.zeros(wl.nvox), np.zeros(wl.nvox)
    host_lib.fit_host(np.ascontiguousarray(wl.meas), hp, np.ascontiguousarray(wl.cfp),
                      np.ascontiguousarray(wl.fixp), hs, None, None, hb, ha)
    assert np.array_equal(hp, p.cpu().numpy())
    assert np.array_equal(hs, s.cpu().numpy())
    assert np.array_equal(hb, bic.cpu().numpy()) and np.array_equal(ha, aic.cpu().numpy())
    st = host_lib.stats()
    assert st.lm_iterations == ref_stats.lm_iterations and st.lm_successes == ref_stats.lm_successes
