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
