"""The persistent multi-model MCMC kernel (include/cdm_hetero.h): several
fits of different models, protocols (71, 134 and 288 measurements), lane
counts and likelihoods run in ONE launch whose CTAs take tiles from a
device counter, and each fit's chains are those of its own library's
cdm_mcmc on the same inputs: the same chain code with the tile in place of
the block index, on the same counter-based draws. The kernel compiles
that code separately from the model library, so a chain may part from its
library twin where the two compilations round an operation differently
and a borderline accept/reject then goes the other way: every fit must
agree sample for sample on at least 99 % of its voxels, and its final
parameters likewise."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi, hetero
from tests.helpers import b2s, dt, watson

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)


# model, workload, voxels, lanes, rician, first voxel; the last two share
# model, lanes and likelihood, so they take two launches
FITS = [("DiffusionTensor", dt, 1000, 1, 0, 0),
        ("Ball_2_Sticks", b2s, 701, 2, 1, 0),
        ("NODDI_Watson", watson, 1303, 4, 0, 0),
        ("NODDI_Watson", watson, 517, 2, 0, 40000),
        ("NODDI_Watson", watson, 300, 2, 0, 90000)]


def _fit_inputs(dev):
    out = []
    for k, (model, wl_fn, n, lanes, rician, fv) in enumerate(FITS):
        wl = wl_fn(n, seed=100 + k)
        cfg = capi.model_cfg(model, run_mcmc=1, nburn=100, njumps=200, sampleevery=10,
                             lanes_mcmc=lanes, rician=rician, first_voxel=fv)
        out.append((model, cfg, wl, rician))
    return out


def _arrays(model, wl, rician, dev):
    s = torch.zeros(wl.nvox, wl.init.shape[1], 20, dtype=torch.float64, device=dev)
    tau = torch.zeros(wl.nvox, 20, dtype=torch.float64, device=dev) if rician else None
    return T(wl.meas, dev), T(wl.init, dev), T(wl.cfp, dev), T(wl.fixp, dev), s, tau


def test_hetero_mcmc_equals_per_model(built, cuda):
    fits = _fit_inputs(cuda)
    ref = []
    for model, cfg, wl, rician in fits:
        m, p, c, f, s, tau = _arrays(model, wl, rician, cuda)
        capi.Cudimot(model, cfg).mcmc(m, p, c, f, s, tau=tau)
        ref.append((p, s, tau))
    torch.cuda.synchronize()
    h = hetero.Hetero()
    ctxs, works, got = [], [], []
    for model, cfg, wl, rician in fits:
        ctx = capi.Cudimot(model, cfg)  # one context per fit: each keeps its packed signals
        m, p, c, f, s, tau = _arrays(model, wl, rician, cuda)
        works.append(h.prepare(ctx, m, p, c, f, s, tau))
        ctxs.append((ctx, m, c, f))
        got.append((p, s, tau))
    assert [w.ntiles for w in works] == [-(-n // (128 // g)) for _, _, n, g, _, _ in FITS]
    h.mcmc(works)
    torch.cuda.synchronize()
    for ctx, *_ in ctxs:
        ctx.synchronize()
    assert 0 < h.last_grid <= sum(w.ntiles for w in works)
    assert h.last_launches == 2
    for k, ((p0, s0, t0), (p1, s1, t1)) in enumerate(zip(ref, got)):
        same = (s0 == s1).flatten(1).all(1)
        if t0 is not None:
            same &= (t0 == t1).all(1)
        assert same.double().mean() >= 0.99, (k, FITS[k][0], float(same.double().mean()))
        assert (p0 == p1).all(1).double().mean() >= 0.99, (k, FITS[k][0])
    # the runs did something: chains moved away from the start
    assert not torch.equal(got[2][1][:, :, 0], got[2][1][:, :, -1])


def test_hetero_rejects_what_is_not_linked(built, cuda):
    h = hetero.Hetero()
    wl = watson(64, seed=3)
    m, p, c, f, s, _ = _arrays("NODDI_Watson", wl, 0, cuda)
    # a lane count the library was not built with: rejected before any launch
    ctx = capi.Cudimot("NODDI_Watson", capi.model_cfg("NODDI_Watson", run_mcmc=1, nburn=10,
                                                      njumps=20, sampleevery=10, lanes_mcmc=8))
    w = h.prepare(ctx, m, p, c, f, s[:, :, :2].contiguous())
    with pytest.raises(capi.CdmError, match="lanes"):
        h.mcmc([w])
    # a model that is not linked
    from tests.helpers import b1s
    wb = b1s(64, seed=4)
    ctx = capi.Cudimot("Ball_1_Stick", capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=10,
                                                      njumps=20, sampleevery=10, lanes_mcmc=2))
    sb = torch.zeros(64, 5, 2, dtype=torch.float64, device=cuda)
    w = h.prepare(ctx, T(wb.meas, cuda), T(wb.init, cuda), T(wb.cfp, cuda), T(wb.fixp, cuda), sb)
    with pytest.raises(capi.CdmError, match="not linked"):
        h.mcmc([w])
    # nothing to do
    h.mcmc([])
    assert h.last_grid == 0
