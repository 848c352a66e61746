"""Heterogeneous batch: DiffusionTensor, Ball_2_Sticks and NODDI-Watson
contexts, each with its own protocol and volume, recorded as branches of one
CUDA graph (cdm_batch) and launched once. Every kernel is deterministic
(Philox draws keyed by seed, voxel, iteration and parameter), so each
model's results must equal a separate cdm_fit of the same inputs bit for
bit; a second launch of the captured graph must repeat them."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from tests.helpers import b2s, dt, watson

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def test_batch_equals_separate_fits(built, cuda):
    vols = [("DiffusionTensor", dt(1200, seed=4)), ("Ball_2_Sticks", b2s(900, seed=4)),
            ("NODDI_Watson", watson(1500, seed=4))]
    batch = capi.Batch()
    runs = []
    for model, wl in vols:
        cfg = capi.model_cfg(model, run_mcmc=1, nburn=200, njumps=200, sampleevery=20)
        npar = wl.truth.shape[1]
        ns = cfg.njumps // cfg.sampleevery
        fits = {}
        for mode in ("batch", "alone"):
            lib = capi.Cudimot(model, cfg)
            d = dict(meas=T(wl.meas, cuda), params=T(wl.init, cuda), cfp=T(wl.cfp, cuda),
                     fixp=T(wl.fixp, cuda),
                     samples=torch.zeros(wl.nvox, npar, ns, dtype=torch.float64, device=cuda))
            fits[mode] = (lib, d)
        lib, d = fits["batch"]
        batch.add(lib, d["meas"], d["params"], d["cfp"], d["fixp"], d["samples"])
        lib, d = fits["alone"]
        lib.fit(d["meas"], d["params"], d["cfp"], d["fixp"], d["samples"])
        runs.append((model, wl, fits))
    batch.run()
    torch.cuda.synchronize()
    for model, wl, fits in runs:
        a, b = fits["alone"][1], fits["batch"][1]
        assert torch.equal(a["params"], b["params"]), model
        assert torch.equal(a["samples"], b["samples"]), model
        assert torch.isfinite(b["samples"]).all(), model
    # relaunch the captured graph from the same starting parameters
    first = [fits["batch"][1]["samples"].clone() for _, _, fits in runs]
    for model, wl, fits in runs:
        fits["batch"][1]["params"].copy_(T(wl.init, cuda))
    batch.run()
    torch.cuda.synchronize()
    for s0, (model, _, fits) in zip(first, runs):
        assert torch.equal(s0, fits["batch"][1]["samples"]), model
