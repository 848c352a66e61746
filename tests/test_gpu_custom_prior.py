"""custom() priors see the whole protocol, as in CUDIMOT: custom_priors(id,
P, nmeas, CFP, FixP) receives the [nmeas][CFP_Tsize] array of every
measurement (MCMC.cu:134, :186; the kernel's copy of the CFP at :382-384).

The test plugin (tests/plugins/Monoexp_BPrior: S = S0 exp(-b D)) centres a
Gaussian prior on D at 0.5 / mean(b) over all measurements. Its chains on
the GPU are compared with the FP64 oracle's chains for the same plugin
(posterior means within Monte Carlo error), and the prior must visibly pull
D below the chains without it."""
import os

import numpy as np
import pytest
import torch

from cudimot_gb300 import build, capi
from oracle import build_oracle
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

NAME = "Monoexp_BPrior"
PLUGIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "plugins", NAME)


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)


@pytest.fixture(scope="module")
def plugin():
    out, err = build.build_model(PLUGIN, name=NAME)
    assert not err, err
    ora = os.path.join(os.path.dirname(build_oracle.__file__), "_build", f"liboracle_{NAME}.so")
    _, err = build_oracle.compile_one(PLUGIN, NAME, ora)
    assert not err, err
    return out, Oracle(NAME, build=False)


def workload(n=256, seed=77):
    rng = np.random.default_rng(seed)
    b = np.linspace(0.0, 3000.0, 60)
    g = rng.standard_normal((b.size, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    cfp = np.concatenate([g, b[:, None]], 1)
    P = np.stack([rng.uniform(800, 1200, n), rng.uniform(0.8e-3, 1.5e-3, n)], 1)
    S = P[:, :1] * np.exp(-P[:, 1:] * b[None, :])
    meas = S + rng.standard_normal(S.shape) * (P[:, :1] / 20.0)
    return meas, P.copy(), cfp


def cfg_for(prior):
    return capi.make_cfg(2, bounds={0: (0.0, None), 1: (0.0, 0.01)},
                         priors={1: (prior,)} if prior else None, run_mcmc=1, run_levmar=0,
                         nburn=500, njumps=1000, sampleevery=10)


def se(x):  # batch means, 10 batches of 10 thinned samples
    b = x.reshape(x.shape[0], 10, -1).mean(2)
    return b.std(1, ddof=1) / np.sqrt(10)


def test_custom_prior_sees_every_measurement(built, cuda, plugin):
    path, ora = plugin
    meas, init, cfp = workload()
    n = meas.shape[0]
    fixp = np.zeros((n, 0))
    chains = {}
    for prior in (capi.CUSTOM, None):
        cfg = cfg_for(prior)
        lib = capi.Cudimot(NAME, cfg, path=path)
        s = torch.zeros(n, 2, 100, dtype=torch.float64, device=cuda)
        lib.mcmc(T(meas, cuda), T(init, cuda), T(cfp, cuda), T(fixp, cuda), s)
        torch.cuda.synchronize()
        chains[prior] = s.cpu().numpy()
    g = chains[capi.CUSTOM][:, 1]
    _, r, _ = ora.mcmc(cfg_for(capi.CUSTOM), meas, init, cfp, fixp)
    r = r[:, 1]
    z = (g.mean(1) - r.mean(1)) / np.sqrt(se(g) ** 2 + se(r) ** 2 + 1e-30)
    assert abs(np.median(z)) < 0.6, float(np.median(z))
    assert np.mean(np.abs(z) < 4) > 0.9, float(np.mean(np.abs(z) < 4))
    # the prior (centre 0.5 / 1500 = 3.3e-4) pulls D down on every voxel
    free = chains[None][:, 1].mean(1)
    assert np.all(g.mean(1) < free), int(np.sum(g.mean(1) >= free))
    assert np.median(free - g.mean(1)) > 5 * np.median(se(g)), (np.median(free - g.mean(1)),
                                                                np.median(se(g)))
