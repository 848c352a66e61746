"""Rician-likelihood MCMC (CUDIMOT's --rician: tau sampled with the
parameters, log I0 of Abramowitz & Stegun 9.8.1/9.8.2, MCMC.cu:32-49 and
254-324) and the Rician BIC/AIC (BIC_AIC.cu:160-201):
  * posterior means of the parameters and of tau agree with the FP64 CPU
    oracle's chain (different random streams) within Monte Carlo error;
  * the same against CUDIMOT's own Rician MCMC kernel;
  * BIC/AIC from given samples and tau equal the oracle's (5e-6 relative)."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import capi
from tests.helpers import b1s, oracle

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def _z(g, r):
    def se(x):
        b = x.reshape(x.shape[0], 10, -1).mean(-1)
        return b.std(1, ddof=1) / np.sqrt(10)
    return (g.mean(-1) - r.mean(-1)) / np.sqrt(se(g) ** 2 + se(r) ** 2 + 1e-30)


def _run_ours(wl, start, cfg, cuda):
    lib = capi.Cudimot("Ball_1_Stick", cfg)
    ns = cfg.njumps // cfg.sampleevery
    s = torch.zeros(wl.nvox, 5, ns, dtype=torch.float64, device=cuda)
    tau = torch.zeros(wl.nvox, ns, dtype=torch.float64, device=cuda)
    lib.mcmc(T(wl.meas, cuda), T(start, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda), s, tau)
    torch.cuda.synchronize()
    return s.cpu().numpy(), tau.cpu().numpy()


def test_rician_mcmc_matches_oracle(built, cuda):
    wl = b1s(256, seed=41)
    o = oracle("Ball_1_Stick")
    cfg = capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=500, njumps=2000, sampleevery=10,
                         rician=1)
    start, _, _, _ = o.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    g, gt = _run_ours(wl, start, cfg, cuda)
    cfg2 = capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=500, njumps=2000, sampleevery=10,
                          rician=1, seed=777)
    _, r, rt = o.mcmc(cfg2, wl.meas, start, wl.cfp, wl.fixp)
    assert np.all(gt > 0)
    for x, y in [(g[:, p], r[:, p]) for p in (0, 1, 2)] + [(gt, rt)]:
        z = _z(x, y)
        assert abs(np.median(z)) < 0.5, np.median(z)
        assert np.mean(np.abs(z) < 4) > 0.95, np.mean(np.abs(z) < 4)


def test_rician_mcmc_matches_reference_kernels(built, cuda):
    rk = pytest.importorskip("oracle.refkernels.refkernels")
    if not rk.available("Ball_1_Stick"):
        pytest.skip("reference cubins not built")
    wl = b1s(512, seed=42)
    o = oracle("Ball_1_Stick")
    cfg = capi.model_cfg("Ball_1_Stick", run_mcmc=1, nburn=500, njumps=2000, sampleevery=10,
                         rician=1)
    start, _, _, _ = o.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    g, gt = _run_ours(wl, start, cfg, cuda)
    ref = rk.RefKernels("Ball_1_Stick", 5)
    sr = torch.zeros(wl.nvox, 5, 200, dtype=torch.float64, device=cuda)
    tr = torch.zeros(wl.nvox, 200, dtype=torch.float64, device=cuda)
    ref.mcmc(cfg, T(wl.meas, cuda), T(start, cuda), T(wl.cfp, cuda), None, sr, tr)
    torch.cuda.synchronize()
    r, rt = sr.cpu().numpy(), tr.cpu().numpy()
    for x, y in [(g[:, p], r[:, p]) for p in (0, 1, 2)] + [(gt, rt)]:
        z = _z(x, y)
        assert abs(np.median(z)) < 0.5, np.median(z)
        assert np.mean(np.abs(z) < 4) > 0.95, np.mean(np.abs(z) < 4)


def test_rician_bic_aic(built, cuda):
    wl = b1s(1000, seed=43)
    o = oracle("Ball_1_Stick")
    rng = np.random.default_rng(1)
    samples = wl.truth[:, :, None] * (1 + 0.01 * rng.standard_normal((wl.nvox, 5, 4)))
    tau = rng.uniform(1e-5, 1e-4, (wl.nvox, 4))
    lib = capi.Cudimot("Ball_1_Stick", capi.model_cfg("Ball_1_Stick", rician=1, run_mcmc=1))
    bic = torch.zeros(wl.nvox, dtype=torch.float64, device=cuda)
    aic = torch.zeros_like(bic)
    lib.bic_aic(T(wl.meas, cuda), T(samples, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda), bic, aic,
                tau=T(tau, cuda))
    torch.cuda.synchronize()
    rb, ra = o.bic_aic(wl.meas, samples, wl.cfp, wl.fixp, tau=tau, rician=True)
    np.testing.assert_allclose(bic.cpu().numpy(), rb, rtol=5e-6)
    np.testing.assert_allclose(aic.cpu().numpy(), ra, rtol=5e-6)
