"""GPU utilities against numpy references:
  * the log-linear tensor fit (S0, eigenvalues, FA, MD to 1e-9 relative;
    V1/V2 axes to 1e-6 rad; psi as the angle of V2 in the fibre-orthogonal
    plane);
  * sample means/SDs, dyadic vectors (principal eigenvector of the mean
    dyad, sign-free) with their dispersion, OD = 2/pi atan(1/kappa)."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import synth, utils

pytestmark = pytest.mark.gpu


def test_dti_fit_matches_numpy(built, cuda):
    wl = synth.diffusion_tensor(3000, seed=2)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=cuda)  # noqa
    out = utils.dti_fit(t(wl.meas), t(wl.cfp[:, :3]), t(wl.cfp[:, 3])).cpu().numpy()
    S0, tens, w, V = synth.dti_fit(wl.meas, wl.cfp)
    np.testing.assert_allclose(out[:, 0], S0, rtol=1e-9)
    np.testing.assert_allclose(out[:, 1:4], w, rtol=1e-8, atol=1e-12)
    for k, col in ((0, 4), (1, 7)):
        dot = np.abs(np.sum(out[:, col:col + 3] * V[:, :, k], 1))
        assert np.all(dot > 1 - 1e-9)
    md = w.mean(1)
    fa = np.sqrt(1.5 * np.sum((w - md[:, None]) ** 2, 1) / np.sum(w * w, 1))
    np.testing.assert_allclose(out[:, 10], fa, rtol=1e-8)
    np.testing.assert_allclose(out[:, 11], md, rtol=1e-8)
    psi = synth.dti_psi(V, out[:, 12], out[:, 13])
    d = np.angle(np.exp(2j * (out[:, 16] - psi)))   # psi is an axis angle (mod pi)
    assert np.max(np.abs(d)) < 1e-6


def test_stats_dyads_od(built, cuda):
    rng = np.random.default_rng(4)
    n, ns = 500, 60
    th0, ph0 = synth.sphere_angles(n, rng)
    s = np.zeros((n, 5, ns))
    s[:, 0] = rng.uniform(0.1, 0.3, (n, ns))
    s[:, 2] = rng.uniform(1, 10, (n, ns))
    s[:, 3] = th0[:, None] + 0.05 * rng.standard_normal((n, ns))
    s[:, 4] = ph0[:, None] + 0.05 * rng.standard_normal((n, ns))
    st = torch.as_tensor(s, device=cuda)
    mean, sd = utils.sample_stats(st)
    np.testing.assert_allclose(mean.cpu().numpy(), s.mean(2), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(sd.cpu().numpy(), s.std(2, ddof=1), rtol=1e-10, atol=1e-12)
    dy = utils.dyads(st, 3, 4).cpu().numpy()
    v = np.stack([np.sin(s[:, 3]) * np.cos(s[:, 4]), np.sin(s[:, 3]) * np.sin(s[:, 4]), np.cos(s[:, 3])], -1)
    T = np.einsum("nsi,nsj->nij", v, v) / ns
    w, E = np.linalg.eigh(T)
    assert np.all(np.abs(np.sum(dy[:, :3] * E[:, :, 2], 1)) > 1 - 1e-9)
    np.testing.assert_allclose(dy[:, 3], 1 - w[:, 2], atol=1e-10)
    od = utils.od_from_kappa(mean[:, 2]).cpu().numpy()
    np.testing.assert_allclose(od, 2 / np.pi * np.arctan(1 / s[:, 2].mean(1)), rtol=1e-12)
