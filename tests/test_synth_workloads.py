"""The seeded synthetic workloads that stand in for acquisitions: shapes,
protocols, parameter ranges and reproducibility of the benchmark
configurations (C0 Ball_1_Stick 134 measurements; C1 NODDI-Watson 288
measurements with the 968-combination grid; C4's DiffusionTensor 71 and
Ball_2_Sticks 134 measurements; C2 NODDI-Bingham on the C1 protocol).
"""
import numpy as np

from cudimot_gb300 import synth
from tests.helpers import bingham, watson


def _shells(cfp):
    b, counts = np.unique(cfp[:, 3], return_counts=True)
    return dict(zip(b.tolist(), counts.tolist()))


def _unit(cfp):
    g = cfp[cfp[:, 3] > 0, :3]
    return np.allclose(np.linalg.norm(g, axis=1), 1.0)


def test_c0_ball_1_stick():
    wl = synth.ball_1_stick(500)
    assert wl.meas.shape == (500, 134) and _shells(wl.cfp) == {0.0: 6, 1000.0: 64, 2000.0: 64}
    assert _unit(wl.cfp)
    S0, d, f = wl.truth[:, 0], wl.truth[:, 1], wl.truth[:, 2]
    assert S0.min() >= 500 and S0.max() <= 1500
    assert d.min() >= 0.5e-3 and d.max() <= 2.5e-3 and f.min() >= 0.05 and f.max() <= 0.8
    assert np.all(wl.meas > 0)


def test_c1_noddi_watson(built):
    wl = watson(400)
    assert wl.meas.shape == (400, 288)
    assert _shells(wl.cfp) == {0.0: 18, 1000.0: 90, 2000.0: 90, 3000.0: 90} and _unit(wl.cfp)
    fiso, fin, kappa = wl.truth[:, 0], wl.truth[:, 1], wl.truth[:, 2]
    assert fiso.min() >= 0 and fiso.max() <= 0.3 and fin.min() >= 0.2 and fin.max() <= 0.8
    assert kappa.min() >= 0.5 and kappa.max() <= 32
    # FixP S0 = mean of the noisy b = 0 signals
    np.testing.assert_allclose(wl.fixp[:, 0], wl.meas[:, wl.cfp[:, 3] == 0].mean(axis=1))
    combs = np.prod([len(v) for v in wl.grid.values()])
    assert combs == 968 and sorted(wl.grid) == [0, 1, 2]


def test_c4_models():
    dt = synth.diffusion_tensor(300)
    assert dt.meas.shape == (300, 71) and _shells(dt.cfp) == {0.0: 7, 1000.0: 64}
    b2 = synth.ball_2_sticks(300)
    assert b2.meas.shape == (300, 134)
    f1, f2 = b2.truth[:, 2], b2.truth[:, 5]
    assert f1.min() >= 0.2 and f1.max() <= 0.6 and np.all(f2 <= f1)


def test_c2_bingham_on_the_c1_protocol(built):
    wl = bingham(200)
    assert wl.meas.shape == (200, 288)
    assert _shells(wl.cfp) == {0.0: 18, 1000.0: 90, 2000.0: 90, 3000.0: 90}


def test_seeded_and_reproducible(built):
    a, b = synth.ball_1_stick(100), synth.ball_1_stick(100)
    assert np.array_equal(a.meas, b.meas) and np.array_equal(a.cfp, b.cfp)
    c = synth.ball_1_stick(100, seed=1)
    assert not np.array_equal(a.meas, c.meas)
    w1, w2 = watson(50), watson(50)
    assert np.array_equal(w1.meas, w2.meas) and np.array_equal(w1.init, w2.init)
