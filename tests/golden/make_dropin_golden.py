"""Generate the fixtures of two more of CUDIMOT's unchanged plugins for the
drop-in tests (toymodel, Ball_2_Sticks_1Shell_SSFP).

    python oracle/build_oracle.py --reference CUDIMOT_TREE
    python tests/golden/make_dropin_golden.py

Like make_golden.py: the plugins as compiled for the host into oracle/_ref/
(libref_<Model>.so, the FP64 oracle restatement of CUDIMOT's fitting loops
around the unchanged plugin) give the signals and LM fits of seeded inputs,
stored here as small .npz files that the GPU tests read.

toymodel: S = P0 exp(-P1 b), b in 0..3000 s/mm^2 (134 values), P0 ~
U(500, 1500), P1 ~ U(0.5e-3, 3e-3), Rician noise sigma = P0 / 30; LM from
(P0 = max signal, P1 = 1e-3).

Ball_2_Sticks_1Shell_SSFP (diffusion-weighted SSFP, CUDIMOT's parameter
layout: d, f1, th1, ph1, f2, th2, ph2, S0; CFP = bvec, b, TR, gradient
amplitude, gradient duration, flip angle, noise floor; FixP = T1, T2, B1):
12 non-diffusion rows and 120 directions, TR 0.028 s, 5.2 G/cm, 13 ms,
flip 24 deg (alternating 24/48 deg between directions), noise floor 0;
T1 ~ U(400, 700) ms, T2 ~ U(30, 70) ms, B1 ~ U(0.9, 1.1); d ~ U(2e-4,
8e-4), f1 ~ U(0.3, 0.7), f2 ~ U(0, min(f1, 1 - f1)), orientations uniform,
S0 ~ U(0.5e5, 1.5e5); Rician noise at SNR 40 relative to the mean signal.
The plugin's Partial_Derivatives is empty (the model is meant for MCMC), so
its fixture holds MCMC samples instead of an LM fit: 500 burn-in + 1000
jumps, every 10th kept, from the truth perturbed (fractions +-0.05, angles
+-0.1 rad, d x1.2, S0 x0.9).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cudimot_gb300 import capi, synth  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402


def toymodel(rng, n=48):
    b = np.linspace(0.0, 3000.0, 134)
    cfp = b[:, None].copy()
    P = np.stack([rng.uniform(500, 1500, n), rng.uniform(0.5e-3, 3e-3, n)], 1)
    F = np.zeros((n, 0))
    return P, cfp, F


def ssfp(rng, n=48):
    ndir = 120
    g = rng.standard_normal((ndir, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    g = np.concatenate([np.tile([1.0, 0.0, 0.0], (12, 1)), g])
    nm = g.shape[0]
    amp = np.concatenate([np.zeros(12), np.full(ndir, 5.2)])
    flip = np.where(np.arange(nm) % 2 == 0, 24.0, 48.0)
    cfp = np.stack([g[:, 0], g[:, 1], g[:, 2], np.where(amp > 0, 1000.0, 0.0), np.full(nm, 0.028),
                    amp, np.full(nm, 0.013), flip, np.zeros(nm)], 1)
    f1 = rng.uniform(0.3, 0.7, n)
    f2 = rng.uniform(0, 1, n) * np.minimum(f1, 1 - f1)
    th1, ph1 = synth.sphere_angles(n, rng)
    th2, ph2 = synth.sphere_angles(n, rng)
    P = np.stack([rng.uniform(2e-4, 8e-4, n), f1, th1, ph1, f2, th2, ph2,
                  rng.uniform(0.5e5, 1.5e5, n)], 1)
    F = np.stack([rng.uniform(400, 700, n), rng.uniform(30, 70, n), rng.uniform(0.9, 1.1, n)], 1)
    return P, cfp, F


def main():
    rng = np.random.default_rng(20240604)
    model = "toymodel"
    ref = Oracle(model, reference=True)
    P, cfp, F = toymodel(rng)
    S = ref.signal(P, cfp, F)
    meas = synth.rician(S, P[:, 0] / 30.0, rng)
    init = np.stack([meas.max(1), np.full(len(P), 1e-3)], 1)
    cfg = capi.model_cfg(model)
    lm, it, su, co = ref.levmar(cfg, meas, init, cfp, F)
    np.savez_compressed(os.path.join(HERE, f"fit_{model}.npz"), params=P, cfp=cfp, fixp=F,
                        signal=S, meas=meas, init=init, lm=lm, lm_iters=it, lm_cost=co)
    print(model, "done")

    model = "Ball_2_Sticks_1Shell_SSFP"
    ref = Oracle(model, reference=True)
    P, cfp, F = ssfp(rng)
    S = ref.signal(P, cfp, F)
    meas = synth.rician(S, S.mean(1) / 40.0, rng)
    init = P.copy()
    init[:, 0] *= 1.2
    init[:, 1] += rng.uniform(-0.05, 0.05, len(P))
    init[:, 4] = np.clip(init[:, 4] + rng.uniform(-0.05, 0.05, len(P)), 0.0, None)
    for k in (2, 3, 5, 6):
        init[:, k] += rng.uniform(-0.1, 0.1, len(P))
    init[:, 7] *= 0.9
    cfg = capi.model_cfg(model, run_mcmc=1, nburn=500, njumps=1000, sampleevery=10, seed=12345)
    _, samples, _ = ref.mcmc(cfg, meas, init, cfp, F)
    np.savez_compressed(os.path.join(HERE, f"fit_{model}.npz"), params=P, cfp=cfp, fixp=F,
                        signal=S, meas=meas, init=init, samples=samples.astype(np.float32))
    print(model, "done", "posterior mean of d / truth (median)",
          float(np.median(samples[:, 0].mean(1) / P[:, 0])))


if __name__ == "__main__":
    main()
