"""Generate the golden fixtures that pin the oracle to CUDIMOT's own plugins.

    python oracle/build_oracle.py --reference CUDIMOT_TREE
    python tests/golden/make_golden.py

Runs CUDIMOT's unchanged plugins, compiled for the host into oracle/_ref/
(libref_<Model>.so), on seeded inputs and stores inputs and outputs here as
small .npz files; the tests read only these files (the reference tree is not
needed to run them):

  plugin_<Model>.npz  Predicted_Signal and Partial_Derivatives of the
                      reference plugin on 64 parameter vectors x 96
                      measurements (FP64);
  fit_<Model>.npz     grid search (Watson) and LM results of the oracle's
                      fitting loops driven by the reference plugin on
                      48 synthetic voxels.
Models: Ball_1_Stick, NODDI_Watson, DiffusionTensor, Ball_2_Sticks, NODDI_Bingham.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cudimot_gb300 import capi, synth  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402


def plugin_inputs(model, rng):
    cfp = synth.protocol(6, [(30, 1000.0), (30, 2000.0), (30, 3000.0)], rng)
    n = 64
    if model == "Ball_1_Stick":
        P = np.stack([rng.uniform(500, 1500, n), rng.uniform(0.3e-3, 3e-3, n),
                      rng.uniform(0.02, 0.95, n), rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)], 1)
        F = np.zeros((n, 0))
    elif model == "DiffusionTensor":
        lam = np.stack([rng.uniform(1e-3, 2.5e-3, n), rng.uniform(0.1e-3, 1e-3, n),
                        rng.uniform(0.1e-3, 1e-3, n)], 1)
        R = synth.random_rotations(n, rng)
        D = np.einsum("nij,nj,nkj->nik", R, lam, R)
        P = np.stack([rng.uniform(500, 1500, n), D[:, 0, 0], D[:, 0, 1], D[:, 0, 2], D[:, 1, 1],
                      D[:, 1, 2], D[:, 2, 2]], 1)
        F = np.zeros((n, 0))
    elif model == "Ball_2_Sticks":
        f1 = rng.uniform(0.05, 0.7, n)
        P = np.stack([rng.uniform(500, 1500, n), rng.uniform(0.3e-3, 3e-3, n), f1,
                      rng.uniform(-3, 3, n), rng.uniform(-3, 3, n), rng.uniform(0, 1, n) * (1 - f1),
                      rng.uniform(-3, 3, n), rng.uniform(-3, 3, n)], 1)
        F = np.zeros((n, 0))
    elif model == "NODDI_Bingham":
        k = np.exp(rng.uniform(np.log(0.3), np.log(64), n))
        P = np.stack([rng.uniform(0, 0.6, n), rng.uniform(0.05, 1, n), k,
                      rng.uniform(0, 1.1, n) * k, rng.uniform(-3, 3, n), rng.uniform(-3, 3, n),
                      rng.uniform(-3, 3, n)], 1)
        F = rng.uniform(500, 1500, (n, 1))
    else:
        k = np.concatenate([np.exp(rng.uniform(np.log(1e-3), np.log(64), n - 6)),
                            [0.0, 0.2, 2.0, 5.0, 12.0, 40.0]])
        P = np.stack([rng.uniform(0, 1, n), rng.uniform(0, 1, n), k, rng.uniform(-3, 3, n),
                      rng.uniform(-3, 3, n)], 1)
        F = rng.uniform(500, 1500, (n, 1))
    return P, cfp, F


def watson_exact(P, cfp, S0):
    """NODDI-Watson by quadrature: Watson moments and Legendre-Gaussian
    integrals from scipy.integrate.quad (the kappa <= 0.4 series and
    kappa > 30 fits of the model definition are kept), for pinning where the
    reference plugin's own numerics lose precision."""
    from scipy import integrate, special
    Dpar, Diso = 0.0017, 0.003
    fits = [[7.52308, 0.411538, -0.214588, 0.0784091, -0.023981, 0.00731537, -0.0026467],
            [8.93718, 1.62147, -0.733421, 0.191568, -0.0202906, -0.00779095, 0.00574847],
            [8.87905, 3.35689, -1.15935, 0.0673053, 0.121857, -0.066642, 0.0180215],
            [7.84352, 5.03178, -1.0193, -0.426362, 0.328816, -0.0688176, -0.0229398],
            [6.30113, 6.09914, -0.16088, -1.05578, 0.338069, 0.0937157, -0.106935],
            [4.65678, 6.30069, 1.13754, -1.38393, -0.0134758, 0.331686, -0.105954]]
    q = lambda f: integrate.quad(f, 0, 1, epsabs=0, epsrel=1e-12, limit=200)[0]

    def moments(k):
        Z = q(lambda t: np.exp(k * (t * t - 1)))
        return [q(lambda t: special.eval_legendre(2 * l, t) * np.exp(k * (t * t - 1))) / Z
                for l in range(7)]

    def coeffs(k):
        if k > 30:
            L = np.log(k / 30.0)
            return [2 * np.sqrt(np.pi)] + [sum(c * L ** j for j, c in enumerate(f)) for f in fits]
        if k <= 0.4:
            sp = np.sqrt(np.pi)
            return [2 * sp, (4 / 3 * k + 8 / 63 * k ** 2) * np.sqrt(np.pi / 5),
                    (8 / 21 * k ** 2 + 32 / 693 * k ** 3) * sp * 0.2,
                    (16 / 693 * k ** 3 + 32 / 10395 * k ** 4) * np.sqrt(np.pi / 13),
                    32 / 19305 * k ** 4 * np.sqrt(np.pi / 17),
                    64 * np.sqrt(np.pi / 21) * k ** 5 / 692835,
                    128 * sp * k ** 6 / 152108775]
        m = moments(k)
        return [2 * np.sqrt(np.pi) * np.sqrt(4 * l + 1) * m[l] for l in range(7)]

    def lgi(x):
        if x <= 0.05:
            return [2 - 2 * x / 3 + x ** 2 / 5 - x ** 3 / 21 + x ** 4 / 108,
                    -4 * x / 15 + 4 * x ** 2 / 35 - 2 * x ** 3 / 63 + 2 * x ** 4 / 297,
                    8 * x ** 2 / 315 - 8 * x ** 3 / 693 + 4 * x ** 4 / 1287,
                    -16 * x ** 3 / 9009 + 16 * x ** 4 / 19305, 32 * x ** 4 / 328185,
                    -64 * x ** 5 / 14549535, 128 * x ** 6 / 760543875]
        return [2 * q(lambda t: special.eval_legendre(2 * l, t) * np.exp(-x * t * t)) for l in range(7)]

    lg = {b: lgi(b * Dpar) for b in np.unique(cfp[:, 3])}
    out = np.zeros((P.shape[0], cfp.shape[0]))
    for i, (fiso, fin, k, th, ph) in enumerate(P):
        c = coeffs(k)
        p2 = (moments(k)[1] if k >= 1e-5 else 2 * k / 15 + 4 * k * k / 315) if k <= 30 else None
        if p2 is None:  # kappa > 30: exact <t^2> from the Dawson function
            s = np.sqrt(k)
            r1 = (s / special.dawsn(s) - 1) / (2 * k)
            p2 = (3 * r1 - 1) / 2
        dperp = Dpar * (1 - fin)
        dperp_eq = dperp + (Dpar - dperp) * (1 - p2) / 3
        dd = (Dpar - dperp) * p2
        v = np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
        for m, row in enumerate(cfp):
            b = row[3]
            xv = row[:3] @ v
            E = np.exp(-b * (dd * xv * xv + dperp_eq))
            x = min(max(xv, -1.0), 1.0)
            I = sum(lg[b][l] * c[l] * np.sqrt((l + 0.25) / np.pi) * special.eval_legendre(2 * l, x)
                    for l in range(7))
            I = 0.5 * (I if I >= 0 else 1e-3)
            out[i, m] = S0[i, 0] * ((1 - fiso) * ((1 - fin) * E + fin * I) + fiso * np.exp(-b * Diso))
    return out


def main():
    rng = np.random.default_rng(20240601)
    for model in ("Ball_1_Stick", "NODDI_Watson"):
        ref = Oracle(model, reference=True)
        P, cfp, F = plugin_inputs(model, rng)
        S, J = ref.signal(P, cfp, F, jac=True)
        extra = {}
        if model == "NODDI_Watson":
            extra["signal_exact"] = watson_exact(P, cfp, F)
        np.savez_compressed(os.path.join(HERE, f"plugin_{model}.npz"), params=P, cfp=cfp,
                            fixp=F, signal=S, jacobian=J, **extra)
        # fitting loops driven by the reference plugin
        if model == "Ball_1_Stick":
            wl = synth.ball_1_stick(48, seed=77)
            cfg = capi.model_cfg(model)
            lm, it, su, co = ref.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
            np.savez_compressed(os.path.join(HERE, f"fit_{model}.npz"), cfp=wl.cfp, meas=wl.meas,
                                init=wl.init, fixp=wl.fixp, lm=lm, lm_iters=it, lm_cost=co)
        else:
            wl = synth.noddi_watson(48, seed=77,
                                    signal_fn=lambda t, c, s0: ref.signal(t, c, s0[:, None]))
            cfg = capi.model_cfg(model, grid=wl.grid)
            gs, best, bc = ref.gridsearch(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
            lm, it, su, co = ref.levmar(cfg, wl.meas, gs, wl.cfp, wl.fixp)
            np.savez_compressed(os.path.join(HERE, f"fit_{model}.npz"), cfp=wl.cfp, meas=wl.meas,
                                init=wl.init, fixp=wl.fixp, gs=gs, gs_best=best, gs_cost=bc,
                                lm=lm, lm_iters=it, lm_cost=co)
        print(model, "done")
    # models added later draw from their own stream (earlier fixtures unchanged)
    rng = np.random.default_rng(20240602)
    makers = {"DiffusionTensor": synth.diffusion_tensor, "Ball_2_Sticks": synth.ball_2_sticks}
    for model in ("DiffusionTensor", "Ball_2_Sticks"):
        ref = Oracle(model, reference=True)
        P, cfp, F = plugin_inputs(model, rng)
        S, J = ref.signal(P, cfp, F, jac=True)
        np.savez_compressed(os.path.join(HERE, f"plugin_{model}.npz"), params=P, cfp=cfp,
                            fixp=F, signal=S, jacobian=J)
        wl = makers[model](48, seed=77)
        cfg = capi.model_cfg(model)
        lm, it, su, co = ref.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
        np.savez_compressed(os.path.join(HERE, f"fit_{model}.npz"), cfp=wl.cfp, meas=wl.meas,
                            init=wl.init, fixp=wl.fixp, lm=lm, lm_iters=it, lm_cost=co)
        print(model, "done")
    rng = np.random.default_rng(20240603)
    model = "NODDI_Bingham"
    ref = Oracle(model, reference=True)
    P, cfp, F = plugin_inputs(model, rng)
    S, J = ref.signal(P, cfp, F, jac=True)
    np.savez_compressed(os.path.join(HERE, f"plugin_{model}.npz"), params=P, cfp=cfp, fixp=F,
                        signal=S, jacobian=J)
    wl = synth.noddi_bingham(48, seed=77, signal_fn=lambda t, c, s0: ref.signal(t, c, s0[:, None]))
    cfg = capi.model_cfg(model, grid=wl.grid)
    gs, best, bc = ref.gridsearch(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    lm, it, su, co = ref.levmar(cfg, wl.meas, gs, wl.cfp, wl.fixp)
    np.savez_compressed(os.path.join(HERE, f"fit_{model}.npz"), cfp=wl.cfp, meas=wl.meas,
                        init=wl.init, fixp=wl.fixp, gs=gs, gs_best=best, gs_cost=bc, lm=lm,
                        lm_iters=it, lm_cost=co)
    print(model, "done")


if __name__ == "__main__":
    main()
