"""Seeded synthetic diffusion-MRI workloads.

There is no public dataset for CUDIMOT's path; these generators stand in for
real acquisitions with the shapes, parameter ranges and noise of the
benchmark configurations:

* protocols: b=0 volumes plus shells of directions drawn uniformly on the
  sphere (normalised N(0, I3) draws); rows of CFP are (gx, gy, gz, b) as
  CUDIMOT's bvecs/bvals CFP files give them (Parameters.cu:105-121);
* true parameters drawn from each configuration's ranges;
* Rician noise y = |S + sigma (n1 + i n2)|.

Streams come from numpy's PCG64 seeded with 8219 (CUDIMOT's default
--seed), one spawned child per purpose, so every array is reproducible.
"""
from __future__ import annotations

import dataclasses
import numpy as np

DEFAULT_SEED = 8219


def _streams(seed: int, n: int):
    ss = np.random.SeedSequence(seed)
    return [np.random.Generator(np.random.PCG64(s)) for s in ss.spawn(n)]


def protocol(n_b0: int, shells, rng) -> np.ndarray:
    """CFP [nmeas][4] = (gx, gy, gz, b): n_b0 rows of b=0 then each shell."""
    rows = [np.tile([1.0, 0.0, 0.0, 0.0], (n_b0, 1))]
    for n, b in shells:
        g = rng.standard_normal((n, 3))
        g /= np.linalg.norm(g, axis=1, keepdims=True)
        rows.append(np.concatenate([g, np.full((n, 1), float(b))], axis=1))
    return np.ascontiguousarray(np.concatenate(rows, axis=0))


def rician(signal: np.ndarray, sigma, rng) -> np.ndarray:
    sigma = np.asarray(sigma, dtype=np.float64)
    if sigma.ndim == 1:
        sigma = sigma[:, None]
    n1 = rng.standard_normal(signal.shape)
    n2 = rng.standard_normal(signal.shape)
    return np.sqrt((signal + sigma * n1) ** 2 + (sigma * n2) ** 2)


def sphere_angles(n, rng):
    th = np.arccos(rng.uniform(-1.0, 1.0, n))
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    return th, ph


@dataclasses.dataclass
class Workload:
    name: str
    model: str
    cfp: np.ndarray          # [nmeas][4]
    meas: np.ndarray         # [nvox][nmeas]
    truth: np.ndarray        # [nvox][NPARAMS]
    init: np.ndarray         # [nvox][NPARAMS]
    fixp: np.ndarray         # [nvox][FixP_Tsize] (may have 0 columns)
    grid: dict | None = None  # {param index: values}

    @property
    def nvox(self):
        return self.meas.shape[0]

    @property
    def nmeas(self):
        return self.meas.shape[1]


def b1s_signal(P, cfp):
    """Ball & 1 Stick signal, numpy, for generating data."""
    S0, d, f, th, ph = (P[:, i:i + 1] for i in range(5))
    g = cfp[None, :, :3]
    b = cfp[None, :, 3]
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=-1)
    gv = np.sum(g * v, axis=-1)
    return S0 * ((1 - f) * np.exp(-b * d) + f * np.exp(-b * d * gv * gv))


def dti_fit(meas, cfp):
    """Log-linear tensor fit per voxel -> (S0 [n], tensor entries [n][6] in
    the order Dxx, Dxy, Dxz, Dyy, Dyz, Dzz, eigenvalues [n][3] descending,
    eigenvectors [n][3][3] with column k the k-th eigenvector)."""
    g = cfp[:, :3]
    b = cfp[:, 3]
    X = np.stack([np.ones_like(b), -b * g[:, 0] ** 2, -2 * b * g[:, 0] * g[:, 1],
                  -2 * b * g[:, 0] * g[:, 2], -b * g[:, 1] ** 2, -2 * b * g[:, 1] * g[:, 2],
                  -b * g[:, 2] ** 2], axis=1)
    y = np.log(np.maximum(meas, 1e-3))
    coef, *_ = np.linalg.lstsq(X, y.T, rcond=None)
    coef = coef.T
    S0 = np.exp(coef[:, 0])
    t = coef[:, 1:]
    D = np.zeros((meas.shape[0], 3, 3))
    D[:, 0, 0], D[:, 1, 1], D[:, 2, 2] = t[:, 0], t[:, 3], t[:, 5]
    D[:, 0, 1] = D[:, 1, 0] = t[:, 1]
    D[:, 0, 2] = D[:, 2, 0] = t[:, 2]
    D[:, 1, 2] = D[:, 2, 1] = t[:, 4]
    w, V = np.linalg.eigh(D)
    return S0, t, w[:, ::-1].copy(), V[:, :, ::-1].copy()


def _angles(v):
    return np.arccos(np.clip(v[:, 2], -1.0, 1.0)), np.arctan2(v[:, 1], v[:, 0])


def dti_init(meas, cfp):
    """Log-linear tensor fit per voxel -> (S0, mean diffusivity, FA, V1).

    Stands in for dtifit + utils/cart2spherical.cc, which CUDIMOT's
    pipelines use to initialise orientations (Pipeline_NODDI_Watson.sh)."""
    g = cfp[:, :3]
    b = cfp[:, 3]
    X = np.stack([np.ones_like(b), -b * g[:, 0] ** 2, -b * g[:, 1] ** 2, -b * g[:, 2] ** 2,
                  -2 * b * g[:, 0] * g[:, 1], -2 * b * g[:, 0] * g[:, 2],
                  -2 * b * g[:, 1] * g[:, 2]], axis=1)
    y = np.log(np.maximum(meas, 1e-3))
    coef, *_ = np.linalg.lstsq(X, y.T, rcond=None)
    coef = coef.T
    S0 = np.exp(coef[:, 0])
    D = np.zeros((meas.shape[0], 3, 3))
    D[:, 0, 0], D[:, 1, 1], D[:, 2, 2] = coef[:, 1], coef[:, 2], coef[:, 3]
    D[:, 0, 1] = D[:, 1, 0] = coef[:, 4]
    D[:, 0, 2] = D[:, 2, 0] = coef[:, 5]
    D[:, 1, 2] = D[:, 2, 1] = coef[:, 6]
    w, V = np.linalg.eigh(D)
    v1 = V[:, :, 2]
    md = w.mean(axis=1)
    fa = np.sqrt(1.5 * np.sum((w - md[:, None]) ** 2, axis=1) / np.maximum(np.sum(w * w, axis=1), 1e-30))
    th = np.arccos(np.clip(v1[:, 2], -1.0, 1.0))
    ph = np.arctan2(v1[:, 1], v1[:, 0])
    return S0, md, fa, th, ph


def ball_1_stick(nvox=10_000, seed=DEFAULT_SEED) -> Workload:
    """Ball & 1 Stick, plain LM: 6 b0 + 64@1000 + 64@2000 (134 measurements),
    S0~U(500,1500), d~U(0.5e-3,2.5e-3), f~U(0.05,0.8), orientation uniform,
    Rician sigma = S0/30; LM initialised from a log-linear DTI fit."""
    r_proto, r_par, r_noise = _streams(seed, 3)
    cfp = protocol(6, [(64, 1000.0), (64, 2000.0)], r_proto)
    S0 = r_par.uniform(500, 1500, nvox)
    d = r_par.uniform(0.5e-3, 2.5e-3, nvox)
    f = r_par.uniform(0.05, 0.8, nvox)
    th, ph = sphere_angles(nvox, r_par)
    truth = np.stack([S0, d, f, th, ph], axis=1)
    meas = rician(b1s_signal(truth, cfp), S0 / 30.0, r_noise)
    s0i, md, fa, thi, phi = dti_init(meas, cfp)
    init = np.stack([s0i, np.clip(md, 1e-5, 5e-3), np.clip(fa, 0.05, 0.95), thi, phi], axis=1)
    return Workload("ball_1_stick_lm", "Ball_1_Stick", cfp, meas, truth, init,
                    np.zeros((nvox, 0)))


def watson_truth(nvox, rng):
    fiso = rng.uniform(0.0, 0.3, nvox)
    fin = rng.uniform(0.2, 0.8, nvox)
    kappa = np.exp(rng.uniform(np.log(0.5), np.log(32.0), nvox))
    th, ph = sphere_angles(nvox, rng)
    S0 = rng.uniform(500, 1500, nvox)
    return np.stack([fiso, fin, kappa, th, ph], axis=1), S0


WATSON_GRID = {0: np.round(np.arange(0.0, 1.0001, 0.1), 10),
               1: np.round(np.arange(0.0, 1.0001, 0.1), 10),
               2: np.arange(1.0, 8.0001, 1.0)}


def noddi_watson(nvox=200_000, seed=DEFAULT_SEED, signal_fn=None, snr=20.0) -> Workload:
    """NODDI-Watson, grid search -> LM -> MCMC: 18 b0 + 90 directions at each
    of b = 1000/2000/3000 (288 measurements); fiso~U(0,0.3),
    fintra~U(0.2,0.8), kappa log-uniform in [0.5,32], orientation uniform,
    S0~U(500,1500); Rician noise at SNR 20 (sigma = S0/20). FixP S0 = mean of
    the noisy b=0 signals; grid fiso, fintra in 0:0.1:1 and kappa 1..8
    (968 combinations); orientation initialised from a DTI fit.

    signal_fn(params [nvox][5], cfp, S0 [nvox]) -> [nvox][nmeas] computes the
    noiseless signal (the oracle's Predicted_Signal)."""
    r_proto, r_par, r_noise = _streams(seed, 3)
    cfp = protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], r_proto)
    truth, S0 = watson_truth(nvox, r_par)
    if signal_fn is None:
        raise ValueError("noddi_watson needs signal_fn (the model's Predicted_Signal)")
    clean = signal_fn(truth, cfp, S0)
    meas = rician(clean, S0 / snr, r_noise)
    b0 = cfp[:, 3] == 0
    s0_est = meas[:, b0].mean(axis=1)
    _, _, _, thi, phi = dti_init(meas, cfp)
    init = np.stack([np.full(nvox, 0.4), np.full(nvox, 0.8), np.full(nvox, 5.0), thi, phi], axis=1)
    return Workload("noddi_watson_gs_lm_mcmc", "NODDI_Watson", cfp, meas, truth, init,
                    s0_est[:, None].copy(), grid=WATSON_GRID)


def dt_signal(P, cfp):
    """Diffusion-tensor signal S0 exp(-b g^T D g), numpy."""
    g = cfp[:, :3]
    b = cfp[:, 3]
    q = np.stack([b * g[:, 0] ** 2, 2 * b * g[:, 0] * g[:, 1], 2 * b * g[:, 0] * g[:, 2],
                  b * g[:, 1] ** 2, 2 * b * g[:, 1] * g[:, 2], b * g[:, 2] ** 2], axis=1)
    return P[:, :1] * np.exp(-(P[:, 1:7] @ q.T))


def random_rotations(n, rng):
    """Uniform random rotation matrices (QR of Gaussian matrices, sign-fixed)."""
    A = rng.standard_normal((n, 3, 3))
    Q, R = np.linalg.qr(A)
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    det = np.linalg.det(Q)
    Q[:, :, 0] *= det[:, None]
    return Q


def diffusion_tensor(nvox=400_000, seed=DEFAULT_SEED, snr=25.0) -> Workload:
    """Diffusion tensor, LM (+ MCMC): 7 b0 + 64@1000 (71 measurements);
    eigenvalues l1~U(1.2e-3,2e-3), l2,l3~U(0.2e-3,0.8e-3) under a uniform
    random rotation, S0~U(500,1500); Rician noise sigma = S0/snr; initialised
    from the log-linear tensor fit."""
    r_proto, r_par, r_noise = _streams(seed, 3)
    cfp = protocol(7, [(64, 1000.0)], r_proto)
    S0 = r_par.uniform(500, 1500, nvox)
    lam = np.stack([r_par.uniform(1.2e-3, 2e-3, nvox), r_par.uniform(0.2e-3, 0.8e-3, nvox),
                    r_par.uniform(0.2e-3, 0.8e-3, nvox)], axis=1)
    R = random_rotations(nvox, r_par)
    D = np.einsum("nij,nj,nkj->nik", R, lam, R)
    truth = np.stack([S0, D[:, 0, 0], D[:, 0, 1], D[:, 0, 2], D[:, 1, 1], D[:, 1, 2], D[:, 2, 2]],
                     axis=1)
    meas = rician(dt_signal(truth, cfp), S0 / snr, r_noise)
    s0i, t, _, _ = dti_fit(meas, cfp)
    init = np.concatenate([np.clip(s0i, 1.0, 9000.0)[:, None], t], axis=1)
    for k in (1, 4, 6):
        init[:, k] = np.clip(init[:, k], 1e-6, 9e-3)
    return Workload("diffusion_tensor", "DiffusionTensor", cfp, meas, truth, init,
                    np.zeros((nvox, 0)))


def b2s_signal(P, cfp):
    """Ball & 2 Sticks signal, numpy."""
    S0, d, f1, t1, p1, f2, t2, p2 = (P[:, i:i + 1] for i in range(8))
    g = cfp[None, :, :3]
    b = cfp[None, :, 3]

    def dot(th, ph):
        v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=-1)
        return np.sum(g * v, axis=-1)

    x1, x2 = dot(t1, p1), dot(t2, p2)
    return S0 * ((1 - f1 - f2) * np.exp(-b * d) + f1 * np.exp(-b * d * x1 * x1) +
                 f2 * np.exp(-b * d * x2 * x2))


def ball_2_sticks(nvox=300_000, seed=DEFAULT_SEED, snr=25.0) -> Workload:
    """Ball & 2 Sticks, LM (+ MCMC): 6 b0 + 64@1000 + 64@2000 (134
    measurements); S0~U(500,1500), d~U(0.5e-3,2.5e-3), f1~U(0.2,0.6),
    f2~U(0,f1), orientations uniform; Rician sigma = S0/snr. Initialised as
    CUDIMOT's Ball_2_Sticks pipeline does from dtifit: S0, L1, FA, V1, FA/4,
    V2."""
    r_proto, r_par, r_noise = _streams(seed, 3)
    cfp = protocol(6, [(64, 1000.0), (64, 2000.0)], r_proto)
    S0 = r_par.uniform(500, 1500, nvox)
    d = r_par.uniform(0.5e-3, 2.5e-3, nvox)
    f1 = r_par.uniform(0.2, 0.6, nvox)
    f2 = r_par.uniform(0.0, 1.0, nvox) * f1
    t1, p1 = sphere_angles(nvox, r_par)
    t2, p2 = sphere_angles(nvox, r_par)
    truth = np.stack([S0, d, f1, t1, p1, f2, t2, p2], axis=1)
    meas = rician(b2s_signal(truth, cfp), S0 / snr, r_noise)
    s0i, _, w, V = dti_fit(meas, cfp)
    md = w.mean(axis=1)
    fa = np.sqrt(1.5 * np.sum((w - md[:, None]) ** 2, axis=1) / np.maximum(np.sum(w * w, axis=1), 1e-30))
    fa = np.clip(fa, 0.02, 0.95)
    th1, ph1 = _angles(V[:, :, 0])
    th2, ph2 = _angles(V[:, :, 1])
    init = np.stack([np.clip(s0i, 1.0, 9000.0), np.clip(w[:, 0], 1e-5, 9e-3), fa, th1, ph1,
                     fa / 4.0, th2, ph2], axis=1)
    return Workload("ball_2_sticks", "Ball_2_Sticks", cfp, meas, truth, init, np.zeros((nvox, 0)))


# Grid of CUDIMOT's NODDI-Bingham pipeline (fiso, fintra, kappa, beta):
# 5 x 10 x 17 x 13 = 11,050 combinations.
BINGHAM_GRID = {0: np.array([0.0, 0.05, 0.1, 0.2, 0.3]),
                1: np.array([0.3, 0.5, 0.6, 0.7, 0.75, 0.8, 0.85, 0.9, 0.95, 1.0]),
                2: np.array([0.5, 1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 15, 20, 25, 30, 40, 50], float),
                3: np.array([0.2, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 4.5, 6.5, 9, 12, 16, 20])}


def bingham_truth(nvox, rng):
    """NODDI-Watson parameters as noddi_watson draws them, plus
    beta = U(0, 0.9) kappa and psi ~ U(0, pi)."""
    P, S0 = watson_truth(nvox, rng)
    beta = rng.uniform(0.0, 0.9, nvox) * P[:, 2]
    psi = rng.uniform(0.0, np.pi, nvox)
    return np.stack([P[:, 0], P[:, 1], P[:, 2], beta, P[:, 3], P[:, 4], psi], axis=1), S0


def dti_psi(V, th, ph):
    """Fanning angle psi from the second tensor eigenvector, as
    utils/initialise_Psi.cc in CUDIMOT does: the angle of V2 in the plane
    orthogonal to the fibre, measured from the fanning direction at psi = 0."""
    v2 = V[:, :, 1]
    f0 = np.stack([-np.sin(ph), np.cos(ph), np.zeros_like(ph)], axis=1)       # psi = 0
    h0 = np.stack([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)], axis=1)
    return np.arctan2(-np.sum(v2 * h0, axis=1), np.sum(v2 * f0, axis=1))


def noddi_bingham(nvox=1_000_000, seed=DEFAULT_SEED, signal_fn=None, snr=20.0) -> Workload:
    """NODDI-Bingham precision study: the NODDI-Watson protocol (288
    measurements) and parameters plus beta = U(0,0.9) kappa and psi ~
    U(0, pi); Rician noise at SNR 20; S0 = mean noisy b=0 signal; theta,
    phi from a DTI fit and psi from its second eigenvector; grid of
    CUDIMOT's Bingham pipeline (11,050 combinations)."""
    r_proto, r_par, r_noise = _streams(seed, 3)
    cfp = protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], r_proto)
    truth, S0 = bingham_truth(nvox, r_par)
    if signal_fn is None:
        raise ValueError("noddi_bingham needs signal_fn (the model's Predicted_Signal)")
    meas = rician(signal_fn(truth, cfp, S0), S0 / snr, r_noise)
    b0 = cfp[:, 3] == 0
    s0_est = meas[:, b0].mean(axis=1)
    _, _, w, V = dti_fit(meas, cfp)
    thi, phi = _angles(V[:, :, 0])
    psi = dti_psi(V, thi, phi)
    init = np.stack([np.full(nvox, 0.2), np.full(nvox, 0.7), np.full(nvox, 5.0), np.full(nvox, 2.0),
                     thi, phi, psi], axis=1)
    return Workload("noddi_bingham_gs_lm_mcmc", "NODDI_Bingham", cfp, meas, truth, init,
                    s0_est[:, None].copy(), grid=BINGHAM_GRID)
