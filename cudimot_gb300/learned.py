"""Learned initialiser for the fitting path (no CUDIMOT counterpart).

A network (include/cdm_mlp.h) maps each voxel's S0-normalised signal to the
plugin's head (hooks MLP_Encode / MLP_Decode in modelfunctions.h): parameter
means and log standard deviations. The means seed LM in place of the grid
search, the standard deviations seed the MCMC proposal widths.

Training data are made by the method itself, all on the GPU:
  * `n_prior` voxels with parameters drawn from a prior, signals from the
    plugin's Predicted_Signal with Rician noise at SNR ~ U(snr_lo, snr_hi)
    (cdm_synth_signals), targets = the drawn parameters;
  * `n_lm` voxels drawn the same way and fitted by the plain path (grid
    search + LM), targets = the LM fits.
The network is trained with Adam on the Gaussian NLL (cdm_mlp_train_step).

`fit` runs the surrogate-initialised path: network -> LM -> refit of the
voxels the judge flags by the plain path (grid search + LM) -> MCMC. The
judge must not need the plain fit of every voxel (that would pay for the
grid search the network replaces), so by default it is a goodness-of-fit
test on the voxel's own data: the LM cost against (nmeas - nparams) times
the variance of the voxel's b = 0 signals, flagged above an upper quantile
of the F(nmeas - nparams, n_b0 - 1) distribution of that ratio for a good
fit. A caller that has the plain fit's cost anyway can pass it instead
(plain_cost, margin): the yardstick of the spec description.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import capi, mlp


def watson_prior(n, gen, device):
    """NODDI-Watson parameters and S0 as the benchmark draws them: fiso
    U(0,0.3), fintra U(0.2,0.8), kappa log-uniform [0.5,32], orientation
    uniform on the sphere, S0 U(500,1500)."""
    import torch
    u = torch.rand(n, 6, generator=gen, device=device, dtype=torch.float64)
    P = torch.empty(n, 5, dtype=torch.float64, device=device)
    P[:, 0] = 0.3 * u[:, 0]
    P[:, 1] = 0.2 + 0.6 * u[:, 1]
    P[:, 2] = torch.exp(math.log(0.5) + (math.log(32.0) - math.log(0.5)) * u[:, 2])
    P[:, 3] = torch.acos(1.0 - 2.0 * u[:, 3])
    P[:, 4] = 2.0 * math.pi * u[:, 4]
    S0 = (500.0 + 1000.0 * u[:, 5]).unsqueeze(1).contiguous()
    return P.contiguous(), S0


PRIORS = {"NODDI_Watson": watson_prior}


def he_init(dims, seed):
    """fp32 weights N(0, 2/fan_in) (output layer x0.1), zero biases."""
    rng = np.random.default_rng(seed)
    W, b = [], []
    for l in range(4):
        s = math.sqrt(2.0 / dims[l]) * (0.1 if l == 3 else 1.0)
        W.append((rng.standard_normal((dims[l + 1], dims[l])) * s).astype(np.float32))
        b.append(np.zeros(dims[l + 1], np.float32))
    return W, b


class LearnedInit:
    def __init__(self, model: str, cfp, grid=None, seed: int = 8219, mlp_cfg=None, device=None,
                 snr=(10.0, 50.0)):
        import torch
        self.torch = torch
        self.model = model
        self.dev = device or torch.device("cuda:0")
        self.cfp = torch.as_tensor(np.ascontiguousarray(cfp), dtype=torch.float64, device=self.dev)
        self.nmeas = self.cfp.shape[0]
        self.n_in = (self.nmeas + 7) // 8 * 8
        self.grid = grid
        self.seed = seed
        self.snr = snr
        self.lib = capi.Cudimot(model, capi.model_cfg(model))
        n_mu, n_sig, group = self.lib.mlp_head()
        self.n_mu = n_mu
        cfg = mlp_cfg or mlp.default_cfg()
        cfg.n_in = self.n_in
        cfg.n_mu, cfg.n_sig = n_mu, n_sig
        for j, g in enumerate(group):
            cfg.group[j] = g
        self.net = mlp.Mlp(cfg)
        self.net.set_params(*he_init(self.net.dims(), seed))
        self.history = []
        self.train_seconds = 0.0

    # ---------------------------------------------------------------- data
    def synth(self, n, seed, snr=None, meas=False):
        """n prior draws -> dict(x bf16, params, S0 true, meas (optional),
        s0 = noisy b0 mean)."""
        torch = self.torch
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(seed)
        P, S0 = PRIORS[self.model](n, gen, self.dev)
        x = torch.empty(n, self.n_in, dtype=torch.bfloat16, device=self.dev)
        m = torch.empty(n, self.nmeas, dtype=torch.float64, device=self.dev) if meas else None
        s0e = torch.empty(n, 1, dtype=torch.float64, device=self.dev)
        self.lib.synth(self.cfp, P, S0, snr=snr or self.snr, seed=seed, meas=m, s0=s0e, x=x)
        return dict(x=x, params=P, S0=S0, meas=m, s0=s0e)

    def targets(self, params):
        t = self.torch.empty(params.shape[0], self.n_mu, dtype=self.torch.float32, device=self.dev)
        self.lib.mlp_targets(params, t)
        return t

    def plain_fit(self, meas, s0, init=None, lm=True):
        """Grid search (+ LM) from CUDIMOT's default start; returns params."""
        torch = self.torch
        n = meas.shape[0]
        cfg = capi.model_cfg(self.model, grid=self.grid)
        lib = capi.Cudimot(self.model, cfg)
        p = init.clone() if init is not None else self._default_init(n)
        lib.gridsearch(meas, p, self.cfp, s0)
        if lm:
            lib.levmar(meas, p, self.cfp, s0)
        torch.cuda.synchronize()
        return p

    def _default_init(self, n):
        torch = self.torch
        p = torch.zeros(n, self.lib.nparams, dtype=torch.float64, device=self.dev)
        p[:, 3] = 1.5
        p[:, 4] = 1.5
        return p

    def make_training_set(self, n_prior, n_lm, seed=None):
        """Returns (x bf16 [N][n_in], targets fp32 [N][n_mu])."""
        torch = self.torch
        seed = self.seed if seed is None else seed
        xs, ts = [], []
        chunk = 1 << 21
        for k, r0 in enumerate(range(0, n_prior, chunk)):
            d = self.synth(min(chunk, n_prior - r0), seed + 1 + k)
            xs.append(d["x"])
            ts.append(self.targets(d["params"]))
        if n_lm > 0:
            d = self.synth(n_lm, seed + 1000003, meas=True)
            init = self._default_init(n_lm)
            init[:, 3:5] = d["params"][:, 3:5]  # orientation start as a DTI fit would give
            fit = self.plain_fit(d["meas"], d["s0"], init=init)
            xs.append(d["x"])
            ts.append(self.targets(fit))
        x = torch.cat(xs)
        t = torch.cat(ts)
        torch.cuda.synchronize()
        return x, t

    # ------------------------------------------------------------ training
    def train(self, x, t, epochs=2, batch=4096, seed=None, log_every=500):
        torch = self.torch
        n = x.shape[0]
        steps_per_epoch = n // batch
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(self.seed if seed is None else seed)
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        xb = torch.empty(batch, x.shape[1], dtype=x.dtype, device=self.dev)
        tb = torch.empty(batch, t.shape[1], dtype=t.dtype, device=self.dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step = 0
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen, device=self.dev)
            for s in range(steps_per_epoch):
                idx = perm[s * batch:(s + 1) * batch]
                torch.index_select(x, 0, idx, out=xb)
                torch.index_select(t, 0, idx, out=tb)
                self.net.train_step(xb, tb, loss)
                if step % log_every == 0:
                    self.history.append((step, float(loss.item())))
                step += 1
        torch.cuda.synchronize()
        self.history.append((step, float(loss.item())))
        self.train_seconds += time.perf_counter() - t0
        self.net.check()
        return self.history

    # ----------------------------------------------------------- inference
    def predict(self, meas, s0):
        """params [n][NPARAMS] and proposal widths from signals + S0."""
        torch = self.torch
        x = mlp.prep_input(meas, s0, ld=self.n_in)
        out = self.net.forward(x)
        n = meas.shape[0]
        P = torch.empty(n, self.lib.nparams, dtype=torch.float64, device=self.dev)
        sd = torch.empty_like(P)
        self.lib.mlp_decode(out, P, sd)
        return P, sd

    def cost(self, meas, params, s0, out=None):
        """Per-voxel sum of squared residuals (the LM cost), on the GPU."""
        torch = self.torch
        if out is None:
            out = torch.empty(meas.shape[0], dtype=torch.float64, device=self.dev)
        self.lib.cost(meas, params, self.cfp, s0, out)
        return out

    def contexts(self, fit_cfg, nvox, refit_cap=None):
        """Fitting contexts and buffers of `fit` (LM/MCMC; grid search + LM
        for the refit, in chunks of refit_cap voxels), allocated now."""
        torch = self.torch
        lib = capi.Cudimot(self.model, fit_cfg)
        g = capi.Cudimot(self.model, capi.model_cfg(self.model, grid=self.grid))
        cap = max(1, min(nvox, refit_cap or max(4096, nvox // 16)))
        lib.fit_reserve(nvox, self.nmeas)
        g.fit_reserve(cap, self.nmeas)
        npar = self.lib.nparams
        f = lambda *shape: torch.empty(*shape, dtype=torch.float64, device=self.dev)  # noqa: E731
        buf = dict(cost=f(nvox), yard=f(nvox), idx=torch.empty(nvox, dtype=torch.int32, device=self.dev),
                   count=torch.zeros(1, dtype=torch.int32, device=self.dev),
                   m=f(cap, self.nmeas), s0=f(cap, 1), p=f(cap, npar), cap=cap)
        return lib, g, buf

    def chi2_yardstick(self, meas, quantile=0.99, b_col=3, b0_max=50.0, out=None):
        """Per-voxel refit threshold from the voxel's own signals: (nmeas -
        nparams) x var(b = 0 signals) x F quantile. A fit whose cost exceeds
        it fits worse than noise of that variance explains (probability
        1 - quantile for a correct fit at Gaussian noise)."""
        torch = self.torch
        key = (quantile, b_col, b0_max)
        if getattr(self, "_yard_key", None) != key:
            b0 = torch.nonzero(self.cfp[:, b_col] <= b0_max).flatten()
            if b0.numel() < 3:
                raise ValueError("the goodness-of-fit judge needs at least 3 b = 0 measurements")
            dof = self.nmeas - self.lib.nparams
            from scipy import stats
            self._yard = (b0, dof * float(stats.f.ppf(quantile, dof, b0.numel() - 1)))
            self._yard_key = key
        b0, scale = self._yard
        var = meas.index_select(1, b0).var(dim=1, unbiased=True)
        if out is None:
            return var * scale
        torch.mul(var, scale, out=out)
        return out

    def fit(self, meas, s0, fit_cfg, samples, plain_cost=None, margin=0.01, ctx=None,
            judge="chi2", quantile=0.99, keep_lm=None):
        """Surrogate-initialised fit: network -> LM -> refit by grid search +
        LM of the voxels the judge flags -> MCMC with network-seeded proposal
        widths. judge "chi2": the goodness-of-fit threshold of chi2_yardstick
        (its cost is part of this call); with plain_cost given, voxels whose
        LM cost exceeds it by more than margin instead; judge None: no refit.
        keep_lm: a tensor that receives the parameters before MCMC.
        Returns (params, info)."""
        torch = self.torch
        n = meas.shape[0]
        lib, g, buf = ctx or self.contexts(fit_cfg, n)
        ev = []

        def mark():
            e = torch.cuda.Event(enable_timing=True)
            e.record(torch.cuda.current_stream())
            ev.append(e)

        mark()
        P, sd = self.predict(meas, s0)
        mark()
        lib.levmar(meas, P, self.cfp, s0)
        mark()
        info = {"refit": 0, "judge": "plain_cost" if plain_cost is not None else judge}
        if plain_cost is not None or judge == "chi2":
            self.cost(meas, P, s0, out=buf["cost"])
            if plain_cost is not None:
                ref, mg = plain_cost, margin
            else:
                ref, mg = self.chi2_yardstick(meas, quantile, out=buf["yard"]), 0.0
            lib.select_worse(buf["cost"], ref, mg, buf["idx"], buf["count"])
            nbad = int(buf["count"].item())
            info["refit"] = nbad
            cap = buf["cap"]
            for k0 in range(0, nbad, cap):
                k = min(cap, nbad - k0)
                idx = buf["idx"][k0:k0 + k]
                sm, ss, sp = buf["m"][:k], buf["s0"][:k], buf["p"][:k]
                lib.rows(k, idx, meas, sm, 0)
                lib.rows(k, idx, s0, ss, 0)
                lib.rows(k, idx, P, sp, 0)
                # the grid search replaces the grid parameters, keeps the rest
                g.gridsearch(sm, sp, self.cfp, ss)
                g.levmar(sm, sp, self.cfp, ss)
                lib.rows(k, idx, sp, P, 1)
                lib.rows(k, idx, None, sd, 2, 0.0)  # MCMC starts these from P/10
        if keep_lm is not None:
            keep_lm.copy_(P)
        mark()
        if fit_cfg.run_mcmc:
            lib.mcmc_seeded(meas, P, self.cfp, s0, samples, sd)
        mark()
        torch.cuda.synchronize()
        info["ms"] = {k: ev[i].elapsed_time(ev[i + 1])
                      for i, k in enumerate(("network", "levmar", "refit", "mcmc"))}
        return P, info
