"""The lane autotuner: it times every lane count on the caller's data,
returns valid choices, caches them per GPU/model/shape, and a fit with the
tuned lane counts still matches the oracle (LM cost within 1e-4)."""
import numpy as np
import pytest
import torch

from cudimot_gb300 import autotune, capi
from tests.helpers import b1s, oracle

pytestmark = pytest.mark.gpu


def T(x, dev):
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float64), device=dev)


def test_autotune_choices_cache_and_parity(built, cuda, tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE_DIR", str(tmp_path))
    wl = b1s(20000, seed=12)
    m, p, c, f = T(wl.meas, cuda), T(wl.init, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda)
    choice = autotune.tune("Ball_1_Stick", m, p, c, f, stages=("levmar", "mcmc"), sample=8192,
                           reps=1, mcmc_iters=20)
    assert set(choice) == {"levmar", "mcmc"}
    assert all(g in autotune.LANES for g in choice.values())

    def no_timing(*a, **k):
        raise AssertionError("cached choice was timed again")
    monkeypatch.setattr(autotune, "_time_stage", no_timing)
    assert autotune.tune("Ball_1_Stick", m, p, c, f, stages=("levmar", "mcmc")) == choice

    cfg = capi.model_cfg("Ball_1_Stick", **autotune.lanes_kwargs(choice))
    lib = capi.Cudimot("Ball_1_Stick", cfg)
    q = p.clone()
    lib.levmar(m, q, c, f)
    torch.cuda.synchronize()
    o = oracle("Ball_1_Stick")
    ref, _, _, _ = o.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    cg = o.cost(wl.meas, q.cpu().numpy(), wl.cfp, wl.fixp)
    cr = o.cost(wl.meas, ref, wl.cfp, wl.fixp)
    assert np.mean((cg - cr) / cr <= 1e-4) >= 0.995


def test_autotune_build_variants(built, cuda, tmp_path, monkeypatch):
    """The build-variant tuner compiles the variants it is given (CTA size
    here), times them on the caller's data, caches the winner, and the
    winning library fits like the default one (LM against the oracle)."""
    monkeypatch.setattr(autotune, "CACHE_DIR", str(tmp_path))
    wl = b1s(20000, seed=13)
    m, p, c, f = T(wl.meas, cuda), T(wl.init, cuda), T(wl.cfp, cuda), T(wl.fixp, cuda)
    tags = ["default", "nt64_b8"]
    got = autotune.tune_build("Ball_1_Stick", m, p, c, f, variants=tags, sample=8192, reps=1,
                              mcmc_iters=20)
    assert got["variant"] in tags and set(got["ms"]) == set(tags)

    def no_timing(*a, **k):
        raise AssertionError("cached variant was timed again")
    monkeypatch.setattr(autotune, "_time_variant", no_timing)
    again = autotune.tune_build("Ball_1_Stick", m, p, c, f, variants=tags)
    assert again["variant"] == got["variant"] and again["path"] == got["path"]

    cfg = capi.model_cfg("Ball_1_Stick")
    lib = capi.Cudimot("Ball_1_Stick", cfg, path=got["path"])
    q = p.clone()
    lib.levmar(m, q, c, f)
    torch.cuda.synchronize()
    o = oracle("Ball_1_Stick")
    ref, _, _, _ = o.levmar(cfg, wl.meas, wl.init, wl.cfp, wl.fixp)
    cg = o.cost(wl.meas, q.cpu().numpy(), wl.cfp, wl.fixp)
    cr = o.cost(wl.meas, ref, wl.cfp, wl.fixp)
    assert np.mean((cg - cr) / cr <= 1e-4) >= 0.995
