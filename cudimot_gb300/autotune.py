"""Lane-group autotuner for the fitting kernels.

Each stage maps a voxel to a group of G lanes (G in 1, 2, 4, 8, 16, 32;
`cdm_model_cfg.lanes_*`, 0 = the library's built-in choice). The best G
depends on the model (registers, work per measurement), the number of
measurements (work per lane, tail of the last chunk) and the number of
voxels (how many groups fill the 152 SMs). `tune` times every G for every
requested stage on a sample of the caller's own data, picks the fastest,
and caches the choice in `cudimot_gb300/_tune/<gpu>.json` keyed by model,
nmeas and the voxel-count bucket, so later calls with the same shape reuse
it without timing.

Timing: CUDA events around each stage call on the current stream, best of
`reps` after one warm-up call; MCMC with a shortened chain (`mcmc_iters`
burn-in + recorded iterations) since its cost is linear in iterations.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from . import capi

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE_DIR = os.path.join(HERE, "_tune")
LANES = (1, 2, 4, 8, 16, 32)
STAGES = ("gridsearch", "levmar", "mcmc")


def _gpu_name():
    import torch
    return torch.cuda.get_device_name(0).replace(" ", "_")


def _bucket(nvox):
    """Voxel-count bucket: powers of two (launch shapes change with size)."""
    return 1 << max(0, int(math.ceil(math.log2(max(nvox, 1)))))


def _key(model, nmeas, nvox):
    return f"{model}|nmeas={nmeas}|nvox~{_bucket(nvox)}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time_stage(model, cfg_kw, stage, G, meas, params0, cfp, fixp, reps, mcmc_iters):
    import torch
    kw = dict(cfg_kw)
    kw["lanes_" + stage] = G
    if stage == "mcmc":
        kw.update(run_mcmc=1, nburn=mcmc_iters, njumps=mcmc_iters, sampleevery=mcmc_iters)
    cfg = capi.model_cfg(model, **kw)
    lib = capi.Cudimot(model, cfg)
    n = meas.shape[0]
    samples = torch.zeros(n, params0.shape[1], 1, dtype=torch.float64, device=meas.device)
    best = float("inf")
    for r in range(reps + 1):
        p = params0.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if stage == "gridsearch":
            lib.gridsearch(meas, p, cfp, fixp)
        elif stage == "levmar":
            lib.levmar(meas, p, cfp, fixp)
        else:
            lib.mcmc(meas, p, cfp, fixp, samples)
        e1.record()
        torch.cuda.synchronize()
        if r > 0:
            best = min(best, e0.elapsed_time(e1))
    lib.synchronize(timeout_ms=60000)
    return best


def tune(model, meas, params, cfp, fixp, grid=None, stages=STAGES, sample=65536, reps=2,
         mcmc_iters=50, cache=True, verbose=False, **cfg_kw):
    """Best lane count per stage for this model and shape.

    meas, params, cfp, fixp: CUDA float64 tensors in the library's layouts
    (a sample of at most `sample` voxels is timed). Returns {stage: G}; the
    dict can be passed to capi.model_cfg as lanes_<stage>=G."""
    n, nmeas = meas.shape
    path = os.path.join(CACHE_DIR, _gpu_name() + ".json")
    key = _key(model, nmeas, n)
    table = _load(path) if cache else {}
    hit = table.get(key, {})
    todo = [s for s in stages if s not in hit and not (s == "gridsearch" and grid is None)]
    if todo:
        k = min(n, sample)
        m, p0 = meas[:k].contiguous(), params[:k].contiguous()
        f = fixp[:k].contiguous()
        if grid is not None:
            cfg_kw = dict(cfg_kw, grid=grid)
        for stage in todo:
            times = {}
            for G in LANES:
                times[G] = _time_stage(model, cfg_kw, stage, G, m, p0, cfp, f, reps, mcmc_iters)
            best = min(times, key=times.get)
            hit[stage] = int(best)
            hit[stage + "_ms"] = {str(g): round(t, 4) for g, t in times.items()}
            if verbose:
                print(f"[autotune] {key} {stage}: " +
                      " ".join(f"G={g}:{t:.3f}ms" for g, t in times.items()) + f" -> {best}")
        table[key] = hit
        if cache:
            os.makedirs(CACHE_DIR, exist_ok=True)
            tmp = path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(table, fh, indent=1, sort_keys=True)
            os.replace(tmp, path)
    return {s: hit[s] for s in stages if s in hit}


def lanes_kwargs(choice):
    """{stage: G} -> keyword arguments of capi.model_cfg."""
    return {"lanes_" + s: int(g) for s, g in choice.items() if s in STAGES}
