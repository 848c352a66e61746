"""Autotuner for the fitting kernels: lane groups (`tune`) and compile-time
tile shape and loop depth (`tune_build`, below).

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


# ---------------------------------------------------------------------------
# Build variants: compile-time tile shape and loop depth.
#
# Beside the lane count, three compile-time choices shape the fitting
# kernels: the threads per CTA (CDM_NT; with the lane count it sets the
# voxels per CTA, i.e. how many voxels share one staged protocol and pair
# table in shared memory), the depth of the paired measurement loop
# (CDM_PAIR_UNROLL: how many measurement pairs are in flight per lane, i.e.
# how far shared-memory and signal loads run ahead of the arithmetic), and
# the resident CTAs per SM the MCMC kernel is compiled for
# (CDM_MCMC_MIN_BLOCKS, which caps its registers). `tune_build` compiles the
# model library once per variant (cudimot_gb300/build.py, in parallel),
# times MCMC and grid search of each on a sample of the caller's data, and
# caches the fastest per GPU, model and shape like `tune`.
VARIANTS = {
    "default": [],  # 128 threads, 4 CTAs/SM, the plugin's default unroll
    "nt64_b8": ["-DCDM_NT=64", "-DCDM_MCMC_MIN_BLOCKS=8"],
    "nt256_b2": ["-DCDM_NT=256", "-DCDM_MCMC_MIN_BLOCKS=2"],
    "u1": ["-DCDM_PAIR_UNROLL=1", "-DCDM_SHELL_UNROLL=1"],
    "u2": ["-DCDM_PAIR_UNROLL=2", "-DCDM_SHELL_UNROLL=2"],
    "u3": ["-DCDM_PAIR_UNROLL=3", "-DCDM_SHELL_UNROLL=3"],
    "u4": ["-DCDM_PAIR_UNROLL=4", "-DCDM_SHELL_UNROLL=4"],
    "b3": ["-DCDM_MCMC_MIN_BLOCKS=3"],
}


def variant_lib(model, tag, model_dir=None):
    """Build (or reuse) the library of one variant; returns its path."""
    from . import build
    flags = VARIANTS[tag]
    name = model if not flags else f"{model}__{tag}"
    out, err = build.build_model(model_dir or os.path.join(build.MODELS, model), name=name,
                                 extra_flags=flags)
    if err:
        raise RuntimeError(f"variant {tag} of {model} did not build:\n{err[-2000:]}")
    return out


def _time_variant(model, path, cfg_kw, meas, params0, cfp, fixp, reps, mcmc_iters, grid):
    import torch
    kw = dict(cfg_kw, run_mcmc=1, nburn=mcmc_iters, njumps=mcmc_iters, sampleevery=mcmc_iters)
    if grid is not None:
        kw["grid"] = grid
    lib = capi.Cudimot(model, capi.model_cfg(model, **kw), path=path)
    n = meas.shape[0]
    samples = torch.zeros(n, params0.shape[1], 1, dtype=torch.float64, device=meas.device)
    best = float("inf")
    for r in range(reps + 1):
        p = params0.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        if grid is not None:
            lib.gridsearch(meas, p, cfp, fixp)
        lib.mcmc(meas, p, cfp, fixp, samples)
        e1.record()
        torch.cuda.synchronize()
        if r > 0:
            best = min(best, e0.elapsed_time(e1))
    lib.synchronize(timeout_ms=60000)
    return best


def tune_build(model, meas, params, cfp, fixp, grid=None, variants=None, sample=65536, reps=2,
               mcmc_iters=50, cache=True, verbose=False, jobs=None, **cfg_kw):
    """Fastest build variant (VARIANTS) for this model and shape, timed on
    grid search (when a grid is given) + MCMC of a sample of the caller's
    data. Returns {"variant": tag, "flags": [...], "path": library}; pass
    the path to capi.Cudimot(model, cfg, path=...)."""
    import concurrent.futures as cf
    tags = list(variants or VARIANTS)
    n, nmeas = meas.shape
    path = os.path.join(CACHE_DIR, _gpu_name() + ".json")
    key = _key(model, nmeas, n) + "|build"
    table = _load(path) if cache else {}
    hit = table.get(key)
    if hit and hit.get("variant") in tags:
        return {"variant": hit["variant"], "flags": VARIANTS[hit["variant"]],
                "path": variant_lib(model, hit["variant"])}
    with cf.ThreadPoolExecutor(jobs or min(len(tags), os.cpu_count() or 1)) as ex:
        paths = dict(zip(tags, ex.map(lambda t: variant_lib(model, t), tags)))
    k = min(n, sample)
    m, p0, f = meas[:k].contiguous(), params[:k].contiguous(), fixp[:k].contiguous()
    times = {t: _time_variant(model, paths[t], cfg_kw, m, p0, cfp, f, reps, mcmc_iters, grid)
             for t in tags}
    best = min(times, key=times.get)
    if verbose:
        print(f"[autotune] {key}: " + " ".join(f"{t}:{ms:.3f}ms" for t, ms in times.items()) +
              f" -> {best}")
    table[key] = {"variant": best, "ms": {t: round(ms, 4) for t, ms in times.items()}}
    if cache:
        os.makedirs(CACHE_DIR, exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(table, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    return {"variant": best, "flags": VARIANTS[best], "path": paths[best], "ms": times}
