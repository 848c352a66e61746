"""Throughput benchmark: NODDI-Watson grid search -> LM -> MCMC.

Workload (one step = one fit of the whole batch): 200,000 voxels,
288 measurements (18 b=0 + 90 directions at each of b = 1000/2000/3000),
grid fiso, fintra in 0:0.1:1 x kappa 1..8 (968 combinations), LM up to 200
iterations, MCMC 1250 burn-in + 1250 jumps keeping every 25th (50 samples).
Synthetic data: true parameters from the configuration's ranges, signals
from the library's own Predicted_Signal, Rician noise at SNR 20, S0 fixed to
the mean b=0 signal, orientation initialised by a log-linear tensor fit.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value: voxels/s with inputs resident in HBM (signals 2 x 230 MB > L2, so
no flush is needed). e2e: the same through cdm_fit_host from pinned host
buffers, copies included. The reference arm times the CPU oracle (the
restated CUDIMOT fitting loops, FP64, OpenMP over all host cores) on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxels/s fitted (LM+MCMC) at matched param error; surrogate-init vs grid-init"
MODEL = "NODDI_Watson"
NVOX = 200_000
NBURN, NJUMPS, SE = 1250, 1250, 25


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nvox", type=int, default=None,
                    help="voxels (default: the workload's own size)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0, help="voxels for the CPU baseline")
    ap.add_argument("--profile-stage",
                    choices=["gridsearch", "levmar", "mcmc", "mlp_forward", "hetero_mcmc"],
                    default=None,
                    help="run the preceding stages, then one launch of this stage (for ncu); "
                         "mlp_forward: two inference passes of the network on --nvox voxels; "
                         "hetero_mcmc: the MCMC of one NODDI-Watson fit through the model "
                         "library, then through the persistent multi-model kernel")
    ap.add_argument("--lanes", type=int, default=None,
                    help="with --profile-stage: lanes per voxel (default: those the 200,000-voxel "
                         "headline runs with, 2 for grid search and MCMC, 4 for LM; the automatic "
                         "rule would widen the groups of a small case)")
    ap.add_argument("--rician", action="store_true",
                    help="with --profile-stage mcmc: the Rician likelihood (tau sampled)")
    ap.add_argument("--nburn", type=int, default=NBURN)
    ap.add_argument("--njumps", type=int, default=NJUMPS)
    ap.add_argument("--workload", default="noddi_watson",
                    choices=["noddi_watson", "noddi_watson_rician", "ball_1_stick_lm", "heterogeneous",
                             "learned_init", "noddi_bingham"],
                    help="noddi_watson: the headline (200k voxels GS->LM->MCMC); "
                         "ball_1_stick_lm: 10k voxels plain LM; heterogeneous: DiffusionTensor "
                         "400k + Ball_2_Sticks 300k + NODDI_Watson 500k LM+MCMC in one graph; "
                         "learned_init: network-initialised vs grid-initialised NODDI_Watson; "
                         "noddi_bingham: 1M voxels GS (11,050) -> LM -> MCMC, precision study; "
                         "noddi_watson_rician: the headline fit with the Rician likelihood")
    ap.add_argument("--train-signals", type=int, default=20_000_000)
    ap.add_argument("--lm-targets", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--eval-voxels", type=int, default=1_000_000)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_cfg(grid=True):
    from cudimot_gb300 import capi, synth
    cfg = capi.model_cfg(MODEL, grid=synth.WATSON_GRID if grid else None, run_mcmc=1,
                         nburn=NBURN, njumps=NJUMPS, sampleevery=SE, iter_levmar=200)
    return cfg


def make_workload(nvox, seed, dev, snr=20.0):
    """Synthetic C1 inputs; the clean signal comes from the library itself."""
    import torch
    from cudimot_gb300 import capi, synth
    r_proto, r_par, r_noise = [np.random.Generator(np.random.PCG64(s))
                               for s in np.random.SeedSequence(seed).spawn(3)]
    cfp = synth.protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], r_proto)
    truth, S0 = synth.watson_truth(nvox, r_par)
    lib = capi.Cudimot(MODEL, capi.model_cfg(MODEL))
    clean = torch.zeros(nvox, cfp.shape[0], dtype=torch.float64, device=dev)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    lib.predicted_signal(t(truth[:, :, None]), t(cfp), t(S0[:, None]), clean)
    torch.cuda.synchronize()
    clean = clean.cpu().numpy()
    lib.close()
    meas = synth.rician(clean, S0 / snr, r_noise)
    b0 = cfp[:, 3] == 0
    fixp = meas[:, b0].mean(axis=1, keepdims=True)
    _, _, _, th, ph = synth.dti_init(meas, cfp)
    init = np.stack([np.full(nvox, 0.4), np.full(nvox, 0.8), np.full(nvox, 5.0), th, ph], axis=1)
    return cfp, meas, fixp, init, truth


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def cpu_baseline(cfp, meas, fixp, init, n, cfg, prec=0):
    """CPU oracle on n voxels: grid search -> LM -> MCMC, all host threads;
    prec 0 = T double (as the plugins ship), 1 = T float."""
    from oracle.oracle import Oracle
    o = Oracle(MODEL)
    threads = o.max_threads()
    sl = slice(0, n)
    t0 = time.perf_counter()
    p, _, _ = o.gridsearch(cfg, meas[sl], init[sl], cfp, fixp[sl], prec=prec, threads=threads)
    p, _, _, _ = o.levmar(cfg, meas[sl], p, cfp, fixp[sl], prec=prec, threads=threads)
    p, s, _ = o.mcmc(cfg, meas[sl], p, cfp, fixp[sl], prec=prec, threads=threads)
    dt = time.perf_counter() - t0
    return n / dt, threads, dt


def flop_model():
    """Algorithmic FP32 work per voxel of the MCMC stage: operations of one
    likelihood (Derived_P after a one-parameter change + nmeas x (signal + 3))
    x free parameters x (burn-in + jumps), counted by the library's
    operation-count build of the plugin (cudimot_gb300/flops.py)."""
    try:
        from cudimot_gb300 import flops
        return flops.watson_c1_flops_per_voxel()
    except Exception as e:  # noqa: BLE001
        return None


def headline_config(nvox, world):
    """The config dict of the headline line (both arms print the same)."""
    return {"workload": "noddi_watson_gs_lm_mcmc", "model": MODEL, "nvox_per_gpu": nvox,
            "nmeas": 288, "grid_combs": 968, "nburn": NBURN, "njumps": NJUMPS, "sampleevery": SE,
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"voxel shards x{world}"}


CPU_PLUGIN_NOTE = ("the CPU oracle runs this library's NODDI-Watson plugin (59 FLOP per signal), "
                   "not CUDIMOT's as written (620-820 FLOP per signal, FP64 closed forms)")


def run_reference(a, rank, world):
    """CUDIMOT's fitting loops restated on the CPU (the oracle, FP64,
    OpenMP over all host cores): every timed step fits a 2,048-voxel sample
    of the headline workload (warm-up steps 256 voxels)."""
    if rank != 0:
        return
    from cudimot_gb300 import synth
    import torch  # noqa: F401
    cfg = workload_cfg()
    # inputs generated on the host: noiseless signal from the CPU oracle
    from oracle.oracle import Oracle
    o = Oracle(MODEL)
    n = a.cpu_sample or 2048
    wl = synth.noddi_watson(n, signal_fn=lambda t, c, s0: o.signal(t, c, s0[:, None]))
    times = []
    for i in range(a.warmup + a.steps):
        k = n if i >= a.warmup else min(n, 256)
        v, threads, dt = cpu_baseline(wl.cfp, wl.meas, wl.fixp, wl.init, k, cfg)
        if i >= a.warmup:
            times.append(dt)
    dt = float(np.mean(times))
    value = n / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s",
            "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded NODDI-Watson, SNR 20)",
            "config": headline_config(NVOX, world),
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": threads, "kind": "port",
                             "sample": f"{n} voxels of the 200,000-voxel workload per timed step "
                                       "(warm-up steps 256), full grid search -> LM -> MCMC, "
                                       "FP64 CPU oracle",
                             "plugin": CPU_PLUGIN_NOTE},
            "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def profile_mlp_forward(a, dev):
    import torch
    from cudimot_gb300 import synth
    from cudimot_gb300.learned import LearnedInit
    rng = np.random.default_rng(8219)
    cfp = synth.protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], rng)
    li = LearnedInit(MODEL, cfp, grid=synth.WATSON_GRID, seed=8219, device=dev)
    a.nvox = a.nvox or 262144
    d = li.synth(a.nvox, seed=4242, snr=(20.0, 20.0), meas=True)
    li.predict(d["meas"], d["s0"])  # warm-up: 4 GEMM launches
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    li.predict(d["meas"], d["s0"])
    e1.record()
    torch.cuda.synchronize()
    li.net.check()
    print(json.dumps({"stage": "mlp_forward", "nvox": a.nvox, "ms": e0.elapsed_time(e1),
                      "hidden_layer": hidden_layer_roofline(li.net, dev, n=a.nvox)}))


def profile_hetero(a, dev):
    """One NODDI-Watson MCMC (--nvox voxels, --nburn + --njumps, 2 lanes)
    through the model library's kernel, then the same fit through the
    persistent multi-model kernel (libcdm_hetero): two launches to compare."""
    import torch
    from cudimot_gb300 import capi, hetero
    a.nvox = a.nvox or 200_000
    cfp, meas, fixp, init, _ = make_workload(a.nvox, 8219, dev)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f, i = t(meas), t(cfp), t(fixp), t(init)
    cfg = capi.model_cfg(MODEL, run_mcmc=1, nburn=a.nburn, njumps=a.njumps, sampleevery=SE,
                         lanes_mcmc=a.lanes or 2)
    ns = max(a.njumps // SE, 1)
    res = {}
    h = hetero.Hetero()
    keep = []
    for path in ("library", "persistent"):
        ctx = capi.Cudimot(MODEL, cfg)
        p = i.clone()
        s = torch.zeros(a.nvox, 5, ns, dtype=torch.float64, device=dev)
        keep.append((ctx, p, s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if path == "library":
            e0.record()
            ctx.mcmc(m, p, c, f, s)
        else:
            w = h.prepare(ctx, m, p, c, f, s)
            e0.record()
            h.mcmc([w])
        e1.record()
        torch.cuda.synchronize()
        res[path] = e0.elapsed_time(e1)
    res["samples_equal"] = bool(torch.equal(keep[0][2], keep[1][2]))
    print(json.dumps({"stage": "hetero_mcmc", "nvox": a.nvox, "ms": res}))


def profile_stage(a):
    """One launch of one stage on a small case, for ncu captures."""
    import torch
    from cudimot_gb300 import capi, synth
    dev = torch.device("cuda:0")
    if a.profile_stage == "mlp_forward":
        profile_mlp_forward(a, dev)
        return
    if a.profile_stage == "hetero_mcmc":
        profile_hetero(a, dev)
        return
    a.nvox = a.nvox or 20000
    model, grid = MODEL, synth.WATSON_GRID
    if a.workload == "noddi_bingham":  # the Bingham workload and grid
        model, grid = "NODDI_Bingham", synth.BINGHAM_GRID
        wl = bingham_workload(a.nvox, dev)
        cfp, meas, fixp, init = wl.cfp, wl.meas, wl.fixp, wl.init
    else:
        cfp, meas, fixp, init, _ = make_workload(a.nvox, 8219, dev)
    lanes = a.lanes or {"levmar": 4}.get(a.profile_stage, 2)
    lk = dict(lanes_gridsearch=2, lanes_levmar=4, lanes_mcmc=2)
    lk[f"lanes_{a.profile_stage}"] = lanes
    cfg = capi.model_cfg(model, grid=grid, run_mcmc=1, nburn=a.nburn,
                         njumps=a.njumps, sampleevery=SE, rician=int(a.rician), **lk)
    lib = capi.Cudimot(model, cfg)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f, p = t(meas), t(cfp), t(fixp), t(init)
    if a.profile_stage in ("levmar", "mcmc"):
        lib.gridsearch(m, p, c, f)
    if a.profile_stage == "mcmc":
        lib.levmar(m, p, c, f)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    if a.profile_stage == "gridsearch":
        lib.gridsearch(m, p, c, f)
    elif a.profile_stage == "levmar":
        lib.levmar(m, p, c, f)
    else:
        ns = max(a.njumps // SE, 1)
        s = torch.zeros(a.nvox, init.shape[1], ns, dtype=torch.float64, device=dev)
        tau = torch.zeros(a.nvox, ns, dtype=torch.float64, device=dev) if a.rician else None
        lib.mcmc(m, p, c, f, s, tau=tau)
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"stage": a.profile_stage, "model": model, "rician": a.rician, "nvox": a.nvox,
                      "lanes": lanes, "ms": e0.elapsed_time(e1)}))


def measured_traffic(kernel, config):
    """DRAM bytes per launch of a kernel from bench_traffic.json (one ncu
    capture per kernel, tagged with the configuration it was taken on).
    Returned as captured when this run's configuration matches; when only
    the voxel count differs, scaled by voxels (the kernel reads each voxel's
    signals once and writes its samples once); else None."""
    try:
        rec = json.load(open(os.path.join(ROOT, "bench_traffic.json")))[kernel]
    except (OSError, ValueError, KeyError):
        return None, None
    cap = rec["config"]
    same = {k: v for k, v in cap.items() if k != "nvox"} == {k: v for k, v in config.items()
                                                              if k != "nvox"}
    if not same:
        return None, None
    b = float(rec["dram_bytes_per_launch"])
    if cap["nvox"] == config["nvox"]:
        return b, f"ncu capture of this configuration ({rec['command']})"
    return b * config["nvox"] / cap["nvox"], (f"ncu capture at {cap['nvox']} voxels scaled to "
                                              f"{config['nvox']} ({rec['command']})")


def timed_events(fn, steps, flush=None):
    """CUDA-event time (ms) of each call of fn on the current stream; flush
    (untimed) before each call when given."""
    import torch
    st = torch.cuda.current_stream()
    out = []
    for _ in range(steps):
        if flush is not None:
            flush()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return out


def base_line(metric, value, unit, a, ms, config, clocks, dtype="f32 model / f64 sums", **kw):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": a.steps,
         "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config,
         "clocks": clocks}
    d.update(kw)
    return d


def bench_b1s_lm(a, dev):
    """Ball & 1 Stick plain LM, 10,000 voxels x 134 measurements, LM <= 200
    iterations from a log-linear tensor fit. Inputs (5 MB) fit in L2, so a
    256 MB buffer is written before every timed step."""
    import torch
    from cudimot_gb300 import capi, synth
    n = a.nvox or 10_000
    wl = synth.ball_1_stick(n)
    cfg = capi.model_cfg("Ball_1_Stick", iter_levmar=200)
    lib = capi.Cudimot("Ball_1_Stick", cfg)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f, p0 = t(wl.meas), t(wl.cfp), t(wl.fixp), t(wl.init)
    p = p0.clone()
    s = torch.zeros(n, 5, 1, dtype=torch.float64, device=dev)
    junk = torch.empty(64 << 20, dtype=torch.float32, device=dev)

    def flush():
        junk.fill_(1.0)
        p.copy_(p0)

    def step():
        lib.fit(m, p, c, f, s)

    timed_events(step, a.warmup, flush)
    with ClockSampler(dev.index or 0) as clk:
        ms = timed_events(step, max(a.steps, 10), flush)
    ms_step = statistics.median(ms)
    st = lib.stats()
    # e2e: host arrays through cdm_fit_host
    hm, hc, hf = wl.meas.copy(), wl.cfp.copy(), wl.fixp.copy()
    hs = np.zeros((n, 5, 1))
    e2e = []
    for _ in range(3):
        hp = wl.init.copy()
        t0 = time.perf_counter()
        lib.fit_host(hm, hp, hc, hf, hs)
        e2e.append(time.perf_counter() - t0)
    # roofline of the step: the LM kernel's work (passes from the device
    # counter) over the step's time, against the FP32 peak
    from cudimot_gb300 import flops
    ops = flops.count_ops("Ball_1_Stick", wl.truth, wl.cfp, wl.fixp)
    fl_pass = flops.levmar_pass_flops(ops, 134, 5)
    pk = fp32_peak_tflops(dev)
    achieved = fl_pass * st.lm_iterations / (ms_step / 1e3) / 1e12
    roof = {"bound": "latency", "kernel": "cdm_levmar_kernel", "achieved": achieved,
            "unit": "TFLOP/s", "peak": pk["tflops"] if pk else None,
            "frac": achieved / pk["tflops"] if pk else None,
            "peak_source": pk["source"] if pk else None, "flop_per_pass": fl_pass,
            "note": "10,000 voxels x 4 lanes are 40,000 threads, half of the 77,824 the GPU "
                    "holds at once: one partial wave of ~7 dependent LM passes, so the fit "
                    "is bound by pass latency, not by a pipe"}
    line = base_line("voxels/s fitted (plain LM)", n / (ms_step / 1e3), "voxels/s", a, ms_step,
                     {"workload": "ball_1_stick_lm", "model": "Ball_1_Stick", "nvox": n, "nmeas": 134,
                      "iter_levmar": 200, "l2": "256 MB written before each step (inputs fit in L2)"},
                     clk.summary(), lm_iterations_per_voxel=st.lm_iterations / n,
                     roofline=roof, gpu_launches=3 * max(a.steps, 10),
                     e2e={"value": n / statistics.median(e2e), "unit": "voxels/s",
                          "h2d_bytes_per_step": int(hm.nbytes + hc.nbytes + wl.init.nbytes),
                          "d2h_bytes_per_step": int(wl.init.nbytes + hs.nbytes)})
    print(json.dumps(line))


def bench_heterogeneous(a, dev):
    """Three volumes, three models, three protocols - DiffusionTensor 400k x
    71, Ball_2_Sticks 300k x 134, NODDI_Watson 500k x 288 (SNR 25), LM +
    MCMC (1250 + 1250, every 25th) - recorded as branches of one CUDA graph
    (cdm_batch) and launched once per step; the same fits run one model
    after another are timed too."""
    import torch
    from cudimot_gb300 import capi, synth
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    scale = a.nvox / 1_200_000 if a.nvox else 1.0
    vols = []
    wdt = synth.diffusion_tensor(int(400_000 * scale), snr=25.0)
    wb2 = synth.ball_2_sticks(int(300_000 * scale), snr=25.0)
    cfp, meas, fixp, init, _ = make_workload(int(500_000 * scale), 8219, dev, snr=25.0)
    from cudimot_gb300 import autotune
    tuned = {}
    for model, m, c, f, i in (("DiffusionTensor", wdt.meas, wdt.cfp, wdt.fixp, wdt.init),
                              ("Ball_2_Sticks", wb2.meas, wb2.cfp, wb2.fixp, wb2.init),
                              ("NODDI_Watson", meas, cfp, fixp, init)):
        dm, dc, df, di = t(m), t(c), t(f), t(i)
        # lane counts per stage from the autotuner, timed on this volume's data
        choice = autotune.tune(model, dm, di, dc, df, stages=("levmar", "mcmc"), reps=1)
        tuned[model] = choice
        cfg = capi.model_cfg(model, run_mcmc=1, nburn=NBURN, njumps=NJUMPS, sampleevery=SE,
                             **autotune.lanes_kwargs(choice))
        npar = i.shape[1]
        d = dict(model=model, lib=capi.Cudimot(model, cfg), meas=dm, cfp=dc, fixp=df,
                 init=di, params=di.clone(),
                 samples=torch.zeros(m.shape[0], npar, NJUMPS // SE, dtype=torch.float64, device=dev))
        vols.append(d)
    total = sum(v["meas"].shape[0] for v in vols)
    batch = capi.Batch()
    for v in vols:
        batch.add(v["lib"], v["meas"], v["params"], v["cfp"], v["fixp"], v["samples"],
                  work=float(v["meas"].numel()) * v["init"].shape[1])

    def reset():
        for v in vols:
            v["params"].copy_(v["init"])

    def run_batch():
        batch.run()

    def run_seq():
        for v in vols:
            v["lib"].fit(v["meas"], v["params"], v["cfp"], v["fixp"], v["samples"])

    # the persistent multi-model kernel: LM per volume, then every volume's
    # MCMC tiles in one launch. MCMC at 2 lanes for every model: one CTA
    # holds the largest fit's tables and the largest sample staging of all
    # of them, and at 1 lane (128 voxels per CTA) the staging alone is 32 KB
    # for the tensor model, which leaves room for 3 CTAs per SM instead of 4
    from cudimot_gb300 import hetero
    hx = hetero.Hetero()
    for v in vols:
        lk = autotune.lanes_kwargs(tuned[v["model"]])
        lk["lanes_mcmc"] = 2
        v["hx_lanes"] = lk["lanes_mcmc"]
        v["hx_lib"] = capi.Cudimot(v["model"], capi.model_cfg(
            v["model"], run_mcmc=1, nburn=NBURN, njumps=NJUMPS, sampleevery=SE, **lk))

    def run_persistent():
        for v in vols:
            v["hx_lib"].levmar(v["meas"], v["params"], v["cfp"], v["fixp"])
        hx.mcmc([hx.prepare(v["hx_lib"], v["meas"], v["params"], v["cfp"], v["fixp"], v["samples"])
                 for v in vols])

    timed_events(run_batch, a.warmup, reset)
    timed_events(run_seq, 1, reset)
    timed_events(run_persistent, 1, reset)
    with ClockSampler(dev.index or 0) as clk:
        ms = timed_events(run_batch, a.steps, reset)
    ms_seq = timed_events(run_seq, a.steps, reset)
    ms_per = timed_events(run_persistent, a.steps, reset)
    ms_b, ms_s = statistics.median(ms), statistics.median(ms_seq)
    ms_p = statistics.median(ms_per)
    line = base_line("voxels/s fitted (LM+MCMC), heterogeneous batch", total / (ms_b / 1e3),
                     "voxels/s", a, ms_b,
                     {"workload": "heterogeneous_lm_mcmc",
                      "volumes": [{"model": v["model"], "nvox": int(v["meas"].shape[0]),
                                   "nmeas": int(v["meas"].shape[1])} for v in vols],
                      "nburn": NBURN, "njumps": NJUMPS, "sampleevery": SE,
                      "l2": "inputs larger than L2 (no flush)",
                      "launch": "one CUDA graph, one branch per volume",
                      "lanes_from_autotuner": tuned},
                     clk.summary(), sequential={"value": total / (ms_s / 1e3), "ms_per_step": ms_s},
                     persistent={"value": total / (ms_p / 1e3), "ms_per_step": ms_p,
                                 "launch": "LM per volume, then one persistent MCMC launch over "
                                           "every volume's tiles (libcdm_hetero)",
                                 "grid": hx.last_grid, "launches": hx.last_launches,
                                 "mcmc_lanes": {v["model"]: v["hx_lanes"] for v in vols}},
                     gpu_launches=sum(9 for _ in vols) * a.steps)
    print(json.dumps(line))


def param_error(m, truth):
    """Posterior means (or fits) against the true NODDI-Watson parameters."""
    ang = np.degrees(np.arccos(np.clip(np.abs(
        np.sin(m[:, 3]) * np.sin(truth[:, 3]) * np.cos(m[:, 4] - truth[:, 4]) +
        np.cos(m[:, 3]) * np.cos(truth[:, 3])), 0, 1)))
    return {"fiso_rmse": float(np.sqrt(np.mean((m[:, 0] - truth[:, 0]) ** 2))),
            "fintra_rmse": float(np.sqrt(np.mean((m[:, 1] - truth[:, 1]) ** 2))),
            "log_kappa_rmse": float(np.sqrt(np.mean((np.log(np.maximum(m[:, 2], 1e-3)) -
                                                     np.log(truth[:, 2])) ** 2))),
            "orientation_median_deg": float(np.median(ang))}


def hidden_layer_roofline(net, dev, n=262_144, reps=20):
    """The network's second hidden layer (262,144 x 256 x 256, bias + GELU,
    bf16 out; the persistent tcgen05 kernel) timed alone with CUDA events on
    the launching stream, against the measured bf16 peak; HBM bytes are the
    bf16 input read once and the output written once."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(5)
    x = (torch.rand(n, net.cfg.hidden, generator=g) * 1.2).to(torch.bfloat16).to(dev)
    out = torch.empty_like(x)
    for _ in range(3):
        net.hidden_layer(1, x, out)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        net.hidden_layer(1, x, out)
    e1.record(st)
    torch.cuda.synchronize()
    net.check()
    ms = e0.elapsed_time(e1) / reps
    flop = 2.0 * n * net.cfg.hidden * net.cfg.hidden
    tf = flop / (ms / 1e3) / 1e12
    peaks = measured_peaks()
    peak = peaks.get("bf16_tflops")
    hbm = 2.0 * x.numel() * 2 / (ms / 1e3) / 1e9
    return {"kernel": "umma_gelu_persistent_kernel", "shape": [n, net.cfg.hidden, net.cfg.hidden],
            "launch_ms": ms, "achieved": tf, "unit": "TFLOP/s", "bound": "tensor",
            "peak": peak, "frac": tf / peak if peak else None,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)",
            "hbm_gbs": hbm, "hbm_frac": hbm / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None}


def learned_comparison(dev, train_signals=20_000_000, lm_targets=1_000_000, epochs=2,
                       n=1_000_000):
    """Network-initialised vs grid-initialised NODDI-Watson fits of the same
    n voxels (SNR 20) on the same GPU, each LM -> MCMC (1250 + 1250, every
    25th). The network (288 -> 256 -> 256 -> 256 -> 12, BF16 tensor cores)
    is trained first on train_signals synthetic signals (SNR U(10,50)) plus
    lm_targets grid-search + LM fits. The surrogate path's time includes the
    network, its LM, the refit judge (goodness of fit against the variance
    of each voxel's b = 0 signals) and the grid search + LM refit of the
    voxels it flags. Since both paths fit every voxel here, the audit
    compares their LM costs voxel by voxel (outside the timing)."""
    import torch
    from cudimot_gb300 import capi, synth
    from cudimot_gb300.learned import LearnedInit
    rng = np.random.default_rng(8219)
    cfp = synth.protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], rng)
    li = LearnedInit(MODEL, cfp, grid=synth.WATSON_GRID, seed=8219, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, tg = li.make_training_set(train_signals, lm_targets)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    li.train(x, tg, epochs=epochs, batch=4096)
    n_train = x.shape[0]
    del x, tg
    steps = epochs * (n_train // 4096)
    flop_sample = 2 * sum(d0 * d1 for d0, d1 in zip(li.net.dims()[:-1], li.net.dims()[1:]))
    d = li.synth(n, seed=4242, snr=(20.0, 20.0), meas=True)
    meas, s0, truth = d["meas"], d["s0"], d["params"].cpu().numpy()
    _, _, _, th, ph = synth.dti_init(meas.cpu().numpy(), cfp)
    init = li._default_init(n)
    init[:, 3] = torch.as_tensor(th, device=dev)
    init[:, 4] = torch.as_tensor(ph, device=dev)
    fit_cfg = capi.model_cfg(MODEL, run_mcmc=1, nburn=NBURN, njumps=NJUMPS, sampleevery=SE)
    gs_cfg = capi.model_cfg(MODEL, grid=synth.WATSON_GRID, run_mcmc=1, nburn=NBURN, njumps=NJUMPS,
                            sampleevery=SE)
    plain = capi.Cudimot(MODEL, gs_cfg)
    ns = NJUMPS // SE
    sp = torch.zeros(n, 5, ns, dtype=torch.float64, device=dev)
    ss = torch.zeros_like(sp)
    st = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    # scratch buffers, the network's inference buffers and every kernel of
    # both paths loaded before timing (a short run of each on 4096 voxels)
    plain.fit_reserve(n, 288)
    ctx = li.contexts(fit_cfg, n)
    li.predict(meas, s0)
    w = min(n, 4096)
    wcfg = capi.model_cfg(MODEL, grid=synth.WATSON_GRID, run_mcmc=1, nburn=25, njumps=25,
                          sampleevery=25)
    wp = init[:w].clone()
    wl = capi.Cudimot(MODEL, wcfg)
    wl.gridsearch(meas[:w], wp, li.cfp, s0[:w])
    wl.levmar(meas[:w], wp, li.cfp, s0[:w])
    wsamp = torch.zeros(w, 5, 1, dtype=torch.float64, device=dev)
    wl.mcmc(meas[:w], wp, li.cfp, s0[:w], wsamp)
    li.fit(meas[:w].contiguous(), s0[:w].contiguous(), wcfg, wsamp)
    lm_plain = torch.empty(n, 5, dtype=torch.float64, device=dev)
    lm_sur = torch.empty_like(lm_plain)
    torch.cuda.synchronize()
    # grid-initialised path: GS -> LM -> MCMC
    p = init.clone()
    e = [ev() for _ in range(4)]
    e[0].record(st)
    plain.gridsearch(meas, p, li.cfp, s0)
    e[1].record(st)
    plain.levmar(meas, p, li.cfp, s0)
    e[2].record(st)
    lm_plain.copy_(p)
    plain.mcmc(meas, p, li.cfp, s0, sp)
    e[3].record(st)
    torch.cuda.synchronize()
    plain_ms = {"gridsearch": e[0].elapsed_time(e[1]), "levmar": e[1].elapsed_time(e[2]),
                "mcmc": e[2].elapsed_time(e[3])}
    t_plain = e[0].elapsed_time(e[3])
    lm_it_plain = plain.stats().lm_iterations / n
    # network-initialised path: network -> LM -> judge -> refit -> MCMC
    f0, f1 = ev(), ev()
    f0.record(st)
    _, info = li.fit(meas, s0, fit_cfg, ss, ctx=ctx, keep_lm=lm_sur)
    f1.record(st)
    torch.cuda.synchronize()
    t_sur = f0.elapsed_time(f1)
    # audit: the surrogate path's LM cost against the plain path's, per voxel
    c_plain = li.cost(meas, lm_plain, s0).cpu().numpy()
    c_sur = li.cost(meas, lm_sur, s0).cpu().numpy()
    rel = (c_sur - c_plain) / c_plain
    gp, gs_ = sp.cpu().numpy().mean(2), ss.cpu().numpy().mean(2)
    return {"workload": "learned_init_noddi_watson", "nvox": n, "nmeas": 288, "snr": 20,
            "nburn": NBURN, "njumps": NJUMPS, "sampleevery": SE,
            "network": "288-256-256-256-12 GELU, bf16 tensor cores",
            "surrogate_init": {"value": n / (t_sur / 1e3), "ms": t_sur, "stages_ms": info["ms"],
                               "lm_iterations_per_voxel": ctx[0].stats().lm_iterations / n,
                               "judge": "LM cost > (nmeas - 5) var(b=0 signals) F.ppf(0.99)",
                               "refit_voxels": info["refit"],
                               "param_error": param_error(gs_, truth)},
            "grid_init": {"value": n / (t_plain / 1e3), "ms": t_plain, "stages_ms": plain_ms,
                          "lm_iterations_per_voxel": lm_it_plain,
                          "param_error": param_error(gp, truth)},
            "speedup": t_plain / t_sur,
            "audit_lm_cost_vs_grid_init": {
                "voxels_worse_by_1pct": int(np.sum(rel > 0.01)),
                "voxels_better_by_1pct": int(np.sum(rel < -0.01)),
                "median_rel": float(np.median(rel)), "max_rel": float(rel.max())},
            "network_hidden_layer": hidden_layer_roofline(li.net, dev),
            "training": {"signals": int(n_train), "epochs": epochs, "steps": int(steps),
                         "seconds": li.train_seconds, "data_seconds": t_data,
                         "tflops": 3 * flop_sample * steps * 4096 / li.train_seconds / 1e12,
                         "loss_first": li.history[0][1], "loss_last": li.history[-1][1]}}


def bench_learned(a, dev):
    """The learned-initialiser comparison (learned_comparison) as its own line."""
    with ClockSampler(dev.index or 0) as clk:
        res = learned_comparison(dev, a.train_signals, a.lm_targets, a.epochs, a.eval_voxels)
    sur = res["surrogate_init"]
    line = base_line(METRIC, sur["value"], "voxels/s", a, sur["ms"],
                     {k: res[k] for k in ("workload", "nvox", "nmeas", "snr", "nburn", "njumps",
                                          "sampleevery", "network")} |
                     {"l2": "inputs larger than L2 (no flush)"},
                     clk.summary(), **{k: v for k, v in res.items() if k in (
                         "surrogate_init", "grid_init", "speedup", "audit_lm_cost_vs_grid_init",
                         "network_hidden_layer", "training")})
    line["steps"], line["warmup"] = 1, 1
    print(json.dumps(line))


# FP32 operations of the Rician term per measurement beyond the signal:
# -tau/2 (y^2 + S^2) (4), tau S y (2), the accumulation (1) and log I0
# (cdm_log_i0: the x / 3.75 scaling, its square and a degree-6 polynomial,
# 16; its logarithm is a transcendental, not counted)
F_RICIAN = 23


def bench_rician(a, dev):
    """The headline fit (200k NODDI-Watson voxels, GS -> LM -> MCMC 1250 +
    1250) with the Rician likelihood (--rician: tau sampled with the
    parameters, CUDIMOT's MCMC.cu Rician energy), device-resident inputs."""
    import torch
    from cudimot_gb300 import capi, flops
    nvox = a.nvox or NVOX
    cfp, meas, fixp, init, truth = make_workload(nvox, 8219, dev)
    cfg = workload_cfg()
    cfg.rician = 1
    lib = capi.Cudimot(MODEL, cfg)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f, p0 = t(meas), t(cfp), t(fixp), t(init)
    p = p0.clone()
    ns = NJUMPS // SE
    samples = torch.zeros(nvox, 5, ns, dtype=torch.float64, device=dev)
    tau = torch.zeros(nvox, ns, dtype=torch.float64, device=dev)

    def step():
        p.copy_(p0)
        lib.fit(m, p, c, f, samples, tau=tau)

    for _ in range(a.warmup):
        step()
    with ClockSampler(dev.index or 0) as clk:
        ms = statistics.median(timed_events(step, a.steps))
    # the MCMC launch alone, from the grid-search + LM start
    q = p0.clone()
    lib.gridsearch(m, q, c, f)
    lib.levmar(m, q, c, f)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    lib.mcmc(m, q, c, f, samples, tau=tau)
    e1.record(st)
    torch.cuda.synchronize()
    mcmc_ms = e0.elapsed_time(e1)
    fl = flops.watson_c1_flops_per_voxel()
    ops = fl["ops"]
    like = ops["derived_p_one_param"] + 288 * (ops["signal"] + F_RICIAN)
    like_tau = 288 * (ops["signal"] + F_RICIAN)
    per_voxel = (NBURN + NJUMPS) * (5 * like + like_tau)
    peak = fp32_peak_tflops(dev)
    achieved = per_voxel * nvox / (mcmc_ms / 1e3) / 1e12
    roof = None
    if peak:
        roof = {"bound": "fp32", "kernel": "cdm_mcmc_kernel", "achieved": achieved,
                "peak": peak["tflops"], "unit": "TFLOP/s", "frac": achieved / peak["tflops"],
                "peak_source": peak["source"], "flop_per_voxel": per_voxel, "launch_ms": mcmc_ms,
                "flop_note": f"signal from the operation-count build + {F_RICIAN} per measurement for the "
                             "Rician term; one tau proposal per iteration besides the 5 parameters"}
    s = samples.cpu().numpy().mean(2)
    line = base_line("voxels/s fitted (GS+LM+MCMC), NODDI-Watson, Rician likelihood",
                     nvox / (ms / 1e3), "voxels/s", a, ms,
                     {"workload": "noddi_watson_rician_gs_lm_mcmc", "model": MODEL, "nvox": nvox,
                      "nmeas": 288, "grid_combs": 968, "nburn": NBURN, "njumps": NJUMPS,
                      "sampleevery": SE, "likelihood": "rician",
                      "l2": "inputs larger than L2 (no flush)"},
                     clk.summary(), roofline=roof, gpu_launches=gpu_launches_per_step(cfg) * a.steps,
                     posterior_mean_vs_truth={
                         "fiso_rmse": float(np.sqrt(np.mean((s[:, 0] - truth[:, 0]) ** 2))),
                         "fintra_rmse": float(np.sqrt(np.mean((s[:, 1] - truth[:, 1]) ** 2)))})
    print(json.dumps(line))


def bingham_workload(n, dev):
    """The NODDI-Bingham workload; clean signals from the library's plugin."""
    import torch
    from cudimot_gb300 import capi, synth
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    lib0 = capi.Cudimot("NODDI_Bingham", capi.model_cfg("NODDI_Bingham"))

    def signal(truth, cfp, S0):
        out = np.empty((truth.shape[0], cfp.shape[0]))
        for r0 in range(0, truth.shape[0], 1 << 18):
            tr = truth[r0:r0 + (1 << 18)]
            clean = torch.zeros(tr.shape[0], cfp.shape[0], dtype=torch.float64, device=dev)
            lib0.predicted_signal(t(tr[:, :, None]), t(cfp), t(S0[r0:r0 + tr.shape[0], None]), clean)
            out[r0:r0 + tr.shape[0]] = clean.cpu().numpy()
        return out

    return synth.noddi_bingham(n, signal_fn=signal)


def bench_bingham(a, dev):
    """NODDI-Bingham precision study: --nvox voxels (default 1,000,000) of
    the NODDI-Watson protocol and parameters plus beta = U(0,0.9) kappa and
    psi ~ U(0,pi), SNR 20; grid search over CUDIMOT's 11,050-combination
    Bingham grid -> LM -> MCMC (1250 + 1250, every 25th), FP32 model. The
    per-parameter error of the GPU fit against the FP64 CPU oracle's fit of
    the same voxels (LM from the same grid-search start, 256 voxels) and
    the posterior-mean error against the truth are reported."""
    import torch
    from cudimot_gb300 import capi, synth
    model = "NODDI_Bingham"
    n = a.nvox or 1_000_000
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    wl = bingham_workload(n, dev)
    cfg = capi.model_cfg(model, grid=synth.BINGHAM_GRID, run_mcmc=1, nburn=NBURN, njumps=NJUMPS,
                         sampleevery=SE)
    lib = capi.Cudimot(model, cfg)
    m, c, f, p0 = t(wl.meas), t(wl.cfp), t(wl.fixp), t(wl.init)
    p = p0.clone()
    samples = torch.zeros(n, 7, NJUMPS // SE, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with ClockSampler(dev.index or 0) as clk:
        torch.cuda.synchronize()
        ev[0].record(st)
        lib.gridsearch(m, p, c, f)
        ev[1].record(st)
        lib.levmar(m, p, c, f)
        ev[2].record(st)
        gs_lm = p.clone()
        lib.mcmc(m, p, c, f, samples)
        ev[3].record(st)
        torch.cuda.synchronize()
    ms = {"gridsearch": ev[0].elapsed_time(ev[1]), "levmar": ev[1].elapsed_time(ev[2]),
          "mcmc": ev[2].elapsed_time(ev[3])}
    total = sum(ms.values())
    lm_passes = lib.stats().lm_iterations
    # per-stage FP32 rates from the plugin's operation counts (FLOPs of
    # the library's Bingham plugin, averaged over the workload's voxels)
    from cudimot_gb300 import flops
    ops = flops.count_ops(model, wl.truth[:512], wl.cfp, wl.fixp[:512])
    like = flops.likelihood_flops(ops, 288)
    like_prop = ops["derived_p_one_param"] + 288 * (ops["signal"] + 3.0)
    work = {"gridsearch": 11050 * like * n, "levmar": flops.levmar_pass_flops(ops, 288, 7) * lm_passes,
            "mcmc": (NBURN + NJUMPS) * 7 * like_prop * n}
    pk = fp32_peak_tflops(dev)
    stage_rate = {st_: work[st_] / (ms[st_] / 1e3) / 1e12 for st_ in ms}
    roof = {"bound": "fp32", "kernel": "cdm_mcmc_kernel", "achieved": stage_rate["mcmc"],
            "unit": "TFLOP/s", "peak": pk["tflops"] if pk else None,
            "frac": stage_rate["mcmc"] / pk["tflops"] if pk else None,
            "peak_source": pk["source"] if pk else None,
            "flop_per_signal": ops["signal"], "stages_tflops": stage_rate,
            "note": "FP32 work of the plugin as the library evaluates it (the saddlepoint 1F1 "
                    "restated for single precision); the LM solve and the energies are FP64 "
                    "and not counted"}
    # precision study on a subset: LM in FP32 (GPU) vs FP64 (oracle) from the same start
    from oracle.oracle import Oracle
    o = Oracle(model)
    k = 256
    gs_only = p0[:k].clone()
    lib.gridsearch(m[:k].contiguous(), gs_only, c, f[:k].contiguous())
    torch.cuda.synchronize()
    start = gs_only.cpu().numpy()
    gpu_lm = start.copy()
    q = t(start)
    lib.levmar(m[:k].contiguous(), q, c, f[:k].contiguous())
    torch.cuda.synchronize()
    gpu_lm = q.cpu().numpy()
    ref_lm, _, _, _ = o.levmar(cfg, wl.meas[:k], start, wl.cfp, wl.fixp[:k])
    names = ["fiso", "fintra", "kappa", "beta"]
    vs_oracle = {nm: float(np.median(np.abs(gpu_lm[:, i] - ref_lm[:, i]) /
                                     np.maximum(np.abs(ref_lm[:, i]), 1e-3)))
                 for i, nm in enumerate(names)}
    nf = lambda th, ph: np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)  # noqa
    ang = np.degrees(np.arccos(np.clip(np.abs(np.sum(nf(gpu_lm[:, 4], gpu_lm[:, 5]) *
                                                      nf(ref_lm[:, 4], ref_lm[:, 5]), 1)), 0, 1)))
    vs_oracle["orientation_deg_median"] = float(np.median(ang))
    c_gpu = o.cost(wl.meas[:k], gpu_lm, wl.cfp, wl.fixp[:k])
    c_ref = o.cost(wl.meas[:k], ref_lm, wl.cfp, wl.fixp[:k])
    vs_oracle["cost_rel_median"] = float(np.median((c_gpu - c_ref) / c_ref))
    pm = samples.mean(2).cpu().numpy()
    truth = wl.truth
    vs_truth = {nm: float(np.sqrt(np.mean((pm[:, i] - truth[:, i]) ** 2))) for i, nm in
                enumerate(names[:2])}
    vs_truth["log_kappa_rmse"] = float(np.sqrt(np.mean((np.log(np.maximum(pm[:, 2], 1e-3)) -
                                                        np.log(truth[:, 2])) ** 2)))
    vs_truth["beta_over_kappa_rmse"] = float(np.sqrt(np.mean((pm[:, 3] / pm[:, 2] -
                                                               truth[:, 3] / truth[:, 2]) ** 2)))
    # CUDIMOT's own kernels (double, as shipped) on the first 512 voxels
    refk = None
    if os.environ.get("CDM_BENCH_REFK", "1") != "0":
        try:
            import time as _time
            from oracle.refkernels.refkernels import RefKernels, available
            if available(model):
                rk = RefKernels(model, 7)
                r = 512
                pr = p0[:r].clone()
                sr = torch.zeros(r, 7, NJUMPS // SE, dtype=torch.float64, device=dev)
                torch.cuda.synchronize()
                t0 = _time.perf_counter()
                rk.gridsearch(cfg, m[:r].contiguous(), pr, c, f[:r].contiguous(), t(cfg.grid_array))
                rk.levmar(cfg, m[:r].contiguous(), pr, c, f[:r].contiguous())
                rk.mcmc(cfg, m[:r].contiguous(), pr, c, f[:r].contiguous(), sr)
                torch.cuda.synchronize()
                dt = _time.perf_counter() - t0
                refk = {"value": r / dt, "unit": "voxels/s", "seconds": dt,
                        "sample": f"first {r} voxels, grid search -> LM -> MCMC, CUDIMOT kernels"}
        except Exception as e:  # noqa: BLE001
            refk = {"unavailable": f"{type(e).__name__}: {e}"}
    line = base_line("voxels/s fitted (GS+LM+MCMC), NODDI-Bingham", n / (total / 1e3), "voxels/s",
                     a, total,
                     {"workload": "noddi_bingham_gs_lm_mcmc", "model": model, "nvox": n, "nmeas": 288,
                      "grid_combs": 11050, "nburn": NBURN, "njumps": NJUMPS, "sampleevery": SE,
                      "l2": "inputs larger than L2 (no flush)"},
                     clk.summary(), stages_ms=ms, roofline=roof,
                     lm_iterations_per_voxel=lm_passes / n,
                     fp32_vs_fp64_oracle_lm=vs_oracle, posterior_mean_vs_truth=vs_truth,
                     reference_kernels=refk, gpu_launches=9)
    # one pass of the 1M-voxel fit (a few minutes) is the measurement
    line["steps"], line["warmup"] = 1, 0
    print(json.dumps(line))


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.profile_stage:
        profile_stage(a)
        return
    if a.impl == "ours" and a.workload != "noddi_watson":
        import torch
        torch.cuda.set_device(local)
        dev = torch.device("cuda", local)
        {"ball_1_stick_lm": bench_b1s_lm, "heterogeneous": bench_heterogeneous,
         "learned_init": bench_learned, "noddi_bingham": bench_bingham,
         "noddi_watson_rician": bench_rician}[a.workload](a, dev)
        return
    if a.impl == "reference":
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_reference(a, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cudimot_gb300 import capi
    nvox = a.nvox or NVOX
    cfp, meas, fixp, init, truth = make_workload(nvox, 8219 + rank, dev)
    cfg = workload_cfg()
    lib = capi.Cudimot(MODEL, cfg)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    d_meas, d_cfp, d_fixp, d_init = t(meas), t(cfp), t(fixp), t(init)
    d_params = d_init.clone()
    ns = NJUMPS // SE
    d_samples = torch.zeros(nvox, 5, ns, dtype=torch.float64, device=dev)

    def step():
        d_params.copy_(d_init)
        lib.fit(d_meas, d_params, d_cfp, d_fixp, d_samples)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(a.warmup):
        step()
    barrier()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(a.steps):
            step()
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / a.steps
    if world > 1:
        tt = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms = float(tt.item())
    value = nvox * world / (ms / 1e3)
    stats = lib.stats()
    # kernel-level timing of the dominant kernel (MCMC) on the same stream
    mcmc_ms = kernel_time_mcmc(lib, d_meas, d_init, d_cfp, d_fixp, d_samples, stream)

    e2e = None
    if not a.no_e2e:
        e2e = run_e2e(lib, meas, init, cfp, fixp, nvox, ns, a, world)

    if rank != 0:
        return
    fl = flop_model()
    roofline = None
    fp32_peak = fp32_peak_tflops(dev)
    if fl is not None and fp32_peak:
        per_voxel_mcmc = fl["mcmc"]
        achieved = per_voxel_mcmc * nvox / (mcmc_ms / 1e3) / 1e12
        traffic, traffic_src = measured_traffic(
            "cdm_mcmc_kernel", {"nvox": nvox, "nburn": NBURN, "njumps": NJUMPS, "sampleevery": SE,
                                "rician": False})
        roofline = {"bound": "fp32", "kernel": "cdm_mcmc_kernel", "achieved": achieved,
                    "peak": fp32_peak["tflops"], "unit": "TFLOP/s", "frac": achieved / fp32_peak["tflops"],
                    "peak_source": fp32_peak["source"], "traffic": traffic,
                    "traffic_source": traffic_src,
                    "flop_per_voxel": per_voxel_mcmc, "launch_ms": mcmc_ms}
    post = d_samples.mean(2).cpu().numpy()
    line = {"metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 model / f64 sums", "data": "synthetic (seeded NODDI-Watson, SNR 20)",
            "config": headline_config(nvox, world),
            "gpu_launches": gpu_launches_per_step(cfg) * a.steps,
            "clocks": clk.summary(),
            # cdm_fit clears the counters, so they hold the last step alone
            "lm_iterations_per_voxel": stats.lm_iterations / max(nvox, 1),
            "gs_recheck_voxels": stats.gs_recheck_voxels,
            # posterior means of the last step against the true parameters
            "param_error": param_error(post, truth),
            "roofline": roofline, "e2e": e2e}
    if os.environ.get("CDM_BENCH_CPU", "1") != "0":
        n = a.cpu_sample or 4096
        from oracle.oracle import Oracle  # noqa: F401
        v, threads, dt = cpu_baseline(cfp, meas, fixp, init, n, cfg)
        line["cpu_baseline"] = {"value": v, "unit": "voxels/s", "cores": threads, "kind": "port",
                                "sample": f"{n} voxels of this workload, grid search -> LM -> MCMC, "
                                          f"FP64 CPU oracle, {dt:.1f} s",
                                "plugin": CPU_PLUGIN_NOTE}
        nf = max(n // 2, 1)
        vf, _, dtf = cpu_baseline(cfp, meas, fixp, init, nf, cfg, prec=1)
        line["cpu_baseline"]["float"] = {
            "value": vf, "unit": "voxels/s", "cores": threads,
            "sample": f"{nf} voxels, the same CPU oracle with T = float, {dtf:.1f} s"}
    part = min(12_800, nvox)
    if os.environ.get("CDM_BENCH_REFK", "1") != "0":
        line["reference_kernels"] = reference_kernels_leg(cfp, meas, fixp, init, cfg, dev, truth,
                                                          post, n=part, n_float=part)
    if os.environ.get("CDM_BENCH_DROPIN", "1") != "0":
        line["dropin_unchanged_plugin"] = dropin_leg(cfp, meas, fixp, init, truth, post, dev, part)
    if os.environ.get("CDM_BENCH_LEARNED", "1") != "0":
        line["surrogate_vs_grid"] = learned_comparison(dev)
    print(json.dumps(line))


def reference_kernels_leg(cfp, meas, fixp, init, cfg, dev, truth, post, n=12_800, n_float=12_800):
    """CUDIMOT's own GridSearch/LM/MCMC kernels (unmodified sources compiled
    for sm_103a) on the first n voxels of this workload (one of CUDIMOT's
    12,800-voxel parts, gridOptions.h SIZE_PART), same GPU: wall time of the
    three stages, and the posterior means' error against the truth beside
    this library's on the same voxels. T = double as the plugins ship, and
    CUDIMOT's float instantiation of the same kernels."""
    import time
    import torch
    try:
        from oracle.refkernels.refkernels import RefKernels, available
        if not available(MODEL):
            return {"unavailable": "CUDIMOT kernels were not compiled (source tree absent at build time)"}
        RefKernels(MODEL, 5)
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}

    def run(k, real):
        ref = RefKernels(MODEL, 5, real=real)
        t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=real, device=dev)  # noqa
        m, c, f, p = t(meas[:k]), t(cfp), t(fixp[:k]), t(init[:k])
        s = torch.zeros(k, 5, NJUMPS // SE, dtype=real, device=dev)
        grid = t(cfg.grid_array)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ref.gridsearch(cfg, m, p, c, f, grid)
        ref.levmar(cfg, m, p, c, f)
        ref.mcmc(cfg, m, p, c, f, s)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, s.double().mean(2).cpu().numpy()

    out = {"library_param_error_same_voxels": param_error(post[:n], truth[:n])}
    dt, pm = run(n, torch.float64)
    out.update({"value": n / dt, "unit": "voxels/s", "seconds": dt,
                "sample": f"first {n} voxels of this workload (one {n}-voxel part), grid search -> "
                          "LM -> MCMC, one warp per voxel as CUDIMOT launches them, T = double",
                "param_error": param_error(pm, truth[:n])})
    try:
        k = min(n_float, len(meas))
        dtf, pmf = run(k, torch.float32)
        fin = np.isfinite(pmf).all(1)
        out["float"] = {"value": k / dtf, "unit": "voxels/s", "seconds": dtf,
                        "sample": f"first {k} voxels, CUDIMOT's float instantiation "
                                  "(MyType = float) of the same kernels",
                        "finite_posterior_means": float(fin.mean()),
                        "param_error": param_error(pmf[fin], truth[:k][fin])}
    except Exception as e:  # noqa: BLE001
        out["float"] = {"unavailable": f"{type(e).__name__}: {e}"}
    return out


def dropin_leg(cfp, meas, fixp, init, truth, post, dev, n=12_800):
    """A drop-in user's throughput: this library built from CUDIMOT's
    unchanged NODDI-Watson plugin (split build, plugin evaluated in double:
    its closed forms need it) on the first n voxels of this workload, grid
    search -> LM -> MCMC through cdm_fit, and the posterior means' error
    against the truth."""
    import torch
    from cudimot_gb300 import capi, synth
    try:
        from oracle import build_dropin
        if not build_dropin.available(MODEL, "double"):
            return {"unavailable": "device module not compiled (CUDIMOT's tree absent at build time)"}
        errs = build_dropin.build_all()
        if errs:
            return {"unavailable": "host half did not build: " + next(iter(errs.values()))[-300:]}
        cfg = capi.model_cfg(MODEL, grid=synth.WATSON_GRID, run_mcmc=1, nburn=NBURN,
                             njumps=NJUMPS, sampleevery=SE, iter_levmar=200)
        lib = capi.Cudimot(MODEL, cfg, path=build_dropin.lib_path(MODEL, "double"))
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f, p0 = t(meas[:n]), t(cfp), t(fixp[:n]), t(init[:n])
    s = torch.zeros(n, 5, NJUMPS // SE, dtype=torch.float64, device=dev)
    w = min(n, 256)  # kernels loaded on a small fit first
    pw = p0[:w].clone()
    lib.fit(m[:w].contiguous(), pw, c, f[:w].contiguous(), s[:w].contiguous())
    torch.cuda.synchronize()
    p = p0.clone()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    lib.fit(m, p, c, f, s)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    pm = s.mean(2).cpu().numpy()
    out = {"value": n / (ms / 1e3), "unit": "voxels/s", "ms": ms,
           "sample": f"first {n} voxels of this workload, grid search -> LM -> MCMC (cdm_fit)",
           "plugin": "CUDIMOT's mymodels/NODDI_Watson unchanged, evaluated in double",
           "param_error": param_error(pm, truth[:n]),
           "library_param_error_same_voxels": param_error(post[:n], truth[:n])}
    # the same plugin evaluated in single precision: what its closed forms do there
    if build_dropin.available(MODEL, "float"):
        try:
            lf = capi.Cudimot(MODEL, cfg, path=build_dropin.lib_path(MODEL, "float"))
            pf = p0.clone()
            sf = torch.zeros_like(s)
            lf.fit(m[:w].contiguous(), pf[:w].clone(), c, f[:w].contiguous(), sf[:w].contiguous())
            torch.cuda.synchronize()
            e0.record(st)
            lf.fit(m, pf, c, f, sf)
            e1.record(st)
            torch.cuda.synchronize()
            pmf = sf.mean(2).cpu().numpy()
            fin = np.isfinite(pmf).all(1)
            out["float"] = {"value": n / (e0.elapsed_time(e1) / 1e3), "unit": "voxels/s",
                            "finite_posterior_means": float(fin.mean()),
                            "param_error": param_error(pmf[fin], truth[:n][fin])}
        except Exception as e:  # noqa: BLE001
            out["float"] = {"unavailable": f"{type(e).__name__}: {e}"}
    return out


def gpu_launches_per_step(cfg):
    # prep+pack+gs+recheck, prep+pack+lm, prep+pack+mcmc
    n = 0
    if cfg.run_gridsearch:
        n += 4
    if cfg.run_levmar:
        n += 3
    n += 3 if cfg.run_mcmc else 1
    return n


def kernel_time_mcmc(lib, d_meas, d_init, d_cfp, d_fixp, d_samples, stream):
    """CUDA-event time of one MCMC stage launch (prep+pack+kernel) on the
    launching stream, from the grid-search/LM start point."""
    import torch
    p = d_init.clone()
    lib.gridsearch(d_meas, p, d_cfp, d_fixp)
    lib.levmar(d_meas, p, d_cfp, d_fixp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q = p.clone()
    e0.record(stream)
    lib.mcmc(d_meas, q, d_cfp, d_fixp, d_samples)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def fp32_peak_tflops(dev):
    """FP32 FMA peak measured on this GPU by the library's own FFMA loop."""
    try:
        from cudimot_gb300 import peak
        return peak.measure_fp32(dev)
    except Exception:  # noqa: BLE001
        return None


def run_e2e(lib, meas, init, cfp, fixp, nvox, ns, a, world):
    import torch
    pin = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64).pin_memory()  # noqa
    h_meas, h_cfp, h_fixp, h_init = pin(meas), pin(cfp), pin(fixp), pin(init)
    h_params = pin(init)
    h_samples = torch.zeros(nvox, 5, ns, dtype=torch.float64).pin_memory()
    ptr = lambda x: C.c_void_p(x.data_ptr())  # noqa

    def step():
        h_params.copy_(h_init)
        st = lib.lib.cdm_fit_host(lib.ctx, nvox, meas.shape[1], ptr(h_meas), ptr(h_params),
                                  ptr(h_cfp), ptr(h_fixp), ptr(h_samples), None, None, None, None,
                                  0, 600000)
        if st != 0:
            raise RuntimeError(lib.lib.cdm_last_error().decode())

    for _ in range(max(1, min(a.warmup, 2))):
        step()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        step()
    dt = (time.perf_counter() - t0) / a.steps
    if world > 1:
        tt = torch.tensor([dt])
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        dt = float(tt.item())
    h2d = (meas.size + init.size + cfp.size + fixp.size) * 8
    d2h = (init.size + nvox * 5 * ns) * 8
    return {"value": nvox * world / dt, "unit": "voxels/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": dt * 1e3}


if __name__ == "__main__":
    main()
