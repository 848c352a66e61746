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
    ap.add_argument("--nvox", type=int, default=NVOX)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0, help="voxels for the CPU baseline")
    ap.add_argument("--profile-stage", choices=["gridsearch", "levmar", "mcmc"], default=None,
                    help="run the preceding stages, then one launch of this stage (for ncu)")
    ap.add_argument("--nburn", type=int, default=NBURN)
    ap.add_argument("--njumps", type=int, default=NJUMPS)
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


def make_workload(nvox, seed, dev):
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
    meas = synth.rician(clean, S0 / 20.0, r_noise)
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


def cpu_baseline(cfp, meas, fixp, init, n, cfg):
    """CPU oracle on n voxels: grid search -> LM -> MCMC, all host threads."""
    from oracle.oracle import Oracle
    o = Oracle(MODEL)
    threads = o.max_threads()
    sl = slice(0, n)
    t0 = time.perf_counter()
    p, _, _ = o.gridsearch(cfg, meas[sl], init[sl], cfp, fixp[sl], threads=threads)
    p, _, _, _ = o.levmar(cfg, meas[sl], p, cfp, fixp[sl], threads=threads)
    p, s, _ = o.mcmc(cfg, meas[sl], p, cfp, fixp[sl], threads=threads)
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


def run_reference(a, rank, world):
    if rank != 0:
        return
    from cudimot_gb300 import synth
    import torch  # noqa: F401
    cfg = workload_cfg()
    # inputs generated on the host: noiseless signal from the CPU oracle
    from oracle.oracle import Oracle
    o = Oracle(MODEL)
    n = a.cpu_sample or 24 * o.max_threads()
    wl = synth.noddi_watson(n, signal_fn=lambda t, c, s0: o.signal(t, c, s0[:, None]))
    times = []
    for i in range(a.warmup + a.steps):
        v, threads, dt = cpu_baseline(wl.cfp, wl.meas, wl.fixp, wl.init, n, cfg)
        if i >= a.warmup:
            times.append(dt)
    dt = float(np.mean(times))
    value = n / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s",
            "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded NODDI-Watson, SNR 20)",
            "config": {"workload": "noddi_watson_gs_lm_mcmc", "model": MODEL, "nvox_full": NVOX,
                       "nvox_sample": n, "nmeas": 288, "grid_combs": 968, "nburn": NBURN,
                       "njumps": NJUMPS, "sampleevery": SE},
            "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": threads, "kind": "port",
                             "sample": f"{n} voxels of the 200k-voxel workload per step, full "
                                       "grid search -> LM -> MCMC, FP64 CPU oracle"},
            "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def profile_stage(a):
    """One launch of one stage on a small case, for ncu captures."""
    import torch
    from cudimot_gb300 import capi, synth
    dev = torch.device("cuda:0")
    cfp, meas, fixp, init, _ = make_workload(a.nvox, 8219, dev)
    cfg = capi.model_cfg(MODEL, grid=synth.WATSON_GRID, run_mcmc=1, nburn=a.nburn,
                         njumps=a.njumps, sampleevery=SE)
    lib = capi.Cudimot(MODEL, cfg)
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
        s = torch.zeros(a.nvox, 5, max(a.njumps // SE, 1), dtype=torch.float64, device=dev)
        lib.mcmc(m, p, c, f, s)
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"stage": a.profile_stage, "nvox": a.nvox, "ms": e0.elapsed_time(e1)}))


def profiled_traffic():
    """Per-launch DRAM bytes of the MCMC kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "mcmc_kernel_noddi_watson.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.profile_stage:
        profile_stage(a)
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
    nvox = a.nvox
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
    peaks = measured_peaks()
    fl = flop_model()
    roofline = None
    fp32_peak = fp32_peak_tflops(dev)
    if fl is not None and fp32_peak:
        per_voxel_mcmc = fl["mcmc"]
        achieved = per_voxel_mcmc * nvox / (mcmc_ms / 1e3) / 1e12
        roofline = {"bound": "fp32", "kernel": "cdm_mcmc_kernel", "achieved": achieved,
                    "peak": fp32_peak["tflops"], "unit": "TFLOP/s", "frac": achieved / fp32_peak["tflops"],
                    "peak_source": fp32_peak["source"], "traffic": profiled_traffic(),
                    "traffic_source": "profiles/mcmc_kernel_noddi_watson.md (small-case ncu capture scaled by voxels)",
                    "flop_per_voxel": per_voxel_mcmc, "launch_ms": mcmc_ms}
    line = {"metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 model / f64 sums", "data": "synthetic (seeded NODDI-Watson, SNR 20)",
            "config": {"workload": "noddi_watson_gs_lm_mcmc", "model": MODEL, "nvox_per_gpu": nvox,
                       "nmeas": 288, "grid_combs": 968, "nburn": NBURN, "njumps": NJUMPS,
                       "sampleevery": SE, "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"voxel shards x{world}"},
            "gpu_launches": gpu_launches_per_step(cfg) * a.steps,
            "clocks": clk.summary(),
            # cdm_fit clears the counters, so they hold the last step alone
            "lm_iterations_per_voxel": stats.lm_iterations / max(nvox, 1),
            "gs_recheck_voxels": stats.gs_recheck_voxels,
            "roofline": roofline, "e2e": e2e}
    if os.environ.get("CDM_BENCH_CPU", "1") != "0":
        n = a.cpu_sample or 4096
        from oracle.oracle import Oracle  # noqa: F401
        v, threads, dt = cpu_baseline(cfp, meas, fixp, init, n, cfg)
        line["cpu_baseline"] = {"value": v, "unit": "voxels/s", "cores": threads, "kind": "port",
                                "sample": f"{n} voxels of this workload, grid search -> LM -> MCMC, "
                                          f"FP64 CPU oracle, {dt:.1f} s"}
    if os.environ.get("CDM_BENCH_REFK", "1") != "0":
        line["reference_kernels"] = reference_kernels_leg(cfp, meas, fixp, init, cfg, dev)
    print(json.dumps(line))


def reference_kernels_leg(cfp, meas, fixp, init, cfg, dev, n=2048):
    """CUDIMOT's own GridSearch/LM/MCMC kernels (unmodified sources compiled
    for sm_103a, T = double as shipped) on the first n voxels of this
    workload, same GPU; wall time of the three stages."""
    import time
    import torch
    try:
        from oracle.refkernels.refkernels import RefKernels, available
        if not available(MODEL):
            return {"unavailable": "CUDIMOT kernels were not compiled (source tree absent at build time)"}
        ref = RefKernels(MODEL, 5)
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f, p = t(meas[:n]), t(cfp), t(fixp[:n]), t(init[:n])
    s = torch.zeros(n, 5, NJUMPS // SE, dtype=torch.float64, device=dev)
    grid = t(cfg.grid_array)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref.gridsearch(cfg, m, p, c, f, grid)
    ref.levmar(cfg, m, p, c, f)
    ref.mcmc(cfg, m, p, c, f, s)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "voxels/s", "seconds": dt,
            "sample": f"first {n} voxels of this workload, grid search -> LM -> MCMC, "
                      "one warp per voxel as CUDIMOT launches them"}


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
