"""Time CUDIMOT's own kernels (double, as shipped) against the GPU library on
the same GPU and inputs: NODDI-Watson grid search -> LM -> MCMC on the
benchmark protocol. Test infrastructure; prints one JSON line.

    python oracle/refkernels/time_ref.py [--nvox 16000] [--bi 1250 --nj 1250]
"""
import argparse
import json
import os
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from cudimot_gb300 import capi, synth  # noqa: E402
from oracle.refkernels.refkernels import RefKernels  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nvox", type=int, default=16000)
    ap.add_argument("--bi", type=int, default=1250)
    ap.add_argument("--nj", type=int, default=1250)
    a = ap.parse_args()
    import bench
    dev = torch.device("cuda:0")
    cfp, meas, fixp, init, truth = bench.make_workload(a.nvox, 8219, dev)
    cfg = capi.model_cfg("NODDI_Watson", grid=synth.WATSON_GRID, run_mcmc=1, nburn=a.bi,
                         njumps=a.nj, sampleevery=25)
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa
    m, c, f = t(meas), t(cfp), t(fixp)
    ns = a.nj // 25
    out = {"nvox": a.nvox, "nburn": a.bi, "njumps": a.nj}

    def stage(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    ref = RefKernels("NODDI_Watson", 5)
    grid = t(cfg.grid_array)
    p = t(init)
    s = torch.zeros(a.nvox, 5, ns, dtype=torch.float64, device=dev)
    out["ref_gridsearch_s"] = stage(lambda: ref.gridsearch(cfg, m, p, c, f, grid))
    out["ref_levmar_s"] = stage(lambda: ref.levmar(cfg, m, p, c, f))
    out["ref_mcmc_s"] = stage(lambda: ref.mcmc(cfg, m, p, c, f, s))
    ours = capi.Cudimot("NODDI_Watson", cfg)
    q = t(init)
    s2 = torch.zeros_like(s)
    ours.fit(m, q, c, f, s2)  # warm-up (graph capture)
    torch.cuda.synchronize()
    q.copy_(t(init))
    out["ours_fit_s"] = stage(lambda: ours.fit(m, q, c, f, s2))
    ref_total = out["ref_gridsearch_s"] + out["ref_levmar_s"] + out["ref_mcmc_s"]
    out["ref_voxels_per_s"] = a.nvox / ref_total
    out["ours_voxels_per_s"] = a.nvox / out["ours_fit_s"]
    out["speedup"] = ref_total / out["ours_fit_s"]
    g, r = s2.cpu().numpy(), s.cpu().numpy()
    out["posterior_mean_abs_diff"] = {n: float(np.median(np.abs(g[:, i].mean(1) - r[:, i].mean(1))))
                                      for i, n in enumerate(["fiso", "fintra", "kappa"])}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
