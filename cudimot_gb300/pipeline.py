"""Multi-stage fitting pipelines on the GPU, captured as one CUDA graph.

Restates the pipeline scripts of CUDIMOT's models (what their
Pipeline_<Model>.sh queue as separate jobs) as one sequence of device
work on the same arrays:
  S0 (mean of the b <= 50 volumes, Pipeline_NODDI_Watson.sh:155-170)
  -> log-linear tensor fit (dtifit + cart2spherical + initialise_Psi)
  -> the model's steps (grid search with some parameters fixed, fits of a
     subset, the full fit with LM and optionally MCMC)
  -> *_finish.sh post-processing (sample means, dyadic vectors, OD).
Every step updates one parameter array in place: a parameter a step keeps
fixed reaches the next step unchanged, which is how the scripts pass
Param_<i>_samples of one step as the next step's --init_params.

`Pipeline.run()` records all of it once with CUDA stream capture (each
step through cdm_fit_enqueue, the rest through libcdm_utils) and then
replays the graph: one launch per volume.
"""
from __future__ import annotations

import numpy as np

from . import capi, synth, utils

# initialisation from the tensor fit: (parameter, DTI column, scale); a
# column of None sets the constant `scale`
DTI = {c: k for k, c in enumerate(utils.DTI_COLS)}

PIPELINES = {
    # Pipeline_Ball_1_Stick.sh:160-171: one fit from dtifit's S0, L1, FA, V1
    "Ball_1_Stick": dict(
        s0_fixp=False,
        init=[(0, "S0", 1.0), (1, "L1", 1.0), (2, "FA", 1.0), (3, "TH1", 1.0), (4, "PH1", 1.0)],
        steps=[dict(name="fit", last=True)]),
    # Pipeline_Ball_2_Sticks.sh:150-168: S0, L1, FA, V1, FA/4, V2
    "Ball_2_Sticks": dict(
        s0_fixp=False,
        init=[(0, "S0", 1.0), (1, "L1", 1.0), (2, "FA", 1.0), (3, "TH1", 1.0), (4, "PH1", 1.0),
              (5, "FA", 0.25), (6, "TH2", 1.0), (7, "PH2", 1.0)],
        steps=[dict(name="fit", last=True)]),
    # Pipeline_NODDI_Watson.sh:183-247: grid search with the orientation
    # fixed, then the fractions with kappa and orientation fixed, then all
    "NODDI_Watson": dict(
        s0_fixp=True,
        init=[(0, None, 0.0), (1, None, 0.0), (2, None, 0.0), (3, "TH1", 1.0), (4, "PH1", 1.0)],
        steps=[dict(name="GridSearch", grid="watson", levmar=False, fixed=(3, 4)),
               dict(name="FitFractions", fixed=(2, 3, 4)),
               dict(name="fit", last=True)],
        finish=dict(theta=3, phi=4, kappa=2)),
    # Pipeline_NODDI_Bingham.sh:190-235: grid search + LM with the
    # orientation fixed, then all but fiso
    "NODDI_Bingham": dict(
        s0_fixp=True,
        init=[(0, None, 0.0), (1, None, 0.0), (2, None, 0.0), (3, None, 0.0), (4, "TH1", 1.0),
              (5, "PH1", 1.0), (6, "PSI", 1.0)],
        steps=[dict(name="GridSearch", grid="bingham", fixed=(4, 5)),
               dict(name="fit", fixed=(0,), last=True)],
        finish=dict(theta=4, phi=5, kappa=2)),
}

GRIDS = {"watson": synth.WATSON_GRID, "bingham": synth.BINGHAM_GRID}


class Pipeline:
    """One model's pipeline on one volume (meas [nvox][nmeas] CUDA float64,
    bvecs [nmeas][3] and bvals [nmeas] numpy)."""

    def __init__(self, model, meas, bvecs, bvals, run_mcmc=False, nburn=1250, njumps=1250,
                 sampleevery=25, b0_max=50.0, lanes=None):
        import torch
        self.torch = torch
        self.model = model
        self.spec = PIPELINES[model]
        self.meas = meas
        dev = meas.device
        self.dev = dev
        n, nm = meas.shape
        self.n = n
        self.bvecs = np.ascontiguousarray(bvecs, dtype=np.float64)
        self.bvals = np.ascontiguousarray(bvals, dtype=np.float64)
        self.cfp = torch.as_tensor(np.concatenate([self.bvecs, self.bvals[:, None]], 1),
                                   dtype=torch.float64, device=dev)
        info = capi.Cudimot(model, capi.model_cfg(model)).info
        self.nparams = info.nparams
        self.fixp = torch.zeros(n, max(info.fixp_tsize, 1), dtype=torch.float64, device=dev)
        self.b0 = torch.as_tensor(np.nonzero(self.bvals <= b0_max)[0].astype(np.int32), device=dev)
        self.dti = torch.zeros(n, len(utils.DTI_COLS), dtype=torch.float64, device=dev)
        self.params = torch.zeros(n, self.nparams, dtype=torch.float64, device=dev)
        self.ctx = []
        for st in self.spec["steps"]:
            kw = dict(fixed=st.get("fixed", ()), run_levmar=int(st.get("levmar", True)))
            if "grid" in st:
                kw["grid"] = GRIDS[st["grid"]]
            if st.get("last") and run_mcmc:
                kw.update(run_mcmc=1, nburn=nburn, njumps=njumps, sampleevery=sampleevery)
            if lanes:
                kw.update(lanes)
            cfg = capi.model_cfg(model, **kw)
            lib = capi.Cudimot(model, cfg)
            lib.fit_reserve(n, nm)
            ns = njumps // sampleevery if (st.get("last") and run_mcmc) else 1
            samples = torch.zeros(n, self.nparams, ns, dtype=torch.float64, device=dev)
            self.ctx.append((st, lib, samples))
        self.samples = self.ctx[-1][2]
        self.mean = torch.zeros(n, self.nparams, dtype=torch.float64, device=dev)
        self.sd = torch.zeros_like(self.mean)
        fin = self.spec.get("finish")
        self.dyads = torch.zeros(n, 4, dtype=torch.float64, device=dev) if fin else None
        self.od = torch.zeros(n, dtype=torch.float64, device=dev) if fin else None
        self.graph = None

    def _record(self):
        if self.spec["s0_fixp"]:
            utils.mean_columns(self.meas, self.b0, self.fixp)
        utils.dti_fit(self.meas, self.bvecs, self.bvals, out=self.dti)
        for p, col, scale in self.spec["init"]:
            if col is None:
                utils.copy_columns(None, 0, self.params, p, 1, scale)
            else:
                utils.copy_columns(self.dti, DTI[col], self.params, p, 1, scale)
        for st, lib, samples in self.ctx:
            lib.fit_enqueue(self.meas, self.params, self.cfp, self.fixp, samples)
        utils.sample_stats_into(self.samples, self.mean, self.sd)
        fin = self.spec.get("finish")
        if fin:
            utils.dyads_into(self.samples, fin["theta"], fin["phi"], self.dyads)
            utils.od_from_kappa(self.mean[:, fin["kappa"]], out=self.od)

    def run(self, graph=True):
        """Run the pipeline; with graph=True the first call captures it and
        every call replays the captured graph."""
        torch = self.torch
        if not graph:
            self._record()
            return
        if self.graph is None:
            torch.cuda.synchronize()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s, capture_error_mode="thread_local"):
                self._record()
            self.graph = g
            torch.cuda.current_stream().wait_stream(s)
        self.graph.replay()
