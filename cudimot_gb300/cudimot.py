"""CUDIMOT's three command-line tools over this library, with CUDIMOT's
options and part files:

    python -m cudimot_gb300.cudimot split --model M --data D --maskfile MASK \\
        --partsdir P --nParts N [--init_params LIST] [--FixP LIST]
    python -m cudimot_gb300.cudimot fit --model M --partsdir P --idPart I --nParts N \\
        --CFP LIST [--gridSearch GRID] [--no_LevMar] [--runMCMC --bi B --nj J --se S] ...
    python -m cudimot_gb300.cudimot merge --model M --maskfile MASK --partsdir P --nParts N \\
        --outputdir O [--runMCMC --nj J --se S] [--getPredictedSignal] [--BIC_AIC] [--rician]

`split` is split_parts_<Model> (split_parts.cc:38-277), `fit` is
cudimot_<Model> for one part (cudimot.cc:25-125 with the part files of
dMRI_Data.cu:37-62 and Parameters.cu:30-235,383-520) and `merge` is
merge_parts_<Model> (merge_parts.cc:64-151). `run` does all three for every
part in one process. The model's default priors file is its modelpriors
(CUDIMOT's <binary>_priors); --priors overrides it.

The fit runs on the GPU through cdm_fit_host; with --rician the signals
are cleaned first as dMRI_Data::getMeasPart does (cdm_clean_signals).
Options CUDIMOT accepts that change nothing here: --ld/--logdir, --forcedir,
--upe (CUDIMOT adapts the proposals every --se jumps, MCMC.cu:711),
--keepTmp for split/fit, --debug (per-voxel printing is not restated).
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import shutil
import sys

import numpy as np

from . import capi, utils, volumes
from .build import MODELS


def _add_common(ap):
    ap.add_argument("--model", required=True, help="model library (mymodels/<Model>)")
    ap.add_argument("--partsdir", required=True)
    ap.add_argument("--nParts", type=int, required=True)
    ap.add_argument("--priors", default="")
    ap.add_argument("--ld", "--logdir", dest="logdir", default="logdir")
    ap.add_argument("--forcedir", action="store_true")
    ap.add_argument("--debug", default="")


def _add_fit(ap):
    ap.add_argument("--nj", "--njumps", dest="njumps", type=int, default=1250)
    ap.add_argument("--bi", "--burnin", dest="nburn", type=int, default=1000)
    ap.add_argument("--se", "--sampleevery", dest="sampleevery", type=int, default=25)
    ap.add_argument("--upe", "--updateproposalevery", dest="upe", type=int, default=40)
    ap.add_argument("--no_updateproposal", action="store_true")
    ap.add_argument("--seed", type=int, default=8219)
    ap.add_argument("--no_LevMar", action="store_true")
    ap.add_argument("--no_Marquardt", action="store_true")
    ap.add_argument("--iterLevMar", type=int, default=200)
    ap.add_argument("--gridSearch", default="")
    ap.add_argument("--runMCMC", action="store_true")
    ap.add_argument("--rician", action="store_true")
    ap.add_argument("--keepTmp", action="store_true")
    ap.add_argument("--getPredictedSignal", action="store_true")
    ap.add_argument("--CFP", default="")
    ap.add_argument("--FixP", default="")
    ap.add_argument("--fixed", default="")
    ap.add_argument("--init_params", default="")
    ap.add_argument("--BIC_AIC", action="store_true")


def parser():
    ap = argparse.ArgumentParser(prog="cudimot_gb300.cudimot", description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    sp = sub.add_parser("split")
    _add_common(sp)
    _add_fit(sp)
    sp.add_argument("--data", required=True)
    sp.add_argument("--maskfile", required=True)
    fp = sub.add_parser("fit")
    _add_common(fp)
    _add_fit(fp)
    fp.add_argument("--idPart", type=int, required=True)
    mp = sub.add_parser("merge")
    _add_common(mp)
    _add_fit(mp)
    mp.add_argument("--maskfile", required=True)
    mp.add_argument("--outputdir", required=True)
    rp = sub.add_parser("run")
    _add_common(rp)
    _add_fit(rp)
    rp.add_argument("--data", required=True)
    rp.add_argument("--maskfile", required=True)
    rp.add_argument("--outputdir", required=True)
    return ap


class CudimotError(RuntimeError):
    pass


def _need_method(o):
    # cudimot.cc:37-41, split_parts.cc:45-49
    if o.gridSearch == "" and o.no_LevMar and not o.runMCMC:
        raise CudimotError("You must select at least one method to fit the model: GridSearch, "
                           "Levenberg_Marquardt or MCMC")


def _priors_path(o):
    if o.priors:
        return o.priors
    p = os.path.join(MODELS, o.model, "modelpriors")
    if not os.path.exists(p):
        raise CudimotError(f"no modelpriors for {o.model}: give --priors")
    return p


def model_info(model):
    lib = capi.load_library(model)
    info = capi.ModelInfo()
    capi._check(lib, lib.cdm_get_model_info(C.byref(info)), "model info")
    return lib, info


def make_cfg(o, info, lib):
    """The cdm_model_cfg cudimot.cc builds from the options and the model's
    priors file (Model.cu:16-393)."""
    cfg, p_init = capi.parse_priors(o.model, _priors_path(o), info.nparams)
    s = cfg.struct
    if o.gridSearch:
        ngp, combs = C.c_int(), C.c_int()
        gp = (C.c_int * capi.CDM_MAX_PARAMS)()
        capi._check(lib, lib.cdm_parse_grid(o.gridSearch.encode(), C.byref(ngp), C.cast(gp, C.c_void_p),
                                            C.byref(combs), None, 0), "gridSearch")
        grid = np.zeros((combs.value, ngp.value))
        capi._check(lib, lib.cdm_parse_grid(o.gridSearch.encode(), C.byref(ngp), C.cast(gp, C.c_void_p),
                                            C.byref(combs), grid.ctypes.data_as(C.c_void_p), grid.size),
                    "gridSearch")
        cfg._grid = grid
        s.n_grid_params = ngp.value
        for k in range(ngp.value):
            s.grid_params[k] = gp[k]
        s.grid_combs = combs.value
        s.grid = grid.ctypes.data_as(C.POINTER(C.c_double))
        s.run_gridsearch = 1
    if o.fixed:
        fx = (C.c_int * capi.CDM_MAX_PARAMS)()
        capi._check(lib, lib.cdm_parse_fixed(o.fixed.encode(), C.cast(fx, C.c_void_p)), "--fixed")
        for k in range(info.nparams):
            s.fixed[k] = fx[k]
    s.run_levmar = 0 if o.no_LevMar else 1
    s.marquardt = 0 if o.no_Marquardt else 1
    s.iter_levmar = o.iterLevMar
    s.run_mcmc = 1 if o.runMCMC else 0
    s.nburn, s.njumps, s.sampleevery = o.nburn, o.njumps, o.sampleevery
    s.update_proposal = 0 if o.no_updateproposal else 1
    s.rician = 1 if o.rician else 0
    s.get_predicted = 1 if o.getPredictedSignal else 0
    s.bic_aic = 1 if o.BIC_AIC else 0
    s.seed = o.seed
    s.id_part = getattr(o, "idPart", 0)
    return cfg, p_init


def nsamples(o):
    # Parameters.cu:334-339, merge_parts.cc:74-79
    return o.njumps // o.sampleevery if o.runMCMC else 1


def split(o):
    """split_parts_<Model>."""
    _need_method(o)
    lib, info = model_info(o.model)
    p_init = None
    if o.init_params:
        _, p_init = capi.parse_priors(o.model, _priors_path(o), info.nparams)
    sizes = [info.fixp_size[i] for i in range(info.nfixp)]
    return volumes.split_volumes(o.partsdir, o.nParts, o.data, o.maskfile, info.nparams,
                                 init_list=o.init_params or None, init_values=p_init,
                                 fixp_list=o.FixP or None, fixp_sizes=sizes)


def _read_part(partsdir, idp, name, nvox, rows, what):
    a = utils.part_read(utils.part_path(partsdir, idp, name))
    if a.shape != (nvox, rows):
        raise CudimotError(f"The amount of data in the input file {name} for {what} is not correct")
    return a


def fit_part(o):
    """cudimot_<Model> on part --idPart: returns the arrays it wrote."""
    _need_method(o)
    lib, info = model_info(o.model)
    cfg, p_init = make_cfg(o, info, lib)
    pd = o.partsdir
    meas = utils.part_read(utils.part_path(pd, o.idPart, "data"))   # dMRI_Data.cu:37-62
    nvox, nmeas = meas.shape
    if nvox <= 0 or nmeas <= 0:
        raise CudimotError("The number of voxels and diffusion-weighted measurements in the input "
                           "file must be greater than 0")
    npar = info.nparams
    params = np.zeros((nvox, npar))
    if o.init_params:                                                   # Parameters.cu:42-75
        for p in range(npar):
            params[:, p] = _read_part(pd, o.idPart, f"ParamInit_{p}", nvox, 1, "initializing the parameters")[:, 0]
    elif p_init is not None:                                            # Parameters.cu:77-88
        params[:] = np.asarray(p_init)[None, :npar]
    cfp = np.zeros((nmeas, max(info.cfp_tsize, 1)))
    if info.cfp_tsize:
        if not o.CFP:
            raise CudimotError("The user must provide a file with a list of Common Fixed Parameters: "
                               "Use option --CFP")
        capi._check(lib, lib.cdm_read_cfp_list(o.CFP.encode(), nmeas, cfp.ctypes.data_as(C.c_void_p)),
                    "--CFP")
    fixp = np.zeros((nvox, max(info.fixp_tsize, 1)))
    if info.fixp_tsize:                                                 # Parameters.cu:150-203
        if not o.FixP:
            raise CudimotError("The user must provide a file with a list of Fixed Parameters for "
                               "this model: Use option --FixP")
        col = 0
        for i in range(info.nfixp):
            w = info.fixp_size[i]
            fixp[:, col:col + w] = _read_part(pd, o.idPart, f"FixParam_{i}", nvox, w, "Fixed Parameters")
            col += w
    ns = nsamples(o)
    samples = np.zeros((nvox, npar, ns))
    tau = np.zeros((nvox, ns)) if (o.rician and o.runMCMC) else None
    pred = np.zeros((nvox, nmeas)) if o.getPredictedSignal else None
    bic = np.zeros(nvox) if o.BIC_AIC else None
    aic = np.zeros(nvox) if o.BIC_AIC else None
    fit = capi.Cudimot(o.model, cfg)
    try:
        fit.fit_host(meas, params, cfp, fixp, samples, tau, pred, bic, aic)
    finally:
        fit.close()
    out = {f"Param_{p}_samples": samples[:, p, :] for p in range(npar)}   # Parameters.cu:383-421
    if tau is not None:
        out["Tau_samples"] = tau
    if pred is not None:
        out["PredictedSignal"] = pred
    if bic is not None:
        out["BIC"] = bic[:, None]
        out["AIC"] = aic[:, None]
    for name, a in out.items():
        utils.part_write(utils.part_path(pd, o.idPart, name), a)
    return out


def merge(o):
    """merge_parts_<Model>: the outputs as NIfTI volumes in --outputdir."""
    lib, info = model_info(o.model)
    ns = nsamples(o)
    if ns <= 0:
        raise CudimotError("The number of samples must be greater than 0")
    os.makedirs(o.outputdir, exist_ok=True)
    ext = ".nii.gz" if volumes.gzip_supported() else ".nii"
    jobs = [(f"Param_{p}_samples", ns) for p in range(info.nparams)]
    if o.getPredictedSignal:
        jobs.append(("PredictedSignal", -1))
    if o.BIC_AIC:
        jobs += [("BIC", 1), ("AIC", 1)]
    if o.rician and o.runMCMC:
        jobs.append(("Tau_samples", ns))
    written = []
    for name, rows in jobs:
        out = os.path.join(o.outputdir, name + ext)
        volumes.merge_volumes(o.partsdir, o.nParts, name, o.maskfile, out, nrows=rows)
        written.append(out)
    if not o.keepTmp:                                                   # merge_parts.cc:143-146
        shutil.rmtree(o.partsdir, ignore_errors=True)
    return written


def run(o):
    split(o)
    keep = o.keepTmp
    for i in range(o.nParts):
        o.idPart = i
        fit_part(o)
    o.keepTmp = keep
    return merge(o)


def main(argv=None):
    o = parser().parse_args(argv)
    try:
        {"split": split, "fit": fit_part, "merge": merge, "run": run}[o.cmd](o)
    except (CudimotError, capi.CdmError) as e:
        print(f"CUDIMOT Error: {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
