"""Algorithmic FP32 work per voxel, from the operation-count build of the
plugin (csrc/host/cdm_flops.cpp).

Work model (per voxel, one parameter proposal = one likelihood):
  likelihood  = Derived_P + nmeas * (Predicted_Signal + 3)   [r=s-y, r*r, +]
  MCMC        = (nburn + njumps) * free_params * likelihood, with Derived_P
                counted after a single-parameter change (cached blocks reused)
  grid search = combinations * likelihood, Derived_P from scratch
Counts +, -, *, / as one FLOP each; transcendental and square-root calls
are reported separately (they run on the SFU/MUFU path).
"""
import ctypes as C
import os

import numpy as np

from .capi import LIBDIR


def count_ops(model, params, cfp, fixp):
    lib = C.CDLL(os.path.join(LIBDIR, f"libcdm_flops_{model}.so"))
    lib.cdm_count_ops.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.cdm_count_ops.restype = C.c_int
    params = np.ascontiguousarray(params, dtype=np.float64)
    cfp = np.ascontiguousarray(cfp, dtype=np.float64)
    fixp = np.ascontiguousarray(fixp, dtype=np.float64)
    out = np.zeros(8)
    lib.cdm_count_ops(params.shape[0], params.ctypes.data, cfp.shape[0], cfp.ctypes.data,
                      fixp.ctypes.data, out.ctypes.data)
    keys = ("derived_p", "signal", "jacobian", "derived_p_mufu", "signal_mufu", "jacobian_mufu",
            "derived_p_one_param", "derived_p_one_param_mufu")
    return dict(zip(keys, out.tolist()))


def likelihood_flops(ops, nmeas):
    return ops["derived_p"] + nmeas * (ops["signal"] + 3.0)


def levmar_pass_flops(ops, nmeas, nparams):
    """One LM pass of the fused kernel per voxel: for every measurement the
    signal, the Jacobian row, the residual, J^T r (2 per parameter) and the
    upper triangle of J^T J (2 per entry); plus Derived_P. The FP64 solve is
    not counted (it runs on the FP64 pipe, n^3/6 multiply-adds)."""
    per_meas = ops["signal"] + ops["jacobian"] + 1.0 + 2.0 * nparams + nparams * (nparams + 1)
    return ops["derived_p"] + nmeas * per_meas


def watson_c1_flops_per_voxel(nburn=1250, njumps=1250, combs=968, nmeas=288, n=512, seed=1):
    """NODDI-Watson FLOPs per voxel of the C1 workload, averaged over
    parameters drawn from its prior and its 288-measurement protocol."""
    from . import synth
    rng = np.random.default_rng(seed)
    cfp = synth.protocol(18, [(90, 1000.0), (90, 2000.0), (90, 3000.0)], rng)
    truth, S0 = synth.watson_truth(n, rng)
    ops = count_ops("NODDI_Watson", truth, cfp, S0[:, None])
    like = likelihood_flops(ops, nmeas)
    like_prop = ops["derived_p_one_param"] + nmeas * (ops["signal"] + 3.0)
    return {"ops": ops, "likelihood": like, "likelihood_proposal": like_prop,
            "mcmc": (nburn + njumps) * 5 * like_prop, "gridsearch": combs * like}
