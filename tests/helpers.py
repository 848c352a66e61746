"""Shared workload builders for the tests (signals from the CPU oracle)."""
import numpy as np

from cudimot_gb300 import capi, synth
from oracle.oracle import Oracle

_ORACLES = {}


def oracle(model):
    if model not in _ORACLES:
        _ORACLES[model] = Oracle(model)
    return _ORACLES[model]


def watson(nvox, seed=8219, snr=20.0):
    o = oracle("NODDI_Watson")
    return synth.noddi_watson(nvox, seed=seed, snr=snr,
                              signal_fn=lambda t, cfp, s0: o.signal(t, cfp, s0[:, None]))


def b1s(nvox, seed=8219):
    return synth.ball_1_stick(nvox, seed=seed)


def dt(nvox, seed=8219):
    return synth.diffusion_tensor(nvox, seed=seed)


def b2s(nvox, seed=8219):
    return synth.ball_2_sticks(nvox, seed=seed)


def bingham(nvox, seed=8219, snr=20.0):
    o = oracle("NODDI_Bingham")
    return synth.noddi_bingham(nvox, seed=seed, snr=snr,
                               signal_fn=lambda t, cfp, s0: o.signal(t, cfp, s0[:, None]))


def angle_deg(th1, ph1, th2, ph2):
    """Angle between two axes (sign-insensitive), degrees."""
    v1 = np.stack([np.sin(th1) * np.cos(ph1), np.sin(th1) * np.sin(ph1), np.cos(th1)], -1)
    v2 = np.stack([np.sin(th2) * np.cos(ph2), np.sin(th2) * np.sin(ph2), np.cos(th2)], -1)
    c = np.abs(np.sum(v1 * v2, -1)).clip(0, 1)
    return np.degrees(np.arccos(c))


def lm_voxelwise(c_got, c_ref, ang=None, rtol=1e-4, adeg=0.5):
    """LM parity voxel by voxel: the library's final cost within rtol
    (relative) of the reference's and, where the angle between the fitted
    orientations is given, within adeg degrees; or else the library's cost
    lower than the reference's. Returns (mask of voxels that are neither,
    report: their number and largest cost excess, and how many voxels ended
    lower by more than rtol)."""
    rel = (c_got - c_ref) / c_ref
    agree = np.abs(rel) <= rtol
    if ang is not None:
        agree &= ang <= adeg
    bad = ~(agree | (c_got < c_ref))
    rep = {"voxels": int(rel.size), "failing": int(bad.sum()),
           "max_excess": float(rel[bad].max()) if bad.any() else 0.0,
           "lower_by_more_than_rtol": int(np.sum(rel < -rtol)),
           "max_rel": float(rel.max())}
    return bad, rep


def assert_lm_voxelwise(c_got, c_ref, ang=None, max_frac=0.0, max_excess=0.0):
    """lm_voxelwise, asserted. A single-precision LM and an FP64 one from
    the same start can part ways at a saddle or on a flat valley floor and
    end at different stationary points, either side: voxels that neither
    agree nor end lower are allowed up to max_frac of the voxels, each at
    most max_excess (relative cost) above the reference. The report says how
    many ended lower instead."""
    bad, rep = lm_voxelwise(c_got, c_ref, ang)
    assert bad.mean() <= max_frac and rep["max_excess"] <= max_excess, rep
    return rep
