"""CUDIMOT's tools end to end on the GPU: split_parts -> cudimot (every part)
-> merge_parts on NIfTI volumes, against the same fit called directly on
the voxels inside the mask; and the Rician signal cleaning of
dMRI_Data.cu:15-30,133 against its oracle (bit-exact)."""
import os

import numpy as np
import pytest
import torch

from cudimot_gb300 import capi, cudimot, volumes
from oracle.data_oracle import remove_nonpositive
from tests.helpers import b1s, watson
from tests.test_volumes import make_nifti, parse_nifti

pytestmark = pytest.mark.gpu


def test_clean_signals_matches_oracle(built, cuda):
    rng = np.random.default_rng(5)
    meas = rng.uniform(-50, 1000, size=(3000, 97))
    meas[::7] = np.abs(meas[::7])                 # voxels without non-positive entries
    meas[::11] = -np.abs(meas[::11])              # voxels without positive entries
    meas[5, :] = 0.0
    meas[9, 3] = 1e-300                           # positive, but 0 as a float
    meas[13, ::2] = 0.0
    fit = capi.Cudimot("Ball_1_Stick", capi.model_cfg("Ball_1_Stick"))
    d = torch.as_tensor(meas, device=cuda)
    fit.clean_signals(d)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), remove_nonpositive(meas))


def _scene(tmp, wl, shape, seed):
    """Embed a workload's voxels in a volume: (mask, paths)."""
    rng = np.random.default_rng(seed)
    nx = int(np.prod(shape))
    sel = np.sort(rng.choice(nx, wl.nvox, replace=False))
    mask = np.zeros(nx)
    mask[sel] = 1.0
    mask = mask.reshape(shape)
    data = volumes.mask_scatter(wl.meas, mask)
    p = {"mask": str(tmp / "mask.nii"), "data": str(tmp / "data.nii")}
    make_nifti(p["mask"], mask.astype(np.uint8), datatype=2)
    make_nifti(p["data"], data, datatype=64)
    np.savetxt(tmp / "bvecs", wl.cfp[:, :3].T)
    np.savetxt(tmp / "bvals", wl.cfp[:, 3:4].T)
    (tmp / "cfp.txt").write_text(f"{tmp / 'bvecs'}\n{tmp / 'bvals'}\n")
    p["cfp"] = str(tmp / "cfp.txt")
    return mask, p


def parts(nvox, nparts):
    """Voxel ranges of split_parts (split_parts.cc:80-94)."""
    size = nvox // nparts
    return [(i * size, nvox if i == nparts - 1 else (i + 1) * size) for i in range(nparts)]


def _nifti_voxels(path, mask):
    r = parse_nifti(path)["data"]
    return r.reshape(r.shape[0], -1)[:, mask.ravel() > 0].T


def test_b1s_lm_through_the_tools(built, cuda, tmp_path):
    wl = b1s(500, seed=4)
    mask, p = _scene(tmp_path, wl, (10, 9, 8), 1)
    init = []
    for k in range(5):
        f = tmp_path / f"init{k}.nii"
        make_nifti(str(f), volumes.mask_scatter(wl.init[:, k], mask)[0], datatype=64)
        init.append(str(f))
    (tmp_path / "init.txt").write_text("\n".join(init) + "\n")
    out = str(tmp_path / "out")
    rc = cudimot.main(["run", "--model", "Ball_1_Stick", "--data", p["data"], "--maskfile", p["mask"],
                       "--partsdir", str(tmp_path / "parts"), "--nParts", "3", "--outputdir", out,
                       "--CFP", p["cfp"], "--init_params", str(tmp_path / "init.txt"), "--BIC_AIC"])
    assert rc == 0
    cfg = capi.model_cfg("Ball_1_Stick", bic_aic=1)
    fit = capi.Cudimot("Ball_1_Stick", cfg)
    ext = ".nii.gz" if volumes.gzip_supported() else ".nii"
    # the same fit called directly on each part's voxels (the lane-group
    # width, and so the summation order, is chosen from the part's size)
    params = wl.init.copy()
    samples = np.zeros((wl.nvox, 5, 1))
    bic, aic = np.zeros(wl.nvox), np.zeros(wl.nvox)
    for v0, v1 in parts(wl.nvox, 3):
        sl = slice(v0, v1)
        fit.fit_host(np.ascontiguousarray(wl.meas[sl]), params[sl], np.ascontiguousarray(wl.cfp),
                     np.zeros((v1 - v0, 1)), samples[sl], None, None, bic[sl], aic[sl])
    for k in range(5):
        np.testing.assert_array_equal(_nifti_voxels(os.path.join(out, f"Param_{k}_samples{ext}"), mask)[:, 0],
                                      samples[:, k, 0])
    np.testing.assert_array_equal(_nifti_voxels(os.path.join(out, "BIC" + ext), mask)[:, 0], bic)
    np.testing.assert_array_equal(_nifti_voxels(os.path.join(out, "AIC" + ext), mask)[:, 0], aic)


def test_watson_gs_lm_mcmc_rician_through_the_tools(built, cuda, tmp_path):
    wl = watson(400, seed=6)
    wl.meas = np.array(wl.meas)
    wl.meas[::17, 3] = 0.0                         # non-positive entries for the Rician cleaning
    wl.meas[::23, 10] = -5.0
    mask, p = _scene(tmp_path, wl, (9, 8, 7), 2)
    make_nifti(str(tmp_path / "S0.nii"), volumes.mask_scatter(wl.fixp[:, 0], mask)[0], datatype=64)
    (tmp_path / "fixp.txt").write_text(f"{tmp_path / 'S0.nii'}\n")
    lines = ["", "", ""]
    for k in (3, 4):
        f = tmp_path / f"init{k}.nii"
        make_nifti(str(f), volumes.mask_scatter(wl.init[:, k], mask)[0], datatype=64)
        lines.append(str(f))
    (tmp_path / "init.txt").write_text("\n".join(lines) + "\n")
    gridf = tmp_path / "grid"
    gridf.write_text("search[0]=(0.0,0.3,0.6)\nsearch[1]=(0.2,0.5,0.8)\nsearch[2]=(1,4,16)\n")
    out = str(tmp_path / "out")
    common = ["--model", "NODDI_Watson", "--partsdir", str(tmp_path / "parts"), "--nParts", "2",
              "--CFP", p["cfp"], "--FixP", str(tmp_path / "fixp.txt"), "--init_params",
              str(tmp_path / "init.txt"), "--gridSearch", str(gridf), "--runMCMC", "--bi", "100",
              "--nj", "100", "--se", "10", "--rician", "--getPredictedSignal", "--BIC_AIC"]
    rc = cudimot.main(["run", "--data", p["data"], "--maskfile", p["mask"], "--outputdir", out] + common)
    assert rc == 0
    # the same fit called directly on each part's voxels, with the part id
    # (MCMC draws are keyed by seed, part id and the voxel's index in its
    # part, as CUDIMOT seeds each part with seed + idPart, MCMC.cu:765);
    # cdm_fit_host cleans the signals (rician) as the tools' fit does
    n = wl.nvox
    lib, info = cudimot.model_info("NODDI_Watson")
    params = np.zeros((n, 5))
    params[:, 3:5] = wl.init[:, 3:5]
    samples = np.zeros((n, 5, 10))
    tau = np.zeros((n, 10))
    pred = np.zeros((n, wl.nmeas))
    bic, aic = np.zeros(n), np.zeros(n)
    for i, (v0, v1) in enumerate(parts(n, 2)):
        o = cudimot.parser().parse_args(["fit", "--idPart", str(i)] + common)
        cfg, p_init = cudimot.make_cfg(o, info, lib)
        if p_init is not None:
            params[v0:v1, :3] = np.asarray(p_init)[:3]
        fit = capi.Cudimot("NODDI_Watson", cfg)
        sl = slice(v0, v1)
        fit.fit_host(np.ascontiguousarray(wl.meas[sl]), params[sl], np.ascontiguousarray(wl.cfp),
                     np.ascontiguousarray(wl.fixp[sl]), samples[sl], tau[sl], pred[sl], bic[sl], aic[sl])
        fit.close()
    ext = ".nii.gz" if volumes.gzip_supported() else ".nii"
    for k in range(5):
        np.testing.assert_array_equal(_nifti_voxels(os.path.join(out, f"Param_{k}_samples{ext}"), mask),
                                      samples[:, k])
    for name, ref in (("Tau_samples", tau), ("PredictedSignal", pred), ("BIC", bic[:, None]),
                      ("AIC", aic[:, None])):
        np.testing.assert_array_equal(_nifti_voxels(os.path.join(out, name + ext), mask), ref)
    # the cleaned entries were fitted as the smallest positive value
    assert np.all(np.isfinite(tau)) and np.all(tau > 0)
