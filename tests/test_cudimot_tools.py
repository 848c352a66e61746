"""CUDIMOT's command-line tools over the library (cudimot_gb300.cudimot):
split_parts and merge_parts on NIfTI volumes with CUDIMOT's options and
checks, and the oracle of dMRI_Data's Rician signal cleaning. CPU only; the
fit step on the GPU is in test_gpu_cudimot_tools.py."""
import os

import numpy as np
import pytest

from cudimot_gb300 import cudimot, utils, volumes
from oracle.data_oracle import remove_nonpositive, remove_nonpositive_voxel
from tests.test_volumes import make_nifti, parse_nifti


def write_scene(tmp, nvox_shape=(4, 5, 3), nmeas=12, seed=3, fixp=True):
    rng = np.random.default_rng(seed)
    mask = (rng.uniform(size=nvox_shape) > 0.35).astype(np.uint8)
    data = rng.uniform(100, 1000, size=(nmeas,) + nvox_shape)
    paths = {"mask": str(tmp / "mask.nii"), "data": str(tmp / "data.nii")}
    make_nifti(paths["mask"], mask, datatype=2)
    make_nifti(paths["data"], data, datatype=64)
    if fixp:
        s0 = rng.uniform(500, 1500, size=nvox_shape)
        paths["S0"] = str(tmp / "S0.nii")
        make_nifti(paths["S0"], s0, datatype=64)
        (tmp / "fixp.txt").write_text(paths["S0"] + "\n")
        paths["fixp_list"] = str(tmp / "fixp.txt")
    return mask.astype(np.float64), data, paths


def test_remove_nonpositive_oracle_known_answers():
    # the smallest positive value replaces every non-positive entry
    np.testing.assert_array_equal(remove_nonpositive_voxel([5.0, -1.0, 0.0, 3.0]), [5.0, 3.0, 3.0, 3.0])
    # all non-positive, or none: unchanged
    np.testing.assert_array_equal(remove_nonpositive_voxel([0.0, -2.0]), [0.0, -2.0])
    np.testing.assert_array_equal(remove_nonpositive_voxel([1.0, 2.0]), [1.0, 2.0])
    # values are float-rounded as the reference's float MinS
    r = remove_nonpositive_voxel([0.1, -1.0, 7.0])
    assert r[1] == float(np.float32(0.1)) and r[0] == 0.1
    # a positive double that is 0 as a float counts as non-positive
    r = remove_nonpositive_voxel([1e-300, 0.5, -3.0])
    assert r[0] == r[2] == 0.5
    # the single positive entry
    np.testing.assert_array_equal(remove_nonpositive_voxel([-1.0, 2.5, -4.0]), [2.5, 2.5, 2.5])
    m = np.array([[1.0, -1.0], [0.0, 0.0]])
    np.testing.assert_array_equal(remove_nonpositive(m), [[1.0, 1.0], [0.0, 0.0]])


def test_split_fixp_and_init(built, tmp_path):
    mask, data, p = write_scene(tmp_path)
    th = np.random.default_rng(1).uniform(0, 3, size=mask.shape)
    make_nifti(str(tmp_path / "th.nii"), th, datatype=64)
    lst = tmp_path / "init.txt"
    lst.write_text(f"\n\n\n{tmp_path / 'th.nii'}\n\n")
    parts = str(tmp_path / "parts")
    rc = cudimot.main(["split", "--model", "NODDI_Watson", "--data", p["data"], "--maskfile", p["mask"],
                       "--partsdir", parts, "--nParts", "2", "--FixP", p["fixp_list"],
                       "--init_params", str(lst), "--runMCMC"])
    assert rc == 0
    m = mask.ravel() > 0
    n = int(m.sum())
    np.testing.assert_array_equal(utils.merge_parts(parts, 2, "data"), data.reshape(data.shape[0], -1)[:, m].T)
    np.testing.assert_array_equal(utils.merge_parts(parts, 2, "ParamInit_3")[:, 0], th.ravel()[m])
    # empty lines take the modelpriors' P_init when it has one, else 0
    assert utils.merge_parts(parts, 2, "ParamInit_0").shape == (n, 1)
    s0 = parse_nifti(p["S0"])["data"].reshape(-1)[m]
    np.testing.assert_array_equal(utils.merge_parts(parts, 2, "FixParam_0")[:, 0], s0)


def test_split_checks(built, tmp_path, capsys):
    mask, data, p = write_scene(tmp_path)
    parts = str(tmp_path / "parts")
    base = ["split", "--model", "NODDI_Watson", "--data", p["data"], "--maskfile", p["mask"],
            "--partsdir", parts, "--nParts", "2"]
    assert cudimot.main(base + ["--FixP", p["fixp_list"], "--no_LevMar"]) == 1   # no method
    assert "at least one method" in capsys.readouterr().err
    assert cudimot.main(base) == 1                                               # FixP list missing
    assert "Fixed Parameters" in capsys.readouterr().err
    assert cudimot.main(["split", "--model", "Ball_1_Stick", "--data", p["data"], "--maskfile", p["mask"],
                         "--partsdir", parts, "--nParts", "2", "--FixP", p["fixp_list"]]) == 1
    assert "does not need any Fixed Parameter" in capsys.readouterr().err


def test_merge_outputs(built, tmp_path):
    mask, data, p = write_scene(tmp_path, fixp=False)
    m = mask.ravel() > 0
    n = int(m.sum())
    parts = str(tmp_path / "parts")
    rng = np.random.default_rng(4)
    ns, nmeas = 4, data.shape[0]
    arrays = {f"Param_{i}_samples": rng.normal(size=(n, ns)) for i in range(5)}
    arrays["PredictedSignal"] = rng.normal(size=(n, nmeas))
    arrays["BIC"] = rng.normal(size=(n, 1))
    arrays["AIC"] = rng.normal(size=(n, 1))
    arrays["Tau_samples"] = rng.normal(size=(n, ns))
    for k, a in arrays.items():
        utils.split_parts(parts, 3, k, a)
    out = str(tmp_path / "out")
    rc = cudimot.main(["merge", "--model", "Ball_1_Stick", "--maskfile", p["mask"], "--partsdir", parts,
                       "--nParts", "3", "--outputdir", out, "--runMCMC", "--nj", "100", "--se", "25",
                       "--getPredictedSignal", "--BIC_AIC", "--rician"])
    assert rc == 0
    assert not os.path.exists(parts)      # removed without --keepTmp (merge_parts.cc:143-146)
    ext = ".nii.gz" if volumes.gzip_supported() else ".nii"
    for k, a in arrays.items():
        r = parse_nifti(os.path.join(out, k + ext))
        exp = np.zeros((a.shape[1], m.size))
        exp[:, m] = a.T
        np.testing.assert_array_equal(r["data"].reshape(a.shape[1], -1), exp)
