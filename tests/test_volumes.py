"""NIfTI-1 volumes, masks and split_parts / merge_parts on volumes
(include/cdm_volumes.h), checked against an independent reader and writer
of the NIfTI-1 format written here with `struct` (CPU only).

What the library restates: split_parts.cc:41-277 (data, --init_params and
--FixP lists into part files, with their checks) and merge_parts.cc:21-59
(parts back into a volume on the mask's grid)."""
import gzip
import os
import struct

import numpy as np
import pytest

from cudimot_gb300 import utils, volumes
from cudimot_gb300.capi import CdmError

NP_TYPES = {2: "u1", 4: "i2", 8: "i4", 16: "f4", 64: "f8", 256: "i1", 512: "u2", 768: "u4",
            1024: "i8", 1280: "u8"}


def make_nifti(path, data, datatype=16, endian="<", slope=0.0, inter=0.0, pixdim=(2.0, 2.0, 2.5, 1.0),
               srow=None, magic=b"n+1\0", sizeof_hdr=348, vox_offset=352, gz=False):
    """Independent NIfTI-1 writer: data [nt][nz][ny][nx] or [nz][ny][nx]."""
    data = np.asarray(data)
    if data.ndim == 3:
        data = data[None]
    nt, nz, ny, nx = data.shape
    h = bytearray(348)
    e = endian
    struct.pack_into(e + "i", h, 0, sizeof_hdr)
    dim = [4 if nt > 1 else 3, nx, ny, nz, nt, 1, 1, 1]
    struct.pack_into(e + "8h", h, 40, *dim)
    bits = np.dtype(NP_TYPES[datatype]).itemsize * 8
    struct.pack_into(e + "hh", h, 70, datatype, bits)
    pd = [1.0, *pixdim] + [0.0] * (7 - len(pixdim))
    struct.pack_into(e + "8f", h, 76, *pd)
    struct.pack_into(e + "f", h, 108, float(vox_offset))
    struct.pack_into(e + "ff", h, 112, slope, inter)
    struct.pack_into(e + "hh", h, 252, 1, 2)  # qform_code, sform_code
    srow = srow if srow is not None else [[-2, 0, 0, 90], [0, 2, 0, -126], [0, 0, 2.5, -72]]
    struct.pack_into(e + "12f", h, 280, *[float(v) for r in srow for v in r])
    h[344:348] = magic
    body = np.ascontiguousarray(data).astype(np.dtype(NP_TYPES[datatype]).newbyteorder(e)).tobytes()
    blob = bytes(h) + b"\0" * (vox_offset - 348) + body
    if gz:
        with gzip.open(path, "wb") as f:
            f.write(blob)
    else:
        with open(path, "wb") as f:
            f.write(blob)


def parse_nifti(path):
    """Independent NIfTI-1 reader (little-endian, as the library writes)."""
    with open(path, "rb") as f:
        blob = f.read()
    if blob[:2] == b"\x1f\x8b":
        blob = gzip.decompress(blob)
    h = blob[:348]
    out = {"sizeof_hdr": struct.unpack_from("<i", h, 0)[0],
           "dim": struct.unpack_from("<8h", h, 40),
           "datatype": struct.unpack_from("<h", h, 70)[0],
           "bitpix": struct.unpack_from("<h", h, 72)[0],
           "pixdim": struct.unpack_from("<8f", h, 76),
           "vox_offset": struct.unpack_from("<f", h, 108)[0],
           "scl": struct.unpack_from("<ff", h, 112),
           "cal_max": struct.unpack_from("<f", h, 124)[0],
           "cal_min": struct.unpack_from("<f", h, 128)[0],
           "codes": struct.unpack_from("<hh", h, 252),
           "srow": struct.unpack_from("<12f", h, 280),
           "magic": h[344:348]}
    d = out["dim"]
    nt = int(np.prod(d[4:d[0] + 1])) if d[0] >= 4 else 1
    dt = np.dtype(NP_TYPES[out["datatype"]]).newbyteorder("<")
    off = int(out["vox_offset"])
    out["data"] = np.frombuffer(blob[off:], dtype=dt, count=nt * d[1] * d[2] * d[3]).reshape(
        nt, d[3], d[2], d[1]).astype(np.float64)
    return out


def test_read_datatypes_and_byte_orders(built, tmp_path):
    rng = np.random.default_rng(1)
    for dt, npt in NP_TYPES.items():
        info = np.iinfo(npt) if np.dtype(npt).kind in "iu" else None
        lo, hi = (max(info.min, -1000), min(info.max, 1000)) if info else (-1e3, 1e3)
        x = rng.uniform(lo, hi, size=(3, 4, 5, 6)).astype(npt)
        for e in "<>":
            p = str(tmp_path / f"t{dt}{'le' if e == '<' else 'be'}.nii")
            make_nifti(p, x, datatype=dt, endian=e)
            h, v = volumes.read(p)
            assert h.datatype == dt and tuple(h.dim[:5]) == (4, 6, 5, 4, 3)
            np.testing.assert_array_equal(v, x.astype(np.float64))
            assert h.pixdim[1] == 2.0 and h.pixdim[3] == 2.5


def test_scaling_applied(built, tmp_path):
    x = np.arange(60, dtype=np.int16).reshape(1, 3, 4, 5)
    p = str(tmp_path / "s.nii")
    make_nifti(p, x, datatype=4, slope=0.5, inter=-3.0)
    _, v = volumes.read(p)
    np.testing.assert_allclose(v, x * 0.5 - 3.0)
    make_nifti(p, x, datatype=4, slope=0.0, inter=7.0)  # slope 0: no scaling
    _, v = volumes.read(p)
    np.testing.assert_array_equal(v, x)


def test_extension_bytes_skipped(built, tmp_path):
    x = np.random.default_rng(2).normal(size=(2, 3, 4, 5)).astype(np.float32)
    p = str(tmp_path / "ext.nii")
    make_nifti(p, x, vox_offset=352 + 64)
    _, v = volumes.read(p)
    np.testing.assert_array_equal(v, x.astype(np.float64))


def test_gzip_read_and_write(built, tmp_path):
    if not volumes.gzip_supported():
        pytest.skip("library built without zlib")
    x = np.random.default_rng(3).normal(size=(4, 3, 5, 6))
    p = str(tmp_path / "g.nii.gz")
    make_nifti(p, x, datatype=64, gz=True)
    h, v = volumes.read(p)
    np.testing.assert_array_equal(v, x)
    q = str(tmp_path / "out.nii.gz")
    volumes.write(q, h, v)
    with open(q, "rb") as f:
        assert f.read(2) == b"\x1f\x8b"
    np.testing.assert_array_equal(parse_nifti(q)["data"], x)


def test_write_header_and_geometry(built, tmp_path):
    x = np.random.default_rng(4).normal(size=(3, 4, 5))
    p = str(tmp_path / "mask.nii")
    srow = [[-1.5, 0.1, 0, 80], [0, 1.5, 0.2, -100], [0.3, 0, 2.0, -60]]
    make_nifti(p, x, datatype=16, srow=srow, pixdim=(1.5, 1.5, 2.0))
    like = volumes.read_header(p)
    y = np.random.default_rng(5).normal(size=(7, 3, 4, 5))
    q = str(tmp_path / "o.nii")
    volumes.write(q, like, y)
    r = parse_nifti(q)
    assert r["sizeof_hdr"] == 348 and r["magic"] == b"n+1\0" and r["vox_offset"] == 352
    assert r["dim"][:5] == (4, 5, 4, 3, 7) and r["datatype"] == 64 and r["bitpix"] == 64
    assert r["scl"] == (1.0, 0.0)
    assert r["codes"] == (1, 2)
    np.testing.assert_allclose(r["srow"], np.float32(np.ravel(srow)))
    np.testing.assert_allclose(r["pixdim"][1:4], (1.5, 1.5, 2.0))
    assert r["cal_min"] == np.float32(y.min()) and r["cal_max"] == np.float32(y.max())
    np.testing.assert_array_equal(r["data"], y)
    volumes.write(q, like, y[0], datatype=volumes.FLOAT32)
    r = parse_nifti(q)
    assert r["dim"][0] == 3 and r["datatype"] == 16
    np.testing.assert_array_equal(r["data"][0], y[0].astype(np.float32))


def test_rejected_images(built, tmp_path):
    x = np.zeros((2, 2, 2), np.float32)
    cases = {
        "nifti2.nii": dict(sizeof_hdr=540),
        "pair.nii": dict(magic=b"ni1\0"),
        "analyze.nii": dict(magic=b"\0\0\0\0"),
        "garbage.nii": dict(sizeof_hdr=12345),
    }
    for name, kw in cases.items():
        p = str(tmp_path / name)
        make_nifti(p, x, **kw)
        with pytest.raises(CdmError):
            volumes.read(p)
    p = str(tmp_path / "short.nii")
    make_nifti(p, np.zeros((4, 4, 4), np.float32))
    with open(p, "r+b") as f:
        f.truncate(352 + 100)
    with pytest.raises(CdmError):
        volumes.read(p)
    with pytest.raises(CdmError):
        volumes.read(str(tmp_path / "missing.nii"))


def test_mask_gather_scatter_order(built):
    rng = np.random.default_rng(6)
    mask = (rng.uniform(size=(4, 5, 6)) > 0.4).astype(np.float64)
    mask[0, 0, 0] = -1.0  # not positive: outside
    vol = rng.normal(size=(3, 4, 5, 6))
    g = volumes.mask_gather(vol, mask)
    sel = mask.ravel() > 0
    np.testing.assert_array_equal(g, vol.reshape(3, -1)[:, sel].T)
    s = volumes.mask_scatter(g, mask)
    np.testing.assert_array_equal(s.reshape(3, -1)[:, sel], vol.reshape(3, -1)[:, sel])
    assert np.all(s.reshape(3, -1)[:, ~sel] == 0)


@pytest.fixture()
def scene(built, tmp_path):
    """A 4-D data volume, its mask, an init volume and a 2-volume FixP."""
    rng = np.random.default_rng(7)
    shp = (3, 4, 5)
    mask = (rng.uniform(size=shp) > 0.3).astype(np.uint8)
    data = rng.normal(size=(6,) + shp)
    init = rng.normal(size=shp)
    fixp = rng.normal(size=(2,) + shp)
    d = {k: str(tmp_path / f"{k}.nii") for k in ("mask", "data", "init", "fixp", "init4d")}
    make_nifti(d["mask"], mask, datatype=2)
    make_nifti(d["data"], data, datatype=64)
    make_nifti(d["init"], init, datatype=64)
    make_nifti(d["fixp"], fixp, datatype=64)
    make_nifti(d["init4d"], fixp, datatype=64)
    return dict(paths=d, mask=mask.astype(np.float64), data=data, init=init, fixp=fixp,
                parts=str(tmp_path / "parts"), tmp=tmp_path)


def test_split_volumes_as_split_parts(scene):
    sc, p = scene, scene["paths"]
    lst = sc["tmp"] / "init.txt"
    lst.write_text(f"{p['init']}\n\n{p['init']}\n")
    fl = sc["tmp"] / "fixp.txt"
    fl.write_text(f"{p['fixp']}\n")
    n = volumes.split_volumes(sc["parts"], 3, p["data"], p["mask"], 3, init_list=str(lst),
                              init_values=[0.0, 4.5, 0.0], fixp_list=str(fl), fixp_sizes=[2])
    m = sc["mask"].ravel() > 0
    assert n == int(m.sum())
    vox = sc["data"].reshape(6, -1)[:, m].T
    np.testing.assert_array_equal(utils.merge_parts(sc["parts"], 3, "data"), vox)
    size = n // 3
    assert utils.part_read(utils.part_path(sc["parts"], 0, "data")).shape == (size, 6)
    assert utils.part_read(utils.part_path(sc["parts"], 2, "data")).shape == (n - 2 * size, 6)
    iv = sc["init"].ravel()[m][:, None]
    np.testing.assert_array_equal(utils.merge_parts(sc["parts"], 3, "ParamInit_0"), iv)
    np.testing.assert_array_equal(utils.merge_parts(sc["parts"], 3, "ParamInit_1"), np.full((n, 1), 4.5))
    np.testing.assert_array_equal(utils.merge_parts(sc["parts"], 3, "ParamInit_2"), iv)
    np.testing.assert_array_equal(utils.merge_parts(sc["parts"], 3, "FixParam_0"),
                                  sc["fixp"].reshape(2, -1)[:, m].T)


def test_split_volumes_checks(scene):
    sc, p, t = scene, scene["paths"], scene["tmp"]

    def split(**kw):
        args = dict(nparams=2)
        args.update(kw)
        return volumes.split_volumes(sc["parts"], 2, p["data"], p["mask"], **args)

    (t / "three.txt").write_text(f"{p['init']}\n\n{p['init']}\n")
    (t / "one.txt").write_text(f"{p['init']}\n")
    (t / "4d.txt").write_text(f"{p['init4d']}\n\n")
    (t / "fp_empty.txt").write_text("\n")
    (t / "fp_bad.txt").write_text(f"{p['init']}\n")
    for kw in (dict(init_list=str(t / "three.txt")),        # too many lines
               dict(init_list=str(t / "one.txt")),          # too few lines
               dict(init_list=str(t / "4d.txt")),           # not a 3-D volume
               dict(init_list=str(t / "nofile.txt")),       # missing list
               dict(fixp_list=str(t / "fp_bad.txt")),       # FixP given to a model without
               dict(fixp_sizes=[2]),                        # FixP list missing
               dict(fixp_list=str(t / "fp_empty.txt"), fixp_sizes=[2]),  # empty line
               dict(fixp_list=str(t / "fp_bad.txt"), fixp_sizes=[2])):   # wrong volume count
        with pytest.raises(CdmError):
            split(**kw)
    with pytest.raises(CdmError):  # more parts than voxels
        volumes.split_volumes(sc["parts"], 10_000, p["data"], p["mask"], 2)
    other = str(t / "other_mask.nii")
    make_nifti(other, np.ones((3, 4, 6), np.uint8), datatype=2)
    with pytest.raises(CdmError):  # grids differ
        volumes.split_volumes(sc["parts"], 2, p["data"], other, 2)


def test_merge_volumes_as_merge_parts(scene):
    sc, p = scene, scene["paths"]
    m = sc["mask"].ravel() > 0
    n = int(m.sum())
    samples = np.random.default_rng(8).normal(size=(n, 5))
    utils.split_parts(sc["parts"], 4, "Param_0_samples", samples)
    out = str(sc["tmp"] / "Param_0_samples.nii")
    volumes.merge_volumes(sc["parts"], 4, "Param_0_samples", p["mask"], out, nrows=5)
    r = parse_nifti(out)
    assert r["dim"][:5] == (4, 5, 4, 3, 5) and r["datatype"] == 64
    exp = np.zeros((5, m.size))
    exp[:, m] = samples.T
    np.testing.assert_array_equal(r["data"].reshape(5, -1), exp)
    assert r["cal_min"] == np.float32(exp.min()) and r["cal_max"] == np.float32(exp.max())
    volumes.merge_volumes(sc["parts"], 4, "Param_0_samples", p["mask"], out)  # rows from part 0
    np.testing.assert_array_equal(parse_nifti(out)["data"].reshape(5, -1), exp)
    with pytest.raises(CdmError):  # a part with other rows
        volumes.merge_volumes(sc["parts"], 4, "Param_0_samples", p["mask"], out, nrows=1)
    with pytest.raises(CdmError):  # parts cover fewer voxels than the mask
        volumes.merge_volumes(sc["parts"], 3, "Param_0_samples", p["mask"], out)
    with pytest.raises(CdmError):  # a missing part
        volumes.merge_volumes(sc["parts"], 5, "Param_0_samples", p["mask"], out)
    assert os.path.exists(out)
