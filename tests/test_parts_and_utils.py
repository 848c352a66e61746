"""CUDIMOT's binary part files, written and read by libcdm_utils: the byte
layout (int32 nvox, int32 nrows, int64 nbytes, then nrows x nvox doubles,
one row per measurement/sample/value, Parameters.cu:405-420), round trips,
CUDIMOT's split sizes (nvox/nparts per part, the last takes the remainder,
split_parts.cc:80-94), merging, and rejected inputs. No GPU needed."""
import ctypes as C
import os
import re
import struct

import numpy as np
import pytest

from cudimot_gb300 import capi, utils

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include")


@pytest.mark.parametrize("header", ["cdm_utils.h", "cdm_volumes.h"])
def test_exports(built, header):
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(INCLUDE, header)).read(), flags=re.S)
    names = set(re.findall(r"\b(cdm_[a-z_0-9]+)\s*\(", text))
    assert len(names) >= 8
    lib = C.CDLL(os.path.join(capi.LIBDIR, "libcdm_utils.so"))
    for n in names:
        assert hasattr(lib, n), n


def test_part_file_bytes(built, tmp_path):
    data = np.arange(12, dtype=np.float64).reshape(4, 3)  # 4 voxels x 3 rows
    p = str(tmp_path / "x")
    utils.part_write(p, data)
    raw = open(p, "rb").read()
    nvox, nrows, nbytes = struct.unpack("<iiq", raw[:16])
    assert (nvox, nrows, nbytes) == (4, 3, 96)
    body = np.frombuffer(raw[16:], dtype="<f8").reshape(3, 4)   # [row][voxel]
    assert np.array_equal(body, data.T)
    assert np.array_equal(utils.part_read(p), data)


def test_read_a_hand_made_part_file(built, tmp_path):
    rows = np.array([[1.5, 2.5, 3.5]])      # one value (e.g. ParamInit_k) for 3 voxels
    p = tmp_path / "ParamInit_0"
    p.write_bytes(struct.pack("<iiq", 3, 1, 24) + rows.astype("<f8").tobytes())
    assert np.array_equal(utils.part_read(str(p))[:, 0], rows[0])


def test_split_and_merge(built, tmp_path):
    rng = np.random.default_rng(0)
    data = rng.standard_normal((103, 5))
    d = str(tmp_path / "parts")
    utils.split_parts(d, 4, "data", data)
    sizes = [utils.part_read(utils.part_path(d, i, "data")).shape[0] for i in range(4)]
    assert sizes == [25, 25, 25, 28]
    assert np.array_equal(utils.merge_parts(d, 4, "data"), data)


def test_rejects_bad_files(built, tmp_path):
    p = tmp_path / "bad"
    p.write_bytes(struct.pack("<iiq", 3, 2, 40) + b"\0" * 48)   # nbytes disagrees with 3 x 2
    with pytest.raises(capi.CdmError):
        utils.part_read(str(p))
    p.write_bytes(struct.pack("<iiq", 3, 2, 48) + b"\0" * 10)   # short payload
    with pytest.raises(capi.CdmError):
        utils.part_read(str(p))
    with pytest.raises(capi.CdmError):
        utils.part_read(str(tmp_path / "missing"))
    with pytest.raises(capi.CdmError):
        utils.split_parts(str(tmp_path / "q"), 5, "data", np.zeros((3, 2)))
