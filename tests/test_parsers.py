"""modelpriors / grid / --fixed / CFP-list readers of the C ABI, with
CUDIMOT's parsing rules (Model.cu:16-393, Parameters.cu:93-149). The model
libraries load without a GPU; these calls are host-only."""
import ctypes as C
import os

import numpy as np
import pytest

from cudimot_gb300 import capi


@pytest.fixture(scope="module")
def lib(built):
    return capi.load_library("NODDI_Watson")


def parse_priors(lib, text, tmp_path):
    p = tmp_path / "priors"
    p.write_text(text)
    cfg = capi.Cfg(5)
    lib.cdm_default_cfg(C.byref(cfg.struct))
    init = (C.c_double * 32)()
    given = C.c_int(0)
    st = lib.cdm_parse_priors(str(p).encode(), C.byref(cfg.struct), C.cast(init, C.c_void_p),
                              C.byref(given))
    return st, cfg.struct, list(init)[:5], given.value


def test_shipped_modelpriors(lib):
    path = os.path.join(capi.HERE, "mymodels", "NODDI_Watson", "modelpriors")
    cfg, init = capi.parse_priors("NODDI_Watson", path, 5)
    assert init == [0.4, 0.8, 5.0, 1.5, 1.5]
    assert list(cfg.bound_types)[:5] == [capi.BMINMAX] * 5
    assert cfg.bounds_max[2] == 64.0
    assert cfg.prior_types[3] == capi.SINPRIOR


def test_priors_rules(lib, tmp_path):
    text = "\n".join([
        "P_init[0.1,0.2,3,1,2]",
        "bounds[0]=(1e-9,)",       # min only
        "bounds[1]=(,5)",          # max only
        "bounds[2]=(0,64) // a comment anywhere skips the whole line",
        "prior[0]=Gaussian(2,0.5)",
        "priors[3]=sin()",         # not recognised: 'priors[' has no 'prior['
        "prior[1]=Gamma(3,4)",
        "prior[4]=ARD(1.5)",
    ])
    st, c, init, given = parse_priors(lib, text, tmp_path)
    assert st == 0 and given == 1 and init == [0.1, 0.2, 3.0, 1.0, 2.0]
    assert c.bound_types[0] == capi.BMIN and c.bounds_min[0] == 1e-9
    assert c.bound_types[1] == capi.BMAX and c.bounds_max[1] == 5.0
    assert c.bound_types[2] == capi.NOBOUNDS
    assert (c.prior_types[0], c.priors_a[0], c.priors_b[0]) == (capi.GAUSSPRIOR, 2.0, 0.5)
    assert c.prior_types[3] == capi.NOPRIOR
    assert (c.prior_types[1], c.priors_a[1], c.priors_b[1]) == (capi.GAMMAPRIOR, 3.0, 4.0)
    assert (c.prior_types[4], c.priors_a[4]) == (capi.ARDPRIOR, 1.5)


@pytest.mark.parametrize("text, code", [
    ("P_init[1,2,3]", 1),                 # wrong count
    ("bounds[7]=(0,1)", 1),               # parameter id out of range
    ("bounds[0]=(,)", 1),                 # neither min nor max
    ("prior[0]=Cauchy(1,2)", 1),          # unknown prior
    ("prior[0]=Gaussian(,2)", 1),         # missing first argument
])
def test_priors_errors(lib, tmp_path, text, code):
    st, *_ = parse_priors(lib, text, tmp_path)
    assert st == code
    assert lib.cdm_last_error()


def test_priors_missing_file(lib):
    cfg = capi.Cfg(5)
    st = lib.cdm_parse_priors(b"/nonexistent/priors", C.byref(cfg.struct), None, None)
    assert st == 5  # CDM_IO_ERROR


def test_grid_order_lowest_id_outermost(lib, tmp_path):
    p = tmp_path / "grid"
    p.write_text("// comment\nsearch[2]=(1,2,3)\nsearch[0]=(0.1,0.2)\n")
    ngp, combs = C.c_int(), C.c_int()
    ids = (C.c_int * 32)()
    assert lib.cdm_parse_grid(str(p).encode(), C.byref(ngp), C.cast(ids, C.c_void_p),
                              C.byref(combs), None, 0) == 0
    assert (ngp.value, combs.value, ids[0], ids[1]) == (2, 6, 0, 2)
    buf = (C.c_double * 12)()
    assert lib.cdm_parse_grid(str(p).encode(), C.byref(ngp), C.cast(ids, C.c_void_p),
                              C.byref(combs), C.cast(buf, C.c_void_p), 12) == 0
    got = np.array(list(buf)).reshape(6, 2)
    want = np.array([[0.1, 1], [0.1, 2], [0.1, 3], [0.2, 1], [0.2, 2], [0.2, 3]])
    assert np.array_equal(got, want)
    # the Python grid builder enumerates identically
    cfg = capi.make_cfg(5, grid={2: [1, 2, 3], 0: [0.1, 0.2]})
    assert np.array_equal(cfg.grid_array, want)


def test_fixed_list(lib):
    fixed = (C.c_int * 32)()
    assert lib.cdm_parse_fixed(b"1,3", C.cast(fixed, C.c_void_p)) == 0
    assert list(fixed)[:5] == [0, 1, 0, 1, 0]
    assert lib.cdm_parse_fixed(b"7", C.cast(fixed, C.c_void_p)) == 1


def test_cfp_list(lib, tmp_path):
    bvecs = np.array([[1, 0, 0.6], [0, 1, 0.8], [0, 0, 0.0]])
    bvals = np.array([[0, 1000, 2000]])
    np.savetxt(tmp_path / "bvecs", bvecs)
    np.savetxt(tmp_path / "bvals", bvals)
    (tmp_path / "list").write_text(f"{tmp_path / 'bvecs'}\n\n{tmp_path / 'bvals'}\n")
    out = np.zeros((3, 4))
    assert lib.cdm_read_cfp_list(str(tmp_path / "list").encode(), 3, out.ctypes.data_as(C.c_void_p)) == 0
    assert np.array_equal(out, np.concatenate([bvecs.T, bvals.T], axis=1))
    assert lib.cdm_read_cfp_list(str(tmp_path / "list").encode(), 4, out.ctypes.data_as(C.c_void_p)) == 1
