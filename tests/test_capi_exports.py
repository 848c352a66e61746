"""Every model library loads without a GPU and exports every function the
public header declares; model facts agree with the oracle; bad arguments
are rejected with a status (never exit)."""
import ctypes as C
import os
import re

import pytest

from cudimot_gb300 import capi

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "cudimot_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cdm_[a-z_0-9]+)\s*\(", text)))


MODELS = ["Ball_1_Stick", "NODDI_Watson", "DiffusionTensor", "Ball_2_Sticks", "NODDI_Bingham"]


@pytest.mark.parametrize("model", MODELS)
def test_exports(built, model):
    lib = C.CDLL(capi.lib_path(model))
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(capi.EXPORTED) <= set(names)


@pytest.mark.parametrize("model", MODELS)
def test_model_info_matches_oracle(built, model):
    from tests.helpers import oracle
    lib = capi.load_library(model)
    info = capi.ModelInfo()
    assert lib.cdm_get_model_info(C.byref(info)) == 0
    o = oracle(model).info
    for f in ("nparams", "ncfp", "nfixp", "cfp_tsize", "fixp_tsize", "derived_cfp", "derived_p"):
        assert getattr(info, f) == getattr(o, f), f
    assert info.name.decode() == model


def test_create_rejects_bad_cfg(built):
    lib = capi.load_library("NODDI_Watson")
    ctx = C.c_void_p()
    bad = capi.model_cfg("NODDI_Watson")
    bad.nparams = 4
    assert lib.cdm_create(C.byref(bad.struct), C.byref(ctx)) == 1
    bad = capi.model_cfg("NODDI_Watson", run_mcmc=1, njumps=10, sampleevery=25)
    assert lib.cdm_create(C.byref(bad.struct), C.byref(ctx)) == 1
    assert b"--nj" in lib.cdm_last_error()
    bad = capi.model_cfg("NODDI_Watson", lanes_mcmc=3)
    assert lib.cdm_create(C.byref(bad.struct), C.byref(ctx)) == 1


def test_status_strings(built):
    lib = capi.load_library("Ball_1_Stick")
    assert [lib.cdm_status_string(i).decode() for i in range(6)] == \
        ["OK", "BAD_ARG", "CUDA_ERROR", "TIMEOUT", "NOT_SUPPORTED", "IO_ERROR"]


def test_hetero_exports(built):
    """cdm_hetero.h: cdm_mcmc_prepare in every model library, the rest in
    the multi-model library (which loads without a GPU)."""
    from cudimot_gb300 import build, hetero
    text = open(os.path.join(os.path.dirname(HEADER), "cdm_hetero.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = sorted(set(re.findall(r"\b(cdm_[a-z_0-9]+)\s*\(", text)))
    assert "cdm_mcmc_prepare" in names
    for model in MODELS:
        assert hasattr(C.CDLL(capi.lib_path(model)), "cdm_mcmc_prepare"), model
    lib = hetero.load()
    for n in names:
        if n != "cdm_mcmc_prepare":
            assert hasattr(lib, n), n
    assert set(hetero.EXPORTED) == set(names) - {"cdm_mcmc_prepare"}
    # the linked set, without a device
    s = lib.cdm_hetero_models(None, 0)
    buf = C.create_string_buffer(s + 1)
    lib.cdm_hetero_models(buf, s + 1)
    models = buf.value.decode().split(",")
    assert [m.split("/")[0] for m in models] == list(build.HETERO_MODELS)
    assert all(m.endswith("/f32/1:2:4") for m in models)
    assert hetero.TileWork.args.offset == 104 and C.sizeof(hetero.TileWork) == 1128
