"""CUDIMOT's command-line options mapped onto cdm_model_cfg (no GPU).

The `fit` tool builds the configuration the way cudimot.cc does
(cudimot.cc:25-125 with the defaults of cudimotoptions.h:78-168): the
priors file, --gridSearch and --fixed go through the library's parsers;
the flags set the stage switches and MCMC settings.
"""
import numpy as np
import pytest

from cudimot_gb300 import cudimot
from cudimot_gb300.cudimot import CudimotError


def _fit_opts(*extra):
    return cudimot.parser().parse_args(
        ["fit", "--model", "NODDI_Watson", "--partsdir", "parts", "--nParts", "4",
         "--idPart", "2", *extra])


def test_defaults_match_the_library(built):
    o = _fit_opts()
    lib, info = cudimot.model_info("NODDI_Watson")
    cfg, _ = cudimot.make_cfg(o, info, lib)
    s = cfg.struct
    assert (s.nburn, s.njumps, s.sampleevery, s.iter_levmar, s.seed) == (1000, 1250, 25, 200, 8219)
    assert (s.run_gridsearch, s.run_levmar, s.run_mcmc, s.marquardt, s.update_proposal) == \
        (0, 1, 0, 1, 1)
    assert (s.rician, s.get_predicted, s.bic_aic, s.id_part) == (0, 0, 0, 2)
    assert list(s.fixed)[:5] == [0] * 5
    assert cudimot.nsamples(o) == 1


def test_every_option_reaches_the_cfg(built, tmp_path):
    grid = tmp_path / "grid"
    grid.write_text("search[0]=(0.0,0.5)\nsearch[2]=(1,2,4)\n")
    o = _fit_opts("--gridSearch", str(grid), "--fixed", "1,3", "--runMCMC", "--bi", "300",
                  "--nj", "400", "--se", "20", "--no_updateproposal", "--seed", "77",
                  "--no_Marquardt", "--iterLevMar", "50", "--rician", "--getPredictedSignal",
                  "--BIC_AIC")
    lib, info = cudimot.model_info("NODDI_Watson")
    cfg, _ = cudimot.make_cfg(o, info, lib)
    s = cfg.struct
    assert (s.run_gridsearch, s.n_grid_params, s.grid_combs) == (1, 2, 6)
    assert (s.grid_params[0], s.grid_params[1]) == (0, 2)
    g = np.ctypeslib.as_array(s.grid, shape=(6, 2))
    assert np.array_equal(g, [[0, 1], [0, 2], [0, 4], [0.5, 1], [0.5, 2], [0.5, 4]])
    assert list(s.fixed)[:5] == [0, 1, 0, 1, 0]
    assert (s.run_mcmc, s.nburn, s.njumps, s.sampleevery, s.update_proposal, s.seed) == \
        (1, 300, 400, 20, 0, 77)
    assert (s.run_levmar, s.marquardt, s.iter_levmar) == (1, 0, 50)
    assert (s.rician, s.get_predicted, s.bic_aic) == (1, 1, 1)
    assert cudimot.nsamples(o) == 20


def test_no_method_is_rejected():
    # cudimot.cc:37-41: at least one of grid search, LM or MCMC
    with pytest.raises(CudimotError, match="at least one method"):
        cudimot._need_method(_fit_opts("--no_LevMar"))
    cudimot._need_method(_fit_opts("--no_LevMar", "--runMCMC"))


def test_bad_fixed_list_is_rejected(built):
    lib, info = cudimot.model_info("NODDI_Watson")
    with pytest.raises(Exception, match="Wrong number of parameter 7"):
        cudimot.make_cfg(_fit_opts("--fixed", "7"), info, lib)
