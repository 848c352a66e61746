"""GB300-native voxelwise diffusion-MRI model fitting with CUDIMOT's plugin
surface: grid search, Levenberg-Marquardt, MCMC, predicted signal and
BIC/AIC as hand-written sm_103a kernels behind a C ABI
(include/cudimot_gb300.h), one library per model plugin."""
from .capi import (Cfg, Cudimot, CdmError, make_cfg, model_cfg, load_library,  # noqa: F401
                   parse_priors, lib_path)
