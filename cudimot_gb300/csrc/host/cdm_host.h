// cdm_host.h - host-side helpers shared by every model library: error
// state, option defaults, and the readers of CUDIMOT's text inputs.
#pragma once
#include <string>
#include <vector>
#include "cudimot_gb300.h"

// Record `msg` as this thread's last error and return `s`.
cdm_status cdm_fail(cdm_status s, const std::string& msg);

void cdm_fill_default_cfg(cdm_model_cfg* cfg, int nparams);
cdm_status cdm_validate_cfg(const cdm_model_cfg* cfg, int nparams);

cdm_status cdm_parse_priors_impl(const char* path, int nparams, cdm_model_cfg* cfg,
                                 double* p_init, int* p_init_given);
cdm_status cdm_parse_grid_impl(const char* path, int nparams, int* n_grid_params,
                               int* grid_params, int* grid_combs, double* grid,
                               int64_t grid_capacity);
cdm_status cdm_parse_fixed_impl(const char* list, int nparams, int* fixed);
cdm_status cdm_read_cfp_list_impl(const char* path, int nmeas, const std::vector<int>& sizes,
                                  double* cfp);
