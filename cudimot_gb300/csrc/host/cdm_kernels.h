// cdm_kernels.h - the kernels of a model library by family, and their names
// in a separately compiled device module.
//
// A model library either carries its kernels (normal build: the host code
// takes their addresses) or loads them from a device module compiled
// separately from the plugin (split build: cdm_module.cu, looked up by
// name). Kernels of the lane-templated families exist for 1, 2, 4, 8, 16
// and 32 lanes per voxel; their module names end in _<lanes>.
#pragma once

enum cdm_kfam : int {
  // lane-templated
  CDM_K_GRIDSEARCH = 0,
  CDM_K_LEVMAR,
  CDM_K_MCMC,
  CDM_K_MCMC_RICIAN,
  CDM_K_PACK_SIGNALS,
  CDM_K_PREP_SHELLS,
  CDM_K_PACK_SHELL_SIGNALS,
  CDM_K_NLANE_FAMILIES,
  // one instance each
  CDM_K_GS_RECHECK = CDM_K_NLANE_FAMILIES,
  CDM_K_PREDICTED,
  CDM_K_BIC_AIC,
  CDM_K_SELECT_WORSE,
  CDM_K_ROWS,
  CDM_K_PREP_PROTOCOL,
  CDM_K_PARAMS_TO_SAMPLES,
  CDM_K_SYNTH,
  CDM_K_MLP_ENCODE,
  CDM_K_MLP_DECODE,
  CDM_K_CLEAN_SIGNALS,
  CDM_K_WAIT_SELFTEST,
  CDM_K_COUNT
};

// Module kernel name: "cdm_k_" + this + ("_" + lanes for the lane-templated).
inline const char* cdm_kfam_name(int fam) {
  static const char* const names[CDM_K_COUNT] = {
      "gridsearch", "levmar",   "mcmc",        "mcmc_rician", "pack_signals",
      "prep_shells", "pack_shell_signals",
      "gs_recheck", "predicted", "bic_aic",    "select_worse",
      "rows",       "prep_protocol", "params_to_samples", "synth", "mlp_encode",
      "mlp_decode", "clean_signals", "wait_selftest"};
  return fam >= 0 && fam < CDM_K_COUNT ? names[fam] : "";
}

// Index of a lane count in {1, 2, 4, 8, 16, 32}, or -1.
inline int cdm_lane_index(int lanes) {
  switch (lanes) {
    case 1: return 0;
    case 2: return 1;
    case 4: return 2;
    case 8: return 3;
    case 16: return 4;
    case 32: return 5;
  }
  return -1;
}
