// refharness.cpp - runs CUDIMOT's own GPU kernels, unmodified, on the
// current device. TEST INFRASTRUCTURE: pins the fitting loops of the GPU
// library against the reference implementation and times the reference.
//
// The kernels come from cubins that oracle/refkernels/build_ref_kernels.py
// compiles from CUDIMOT's GridSearch.cu, Levenberg_Marquardt.cu, MCMC.cu,
// BIC_AIC.cu and getPredictedSignal.cu for sm_103a. The CUDIMOT host classes
// need FSL, so this file does what their constructors and run() methods do
// (same __constant__ uploads, launch shapes and dynamic shared memory),
// through the CUDA driver API, for T = double (the MyType of the plugins)
// or T = float (CUDIMOT instantiates every method for both, e.g.
// GridSearch.cu:320-321; ref_set_real selects which). Line references are
// to those files.
//
// The reference kernels process whole blocks of voxels without a bounds
// check (VOXELS_BLOCK = 8 for GridSearch/MCMC/BIC/predicted signal, 2 for
// LM), relying on arrays padded to a multiple of 8 voxels
// (dMRI_Data.cu:82-88). Every entry point here therefore requires nvox to be
// a multiple of 8 and returns -1 otherwise.
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

CUmodule g_mod[5] = {};
enum { M_GS = 0, M_LM, M_MCMC, M_BIC, M_PRED };
const char* kFiles[5] = {"GridSearch", "Levenberg_Marquardt", "MCMC", "BIC_AIC", "getPredictedSignal"};
char g_err[512];
// T of the launched kernels: 'd' (double) or 'f' (float), its size in bytes
char g_t = 'd';
size_t g_ts = sizeof(double);

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
  return (int)r;
}
#define DRV(call)                          \
  do {                                     \
    CUresult r_ = (call);                  \
    if (r_ != CUDA_SUCCESS) return fail(#call, r_); \
  } while (0)

int set_const(int mod, const char* name, const void* src, size_t bytes) {
  CUdeviceptr p;
  size_t sz;
  DRV(cuModuleGetGlobal(&p, &sz, g_mod[mod], name));
  if (sz < bytes) {
    std::snprintf(g_err, sizeof(g_err), "constant %s too small", name);
    return -1;
  }
  DRV(cuMemcpyHtoD(p, src, bytes));
  return 0;
}

int get_fn(int mod, const std::string& name, CUfunction* f) {
  DRV(cuModuleGetFunction(f, g_mod[mod], name.c_str()));
  return 0;
}

int launch(CUfunction f, int blocks, int threads, size_t smem, void** args) {
  if (smem > 48 * 1024) DRV(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem));
  DRV(cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, (unsigned)smem, 0, args, nullptr));
  DRV(cuCtxSynchronize());
  return 0;
}

const char* b(int v) { return v ? "1" : "0"; }

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err; }

// Select T for the following calls: bytes 8 = double, 4 = float. Every
// array argument (meas, params, CFP, FixP, grid, samples, tau, outputs) is
// then a T array.
int ref_set_real(int bytes) {
  if (bytes != 4 && bytes != 8) return -1;
  g_t = bytes == 4 ? 'f' : 'd';
  g_ts = (size_t)bytes;
  return 0;
}

// Load the five cubins of one model from dir/<File>.cubin into the primary
// context of device 0 (the context the CUDA runtime uses too).
int ref_load(const char* dir) {
  DRV(cuInit(0));
  CUdevice dev;
  DRV(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
  DRV(cuCtxSetCurrent(ctx));
  for (int i = 0; i < 5; i++) {
    std::string path = std::string(dir) + "/" + kFiles[i] + ".cubin";
    DRV(cuModuleLoad(&g_mod[i], path.c_str()));
  }
  return 0;
}

// GridSearch<T>::GridSearch + run (GridSearch.cu:252-317).
int ref_gridsearch(int nparams, int nvox, int nmeas, int cfp_size, int fixp_size, CUdeviceptr meas,
                   CUdeviceptr params, CUdeviceptr cfp, CUdeviceptr fixp, int ngp,
                   const int* grid_params, int combs, CUdeviceptr grid, const int* btypes,
                   const float* bmin, const float* bmax) {
  if (nvox % 8) return -1;
  std::vector<int> gp(nparams, 0);
  for (int i = 0; i < ngp; i++) gp[i] = grid_params[i];
  if (set_const(M_GS, "_ZN7Cudimot10gridParamsE", gp.data(), nparams * sizeof(int)) ||
      set_const(M_GS, "_ZN7Cudimot13GSbound_typesE", btypes, nparams * sizeof(int)) ||
      set_const(M_GS, "_ZN7Cudimot12GSbounds_minE", bmin, nparams * sizeof(float)) ||
      set_const(M_GS, "_ZN7Cudimot12GSbounds_maxE", bmax, nparams * sizeof(float)))
    return -1;
  CUfunction f;
  if (get_fn(M_GS, std::string("_ZN7Cudimot17gridSearch_kernelI") + g_t + "Lb0EEEviiiiiPT_S2_S2_S2_S2_i", &f))
    return -1;
  const size_t smem = 2 * 8 * sizeof(double) + (size_t)nmeas * cfp_size * g_ts +
                      2 * (size_t)nparams * 8 * g_ts + 8 * sizeof(int);  // :298-303
  int dbg = -1;
  void* args[] = {&ngp, &combs, &nmeas, &cfp_size, &fixp_size, &meas, &grid, &params, &cfp, &fixp, &dbg};
  return launch(f, nvox / 8, 8 * 32, smem, args);
}

// Levenberg_Marquardt<T>::Levenberg_Marquardt + run (Levenberg_Marquardt.cu:627-704).
int ref_levmar(int nparams, int nvox, int nmeas, int cfp_size, int fixp_size, CUdeviceptr meas,
               CUdeviceptr params, CUdeviceptr cfp, CUdeviceptr fixp, int max_iters, int marquardt,
               const int* btypes, const float* bmin, const float* bmax, const int* fixed) {
  if (nvox % 8) return -1;
  if (set_const(M_LM, "_ZN7Cudimot13LMbound_typesE", btypes, nparams * sizeof(int)) ||
      set_const(M_LM, "_ZN7Cudimot12LMbounds_minE", bmin, nparams * sizeof(float)) ||
      set_const(M_LM, "_ZN7Cudimot12LMbounds_maxE", bmax, nparams * sizeof(float)) ||
      set_const(M_LM, "_ZN7Cudimot7LMfixedE", fixed, nparams * sizeof(int)))
    return -1;
  CUfunction f;
  std::string name = std::string("_ZN7Cudimot16levenberg_kernelI") + g_t + "Lb" + b(marquardt) +
                     "ELb0EEEviiiPT_S2_S2_S2_ii";
  if (get_fn(M_LM, name, &f)) return -1;
  const size_t np = nparams;
  const size_t smem = 4 * 2 * sizeof(double) + (size_t)nmeas * cfp_size * g_ts +
                      3 * np * 2 * g_ts + np * np * 2 * g_ts + 2 * 2 * sizeof(int) +
                      np * 2 * g_ts;  // :674-682
  int dbg = -1;
  void* args[] = {&nmeas, &cfp_size, &fixp_size, &meas, &params, &cfp, &fixp, &max_iters, &dbg};
  return launch(f, nvox / 2, 2 * 32, smem, args);
}

// MCMC<T>::MCMC + run (MCMC.cu:691-848): random states seeded as
// srand(seed + idPart); curand_init(rand(), id, 0), burn-in launch then
// recording launch.
int ref_mcmc(int nparams, int nvox, int nmeas, int cfp_size, int fixp_size, CUdeviceptr meas,
             CUdeviceptr params, CUdeviceptr cfp, CUdeviceptr fixp, CUdeviceptr samples,
             CUdeviceptr tau, int nburn, int njumps, int sampleevery, int update_proposal,
             int rician, int seed, int id_part, const int* btypes, const float* bmin,
             const float* bmax, const int* ptypes, const float* pa, const float* pb,
             const int* fixed) {
  if (nvox % 8) return -1;
  // iteration njumps-1 records sample (njumps-1)/se, which CUDIMOT does not
  // bound-check against nsamples = njumps/se (MCMC.cu:616-621)
  if (sampleevery <= 0 || njumps % sampleevery) return -1;
  if (set_const(M_MCMC, "_ZN7Cudimot13MCbound_typesE", btypes, nparams * sizeof(int)) ||
      set_const(M_MCMC, "_ZN7Cudimot12MCbounds_minE", bmin, nparams * sizeof(float)) ||
      set_const(M_MCMC, "_ZN7Cudimot12MCbounds_maxE", bmax, nparams * sizeof(float)) ||
      set_const(M_MCMC, "_ZN7Cudimot13MCprior_typesE", ptypes, nparams * sizeof(int)) ||
      set_const(M_MCMC, "_ZN7Cudimot10MCpriors_aE", pa, nparams * sizeof(float)) ||
      set_const(M_MCMC, "_ZN7Cudimot10MCpriors_bE", pb, nparams * sizeof(float)) ||
      set_const(M_MCMC, "_ZN7Cudimot7MCfixedE", fixed, nparams * sizeof(int)))
    return -1;
  if (nburn < 1) nburn = 1;  // :702-703
  const int nsamples = njumps / sampleevery;
  const int upe = sampleevery;  // :711
  const size_t state_bytes = 48;  // sizeof(curandStateXORWOW)
  const int blocks_rand = (nvox + 255) / 256;
  CUdeviceptr states, propsd, taupsd;
  DRV(cuMemAlloc(&states, (size_t)blocks_rand * 256 * state_bytes));
  DRV(cuMemAlloc(&propsd, (size_t)nvox * nparams * g_ts));
  DRV(cuMemAlloc(&taupsd, (size_t)nvox * g_ts));
  CUfunction fs;
  int rc = get_fn(M_MCMC, "_ZN7Cudimot20setup_randoms_kernelEP17curandStateXORWOWd", &fs);
  if (!rc) {
    srand(seed + id_part);
    double s = (double)rand();
    void* a0[] = {&states, &s};
    rc = launch(fs, blocks_rand, 256, 0, a0);
  }
  const size_t np = nparams;
  const size_t smem = 8 * state_bytes + (size_t)nmeas * cfp_size * g_ts + 3 * np * 8 * g_ts +
                      2 * 8 * g_ts + 3 * 8 * g_ts + 3 * 8 * g_ts + 2 * np * 8 * sizeof(int) +
                      2 * 8 * sizeof(int);  // :780-791
  int dbg = -1;
  for (int phase = 0; phase < 2 && !rc; phase++) {
    const int rec = phase;
    const int upd = rec ? update_proposal : 1;
    int niters = rec ? njumps : nburn;
    std::string name = std::string("_ZN7Cudimot11mcmc_kernelI") + g_t + "Lb" + b(rec) + "ELb" + b(upd) +
                       "ELb" + b(rician) + "ELb0EEEvP17curandStateXORWOWiiiiiiiPT_S4_S4_S4_S4_S4_S4_S4_i";
    CUfunction f;
    rc = get_fn(M_MCMC, name, &f);
    if (rc) break;
    int ns = nsamples, se = sampleevery, up = upe;
    void* args[] = {&states, &nmeas, &cfp_size, &fixp_size, &niters, &ns, &se, &up, &meas, &params,
                    &propsd, &cfp, &fixp, &samples, &tau, &taupsd, &dbg};
    rc = launch(f, nvox / 8, 8 * 32, smem, args);
  }
  cuMemFree(states);
  cuMemFree(propsd);
  cuMemFree(taupsd);
  return rc;
}

// BIC_AIC<T>::run (BIC_AIC.cu:212-243).
int ref_bic_aic(int nparams, int nvox, int nmeas, int nsamples, int cfp_size, int fixp_size,
                CUdeviceptr meas, CUdeviceptr samples, CUdeviceptr cfp, CUdeviceptr fixp,
                CUdeviceptr bic, CUdeviceptr aic, CUdeviceptr tau, int rician) {
  if (nvox % 8) return -1;
  CUfunction f;
  std::string name = std::string("_ZN7Cudimot14bic_aic_kernelI") + g_t + "Lb" + b(rician) +
                     "EEEviiiiPT_S2_S2_S2_S2_S2_S2_";
  if (get_fn(M_BIC, name, &f)) return -1;
  const size_t smem = (size_t)nmeas * cfp_size * g_ts + (size_t)nparams * 8 * g_ts +
                      3 * 8 * g_ts;  // :223-228
  void* args[] = {&nmeas, &nsamples, &cfp_size, &fixp_size, &meas, &samples, &cfp, &fixp, &bic, &aic, &tau};
  return launch(f, nvox / 8, 8 * 32, smem, args);
}

// getPredictedSignal<T>::run (getPredictedSignal.cu:100-117).
int ref_predicted(int nparams, int nvox, int nmeas, int nsamples, int cfp_size, int fixp_size,
                  CUdeviceptr samples, CUdeviceptr cfp, CUdeviceptr fixp, CUdeviceptr pred) {
  if (nvox % 8) return -1;
  CUfunction f;
  if (get_fn(M_PRED, std::string("_ZN7Cudimot25getPredictedSignal_kernelI") + g_t + "EEviiiiiPT_S2_S2_S2_", &f))
    return -1;
  const size_t smem = (size_t)nmeas * cfp_size * g_ts + (size_t)nparams * 8 * g_ts;
  void* args[] = {&nvox, &nmeas, &nsamples, &cfp_size, &fixp_size, &samples, &cfp, &fixp, &pred};
  return launch(f, nvox / 8, 8 * 32, smem, args);
}

}  // extern "C"
