// cdm_host.cpp - host-side helpers shared by every model library.
#include "cdm_host.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace {
thread_local std::string g_last_error;
}

cdm_status cdm_fail(cdm_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

extern "C" const char* cdm_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* cdm_status_string(cdm_status s) {
  switch (s) {
    case CDM_OK: return "OK";
    case CDM_BAD_ARG: return "BAD_ARG";
    case CDM_CUDA_ERROR: return "CUDA_ERROR";
    case CDM_TIMEOUT: return "TIMEOUT";
    case CDM_NOT_SUPPORTED: return "NOT_SUPPORTED";
    case CDM_IO_ERROR: return "IO_ERROR";
  }
  return "UNKNOWN";
}

// Option defaults of cudimotoptions.h:78-168.
void cdm_fill_default_cfg(cdm_model_cfg* c, int nparams) {
  std::memset(c, 0, sizeof(*c));
  c->nparams = nparams;
  c->run_levmar = 1;
  c->iter_levmar = 200;
  c->marquardt = 1;
  c->nburn = 1000;
  c->njumps = 1250;
  c->sampleevery = 25;
  c->update_proposal = 1;
  c->seed = 8219;
}

cdm_status cdm_validate_cfg(const cdm_model_cfg* c, int nparams) {
  for (int p = 0; p < nparams; p++) {
    if (c->bound_types[p] < CDM_NOBOUNDS || c->bound_types[p] > CDM_BMINMAX)
      return cdm_fail(CDM_BAD_ARG, "bad bound type for parameter " + std::to_string(p));
    if (c->prior_types[p] < CDM_NOPRIOR || c->prior_types[p] > CDM_CUSTOM)
      return cdm_fail(CDM_BAD_ARG, "bad prior type for parameter " + std::to_string(p));
  }
  if (c->run_gridsearch) {
    if (c->n_grid_params <= 0 || c->n_grid_params > nparams || c->grid_combs <= 0 || !c->grid)
      return cdm_fail(CDM_BAD_ARG, "grid search enabled without a grid");
    for (int i = 0; i < c->n_grid_params; i++)
      if (c->grid_params[i] < 0 || c->grid_params[i] >= nparams)
        return cdm_fail(CDM_BAD_ARG, "grid parameter id out of range");
  }
  if (c->run_levmar && c->iter_levmar < 0) return cdm_fail(CDM_BAD_ARG, "iter_levmar < 0");
  if (c->run_mcmc) {
    if (c->njumps <= 0 || c->sampleevery <= 0 || c->njumps < c->sampleevery)
      return cdm_fail(CDM_BAD_ARG,
                      "MCMC must record at least one sample: --nj must be >= --se (MCMC.cu:707)");
    if (c->nburn < 0) return cdm_fail(CDM_BAD_ARG, "nburn < 0");
  }
  for (int l : {c->lanes_gridsearch, c->lanes_levmar, c->lanes_mcmc})
    if (!(l == 0 || l == 1 || l == 2 || l == 4 || l == 8 || l == 16 || l == 32))
      return cdm_fail(CDM_BAD_ARG, "lanes per voxel must be 0, 1, 2, 4, 8, 16 or 32");
  if (c->first_voxel < 0 || c->first_voxel > 0xFFFFFFFFll)
    return cdm_fail(CDM_BAD_ARG, "first_voxel must be in 0 .. 2^32 - 1");
  return CDM_OK;
}

namespace {
// std::string::find returns npos; CUDIMOT stores it in an int and tests >= 0.
bool has(const std::string& s, const std::string& m, size_t* pos) {
  *pos = s.find(m);
  return *pos != std::string::npos;
}

std::vector<double> split_values(std::string vals) {
  std::vector<double> out;
  size_t p;
  while ((p = vals.find(',')) != std::string::npos) {
    out.push_back(std::strtod(vals.substr(0, p).c_str(), nullptr));
    vals.erase(0, p + 1);
  }
  out.push_back(std::strtod(vals.c_str(), nullptr));
  return out;
}
}  // namespace

// Model::Modelparser (Model.cu:16-299), with its rules: a line containing
// "//" anywhere is skipped; the markers are "P_init[", "bounds[" and
// "prior[" (so "priors[i]=..." is not recognised); bounds "(min,max)",
// "(min,)" or "(,max)"; priors Gaussian(mean,std), Gamma(a,b), ARD(f),
// sin(), custom().
cdm_status cdm_parse_priors_impl(const char* path, int nparams, cdm_model_cfg* cfg,
                                 double* p_init, int* p_init_given) {
  if (!path || !cfg) return cdm_fail(CDM_BAD_ARG, "null argument");
  std::ifstream f(path);
  if (!f.is_open())
    return cdm_fail(CDM_IO_ERROR, std::string("Unable to open file with Priors information: ") + path);
  for (int p = 0; p < nparams; p++) {
    cfg->bound_types[p] = CDM_NOBOUNDS;
    cfg->bounds_min[p] = cfg->bounds_max[p] = 0.0;
    cfg->prior_types[p] = CDM_NOPRIOR;
    cfg->priors_a[p] = cfg->priors_b[p] = 0.0;
  }
  if (p_init_given) *p_init_given = 0;
  std::string line;
  while (std::getline(f, line)) {
    size_t pos0, pos1;
    if (has(line, "//", &pos0)) continue;
    if (has(line, "P_init[", &pos0)) {
      pos0 += 7;
      pos1 = line.rfind(']');
      std::vector<double> v = split_values(line.substr(pos0, pos1 - pos0));
      if ((int)v.size() != nparams)
        return cdm_fail(CDM_BAD_ARG, "The number of values for initializating the parameters " +
                                         std::to_string(v.size()) +
                                         " do not match the number of parameters of this model " +
                                         std::to_string(nparams));
      if (p_init)
        for (int i = 0; i < nparams; i++) p_init[i] = v[i];
      if (p_init_given) *p_init_given = 1;
    }
    if (has(line, "bounds[", &pos0)) {
      pos0 += 7;
      pos1 = line.rfind(']');
      const int id = std::atoi(line.substr(pos0, pos1 - pos0).c_str());
      if (id >= nparams || id < 0)
        return cdm_fail(CDM_BAD_ARG, "Wrong number of parameter [" + std::to_string(id) +
                                         "] when specifying the bounds");
      cfg->bound_types[id] = CDM_BMINMAX;
      pos1 = line.rfind('(');
      pos0 = pos1 + 1;
      size_t comma = line.rfind(',');
      if (comma == std::string::npos || comma < pos0)
        return cdm_fail(CDM_BAD_ARG, "bounds[" + std::to_string(id) + "] needs (min,max)");
      if (comma - pos0 == 0)
        cfg->bound_types[id] = CDM_BMAX;
      else
        cfg->bounds_min[id] = std::strtod(line.substr(pos0, comma - pos0).c_str(), nullptr);
      pos0 = comma + 1;
      pos1 = line.rfind(')');
      const size_t len = (pos1 == std::string::npos || pos1 < pos0) ? 0 : pos1 - pos0;
      if (len == 0 && cfg->bound_types[id] == CDM_BMINMAX)
        cfg->bound_types[id] = CDM_BMIN;
      else if (len == 0)
        return cdm_fail(CDM_BAD_ARG,
                        "For bounded priors, at least a min or a max value must be specified");
      else
        cfg->bounds_max[id] = std::strtod(line.substr(pos0, len).c_str(), nullptr);
    }
    if (has(line, "prior[", &pos0)) {
      pos0 += 6;
      pos1 = line.rfind(']');
      const int id = std::atoi(line.substr(pos0, pos1 - pos0).c_str());
      if (id >= nparams || id < 0)
        return cdm_fail(CDM_BAD_ARG, "Wrong number of parameter [" + std::to_string(id) +
                                         "] when specifying the priors");
      pos0 = line.rfind('=') + 1;
      pos1 = line.rfind('(');
      const std::string type = line.substr(pos0, pos1 - pos0);
      int t;
      if (type == "Gaussian") t = CDM_GAUSSPRIOR;
      else if (type == "Gamma") t = CDM_GAMMAPRIOR;
      else if (type == "ARD") t = CDM_ARDPRIOR;
      else if (type == "sin") t = CDM_SINPRIOR;
      else if (type == "custom") t = CDM_CUSTOM;
      else return cdm_fail(CDM_BAD_ARG, "Prior " + type + " is a not a recognised prior type");
      cfg->prior_types[id] = t;
      if (t <= CDM_ARDPRIOR) {
        pos0 = pos1 + 1;
        size_t comma = line.rfind(',');
        size_t close = line.rfind(')');
        size_t end1 = (t <= CDM_GAMMAPRIOR) ? comma : close;
        if (end1 == std::string::npos || end1 <= pos0)
          return cdm_fail(CDM_BAD_ARG, "A prior of type " + type + " needs a first argument");
        cfg->priors_a[id] = std::strtod(line.substr(pos0, end1 - pos0).c_str(), nullptr);
        if (t <= CDM_GAMMAPRIOR) {
          pos0 = comma + 1;
          if (close == std::string::npos || close <= pos0)
            return cdm_fail(CDM_BAD_ARG, "A prior of type " + type + " needs a second argument");
          cfg->priors_b[id] = std::strtod(line.substr(pos0, close - pos0).c_str(), nullptr);
        }
      }
    }
  }
  return CDM_OK;
}

// Model::Parser_gridSearch and set_grid (Model.cu:302-393): search[i]=(...)
// lines; combinations enumerate the lowest parameter id outermost.
cdm_status cdm_parse_grid_impl(const char* path, int nparams, int* n_grid_params,
                               int* grid_params, int* grid_combs, double* grid,
                               int64_t grid_capacity) {
  if (!path || !n_grid_params || !grid_combs) return cdm_fail(CDM_BAD_ARG, "null argument");
  std::ifstream f(path);
  if (!f.is_open())
    return cdm_fail(CDM_IO_ERROR, std::string("Unable to open GridSearch file configuration: ") + path);
  std::vector<std::vector<double>> values(nparams);
  std::string line;
  while (std::getline(f, line)) {
    size_t pos0, pos1;
    if (has(line, "//", &pos0)) continue;
    if (has(line, "search[", &pos0)) {
      pos0 += 7;
      pos1 = line.rfind(']');
      const int id = std::atoi(line.substr(pos0, pos1 - pos0).c_str());
      if (id >= nparams || id < 0)
        return cdm_fail(CDM_BAD_ARG, "Wrong number of parameter [" + std::to_string(id) +
                                         "] when specifying the GridSearch values");
      pos0 = line.rfind('(') + 1;
      pos1 = line.rfind(')');
      std::vector<double> v = split_values(line.substr(pos0, pos1 - pos0));
      values[id].insert(values[id].end(), v.begin(), v.end());
    }
  }
  int ngp = 0;
  int64_t combs = 1;
  std::vector<int> ids;
  for (int i = 0; i < nparams; i++)
    if (!values[i].empty()) {
      ids.push_back(i);
      ngp++;
      combs *= (int64_t)values[i].size();
    }
  if (ngp == 0) combs = 0;
  if (combs > (int64_t)1 << 30) return cdm_fail(CDM_BAD_ARG, "grid too large");
  *n_grid_params = ngp;
  *grid_combs = (int)combs;
  if (grid_params)
    for (int i = 0; i < ngp; i++) grid_params[i] = ids[i];
  if (!grid) return CDM_OK;
  if (grid_capacity < combs * ngp) return cdm_fail(CDM_BAD_ARG, "grid buffer too small");
  std::vector<size_t> idx(ngp, 0);
  for (int64_t c = 0; c < combs; c++) {
    for (int k = 0; k < ngp; k++) grid[c * ngp + k] = values[ids[k]][idx[k]];
    for (int k = ngp - 1; k >= 0; k--) {  // last parameter varies fastest
      if (++idx[k] < values[ids[k]].size()) break;
      idx[k] = 0;
    }
  }
  return CDM_OK;
}

// --fixed=i,j (Model.cu:279-298).
cdm_status cdm_parse_fixed_impl(const char* list, int nparams, int* fixed) {
  if (!fixed) return cdm_fail(CDM_BAD_ARG, "null argument");
  for (int p = 0; p < nparams; p++) fixed[p] = 0;
  if (!list || !*list) return CDM_OK;
  std::stringstream ss(list);
  int i;
  std::vector<int> v;
  while (ss >> i) {
    if (i >= nparams || i < 0)
      return cdm_fail(CDM_BAD_ARG, "Wrong number of parameter " + std::to_string(i) +
                                       " when specifying the fixed parameters");
    v.push_back(i);
    if (ss.peek() == ',') ss.ignore();
  }
  for (int k : v) fixed[k] = 1;
  return CDM_OK;
}

namespace {
// Whitespace- or comma-separated ASCII matrix, one row per non-empty line.
bool read_ascii_matrix(const std::string& path, std::vector<std::vector<double>>& m) {
  std::ifstream f(path);
  if (!f.is_open()) return false;
  std::string line;
  while (std::getline(f, line)) {
    for (char& ch : line)
      if (ch == ',' || ch == '\t') ch = ' ';
    std::stringstream ss(line);
    std::vector<double> row;
    double x;
    while (ss >> x) row.push_back(x);
    if (!row.empty()) m.push_back(row);
  }
  return true;
}
}  // namespace

// Parameters.cu:93-149: each non-empty line of the list names an ASCII
// matrix with CFP_size[k] rows and nmeas columns.
cdm_status cdm_read_cfp_list_impl(const char* path, int nmeas, const std::vector<int>& sizes,
                                  double* cfp) {
  if (!path || !cfp) return cdm_fail(CDM_BAD_ARG, "null argument");
  std::ifstream f(path);
  if (!f.is_open())
    return cdm_fail(CDM_IO_ERROR, std::string("Unable to open file with Common Fixed Parameters: ") + path);
  int tsize = 0;
  for (int s : sizes) tsize += s;
  int k = 0, cum = 0;
  std::string line;
  while (std::getline(f, line)) {
    while (!line.empty() && (line.back() == '\r' || line.back() == ' ')) line.pop_back();
    if (line.empty()) continue;
    if (k >= (int)sizes.size())
      return cdm_fail(CDM_BAD_ARG, "more Common Fixed Parameter files than the model has");
    std::vector<std::vector<double>> m;
    if (!read_ascii_matrix(line, m)) return cdm_fail(CDM_IO_ERROR, "cannot read " + line);
    if ((int)m.size() != sizes[k])
      return cdm_fail(CDM_BAD_ARG, "Common Fixed Parameters number " + std::to_string(k) +
                                       " and file " + line +
                                       " do not match the dimensions specified for this model");
    for (const auto& row : m)
      if ((int)row.size() != nmeas)
        return cdm_fail(CDM_BAD_ARG, "Common Fixed Parameters number " + std::to_string(k) +
                                         " and file " + line +
                                         " do not match the number of measurements");
    for (int i = 0; i < sizes[k]; i++)
      for (int j = 0; j < nmeas; j++) cfp[cum + i + (size_t)j * tsize] = m[i][j];
    cum += sizes[k];
    k++;
  }
  if (k != (int)sizes.size())
    return cdm_fail(CDM_BAD_ARG, "The number of Common Fixed Parameters provided is not correct");
  return CDM_OK;
}
