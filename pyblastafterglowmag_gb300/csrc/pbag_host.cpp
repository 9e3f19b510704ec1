// pbag_host.cpp - host-side parts of the comoving-radiation step that run once
// per grid or once per step on scalars:
//   * the electron and photon grids of one CommonTables entry
//     (base_state.h:217-253, utils.h MakeLogspaceVec);
//   * the per-step shock scalars B, gamma_min, gamma_max, gamma_c, accel_frac,
//     Theta, z_cool that ElectronAndRadiaionBase::updateSockProperties +
//     computeEleSpectrumLimits set (microphysics_base.h:575-966), one call
//     after another (the per-call arithmetic is pbag_limits.cuh, shared with
//     the device kernel of pbag_limits.cu).
// Paths are relative to the reference project's src/ directory.
#include <cmath>
#include <cstring>

#include "pbag.h"
#include "pbag_const.h"
#include "pbag_internal.h"
#include "pbag_limits.cuh"

using namespace pbag::cgs;

namespace pbag {

void build_grids(const pbag_grid_desc* g, double* gam, double* freq) {
  const int G = g->ngam, F = g->nfreq;
  // base_state.h:229-236: e[i] = step^i with step = exp(ln(gam2)/G)
  double step = std::exp(std::log(g->gam2) / (double)G);
  for (int i = 0; i < G; i++) gam[i] = std::pow(step, (double)i);
  // utils.h MakeLogspaceVec: x0 = 10^start, x_{i+1} = x_i * 10^((stop-start)/num);
  // one extra point (index F) defines the one-past-the-end read of
  // computeSSCSpectrum (numeric_model.h:269-272).
  double start = std::log10(g->freq1), stop = std::log10(g->freq2);
  double cur = std::pow(10., start);
  double base = std::pow(10., (stop - start) / F);
  for (int i = 0; i <= F; i++) {
    freq[i] = cur;
    cur *= base;
  }
}

}  // namespace pbag

extern "C" {

int pbag_abi_version(void) { return PBAG_ABI_VERSION; }

size_t pbag_sizeof(int which) {
  switch (which) {
    case 0: return sizeof(pbag_grid_desc);
    case 1: return sizeof(pbag_shock_params);
    case 2: return sizeof(pbag_step_rec);
    case 3: return sizeof(pbag_outputs);
    case 4: return sizeof(pbag_status);
    case 5: return sizeof(pbag_limits_opts);
    case 6: return sizeof(pbag_shock_state);
    case 7: return sizeof(pbag_limits);
    case 8: return sizeof(pbag_flux_opts);
    case 9: return sizeof(pbag_flux_query);
    default: return 0;
  }
}

int pbag_build_grids(const pbag_grid_desc* g, double* gam, double* freq) {
  if (!g || !gam || !freq || g->ngam < PBAG_MIN_BINS || g->ngam > PBAG_MAX_BINS || g->nfreq < PBAG_MIN_BINS ||
      g->nfreq > PBAG_MAX_BINS || !(g->gam2 > 1.) || !(g->freq1 > 0.) || !(g->freq2 > g->freq1))
    return PBAG_ERR_ARG;
  pbag::build_grids(g, gam, freq);
  return PBAG_OK;
}

int pbag_shock_limits(const pbag_limits_opts* o, const double* gam, int ngam, int n, const pbag_shock_state* in,
                      double* state, pbag_limits* out) {
  if (!o || !gam || ngam < 2 || n < 0 || (n > 0 && (!in || !out)) || !state) return PBAG_ERR_ARG;
  pbag::LimState s{};
  s.o = o;
  s.gamma_min = state[0];
  s.gamma_max = state[1];
  s.gamma_c = state[2];
  s.accel_frac = state[3];
  s.B = state[4];
  s.Theta = state[5];
  s.z_cool = state[6];
  for (int i = 0; i < n; ++i) {
    int valid = 0, accel_set = 0;
    const int rc = pbag::lim_one(s, in[i], gam[0], gam[ngam - 1], &valid, &accel_set);
    if (rc != PBAG_OK) return rc;
    pbag::lim_store(s, valid, out[i]);
  }
  state[0] = s.gamma_min;
  state[1] = s.gamma_max;
  state[2] = s.gamma_c;
  state[3] = s.accel_frac;
  state[4] = s.B;
  state[5] = s.Theta;
  state[6] = s.z_cool;
  return PBAG_OK;
}

const char* pbag_status_string(int code) {
  switch (code) {
    case PBAG_OK: return "ok";
    case PBAG_ERR_ARG: return "bad argument";
    case PBAG_ERR_CUDA: return "CUDA runtime error";
    case PBAG_ERR_NONFINITE: return "non-finite or negative value";
    case PBAG_ERR_NELE: return "total electron number <= 0";
    case PBAG_ERR_PARAM: return "invalid shock parameters";
    case PBAG_ERR_DLNVDT: return "invalid dlnV/dt";
    case PBAG_ERR_UNSUPPORTED: return "option not supported by the GPU path";
    case PBAG_ERR_TIMEOUT: return "device-side wait timed out";
    case PBAG_ERR_NOMEM: return "device allocation failed";
    default: return "unknown status";
  }
}

}  // extern "C"
