// pbag_host.cpp - host-side parts of the comoving-radiation step that run once
// per grid or once per step on scalars:
//   * the electron and photon grids of one CommonTables entry
//     (base_state.h:217-253, utils.h MakeLogspaceVec);
//   * the per-step shock scalars B, gamma_min, gamma_max, gamma_c, accel_frac,
//     Theta, z_cool that ElectronAndRadiaionBase::updateSockProperties +
//     computeEleSpectrumLimits set (microphysics_base.h:575-966).
// Paths are relative to the reference project's src/ directory.
#include <cmath>
#include <cstring>

#include "pbag.h"
#include "pbag_const.h"
#include "pbag_internal.h"

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

namespace {

inline double beta_from_gamma(double gam) {  // blastwave_components.h:36-39
  return std::sqrt((gam - 1.) * (gam + 1.)) / gam;
}

struct LimState {  // the ElectronAndRadiaionBase members the prep reads and writes
  const pbag_limits_opts* o;
  double e_prime, Gamma, GammaSh, betaSh, t_e, tcomov, n_prime;
  double B, gamma_min, gamma_max, gamma_c, accel_frac, Theta, z_cool;
};

// microphysics_base.h:792-806 gammaMinFunc (the p==1 and p==2 branches use the
// member gamma_min, not the bracketing variable, exactly as the reference does)
double gamma_min_func(double x, const LimState& s) {
  const double p = s.o->p;
  double gamma_ave = s.o->eps_e * s.e_prime / (s.n_prime * m_e * c_light * c_light);
  if (p == 1)
    return (s.gamma_max - s.gamma_min) / (std::log(s.gamma_max) - std::log(s.gamma_min)) - gamma_ave;
  else if (p == 2)
    return (std::log(s.gamma_max) - std::log(s.gamma_min)) / (-1. / s.gamma_max + 1. / s.gamma_min) - gamma_ave;
  return (p - 1) / (p - 2) * (std::pow(s.gamma_max, -p + 2) - std::pow(x, -p + 2)) /
             (std::pow(s.gamma_max, -p + 1) - std::pow(x, -p + 1)) -
         gamma_ave;
}

// rootfinders.h:17-58 Bisect (status -1 on failure)
double bisect(double xa, double xb, double xtol, double rtol, int iter, const LimState& s, int& status) {
  status = 0;
  double fa = gamma_min_func(xa, s), fb = gamma_min_func(xb, s);
  if (fa * fb > 0) {
    status = -1;
    return 0.;
  }
  if (fa == 0) {
    status = -1;
    return xa;
  }
  if (fb == 0) {
    status = -1;
    return xb;
  }
  double dm = xb - xa;
  for (int i = 0; i < iter; i++) {
    dm *= 0.5;
    double xm = xa + dm;
    double fm = gamma_min_func(xm, s);
    if (fm * fa >= 0) xa = xm;
    if (fm == 0 || std::fabs(dm) < xtol + rtol * std::fabs(xm)) return xm;
  }
  status = -1;
  return xa;
}

}  // namespace

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
  LimState s{};
  s.o = o;
  s.gamma_min = state[0];
  s.gamma_max = state[1];
  s.gamma_c = state[2];
  s.accel_frac = state[3];
  s.B = state[4];
  s.Theta = state[5];
  s.z_cool = state[6];
  const bool numeric = !o->ele_analytic;
  for (int i = 0; i < n; ++i) {
    const pbag_shock_state& a = in[i];
    // updateSockProperties (microphysics_base.h:575-605)
    s.GammaSh = a.GammaSh;
    s.e_prime = a.e_prime;
    s.Gamma = a.Gamma;
    s.betaSh = beta_from_gamma(a.GammaSh);
    s.t_e = a.t_e;
    s.tcomov = a.tcomov;
    s.n_prime = a.n_prime;
    // checkParams (microphysics_base.h:736-787)
    int valid = s.betaSh < o->beta_min ? 0 : 1;
    if (valid) {
      if (o->eps_e <= 0 || o->eps_b <= 0 || o->eps_t < 0 || o->p <= 0 || s.n_prime <= 0 || s.e_prime < 0 ||
          !std::isfinite(s.e_prime))
        return PBAG_ERR_PARAM;
      // computeMagneticField (microphysics_base.h:808-823)
      double U_b = s.e_prime * o->eps_b;
      double B1 = std::sqrt(8. * pi_ * U_b);
      double B2 = std::sqrt(32. * M_PI * o->eps_b * (s.GammaSh - 1.) * (s.GammaSh + 3. / 4) * s.n_prime * m_p *
                            (c_light * c_light));
      double B3 = std::sqrt(9.0 * M_PI * o->eps_b * s.n_prime * o->mu * m_p) * (s.betaSh * c_light);
      s.B = o->method_B == 0 ? B1 : (o->method_B == 2 ? B2 : B3);
      // computeGammaMax (microphysics_base.h:824-837)
      double gmax1 = std::sqrt(6.0 * pi_ * q_e / sigma_T / s.B);
      if (o->method_gamma_max == 0) s.gamma_max = gmax1;
      if (numeric && s.gamma_max > 0.99 * gam[ngam - 1]) s.gamma_max = 0.99 * gam[ngam - 1];
      // computeGammaMin (microphysics_base.h:838-937)
      const double p = o->p;
      int status = 0;
      double U_e = s.e_prime * o->eps_e;
      double gm1 = (p - 2.) / (p - 1.) * U_e / (s.n_prime * m_e * c_light * c_light);
      double gm2 = (p - 2.) / (p - 1.) * (m_p / m_e) * o->eps_e * beta_from_gamma(s.GammaSh);
      double gm3 = (p - 2.) / (p - 1.) * (o->eps_e * m_p / m_e * (s.GammaSh - 1.) + 1.);
      {  // Margalit21::Theta_fun (analytic_models.h:57-64)
        double th0 = o->eps_t * (9.0 * o->mu * m_p / (32.0 * o->mu_e * m_e)) * s.betaSh * s.betaSh;
        s.Theta = (5.0 * th0 - 6.0 + std::sqrt(25.0 * th0 * th0 + 180.0 * th0 + 36.0)) / 30.0;
      }
      s.z_cool = (6.0 * M_PI * m_e * c_light / (sigma_T * s.B * s.B * s.t_e)) / s.Theta;
      // Margalit21::gamma_m_fun / a_fun (analytic_models.h:29-32, 80-82)
      double gm4 = 1. + (6.0 + 15.0 * s.Theta) / (4.0 + 5.0 * s.Theta) * s.Theta;
      switch (o->method_gamma_min) {
        case 0: s.gamma_min = gm1; break;
        case 2: s.gamma_min = gm2; break;
        case 3: s.gamma_min = gm3; break;
        case 1:
          s.gamma_min = bisect(1., 1.e8, 0., .001, 100, s, status);
          if ((status < 0) && (gm1 > 1.5)) s.gamma_min = gm1;
          break;
        case 4: s.gamma_min = gm4; break;
        default: return PBAG_ERR_ARG;
      }
      double af_ayache = (std::pow(s.gamma_max, 2 - p) - std::pow(s.gamma_min - 1., 2. - p)) /
                         (std::pow(s.gamma_max, 2. - p) - 1.) * (std::pow(s.gamma_max, 1. - p) - 1.) /
                         (std::pow(s.gamma_max, 1. - p) - std::pow(s.gamma_min - 1., 1. - p));
      double af_sironi = (p - 2.0) / (p - 1.0) * o->eps_e * s.e_prime / (s.n_prime * m_e * c_light * c_light);
      if ((s.gamma_min < 2.) || (status < 0)) {
        switch (o->method_nonrel) {
          case 0: s.accel_frac = 1; break;
          case 1: s.accel_frac = s.gamma_min; break;
          case 2:
            if (p < 2.) return PBAG_ERR_PARAM;
            s.accel_frac = af_ayache;
            break;
          case 3:
            if (p < 2.) return PBAG_ERR_PARAM;
            s.accel_frac = af_sironi;
            break;
          default: return PBAG_ERR_ARG;
        }
        s.accel_frac = s.accel_frac > 1. ? 1 : s.accel_frac;
        s.gamma_min = s.gamma_min < 1. ? 1 : s.gamma_min;
      }
      if (!std::isfinite(s.gamma_min) || !std::isfinite(s.accel_frac) || s.accel_frac < 0) return PBAG_ERR_NONFINITE;
      if (numeric && s.gamma_min < gam[0]) {
        s.gamma_min = gam[0];
        if (s.gamma_min > 1e8) return PBAG_ERR_PARAM;
      }
      // computeGammaCool (microphysics_base.h:938-966)
      double gc1 = 6. * pi_ * m_e * c_light / (sigma_T * s.B * s.B) * a.t_e / s.Gamma;
      double gc2 = ((6. * pi_ * m_e * c_light) / (sigma_T * s.B * s.B * (s.tcomov)));
      if (o->method_gamma_c == 0) s.gamma_c = gc1;
      if (o->method_gamma_c == 1) s.gamma_c = gc2;
      if (s.gamma_c <= 1.) s.gamma_c = 1.001;
      if (numeric && s.gamma_c > s.gamma_max) s.gamma_c = s.gamma_max;
    }
    pbag_limits& r = out[i];
    r.B = s.B;
    r.gamma_min = s.gamma_min;
    r.gamma_max = s.gamma_max;
    r.gamma_c = s.gamma_c;
    r.accel_frac = s.accel_frac;
    r.Theta = s.Theta;
    r.z_cool = s.z_cool;
    r.valid = valid;
    r.reserved = 0;
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
