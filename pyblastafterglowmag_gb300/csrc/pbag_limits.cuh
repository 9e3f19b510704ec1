// pbag_limits.cuh - the per-step shock scalars that
// ElectronAndRadiaionBase::updateSockProperties + computeEleSpectrumLimits set
// (microphysics_base.h:575-605, 642-652, 736-966; Bisect rootfinders.h:17-58),
// for one call, shared by the host loop (pbag_host.cpp) and the device kernel
// (pbag_limits.cu). Paths are relative to the reference project's src/.
#ifndef PBAG_LIMITS_CUH
#define PBAG_LIMITS_CUH

#include <cmath>

#include "pbag.h"
#include "pbag_const.h"

#ifdef __CUDACC__
#define PBAG_HD __host__ __device__
#else
#define PBAG_HD
#endif

namespace pbag {

#ifndef __CUDACC__
using std::isfinite;
#endif

// The ElectronAndRadiaionBase members the prep reads and writes.
struct LimState {
  const pbag_limits_opts* o;
  double e_prime, Gamma, GammaSh, betaSh, t_e, tcomov, n_prime;
  double B, gamma_min, gamma_max, gamma_c, accel_frac, Theta, z_cool;
};

PBAG_HD inline double lim_beta(double gam) {  // EQS::BetaFromGamma (blastwave_components.h:36-39)
  return sqrt((gam - 1.) * (gam + 1.)) / gam;
}

// gammaMinFunc (microphysics_base.h:792-806): the p==1 and p==2 branches use
// the member gamma_min, not the bracketing variable, as the reference does
PBAG_HD inline double lim_gm_func(double x, const LimState& s) {
  using namespace cgs;
  const double p = s.o->p;
  const double gamma_ave = s.o->eps_e * s.e_prime / (s.n_prime * m_e * c_light * c_light);
  if (p == 1) return (s.gamma_max - s.gamma_min) / (log(s.gamma_max) - log(s.gamma_min)) - gamma_ave;
  if (p == 2) return (log(s.gamma_max) - log(s.gamma_min)) / (-1. / s.gamma_max + 1. / s.gamma_min) - gamma_ave;
  return (p - 1) / (p - 2) * (pow(s.gamma_max, -p + 2) - pow(x, -p + 2)) / (pow(s.gamma_max, -p + 1) - pow(x, -p + 1)) -
         gamma_ave;
}

// Bisect (rootfinders.h:17-58); status -1 on failure
PBAG_HD inline double lim_bisect(double xa, double xb, double xtol, double rtol, int iter, const LimState& s,
                                 int& status) {
  status = 0;
  const double fa = lim_gm_func(xa, s), fb = lim_gm_func(xb, s);
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
    const double xm = xa + dm;
    const double fm = lim_gm_func(xm, s);
    if (fm * fa >= 0) xa = xm;
    if (fm == 0 || fabs(dm) < xtol + rtol * fabs(xm)) return xm;
  }
  status = -1;
  return xa;
}

// One call of updateSockProperties + computeEleSpectrumLimits on the members
// in s. Returns PBAG_OK, or the code where the reference exits; *valid = 0
// when checkParams() refused the state and nothing was recomputed;
// *accel_set = 1 when this call assigned accel_frac (the non-relativistic
// branch), else accel_frac keeps its earlier value. gam_lo / gam_hi: first and
// last points of the electron grid (they cap gamma_min and gamma_max).
PBAG_HD inline int lim_one(LimState& s, const pbag_shock_state& a, double gam_lo, double gam_hi, int* valid,
                           int* accel_set) {
  using namespace cgs;
  const pbag_limits_opts* o = s.o;
  const bool numeric = !o->ele_analytic;
  // updateSockProperties (microphysics_base.h:575-605)
  s.GammaSh = a.GammaSh;
  s.e_prime = a.e_prime;
  s.Gamma = a.Gamma;
  s.betaSh = lim_beta(a.GammaSh);
  s.t_e = a.t_e;
  s.tcomov = a.tcomov;
  s.n_prime = a.n_prime;
  *accel_set = 0;
  // checkParams (microphysics_base.h:736-787)
  *valid = s.betaSh < o->beta_min ? 0 : 1;
  if (!*valid) return PBAG_OK;
  if (o->eps_e <= 0 || o->eps_b <= 0 || o->eps_t < 0 || o->p <= 0 || s.n_prime <= 0 || s.e_prime < 0 ||
      !isfinite(s.e_prime))
    return PBAG_ERR_PARAM;
  // computeMagneticField (microphysics_base.h:808-823)
  const double U_b = s.e_prime * o->eps_b;
  const double B1 = sqrt(8. * pi_ * U_b);
  const double B2 =
      sqrt(32. * M_PI * o->eps_b * (s.GammaSh - 1.) * (s.GammaSh + 3. / 4) * s.n_prime * m_p * (c_light * c_light));
  const double B3 = sqrt(9.0 * M_PI * o->eps_b * s.n_prime * o->mu * m_p) * (s.betaSh * c_light);
  s.B = o->method_B == 0 ? B1 : (o->method_B == 2 ? B2 : B3);
  // computeGammaMax (microphysics_base.h:824-837)
  const double gmax1 = sqrt(6.0 * pi_ * q_e / sigma_T / s.B);
  if (o->method_gamma_max == 0) s.gamma_max = gmax1;
  if (numeric && s.gamma_max > 0.99 * gam_hi) s.gamma_max = 0.99 * gam_hi;
  // computeGammaMin (microphysics_base.h:838-937)
  const double p = o->p;
  int status = 0;
  const double U_e = s.e_prime * o->eps_e;
  const double gm1 = (p - 2.) / (p - 1.) * U_e / (s.n_prime * m_e * c_light * c_light);
  const double gm2 = (p - 2.) / (p - 1.) * (m_p / m_e) * o->eps_e * lim_beta(s.GammaSh);
  const double gm3 = (p - 2.) / (p - 1.) * (o->eps_e * m_p / m_e * (s.GammaSh - 1.) + 1.);
  {  // Margalit21::Theta_fun (analytic_models.h:57-64)
    const double th0 = o->eps_t * (9.0 * o->mu * m_p / (32.0 * o->mu_e * m_e)) * s.betaSh * s.betaSh;
    s.Theta = (5.0 * th0 - 6.0 + sqrt(25.0 * th0 * th0 + 180.0 * th0 + 36.0)) / 30.0;
  }
  s.z_cool = (6.0 * M_PI * m_e * c_light / (sigma_T * s.B * s.B * s.t_e)) / s.Theta;
  // Margalit21::gamma_m_fun / a_fun (analytic_models.h:29-32, 80-82)
  const double gm4 = 1. + (6.0 + 15.0 * s.Theta) / (4.0 + 5.0 * s.Theta) * s.Theta;
  switch (o->method_gamma_min) {
    case 0: s.gamma_min = gm1; break;
    case 2: s.gamma_min = gm2; break;
    case 3: s.gamma_min = gm3; break;
    case 1:
      s.gamma_min = lim_bisect(1., 1.e8, 0., .001, 100, s, status);
      if ((status < 0) && (gm1 > 1.5)) s.gamma_min = gm1;
      break;
    case 4: s.gamma_min = gm4; break;
    default: return PBAG_ERR_ARG;
  }
  const double af_ayache = (pow(s.gamma_max, 2 - p) - pow(s.gamma_min - 1., 2. - p)) / (pow(s.gamma_max, 2. - p) - 1.) *
                           (pow(s.gamma_max, 1. - p) - 1.) / (pow(s.gamma_max, 1. - p) - pow(s.gamma_min - 1., 1. - p));
  const double af_sironi = (p - 2.0) / (p - 1.0) * o->eps_e * s.e_prime / (s.n_prime * m_e * c_light * c_light);
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
    *accel_set = 1;
  }
  if (!isfinite(s.gamma_min) || !isfinite(s.accel_frac) || s.accel_frac < 0) return PBAG_ERR_NONFINITE;
  if (numeric && s.gamma_min < gam_lo) {
    s.gamma_min = gam_lo;
    if (s.gamma_min > 1e8) return PBAG_ERR_PARAM;
  }
  // computeGammaCool (microphysics_base.h:938-966)
  const double gc1 = 6. * pi_ * m_e * c_light / (sigma_T * s.B * s.B) * a.t_e / s.Gamma;
  const double gc2 = ((6. * pi_ * m_e * c_light) / (sigma_T * s.B * s.B * (s.tcomov)));
  if (o->method_gamma_c == 0) s.gamma_c = gc1;
  if (o->method_gamma_c == 1) s.gamma_c = gc2;
  if (s.gamma_c <= 1.) s.gamma_c = 1.001;
  if (numeric && s.gamma_c > s.gamma_max) s.gamma_c = s.gamma_max;
  return PBAG_OK;
}

PBAG_HD inline void lim_store(const LimState& s, int valid, pbag_limits& r) {
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

}  // namespace pbag

#endif
