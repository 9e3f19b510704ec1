// pbag_rhs.cuh - the right-hand side of one blastwave's ODE system (forward
// shock, or forward and reverse shock), compiled for the host and the device:
// BlastWave::rhs_fs and BlastWave::rhs_fsrs (blastwave/blastwave.h:1515-1768,
// 1771-2118) with the pieces they call - the jet's density profile
// (RhoISM::evaluateRhoDrhoDrDefault, blastwave_components.h:846-891), the
// adiabatic index (EOSadi, :914-950), lateral spreading (LatSpread, :952-1143),
// the EQS formulas (:36-450), the layer centre (EjectaID2::ctheta,
// ejecta/ejecta_id.h:81-116) and the radiative-loss term
// (ElectronAndRadiation::computeRadiationLoss, microphysics/microphysics.h:
// 749-791, with computePtot :204-219, the limits it recomputes,
// microphysics_base.h:575-605, 736-966, and the analytic synchrotron power,
// analytic_models.h:889-909, 1051-1078). Operation order follows the
// reference; its long double intermediates of rhs_fsrs are double here.
// Paths are relative to the reference's src/ directory.
#ifndef PBAG_RHS_CUH
#define PBAG_RHS_CUH

#include <cmath>

#include "pbag.h"
#include "pbag_const.h"

#ifdef __CUDACC__
#define PBAG_RHD __host__ __device__
#else
#define PBAG_RHD
#endif

namespace pbag {
namespace rhs {

using namespace cgs;
constexpr double kMppme = m_p + m_e;  // CGS::mppme

// error sites (pbag_status.site) of the failures where the reference exits
enum Site {
  kSiteRhsInput = 1,        // Gamma < 1, M2 < 0 or theta < 0 (blastwave.h:1527-1545)
  kSiteTheta = 2,           // theta < 0 while spreading (:1585-1588)
  kSiteDmdr = 3,            // dM/dR < 0 (:1624-1627, 1861-1864)
  kSiteDensity = 4,         // rho < 0 or rho > 1 (blastwave_components.h:883-890)
  kSiteCtheta = 5,          // a non-finite layer centre (ejecta_id.h:96-112)
  kSiteLossInput = 6,       // Eint2 < 0, M2 < 0 or Gamma < 1 before the loss term (blastwave.h:1660-1663)
  kSiteUp = 7,              // U' < 0 or not finite (microphysics_base.h:693-696)
  kSiteParams = 8,          // eps_e, eps_b, eps_t, p, n' or e' invalid (microphysics_base.h:750-773)
  kSiteGammaMin = 9,        // gamma_min or accel_frac invalid (microphysics_base.h:918-934)
  kSiteNonfinite = 10,      // a non-finite derivative (blastwave.h:1715-1742, 2073-2091)
  kSiteDGammaDr = 11,       // |dGamma/dt| > Gamma0 (blastwave.h:1743-1756)
  kSiteSpreadMethod = 12,   // dtheta/dr < 0 in the afterglowpy method (blastwave_components.h:1064-1068)
  kSiteNewtonian = 13,      // p < 2 with the Ayache or Sironi non-relativistic fraction (microphysics_base.h:898-910)
};

struct Err {
  int code = PBAG_OK, site = 0;
  PBAG_RHD bool set(int c, int s) {
    if (code == PBAG_OK) {
      code = c;
      site = s;
    }
    return false;
  }
};

PBAG_RHD inline double beta_g(double g) { return sqrt((g - 1.) * (g + 1.)) / g; }  // EQS::BetaFromGamma
PBAG_RHD inline double mom_g(double g) { return g * beta_g(g); }                    // EQS::MomFromGamma
PBAG_RHD inline double beta_mom(double m) { return m / sqrt(m * m + 1.); }          // EQS::BetaFromMom
PBAG_RHD inline bool finite(double x) { return isfinite(x); }

// EjectaID2::ctheta (ejecta_id.h:81-116)
PBAG_RHD inline double ctheta(double theta, int ilayer, int nlayers, Err& e) {
  double ct = 0.;
  if (ilayer > 0) {
    const double fac0 = (double)ilayer / (double)nlayers;
    const double fac1 = (double)(ilayer + 1) / (double)nlayers;
    if (!finite(sin(theta))) return e.set(PBAG_ERR_NONFINITE, kSiteCtheta), 0.;
    const double x2 = fac1 * sin(theta / 2.);
    const double xx2 = 2. * asin(x2);
    const double x1 = fac0 * sin(theta / 2.);
    const double xx1 = 2. * asin(x1);
    ct = 0.5 * (xx1 + xx2);
    if (!finite(ct)) return e.set(PBAG_ERR_NONFINITE, kSiteCtheta), 0.;
  }
  return ct;
}

// RhoISM::evaluateRhoDrhoDrDefault (blastwave_components.h:846-891): uniform
// ISM for n_ism > 0, else the ejecta / wind / ISM step profile
PBAG_RHD inline void density(const pbag_bw_rhs_pars& P, double R, double& rho, double& drhodr, Err& e) {
  if (P.n_ism > 0.0) {
    rho = P.n_ism * kMppme;
    drhodr = 0.0;
  } else {
    if (P.s < 0 || P.A0 < 0) {
      e.set(PBAG_ERR_PARAM, kSiteDensity);
      return;
    }
    if (R < P.R_ej) {
      rho = P.A0 * pow(P.R_ej, -P.s) * kMppme;
      drhodr = 0.0;
    }
    if (P.R_ej <= R && R < P.R_ism) {
      rho = P.A0 * pow(R, -P.s) * kMppme;
      drhodr = rho * (-P.s / R);
    }
    if (P.R_ism <= R) {
      rho = P.A0 * pow(P.R_ism, -P.s) * kMppme;
      drhodr = 0.0;
    }
  }
  if (rho < 0 || rho > 1.) e.set(PBAG_ERR_NONFINITE, kSiteDensity);
}

// EOSadi::getGammaAdi (blastwave_components.h:920-950)
PBAG_RHD inline double gamma_adi(int method, double Gamma, double beta) {
  if (method == PBAG_EOS_NAVA13) return (4.0 + 1.0 / Gamma) / 3.0;
  const double mom = Gamma * beta;
  const double theta = mom / 3.0 * (mom + 1.07 * mom * mom) / (1.0 + mom + 1.07 * mom * mom);
  const double zz = theta / (0.24 + theta);
  return (5.0 - 1.21937 * zz + 0.18203 * pow(zz, 2.) - 0.96583 * pow(zz, 3.) + 2.32513 * pow(zz, 4.) -
          2.39332 * pow(zz, 5.) + 1.07136 * pow(zz, 6.)) /
         3.0;
}

PBAG_RHD inline double gamma_sh(double Gamma, double adi) {  // EQS::GammaSh
  return (Gamma + 1.0) * (adi * (Gamma - 1.0) + 1.0) / (adi * (2.0 - adi) * (Gamma - 1.0) + 2.0);
}

// LatSpread::getDthetaDr (blastwave_components.h:966-1143)
PBAG_RHD inline double dthetadr(const pbag_bw_rhs_pars& P, double Gamma, double GammaSh, double R, double gammaAdi,
                                double theta, Err& e) {
  const double thC = P.spread_theta_c, th0 = P.spread_theta_b0;
  switch (P.method_spread) {
    case PBAG_SPREAD_ADI: {
      const double vperp = sqrt(gammaAdi * (gammaAdi - 1.0) * (Gamma - 1.0) / (1.0 + gammaAdi * (Gamma - 1.0))) * c_light;
      const double beta = beta_g(Gamma);
      return (theta < P.spread_theta_max) ? cos(theta) * cos(theta) * (vperp / R / Gamma / beta / c_light) : 0.0;
    }
    case PBAG_SPREAD_AA:
      return 1. / (R * pow(Gamma, 1. + P.spread_aa) * pow(theta, P.spread_aa));
    case PBAG_SPREAD_AFGPY: {
      if (thC < 0) return e.set(PBAG_ERR_PARAM, kSiteSpreadMethod), 0.;
      double dThdt = 0.;
      const double Q0 = 2.0, Q = sqrt(2.0) * 3.0;
      const double u = mom_g(Gamma);
      const double bes = 4 * u * Gamma / (4 * u * u + 3);
      const double val = sqrt((2 * u * u + 3) / (4 * u * u + 3));
      const double bew = 0.5 * val * bes / Gamma;
      if ((theta < 0.5 * pi_) && (Q0 * u * thC < 1)) {
        double fac = u * thC * Q < 1.0 ? 1.0 : Q * (1 - Q0 * u * thC) / (Q - Q0);
        if (th0 < thC) fac *= tan(0.5 * th0) / tan(0.5 * thC);
        dThdt = fac * bew * c_light / R;
      }
      if (dThdt < 0.) return e.set(PBAG_ERR_NONFINITE, kSiteSpreadMethod), 0.;
      return dThdt * (1. / bes / c_light);
    }
    case PBAG_SPREAD_OUR: {
      const double Q0 = 2.0, Q = sqrt(2.0) * 3.0;
      const double mom = mom_g(GammaSh);
      const double vperp = sqrt(gammaAdi * (gammaAdi - 1.0) * (Gamma - 1.0) / (1.0 + gammaAdi * (Gamma - 1.0))) * c_light;
      if ((theta < 0.5 * pi_) && (Q0 * mom * thC < 1)) {
        double fac = 1.;
        if (mom * thC * Q >= 1.0) fac = Q * (1. - Q0 * mom * thC) / (Q - Q0);
        if (th0 < thC) fac *= tan(0.5 * th0) / tan(0.5 * thC);
        const double beta = beta_g(GammaSh);
        return vperp / R / GammaSh / beta / c_light * fac;
      }
      return 0.;
    }
    default:
      return 0.;
  }
}

// the spreading rate the RHS uses, with its start condition (blastwave.h:1580-1609)
PBAG_RHD inline double spread_rate(const pbag_bw_rhs_pars& P, const pbag_bw_rhs_state& S, double Gamma, double beta,
                                   double GammaSh, double R, double gammaAdi, double theta, bool check_theta, Err& e) {
  double d = 0.0;
  if ((theta < P.theta_max) && (!S.end_spreading)) {
    if (check_theta && theta < 0) return e.set(PBAG_ERR_NONFINITE, kSiteTheta), 0.;  // rhs_fs only
    switch (P.method_limit_spread) {
      case PBAG_LIMIT_SPREAD_NONE:
        d = dthetadr(P, Gamma, GammaSh, R, gammaAdi, theta, e);
        break;
      case PBAG_LIMIT_SPREAD_GAMMA0_FRAC:
        if (Gamma * beta < P.frac_mom0_spread * P.mom0) d = dthetadr(P, Gamma, GammaSh, R, gammaAdi, theta, e);
        break;
      case PBAG_LIMIT_SPREAD_GAMMA_VAL: {
        const double lim = P.mom_spread > P.frac_mom0_spread * P.mom0 ? P.mom_spread : P.frac_mom0_spread * P.mom0;
        if (Gamma * beta < lim) d = dthetadr(P, Gamma, GammaSh, R, gammaAdi, theta, e);
        break;
      }
      case PBAG_LIMIT_SPREAD_RD:
        if (R > P.Rd) d = dthetadr(P, Gamma, GammaSh, R, gammaAdi, theta, e);
        break;
    }
  }
  return d;
}

// swept-up mass rate (EQS::dmdr, blastwave_components.h:88-99)
PBAG_RHD inline double dmdr(const pbag_bw_rhs_pars& P, double Gamma, double R, double dthetadr_, double theta,
                            double rho) {
  if (P.method_dmdr == PBAG_DMDR_USING_A) {
    const double aa = P.spread_aa;
    const double t1 = (aa < 0) ? 0.0 : sin(theta) / (3.0 * pow(Gamma, 1.0 + aa) * pow(theta, aa));
    const double t2 = (cos(P.theta_a) - cos(theta));
    return 2.0 * pi_ * rho * (t1 + t2) * R * R / P.ncells;
  }
  if (P.method_dmdr == PBAG_DMDR_USING_DTHDR)
    return 2. * pi_ * rho * ((1. - cos(theta)) + (1. / 3.) * sin(theta) * R * dthetadr_) * R * R / P.ncells;
  return 0.;
}

PBAG_RHD inline double gamma_eff(double Gamma, double adi) { return (adi * Gamma * Gamma - adi + 1.0) / Gamma; }
PBAG_RHD inline double dgamma_eff(double Gamma, double adi) { return (adi * Gamma * Gamma + adi - 1.0) / (Gamma * Gamma); }

// EQS::evalElapsedTime (blastwave_components.h:165-174)
PBAG_RHD inline double elapsed_time_rate(double R, double mom, double dthetadr_, bool spread) {
  const double xx = 1. + mom * mom * mom / (sqrt(1. + mom * mom));
  const double beta = beta_mom(mom);
  if (spread) return 1. / (c_light * beta) * sqrt(1. + R * R * dthetadr_ * dthetadr_) - (1. / c_light);
  return 1. / (c_light * xx * (1. + beta));
}

// ElectronAndRadiation::computeRadiationLoss (microphysics.h:749-791): the
// fraction of the shocked energy radiated, from the analytic synchrotron power
// of the shock's limits (computePtot :204-219). Reads the shock's tcomov and
// reads and updates its carried gamma_max and accel_frac members; its t_e
// (set from the member x) enters only z_cool and the useTe cooling factor,
// neither of which reaches the power.
PBAG_RHD inline double radiation_loss(const pbag_bw_mphys& M, double m_tcomov, double& m_gamma_max,
                                      double& m_accel_frac, double dmdR, double dEshdR, double R, double Gamma,
                                      double GammaSh, double gammaAdi, double m, double Eint, double rho, double theta,
                                      double ncells, Err& e) {
  if (dmdR == 0 || dEshdR == 0 || m == 0 || rho == 0) return 0.;
  const double rho2 = (gammaAdi * Gamma + 1.) / (gammaAdi - 1.) * rho;  // EQS::rho2t
  // get_shock_Up (microphysics_base.h:676-698)
  double up = 0.;
  if (!(Eint == 0 || m == 0)) {
    const double V2 = m / rho2;
    const double U_p = Eint / V2;
    const double from_gamma = (GammaSh - 1.) * rho2 * c_light * c_light;
    up = M.method_up == 0 ? U_p : from_gamma;
    if (up < 0 || !finite(up)) return e.set(PBAG_ERR_NONFINITE, kSiteUp), 0.;
  }
  // updateSockProperties(U_p, Gamma, GammaSh, x, t_b, tcomov, rho2/mp, m/mp)
  const double eprime = up;
  const double betaSh = beta_g(GammaSh);
  const double n_prime = rho2 / m_p;
  // EQS::shock_thickness(m, rho2, 0., theta, Gamma, R, ncells)
  const double one_min_costheta = (cos(0.) - cos(theta) / ncells);
  const double thickness = m / (2.0 * pi_ * one_min_costheta * rho2 * Gamma * R * R);
  // computePtot
  double p_tot = 0.;
  bool ok = true;
  // checkParams (microphysics_base.h:736-774)
  if (betaSh < M.beta_min) ok = false;
  if (ok) {
    if (M.eps_e <= 0 || M.eps_b <= 0 || M.eps_t < 0 || M.p <= 0 || n_prime <= 0 || eprime < 0 || !finite(eprime))
      return e.set(PBAG_ERR_PARAM, kSiteParams), 0.;
    const double p = M.p;
    // computeMagneticField
    double B;
    const double U_b_prime = eprime * M.eps_b;
    if (M.method_B == 0)
      B = sqrt(8. * pi_ * U_b_prime);
    else if (M.method_B == 2)
      B = sqrt(32. * pi_ * M.eps_b * (GammaSh - 1.) * (GammaSh + 3. / 4) * n_prime * m_p * (c_light * c_light));
    else
      B = sqrt(9.0 * pi_ * M.eps_b * n_prime * M.mu * m_p) * (betaSh * c_light);
    // computeGammaMax
    double gamma_max = m_gamma_max;
    if (M.method_gamma_max == 0) gamma_max = sqrt(6.0 * pi_ * q_e / sigma_T / B);
    if (!M.ele_analytic && gamma_max > 0.99 * M.gam_hi) gamma_max = 0.99 * M.gam_hi;
    // computeGammaMin(igmUprime)
    const double U_e_prime = eprime * M.eps_e;
    double gamma_min = (p - 2.) / (p - 1.) * U_e_prime / (n_prime * m_e * c_light * c_light);
    double accel = m_accel_frac;
    if (gamma_min < 2.) {
      const double ayache = (pow(gamma_max, 2 - p) - pow(gamma_min - 1., 2. - p)) / (pow(gamma_max, 2. - p) - 1.) *
                            (pow(gamma_max, 1. - p) - 1.) / (pow(gamma_max, 1. - p) - pow(gamma_min - 1., 1. - p));
      const double sironi = (p - 2.0) / (p - 1.0) * M.eps_e * eprime / (n_prime * m_e * c_light * c_light);
      switch (M.method_nonrel) {
        case 0:
          accel = 1;
          break;
        case 1:
          accel = gamma_min;
          break;
        case 2:
          if (p < 2.) return e.set(PBAG_ERR_PARAM, kSiteNewtonian), 0.;
          accel = ayache;
          break;
        default:
          if (p < 2.) return e.set(PBAG_ERR_PARAM, kSiteNewtonian), 0.;
          accel = sironi;
          break;
      }
      accel = accel > 1. ? 1 : accel;
      gamma_min = gamma_min < 1. ? 1 : gamma_min;
    }
    if (!finite(gamma_min) || !finite(accel) || accel < 0) return e.set(PBAG_ERR_NONFINITE, kSiteGammaMin), 0.;
    if (!M.ele_analytic && gamma_min < M.gam_lo) {
      gamma_min = M.gam_lo;
      if (gamma_min > 1e8) return e.set(PBAG_ERR_PARAM, kSiteGammaMin), 0.;
    }
    // computeGammaCool(useTcomov)
    double gamma_c = ((6. * pi_ * m_e * c_light) / (sigma_T * B * B * (m_tcomov)));
    if (gamma_c <= 1.) gamma_c = 1.001;
    if (!M.ele_analytic && gamma_c > gamma_max) gamma_c = gamma_max;
    m_gamma_max = gamma_max;
    m_accel_frac = accel;
    // SynchrotronAnalytic::computeAnalyticSynchJOH06_limits(dmdr / mp)
    const double n_an = dmdR / m_p;
    const double gamToNuFactor = (3.0 / (4.0 * pi_)) * (q_e * B) / (m_e * c_light);
    double nu_m, nu_c, p_max;
    if (gamma_min < gamma_c) {
      const double XpS = 0.06 + 0.28 * p;
      nu_m = XpS * gamma_min * gamma_min * gamToNuFactor;
      nu_c = XpS * gamma_c * gamma_c * gamToNuFactor;
      p_max = 11.17 * (p - 1.0) / (3.0 * p - 1.0) * (0.54 + 0.08 * p) * q_e * q_e * q_e * n_an * B /
              (m_e * c_light * c_light);
    } else {
      const double XpF = 0.455 + 0.08 * p;
      const double phipF = 1.89 - 0.935 * p + 0.17 * (p * p);
      nu_m = XpF * gamma_min * gamma_min * gamToNuFactor;
      nu_c = XpF * gamma_c * gamma_c * gamToNuFactor;
      const double phip = 2.234 * phipF;
      p_max = phip * q_e * q_e * q_e * n_an * B / (m_e * c_light * c_light);
    }
    const double nu_M = 3.0 / (4.0 * pi_) * gamma_max * gamma_max * q_e * B / (m_e * c_light);
    // computeIntegratedAnalyticSynchWSPN99(1e6)
    const double nu0 = 1e6;
    double term0, term1, term2;
    if (nu_m <= nu_c) {
      term0 = (3. / 4.) * pow(1. / nu_m, 1. / 3.) * (pow(nu_m, 4. / 3.) - pow(nu0, 4. / 3.));
      term1 = -1. / (3. - p) * (2 * pow(1. / nu_m, 1. / 2. - p / 2.)) *
              (pow(nu_m, 3. / 2. - p / 2.) - pow(nu_c, 3. / 2. - p / 2.));
      term2 = pow(nu_c / nu_m, -(p - 1.) / 2.) * 2. / (p - 2.) * (nu_c * pow(nu_M, p / 2.) - nu_M * pow(nu_c, p / 2.)) *
              pow(nu_c * nu_M / nu_c, -p / 2.);
    } else {
      term0 = (3. / 4.) * pow(1. / nu_c, 1. / 3.) * (pow(nu_c, 4. / 3.) - pow(nu0, 4. / 3.));
      term1 = -2. / sqrt(1. / nu_c) * (sqrt(nu_c) - sqrt(nu_m));
      term2 = 1. / sqrt(nu_m / nu_c) * 2. / (p - 2.) * (nu_m * pow(nu_M, p / 2.) - nu_M * pow(nu_m, p / 2.)) *
              pow(nu_m * nu_M / nu_m, -p / 2.);
    }
    p_tot = (term0 + term1 + term2) * p_max;
  }
  p_tot *= m_accel_frac;
  p_tot = p_tot > 0. ? p_tot : 0.;
  const double drcomov = thickness * GammaSh;
  const double dt_esc = drcomov / c_light;
  const double dErad2dR = p_tot * dt_esc;
  double eps_rad = dErad2dR / (dEshdR * M.eps_e);
  if (eps_rad < 0. || !finite(eps_rad)) eps_rad = 0.;
  return eps_rad;
}

// BlastWave::rhs_fs (blastwave.h:1515-1768)
PBAG_RHD inline int rhs_fs(const pbag_bw_rhs_pars& P, pbag_bw_rhs_state& S, double* out, int* site) {
  Err e;
  const double* Y = S.Y;
  const double R = Y[PBAG_Y_R], Gamma = Y[PBAG_Y_GAMMA], Eint2 = Y[PBAG_Y_EINT2], theta = Y[PBAG_Y_THETA];
  const double M2 = Y[PBAG_Y_M2];
  if (Gamma < 1 || M2 < 0 || theta < 0) return *site = kSiteRhsInput, PBAG_ERR_NONFINITE;
  const double ct = ctheta(theta, P.ilayer, P.nlayers, e);
  double rho_d = 0., drho_d = 0.;
  density(P, R, rho_d, drho_d, e);
  if (e.code) return *site = e.site, e.code;
  const double rho = rho_d / P.M0;
  const double drhodr = drho_d / P.M0;
  (void)ct;  // the uniform and step profiles do not depend on the angle
  const double beta = beta_g(Gamma);
  const double gammaAdi = gamma_adi(P.method_eos, Gamma, beta);
  const double GammaSh = gamma_sh(Gamma, gammaAdi);
  const double dRshdt = beta_g(GammaSh) * c_light;  // EQS::dRsh_dt
  const double dRdt = beta * c_light;
  const double dthdr = spread_rate(P, S, Gamma, beta, GammaSh, R, gammaAdi, theta, true, e);
  if (e.code) return *site = e.site, e.code;
  const double dM2dR = dmdr(P, Gamma, R, dthdr, theta, rho);
  if (dM2dR < 0.) return *site = kSiteDmdr, PBAG_ERR_NONFINITE;
  double dGammadR = 0.;
  if (P.method_dgdr == PBAG_DGDR_OUR) {
    const double GammaEff = gamma_eff(Gamma, gammaAdi);
    const double dGammaEffdGamma = dgamma_eff(Gamma, gammaAdi);
    const double num = ((Gamma - 1.) * (GammaEff + 1.) * dM2dR - GammaEff * (gammaAdi - 1.) * Eint2 * (dM2dR / M2 - drhodr / rho));
    const double denum = ((1. + M2) + Eint2 * dGammaEffdGamma + GammaEff * (gammaAdi - 1.) * Eint2 / Gamma);
    dGammadR = -num / denum;
  } else {  // EQS::dgdr(1, Gamma, beta, M2, gammaAdi, dM2dR) (blastwave_components.h:103-110)
    const double numerator = -(gammaAdi * (Gamma * Gamma - 1.0) - (gammaAdi - 1.0) * Gamma * beta * beta);
    const double denominator = 1 + M2 * (2.0 * gammaAdi * Gamma - (gammaAdi - 1) * (1. + pow(Gamma, -2.)));
    dGammadR = (numerator / denominator) * dM2dR;
  }
  const double dtcomov_dR = 1.0 / mom_g(Gamma) / c_light;
  const double dEsh2dR = (Gamma - 1.0) * dM2dR;
  const double dlnV2dR = dM2dR / M2 - drhodr / rho - dGammadR / Gamma;
  double dEad2dR = 0.0;
  if (P.adiab_loss) dEad2dR = -(gammaAdi - 1.0) * Eint2 * dlnV2dR;
  double eps_rad = P.eps_rad_fs;
  if (P.eps_rad_fs < 0) {
    if (Eint2 < 0 || M2 < 0 || Gamma < 1) return *site = kSiteLossInput, PBAG_ERR_NONFINITE;
    eps_rad = radiation_loss(P.fs, S.fs_tcomov, S.fs_gamma_max, S.fs_accel_frac, dM2dR * P.M0,
                             dEsh2dR * P.M0 * c_light * c_light, R, Gamma, GammaSh, gammaAdi, M2 * P.M0,
                             Eint2 * P.M0 * c_light * c_light, rho * P.M0, theta, P.ncells, e);
    if (e.code) return *site = e.site, e.code;
  }
  const double dErad2dR = eps_rad * P.fs.eps_e * dEsh2dR;
  const double dEint2dR = dEsh2dR + dEad2dR - dErad2dR;
  const bool spread = P.method_spread != PBAG_SPREAD_NULL;
  const double dttdr = elapsed_time_rate(R, mom_g(Gamma), dthdr, spread);
  if (!finite(dRdt) || !finite(dGammadR) || !finite(dlnV2dR) || !finite(dthdr) || !finite(dEint2dR))
    return *site = kSiteNonfinite, PBAG_ERR_NONFINITE;
  if (dthdr < 0) return *site = kSiteNonfinite, PBAG_ERR_NONFINITE;
  if (fabs(dRdt * dGammadR) > P.Gamma0) return *site = kSiteDGammaDr, PBAG_ERR_NONFINITE;
  out[PBAG_Y_R] = dRdt;
  out[PBAG_Y_RSH] = dRshdt;
  out[PBAG_Y_TT] = dRdt * dttdr;
  out[PBAG_Y_TCOMOV] = dRdt * dtcomov_dR;
  out[PBAG_Y_GAMMA] = dRdt * dGammadR;
  out[PBAG_Y_EINT2] = dRdt * dEint2dR;
  out[PBAG_Y_THETA] = dRdt * dthdr;
  out[PBAG_Y_ERAD2] = dRdt * dErad2dR;
  out[PBAG_Y_ESH2] = dRdt * dEsh2dR;
  out[PBAG_Y_EAD2] = dRdt * dEad2dR;
  out[PBAG_Y_M2] = dRdt * dM2dR;
  return PBAG_OK;
}

// BlastWave::rhs_fsrs (blastwave.h:1771-2118)
PBAG_RHD inline int rhs_fsrs(const pbag_bw_rhs_pars& P, pbag_bw_rhs_state& S, double* out, int* site) {
  Err e;
  const double* Y = S.Y;
  const double R = Y[PBAG_Y_R], Eint2 = Y[PBAG_Y_EINT2], theta = Y[PBAG_Y_THETA], M2 = Y[PBAG_Y_M2];
  double Gamma = Y[PBAG_Y_GAMMA], Eint3 = Y[PBAG_Y_EINT3], M3 = Y[PBAG_Y_M3], deltaR4 = Y[PBAG_Y_DELTAR4];
  if (Gamma < 1.) Gamma = S.first_step ? P.Gamma0 : 1. + 1.e-5;
  if (Eint3 < 0) Eint3 = 0.0;
  if (M3 < 0) {
    if (S.first_step) {
      M3 = 0;
      Eint3 = 0;
      deltaR4 = 0;
    }
  }
  const double beta = beta_g(Gamma);
  // EQS::get_Gamma43 (blastwave_components.h:343-362). The reference divides
  // in long double (the numerator is a double product, the denominator
  // 1 + beta beta0 formed in long double) and keeps Gamma43 in long double;
  // Gamma43 - 1 is ~1e-8 and less while the reverse shock starts, so the
  // quotient is carried here as a double-double (hi + lo, ~106 bits): its hi
  // part is the reference's (double)Gamma43, and Gamma43 - 1 keeps the bits
  // the reference's extended precision keeps.
  const double A43 = Gamma * P.Gamma0 *
                     (1.0 / (P.Gamma0 * P.Gamma0) + 1.0 / (Gamma * Gamma) - 1.0 / (Gamma * Gamma) / (P.Gamma0 * P.Gamma0));
  double Gamma43, g43_lo;
  {
    const double pr = beta * P.beta0, pr_e = fma(beta, P.beta0, -pr);  // exact product
    const double dh = 1.0 + pr;                                          // TwoSum(1, pr)
    const double bb = dh - 1.0;
    const double de = ((1.0 - (dh - bb)) + (pr - bb)) + pr_e;
    const double d_hi = dh + de, d_lo = de - (d_hi - dh);                // denominator, normalised
    const double q1 = A43 / d_hi;
    const double r = fma(-q1, d_hi, A43) - q1 * d_lo;                    // A - q1 d
    const double q2 = r / d_hi;
    Gamma43 = q1 + q2;
    g43_lo = q2 - (Gamma43 - q1);
  }
  if (Gamma43 < 1.) {
    Gamma43 = 1.;
    g43_lo = 0.;
  }
  const double g43m1 = (Gamma43 - 1.0) + g43_lo;  // Gamma43 - 1 (Gamma43 - 1 is exact: Sterbenz)
  const double beta43 = beta_g(Gamma43);
  const double gammaAdi3 = gamma_adi(P.method_eos, Gamma43, beta43);
  const double GammaRsh = gamma_sh(Gamma43, gammaAdi3);
  const double dRshRshdt = beta_g(GammaRsh) * c_light;
  const double ct = ctheta(theta, P.ilayer, P.nlayers, e);
  double rho_d = 0., drho_d = 0.;
  density(P, R, rho_d, drho_d, e);
  if (e.code) return *site = e.site, e.code;
  (void)ct;
  const double rho = rho_d / P.M0;
  const double drhodr = drho_d / P.M0;
  const double dRdt = beta * c_light;
  const double gammaAdi = gamma_adi(P.method_eos, Gamma, beta);
  const double GammaSh = gamma_sh(Gamma, gammaAdi);
  const double dRshdt = beta_g(GammaSh) * c_light;
  const double dthdr = spread_rate(P, S, Gamma, beta, GammaSh, R, gammaAdi, theta, false, e);
  if (e.code) return *site = e.site, e.code;
  const double dM2dR = dmdr(P, Gamma, R, dthdr, theta, rho);
  if (dM2dR < 0.) return *site = kSiteDmdr, PBAG_ERR_NONFINITE;
  double ddeltaR4dR = 0., dM3dR = 0., dlnrho4dR = 0.;
  const double rho4 = 0.;  // never set in the reference: the reverse-shock loss term sees rho = 0
  if ((!S.shut_off) && (Gamma < 0.9999 * P.Gamma0)) {
    const double alpha_of = P.tprompt * P.beta0 * c_light;
    const double b = beta, b0 = P.beta0;
    ddeltaR4dR = (1.0 / (b * b * b * b) - 1.0 / (b0 * b0 * b0 * b0)) / (1.0 / b + 1.0 / b0) / (1.0 / (b * b) + 1.0 / (b0 * b0)) * b0;
    const double rho4_scale_factor = -deltaR4 / alpha_of;
    if (P.exponential_rho4) {
      dM3dR = (1.0 / alpha_of) * ddeltaR4dR * exp(rho4_scale_factor);
      dlnrho4dR = -2.0 / R - ddeltaR4dR / alpha_of;
    } else {
      dM3dR = (1.0 / alpha_of) * ddeltaR4dR;
      dlnrho4dR = -2.0 / R;
    }
  }
  const double dlnrhodr = drhodr / rho;
  // EQS::get_dGammadR_fs_rs (blastwave_components.h:402-433)
  double dGammadR;
  {
    const double G0 = P.Gamma0;
    const double dgamma43dGamma = G0 - (G0 * G0 * Gamma - Gamma) / sqrt(Gamma * Gamma * G0 * G0 - G0 * G0 - Gamma * Gamma + 1.0);
    const double GammaEff3 = gamma_eff(Gamma, gammaAdi3);
    const double dGammaEff3dGamma = gammaAdi3 * (1.0 + 1.0 / (Gamma * Gamma)) -
                                    dgamma43dGamma / 3.0 / Gamma43 * Gamma43 * (Gamma - 1.0 / Gamma) - 1.0 / (Gamma * Gamma);
    const double dGammaEffdGamma = dgamma_eff(Gamma, gammaAdi);
    const double GammaEff = gamma_eff(Gamma, gammaAdi);
    const double f_2 = GammaEff * (gammaAdi - 1.0) * Eint2 / Gamma;
    const double h_2 = GammaEff * (gammaAdi - 1.0) * Eint2 * (dM2dR / M2 - dlnrhodr);
    const double fh_factor3 = GammaEff3 * (gammaAdi3 - 1.0) * Eint3;
    const double f_3 = fh_factor3 / (Gamma43) * dgamma43dGamma;
    double h_3 = 0.0;
    if (Eint3 != 0) h_3 = fh_factor3 * (dM3dR / M3 - dlnrho4dR);
    dGammadR = -((Gamma - 1.0) * (GammaEff + 1.0) * dM2dR + (Gamma - G0 + GammaEff3 * g43m1) * dM3dR - h_2 - h_3) /
               ((M2 + M3) + Eint2 * dGammaEffdGamma + Eint3 * dGammaEff3dGamma + f_2 + f_3);
  }
  if (dGammadR > 0) {
    if (Gamma > P.rs_Gamma0_frac_no_exceed * P.Gamma0) dGammadR = 0.0;
  }
  const double dEsh2dR = (Gamma - 1.0) * dM2dR;
  const double dEsh3dR = g43m1 * dM3dR;
  double dEad2dR = 0.0;
  const double dlnV2dR = dM2dR / M2 - drhodr / rho - dGammadR / Gamma;
  if (P.adiab_loss) dEad2dR = -(gammaAdi - 1.0) * Eint2 * dlnV2dR;
  double dEad3dR = 0.;
  if ((!S.shut_off) && (M3 > 0.0)) {
    const double dlnV3dR = dM3dR / M3 - dlnrho4dR - dGammadR / Gamma;
    if (P.adiab_loss_rs) dEad3dR = -(gammaAdi3 - 1) * Eint3 * dlnV3dR;
  }
  double eps_rad = P.eps_rad_fs;
  if (P.eps_rad_fs < 0) {
    eps_rad = radiation_loss(P.fs, S.fs_tcomov, S.fs_gamma_max, S.fs_accel_frac, dM2dR * P.M0,
                             dEsh2dR * P.M0 * c_light * c_light, R, Gamma, GammaSh, gammaAdi, M2 * P.M0,
                             Eint2 * P.M0 * c_light * c_light, rho * P.M0, theta, P.ncells, e);
    if (e.code) return *site = e.site, e.code;
  }
  const double dErad2dR = eps_rad * P.fs.eps_e * dEsh2dR;
  double eps_rad_rs = P.eps_rad_rs;
  if (P.eps_rad_rs < 0) {
    eps_rad_rs = radiation_loss(P.rs, S.rs_tcomov, S.rs_gamma_max, S.rs_accel_frac, dM3dR * P.M0,
                                dEsh3dR * P.M0 * c_light * c_light, R, Gamma, GammaRsh, gammaAdi3, M3 * P.M0,
                                Eint3 * P.M0 * c_light * c_light, rho4 * P.M0, theta, P.ncells, e);
    if (e.code) return *site = e.site, e.code;
  }
  const double dErad3dR = eps_rad_rs * P.rs.eps_e * dEsh3dR;
  const double dEint2dR = dEsh2dR + dEad2dR - dErad2dR;
  const double dEint3dR = dEsh3dR + dEad3dR - dErad3dR;
  const double dtcomov_dR = 1.0 / beta / Gamma / c_light;
  const bool spread = P.method_spread != PBAG_SPREAD_NULL;
  const double dttdr = elapsed_time_rate(R, Gamma * beta, dthdr, spread);
  if (!finite(dRdt) || !finite(dGammadR) || !finite(dlnV2dR) || !finite(dthdr))
    return *site = kSiteNonfinite, PBAG_ERR_NONFINITE;
  out[PBAG_Y_R] = dRdt;
  out[PBAG_Y_RSH] = dRshdt;
  out[PBAG_Y_TT] = dRdt * dttdr;
  out[PBAG_Y_TCOMOV] = dRdt * dtcomov_dR;
  out[PBAG_Y_GAMMA] = dRdt * dGammadR;
  out[PBAG_Y_RRSH] = dRshRshdt;
  out[PBAG_Y_EINT2] = dRdt * dEint2dR;
  out[PBAG_Y_EINT3] = dRdt * dEint3dR;
  out[PBAG_Y_THETA] = dRdt * dthdr;
  out[PBAG_Y_ERAD2] = dRdt * dErad2dR;
  out[PBAG_Y_ERAD3] = dRdt * dErad3dR;
  out[PBAG_Y_ESH2] = dRdt * dEsh2dR;
  out[PBAG_Y_ESH3] = dRdt * dEsh3dR;
  out[PBAG_Y_EAD2] = dRdt * dEad2dR;
  out[PBAG_Y_EAD3] = dRdt * dEad3dR;
  out[PBAG_Y_M2] = dRdt * dM2dR;
  out[PBAG_Y_M3] = dRdt * dM3dR;
  out[PBAG_Y_DELTAR4] = dRdt * ddeltaR4dR;
  return PBAG_OK;
}

PBAG_RHD inline int rhs_one(const pbag_bw_rhs_pars& P, pbag_bw_rhs_state& S, double* out, int* site) {
  if (P.type == PBAG_BW_FS) return rhs_fs(P, S, out, site);
  if (P.type == PBAG_BW_FSRS) return rhs_fsrs(P, S, out, site);
  *site = 0;
  return PBAG_ERR_UNSUPPORTED;
}

}  // namespace rhs
}  // namespace pbag

#endif
