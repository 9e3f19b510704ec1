// pbag_oracle.cpp - FP64 CPU restatement of the reference's comoving-radiation
// step. TEST INFRASTRUCTURE: the checker for the GPU path in tests/, smoke()
// and the CPU-baseline leg of bench.py; never linked by the product.
//
// It follows, line by line, the reference sources cited beside each function
// (paths relative to the reference's src/ directory). Floating-point operations
// are written in the reference's order so that results agree to rounding.
//
// One intentional definition: the reference reads freqs[F] (one past the end)
// in computeSSCSpectrum (microphysics/numeric_model.h:269-272); here that
// value is the next point of the logspace grid, freq[F-1]*base.
#include "pbag_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// utilitites/utils.h:18-60 (CGS constants)
constexpr double c_light = 2.99792458e10;
constexpr double pi_ = 3.141592653589793;
constexpr double cgs2mJy = 1.e26;  // utils.h:40
constexpr double m_p = 1.6726e-24;
constexpr double m_e = 9.1094e-28;
constexpr double q_e = 4.803204e-10;
constexpr double sigma_T = 6.6524e-25;
constexpr double h_pl = 6.6260755e-27;
constexpr double mec2 = 8.187105649650028e-07;
const double h_by_mec2 = h_pl / m_e / c_light / c_light;

// --- synchrotron kernel functions (microphysics/kernels.h) -----------------

inline double nu_crit(double B, double gam) {  // kernels.h:194-197
  return (3. * q_e * B * gam * gam) / (4. * M_PI * m_e * c_light);
}
inline double nu_larmor(double B) {  // kernels.h:199-202
  return (3. * q_e * B) / (2. * pi_ * m_e * c_light);
}

double cheb_eval(const double* coeff, int order, double a, double b, double x) {  // kernels.h:158-173
  double d = 0.0, dd = 0.0;
  double y = (2.0 * x - a - b) / (b - a);
  double y2 = 2.0 * y;
  for (int j = order; j > 0; j--) {
    double temp = d;
    d = y2 * d - dd + coeff[j];
    dd = temp;
  }
  return y * d - dd + 0.5 * coeff[0];
}

// Chebyshev series of the synchrotron function F(x) used by synchGSL
// (kernels.h:213-279): the published GSL "synchrotron_1" expansions.
const double syn1_cs[13] = {30.364682982501076273, 17.079395277408394574, 4.560132133545072889,
                            0.549281246730419979, 0.372976075069301172e-01, 0.161362430201041242e-02,
                            0.481916772120371e-04, 0.10512425288938e-05, 0.174638504670e-07,
                            0.22815486544e-09, 0.240443082e-11, 0.2086588e-13, 0.15167e-15};
const double syn1a_cs[23] = {2.1329305161355000985, 0.741352864954200240e-01, 0.86968099909964198e-02,
                             0.11703826248775692e-02, 0.1645105798619192e-03, 0.240201021420640e-04,
                             0.35827756389389e-05, 0.5447747626984e-06, 0.838802856196e-07,
                             0.13069882684e-07, 0.2053099071e-08, 0.325187537e-09, 0.517914041e-10,
                             0.83002988e-11, 0.13352728e-11, 0.2159150e-12, 0.349967e-13,
                             0.56994e-14, 0.9291e-15, 0.152e-15, 0.249e-16, 0.41e-17, 0.7e-18};
const double syn2_cs[12] = {0.4490721623532660844, 0.898353677994187218e-01, 0.81044573772151290e-02,
                            0.4261716991089162e-03, 0.147609631270746e-04, 0.3628633615300e-06,
                            0.66634807498e-08, 0.949077166e-10, 0.1079125e-11, 0.10022e-13, 0.77e-16,
                            0.5e-18};

double synch_gsl(double B, double nu, double gam) {  // kernels.h:211-342
  double ec = 1.5 * B / 4.14e13;
  double en = nu * h_by_mec2;
  double x = en / (ec * gam * gam);
  const double c0 = M_PI / 1.7320508075688772;
  const double c01 = 0.2257913526447274323630976;
  const double cond1 = 2 * M_SQRT2 * 1.4901161193847656e-08;
  const double cond3 = -8.0 * (-7.0839641853226408e02) / 7.0;
  double result;
  if (x < cond1) {
    double z = std::pow(x, 1.0 / 3.0);
    double cf = 1 - 8.43812762813205e-01 * z * z;
    result = 2.14952824153447863671 * z * cf;
  } else if (x <= 4.0) {
    double px = std::pow(x, 1.0 / 3.0);
    double px11 = std::pow(px, 11.);
    double t = x * x / 8.0 - 1.0;
    double r1 = cheb_eval(syn1_cs, 12, -1.0, 1.0, t);
    double r2 = cheb_eval(syn2_cs, 11, -1.0, 1.0, t);
    result = px * r1 - px11 * r2 - c0 * x;
  } else if (x < cond3) {
    double t = (12.0 - x) / (x + 4.0);
    double r1 = cheb_eval(syn1a_cs, 22, -1.0, 1.0, t);
    result = std::sqrt(x) * r1 * std::exp(c01 - x);
  } else {
    result = 0.0;
  }
  result *= std::sqrt(3.) * std::pow(q_e, 3.) * B / mec2;
  return result;
}

double synch_bessel(double B, double nu, double gam) {  // kernels.h:396-412
  double t = nu / nu_crit(B, gam);
  double res;
  try {
    double k43 = std::cyl_bessel_k(4. / 3., t);
    double k13 = std::cyl_bessel_k(1. / 3., t);
    res = 2 * t * t * (k43 * k13 - 3. / 5 * t * (k43 * k43 - k13 * k13));
  } catch (...) {
    res = 0;
  }
  res *= std::sqrt(3.) * std::pow(q_e, 3.) * B / (m_e * c_light * c_light);
  return res;
}

// Aharonian+2010 eq. D7 fit to the angle-averaged synchrotron function
// (kernels.h:420-427, 463-469).
inline double aharonian_R(double x) {
  double t1n = 1.808 * std::pow(x, 1. / 3.);
  double t1d = std::sqrt(1 + 3.4 * std::pow(x, 2. / 3.));
  double t2n = 1. + 2.21 * std::pow(x, 2. / 3.) + 0.347 * std::pow(x, 4. / 3.);
  double t2d = 1. + 1.353 * std::pow(x, 2. / 3.) + 0.217 * std::pow(x, 4. / 3.);
  return t1n / t1d * t2n / t2d * std::exp(-x);
}

double cyc_synch(double B, double nu, double gam) {  // kernels.h:414-437 ("CSYN")
  double em;
  if (gam > 2.) {
    double x = nu / nu_crit(B, gam);
    em = aharonian_R(x);
    em *= std::sqrt(3.) * std::pow(q_e, 3.) * B / mec2;
  } else {
    double x = nu / nu_larmor(B);
    double psq = gam * gam - 1.;
    em = (2. * psq) / (1. + 3. * psq) * std::exp((2. * (1. - x)) / (1. + 3. * psq));
    em *= std::sqrt(3.) * std::pow(q_e, 3.) * B / mec2;
  }
  return em;
}

double synch_dermer(double B, double nu, double gam) {  // kernels.h:451-473
  double x = nu / nu_crit(B, gam);
  double res = aharonian_R(x);
  res *= std::sqrt(3.) * std::pow(q_e, 3.) * B / (m_e * c_light * c_light);
  return res;
}

// Blumenthal & Gould isotropic Compton kernel, Nava form (kernels.h:96-117).
double ssc_nava(double nu, double gam, double nu_tilde) {
  double en = nu * h_by_mec2;
  double en_t = nu_tilde * h_by_mec2;
  double K = 0.;
  if (en_t / (4. * gam * gam) < en && en <= en_t)
    K = (en / en_t) - (1. / (4. * gam * gam));
  else if (en_t < en && en < (4. * gam * gam * en_t / (1. + 4. * gam * en_t))) {
    double q = en / (4. * gam * en_t * (gam - en));
    K = 2. * q * std::log(q) + (1. + 2. * q) * (1. - q) +
        .5 * (1. - q) * std::pow(4. * gam * en_t * q, 2.) / (1. + 4. * gam * en_t * q);
  } else
    K = 0;
  return K;
}

// Pair-production rate kernel (numeric_model.h:295-303)
inline double pp_R(double nu, double nu_t) {
  double x = nu * nu_t;
  double varbl = x * (h_pl / m_e / c_light / c_light) * (h_pl / m_e / c_light / c_light);
  double res = 0.;
  if (varbl - 1 > 0) res = 0.652 * c_light * sigma_T * (varbl * varbl - 1) * std::log(varbl) / (varbl * varbl * varbl);
  return res;
}

// computePPinjection (numeric_model.h:305-340): pairs injected at the electron
// energy of photon frequency nu from the photon density n[F]
double pp_injection(const std::vector<double>& nu_g, int F, double nu, const std::vector<double>& n) {
  size_t idx = F - 1;
  for (int i = 0; i < F - 1; i++)
    if ((nu_g[i] < nu) && (nu_g[i + 1] >= nu)) {
      idx = i;
      break;
    }
  const double c4 = c_light * c_light * c_light * c_light;
  double integ = 0;
  for (int i = 0; i < F - 1; i++) {
    if (nu_g[i] * nu * h_pl * h_pl / m_e / m_e / c4 < 1.) continue;
    integ += n[i] * pp_R(nu, nu_g[i]) * (nu_g[i + 1] - nu_g[i]);
  }
  double fac = 4. * m_e * (c_light * c_light) / h_pl;
  return fac * n[idx] * integ;  // Eq. 51 of Miceli & Nava
}

// microphysics/microphysics.h:11-58, METHOD_TAU::iAPPROX branch
inline double intensity_approx(double em, double dtau) {
  if (dtau == 0) return em;
  double u = 1. / 2. + std::exp(-dtau) / dtau - (1 - std::exp(-dtau)) / (dtau * dtau);
  return dtau > 1.e-3 ? em * (3. * u / dtau) : em;
}

typedef double (*syn_fn)(double, double, double);
syn_fn pick_syn(int method) {
  switch (method) {
    case PBAG_SYN_DER09: return synch_dermer;
    case PBAG_SYN_GSL: return synch_gsl;
    case PBAG_SYN_BESSEL: return synch_bessel;
    default: return cyc_synch;
  }
}

// Shared read-only tables for one grid (the reference's CommonTables entry).
struct Tables {
  int G = 0, F = 0;
  std::vector<double> e, half, dg, dgb, nu;  // gamma grid, half grid, delta_grid[G+1], delta_grid_bar[G], nu[F+1]
  std::vector<double> K, Kint;               // SSC kernel [F][G][F], its integral [G][F]
  bool has_ssc = false;
};

void build_tables(const pbag_grid_desc* g, bool ssc, Tables& t) {
  int G = g->ngam, F = g->nfreq;
  t.G = G;
  t.F = F;
  t.e.assign(G, 0.);
  t.nu.assign(F + 1, 0.);
  orc_build_grids(g, t.e.data(), t.nu.data());
  // base_state.h:229-250
  double step = std::exp(std::log(g->gam2) / (double)G);
  double sp1 = step + 1.0;
  t.half.assign(G - 1, 0.);
  for (int i = 0; i < G - 1; ++i) t.half[i] = .5 * t.e[i] * sp1;
  t.dg.assign(G + 1, 0.);
  for (int i = 0; i < G - 1; ++i) t.dg[i + 1] = t.e[i + 1] - t.e[i];
  t.dg[0] = t.e[0] * (1 - 1.0 / step);
  t.dg[G] = t.e[G - 1] * (step - 1);
  t.dgb.assign(G, 0.);
  for (int i = 0; i < G; ++i) t.dgb[i] = (t.dg[i] + t.dg[i + 1]) / 2.;
  if (ssc) {
    t.K.assign((size_t)F * G * F, 0.);
    t.Kint.assign((size_t)G * F, 0.);
    orc_ssc_kernel(t.e.data(), G, t.nu.data(), F, t.K.data(), t.Kint.data());
    t.has_ssc = true;
  }
}

// Per-blastwave state and scratch (ElectronAndRadiation members).
struct BW {
  std::vector<double> f, dfde, tmp, gsyn, gadi, gssc, heat, src, a, b, c, d, cp, dp;
  std::vector<double> ker, sj, sa, cj, n, tj, ta, ti, spe, ppa;
  double dr_comov = 0, vol = 0, N = -1;
  bool init = false, syn_seen = false;
  void alloc(int G, int F) {
    for (auto* v : {&f, &dfde, &tmp, &gsyn, &gadi, &gssc, &heat, &src, &a, &b, &c, &d, &cp, &dp, &spe})
      v->assign(G, 0.);
    ker.assign((size_t)F * G, 0.);
    for (auto* v : {&sj, &sa, &cj, &n, &tj, &ta, &ti, &ppa}) v->assign(F, 0.);
  }
};

struct Err {
  int code = PBAG_OK;
};

// microphysics.h:228-280 powerLawElectronDistributionAnalytic
bool power_law(const Tables& T, double gm, double gc, double gM, double p, double n_inj, double* N) {
  bool ok = true;
  if (gm > gc) {
    double Kf = n_inj / (std::pow(gm, 1. - p) * (1. / gc - 1. / gm) + 1. / p * (std::pow(gm, -p) - std::pow(gM, -p)));
    for (int i = 0; i < T.G; i++) {
      double g = T.e[i];
      if ((gc <= g) && (g < gm))
        N[i] = Kf * std::pow(gm, 1. - p) * std::pow(g, -2.);
      else if ((gm < g) && (g <= gM))
        N[i] = Kf * std::pow(g, -p - 1.);
      if (!std::isfinite(N[i]) || N[i] < 0.) ok = false;
    }
  } else {
    double Ks = n_inj / ((1. / (1. - p)) * (std::pow(gc, 1. - p) - std::pow(gm, 1. - p)) -
                         gc / p * (std::pow(gM, -p) - std::pow(gc, -p)));
    for (int i = 0; i < T.G; ++i) {
      double g = T.e[i];
      if ((gm <= g) && (g < gc))
        N[i] = Ks * std::pow(g, -p);
      else if ((gc <= g) && (g <= gM))
        N[i] = Ks * gc * std::pow(g, -p - 1.);
      if (!std::isfinite(N[i]) || N[i] < 0.) ok = false;
    }
  }
  return ok;
}

// numeric_model.h:753-801 setHeatCoolTerms (dispersion_term = 0)
bool heat_cool(const Tables& T, BW& w, double B, double dlnVdt, bool ssc, int inner) {
  const int G = T.G, F = T.F;
  bool ok = true;
  const double const_syn = sigma_T / (6. * M_PI * m_e * c_light);
  const double const_ssc = 3. / 4. * h_pl * sigma_T / m_e / c_light;
  (void)inner;
#pragma omp parallel for num_threads(inner) if (inner > 1) reduction(&& : ok)
  for (int i = 0; i < G - 1; i++) {
    double gam = T.half[i];
    w.gsyn[i] = const_syn * B * B * gam * gam;
    w.gadi[i] = dlnVdt * (gam * gam - 1.) / (3. * gam);
    if (ssc) {
      double res = 0;
      for (int j = 0; j < F - 1; j++)
        res += w.n[j] / T.nu[j] * (T.nu[j + 1] - T.nu[j]) * T.Kint[(size_t)i * F + j];
      w.gssc[i] = const_ssc * res / gam / gam;
    }
    w.heat[i] = w.gsyn[i] + w.gadi[i] + w.gssc[i];
    if (!std::isfinite(w.heat[i])) ok = false;
  }
  w.heat[G - 1] = 0.;
  return ok;
}

// numeric_model.h:539-675 setupVectors with dispersion = delta_j = escape = 0
void setup_vectors(const Tables& T, BW& w, double dt) {
  const int G = T.G;
  for (int k = 0; k < G; ++k) w.a[k] = w.b[k] = w.c[k] = 0.;
  for (int k = G - 2; k > 0; k--) {
    double odgb = 1.0 / T.dgb[k];
    double Bf = w.heat[k], Bb = w.heat[k - 1];
    w.a[k] = odgb * (0. - 0. * Bb);              // compute_n_j_minus_one_term, C=0, delta=0
    w.b[k] = -odgb * ((0. + 0.) + 1. * Bb - 0. * Bf);  // compute_n_j
    w.c[k] = odgb * (1. * Bf + 0.);               // compute_n_j_plus_one
  }
  {  // right boundary
    double odgb = 1.0 / T.dgb[G - 1];
    double Hl = w.heat[G - 1];
    w.a[G - 1] = odgb * (0. - 0. * Hl);
    w.b[G - 1] = -odgb * ((0. + 0.) + 1. * Hl - 0.);
    w.c[G - 1] = 0.;
  }
  {  // left boundary
    double odgb = 1.0 / T.dgb[0];
    w.a[0] = 0.0;
    w.b[0] = -odgb * ((0. + 0.) + 0. * 0. - 0. * w.heat[0]);
    w.c[0] = odgb * (1. * w.heat[0] + 0.);
  }
  for (int i = 0; i < G; i++) {
    w.a[i] *= -dt;
    w.b[i] = (1. - w.b[i] * dt) + 0. * dt;
    w.c[i] *= -dt;
  }
}

// numeric_model.h:682-708 solve -> tridiagonal_solver (:19-43)
bool solve(const Tables& T, BW& w, double dt) {
  const int G = T.G;
  bool ok = true;
  for (int i = 0; i < G; i++) {
    w.d[i] = w.f[i] + w.src[i] * dt;
    if (!std::isfinite(w.f[i]) || w.f[i] < 0.) ok = false;
  }
  for (int i = 0; i < G; i++) {
    w.cp[i] = w.c[i] / w.b[i];
    w.dp[i] = w.d[i] / w.b[i];
  }
  double sum = 0;
  for (int i = 0; i < G; i++) sum += w.a[i];
  if (sum > 0)
    for (int i = 1; i < G; i++) {
      double bm = w.b[i] - w.a[i] * w.cp[i - 1];
      w.cp[i] = w.c[i] / bm;
      w.dp[i] = (w.d[i] - w.a[i] * w.dp[i - 1]) / bm;
    }
  w.f[G - 1] = w.dp[G - 1];
  for (int j = G - 2; j > -1; j--) w.f[j] = w.dp[j] - w.cp[j] * w.f[j + 1];
  return ok;
}

// microphysics.h:359-489 evaluateElectronDistributionNumericMixed
int evolve(const Tables& T, const pbag_shock_params& P, BW& w, const pbag_step_rec& r, int flags,
           int inner) {
  const int G = T.G;
  if ((r.B <= 0) || (r.gamma_min < 1.) || (r.gamma_max <= 1.) || (r.gamma_min >= r.gamma_max) ||
      (r.accel_frac > 1.))
    return PBAG_ERR_PARAM;
  w.dr_comov = r.dr;
  double N_tot = r.m_p1 / m_p;
  std::fill(w.tmp.begin(), w.tmp.end(), 0.);
  if (!power_law(T, r.gamma_min, r.gamma_c, r.gamma_max, P.p, N_tot, w.tmp.data())) return PBAG_ERR_NONFINITE;
  double dt = r.tc_p1 - r.tc;
  double volume = r.m / r.rho;
  double volume_p1 = r.m_p1 / r.rho_p1;
  double dlnVdt = P.adi_on ? 1. / dt * (1. - volume / volume_p1) : 0.;
  if ((!std::isfinite(dlnVdt)) || (dlnVdt < 0)) return PBAG_ERR_DLNVDT;
  // substeps (microphysics.h:412-435)
  double dlog_gam = (T.e[1] - T.e[0]) / T.e[0];
  double dts = sigma_T * r.gamma_max * r.B * r.B / (6. * M_PI * m_e * c_light);
  double dta = (r.gamma_max * r.gamma_max - 1.) / (3. * r.gamma_max * r.gamma_max) * dlnVdt;
  double delta_t = dlog_gam / (dts + dta);
  size_t n_sub;
  const size_t max_sub = (size_t)P.max_substeps;
  if (delta_t >= dt / 1.) {
    delta_t = dt / 1.;
    n_sub = 1;
  } else if (delta_t < dt / (double)max_sub) {
    delta_t = dt / (double)max_sub;
    n_sub = max_sub;
  } else
    n_sub = (size_t)(dt / delta_t);
  w.vol = volume;
  if (P.ele_method == PBAG_ELE_MIX || r.gamma_min <= 2) {
    for (int i = 0; i < G; i++) w.f[i] = w.tmp[i];
    return PBAG_OK;
  }
  w.N = (r.m_p1 - r.m) / m_p / dt;
  // setSourceFunction (numeric_model.h:717-724)
  double index = -P.p;
  double norm = (1 + index) / (std::pow(r.gamma_max, index + 1) - std::pow(r.gamma_min, index + 1));
  for (int i = 0; i < G; i++)
    w.src[i] = ((T.e[i] > r.gamma_min) && (T.e[i] <= r.gamma_max)) ? w.N * norm * std::pow(T.e[i], index) : 0.;
  const bool ssc = P.ssc_on && T.has_ssc;
  // addPPSource (numeric_model.h:727-733): pairs from the photon density of
  // the previous radiating step join the source (microphysics.h:457-459)
  if (ssc && P.pp_on)
    for (int i = 0; i < G; i++) {
      double nu1 = 2. * T.e[i] * m_e * c_light * c_light / h_pl;
      w.src[i] += pp_injection(T.nu, T.F, nu1, w.n) * w.vol;
    }
  if (flags & ORC_HOIST_HEATING) {
    if (!heat_cool(T, w, r.B, dlnVdt, ssc, inner)) return PBAG_ERR_NONFINITE;
    setup_vectors(T, w, delta_t);
  }
  for (size_t s = 0; s < n_sub; s++) {
    if (!(flags & ORC_HOIST_HEATING)) {
      if (!heat_cool(T, w, r.B, dlnVdt, ssc, inner)) return PBAG_ERR_NONFINITE;
      setup_vectors(T, w, delta_t);
    }
    if (!solve(T, w, delta_t)) return PBAG_ERR_NONFINITE;
  }
  return PBAG_OK;
}

// base_state.h:482-536 dfdx (acc=1), stateful: only entries with f>0 are written
void dfdx(const double* x, const double* f, double* df, int n) {
  for (int i = 1; i < n - 1; i++)
    if (f[i] > 0) {
      double dx = x[i] - x[i - 1];
      df[i] = 0.5 * (f[i + 1] - f[i - 1]) / dx;
    }
  if (f[0] > 0) df[0] = -1.5 * f[0] + 2. * f[1] - 0.5 * f[2];
  int i = n - 1;
  if (f[i] > 0) df[i] = 1.5 * f[i] - 2. * f[i - 1] + 0.5 * f[i - 2];
}

// microphysics.h:492-633 computeRadiationNumericMixed (+ storeDenseOutput)
int radiate(const Tables& T, const pbag_shock_params& P, BW& w, const pbag_step_rec& r, size_t row,
            pbag_outputs* out, int inner) {
  const int G = T.G, F = T.F;
  const double B = r.B;
  if (B < 0) return PBAG_ERR_PARAM;
  syn_fn fn = pick_syn(P.syn_method);
  // kernels.h:528-538 evalSynKernel
  for (int k = 0; k < F; k++)
    for (int j = 0; j < G; j++) w.ker[(size_t)k * G + j] = fn(B, T.nu[k], T.e[j]);
  // numeric_model.h:148-184 computeSynSpectrum
  std::fill(w.sj.begin(), w.sj.end(), 0.);
  bool ok = true;
#pragma omp parallel for num_threads(inner) if (inner > 1) reduction(&& : ok)
  for (int i = 0; i < F - 1; i++) {
    double res = 0.;
    for (int j = 0; j < G - 1; j++) res += w.ker[(size_t)i * G + j] * w.f[j] * (T.e[j + 1] - T.e[j]);
    w.sj[i] = res;
    if (!std::isfinite(res) || res < 0.) ok = false;
  }
  if (!ok) return PBAG_ERR_NONFINITE;
  // numeric_model.h:191-238 computeSSA
  if (P.ssa_on) {
    for (int i = 0; i < G; i++) w.tmp[i] = w.f[i] / T.e[i] / T.e[i];
    dfdx(T.e.data(), w.tmp.data(), w.dfde.data(), G);
    std::fill(w.sa.begin(), w.sa.end(), 0.);
#pragma omp parallel for num_threads(inner) if (inner > 1)
    for (int i = 0; i < F; i++) {
      for (int j = 0; j < G - 1; j++)
        w.sa[i] += T.e[j] * T.e[j] * (T.e[j + 1] - T.e[j]) * w.dfde[j] * w.ker[(size_t)i * G + j];
      w.sa[i] *= -1. / (8. * M_PI * m_e * T.nu[i] * T.nu[i]);
      w.sa[i] = std::abs(w.sa[i]);
      if (!std::isfinite(w.sa[i])) w.sa[i] = 1e99;
    }
  }
  // numeric_model.h:247-285 computeSSCSpectrum (photon field of the previous step)
  const bool ssc = P.ssc_on && T.has_ssc;
  if (ssc) {
    std::fill(w.cj.begin(), w.cj.end(), 0.);
#pragma omp parallel for num_threads(inner) if (inner > 1)
    for (int i = 0; i < F; i++) {
      std::vector<double> spe(G - 1, 0.);
      const double* Ki = T.K.data() + (size_t)i * G * F;
      for (int j = 0; j < G - 1; j++)
        for (int k = 0; k < F; k++)
          spe[j] += 3. / 4. * sigma_T * c_light / (T.e[j] * T.e[j]) * w.n[k] / T.nu[k] * (T.nu[k + 1] - T.nu[k]) *
                    Ki[(size_t)j * F + k];
      double acc = 0.;
      for (int j = 0; j < G - 1; j++) acc += w.f[j] * h_pl * T.nu[i] * spe[j] * (T.e[j + 1] - T.e[j]);
      w.cj[i] = acc;
    }
  }
  // computePPabsorption (numeric_model.h:343-356) from the previous photon density
  const bool pp = P.pp_on && ssc;
  if (pp)
    for (int i = 0; i < F; i++) {
      double integ = 0;
      for (int j = 0; j < F - 1; j++) integ += pp_R(T.nu[i], T.nu[j]) * w.n[j] * (T.nu[j + 1] - T.nu[j]);
      w.ppa[i] = integ / c_light;
    }
  // new photon density (microphysics.h:516-523)
  const bool num = P.ele_method == PBAG_ELE_NUMERIC;
  double Tesc = w.dr_comov / c_light;
  double fac = Tesc / w.vol;
  for (int i = 0; i < F; i++) w.n[i] = w.sj[i] * fac / (h_pl * T.nu[i]);
  if (num && ssc)
    for (int i = 0; i < F; i++) w.n[i] += w.cj[i] * fac / (h_pl * T.nu[i]);
  for (int i = 0; i < F; i++) w.tj[i] = w.sj[i];
  if (num && ssc)
    for (int i = 0; i < F; i++) w.tj[i] += w.cj[i];
  for (int i = 0; i < F; i++) w.ta[i] = w.sa[i];
  // total number of electrons (microphysics.h:556-563)
  double n_ele = 0.;
  for (int i = 0; i < G - 1; i++) n_ele += w.f[i] * (T.e[i + 1] - T.e[i]);
  if (n_ele <= 0) return PBAG_ERR_NELE;
  // pair-production attenuation of the total emissivity (microphysics.h:565-574)
  if (num && pp)
    for (int i = 0; i < F; i++) {
      double tau_pp = w.ppa[i] * w.dr_comov;
      double atten = (-std::expm1(-tau_pp) / tau_pp);
      if (tau_pp > 0.) w.tj[i] = w.tj[i] * atten;
    }
  // normalisation (microphysics.h:577-586)
  const double acc = r.accel_frac, np = r.n_prime;
  for (int i = 0; i < F; i++) {
    w.ta[i] = w.ta[i] / n_ele * acc * np;
    double dtau = w.ta[i] * w.dr_comov;
    w.ti[i] = intensity_approx(w.tj[i] * acc, dtau);
    w.tj[i] = w.tj[i] * acc / n_ele;
    if (!std::isfinite(w.tj[i]) || w.tj[i] < 0.) return PBAG_ERR_NONFINITE;
  }
  auto put = [&](double* dst, const std::vector<double>& v, int n) {
    if (dst) std::memcpy(dst + row * n, v.data(), sizeof(double) * n);
  };
  put(out->j_all, w.tj, F);
  put(out->a_all, w.ta, F);
  put(out->f_all, w.n, F);
  put(out->i_all, w.ti, F);
  // storeDenseOutput (microphysics.h:602-633)
  if (out->syn_j_all || out->syn_a_all || out->syn_i_all) {
    std::vector<double> j(F), a(F), in(F);
    for (int i = 0; i < F; i++) {
      j[i] = w.sj[i] * acc;
      a[i] = w.sa[i] / n_ele * acc * np;
      in[i] = intensity_approx(j[i], a[i] * w.dr_comov);
    }
    put(out->syn_j_all, j, F);
    put(out->syn_a_all, a, F);
    put(out->syn_i_all, in, F);
  }
  if (ssc && (out->ssc_j_all || out->ssc_i_all)) {
    std::vector<double> j(F), in(F);
    for (int i = 0; i < F; i++) {
      j[i] = w.cj[i] * acc;
      // ssc.a is the pair-production absorption (0 without it, then I = j)
      double a = pp ? w.ppa[i] / n_ele * acc * np : 0.;
      in[i] = intensity_approx(j[i], a * w.dr_comov);
    }
    put(out->ssc_j_all, j, F);
    put(out->ssc_i_all, in, F);
  }
  put(out->ele_f_all, w.f, G);
  put(out->gdot_syn_all, w.gsyn, G);
  put(out->gdot_adi_all, w.gadi, G);
  put(out->gdot_ssc_all, w.gssc, G);
  if (out->syn_j_all) {  // microphysics.h:627-631: exit if the syn history sums to 0 after step 0
    for (int i = 0; i < F; i++)
      if (w.sj[i] != 0.) w.syn_seen = true;
    if (!w.syn_seen && row > 0) return PBAG_ERR_NONFINITE;
  }
  return PBAG_OK;
}

// microphysics.h:347-357 initializeElectronDistribution
int initialize(const Tables& T, const pbag_shock_params& P, BW& w, const pbag_step_rec& r) {
  w.dr_comov = r.dr;
  w.vol = r.m_p1 / r.rho_p1;
  if (!power_law(T, r.gamma_min, r.gamma_c, r.gamma_max, P.p, r.m_p1 / m_p, w.f.data())) return PBAG_ERR_NONFINITE;
  w.init = true;
  for (int i = 0; i < T.G - 1; i++) w.f[i] *= r.accel_frac;
  return PBAG_OK;
}

int run_one(const Tables& T, const pbag_shock_params& P, const pbag_step_rec* recs, size_t nr, pbag_outputs* o,
            int flags, int inner, int* fail_step) {
  BW w;
  w.alloc(T.G, T.F);
  for (size_t it = 0; it < nr; ++it) {
    const pbag_step_rec& r = recs[it];
    if (r.mode == PBAG_SKIP) continue;
    int rc;
    // blastwave_radiation.h:1160-1175: the first valid step initialises
    if (!w.init)
      rc = initialize(T, P, w, r);
    else
      rc = evolve(T, P, w, r, flags, inner);
    if (rc == PBAG_OK) rc = radiate(T, P, w, r, it, o, inner);
    if (rc != PBAG_OK) {
      *fail_step = (int)it;
      return rc;
    }
  }
  return PBAG_OK;
}

}  // namespace

extern "C" {

int orc_build_grids(const pbag_grid_desc* g, double* gam, double* freq) {
  const int G = g->ngam, F = g->nfreq;
  // base_state.h:229-236: e[i] = step^i, step = exp(ln(gam2)/G)
  double step = std::exp(std::log(g->gam2) / (double)G);
  for (int i = 0; i < G; i++) gam[i] = std::pow(step, (double)i);
  // utils.h MakeLogspaceVec: first = 10^start, base = 10^((stop-start)/num), x *= base
  double start = std::log10(g->freq1), stop = std::log10(g->freq2);
  double cur = std::pow(10., start);
  double base = std::pow(10., (stop - start) / F);
  for (int i = 0; i <= F; i++) {
    freq[i] = cur;
    cur *= base;
  }
  return PBAG_OK;
}

double orc_syn_func(int method, double B, double nu, double gam) { return pick_syn(method)(B, nu, gam); }

double orc_ssc_func(double nu, double gam, double nu_tilde) { return ssc_nava(nu, gam, nu_tilde); }

int orc_ssc_kernel(const double* gam, int G, const double* freq, int F, double* K, double* Kint) {
  std::vector<double> tmp;
  double* KK = K;
  if (!KK) {
    tmp.assign((size_t)F * G * F, 0.);
    KK = tmp.data();
  }
  for (int i = 0; i < F; i++)
    for (int j = 0; j < G; j++)
      for (int k = 0; k < F; k++) KK[((size_t)i * G + j) * F + k] = ssc_nava(freq[i], gam[j], freq[k]);
  for (int j = 0; j < G; j++)
    for (int k = 0; k < F; k++) {
      double res = 0;
      for (int i = 0; i < F - 1; i++)
        res += KK[((size_t)i * G + j) * F + k] * freq[i + 1] * (freq[i + 1] - freq[i]);
      Kint[(size_t)j * F + k] = res;
    }
  return PBAG_OK;
}

int orc_run(const pbag_grid_desc* g, const pbag_shock_params* prm, int nbw, const int64_t* offsets,
            const pbag_step_rec* recs, pbag_outputs* out, int flags, int outer_threads, int inner_threads,
            pbag_status* st) {
  if (!g || !prm || !offsets || !recs || !out || nbw < 0 || g->ngam < 8 || g->nfreq < 8) return PBAG_ERR_ARG;
  bool any_ssc = false;
  for (int b = 0; b < nbw; ++b) any_ssc = any_ssc || prm[b].ssc_on;
  Tables T;
  build_tables(g, any_ssc, T);
  // zero all output rows (skipped steps keep zero rows, like the reference's vectors)
  const size_t nrec = (size_t)offsets[nbw];
  for (size_t fi = 0; fi < 13; ++fi) {
    double* p = ((double**)out)[fi];
    size_t n = fi >= 4 && fi < 8 ? (size_t)T.G : (size_t)T.F;
    if (p) std::memset(p, 0, sizeof(double) * nrec * n);
  }
  int inner = (flags & ORC_INNER_OMP) ? inner_threads : 1;
  std::vector<int> codes(nbw, PBAG_OK), steps(nbw, -1);
  (void)outer_threads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(outer_threads) if (outer_threads > 1)
  for (int b = 0; b < nbw; ++b) {
    size_t r0 = (size_t)offsets[b], nr = (size_t)(offsets[b + 1] - offsets[b]);
    pbag_outputs o = *out;
    for (size_t fi = 0; fi < 13; ++fi) {
      double** p = ((double**)&o) + fi;
      size_t n = fi >= 4 && fi < 8 ? (size_t)T.G : (size_t)T.F;
      if (*p) *p += r0 * n;
    }
    codes[b] = run_one(T, prm[b], recs + r0, nr, &o, flags, inner, &steps[b]);
  }
  for (int b = 0; b < nbw; ++b)
    if (codes[b] != PBAG_OK) {
      if (st) {
        st->code = codes[b];
        st->bw = b;
        st->step = steps[b];
      }
      return codes[b];
    }
  if (st) {
    st->code = PBAG_OK;
    st->bw = -1;
    st->step = -1;
  }
  return PBAG_OK;
}

int orc_contract(const pbag_grid_desc* g, int n, const double* f, const double* B, const double* nph, int syn_method,
                 double* jsyn, double* jssc, int threads) {
  if (!g || n < 0 || !f || g->ngam < 8 || g->nfreq < 8) return PBAG_ERR_ARG;
  const int G = g->ngam, F = g->nfreq;
  std::vector<double> e(G), nu(F + 1);
  orc_build_grids(g, e.data(), nu.data());
  std::vector<double> K;
  if (jssc) {
    if (!nph) return PBAG_ERR_ARG;
    K.assign((size_t)F * G * F, 0.);
    for (int i = 0; i < F; i++)
      for (int j = 0; j < G; j++)
        for (int k = 0; k < F; k++) K[((size_t)i * G + j) * F + k] = ssc_nava(nu[i], e[j], nu[k]);
  }
  if (jsyn && !B) return PBAG_ERR_ARG;
  const auto syn = pick_syn(syn_method);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) if (threads > 1)
  for (int s = 0; s < n; ++s) {
    const double* fs = f + (size_t)s * G;
    if (jsyn) {
      // computeSynSpectrum (numeric_model.h:148-184) with the kernel of SynKernel::evalSynKernel
      // (kernels.h:528-538) at this state's field
      double* js = jsyn + (size_t)s * F;
      for (int i = 0; i < F; ++i) js[i] = 0.;
      for (int i = 0; i < F - 1; ++i) {
        double res = 0.;
        for (int j = 0; j < G - 1; ++j) res += syn(B[s], nu[i], e[j]) * fs[j] * (e[j + 1] - e[j]);
        js[i] = res;
      }
    }
    if (jssc) {
      // computeSSCSpectrum (numeric_model.h:247-285), photon_density = nph[s]
      const double* ph = nph + (size_t)s * F;
      double* jc = jssc + (size_t)s * F;
      std::vector<double> scat(G - 1);
      for (int i = 0; i < F; ++i) {
        for (int j = 0; j < G - 1; ++j) scat[j] = 0.;
        for (int j = 0; j < G - 1; ++j)
          for (int k = 0; k < F; ++k)
            scat[j] += 3. / 4. * sigma_T * c_light / (e[j] * e[j]) * ph[k] / nu[k] * (nu[k + 1] - nu[k]) *
                       K[((size_t)i * G + j) * F + k];
        double r = 0.;
        for (int j = 0; j < G - 1; ++j) r += fs[j] * h_pl * nu[i] * scat[j] * (e[j + 1] - e[j]);
        jc[i] = r;
      }
    }
  }
  return PBAG_OK;
}

}  // extern "C"

namespace {

// ElectronAndRadiation::fluxDens (microphysics.h:1185-1217) with
// computeFluxDensity (:799-867) and computeIntensity (:11-58), FP64, for one
// query on the histories of its blastwave (rows r0 + ia, r0 + ib of J / A
// and R). Returns PBAG_OK, PBAG_ERR_RANGE or PBAG_ERR_NONFINITE.
int flux_dens_one(const double* nu, int F, const pbag_flux_opts* o, const double* J, const double* A,
                  const double* R, int64_t r0, const pbag_flux_query& q, double* out) {
  *out = 0.;
  if (q.freq >= nu[F - 1] || q.freq <= nu[0]) return PBAG_ERR_RANGE;  // microphysics.h:1190-1201
  // findIndex (interpolators.h:13-35)
  size_t ia_nu;
  if (q.freq <= nu[0])
    ia_nu = 0;
  else if (q.freq >= nu[F - 1])
    ia_nu = F - 2;
  else {
    unsigned a = 0, b = (unsigned)F - 1;
    while (b - a > 1u) {
      unsigned i = (b + a) >> 1;
      if (nu[i] > q.freq)
        b = i;
      else
        a = i;
    }
    ia_nu = a;
  }
  const size_t ib_nu = ia_nu + 1;
  // Interp2d::InterpolateBilinear / BilinearInterpolation (interpolators.h:708-801)
  auto interp = [&](const double* Z) {
    double q11 = Z[(r0 + q.ia) * F + ia_nu], q12 = Z[(r0 + q.ib) * F + ia_nu];
    double q21 = Z[(r0 + q.ia) * F + ib_nu], q22 = Z[(r0 + q.ib) * F + ib_nu];
    double x1 = nu[ia_nu], x2 = nu[ib_nu], y1 = R[r0 + q.ia], y2 = R[r0 + q.ib];
    double x2x1 = x2 - x1, y2y1 = y2 - y1, x2x = x2 - q.freq, y2y = y2 - q.r, yy1 = q.r - y1, xx1 = q.freq - x1;
    return 1.0 / (x2x1 * y2y1) * (q11 * x2x * y2y + q21 * xx1 * y2y + q12 * x2x * yy1 + q22 * xx1 * yy1);
  };
  const double em_prime = interp(J), abs_prime = interp(A);
  auto beta_of = [](double gm) { return std::sqrt((gm - 1.) * (gm + 1.)) / gm; };  // blastwave_components.h:36
  double beta = beta_of(q.Gamma);
  double a = 1.0 - beta * q.mu;
  double delta_D = q.Gamma * a;
  double em_lab = em_prime / (delta_D * delta_D);
  double abs_lab = abs_prime * delta_D;
  double beta_shock = o->shock_vel == PBAG_VEL_SHOCK ? beta_of(q.GammaSh) : beta_of(q.Gamma);
  double m2 = q.ne * m_p;
  double dr = m2 / (2. * pi_ * m_p * q.r * q.r * (1. - std::cos(q.theta) / q.ncells) * q.Gamma * q.n_prime);
  double dtau;
  if (q.mu == beta_shock)
    dtau = 1.0e100;
  else
    dtau = abs_lab * dr * (1. - q.mu * beta_shock) / (q.mu - beta_shock);
  double intensity = em_lab;
  if (dtau != 0) {
    double thick = dtau > 0 ? em_lab / dtau : 0.;
    double u = 1. / 2. + std::exp(-dtau) / dtau - (1 - std::exp(-dtau)) / (dtau * dtau);
    double approx = dtau > 1.e-3 ? em_lab * (3. * u / dtau) : em_lab;
    double abs_fac = dtau > 0.0 ? -std::expm1(-dtau) / dtau : std::expm1(dtau) / dtau;
    double smooth = em_lab * abs_fac;
    double sharp = em_lab;
    if (dtau > 1.0)
      sharp = em_lab / dtau;
    else if (dtau < -1.0)
      sharp = 0.0;
    intensity = o->method_tau == PBAG_TAU_THICK    ? thick
                : o->method_tau == PBAG_TAU_SMOOTH ? smooth
                : o->method_tau == PBAG_TAU_SHARP  ? sharp
                                                   : approx;
  }
  if (intensity < 0 || !std::isfinite(intensity)) return PBAG_ERR_NONFINITE;
  double ashock = 1.0 - q.mu * beta_shock;
  double lum = o->method_ne == PBAG_NE_USE_NPRIME
                   ? intensity * q.r * q.r * (dr / ashock)
                   : intensity * q.ne / (2. * pi_ * (1. - std::cos(q.theta) / q.ncells)) / q.Gamma / ashock;
  if (lum < 0 || !std::isfinite(lum)) return PBAG_ERR_NONFINITE;
  *out = lum;
  return PBAG_OK;
}

}  // namespace

extern "C" {

// ElectronAndRadiation::fluxDens for a batch of queries (flux_dens_one each).
int orc_flux_dens(const pbag_grid_desc* g, const pbag_flux_opts* o, const int64_t* offsets, const double* j_all,
                  const double* a_all, const double* r_all, int nq, const pbag_flux_query* qs, double* flux,
                  int* fail_index) {
  const int F = g->nfreq;
  std::vector<double> gam(g->ngam), nu(F + 1);
  orc_build_grids(g, gam.data(), nu.data());
  *fail_index = -1;
  for (int t = 0; t < nq; ++t) {
    const int rc = flux_dens_one(nu.data(), F, o, j_all, a_all, r_all, offsets[qs[t].bw], qs[t], &flux[t]);
    if (rc != PBAG_OK) {
      *fail_index = t;
      return rc;
    }
  }
  return PBAG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Shock scalars (microphysics_base.h:575-966). The members the reference keeps
// on its ElectronAndRadiaionBase object live in `Mem`; every call follows the
// order of computeEleSpectrumLimits: checkParams, computeMagneticField,
// computeGammaMax, computeGammaMin, computeGammaCool.
namespace {

struct Mem {
  const pbag_limits_opts* o;
  double eprime, Gamma, GammaSh, betaSh, t_e, tcomov, n_prime;
  double B, gamma_min, gamma_max, gamma_c, accel_frac, Theta, z_cool;
};

double beta_of(double g) { return std::sqrt((g - 1.) * (g + 1.)) / g; }  // EQS::BetaFromGamma

double gm_func(double x, const Mem& m) {  // gammaMinFunc (microphysics_base.h:792-806)
  const double p = m.o->p;
  const double ave = m.o->eps_e * m.eprime / (m.n_prime * m_e * c_light * c_light);
  if (p == 1) return (m.gamma_max - m.gamma_min) / (std::log(m.gamma_max) - std::log(m.gamma_min)) - ave;
  if (p == 2) return (std::log(m.gamma_max) - std::log(m.gamma_min)) / (-1. / m.gamma_max + 1. / m.gamma_min) - ave;
  return (p - 1) / (p - 2) * (std::pow(m.gamma_max, -p + 2) - std::pow(x, -p + 2)) /
             (std::pow(m.gamma_max, -p + 1) - std::pow(x, -p + 1)) -
         ave;
}

double bisect_gm(double a, double b, double xtol, double rtol, int iters, const Mem& m, int& status) {
  // rootfinders.h:17-58
  status = 0;
  const double fa0 = gm_func(a, m), fb0 = gm_func(b, m);
  if (fa0 * fb0 > 0) { status = -1; return 0.; }
  if (fa0 == 0) { status = -1; return a; }
  if (fb0 == 0) { status = -1; return b; }
  double fa = fa0, d = b - a;
  for (int k = 0; k < iters; ++k) {
    d *= 0.5;
    const double mid = a + d;
    const double fm = gm_func(mid, m);
    if (fm * fa >= 0) a = mid;
    if (fm == 0 || std::fabs(d) < xtol + rtol * std::fabs(mid)) return mid;
  }
  status = -1;
  return a;
}

}  // namespace

extern "C" int orc_shock_limits(const pbag_limits_opts* o, const double* gam, int ngam, int n,
                                const pbag_shock_state* in, double* state, pbag_limits* out) {
  if (!o || !gam || ngam < 2 || n < 0 || !state || (n > 0 && (!in || !out))) return PBAG_ERR_ARG;
  Mem m{};
  m.o = o;
  m.gamma_min = state[0], m.gamma_max = state[1], m.gamma_c = state[2], m.accel_frac = state[3];
  m.B = state[4], m.Theta = state[5], m.z_cool = state[6];
  const bool analytic = o->ele_analytic != 0;
  const double egrid_lo = gam[0], egrid_hi = gam[ngam - 1];
  for (int s = 0; s < n; ++s) {
    const pbag_shock_state& x = in[s];
    m.GammaSh = x.GammaSh, m.eprime = x.e_prime, m.Gamma = x.Gamma, m.betaSh = beta_of(x.GammaSh);
    m.t_e = x.t_e, m.tcomov = x.tcomov, m.n_prime = x.n_prime;
    const bool ok = !(m.betaSh < o->beta_min);  // checkParams
    if (ok) {
      if (o->eps_e <= 0 || o->eps_b <= 0 || o->eps_t < 0 || o->p <= 0 || m.n_prime <= 0 || m.eprime < 0 ||
          !std::isfinite(m.eprime))
        return PBAG_ERR_PARAM;
      // computeMagneticField
      const double Bub = std::sqrt(8. * pi_ * (m.eprime * o->eps_b));
      const double Bsh = std::sqrt(32. * M_PI * o->eps_b * (m.GammaSh - 1.) * (m.GammaSh + 3. / 4) * m.n_prime * m_p *
                                   (c_light * c_light));
      const double Bmag = std::sqrt(9.0 * M_PI * o->eps_b * m.n_prime * o->mu * m_p) * (m.betaSh * c_light);
      m.B = o->method_B == 0 ? Bub : o->method_B == 2 ? Bsh : Bmag;
      // computeGammaMax
      if (o->method_gamma_max == 0) m.gamma_max = std::sqrt(6.0 * pi_ * q_e / sigma_T / m.B);
      if (!analytic && m.gamma_max > 0.99 * egrid_hi) m.gamma_max = 0.99 * egrid_hi;
      // computeGammaMin
      const double p = o->p;
      int status = 0;
      const double g1 = (p - 2.) / (p - 1.) * (m.eprime * o->eps_e) / (m.n_prime * m_e * c_light * c_light);
      const double g2 = (p - 2.) / (p - 1.) * (m_p / m_e) * o->eps_e * beta_of(m.GammaSh);
      const double g3 = (p - 2.) / (p - 1.) * (o->eps_e * m_p / m_e * (m.GammaSh - 1.) + 1.);
      const double th0 = o->eps_t * (9.0 * o->mu * m_p / (32.0 * o->mu_e * m_e)) * m.betaSh * m.betaSh;
      m.Theta = (5.0 * th0 - 6.0 + std::sqrt(25.0 * th0 * th0 + 180.0 * th0 + 36.0)) / 30.0;  // Margalit21::Theta_fun
      m.z_cool = (6.0 * M_PI * m_e * c_light / (sigma_T * m.B * m.B * m.t_e)) / m.Theta;
      const double g4 = 1. + (6.0 + 15.0 * m.Theta) / (4.0 + 5.0 * m.Theta) * m.Theta;  // Margalit21::gamma_m_fun
      if (o->method_gamma_min == 0) m.gamma_min = g1;
      else if (o->method_gamma_min == 2) m.gamma_min = g2;
      else if (o->method_gamma_min == 3) m.gamma_min = g3;
      else if (o->method_gamma_min == 4) m.gamma_min = g4;
      else if (o->method_gamma_min == 1) {
        m.gamma_min = bisect_gm(1., 1.e8, 0., .001, 100, m, status);
        if (status < 0 && g1 > 1.5) m.gamma_min = g1;
      } else {
        return PBAG_ERR_ARG;
      }
      const double gM = m.gamma_max, gm = m.gamma_min;
      const double ayache = (std::pow(gM, 2 - p) - std::pow(gm - 1., 2. - p)) / (std::pow(gM, 2. - p) - 1.) *
                            (std::pow(gM, 1. - p) - 1.) / (std::pow(gM, 1. - p) - std::pow(gm - 1., 1. - p));
      const double sironi = (p - 2.0) / (p - 1.0) * o->eps_e * m.eprime / (m.n_prime * m_e * c_light * c_light);
      if (m.gamma_min < 2. || status < 0) {
        if (o->method_nonrel == 0) m.accel_frac = 1;
        else if (o->method_nonrel == 1) m.accel_frac = m.gamma_min;
        else if (o->method_nonrel == 2 || o->method_nonrel == 3) {
          if (p < 2.) return PBAG_ERR_PARAM;
          m.accel_frac = o->method_nonrel == 2 ? ayache : sironi;
        } else {
          return PBAG_ERR_ARG;
        }
        if (m.accel_frac > 1.) m.accel_frac = 1;
        if (m.gamma_min < 1.) m.gamma_min = 1;
      }
      if (!std::isfinite(m.gamma_min) || !std::isfinite(m.accel_frac) || m.accel_frac < 0) return PBAG_ERR_NONFINITE;
      if (!analytic && m.gamma_min < egrid_lo) {
        m.gamma_min = egrid_lo;
        if (m.gamma_min > 1e8) return PBAG_ERR_PARAM;
      }
      // computeGammaCool
      if (o->method_gamma_c == 0) m.gamma_c = 6. * pi_ * m_e * c_light / (sigma_T * m.B * m.B) * x.t_e / m.Gamma;
      else if (o->method_gamma_c == 1) m.gamma_c = (6. * pi_ * m_e * c_light) / (sigma_T * m.B * m.B * m.tcomov);
      if (m.gamma_c <= 1.) m.gamma_c = 1.001;
      if (!analytic && m.gamma_c > m.gamma_max) m.gamma_c = m.gamma_max;
    }
    pbag_limits& r = out[s];
    r.B = m.B, r.gamma_min = m.gamma_min, r.gamma_max = m.gamma_max, r.gamma_c = m.gamma_c;
    r.accel_frac = m.accel_frac, r.Theta = m.Theta, r.z_cool = m.z_cool;
    r.valid = ok ? 1 : 0;
    r.reserved = 0;
  }
  state[0] = m.gamma_min, state[1] = m.gamma_max, state[2] = m.gamma_c, state[3] = m.accel_frac;
  state[4] = m.B, state[5] = m.Theta, state[6] = m.z_cool;
  return PBAG_OK;
}

// ---------------------------------------------------------------------------
// Adaptive EATS light curve: EATS::evalFluxDensA (eats.h:820-850) with atol 0,
// parsPars' mu array (eats.h:917-948), integrate_theta_phi (:587-700),
// phi_integrand (:449-586) with find_jet_edge (:103-173), costheta_integrand
// (:435-448), integrand (:175-232) with check_emission_time (:24-38), the
// flux of fluxDensAdaptiveWithComov (blastwave_radiation.h:75-150), and the
// quadratures trap (quadratures.h:939-951) and cadre_adapt = m9_adapt with
// cadreInitInterval / cadreProcessInterval / cadreSplitInterval and the mesh9
// heap (quadratures.h:182-208, 657-770, 1613-2113), in their loop structure
// and operation order.
namespace {

struct Iv9 {  // Interval9 (quadratures.h:182-198)
  double a, b, I, err, fa, fll, fl, flr, fm, frl, fr, frr, fb;
  int refinement;
};

struct Mesh9 {  // quadratures.h:201-208, 657-770
  std::vector<Iv9> heap;
  void insert(const Iv9& i) {
    heap.push_back(i);
    size_t c = heap.size() - 1, p = (c - 1) / 2;
    while (c != 0 && heap[p].err < heap[c].err) {
      std::swap(heap[p], heap[c]);
      c = p;
      p = (c - 1) / 2;
    }
  }
  void extract(Iv9* worst) {
    *worst = heap[0];
    heap[0] = heap[heap.size() - 1];
    heap.pop_back();
    size_t p = 0, c1 = 1, c2 = 2;
    while (c1 < heap.size()) {
      size_t c = c1;
      double e = heap[c1].err;
      if (c2 < heap.size() && heap[c2].err > e) {
        c = c2;
        e = heap[c2].err;
      }
      if (e <= heap[p].err) break;
      std::swap(heap[p], heap[c]);
      p = c;
      c1 = 2 * p + 1;
      c2 = c1 + 1;
    }
  }
  double total_I() const {
    double I = 0.0;
    for (const Iv9& i : heap) I += i.I;
    return I;
  }
  double total_err() const {
    double e = 0.0;
    for (const Iv9& i : heap) e += i.err;
    return e;
  }
};

// cadre_adapt over f (a callable double(double)); err() stops the quadrature
// as the reference's errf does (its result is then 0).
template <class Fn, class Err>
struct Cadre {
  Fn& f;
  Err& errf;
  int init(Iv9* i) {  // cadreInitInterval with pfa = pfb = NULL
    int count = 0;
    i->fa = f(i->a);
    count++;
    if (errf()) return count;
    i->fb = f(i->b);
    count++;
    if (errf()) return count;
    i->fm = f(0.5 * (i->a + i->b));
    count++;
    return count;
  }
  int process(Iv9* i) {  // cadreProcessInterval
    const double scaleTol = 0.2;
    int count = 0;
    if (i->refinement < 4) {
      double fa = i->fa, fm = i->fm, fb = i->fb;
      double fl, fr;
      if (i->refinement == 0) {
        fl = f(0.75 * i->a + 0.25 * i->b);
        count++;
        if (errf()) return count;
        fr = f(0.25 * i->a + 0.75 * i->b);
        count++;
        if (errf()) return count;
        i->fl = fl;
        i->fr = fr;
      } else {
        fl = i->fl;
        fr = i->fr;
        i->refinement = 0;
      }
      double h = 0.25 * (i->b - i->a);
      double T0 = 2 * h * (fa + fb);
      double T1 = 0.5 * T0 + 2 * h * fm;
      double T2 = 0.5 * T1 + h * (fl + fr);
      double R0 = (T1 - T0) / (T2 - T1);
      if (R0 > 4 - scaleTol && R0 < 4 + scaleTol) {
        double fll = f(0.875 * i->a + 0.125 * i->b);
        count++;
        if (errf()) return count;
        double flr = f(0.625 * i->a + 0.375 * i->b);
        count++;
        if (errf()) return count;
        double frl = f(0.375 * i->a + 0.625 * i->b);
        count++;
        if (errf()) return count;
        double frr = f(0.125 * i->a + 0.875 * i->b);
        count++;
        if (errf()) return count;
        i->fll = fll;
        i->flr = flr;
        i->frl = frl;
        i->frr = frr;
        i->refinement = 1;
        double T3 = 0.5 * T2 + 0.5 * h * (fll + flr + frl + frr);
        double R1 = (T2 - T1) / (T3 - T2);
        if (R1 > 4 - scaleTol && R1 < 4 + scaleTol) {
          double R11 = (4 * T1 - T0) / 3.0;
          double R21 = (4 * T2 - T1) / 3.0;
          double R22 = (16 * R21 - R11) / 15.0;
          i->fa = T3;
          i->fll = (4 * T3 - T2) / 3.0;
          i->fl = (16 * i->fll - R21) / 15.0;
          i->flr = (64 * i->fl - R22) / 63.0;
          i->I = i->flr;
          i->err = std::fabs((i->fl - R22) / 63.0);
          i->refinement = 4;
          return count;
        }
        double errt = (T3 - T2) / 3.0;
        i->err = std::fabs(errt);
        i->I = T3 + errt;
        return count;
      } else if (R0 >= 4 + scaleTol || R0 < 2 || R0 != R0) {
        double err10 = std::fabs(T1 - T0);
        double err21 = std::fabs(T2 - T1);
        i->err = err10 > err21 ? err10 : err21;
        i->I = T2;
        return count;
      } else {
        double err = -(T2 - T1) * (T2 - T1) / (T2 - 2 * T1 + T0);
        i->err = std::fabs(err);
        if (std::fabs(T2 + err) < 1.0e-14 * std::fabs(T2))
          i->I = 1.0e-14 * T2;
        else
          i->I = T2 + err;
        return count;
      }
    }
    if (i->refinement < 0) return 0;
    int nint = 1;
    for (int n = 0; n < i->refinement; n++) nint *= 2;
    double h = (i->b - i->a) / nint;
    double sum = 0;
    for (int n = 1; n < nint; n += 2) {
      sum += f(i->a + h * n);
      count++;
      if (errf()) return count;
    }
    // the Romberg tableau in fa, fll, fl, flr, fm, frl, fr, frr, fb (m = 1..9)
    double* tab[9] = {&i->fa, &i->fll, &i->fl, &i->flr, &i->fm, &i->frl, &i->fr, &i->frr, &i->fb};
    double T = 0.5 * i->fa + h * sum;
    double Rnm = i->fa;
    double Rnmp = i->fll;
    i->fa = T;
    i->fll = (4.0 * i->fa - Rnm) / 3.0;
    if (i->refinement == 1) {
      i->I = i->fll;
      i->err = std::fabs((i->fa - Rnm) / 3.0);
      i->refinement += 1;
      return count;
    }
    double pw = 4.0;
    for (int m = 2; m <= 8; ++m) {
      pw *= 4.0;
      Rnm = Rnmp;
      Rnmp = *tab[m];
      *tab[m] = (pw * *tab[m - 1] - Rnm) / (pw - 1.0);
      if (i->refinement == m) {
        i->I = *tab[m];
        i->err = std::fabs((*tab[m - 1] - Rnm) / (pw - 1.0));
        i->refinement += 1;
        return count;
      }
    }
    Rnm = Rnmp;  // m = 9
    i->I = (262144 * i->fb - Rnm) / 262143.0;
    i->err = std::fabs((i->fb - Rnm) / 262143.0);
    i->refinement += 1;
    return count;
  }
  int split(Iv9* i0, Iv9* i1, Iv9* i2) {  // cadreSplitInterval
    double xm = 0.5 * (i0->a + i0->b);
    i1->a = i0->a;
    i1->b = xm;
    i2->a = xm;
    i2->b = i0->b;
    i1->fa = i0->fa;
    i1->fl = i0->fll;
    i1->fm = i0->fl;
    i1->fr = i0->flr;
    i1->fb = i0->fm;
    i1->refinement = i0->refinement;
    i2->fa = i0->fm;
    i2->fl = i0->frl;
    i2->fm = i0->fr;
    i2->fr = i0->frr;
    i2->fb = i0->fb;
    i2->refinement = i0->refinement;
    int n = 0;
    n += process(i1);
    n += process(i2);
    return n;
  }
  double adapt(double xa, double xb, int Nmax, double atol, double rtol) {  // m9_adapt
    Mesh9 m;
    Iv9 i{};
    i.a = xa;
    i.b = xb;
    int n = init(&i);
    if (errf()) return 0.0;
    n += process(&i);
    if (errf()) return 0.0;
    m.insert(i);
    double I = i.I, err = i.err;
    int num_intervals = 1, num_iterations = 0, last_check = 0;
    while (n < Nmax && err > atol + rtol * std::fabs(I)) {
      m.extract(&i);
      if (i.refinement >= 4) {
        double oldI = i.I, olderr = i.err;
        n += process(&i);
        if (errf()) return 0.0;
        m.insert(i);
        err += i.err - olderr;
        I += i.I - oldI;
      } else {
        Iv9 i1{}, i2{};
        n += split(&i, &i1, &i2);
        if (errf()) return 0.0;
        m.insert(i1);
        m.insert(i2);
        num_intervals++;
        err += i1.err + i2.err - i.err;
        I += i1.I + i2.I - i.I;
      }
      if (num_iterations == 2 * last_check) {
        err = m.total_err();
        I = m.total_I();
        last_check = num_intervals;
      }
      num_iterations++;
    }
    return m.total_I();
  }
};

template <class Fn, class Err>
double trap_fixed(Fn& f, Err& errf, double xa, double xb, int N) {  // trap (quadratures.h:939-951)
  double dx = (xb - xa) / N;
  double fa = f(xa);
  double I = 0.5 * (fa + f(xb));
  for (int i = 1; i < N; i++) {
    I += f(xa + i * dx);
    if (errf()) return 0.0;
  }
  return I * dx;
}

// findIndex (interpolators.h:13-35)
size_t find_index(double x, const double* arr, size_t N) {
  if (x <= arr[0]) return 0;
  if (x >= arr[N - 1]) return N - 2;
  unsigned a = 0, b = (unsigned)N - 1;
  while (b - a > 1u) {
    unsigned i = (b + a) >> 1;
    if (arr[i] > x)
      b = i;
    else
      a = i;
  }
  return a;
}
double seg_lin(size_t a, size_t b, double x, const double* X, const double* Y) {  // interpSegLin (:98-106)
  return Y[a] + (Y[b] - Y[a]) * (x - X[a]) / (X[b] - X[a]);
}
double seg_log(size_t a, size_t b, double x, const double* X, const double* Y) {  // interpSegLog (:114-122)
  return Y[a] * std::pow(Y[b] / Y[a], std::log(x / X[a]) / std::log(X[b] / X[a]));
}
double obs_angle(double theta, double phi, double a) {  // image.h:361-375
  return std::sin(a) * (std::sin(theta) * std::sin(phi)) + std::cos(a) * std::cos(theta);
}
double obs_angle_cj(double theta, double phi, double a) {  // image.h:376-378
  return std::sin(a) * (std::sin(pi_ - theta) * std::sin(phi)) + std::cos(a) * std::cos(pi_ - theta);
}

// the state an EATS object holds while it integrates one (layer, t_obs, nu_obs)
struct EatsRun {
  const pbag_eats_opts* o;
  const pbag_eats_layer* L;
  int nr;
  const double* dyn;  // [PBAG_EQ_N][nr]
  const double* nu;
  int F;
  const double *J, *A, *Rh;  // histories and their radius rows (the layer's dynamics R)
  int64_t r_fs, r_rs;        // first history rows of the layer's shocks (r_rs < 0: none)
  std::vector<double> mu;
  bool cj = false;
  double t_obs = 0, nu_obs = 0, phi = 0;
  long nevals = 0;
  int code = PBAG_OK;
  const double* q(int k) const { return dyn + (size_t)k * nr; }
  double angle(double th, double ph) const { return cj ? obs_angle_cj(th, ph, o->theta_obs) : obs_angle(th, ph, o->theta_obs); }

  // fluxDensAdaptiveWithComov (blastwave_radiation.h:75-150)
  double flux_a(double theta_in, size_t ia, size_t ib, double mu_, double t_e) {
    const double* tb = q(PBAG_EQ_TBURST);
    const double* R = q(PBAG_EQ_R);
    double r = seg_log(ia, ib, t_e, tb, R);
    if (r <= 0.0 || !std::isfinite(r)) return 0.0;
    double Gamma = seg_log(ia, ib, r, R, q(PBAG_EQ_GAMMA));
    double beta = seg_log(ia, ib, r, R, q(PBAG_EQ_BETA));
    double GammaShock = seg_log(ia, ib, r, R, q(PBAG_EQ_GAMMA_FSH));
    double dr = seg_log(ia, ib, r, R, q(PBAG_EQ_THICKNESS));
    double ne = seg_log(ia, ib, r, R, q(PBAG_EQ_M2)) / m_p;
    double n_prime = seg_log(ia, ib, r, R, q(PBAG_EQ_RHO2)) / m_p;
    double rsh = seg_log(ia, ib, r, R, q(PBAG_EQ_RSH));
    double acc_fac = seg_log(ia, ib, r, R, q(PBAG_EQ_ACC_FRAC));
    double a = 1.0 - beta * mu_;
    double delta_D = Gamma * a;
    double nuprime = (1.0 + o->z) * nu_obs * delta_D;
    double theta = seg_log(ia, ib, r, R, q(PBAG_EQ_THETA));
    (void)theta_in;
    pbag_flux_query fq{};
    fq.ia = (int)ia;
    fq.ib = (int)ib;
    fq.theta = theta;
    fq.ncells = L->ncells;
    fq.freq = nuprime;
    fq.Gamma = Gamma;
    fq.GammaSh = GammaShock;
    fq.acc_fac = acc_fac;
    fq.mu = mu_;
    fq.r = r;
    fq.rsh = rsh;
    fq.dr = dr;
    fq.n_prime = n_prime;
    fq.ne = ne;
    double flux = 0.;
    int rc = flux_dens_one(nu, F, &o->flux, J, A, Rh, r_fs, fq, &flux);
    if (rc != PBAG_OK) {
      code = rc;
      return 0.0;
    }
    if (r_rs >= 0) {
      const double* th_rs = q(PBAG_EQ_THICKNESS_RS);
      if (th_rs[ia] > 0 && th_rs[ib] > 0) {
        fq.GammaSh = seg_log(ia, ib, r, R, q(PBAG_EQ_GAMMA_RSH));
        fq.dr = seg_log(ia, ib, r, R, th_rs);
        fq.ne = seg_log(ia, ib, r, R, q(PBAG_EQ_M3)) / m_p;
        fq.n_prime = seg_log(ia, ib, r, R, q(PBAG_EQ_RHO3)) / m_p;
        fq.rsh = seg_log(ia, ib, r, R, q(PBAG_EQ_RRSH));
        fq.acc_fac = seg_log(ia, ib, r, R, q(PBAG_EQ_ACC_FRAC_RS));
        double frs = 0.;
        rc = flux_dens_one(nu, F, &o->flux, J, A, Rh, r_rs, fq, &frs);
        if (rc != PBAG_OK) {
          code = rc;
          return 0.0;
        }
        flux += frs;
      }
    }
    return flux;
  }
  // integrand (eats.h:175-232)
  double integrand(double i_cos_theta, double i_phi) {
    const double* R = q(PBAG_EQ_R);
    const int ie = L->i_end_r;
    if (R[0] == 0.0 && R[ie - 1] == 0.0) return 0.0;
    double a_theta = 2.0 * std::asin(std::sqrt(0.5 * (1.0 - i_cos_theta)));  // arccos (image.h:357-360)
    double mu_ = angle(a_theta, i_phi);
    if (mu_ < mu[0]) return 0.;
    if (mu_ > mu[ie - 1]) return 0.;
    size_t ia = find_index(mu_, mu.data(), ie), ib = ia + 1;
    double t_e = seg_lin(ia, ib, mu_, mu.data(), q(PBAG_EQ_TBURST));
    // check_emission_time (eats.h:24-38)
    if (mu_ > mu[ie - 1] || mu[0] >= mu_) t_e = -1;
    if (t_e < 0.0 || !std::isfinite(t_e)) return 0.;
    return flux_a(a_theta, ia, ib, mu_, t_e);
  }
  // find_jet_edge (eats.h:103-173)
  double jet_edge(double ph, double th_con_hi) {
    const double* thj = q(PBAG_EQ_THETA);
    const int N = L->i_end_r;
    double mu_ = angle(th_con_hi, ph);
    size_t ia = find_index(mu_, mu.data(), N);
    if (thj[ia] <= th_con_hi && th_con_hi <= thj[ia + 1]) return th_con_hi;
    double theta_a, theta_b;
    if (th_con_hi < thj[ia]) {
      theta_a = th_con_hi;
      theta_b = 0.5 * pi_;
    } else {
      theta_a = 0.0;
      theta_b = th_con_hi;
    }
    int i = 0;
    while (theta_b - theta_a > 1.0e-5 && i < 100) {
      double theta_c_i = 0.5 * (theta_a + theta_b);
      mu_ = angle(theta_c_i, ph);
      ia = find_index(mu_, mu.data(), N);
      if (theta_c_i < thj[ia])
        theta_a = theta_c_i;
      else
        theta_b = theta_c_i;
      i++;
    }
    return theta_a;
  }
  bool stop() const { return code != PBAG_OK; }
  // costheta_integrand (eats.h:435-448)
  double costheta(double aomct) {
    nevals += 1;
    if (nevals > (long)1e7) {
      code = PBAG_ERR_EVALS;
      return 0.0;
    }
    return integrand(1 - aomct, phi);
  }
  // phi_integrand (eats.h:449-586)
  double phi_integrand(double a_phi) {
    phi = a_phi;
    double theta_1 = L->theta_c_h, theta_0 = L->theta_c_l;
    double th_1 = jet_edge(a_phi, theta_1);
    double frac = theta_0 / theta_1;
    double th_0 = frac * th_1;
    theta_0 = th_0;
    theta_1 = th_1;
    if (theta_0 > 0.5 * pi_) theta_0 = 0.5 * pi_;
    if (theta_1 > 0.5 * pi_) theta_1 = 0.5 * pi_;
    double s0 = std::sin(0.5 * theta_0), s1 = std::sin(0.5 * theta_1);
    double omc0 = 2.0 * s0 * s0, omc1 = 2.0 * s1 * s1;
    auto fth = [&](double x) { return costheta(x); };
    auto st = [&]() { return stop(); };
    double result;
    if (o->method_quad == PBAG_QUAD_TRAP_FIXED) {
      result = trap_fixed(fth, st, omc0, omc1, o->nmax_theta);
    } else {
      Cadre<decltype(fth), decltype(st)> c{fth, st};
      result = c.adapt(omc0, omc1, o->nmax_theta, 0.0, o->rtol_theta);
    }
    if (result != result || result < 0.0) return 0.;
    if (nevals > (long)1e7) {
      code = PBAG_ERR_EVALS;
      return 0.;
    }
    return result;
  }
  // integrate_theta_phi (eats.h:587-700)
  double theta_phi() {
    nevals = 0;
    double Fcoeff = cgs2mJy / (4 * pi_ * o->d_l * o->d_l);
    auto fph = [&](double x) { return phi_integrand(x); };
    auto st = [&]() { return stop(); };
    if (o->method_quad == PBAG_QUAD_TRAP_FIXED) return 2 * Fcoeff * trap_fixed(fph, st, 0.0, pi_, o->nmax_phi);
    Cadre<decltype(fph), decltype(st)> c{fph, st};
    return 2 * Fcoeff * c.adapt(0.0, pi_, o->nmax_phi, 0.0, o->rtol_phi);
  }
  // parsPars' mu array (eats.h:941-947)
  void set_mu() {
    const double* tb = q(PBAG_EQ_TBURST);
    const double* R = q(PBAG_EQ_R);
    mu.assign((size_t)nr, 0.0);
    for (int i = 0; i < L->i_end_r; i++) mu[i] = (tb[i] - t_obs / (1.0 + o->z)) / R[i] * c_light;
  }
};

}  // namespace

extern "C" int orc_eats_flux(const pbag_grid_desc* g, const pbag_eats_opts* o, int nl, const pbag_eats_layer* layers,
                             int nr, const double* dyn, const int64_t* offsets, const double* j_all,
                             const double* a_all, int nq, const pbag_eats_query* qs, double* flux, int* fail_index) {
  const int F = g->nfreq;
  std::vector<double> gam(g->ngam), nu(F + 1);
  orc_build_grids(g, gam.data(), nu.data());
  *fail_index = -1;
  // the fluxDens radius rows of every history row: the layer's dynamics R
  int64_t nrec = 0;
  for (int l = 0; l < nl; ++l) {
    nrec = std::max<int64_t>(nrec, offsets[layers[l].bw_fs + 1]);
    if (layers[l].bw_rs >= 0) nrec = std::max<int64_t>(nrec, offsets[layers[l].bw_rs + 1]);
  }
  std::vector<double> Rh((size_t)nrec, 0.0);
  for (int l = 0; l < nl; ++l) {
    const double* R = dyn + ((size_t)l * PBAG_EQ_N + PBAG_EQ_R) * nr;
    for (int b : {layers[l].bw_fs, layers[l].bw_rs}) {
      if (b < 0) continue;
      for (int64_t k = 0; k < offsets[b + 1] - offsets[b] && k < nr; ++k) Rh[offsets[b] + k] = R[k];
    }
  }
  for (int t = 0; t < nq; ++t) {
    const pbag_eats_query& qq = qs[t];
    const pbag_eats_layer& L = layers[qq.layer];
    const double* tb = dyn + ((size_t)qq.layer * PBAG_EQ_N + PBAG_EQ_TBURST) * nr;
    if (L.i_end_r > 0 && (qq.t_obs < tb[0] || qq.t_obs > tb[L.i_end_r - 1])) {  // eats.h:822-827
      flux[t] = 0.;
      *fail_index = t;
      return PBAG_ERR_RANGE;
    }
    EatsRun e{o, &L, nr, dyn + (size_t)qq.layer * PBAG_EQ_N * nr, nu.data(), F, j_all, a_all, Rh.data(),
              offsets[L.bw_fs], L.bw_rs >= 0 ? offsets[L.bw_rs] : -1};
    e.t_obs = qq.t_obs;
    e.nu_obs = qq.nu_obs;
    e.set_mu();
    double fd = e.theta_phi();  // evalFluxDensA: the principal jet
    if (o->counter_jet && e.code == PBAG_OK) {
      e.cj = true;
      e.set_mu();
      fd += e.theta_phi();
    }
    flux[t] = fd;
    if (e.code != PBAG_OK) {
      flux[t] = 0.;
      *fail_index = t;
      return e.code;
    }
  }
  return PBAG_OK;
}
