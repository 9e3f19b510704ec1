// pbag_microphysics.hpp - drop-in replacement of the reference's
// ElectronAndRadiation (src/microphysics/microphysics.h:60-1217) for the
// numeric ("numeric" and "mix") electron paths, over the C ABI of pbag.h.
//
// The class keeps the reference's constructor, the public members its callers
// read and the methods they call, so that the blastwave driver's per-step code
// (src/blastwave/blastwave_radiation.h:976-1182) and the consumers of the
// histories (fluxDens for EATS, the spectrum writer of ejecta.h:354-509) work
// unchanged against it:
//
//   ElectronAndRadiation(loglevel, gam_grid, freq_grid, syn_kernel, ssc_kernel, is_rs)   (microphysics.h:94-98)
//   setPars(pars, opts, nr, ish, il, theta_h, tcomov0, do_allocate)                      (microphysics.h:100-131)
//   updateSockProperties(e_prime, Gamma, GammaSh, t_e, t_b, tcomov, n_prime, n_protons)  (microphysics_base.h:575)
//   computeEleSpectrumLimits()                                                            (microphysics_base.h:642)
//   initializeElectronDistribution(tcomov, m2, rho2, u_p, dr)                            (microphysics.h:347)
//   evaluateElectronDistributionNumericMixed(tc, tc_p1, m, m_p1, rho, rho_p1, r, rp1,
//                                            dr, dr_p1, u_p, u_p_p1)                      (microphysics.h:359)
//   computeRadiationNumericMixed(it)                                                      (microphysics.h:492)
//   fluxDens(eats_method, theta, ncells, ia, ib, freq, Gamma, GammaSh, acc_fac, mu, r,
//            rsh, dr, n_prime, ne, r_arr)                                                 (microphysics.h:1185)
//   members B, gamma_min, gamma_max, gamma_c, Theta, z_cool, n_prime, accel_frac, eps_e,
//   beta_min, m_eleMethod, m_methods_ssa/ssc/pp, is_distribution_initialized, and
//   ele / syn / ssc / total_rad with .e, .numbins and the time-major *_all vectors.
//
// What differs is when the work happens. computeEleSpectrumLimits runs on the
// host at once (pbag_shock_limits, so every member a caller reads after it is
// set as in the reference). The Chang-Cooper evolution and the radiation of a
// step are only recorded: every ElectronAndRadiation built on the same
// SSCKernel joins one batch, and SSCKernel::flush() evolves all of them on the
// GPU and fills their *_all vectors (value k of step it at [k + numbins * it],
// as the reference stores them). fluxDens flushes first if steps are pending;
// a caller that reads the vectors directly (the spectrum writer) calls flush()
// once the evolution has finished. Where the reference logs and calls exit(1),
// an implicit flush logs the first failure in time order and exits the same
// way; flush(&status) returns the status to callers that want it instead.
//
// SynKernel and SSCKernel stand where the reference's CommonTables objects are
// passed (microphysics/common.h:93-117): the synchrotron functions and the SSC
// kernel are tabulated once per grid on the device, and the SSCKernel object
// owns that device context and the batch. Header-only; link libpbag. Not
// thread-safe (neither are the reference's shared kernel objects).
#ifndef PBAG_MICROPHYSICS_HPP
#define PBAG_MICROPHYSICS_HPP

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "pbag.h"

namespace pbag {

// the reference's container types (utilitites/utils.h:13-16)
using Vector = std::vector<double>;
using StrDbMap = std::unordered_map<std::string, double>;
using StrStrMap = std::unordered_map<std::string, std::string>;

// option enums of the numeric path, with the reference's names and order
// (microphysics_base.h:30-54)
enum METHODS_SHOCK_ELE { iShockEleAnalyt, iShockEleNum, iShockEleMix };
enum METHOD_TAU { iAPPROX, iTHICK, iSMOOTH, iSHARP };
enum METHOD_SSC { inoSSC, iNumSSC };
enum METHODS_SSA { iSSAoff, iSSAon };
enum METHOD_PP { iPPoff, iPPnum };
enum METHOD_NE { iusenprime, iuseNe };
enum METHODS_SHOCK_VEL { isameAsBW, ishockVel };

// Electrons / Photons (base_state.h:153-300): the grid (shared, by
// reference), its size, the state of the last flushed step and the dense
// time-major histories.
struct Electrons {
  Vector& e;
  size_t numbins = 0;
  Vector f, f_all, gam_dot_syn_all, gam_dot_adi_all, gam_dot_ssc_all;
  explicit Electrons(Vector& grid) : e(grid) {}
};
struct Photons {
  Vector& e;
  size_t numbins = 0;
  Vector f, j, a, intensity, f_all, j_all, a_all, i_all;
  explicit Photons(Vector& grid) : e(grid) {}
};

class ElectronAndRadiation;

// Stand-in for the reference's SynKernel: the synchrotron functions of all
// four methods are tabulated on the device, so nothing lives on the host.
class SynKernel {};

// Stand-in for the reference's SSCKernel (one per grid, shared by every
// blastwave of a shock type): the device context of that grid and the batch
// of every ElectronAndRadiation constructed with it.
class SSCKernel {
 public:
  explicit SSCKernel(int device = 0) : device_(device) {}
  ~SSCKernel() {
    if (ctx_) pbag_destroy(ctx_);
  }
  SSCKernel(const SSCKernel&) = delete;
  SSCKernel& operator=(const SSCKernel&) = delete;

  // Evolve every recorded step of every member on the GPU and fill their
  // histories. Returns PBAG_OK or the first failure in time order (blastwave =
  // index of the member in construction order, step = time index).
  inline int flush(pbag_status* st = nullptr);
  // Steps recorded since the last flush.
  bool pending() const { return pending_; }
  pbag_ctx* context() const { return ctx_; }

 private:
  friend class ElectronAndRadiation;
  int device_;
  pbag_ctx* ctx_ = nullptr;
  pbag_grid_desc grid_{};
  bool have_grid_ = false, ctx_ssc_ = false, pending_ = false;
  std::vector<ElectronAndRadiation*> members_;
};

class ElectronAndRadiation {
 public:
  // ---- members the reference's callers read (microphysics_base.h:59-120) ----
  Vector& freqs_grid;
  Vector& gams_grid;
  Electrons ele{gams_grid};
  Photons syn{freqs_grid};
  Photons ssc{freqs_grid};
  Photons total_rad{freqs_grid};
  double B = -1, gamma_min = -1, gamma_max = -1, gamma_c = -1;
  double n_prime = -1, n_protons = -1, nn = -1;
  double eprime = -1., Gamma = -1, GammaSh = -1, betaSh = -1., t_e = -1., t_b = -1., tcomov = -1.;
  double accel_frac = 1.;
  double Theta = -1, z_cool = -1;
  double eps_e = -1, eps_b = -1, eps_t = 0, p = -1, beta_min = -1;
  size_t max_substeps = 0;
  METHOD_TAU method_tau = iSMOOTH;
  METHODS_SHOCK_ELE m_eleMethod = iShockEleAnalyt;
  bool num_ele_use_adi_loss = true;
  METHOD_NE m_method_ne = iuseNe;
  METHODS_SHOCK_VEL method_shock_vel = isameAsBW;
  METHODS_SSA m_methods_ssa = iSSAoff;
  METHOD_SSC m_methods_ssc = inoSSC;
  METHOD_PP m_methods_pp = iPPoff;
  bool is_distribution_initialized = false;
  bool is_rs = false;
  bool is_dense_output = false;
  double freq1 = 0, freq2 = 0, gam1 = 0, gam2 = 0;
  size_t nfreq = 0, ngam = 0;

  ElectronAndRadiation(int loglevel, Vector& gam_grid, Vector& freq_grid, SynKernel& syn_kernel,
                       SSCKernel& ssc_kernel, bool _is_rs)
      : freqs_grid(freq_grid), gams_grid(gam_grid), is_rs(_is_rs), loglevel_(loglevel), ssc_kernel_(ssc_kernel) {
    (void)syn_kernel;
    ssc_kernel_.members_.push_back(this);
  }
  ~ElectronAndRadiation() {
    auto& m = ssc_kernel_.members_;
    for (size_t i = 0; i < m.size(); ++i)
      if (m[i] == this) {
        m.erase(m.begin() + (long)i);
        break;
      }
  }
  ElectronAndRadiation(const ElectronAndRadiation&) = delete;
  ElectronAndRadiation& operator=(const ElectronAndRadiation&) = delete;

  // setBasePars + setPars (microphysics_base.h:140-575, microphysics.h:100-131):
  // the parameters and options the numeric path reads, with the reference's
  // names, suffixes (_fs / _rs) and defaults; nr burster times are allocated.
  void setPars(StrDbMap& pars, StrStrMap& opts, size_t nr, size_t ish, size_t il, double theta_h, double tcomov0,
               bool do_allocate) {
    (void)ish;
    (void)il;
    (void)theta_h;
    if (tcomov0 <= 0.) die("Bad value: tcomov=" + std::to_string(tcomov0));
    const std::string s = is_rs ? "_rs" : "_fs";
    eps_e = par(pars, "eps_e" + s, -1, true);
    eps_b = par(pars, "eps_b" + s, -1, true);
    eps_t = par(pars, "eps_t" + s, 0., true);
    p = par(pars, "p" + s, -1, true);
    beta_min = par(pars, "beta_min" + s, 1.e-5, false);
    gamma_max = par(pars, "gamma_max" + s, 1.e7, false);
    max_substeps = (size_t)par(pars, "max_substeps" + s, 1000, false);
    const std::string ele_m = opt(opts, "method_ele" + s, "analytic", {"analytic", "numeric", "mix"});
    m_eleMethod = ele_m == "numeric" ? iShockEleNum : ele_m == "mix" ? iShockEleMix : iShockEleAnalyt;
    if (m_eleMethod == iShockEleAnalyt)
      die("method_ele" + s + " = analytic: this class replaces the numeric and mix paths only");
    num_ele_use_adi_loss = yes(opts, "num_ele_use_adi_loss" + s, true);
    const std::string ne = opt(opts, "method_ne" + s, "useNe", {"useNe", "usenprime"});
    m_method_ne = ne == "usenprime" ? iusenprime : iuseNe;
    const std::string vel = opt(opts, "method_vel" + s, "sameAsBW", {"sameAsBW", "shockVel"});
    method_shock_vel = vel == "shockVel" ? ishockVel : isameAsBW;
    const std::string synm = opt(opts, "method_synchrotron" + s, "CSYN", {"CSYN", "Dermer09", "GSL", "Bessel"});
    syn_method_ = synm == "Dermer09" ? PBAG_SYN_DER09 : synm == "GSL" ? PBAG_SYN_GSL
                  : synm == "Bessel" ? PBAG_SYN_BESSEL : PBAG_SYN_CSYN;
    m_methods_ssc = opt(opts, "method_ssc" + s, "none", {"none", "numeric"}) == "numeric" ? iNumSSC : inoSSC;
    m_methods_pp = opt(opts, "method_pp" + s, "none", {"none", "numeric"}) == "numeric" ? iPPnum : iPPoff;
    if (m_methods_pp == iPPnum && m_methods_ssc == inoSSC) die("method_pp" + s + " = numeric requires SSC");
    const std::string nr_m =
        opt(opts, "method_nonrel_dist" + s, "none", {"none", "use_gamma_min", "use_Ayache", "use_Sironi"});
    lim_.method_nonrel = nr_m == "use_gamma_min" ? 1 : nr_m == "use_Ayache" ? 2 : nr_m == "use_Sironi" ? 3 : 0;
    const std::string gmin =
        opt(opts, "method_gamma_min" + s, "useU_e", {"useU_e", "useNumeric", "useBeta", "useGamma", "useTheta"});
    lim_.method_gamma_min = gmin == "useNumeric" ? 1 : gmin == "useBeta" ? 2 : gmin == "useGamma" ? 3
                            : gmin == "useTheta" ? 4 : 0;
    const std::string bm = opt(opts, "method_B" + s, "useU_b", {"useU_b", "useMAG21", "useGammaSh"});
    lim_.method_B = bm == "useMAG21" ? 1 : bm == "useGammaSh" ? 2 : 0;
    const std::string gmax = opt(opts, "method_gamma_max" + s, "useB", {"useB", "useConst"});
    lim_.method_gamma_max = gmax == "useConst" ? 1 : 0;
    if (lim_.method_gamma_max == 1) gamma_max = par(pars, "gamma_max" + s, 1.e7, true);
    const std::string gc = opt(opts, "method_gamma_c" + s, "useTe", {"useTe", "useTcomov", "useConst"});
    lim_.method_gamma_c = gc == "useTcomov" ? 1 : gc == "useConst" ? 2 : 0;
    if (lim_.method_gamma_c == 2) gamma_c = par(pars, "gamma_c" + s, 1.e5, true);
    m_methods_ssa = yes(opts, "use_ssa" + s, false) ? iSSAon : iSSAoff;
    const std::string tau = opt(opts, "method_tau" + s, "smooth", {"thick", "sharp", "smooth", "approx"});
    method_tau = tau == "thick" ? iTHICK : tau == "sharp" ? iSHARP : tau == "approx" ? iAPPROX : iSMOOTH;
    lim_.p = p, lim_.eps_e = eps_e, lim_.eps_b = eps_b, lim_.eps_t = eps_t;
    lim_.beta_min = beta_min, lim_.mu = 0.62, lim_.mu_e = 1.18, lim_.ele_analytic = 0;
    freq1 = par(pars, "freq1" + s, 1.e7, true);
    freq2 = par(pars, "freq2" + s, 1.e28, true);
    nfreq = (size_t)par(pars, "nfreq" + s, 200, true);
    is_dense_output = yes(opts, "save_spec", false);
    if (do_allocate) allocate(pars, s, nr);
  }

  // updateSockProperties (microphysics_base.h:575-605)
  void updateSockProperties(double e_prime, double Gamma_, double Gamma_shock, double t_e_, double t_b_,
                            double tcomov_, double n_prime_, double n_protons_) {
    GammaSh = Gamma_shock;
    eprime = e_prime;
    Gamma = Gamma_;
    betaSh = std::sqrt((Gamma_shock - 1.) * (Gamma_shock + 1.)) / Gamma_shock;
    t_e = t_e_;
    t_b = t_b_;
    tcomov = tcomov_;
    n_prime = n_prime_;
    n_protons = n_protons_;
    nn = m_method_ne == iusenprime ? n_prime : n_protons;
  }

  // computeEleSpectrumLimits (microphysics_base.h:642-966), on the host
  void computeEleSpectrumLimits() {
    pbag_shock_state in{eprime, Gamma, GammaSh, t_e, t_b, tcomov, n_prime, n_protons};
    double state[7] = {gamma_min, gamma_max, gamma_c, accel_frac, B, Theta, z_cool};
    pbag_limits out{};
    const int rc = pbag_shock_limits(&lim_, gams_grid.data(), (int)gams_grid.size(), 1, &in, state, &out);
    if (rc != PBAG_OK) die(std::string("computeEleSpectrumLimits: ") + pbag_status_string(rc));
    if (!out.valid) return;  // checkParams() refused: nothing recomputed
    B = out.B, gamma_min = out.gamma_min, gamma_max = out.gamma_max, gamma_c = out.gamma_c;
    accel_frac = out.accel_frac, Theta = out.Theta, z_cool = out.z_cool;
  }

  // initializeElectronDistribution (microphysics.h:347-357): recorded
  void initializeElectronDistribution(double tcomov_, double m2, double rho2, double u_p, double dr_comov) {
    next_ = pbag_step_rec{};
    next_.mode = PBAG_INIT;
    next_.tc_p1 = tcomov_;
    next_.m_p1 = m2;
    next_.rho_p1 = rho2;
    next_.u_p_p1 = u_p;
    next_.dr = dr_comov;
    scalars(next_);
    have_next_ = true;
    is_distribution_initialized = true;
  }

  // evaluateElectronDistributionNumericMixed (microphysics.h:359-489): recorded
  void evaluateElectronDistributionNumericMixed(double tc, double tc_p1, double m, double m_p1, double rho_prime,
                                                double rho_prime_p1, double r, double rp1, double dr_comov_,
                                                double drp1_comov, double u_p, double u_p_p1) {
    (void)r;
    (void)rp1;
    if (gams_grid.empty()) die("electon grid is not initialized");
    next_ = pbag_step_rec{};
    next_.mode = PBAG_EVOLVE;
    next_.tc = tc, next_.tc_p1 = tc_p1, next_.m = m, next_.m_p1 = m_p1;
    next_.rho = rho_prime, next_.rho_p1 = rho_prime_p1, next_.dr = dr_comov_, next_.dr_p1 = drp1_comov;
    next_.u_p = u_p, next_.u_p_p1 = u_p_p1;
    scalars(next_);
    have_next_ = true;
  }

  // computeRadiationNumericMixed (microphysics.h:492-599): the recorded step
  // is stored at time index it; its results appear at the next flush
  void computeRadiationNumericMixed(size_t it) {
    if (!have_next_) die("computeRadiationNumericMixed: no electron step recorded before it");
    if (it >= recs_.size()) die("computeRadiationNumericMixed: it beyond the allocated burster times");
    recs_[it] = next_;
    have_next_ = false;
    ssc_kernel_.pending_ = true;
  }

  // fluxDens (microphysics.h:1185-1217) with computeFluxDensity (:799-867),
  // on the flushed histories; eats_method is not used by either
  double fluxDens(int eats_method, double theta, double ncells, size_t ia, size_t ib, double freq, double Gamma_,
                  double GammaSh_, double acc_fac, double mu, double r, double rsh, double dr, double n_prime_,
                  double ne, const Vector& r_arr) {
    (void)eats_method;
    (void)acc_fac;
    (void)rsh;
    (void)dr;
    if (ssc_kernel_.pending_) {
      pbag_status st{};
      if (ssc_kernel_.flush(&st) != PBAG_OK) die_status(st);
    }
    const Vector& nu = total_rad.e;
    const size_t F = total_rad.numbins;
    if (freq >= nu[F - 1]) die("freq_prime > grid freq[-1]: increase 'freq2' parameter");
    if (freq <= nu[0]) die("freq_prime < grid freq[0]: decrease 'freq1' parameter");
    size_t lo = 0, hi = F - 1;  // findIndex (interpolators.h:13-35)
    while (hi - lo > 1) {
      const size_t m = (lo + hi) >> 1;
      if (nu[m] > freq) hi = m; else lo = m;
    }
    const size_t ka = lo, kb = lo + 1;
    auto bilin = [&](const Vector& h) {  // Interp2d::InterpolateBilinear (interpolators.h:708-801)
      const double x1 = nu[ka], x2 = nu[kb], y1 = r_arr[ia], y2 = r_arr[ib];
      const double q11 = h[ka + F * ia], q12 = h[ka + F * ib], q21 = h[kb + F * ia], q22 = h[kb + F * ib];
      const double x2x1 = x2 - x1, y2y1 = y2 - y1, x2x = x2 - freq, y2y = y2 - r, yy1 = r - y1, xx1 = freq - x1;
      return 1.0 / (x2x1 * y2y1) * (q11 * x2x * y2y + q21 * xx1 * y2y + q12 * x2x * yy1 + q22 * xx1 * yy1);
    };
    const double em_prime = bilin(total_rad.j_all), abs_prime = bilin(total_rad.a_all);
    const double pi_ = 3.141592653589793, m_p = 1.6726e-24;
    const double beta = std::sqrt((Gamma_ - 1.) * (Gamma_ + 1.)) / Gamma_;
    const double delta_D = Gamma_ * (1.0 - beta * mu);
    const double em_lab = em_prime / (delta_D * delta_D), abs_lab = abs_prime * delta_D;
    const double gsh = method_shock_vel == ishockVel ? GammaSh_ : Gamma_;
    const double beta_shock = std::sqrt((gsh - 1.) * (gsh + 1.)) / gsh;
    const double dr_ = ne * m_p / (2. * pi_ * m_p * r * r * (1. - std::cos(theta) / ncells) * Gamma_ * n_prime_);
    const double dtau = mu == beta_shock ? 1.0e100 : abs_lab * dr_ * (1. - mu * beta_shock) / (mu - beta_shock);
    const double intensity = intensity_of(em_lab, dtau);
    if (intensity < 0 || !std::isfinite(intensity)) die("intensity < 0 or nan");
    const double ashock = 1.0 - mu * beta_shock;
    const double lum = m_method_ne == iusenprime
                           ? intensity * r * r * (dr_ / ashock)
                           : intensity * ne / (2. * pi_ * (1. - std::cos(theta) / ncells)) / Gamma_ / ashock;
    if (lum < 0 || !std::isfinite(lum)) die("luminosity < 0 or nan");
    return lum;
  }

  // this blastwave's step records (diagnostics, tests)
  const std::vector<pbag_step_rec>& records() const { return recs_; }
  int loglevel() const { return loglevel_; }

 private:
  friend class SSCKernel;
  int loglevel_;
  SSCKernel& ssc_kernel_;
  pbag_limits_opts lim_{};
  int syn_method_ = PBAG_SYN_CSYN;
  size_t nr_ = 0;
  std::vector<pbag_step_rec> recs_;
  pbag_step_rec next_{};
  bool have_next_ = false;

  [[noreturn]] void die(const std::string& msg) const {
    std::fprintf(stderr, "ElectronAndRadiation%s: %s\n", is_rs ? "[rs]" : "[fs]", msg.c_str());
    std::exit(1);
  }
  [[noreturn]] void die_status(const pbag_status& st) const {
    die(std::string(pbag_status_string(st.code)) + " at blastwave " + std::to_string(st.bw) + " step " +
        std::to_string(st.step));
  }
  double par(StrDbMap& pars, const std::string& k, double def, bool required) const {
    auto it = pars.find(k);
    if (it != pars.end()) return it->second;
    if (required && def < 0) die("Required parameter " + k + " not found");
    return def;
  }
  std::string opt(StrStrMap& opts, const std::string& k, const std::string& def,
                  std::initializer_list<const char*> allowed) const {
    auto it = opts.find(k);
    if (it == opts.end()) return def;
    for (const char* a : allowed)
      if (it->second == a) return it->second;
    die("option for: " + k + " given: " + it->second + " is not recognized");
  }
  bool yes(StrStrMap& opts, const std::string& k, bool def) const {
    auto it = opts.find(k);
    if (it == opts.end()) return def;
    if (it->second == "yes") return true;
    if (it->second == "no") return false;
    die("option for: " + k + " given: " + it->second + " is not recognized (yes / no)");
  }
  void scalars(pbag_step_rec& q) const {
    q.B = B, q.gamma_min = gamma_min, q.gamma_max = gamma_max, q.gamma_c = gamma_c;
    q.accel_frac = accel_frac, q.n_prime = n_prime;
  }
  double intensity_of(double em, double dtau) const {  // computeIntensity (microphysics.h:11-58)
    if (dtau == 0) return em;
    switch (method_tau) {
      case iTHICK: return dtau > 0 ? em / dtau : 0.;
      case iSMOOTH: return em * (dtau > 0.0 ? -std::expm1(-dtau) / dtau : std::expm1(dtau) / dtau);
      case iSHARP: return dtau > 1.0 ? em / dtau : dtau < -1.0 ? 0.0 : em;
      default: {
        if (!(dtau > 1.e-3)) return em;
        const double e = std::exp(-dtau);
        const double u = 1. / 2. + e / dtau - (1 - e) / (dtau * dtau);
        return em * (3. * u / dtau);
      }
    }
  }
  // allocateForNumericSpectra (microphysics.h:282-345): grids and histories
  void allocate(StrDbMap& pars, const std::string& s, size_t nr) {
    gam1 = par(pars, "gam1" + s, 1, true);
    gam2 = par(pars, "gam2" + s, 1.e8, true);
    ngam = (size_t)par(pars, "ngam" + s, 250, true);
    pbag_grid_desc g{(int32_t)ngam, (int32_t)nfreq, gam1, gam2, freq1, freq2};
    std::vector<double> gam(ngam), freq(nfreq + 1);
    if (pbag_build_grids(&g, gam.data(), freq.data()) != PBAG_OK) die("bad electron or photon grid");
    gams_grid.assign(gam.begin(), gam.end());
    freqs_grid.assign(freq.begin(), freq.end() - 1);
    SSCKernel& k = ssc_kernel_;
    if (k.have_grid_ && (k.grid_.ngam != g.ngam || k.grid_.nfreq != g.nfreq || k.grid_.gam1 != g.gam1 ||
                         k.grid_.gam2 != g.gam2 || k.grid_.freq1 != g.freq1 || k.grid_.freq2 != g.freq2))
      die("every blastwave of one SSCKernel must share its grid");
    k.grid_ = g;
    k.have_grid_ = true;
    nr_ = nr;
    ele.numbins = ngam;
    syn.numbins = ssc.numbins = total_rad.numbins = nfreq;
    ele.f.assign(ngam, 0.);
    for (Photons* ph : {&syn, &ssc, &total_rad}) {
      ph->f.assign(nfreq, 0.), ph->j.assign(nfreq, 0.), ph->a.assign(nfreq, 0.), ph->intensity.assign(nfreq, 0.);
    }
    total_rad.f_all.assign(nfreq * nr, 0.), total_rad.j_all.assign(nfreq * nr, 0.);
    total_rad.a_all.assign(nfreq * nr, 0.), total_rad.i_all.assign(nfreq * nr, 0.);
    if (is_dense_output) {
      ele.f_all.assign(ngam * nr, 0.), ele.gam_dot_syn_all.assign(ngam * nr, 0.);
      ele.gam_dot_adi_all.assign(ngam * nr, 0.), ele.gam_dot_ssc_all.assign(ngam * nr, 0.);
      syn.f_all.assign(nfreq * nr, 0.), syn.j_all.assign(nfreq * nr, 0.);
      syn.a_all.assign(nfreq * nr, 0.), syn.i_all.assign(nfreq * nr, 0.);
      if (m_methods_ssc == iNumSSC) {
        ssc.f_all.assign(nfreq * nr, 0.), ssc.j_all.assign(nfreq * nr, 0.);
        ssc.a_all.assign(nfreq * nr, 0.), ssc.i_all.assign(nfreq * nr, 0.);
      }
    }
    recs_.assign(nr, pbag_step_rec{});  // PBAG_SKIP until recorded
  }
  pbag_shock_params params() const {
    pbag_shock_params q{};
    q.p = p, q.eps_e = eps_e, q.max_substeps = (int32_t)max_substeps;
    q.ele_method = m_eleMethod == iShockEleMix ? PBAG_ELE_MIX : PBAG_ELE_NUMERIC;
    q.syn_method = syn_method_;
    q.ssa_on = m_methods_ssa == iSSAon, q.ssc_on = m_methods_ssc == iNumSSC;
    q.adi_on = num_ele_use_adi_loss, q.pp_on = m_methods_pp == iPPnum;
    return q;
  }
  // copies rows [row0, row0 + nr) of a batch history into a member's vector
  void take(const std::vector<double>& src, size_t row0, size_t n, Vector& dst) const {
    if (src.empty() || dst.size() != n * nr_) return;
    std::copy(src.begin() + (long)(row0 * n), src.begin() + (long)((row0 + nr_) * n), dst.begin());
  }
  // the state of the last step with a record (the reference's current vectors)
  void take_last(const std::vector<double>& src, size_t row0, size_t n, Vector& dst) const {
    size_t last = nr_;
    for (size_t it = nr_; it-- > 0;)
      if (recs_[it].mode != PBAG_SKIP) {
        last = it;
        break;
      }
    if (src.empty() || last == nr_ || dst.size() != n) return;
    std::copy(src.begin() + (long)((row0 + last) * n), src.begin() + (long)((row0 + last + 1) * n), dst.begin());
  }
};

inline int SSCKernel::flush(pbag_status* st) {
  pbag_status local{};
  pbag_status& s = st ? *st : local;
  s = pbag_status{PBAG_OK, -1, -1, 0};
  if (members_.empty()) return PBAG_OK;
  if (!have_grid_) return s.code = PBAG_ERR_ARG;
  bool want_ssc = false, dense = false;
  for (const ElectronAndRadiation* m : members_) {
    want_ssc = want_ssc || m->m_methods_ssc == iNumSSC;
    dense = dense || m->is_dense_output;
  }
  if (ctx_ && want_ssc && !ctx_ssc_) {
    pbag_destroy(ctx_);
    ctx_ = nullptr;
  }
  if (!ctx_) {
    const int rc = pbag_create(&grid_, device_, want_ssc ? 1 : 0, &ctx_);
    if (rc != PBAG_OK) return s.code = rc;
    ctx_ssc_ = want_ssc;
  }
  std::vector<pbag_shock_params> prm;
  std::vector<int64_t> off{0};
  std::vector<pbag_step_rec> recs;
  for (const ElectronAndRadiation* m : members_) {
    prm.push_back(m->params());
    recs.insert(recs.end(), m->recs_.begin(), m->recs_.end());
    off.push_back((int64_t)recs.size());
  }
  const size_t nrec = recs.size(), F = (size_t)grid_.nfreq, G = (size_t)grid_.ngam;
  // one batch history per output; the dense ones only when a member keeps them
  std::vector<double> h[13];
  pbag_outputs out{};
  double** slot = reinterpret_cast<double**>(&out);
  for (int k = 0; k < 13; ++k) {
    if (k >= 4 && !dense) continue;
    h[k].assign(nrec * ((k >= 4 && k < 8) ? G : F), 0.);
    slot[k] = h[k].data();
  }
  const int rc = pbag_run_batch(ctx_, prm.data(), (int)prm.size(), off.data(), recs.data(), &out, &s);
  for (size_t b = 0; b < members_.size(); ++b) {
    ElectronAndRadiation& m = *members_[b];
    const size_t r0 = (size_t)off[b];
    m.take(h[0], r0, F, m.total_rad.j_all);
    m.take(h[1], r0, F, m.total_rad.a_all);
    m.take(h[2], r0, F, m.total_rad.f_all);
    m.take(h[3], r0, F, m.total_rad.i_all);
    m.take_last(h[0], r0, F, m.total_rad.j);
    m.take_last(h[1], r0, F, m.total_rad.a);
    m.take_last(h[2], r0, F, m.total_rad.f);
    m.take_last(h[3], r0, F, m.total_rad.intensity);
    if (m.is_dense_output) {
      m.take(h[4], r0, G, m.ele.f_all);
      m.take(h[5], r0, G, m.ele.gam_dot_syn_all);
      m.take(h[6], r0, G, m.ele.gam_dot_adi_all);
      m.take(h[7], r0, G, m.ele.gam_dot_ssc_all);
      m.take(h[8], r0, F, m.syn.j_all);
      m.take(h[9], r0, F, m.syn.a_all);
      m.take(h[10], r0, F, m.syn.i_all);
      m.take(h[11], r0, F, m.ssc.j_all);
      m.take(h[12], r0, F, m.ssc.i_all);
      m.take_last(h[4], r0, G, m.ele.f);
    }
  }
  pending_ = false;
  return rc;
}

}  // namespace pbag

#endif
