// ref_driver.cpp - drives the REFERENCE's own microphysics code (compiled in
// place from its headers) so that its outputs can pin the oracle restatement and
// produce golden fixtures.
//
// Test infrastructure only: built by oracle/Makefile into oracle/_ref/libpbaref.so
// when the reference sources are present. Nothing in the product links it.
//
// The reference classes used are ElectronAndRadiation (src/microphysics/
// microphysics.h:60), SynKernel and SSCKernel (src/microphysics/kernels.h:17,175)
// and the per-step scalar prep in ElectronAndRadiaionBase
// (src/microphysics/microphysics_base.h:575-966).
#include "pbag.h"

// The only ejecta type microphysics.h needs (computeFluxDensity signature).
struct EjectaID2 {
  enum STUCT_TYPE { iadaptive, ipiecewise };
};
#include "microphysics/microphysics.h"

#include <cstring>

namespace {

StrDbMap make_pars(const pbag_grid_desc* g, const pbag_shock_params* s, double eps_b) {
  StrDbMap pars;
  pars["eps_e_fs"] = s->eps_e > 0 ? s->eps_e : 0.1;
  pars["eps_b_fs"] = eps_b;
  pars["eps_t_fs"] = 0.;
  pars["p_fs"] = s->p;
  pars["max_substeps_fs"] = (double)s->max_substeps;
  pars["gam1_fs"] = g->gam1;
  pars["gam2_fs"] = g->gam2;
  pars["ngam_fs"] = (double)g->ngam;
  pars["freq1_fs"] = g->freq1;
  pars["freq2_fs"] = g->freq2;
  pars["nfreq_fs"] = (double)g->nfreq;
  return pars;
}

const char* syn_name(int m) {
  switch (m) {
    case PBAG_SYN_DER09: return "Dermer09";
    case PBAG_SYN_GSL: return "GSL";
    case PBAG_SYN_BESSEL: return "Bessel";
    default: return "CSYN";
  }
}

StrStrMap make_opts(const pbag_shock_params* s, bool dense, const char* lfmin, const char* lfcool,
                    const char* lfmax, const char* bmeth, const char* nonrel) {
  StrStrMap opts;
  opts["method_ele_fs"] = s->ele_method == PBAG_ELE_MIX ? "mix" : "numeric";
  opts["method_synchrotron_fs"] = syn_name(s->syn_method);
  opts["method_ssc_fs"] = s->ssc_on ? "numeric" : "none";
  opts["method_pp_fs"] = s->pp_on ? "numeric" : "none";
  opts["use_ssa_fs"] = s->ssa_on ? "yes" : "no";
  opts["num_ele_use_adi_loss_fs"] = s->adi_on ? "yes" : "no";
  opts["save_spec"] = dense ? "yes" : "no";
  opts["method_ne_fs"] = "useNe";
  opts["method_vel_fs"] = "shockVel";
  opts["method_Up_fs"] = "useEint2";
  opts["method_thickness_fs"] = "useJoh06";
  opts["method_tau_fs"] = "approx";
  opts["method_gamma_min_fs"] = lfmin;
  opts["method_gamma_c_fs"] = lfcool;
  opts["method_gamma_max_fs"] = lfmax;
  opts["method_B_fs"] = bmeth;
  opts["method_nonrel_dist_fs"] = nonrel;
  return opts;
}

// The reference reads freqs[F] one past the end in computeSSCSpectrum
// (numeric_model.h:269-272). Make that read deterministic: build the grid the
// way allocateBase would (utils.h MakeLogspaceVec), then park the next
// logspace point in the spare capacity slot.
void make_freq_grid(const pbag_grid_desc* g, Vector& freq) {
  freq = TOOLS::MakeLogspaceVec(std::log10(g->freq1), std::log10(g->freq2), g->nfreq);
  double base = std::pow(10., (std::log10(g->freq2) - std::log10(g->freq1)) / g->nfreq);
  double extra = freq.back() * base;
  freq.reserve(freq.size() + 1);
  freq.push_back(extra);
  freq.pop_back();
}

void copy_rows(double* dst, const Vector& src, size_t nrow, size_t n) {
  if (!dst) return;
  std::memcpy(dst, src.data(), sizeof(double) * nrow * n);
}

}  // namespace

extern "C" {

// Grids exactly as the reference builds them for one CommonTables entry.
int ref_grids(const pbag_grid_desc* g, double* gam_out, double* freq_out, double* freq_extra) {
  Vector freq;
  make_freq_grid(g, freq);
  for (int i = 0; i < g->nfreq; ++i) freq_out[i] = freq[i];
  if (freq_extra) *freq_extra = freq.data()[g->nfreq];
  Vector gam;
  Electrons ele(gam);
  ele.allocate(g->gam1, g->gam2, (size_t)g->ngam, 1, false);
  ele.build_grid_chang_cooper();
  for (int i = 0; i < g->ngam; ++i) gam_out[i] = gam[i];
  return 0;
}

// Synchrotron kernel function values K(nu_k, gamma_j; B), [nfreq][ngam].
int ref_syn_kernel(int method, double B, const double* gam, int ngam, const double* freq, int nfreq,
                   double* out) {
  double (*fn)(double, double, double) = SynKernel::cycSynch;
  if (method == PBAG_SYN_DER09) fn = SynKernel::synchDermer;
  if (method == PBAG_SYN_GSL) fn = SynKernel::synchGSL;
  if (method == PBAG_SYN_BESSEL) fn = SynKernel::synchBessel;
  for (int k = 0; k < nfreq; ++k)
    for (int j = 0; j < ngam; ++j) out[(size_t)k * ngam + j] = fn(B, freq[k], gam[j]);
  return 0;
}

// SSC kernel K[i][j][k] = sscNava(nu_i, gamma_j, nu_k) and its integral
// Kint[j][k] (kernels.h:49-117).
int ref_ssc_kernel(const double* gam, int ngam, const double* freq, int nfreq, double* K,
                   double* Kint) {
  Vector e(gam, gam + ngam), f(freq, freq + nfreq), f2(freq, freq + nfreq);
  SSCKernel k;
  k.allocate((size_t)ngam, (size_t)nfreq, (size_t)nfreq, SSCKernel::sscNava);
  k.evalSSCkernel(e, f, f2);
  const auto& kk = k.getKernel();
  const auto& ki = k.getKernelInteg();
  for (int i = 0; i < nfreq; ++i)
    for (int j = 0; j < ngam; ++j)
      for (int l = 0; l < nfreq; ++l)
        if (K) K[((size_t)i * ngam + j) * nfreq + l] = kk[i][j][l];
  for (int j = 0; j < ngam; ++j)
    for (int l = 0; l < nfreq; ++l) Kint[(size_t)j * nfreq + l] = ki[j][l];
  return 0;
}

// Per-step scalar prep (microphysics_base.h:575-966) for a sequence of shock
// states on one object. in: [n][8] = e_prime, Gamma, GammaSh, t_e, t_b, tcomov,
// n_prime, n_protons. out: [n][8] = B, gamma_min, gamma_max, gamma_c,
// accel_frac, Theta, z_cool, valid(1/0).
int ref_ele_limits(const pbag_grid_desc* g, double p, double eps_e, double eps_b, double eps_t,
                   int lfmin, int lfcool, int lfmax, int bmeth, int nonrel, double gamma_max_const,
                   double gamma_c_const, int n, const double* in, double* out) {
  static const char* lfmin_s[] = {"useU_e", "useNumeric", "useBeta", "useGamma", "useTheta"};
  static const char* lfcool_s[] = {"useTe", "useTcomov", "useConst"};
  static const char* lfmax_s[] = {"useB", "useConst"};
  static const char* b_s[] = {"useU_b", "useMAG21", "useGammaSh"};
  static const char* nr_s[] = {"none", "use_gamma_min", "use_Ayache", "use_Sironi"};
  pbag_shock_params s{};
  s.p = p;
  s.eps_e = eps_e;
  s.max_substeps = 1000;
  s.ele_method = PBAG_ELE_NUMERIC;
  s.ssc_on = 0;
  s.ssa_on = 0;
  s.adi_on = 1;
  StrDbMap pars = make_pars(g, &s, eps_b);
  pars["eps_t_fs"] = eps_t;
  pars["gamma_max_fs"] = gamma_max_const;
  pars["gamma_c_fs"] = gamma_c_const;
  StrStrMap opts = make_opts(&s, false, lfmin_s[lfmin], lfcool_s[lfcool], lfmax_s[lfmax], b_s[bmeth],
                             nr_s[nonrel]);
  Vector gam, freq;
  make_freq_grid(g, freq);
  SynKernel sk;
  SSCKernel ck;
  ElectronAndRadiation er(LOG_SILENT, gam, freq, sk, ck, false);
  er.setPars(pars, opts, 1, 0, 0, 0.1, 1.0, true);
  for (int i = 0; i < n; ++i) {
    const double* a = in + (size_t)i * 8;
    er.updateSockProperties(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]);
    bool valid = er.betaSh >= er.beta_min;
    er.computeEleSpectrumLimits();
    double* o = out + (size_t)i * 8;
    o[0] = er.B;
    o[1] = er.gamma_min;
    o[2] = er.gamma_max;
    o[3] = er.gamma_c;
    o[4] = er.accel_frac;
    o[5] = er.Theta;
    o[6] = er.z_cool;
    o[7] = valid ? 1. : 0.;
  }
  return 0;
}

// Full per-blastwave histories through ElectronAndRadiation, one object per
// blastwave, all sharing one grid and one pair of kernels like CommonTables.
// offsets[nbw+1] index recs; output row r belongs to record r.
int ref_run(const pbag_grid_desc* g, const pbag_shock_params* prm, int nbw, const int64_t* offsets,
            const pbag_step_rec* recs, pbag_outputs* out) {
  Vector gam, freq;
  make_freq_grid(g, freq);
  SynKernel sk;
  SSCKernel ck;
  const bool dense = out->ele_f_all || out->syn_j_all || out->ssc_j_all || out->gdot_syn_all;
  const size_t F = (size_t)g->nfreq, G = (size_t)g->ngam;
  for (int b = 0; b < nbw; ++b) {
    const pbag_shock_params* s = prm + b;
    size_t r0 = (size_t)offsets[b], nr = (size_t)(offsets[b + 1] - offsets[b]);
    if (nr == 0) continue;
    StrDbMap pars = make_pars(g, s, 1e-3);
    StrStrMap opts = make_opts(s, dense, "useU_e", "useTe", "useB", "useU_b", "none");
    ElectronAndRadiation er(LOG_SILENT, gam, freq, sk, ck, false);
    er.setPars(pars, opts, nr, 0, (size_t)b, 0.1, 1.0, true);
    for (size_t it = 0; it < nr; ++it) {
      const pbag_step_rec& q = recs[r0 + it];
      if (q.mode == PBAG_SKIP) continue;
      er.B = q.B;
      er.gamma_min = q.gamma_min;
      er.gamma_max = q.gamma_max;
      er.gamma_c = q.gamma_c;
      er.accel_frac = q.accel_frac;
      er.n_prime = q.n_prime;
      if (!er.is_distribution_initialized)
        er.initializeElectronDistribution(q.tc_p1, q.m_p1, q.rho_p1, q.u_p_p1, q.dr);
      else
        er.evaluateElectronDistributionNumericMixed(q.tc, q.tc_p1, q.m, q.m_p1, q.rho, q.rho_p1, 0., 0.,
                                                    q.dr, q.dr_p1, q.u_p, q.u_p_p1);
      er.computeRadiationNumericMixed(it);
    }
    auto off = [&](double* p, size_t n) { return p ? p + r0 * n : nullptr; };
    copy_rows(off(out->j_all, F), er.total_rad.j_all, nr, F);
    copy_rows(off(out->a_all, F), er.total_rad.a_all, nr, F);
    copy_rows(off(out->f_all, F), er.total_rad.f_all, nr, F);
    copy_rows(off(out->i_all, F), er.total_rad.i_all, nr, F);
    if (dense) {
      copy_rows(off(out->ele_f_all, G), er.ele.f_all, nr, G);
      copy_rows(off(out->gdot_syn_all, G), er.ele.gam_dot_syn_all, nr, G);
      copy_rows(off(out->gdot_adi_all, G), er.ele.gam_dot_adi_all, nr, G);
      copy_rows(off(out->gdot_ssc_all, G), er.ele.gam_dot_ssc_all, nr, G);
      copy_rows(off(out->syn_j_all, F), er.syn.j_all, nr, F);
      copy_rows(off(out->syn_a_all, F), er.syn.a_all, nr, F);
      copy_rows(off(out->syn_i_all, F), er.syn.i_all, nr, F);
      if (s->ssc_on) {
        copy_rows(off(out->ssc_j_all, F), er.ssc.j_all, nr, F);
        copy_rows(off(out->ssc_i_all, F), er.ssc.i_all, nr, F);
      }
    }
  }
  return 0;
}

// ElectronAndRadiation::fluxDens itself on nq queries of one blastwave: an
// object set up with the flux options, its total_rad.j_all / a_all replaced by
// the given histories [nr][F], r_arr the radii of the rows.
int ref_flux_dens(const pbag_grid_desc* g, const pbag_flux_opts* o, int nr, const double* j_all,
                  const double* a_all, const double* r_arr, int nq, const pbag_flux_query* qs, double* flux) {
  static const char* vel_s[] = {"sameAsBW", "shockVel"};
  static const char* ne_s[] = {"usenprime", "useNe"};
  static const char* tau_s[] = {"approx", "thick", "smooth", "sharp"};
  Vector gam, freq;
  make_freq_grid(g, freq);
  SynKernel sk;
  SSCKernel ck;
  pbag_shock_params s{};
  s.p = 2.2;
  s.eps_e = 0.1;
  s.max_substeps = 1000;
  s.ele_method = PBAG_ELE_NUMERIC;
  StrDbMap pars = make_pars(g, &s, 1e-3);
  StrStrMap opts = make_opts(&s, false, "useU_e", "useTe", "useB", "useU_b", "none");
  opts["method_vel_fs"] = vel_s[o->shock_vel];
  opts["method_ne_fs"] = ne_s[o->method_ne];
  opts["method_tau_fs"] = tau_s[o->method_tau];
  ElectronAndRadiation er(LOG_SILENT, gam, freq, sk, ck, false);
  er.setPars(pars, opts, (size_t)nr, 0, 0, 0.1, 1.0, true);
  const size_t F = (size_t)g->nfreq;
  er.total_rad.j_all.assign(j_all, j_all + (size_t)nr * F);
  er.total_rad.a_all.assign(a_all, a_all + (size_t)nr * F);
  Vector r(r_arr, r_arr + nr);
  for (int t = 0; t < nq; ++t) {
    const pbag_flux_query& q = qs[t];
    flux[t] = er.fluxDens(EjectaID2::STUCT_TYPE::ipiecewise, q.theta, q.ncells, (size_t)q.ia, (size_t)q.ib, q.freq,
                          q.Gamma, q.GammaSh, q.acc_fac, q.mu, q.r, q.rsh, q.dr, q.n_prime, q.ne, r);
  }
  return 0;
}

}  // extern "C"
