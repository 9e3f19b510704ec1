// ref_eats.cpp - drives the REFERENCE's adaptive EATS integrator (compiled in
// place from its headers) on given layer dynamics and comoving histories, so
// that its light curves can pin the oracle's restatement of the quadrature.
//
// Test infrastructure only: built by oracle/Makefile (target ref) into
// oracle/_ref/libpbaref_eats.so when the reference sources are present.
// Nothing in the product links it.
//
// Reference code driven: EATS (src/eats.h:44) through its public
// evalFluxDensA (eats.h:820-850), with fluxFuncA = fluxDensAdaptiveWithComov
// (src/blastwave/blastwave_radiation.h:75-150) reading a blastwave Pars
// (src/blastwave/blastwave_pars.h:21) whose m_data holds the given dynamics and
// whose p_mphys / p_mphys_rs are ElectronAndRadiation objects holding the
// given total_rad.j_all / a_all histories (microphysics.h:1185-1217).
#include "pbag.h"

#include "utilitites/utils.h"
#include "utilitites/H5Easy.h"
#include "blastwave/blastwave.h"
#include "ejecta/ejecta.h"

#include <memory>

namespace {

const char* vel_s[] = {"sameAsBW", "shockVel"};
const char* ne_s[] = {"usenprime", "useNe"};
const char* tau_s[] = {"approx", "thick", "smooth", "sharp"};

// an ElectronAndRadiation holding the histories of one shock (the grid and
// options as the library's context and flux options describe them)
std::unique_ptr<ElectronAndRadiation> make_er(const pbag_grid_desc* g, const pbag_flux_opts* fo, bool rs, int nr,
                                              const double* j, const double* a, Vector& gam, Vector& freq,
                                              SynKernel& sk, SSCKernel& ck) {
  const std::string s = rs ? "_rs" : "_fs";
  StrDbMap pars;
  pars["eps_e" + s] = 0.1;
  pars["eps_b" + s] = 1e-3;
  pars["eps_t" + s] = 0.;
  pars["p" + s] = 2.2;
  pars["gam1" + s] = g->gam1;
  pars["gam2" + s] = g->gam2;
  pars["ngam" + s] = (double)g->ngam;
  pars["freq1" + s] = g->freq1;
  pars["freq2" + s] = g->freq2;
  pars["nfreq" + s] = (double)g->nfreq;
  StrStrMap opts;
  opts["method_ele" + s] = "numeric";
  opts["method_synchrotron" + s] = "CSYN";
  opts["method_ssc" + s] = "none";
  opts["method_pp" + s] = "none";
  opts["use_ssa" + s] = "yes";
  opts["num_ele_use_adi_loss" + s] = "yes";
  opts["save_spec"] = "no";
  opts["method_ne" + s] = ne_s[fo->method_ne];
  opts["method_vel" + s] = vel_s[fo->shock_vel];
  opts["method_tau" + s] = tau_s[fo->method_tau];
  opts["method_Up" + s] = "useEint2";
  opts["method_thickness" + s] = "useJoh06";
  opts["method_gamma_min" + s] = "useU_e";
  opts["method_gamma_c" + s] = "useTe";
  opts["method_gamma_max" + s] = "useB";
  opts["method_B" + s] = "useU_b";
  opts["method_nonrel_dist" + s] = "none";
  // the photon grid as CommonTables holds it (setPars allocates the electron grid)
  freq = TOOLS::MakeLogspaceVec(std::log10(g->freq1), std::log10(g->freq2), g->nfreq);
  auto er = std::make_unique<ElectronAndRadiation>(LOG_SILENT, gam, freq, sk, ck, rs);
  er->setPars(pars, opts, (size_t)nr, 0, 0, 0.1, 1.0, true);
  const size_t F = (size_t)g->nfreq;
  er->total_rad.j_all.assign(j, j + (size_t)nr * F);
  er->total_rad.a_all.assign(a, a + (size_t)nr * F);
  return er;
}

}  // namespace

extern "C" {

// One layer: dyn [PBAG_EQ_N][nr] (the pbag_eats_q order), the forward-shock
// histories j_fs / a_fs [nr][nfreq], the reverse-shock ones (NULL: none);
// flux[q] = evalFluxDensA(t_obs[q], nu_obs[q], 0) in mJy.
int ref_eats_flux(const pbag_grid_desc* g, const pbag_eats_opts* o, const pbag_eats_layer* L, int nr,
                  const double* dyn, const double* j_fs, const double* a_fs, const double* j_rs, const double* a_rs,
                  int nq, const double* t_obs, const double* nu_obs, double* flux) {
  VecVector data(BW::Q::i_Wdr + 1, Vector((size_t)nr, 0.));
  VecVector data_tmp(BW::Q::i_Wdr + 1, Vector((size_t)nr, 0.));
  static const int qmap[PBAG_EQ_N] = {
      BW::Q::itburst,  BW::Q::iR,        BW::Q::itheta,     BW::Q::iGamma,        BW::Q::ibeta,
      BW::Q::iGammaFsh, BW::Q::ithickness, BW::Q::iM2,      BW::Q::irho2,         BW::Q::iRsh,
      BW::Q::iacc_frac, BW::Q::ictheta,   BW::Q::iGammaRsh,  BW::Q::ithickness_rs, BW::Q::iM3,
      BW::Q::irho3,    BW::Q::iRrsh,      BW::Q::iacc_frac_rs};
  for (int q = 0; q < PBAG_EQ_N; ++q) data[qmap[q]].assign(dyn + (size_t)q * nr, dyn + (size_t)(q + 1) * nr);
  Pars pars(data, data_tmp, LOG_SILENT);
  Vector gam, freq;  // filled by ElectronAndRadiation::setPars
  Vector gam_rs, freq_rs;
  SynKernel sk;
  SSCKernel ck;
  pars.p_mphys = make_er(g, &o->flux, false, nr, j_fs, a_fs, gam, freq, sk, ck);
  const bool rs = j_rs && a_rs;
  if (rs) pars.p_mphys_rs = make_er(g, &o->flux, true, nr, j_rs, a_rs, gam_rs, freq_rs, sk, ck);
  pars.m_type = rs ? BW_TYPES::iFSRS : BW_TYPES::iFS;
  pars.do_rs_radiation = rs;
  pars.ncells = L->ncells;
  pars.z = o->z;
  pars.nr = (size_t)nr;

  size_t i_end_r = (size_t)L->i_end_r;
  Vector tt = data[BW::Q::itburst];
  CommonTables tables;
  EATS eats(data[BW::Q::itburst], tt, data[BW::Q::iR], data[BW::Q::itheta], data[BW::Q::iGamma],
            data[BW::Q::ibeta], i_end_r, 0, 0, LOG_SILENT, tables, &pars);
  StrDbMap ep;
  ep["nmax_phi"] = (double)o->nmax_phi;
  ep["nmax_theta"] = (double)o->nmax_theta;
  ep["rtol_phi"] = o->rtol_phi;
  ep["rtol_theta"] = o->rtol_theta;
  ep["theta_obs"] = o->theta_obs;
  ep["d_l"] = o->d_l;
  ep["z"] = o->z;
  StrStrMap eo;
  eo["counter_jet"] = o->counter_jet ? "yes" : "no";
  eo["method_quad"] = o->method_quad == PBAG_QUAD_TRAP_FIXED ? "TRAP_FIXED" : "CADRE";
  eo["skymap_remove_mu"] = "no";
  eo["ebl_tbl_fpath"] = "none";
  eats.setEatsPars(ep, eo, 1, (size_t)L->ncells, 0.5 * (L->theta_c_l + L->theta_c_h), L->theta_c_l,
                   L->theta_c_h, L->theta_c_h, L->theta_c_h);
  eats.fluxFuncA = fluxDensAdaptiveWithComov;
  for (int k = 0; k < nq; ++k) flux[k] = eats.evalFluxDensA(t_obs[k], nu_obs[k], 0.);
  return 0;
}

}  // extern "C"
