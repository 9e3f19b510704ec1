// pbag_recorder.hpp - the host side of the drop-in for the numeric path of
// ElectronAndRadiation (src/microphysics/microphysics.h:60-633), in C++ over
// the C ABI of pbag.h.
//
// The reference's blastwave driver calls, per blastwave (layer x shock) and
// burster-time index it,
//   initializeElectronDistribution(tcomov, m2, rho2, u_p, dr)            (microphysics.h:347)
//   evaluateElectronDistributionNumericMixed(tc, tc_p1, m, m_p1, rho, rho_p1,
//                                            r, rp1, dr, dr_p1, u_p, u_p_p1)   (:359)
//   computeRadiationNumericMixed(it)                                          (:492)
// after updateSockProperties + computeEleSpectrumLimits (microphysics_base.h:
// 575-966) set B, gamma_min, gamma_max, gamma_c, accel_frac and n_prime. The
// recorder has the same calls (plus the blastwave and step index and those
// members): they append one pbag_step_rec and return. flush() runs every
// recorded step of every blastwave in one batch on the GPU and writes the
// histories into the caller's vectors in the reference's time-major layout
// (value k of step it at [k + n * it], microphysics.h:602-633), sized for the
// blastwave's nt burster times; steps never recorded stay zero, like the
// reference's zero-initialised *_all vectors. Errors where the reference logs
// and exits come back as the pbag_status of the first failure in time order.
//
// Header-only; link libpbag. Not thread-safe (neither is the reference's
// shared kernel state).
#ifndef PBAG_RECORDER_HPP
#define PBAG_RECORDER_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pbag.h"

namespace pbag {

// The members computeEleSpectrumLimits() leaves for the step (microphysics_base.h:642-966).
struct ShockScalars {
  double B, gamma_min, gamma_max, gamma_c, accel_frac, n_prime;
};

// Where one blastwave's histories go (any pointer may be null: not produced).
struct Histories {
  std::vector<double>* j_all = nullptr;   // total_rad.j_all
  std::vector<double>* a_all = nullptr;   // total_rad.a_all
  std::vector<double>* f_all = nullptr;   // total_rad.f_all
  std::vector<double>* i_all = nullptr;   // total_rad.i_all
  std::vector<double>* ele_f_all = nullptr, *gdot_syn_all = nullptr, *gdot_adi_all = nullptr,
                      *gdot_ssc_all = nullptr;   // ele.* (save_spec)
  std::vector<double>* syn_j_all = nullptr, *syn_a_all = nullptr, *syn_i_all = nullptr;  // syn.*
  std::vector<double>* ssc_j_all = nullptr, *ssc_i_all = nullptr;                         // ssc.*
};

// The datasets the reference's spectrum writer stores for one blastwave
// (Ejecta::computeSaveEjectaSpectrum, ejecta.h:354-455), in its order and with
// its names (suffix "_fs" or "_rs"), pointing at the vectors a Recorder filled.
// syn.f_all and ssc.f_all are never set by the reference (their photon
// densities are commented out, numeric_model.h:182, 283): they are written as
// zeros of the history's size, held here.
struct WriterDatasets {
  std::vector<std::pair<std::string, const std::vector<double>*>> items;
  std::vector<double> zeros;
};
inline WriterDatasets writer_datasets(const Histories& h, bool rs, bool ele_numeric, bool ssa, bool ssc) {
  WriterDatasets d;
  const std::string sfx = rs ? "_rs" : "_fs";
  const size_t n = h.j_all ? h.j_all->size() : 0;
  d.zeros.assign(n, 0.);
  auto add = [&](const char* name, const std::vector<double>* v) {
    if (v) d.items.emplace_back(std::string(name) + sfx, v);
  };
  if (ele_numeric) {
    add("n_ele", h.ele_f_all);
    add("gam_dot_syn", h.gdot_syn_all);
    add("gam_dot_adi", h.gdot_adi_all);
    add("gam_dot_ssc", h.gdot_ssc_all);
  }
  add("syn_f", &d.zeros);
  add("syn_j", h.syn_j_all);
  add("syn_i", h.syn_i_all);
  if (ssa) add("syn_a", h.syn_a_all);
  if (ssc) {
    add("ssc_f", &d.zeros);
    add("ssc_j", h.ssc_j_all);
    add("ssc_i", h.ssc_i_all);
  }
  add("total_f", h.f_all);
  add("total_j", h.j_all);
  add("total_i", h.i_all);
  if (ssa) add("total_a", h.a_all);
  return d;
}

class Recorder {
 public:
  // One recorder per grid (one CommonTables entry of the reference).
  Recorder(const pbag_grid_desc& grid, int device, bool ssc_tables) : grid_(grid) {
    int rc = pbag_create(&grid, device, ssc_tables ? 1 : 0, &ctx_);
    if (rc != PBAG_OK) throw std::runtime_error(std::string("pbag_create: ") + pbag_status_string(rc));
  }
  ~Recorder() { pbag_destroy(ctx_); }
  Recorder(const Recorder&) = delete;
  Recorder& operator=(const Recorder&) = delete;

  pbag_ctx* context() { return ctx_; }

  // A blastwave with its options and nt burster times; returns its index.
  int add_blastwave(const pbag_shock_params& prm, size_t nt, const Histories& out) {
    Bw b;
    b.prm = prm;
    b.recs.assign(nt, pbag_step_rec{});  // PBAG_SKIP until recorded
    b.out = out;
    bws_.push_back(b);
    return (int)bws_.size() - 1;
  }

  // initializeElectronDistribution(tcomov, m2, rho2, u_p, dr) at step it
  void initializeElectronDistribution(int bw, size_t it, double tcomov, double m2, double rho2, double u_p,
                                      double dr, const ShockScalars& s) {
    pbag_step_rec& q = at(bw, it);
    q = pbag_step_rec{};
    q.mode = PBAG_INIT;
    q.tc_p1 = tcomov;
    q.m_p1 = m2;
    q.rho_p1 = rho2;
    q.u_p_p1 = u_p;
    q.dr = dr;
    scalars(q, s);
  }

  // evaluateElectronDistributionNumericMixed(...) at step it (r, rp1 unused, as in the reference)
  void evaluateElectronDistributionNumericMixed(int bw, size_t it, double tc, double tc_p1, double m, double m_p1,
                                                double rho, double rho_p1, double r, double rp1, double dr,
                                                double dr_p1, double u_p, double u_p_p1, const ShockScalars& s) {
    (void)r;
    (void)rp1;
    pbag_step_rec& q = at(bw, it);
    q = pbag_step_rec{};
    q.mode = PBAG_EVOLVE;
    q.tc = tc;
    q.tc_p1 = tc_p1;
    q.m = m;
    q.m_p1 = m_p1;
    q.rho = rho;
    q.rho_p1 = rho_p1;
    q.dr = dr;
    q.dr_p1 = dr_p1;
    q.u_p = u_p;
    q.u_p_p1 = u_p_p1;
    scalars(q, s);
  }

  // The records of one blastwave (diagnostics, tests).
  const std::vector<pbag_step_rec>& records(int bw) const { return bws_.at(bw).recs; }

  // Runs every recorded step on the GPU and fills the histories. Returns
  // PBAG_OK or the first failure (blastwave, step) in *st.
  int flush(pbag_status* st = nullptr) {
    std::vector<pbag_shock_params> prm;
    std::vector<int64_t> off{0};
    std::vector<pbag_step_rec> recs;
    for (const Bw& b : bws_) {
      prm.push_back(b.prm);
      recs.insert(recs.end(), b.recs.begin(), b.recs.end());
      off.push_back((int64_t)recs.size());
    }
    const size_t nrec = recs.size(), F = (size_t)grid_.nfreq, G = (size_t)grid_.ngam;
    // the batch's histories, then split per blastwave into the caller's vectors
    std::vector<double> buf[13];
    pbag_outputs out{};
    double** slot = reinterpret_cast<double**>(&out);
    for (int k = 0; k < 13; ++k) {
      bool want = false;
      for (const Bw& b : bws_) want = want || field(b.out, k) != nullptr;
      if (!want) continue;
      buf[k].assign(nrec * (on_gamma(k) ? G : F), 0.);
      slot[k] = buf[k].data();
    }
    pbag_status s{};
    int rc = pbag_run_batch(ctx_, prm.data(), (int)prm.size(), off.data(), recs.data(), &out, &s);
    if (st) *st = s;
    for (size_t b = 0; b < bws_.size(); ++b)
      for (int k = 0; k < 13; ++k) {
        std::vector<double>* dst = field(bws_[b].out, k);
        if (!dst || !slot[k]) continue;
        const size_t n = on_gamma(k) ? G : F;
        const size_t nt = (size_t)(off[b + 1] - off[b]);
        dst->assign(n * nt, 0.);
        std::copy(buf[k].begin() + (size_t)off[b] * n, buf[k].begin() + (size_t)off[b + 1] * n, dst->begin());
      }
    return rc;
  }

 private:
  struct Bw {
    pbag_shock_params prm{};
    std::vector<pbag_step_rec> recs;
    Histories out;
  };
  static bool on_gamma(int k) { return k >= 4 && k < 8; }
  static std::vector<double>* field(const Histories& h, int k) {
    std::vector<double>* const f[13] = {h.j_all,        h.a_all,        h.f_all,     h.i_all,     h.ele_f_all,
                                        h.gdot_syn_all, h.gdot_adi_all, h.gdot_ssc_all, h.syn_j_all, h.syn_a_all,
                                        h.syn_i_all,    h.ssc_j_all,    h.ssc_i_all};
    return f[k];
  }
  pbag_step_rec& at(int bw, size_t it) {
    Bw& b = bws_.at((size_t)bw);
    if (it >= b.recs.size()) throw std::out_of_range("pbag::Recorder: step index beyond the blastwave's nt");
    return b.recs[it];
  }
  static void scalars(pbag_step_rec& q, const ShockScalars& s) {
    q.B = s.B;
    q.gamma_min = s.gamma_min;
    q.gamma_max = s.gamma_max;
    q.gamma_c = s.gamma_c;
    q.accel_frac = s.accel_frac;
    q.n_prime = s.n_prime;
  }
  pbag_grid_desc grid_;
  pbag_ctx* ctx_ = nullptr;
  std::vector<Bw> bws_;
};

}  // namespace pbag

#endif
