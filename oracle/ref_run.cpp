// ref_run.cpp - runs the REFERENCE's own program (src/main.cpp compiled in
// place, its main renamed) on a parfile, with the HDF5 stand-in of
// shim/H5Cpp.h keeping in memory what it reads and writes: a caller puts the
// ejecta initial data there (what the reference's Python front end would write
// to id_a.h5), runs the program, and reads back what it wrote - the blastwave
// dynamics (saveEjectaBWsDynamics), the comoving spectra
// (computeSaveEjectaSpectrum) and the light curves (computeSaveEjectaLightCurve).
//
// Test infrastructure only: built by oracle/Makefile (target ref) into
// oracle/_ref/libpbaref_run.so when the reference sources are present, used by
// tests/golden/make_reference_run.py to record the reference driver's inputs
// and outputs. Nothing in the product links it.
//
// The ODE right-hand side the program registers with its integrator
// (model_evolve.h:294) is wrapped so that evaluations can be sampled: every
// `every`-th call, the inputs of each GRB blastwave's rhs_dispatcher (its state,
// parameters, flags and the microphysics members its loss term reads) and its
// outputs are recorded in the ABI layout of pbag_bw_rhs (include/pbag.h). The
// reference's headers come first with their private and protected members
// open, the wrapper goes in through SetRHS's one call site.
#include <csignal>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include <fcntl.h>
#include <sys/wait.h>
#include <unistd.h>

#include "utilitites/pch.h"
#define private public
#define protected public
#include "utilitites/utils.h"
#include "utilitites/H5Easy.h"
#include "blastwave/blastwave.h"
#include "ejecta/ejecta.h"
#include "pbag.h"

namespace pbag_rec {
using rhs_fn = void (*)(double*, size_t, double, const double*, void*);
rhs_fn real = nullptr;
void record(double* out, size_t n, double x, const double* Y, void* pars);
inline rhs_fn install(rhs_fn f) {
  real = f;
  return &record;
}
}  // namespace pbag_rec
#define SetRHS(F, N, P) SetRHS(pbag_rec::install(F), N, P)

#define main pbag_reference_main
#include "main.cpp"
#undef main
#undef SetRHS

namespace pbag_rec {

struct Sample {
  int32_t call, layer;
  pbag_bw_rhs_pars pars;
  pbag_bw_rhs_state before, after;
  double dydt[PBAG_Y_N];
};
// Samples go to the store's write-through log as they are taken ('R', size,
// bytes), and record() allocates nothing on the program's heap.
constexpr int kMaxBw = 128;  // GRB blastwaves recorded per call
long g_every = 0;            // 0: recording off
long g_calls = 0;
size_t g_cap = 0, g_n = 0;

void mphys_of(const ElectronAndRadiation* m, pbag_bw_mphys& o) {
  o = pbag_bw_mphys{};
  if (!m) return;
  o.method_B = m->m_methodsB == METHODS_B::iBuseUb ? 0 : m->m_methodsB == METHODS_B::iBasMAG21 ? 1 : 2;
  o.method_gamma_max = m->m_methodsLfmax == METHOD_LFMAX::iuseB ? 0 : 1;
  o.method_nonrel = (int32_t)m->m_method_nonreldist;
  o.method_up = m->m_method_up == METHODS_Up_sh::iuseEint2 ? 0 : 1;
  o.ele_analytic = m->m_eleMethod == METHODS_SHOCK_ELE::iShockEleAnalyt;
  o.eps_e = m->eps_e;
  o.eps_b = m->eps_b;
  o.eps_t = m->eps_t;
  o.p = m->p;
  o.mu = m->mu;
  o.mu_e = m->mu_e;
  o.beta_min = m->beta_min;
  if (!m->ele.e.empty()) {  // a reverse shock's object without a grid where none runs
    o.gam_lo = m->ele.e.front();
    o.gam_hi = m->ele.e.back();
  }
}

void carried(const Pars* p, pbag_bw_rhs_state& s) {
  s.end_spreading = p->end_spreading;
  s.shut_off = p->shutOff;
  s.first_step = p->prev_idx_x == 0;
  if (p->p_mphys) {
    s.fs_tcomov = p->p_mphys->tcomov;
    s.fs_gamma_max = p->p_mphys->gamma_max;
    s.fs_accel_frac = p->p_mphys->accel_frac;
  }
  if (p->p_mphys_rs) {
    s.rs_tcomov = p->p_mphys_rs->tcomov;
    s.rs_gamma_max = p->p_mphys_rs->gamma_max;
    s.rs_accel_frac = p->p_mphys_rs->accel_frac;
  }
}

void record(double* out, size_t n, double x, const double* Y, void* pars) {
  const bool take = g_every > 0 && (g_calls++ % g_every) == 0 && g_n < g_cap;
  if (!take) {
    real(out, n, x, Y, pars);
    return;
  }
  // EvolveODEsystem::Pars is a private type of its class; its leading
  // reference members (model_evolve.h:35-41) read through a mirror of them
  struct ParsHead {
    Vector* t_grid;
    Vector* t_grid_;
    std::unique_ptr<Magnetar>* p_magnetar;
    std::unique_ptr<PWNset>* p_ej_pwn;
    std::unique_ptr<Ejecta>* p_grb;
  };
  const ParsHead* H = reinterpret_cast<const ParsHead*>(pars);
  struct {
    std::unique_ptr<Magnetar>& p_magnetar;
    std::unique_ptr<Ejecta>& p_grb;
  } Pv{*H->p_magnetar, *H->p_grb};
  auto* P = &Pv;
  static Sample now[kMaxBw];
  size_t at[kMaxBw];
  int nnow = 0;
  if (P->p_grb->run_bws) {
    size_t ii = P->p_magnetar->run_magnetar ? P->p_magnetar->getNeq() : 0;
    auto& layers = P->p_grb->getShells();
    for (size_t il = 0; il < layers.size(); il++)
      for (size_t ish = 0; ish < layers[il]->nBWs(); ish++, ii += SOL::neq) {
        auto& bw = layers[il]->getBW(ish);
        const Pars* p = bw->getPars();
        if (p->end_evolution || (p->m_type != BW_TYPES::iFS && p->m_type != BW_TYPES::iFSRS) || nnow >= kMaxBw)
          continue;
        Sample& r = now[nnow];
        r = Sample{};
        r.call = (int32_t)(g_calls - 1);
        r.layer = (int32_t)il;
        pbag_bw_rhs_pars& q = r.pars;
        q.type = p->m_type == BW_TYPES::iFS ? PBAG_BW_FS : PBAG_BW_FSRS;
        q.method_dmdr = (int32_t)p->m_method_dmdr;
        q.method_dgdr = (int32_t)p->m_method_dgdr;
        q.method_limit_spread = (int32_t)p->method_limit_spread;
        q.method_spread = (int32_t)bw->p_spread->m_method;
        q.method_eos = (int32_t)bw->p_eos->m_method;
        q.adiab_loss = p->adiabLoss;
        q.adiab_loss_rs = p->adiabLoss_rs;
        q.exponential_rho4 = p->exponential_rho4;
        q.ilayer = (int32_t)p->ilayer;
        q.nlayers = (int32_t)p->nlayers;
        q.Gamma0 = p->Gamma0;
        q.beta0 = p->beta0;
        q.M0 = p->M0;
        q.mom0 = p->mom0;
        q.ncells = p->ncells;
        q.theta_a = p->theta_a;
        q.theta_max = p->theta_max;
        q.Rd = p->Rd;
        q.frac_mom0_spread = p->fraction_of_mom0_when_spread_start;
        q.mom_spread = p->value_of_mom_when_spread_start;
        q.spread_aa = bw->p_spread->m_aa;
        q.spread_theta_max = bw->p_spread->m_theta_max;
        q.spread_theta_c = bw->p_spread->m_thetaC;
        q.spread_theta_w = bw->p_spread->m_thetaW;
        q.spread_theta_b0 = bw->p_spread->m_theta_b0;
        q.eps_rad_fs = p->epsilon_rad_fs;
        q.eps_rad_rs = p->epsilon_rad_rs;
        q.tprompt = p->tprompt;
        q.rs_Gamma0_frac_no_exceed = p->rs_Gamma0_frac_no_exceed;
        q.n_ism = bw->p_dens->m_nn;
        q.A0 = bw->p_dens->m_A0;
        q.s = bw->p_dens->m_s;
        q.R_ej = bw->p_dens->m_R_EJ;
        q.R_ism = bw->p_dens->m_R_ISM;
        mphys_of(p->p_mphys.get(), q.fs);
        mphys_of(p->p_mphys_rs.get(), q.rs);
        r.before.x = x;
        for (int k = 0; k < PBAG_Y_N; ++k) r.before.Y[k] = Y[ii + k];
        carried(p, r.before);
        at[nnow++] = ii;
      }
  }
  real(out, n, x, Y, pars);
  for (int k = 0; k < nnow; ++k) {
    Sample& r = now[k];
    for (int q = 0; q < PBAG_Y_N; ++q) r.dydt[q] = out[at[k] + q];
    r.after = r.before;
    auto& bw = P->p_grb->getShells()[(size_t)r.layer]->getBW(0);
    carried(bw->getPars(), r.after);
    if (g_n < g_cap) {
      const uint64_t sz = sizeof(Sample);
      pbag_h5::log_bytes("R", 1);
      pbag_h5::log_bytes(&sz, sizeof sz);
      pbag_h5::log_bytes(&r, sizeof r);
      ++g_n;
    }
  }
}

}  // namespace pbag_rec


extern "C" {

// the store of the HDF5 stand-in
void ref_h5_put(const char* file, const char* name, const double* data, const unsigned long long* dims, int ndims) {
  std::vector<unsigned long long> d(dims, dims + ndims);
  size_t n = ndims ? 1 : 0;
  for (unsigned long long x : d) n *= (size_t)x;
  pbag_h5::put(file, name, std::vector<double>(data, data + n), d);
}
void ref_h5_put_attr(const char* file, const char* name, double v) { pbag_h5::put_attr(file, name, v); }
void ref_h5_clear() {
  pbag_h5::datasets().clear();
  pbag_h5::attributes().clear();
}
int ref_h5_count() { return (int)pbag_h5::datasets().size(); }
// key of dataset i (NUL-terminated into buf of len bytes); its element count
long ref_h5_key(int i, char* buf, int len) {
  auto it = pbag_h5::datasets().begin();
  std::advance(it, i);
  std::strncpy(buf, it->first.c_str(), (size_t)len - 1);
  buf[len - 1] = 0;
  return (long)it->second.data.size();
}
// sampling of the ODE right-hand side: every `every`-th call, at most `cap`
// blastwave samples (0: off)
int ref_rhs_record(long every, long cap) {
  using namespace pbag_rec;
  g_every = every > 0 && cap > 0 ? every : 0;
  g_cap = cap > 0 ? (size_t)cap : 0;
  g_n = 0;
  g_calls = 0;
  return 0;
}
int ref_h5_get(const char* key, double* out) {
  const pbag_h5::Entry* e = pbag_h5::find(key);
  if (!e) return -1;
  std::memcpy(out, e->data.data(), e->data.size() * sizeof(double));
  return 0;
}
double ref_h5_get_attr(const char* key, int* found) {
  auto it = pbag_h5::attributes().find(key);
  *found = it != pbag_h5::attributes().end();
  return *found ? it->second : 0.;
}

}  // extern "C"


namespace {

// the program's exit path frees one of its strings twice after its last
// output is written (and may corrupt the heap before that); the child ends
// there with the signal's status, its outputs already in the log
void on_fatal(int sig) { _exit(128 + sig); }

}  // namespace

extern "C" {

// Runs the reference program (argv = {name, working_dir, parfile, loglevel})
// in a child process that logs everything it writes (and the right-hand-side
// samples) to out_path as it writes it (pbag_h5 log format). Returns the
// child's exit status (0, or 128 + the signal that ended it after its outputs
// were written).
int ref_run(const char* working_dir, const char* parfile, const char* loglevel, const char* out_path) {
  std::fflush(nullptr);
  const pid_t pid = fork();
  if (pid < 0) return -1;
  if (pid == 0) {
    const int fd = ::open(out_path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) _exit(127);
    pbag_h5::log_fd() = fd;
    std::signal(SIGSEGV, on_fatal);
    std::signal(SIGABRT, on_fatal);
    char a0[] = "pba.out";
    std::string w(working_dir), p(parfile), l(loglevel);
    char* argv[] = {a0, w.data(), p.data(), l.data(), nullptr};
    const int rc = pbag_reference_main(4, argv);
    std::fflush(nullptr);
    _exit(rc);
  }
  int status = 0;
  if (waitpid(pid, &status, 0) < 0) return -1;
  return WIFEXITED(status) ? WEXITSTATUS(status) : 128 + WTERMSIG(status);
}

}  // extern "C"
