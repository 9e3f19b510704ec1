// Drives pbag::ElectronAndRadiation (include/pbag_microphysics.hpp) with the
// call sequence of the reference's blastwave driver, per burster-time index
// it and per blastwave (blastwave_radiation.h:976-1182):
//   updateSockProperties(U_p, Gamma, GammaSh, t_e, t_b, tcomov, rho2/m_p, M2/m_p)
//   computeEleSpectrumLimits()
//   is_distribution_initialized ? evaluateElectronDistributionNumericMixed(12 values at it-1, it)
//                               : initializeElectronDistribution(tcomov, M2, rho2, U_p, thickness)
//   if (is_distribution_initialized) computeRadiationNumericMixed(it)
// then reads the histories back from the objects' members, as the spectrum
// writer and EATS do, and answers a few fluxDens queries.
//
// Usage: microphysics_driver <in.bin> <out.bin>
// in.bin (little-endian): int32 nbw, nt; doubles grid[6] (ngam, nfreq, gam1,
// gam2, freq1, freq2), shock[6] (eps_e, eps_b, p, use_ssa, use_ssc,
// max_substeps); per blastwave int32 is_rs and 14 arrays of nt doubles (valid,
// U_p, Gamma, GammaSh, t_e, t_b, tcomov, n_prime, n_protons, M2, rho2, R,
// thickness, comoving thickness); int32 nq and nq queries of 16 doubles (bw,
// ia, ib, theta, ncells, freq, Gamma, GammaSh, acc_fac, mu, r, rsh, dr,
// n_prime, ne, unused).
// out.bin: per blastwave its 13 histories in pbag_outputs order (each nt rows,
// zeros where the object keeps none), then its records (nt pbag_step_rec),
// then the nq flux densities.
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <memory>
#include <vector>

#include "pbag_microphysics.hpp"

namespace {

struct Reader {
  std::ifstream f;
  explicit Reader(const char* p) : f(p, std::ios::binary) {}
  template <typename T>
  T get() {
    T v{};
    f.read(reinterpret_cast<char*>(&v), sizeof(T));
    return v;
  }
  std::vector<double> vec(size_t n) {
    std::vector<double> v(n);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(double)));
    return v;
  }
};

enum { kValid, kUp, kGamma, kGammaSh, kTe, kTb, kTcomov, kNprime, kNprot, kM2, kRho2, kR, kThick, kDr, kArrays };

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  Reader in(argv[1]);
  const int nbw = in.get<int32_t>(), nt = in.get<int32_t>();
  const std::vector<double> g = in.vec(6), sh = in.vec(6);

  // the shared tables of one grid (CommonTables) and one object per blastwave
  pbag::Vector gam_grid, freq_grid;
  pbag::SynKernel syn_kernel;
  pbag::SSCKernel ssc_kernel(0);
  std::vector<std::unique_ptr<pbag::ElectronAndRadiation>> bw;
  std::vector<std::vector<std::vector<double>>> data(nbw);
  for (int b = 0; b < nbw; ++b) {
    const bool rs = in.get<int32_t>() != 0;
    for (int a = 0; a < kArrays; ++a) data[b].push_back(in.vec((size_t)nt));
    bw.emplace_back(new pbag::ElectronAndRadiation(0, gam_grid, freq_grid, syn_kernel, ssc_kernel, rs));
    const std::string s = rs ? "_rs" : "_fs";
    pbag::StrDbMap pars{{"eps_e" + s, sh[0]}, {"eps_b" + s, sh[1]}, {"p" + s, sh[2]},
                        {"max_substeps" + s, sh[5]}, {"ngam" + s, g[0]}, {"nfreq" + s, g[1]},
                        {"gam1" + s, g[2]}, {"gam2" + s, g[3]}, {"freq1" + s, g[4]}, {"freq2" + s, g[5]}};
    pbag::StrStrMap opts{{"method_ele" + s, "numeric"}, {"method_synchrotron" + s, "CSYN"},
                         {"method_ssc" + s, sh[4] != 0 ? "numeric" : "none"},
                         {"use_ssa" + s, sh[3] != 0 ? "yes" : "no"}, {"save_spec", "yes"},
                         {"method_ne" + s, "useNe"}, {"method_tau" + s, "smooth"}};
    bw.back()->setPars(pars, opts, (size_t)nt, 0, (size_t)(b / 2), 0.1, 1.0, true);
  }

  // the driver's loop: time index by time index, every blastwave
  for (int it = 0; it < nt; ++it)
    for (int b = 0; b < nbw; ++b) {
      const std::vector<std::vector<double>>& d = data[b];
      if (d[kValid][it] == 0) continue;  // isBlastWaveValidForElectronCalc / considerReverseShock
      pbag::ElectronAndRadiation& m = *bw[b];
      m.updateSockProperties(d[kUp][it], d[kGamma][it], d[kGammaSh][it], d[kTe][it], d[kTb][it], d[kTcomov][it],
                             d[kNprime][it], d[kNprot][it]);
      m.computeEleSpectrumLimits();
      if (!m.is_distribution_initialized)
        m.initializeElectronDistribution(d[kTcomov][it], d[kM2][it], d[kRho2][it], d[kUp][it], d[kThick][it]);
      else
        m.evaluateElectronDistributionNumericMixed(d[kTcomov][it - 1], d[kTcomov][it], d[kM2][it - 1], d[kM2][it],
                                                   d[kRho2][it - 1], d[kRho2][it], d[kR][it - 1], d[kR][it],
                                                   d[kDr][it - 1], d[kDr][it], d[kUp][it - 1], d[kUp][it]);
      if (m.is_distribution_initialized) m.computeRadiationNumericMixed((size_t)it);
    }

  // EATS: fluxDens flushes the recorded steps before its first interpolation
  const int nq = in.get<int32_t>();
  std::vector<double> flux((size_t)nq, 0.);
  for (int q = 0; q < nq; ++q) {
    const std::vector<double> x = in.vec(16);
    const int b = (int)x[0];
    flux[(size_t)q] = bw[b]->fluxDens(0, x[3], x[4], (size_t)x[1], (size_t)x[2], x[5], x[6], x[7], x[8], x[9], x[10],
                                      x[11], x[12], x[13], x[14], data[b][kR]);
  }
  pbag_status st{};
  const int rc = ssc_kernel.flush(&st);  // nothing pending after fluxDens: a no-op flush
  std::ofstream out(argv[2], std::ios::binary);
  for (int b = 0; b < nbw; ++b) {
    pbag::ElectronAndRadiation& m = *bw[b];
    const std::vector<double>* h[13] = {&m.total_rad.j_all,      &m.total_rad.a_all,      &m.total_rad.f_all,
                                        &m.total_rad.i_all,      &m.ele.f_all,            &m.ele.gam_dot_syn_all,
                                        &m.ele.gam_dot_adi_all,  &m.ele.gam_dot_ssc_all,  &m.syn.j_all,
                                        &m.syn.a_all,            &m.syn.i_all,            &m.ssc.j_all,
                                        &m.ssc.i_all};
    for (int k = 0; k < 13; ++k) {
      const size_t n = (size_t)nt * ((k >= 4 && k < 8) ? m.ele.numbins : m.total_rad.numbins);
      std::vector<double> v = h[k]->size() == n ? *h[k] : std::vector<double>(n, 0.);
      out.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(n * sizeof(double)));
    }
    out.write(reinterpret_cast<const char*>(m.records().data()),
              (std::streamsize)(m.records().size() * sizeof(pbag_step_rec)));
  }
  out.write(reinterpret_cast<const char*>(flux.data()), (std::streamsize)(flux.size() * sizeof(double)));
  std::printf("rc %d bw %d step %d grid %zu %zu\n", rc, st.bw, st.step, gam_grid.size(), freq_grid.size());
  return rc == PBAG_OK ? 0 : 1;
}
