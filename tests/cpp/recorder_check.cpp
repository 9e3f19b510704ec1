// Replays step records through pbag::Recorder the way the reference's driver
// calls ElectronAndRadiation (one call per blastwave and step), flushes, and
// writes every blastwave's total_rad.j_all / a_all, concatenated, to a file.
// Usage: recorder_check <grid.bin> <params.bin> <offsets.bin> <records.bin> <out.bin>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <vector>

#include "pbag_recorder.hpp"

template <typename T>
std::vector<T> load(const char* path) {
  std::ifstream f(path, std::ios::binary);
  std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<T> v(raw.size() / sizeof(T));
  std::copy(raw.begin(), raw.begin() + v.size() * sizeof(T), reinterpret_cast<char*>(v.data()));
  return v;
}

int main(int argc, char** argv) {
  if (argc != 6) return 2;
  const auto grid = load<pbag_grid_desc>(argv[1]).at(0);
  const auto prm = load<pbag_shock_params>(argv[2]);
  const auto off = load<int64_t>(argv[3]);
  const auto recs = load<pbag_step_rec>(argv[4]);
  pbag::Recorder rec(grid, 0, true);
  std::vector<std::vector<double>> j(prm.size()), a(prm.size());
  for (size_t b = 0; b < prm.size(); ++b) {
    pbag::Histories h;
    h.j_all = &j[b];
    h.a_all = &a[b];
    const int id = rec.add_blastwave(prm[b], (size_t)(off[b + 1] - off[b]), h);
    for (int64_t r = off[b]; r < off[b + 1]; ++r) {
      const pbag_step_rec& q = recs[(size_t)r];
      const size_t it = (size_t)(r - off[b]);
      const pbag::ShockScalars s{q.B, q.gamma_min, q.gamma_max, q.gamma_c, q.accel_frac, q.n_prime};
      if (q.mode == PBAG_INIT)
        rec.initializeElectronDistribution(id, it, q.tc_p1, q.m_p1, q.rho_p1, q.u_p_p1, q.dr, s);
      else if (q.mode == PBAG_EVOLVE)
        rec.evaluateElectronDistributionNumericMixed(id, it, q.tc, q.tc_p1, q.m, q.m_p1, q.rho, q.rho_p1, 0., 0.,
                                                     q.dr, q.dr_p1, q.u_p, q.u_p_p1, s);
    }
  }
  pbag_status st{};
  const int rc = rec.flush(&st);
  std::ofstream o(argv[5], std::ios::binary);
  for (size_t b = 0; b < prm.size(); ++b) {
    o.write(reinterpret_cast<const char*>(j[b].data()), (std::streamsize)(j[b].size() * sizeof(double)));
    o.write(reinterpret_cast<const char*>(a[b].data()), (std::streamsize)(a[b].size() * sizeof(double)));
  }
  // the spectrum writer's datasets of the first blastwave (total j, a only here)
  pbag::Histories h0;
  h0.j_all = &j[0];
  h0.a_all = &a[0];
  const pbag::WriterDatasets ds = pbag::writer_datasets(h0, false, true, true, true);
  std::printf("datasets");
  for (const auto& it : ds.items) std::printf(" %s:%zu", it.first.c_str(), it.second->size());
  std::printf("\n");
  std::printf("rc %d bw %d step %d\n", rc, st.bw, st.step);
  return rc == PBAG_OK ? 0 : 1;
}
