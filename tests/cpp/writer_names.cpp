// Prints, for every combination of the options that gate the spectrum
// writer's datasets (numeric electrons, SSA, SSC, reverse-shock radiation),
// the datasets pbag::writer_datasets lists for one layer group: the forward
// shock's, then (with reverse-shock radiation) the reverse shock's.
// Output lines: "<ele> <ssa> <ssc> <rs>: name name ...".
#include <cstdio>
#include <vector>

#include "pbag_recorder.hpp"

int main() {
  std::vector<double> v(4, 1.0);
  pbag::Histories h;
  h.j_all = h.a_all = h.f_all = h.i_all = &v;
  h.ele_f_all = h.gdot_syn_all = h.gdot_adi_all = h.gdot_ssc_all = &v;
  h.syn_j_all = h.syn_a_all = h.syn_i_all = h.ssc_j_all = h.ssc_i_all = &v;
  for (int ele = 0; ele < 2; ++ele)
    for (int ssa = 0; ssa < 2; ++ssa)
      for (int ssc = 0; ssc < 2; ++ssc)
        for (int rs = 0; rs < 2; ++rs) {
          std::printf("%d %d %d %d:", ele, ssa, ssc, rs);
          for (int shock = 0; shock <= rs; ++shock) {
            const pbag::WriterDatasets d = pbag::writer_datasets(h, shock == 1, ele, ssa, ssc);
            for (const auto& it : d.items) std::printf(" %s", it.first.c_str());
          }
          std::printf("\n");
        }
  return 0;
}
