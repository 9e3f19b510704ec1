// pbag_internal.h - declarations shared between the host and device
// translation units of libpbag (not part of the C ABI).
#ifndef PBAG_INTERNAL_H
#define PBAG_INTERNAL_H

#include <vector>

#include "pbag.h"

namespace pbag {

// Electron grid gam[G] and photon grid freq[F+1] (see pbag_build_grids).
void build_grids(const pbag_grid_desc* g, double* gam, double* freq);

// Tabulated synchrotron function of the GSL or Bessel method (pbag_syntab.cpp):
// g(u) = R(e^u) e^(-u/3) at kSynTabN points u uniform in [ln kSynTabXmin,
// ln kSynTabXmax].
constexpr int kSynTabN = 16384;
constexpr double kSynTabXmin = 1e-12;
constexpr double kSynTabXmax = 120.;
std::vector<float> syn_table(int method);

}  // namespace pbag

#endif
