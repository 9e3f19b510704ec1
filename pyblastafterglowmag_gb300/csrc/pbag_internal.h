// pbag_internal.h - declarations shared between the host and device
// translation units of libpbag (not part of the C ABI).
#ifndef PBAG_INTERNAL_H
#define PBAG_INTERNAL_H

#include <vector>

#include "pbag.h"

namespace pbag {

// Electron grid gam[G] and photon grid freq[F+1] (see pbag_build_grids).
void build_grids(const pbag_grid_desc* g, double* gam, double* freq);

// Tabulated synchrotron functions (pbag_syntab.cpp): g(u) = R(e^u) e^(-u/3)
// at n <= kSynTabN points u0 + i h covering [ln kSynTabXmin, ln kSynTabXmax]
// (zero after them); syn_table_grid picks h from the electron grid's step
// dlng = ln(e[1] / e[0]). method: GSL, Bessel, or CSYN / Dermer09 (the fit).
constexpr int kSynTabN = 16384;
constexpr double kSynTabXmin = 1e-12;
constexpr double kSynTabXmax = 120.;
void syn_table_grid(double dlng, double* u0, double* h, int* n, int nmax = kSynTabN);
std::vector<float> syn_table(int method, double u0, double h, int n);
// The same function as value / slope pairs (g(u_i), (g(u_{i+1}) - g(u_{i-1})) / 2)
// for interpolation around the nearest point, kSynTab2N pairs; the slope is 0
// at the first point (g is flat there) and value and slope are 0 from the
// last point on.
constexpr int kSynTab2N = 8192;
std::vector<float> syn_table2(int method, double u0, double h, int n);
// The synchrotron function R(x) of a method in FP64 (GSL: F(x); Bessel: the
// K_4/3 K_1/3 form; CSYN and Dermer09: the Aharonian fit), x = nu / nu_crit.
double syn_shape(int method, double x);

}  // namespace pbag

#endif
