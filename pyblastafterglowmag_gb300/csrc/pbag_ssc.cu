// pbag_ssc.cu - host-side construction of the SSC kernel tables of one grid.
//
// The reference fills the Blumenthal-Gould kernel K[i][j][k] = sscNava(nu_i,
// gamma_j, nu_k) once per CommonTables entry and integrates it over the
// scattered frequency for the SSC cooling term (kernels.h:49-117). Here the
// same FP64 values are converted to the operands the device kernels use.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "pbag_kernels.h"

namespace pbag {

using namespace cgs;

namespace {

// kernels.h:96-117 (sscNava): isotropic Compton kernel, Nava et al. form.
double ssc_nava(double nu, double gam, double nu_tilde) {
  const double en = nu * h_by_mec2;
  const double en_t = nu_tilde * h_by_mec2;
  double K = 0.;
  if (en_t / (4. * gam * gam) < en && en <= en_t) {
    K = (en / en_t) - (1. / (4. * gam * gam));
  } else if (en_t < en && en < (4. * gam * gam * en_t / (1. + 4. * gam * en_t))) {
    const double q = en / (4. * gam * en_t * (gam - en));
    K = 2. * q * std::log(q) + (1. + 2. * q) * (1. - q) +
        .5 * (1. - q) * std::pow(4. * gam * en_t * q, 2.) / (1. + 4. * gam * en_t * q);
  }
  return K;
}

}  // namespace

void build_ssc_tables(const double* gam, int G, const double* freq, int F, int Gp, int Gs, std::vector<float>& KintT,
                      std::vector<double>& kscale, std::vector<float>& K32) {
  std::vector<double> K((size_t)F * G * F);
  const unsigned hw = std::thread::hardware_concurrency();
  const int nth = (int)std::max(1u, std::min(hw, 16u));
  auto fill = [&](int t) {
    for (int i = t; i < F; i += nth)
      for (int j = 0; j < G; j++)
        for (int k = 0; k < F; k++) K[((size_t)i * G + j) * F + k] = ssc_nava(freq[i], gam[j], freq[k]);
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nth; ++t) th.emplace_back(fill, t);
  for (auto& t : th) t.join();
  // kernels.h:79-91: integral over the scattered frequency
  std::vector<double> Kint((size_t)G * F, 0.);
  for (int j = 0; j < G; j++)
    for (int k = 0; k < F; k++) {
      double res = 0;
      for (int i = 0; i < F - 1; i++) res += K[((size_t)i * G + j) * F + k] * freq[i + 1] * (freq[i + 1] - freq[i]);
      Kint[(size_t)j * F + k] = res;
    }
  kscale.assign(F, 1.);
  for (int k = 0; k < F; k++) {
    double m = 0.;
    for (int j = 0; j < G; j++) m = std::max(m, Kint[(size_t)j * F + k]);
    if (m > 0. && m < 1e300) {
      int ex;
      std::frexp(m, &ex);
      kscale[k] = std::ldexp(1., ex);  // >= m, so the scaled column is <= 1
    }
  }
  KintT.assign((size_t)F * Gs, 0.f);
  for (int j = 0; j < G; j++)
    for (int k = 0; k < F; k++) KintT[(size_t)k * Gs + j] = (float)(Kint[(size_t)j * F + k] / kscale[k]);
  K32.assign((size_t)F * Gp * F, 0.f);
  for (int i = 0; i < F; i++)
    for (int j = 0; j < G; j++)
      for (int k = 0; k < F; k++) K32[((size_t)i * Gp + j) * F + k] = (float)K[((size_t)i * G + j) * F + k];
}

}  // namespace pbag
