// pbag_syntab.cpp - tabulated synchrotron functions of SynKernel for the GPU
// radiation sums: the "GSL" and "Bessel" methods (kernels.h:211-342, 396-412),
// and the Aharonian fit of "CSYN" / "Dermer09" (kernels.h:420-427, 463-469)
// for the batch contraction, which interpolates instead of evaluating the fit.
//
// Both functions depend on the state only through their argument x: the GSL
// method's F(x) = x int_x^inf K_5/3 (x = h nu / m_e c^2 / (1.5 B / 4.14e13
// gamma^2), kernels.h:282-285), the Bessel method's 2 t^2 (K_4/3 K_1/3 -
// 3/5 t (K_4/3^2 - K_1/3^2)) (t = nu / nu_crit). They are tabulated once per
// context in FP64 on the host as g(u) = R(e^u) e^(-u/3), u = ln x, on a uniform
// grid in u; g is smooth and tends to a constant for x -> 0 (R ~ x^(1/3)), so
// the device interpolates g linearly and multiplies by x^(1/3), which it forms
// from its tabulated factors. Below the table g keeps its first value; above it
// (x > kSynTabXmax, R < e^-120 relative) R is zero.
//
// F(x) is evaluated with the published Chebyshev expansions of GSL's
// synchrotron_1 (the numbers the reference embeds in kernels.h:213-279),
// summed by Clenshaw's recurrence; the Bessel functions come from the C++17
// special functions of the standard library (as the reference's own
// std::cyl_bessel_k, kernels.h:403-404).
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "pbag_internal.h"

namespace pbag {

namespace {

// Clenshaw sum of a Chebyshev series with coefficients c[0..order] at y in [-1, 1]
// (the first term halved, as in the expansions' convention)
double clenshaw(const double* c, int order, double y) {
  double d = 0., dd = 0.;
  const double y2 = 2. * y;
  for (int j = order; j > 0; --j) {
    const double t = d;
    d = y2 * d - dd + c[j];
    dd = t;
  }
  return y * d - dd + 0.5 * c[0];
}

// GSL synchrotron_1 expansions (published coefficients)
const double kSyn1[13] = {30.364682982501076273, 17.079395277408394574, 4.560132133545072889,
                          0.549281246730419979,  0.372976075069301172e-01, 0.161362430201041242e-02,
                          0.481916772120371e-04, 0.10512425288938e-05,    0.174638504670e-07,
                          0.22815486544e-09,     0.240443082e-11,          0.2086588e-13,
                          0.15167e-15};
const double kSyn2[12] = {0.4490721623532660844, 0.898353677994187218e-01, 0.81044573772151290e-02,
                          0.4261716991089162e-03, 0.147609631270746e-04,   0.3628633615300e-06,
                          0.66634807498e-08,      0.949077166e-10,         0.1079125e-11,
                          0.10022e-13,            0.77e-16,                0.5e-18};
const double kSyn1a[23] = {2.1329305161355000985, 0.741352864954200240e-01, 0.86968099909964198e-02,
                           0.11703826248775692e-02, 0.1645105798619192e-03, 0.240201021420640e-04,
                           0.35827756389389e-05,  0.5447747626984e-06,      0.838802856196e-07,
                           0.13069882684e-07,     0.2053099071e-08,         0.325187537e-09,
                           0.517914041e-10,       0.83002988e-11,           0.13352728e-11,
                           0.2159150e-12,         0.349967e-13,             0.56994e-14,
                           0.9291e-15,            0.152e-15,                0.249e-16,
                           0.41e-17,              0.7e-18};

// F(x) = x int_x^inf K_5/3 over the three ranges of kernels.h:282-330
double synchrotron_F(double x) {
  const double c0 = M_PI / std::sqrt(3.);
  const double c01 = 0.2257913526447274323630976;  // ln(sqrt(pi/2))
  const double x_small = 2. * std::sqrt(2.) * 1.4901161193847656e-08;
  const double x_big = -8.0 * (-7.0839641853226408e02) / 7.0;
  if (x < x_small) {
    const double z = std::cbrt(x);
    return 2.14952824153447863671 * z * (1. - 8.43812762813205e-01 * z * z);
  }
  if (x <= 4.) {
    const double px = std::cbrt(x), t = x * x / 8. - 1.;
    return px * clenshaw(kSyn1, 12, t) - std::pow(px, 11.) * clenshaw(kSyn2, 11, t) - c0 * x;
  }
  if (x < x_big) return std::sqrt(x) * clenshaw(kSyn1a, 22, (12. - x) / (x + 4.)) * std::exp(c01 - x);
  return 0.;
}

double synchrotron_bessel(double t) {
  try {
    const double k43 = std::cyl_bessel_k(4. / 3., t), k13 = std::cyl_bessel_k(1. / 3., t);
    return 2. * t * t * (k43 * k13 - 3. / 5. * t * (k43 * k43 - k13 * k13));
  } catch (const std::exception&) {
    return 0.;  // the reference's catch (kernels.h:406-408)
  }
}

// the Aharonian et al. (2010) fit of CSYN and Dermer09 (kernels.h:420-427, 463-469)
double synchrotron_aharonian(double x) {
  const double x13 = std::cbrt(x), x23 = x13 * x13, x43 = x23 * x23;
  return 1.808 * x13 / std::sqrt(1 + 3.4 * x23) * (1. + 2.21 * x23 + 0.347 * x43) /
         (1. + 1.353 * x23 + 0.217 * x43) * std::exp(-x);
}

}  // namespace

double syn_shape(int method, double x) {
  return method == PBAG_SYN_GSL ? synchrotron_F(x) : method == PBAG_SYN_BESSEL ? synchrotron_bessel(x)
                                                                               : synchrotron_aharonian(x);
}

void syn_table_grid(double dlng, double* u0, double* h, int* n, int nmax) {
  // spacing: the step of ln(1/gamma^2) between neighbouring electron bins is
  // m spacings, m odd, so that the lanes of a warp (consecutive bins) read
  // the table at indices m apart: distinct shared-memory banks
  const double span = std::log(kSynTabXmax) - std::log(kSynTabXmin);
  const double step2 = 2. * dlng;
  const double target = 2. * span / nmax;
  int m = (int)std::lround(step2 / target) | 1;
  while (m > 1 && span / (step2 / m) + 2 > nmax) m -= 2;
  *h = step2 / m;
  *u0 = std::log(kSynTabXmin);
  *n = std::min(nmax, (int)std::ceil(span / *h) + 2);
}

std::vector<float> syn_table(int method, double u0, double h, int n) {
  std::vector<float> g(kSynTabN, 0.f);
  for (int i = 0; i < n; ++i) {
    const double u = u0 + i * h, x = std::exp(u);
    const double R = method == PBAG_SYN_GSL      ? synchrotron_F(x)
                     : method == PBAG_SYN_BESSEL ? synchrotron_bessel(x)
                                                 : synchrotron_aharonian(x);
    g[i] = (float)(R * std::exp(-u / 3.));
  }
  return g;
}

std::vector<float> syn_table2(int method, double u0, double h, int n) {
  std::vector<double> g((size_t)n + 1, 0.);
  for (int i = 0; i < n; ++i) {
    const double u = u0 + i * h, x = std::exp(u);
    const double R = method == PBAG_SYN_GSL      ? synchrotron_F(x)
                     : method == PBAG_SYN_BESSEL ? synchrotron_bessel(x)
                                                 : synchrotron_aharonian(x);
    g[i] = R * std::exp(-u / 3.);
  }
  g[n - 1] = 0.;  // from the last point on: zero
  std::vector<float> t((size_t)2 * kSynTab2N, 0.f);
  for (int i = 0; i < n - 1; ++i) {
    t[2 * i] = (float)g[i];
    t[2 * i + 1] = i == 0 ? 0.f : (float)(0.5 * (g[i + 1] - g[i - 1]));
  }
  return t;
}

}  // namespace pbag
