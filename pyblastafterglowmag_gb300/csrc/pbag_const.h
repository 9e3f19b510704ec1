// pbag_const.h - CGS constants of the reference (utilitites/utils.h:18-60),
// usable from host and device code.
#ifndef PBAG_CONST_H
#define PBAG_CONST_H

namespace pbag {
namespace cgs {
constexpr double c_light = 2.99792458e10;          // speed of light [cm/s]
constexpr double pi_ = 3.141592653589793;          // CGS::pi and M_PI
constexpr double m_p = 1.6726e-24;                 // proton mass [g]
constexpr double m_e = 9.1094e-28;                 // electron mass [g]
constexpr double q_e = 4.803204e-10;               // electron charge [esu]
constexpr double sigma_T = 6.6524e-25;             // Thomson cross-section [cm^2]
constexpr double h_pl = 6.6260755e-27;             // Planck constant [erg s]
constexpr double mec2 = 8.187105649650028e-07;     // m_e c^2 [erg]
constexpr double h_by_mec2 = h_pl / m_e / c_light / c_light;
constexpr double sqrt3 = 1.7320508075688772;
}  // namespace cgs
}  // namespace pbag

#endif
