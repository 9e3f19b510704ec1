// pbag_device.cuh - device-side data layout and helpers shared by the step
// kernels. Paths in comments are relative to the reference's src/ directory.
#ifndef PBAG_DEVICE_CUH
#define PBAG_DEVICE_CUH

#include <cstdint>

#include "pbag.h"
#include "pbag_const.h"

namespace pbag {

constexpr int kStepThreads = 128;     // threads per blastwave in the step kernels
constexpr int kKernelClasses = 3;     // evolve, ssc, finalize (pbag_kernel_class)
constexpr int kClassEvolve = PBAG_K_EVOLVE, kClassSsc = PBAG_K_SSC, kClassFinalize = PBAG_K_FINALIZE;
constexpr int kMaxPerThread = (PBAG_MAX_BINS + kStepThreads - 1) / kStepThreads;  // gamma bins per thread

// Read-only tables of one grid (one CommonTables entry), device pointers.
struct DevGrid {
  int G, F, Gp;          // Gp: G rounded up to a multiple of 16 (padded SSC operand)
  int n_cyc;             // number of bins with e[j] <= 2 (cyclotron branch of cycSynch)
  double dlog_gam;       // (e[1]-e[0])/e[0] (microphysics.h:413)
  const float* psq32;    // [G]   e[j]^2 - 1 in FP32 (cyclotron branch)
  const double* e;       // [G]   gamma grid e[i] = step^i
  const double* half;    // [G-1] half grid (base_state.h:237)
  const double* de;      // [G-1] e[j+1]-e[j]
  const double* dgb;     // [G]   delta_grid_bar (base_state.h:248-250)
  const float* ginv2;    // [G]   1/e[j]^2 (FP32, synchrotron argument)
  const double* nu;      // [F+1] frequency grid, nu[F] = next logspace point
  const double* dnu_nu;  // [F]   (nu[k+1]-nu[k])/nu[k]
  const double* Kint;    // [G][F] SSC kernel integral (kernels.h:79-91), FP64
  const float* K32;      // [F][Gp][F] SSC kernel (i, j, k) in FP32, j >= G zero
};

// Per-blastwave state that lives across steps (structure of arrays).
struct DevState {
  double* f;       // [nbw][G]   N(gamma) (ele.f)
  double* dfde;    // [nbw][G]   d(f/gamma^2)/dgamma, stateful (base_state.h:482-536)
  double* gdot;    // [nbw][3][G] gam_dot_syn, _adi, _ssc (last substep)
  double* n;       // [nbw][F]   photon density total_rad.f of the previous step
  double* jsyn;    // [nbw][F]   synchrotron emissivity of this step
  double* asyn;    // [nbw][F]   SSA absorption of this step
  double* jssc;    // [nbw][F]   SSC emissivity of this step
  float* W32;      // [nbw][Gp]  SSC electron weights, scaled to FP32
  float* U32;      // [nbw][F]   SSC seed-photon weights, scaled to FP32
  double* scal;    // [nbw][kScal] per-step scalars handed between kernels
  int* flags;      // [nbw]      kFlag* bits
  int* err;        // [nbw][4]   first error: code, step index, check site, unused
};

enum : int {
  kScalDr = 0,     // dr_comov of this step
  kScalVol = 1,    // source.vol of this step
  kScalNele = 2,   // total electron number
  kScalSW = 3,     // scale of W32 (true value = W32 * sW)
  kScalSU = 4,     // scale of U32
  kScalAcc = 5,    // accel_frac of this step
  kScalNp = 6,     // n_prime of this step
  kScalNsub = 7,   // substeps taken (diagnostic)
  kScal = 8
};

enum : int {
  kFlagInit = 1,     // distribution initialised (is_distribution_initialized)
  kFlagActive = 2,   // blastwave radiates at the current step
  kFlagSynSeen = 4,  // a non-zero synchrotron emissivity was produced (dense check)
  kFlagUValid = 8    // U32/sU hold the previous step's photon field
};

// Power of two close to 1/max|x| (exact rescaling); 1 when max is 0 or not finite.
__host__ __device__ inline double pow2_scale(double maxabs) {
  if (!(maxabs > 0.) || !(maxabs < 1.e308)) return 1.;
  int ex;
  frexp(maxabs, &ex);
  return ldexp(1., -ex);
}

// ---- synchrotron kernel functions in FP32 (kernels.h) ---------------------
// All return the dimensionless shape R; the caller multiplies by the FP64
// prefactor sqrt(3) q^3 B / (m_e c^2) of kernels.h:427,434,471.

// Aharonian+2010 eq. D7 fit (kernels.h:420-427), x = nu / nu_crit. Beyond
// x = 150 the factor exp(-x) is below the smallest FP32 subnormal, so the
// value is 0 (this also keeps x^(4/3) from overflowing for huge x).
__device__ __forceinline__ float aharonian_R32(float x) {
  if (!(x <= 150.f)) return x > 150.f ? 0.f : x;  // NaN propagates
  float y = cbrtf(x);
  float y2 = y * y;
  float y4 = y2 * y2;
  float num = fmaf(0.347f, y4, fmaf(2.21f, y2, 1.f));
  float den = fmaf(0.217f, y4, fmaf(1.353f, y2, 1.f));
  return 1.808f * y * rsqrtf(fmaf(3.4f, y2, 1.f)) * num / den * expf(-x);
}

// Chebyshev recurrence (kernels.h:158-173) on [-1,1].
__device__ __forceinline__ float cheb32(const float* c, int order, float t) {
  float d = 0.f, dd = 0.f, y2 = 2.f * t;
  for (int j = order; j > 0; j--) {
    float tmp = d;
    d = fmaf(y2, d, -dd) + c[j];
    dd = tmp;
  }
  return fmaf(t, d, -dd) + 0.5f * c[0];
}

}  // namespace pbag

#endif
