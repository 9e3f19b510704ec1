// pbag_flux.cu - EATS flux density of cells from the comoving histories:
// ElectronAndRadiation::fluxDens (microphysics.h:1185-1217) and
// computeFluxDensity (microphysics.h:799-867), one thread per query, FP64 in
// the reference's operation order.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_device.cuh"

namespace pbag {

namespace {

constexpr int kFluxThreads = 128;
enum : int { kFluxRange = 1, kFluxNonfinite = 2 };

// EQS::BetaFromGamma (blastwave_components.h:36-39)
__device__ __forceinline__ double beta_from_gamma(double g) { return sqrt((g - 1.) * (g + 1.)) / g; }

// findIndex (interpolators.h:13-35): the grid interval of x by bisection
__device__ int find_index(double x, const double* __restrict__ a, int n) {
  if (x <= a[0]) return 0;
  if (x >= a[n - 1]) return n - 2;
  unsigned lo = 0, hi = (unsigned)n - 1;
  while (hi - lo > 1u) {
    const unsigned m = (hi + lo) >> 1;
    if (a[m] > x)
      hi = m;
    else
      lo = m;
  }
  return (int)lo;
}

// Interp2d::BilinearInterpolation (interpolators.h:786-801)
__device__ __forceinline__ double bilinear(double q11, double q12, double q21, double q22, double x1, double x2,
                                           double y1, double y2, double x, double y) {
  const double x2x1 = x2 - x1, y2y1 = y2 - y1, x2x = x2 - x, y2y = y2 - y, yy1 = y - y1, xx1 = x - x1;
  return 1.0 / (x2x1 * y2y1) * (q11 * x2x * y2y + q21 * xx1 * y2y + q12 * x2x * yy1 + q22 * xx1 * yy1);
}

// computeIntensity (microphysics.h:11-58)
__device__ double intensity_of(double em, double dtau, int method) {
  if (dtau == 0) return em;
  switch (method) {
    case PBAG_TAU_THICK:
      return dtau > 0 ? em / dtau : 0.;
    case PBAG_TAU_SMOOTH: {
      const double abs_fac = dtau > 0.0 ? -expm1(-dtau) / dtau : expm1(dtau) / dtau;
      return em * abs_fac;
    }
    case PBAG_TAU_SHARP:
      return dtau > 1.0 ? em / dtau : dtau < -1.0 ? 0.0 : em;
    default: {
      if (!(dtau > 1.e-3)) return em;
      const double e = exp(-dtau);
      const double u = 1. / 2. + e / dtau - (1 - e) / (dtau * dtau);
      return em * (3. * u / dtau);
    }
  }
}

__device__ __forceinline__ bool bad(double x) { return x < 0 || !isfinite(x); }

__global__ void __launch_bounds__(kFluxThreads)
k_flux_dens(pbag_flux_opts o, int F, const double* __restrict__ nu, const int64_t* __restrict__ off,
            const double* __restrict__ j_all, const double* __restrict__ a_all, const double* __restrict__ r_all,
            int nq, const pbag_flux_query* __restrict__ qs, double* __restrict__ flux,
            unsigned long long* __restrict__ first) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  const pbag_flux_query q = qs[t];
  auto fail = [&](int code) {
    atomicMin(first, ((unsigned long long)t << 4) | (unsigned long long)code);
    flux[t] = 0.;
  };
  // fluxDens: the frequency inside the grid, its interval, the bilinear
  // interpolation of the histories in (frequency, radius)
  if (q.freq >= nu[F - 1] || q.freq <= nu[0]) return fail(kFluxRange);
  const int ia_nu = find_index(q.freq, nu, F), ib_nu = ia_nu + 1;
  const int64_t r0 = off[q.bw];
  const double* ja = j_all + (size_t)(r0 + q.ia) * F;
  const double* jb = j_all + (size_t)(r0 + q.ib) * F;
  const double* aa = a_all + (size_t)(r0 + q.ia) * F;
  const double* ab = a_all + (size_t)(r0 + q.ib) * F;
  const double y1 = r_all[r0 + q.ia], y2 = r_all[r0 + q.ib];
  const double x1 = nu[ia_nu], x2 = nu[ib_nu];
  const double em_prime = bilinear(ja[ia_nu], jb[ia_nu], ja[ib_nu], jb[ib_nu], x1, x2, y1, y2, q.freq, q.r);
  const double abs_prime = bilinear(aa[ia_nu], ab[ia_nu], aa[ib_nu], ab[ib_nu], x1, x2, y1, y2, q.freq, q.r);
  // computeFluxDensity
  const double Gamma = q.Gamma, mu = q.mu, r = q.r;
  const double beta = beta_from_gamma(Gamma);
  const double a = 1.0 - beta * mu;
  const double delta_D = Gamma * a;
  const double em_lab = em_prime / (delta_D * delta_D);
  const double abs_lab = abs_prime * delta_D;
  const double beta_shock = beta_from_gamma(o.shock_vel == PBAG_VEL_SHOCK ? q.GammaSh : Gamma);
  const double m2 = q.ne * cgs::m_p;
  const double dr = m2 / (2. * cgs::pi_ * cgs::m_p * r * r * (1. - cos(q.theta) / q.ncells) * Gamma * q.n_prime);
  const double dtau = mu == beta_shock ? 1.0e100 : abs_lab * dr * (1. - mu * beta_shock) / (mu - beta_shock);
  const double intensity = intensity_of(em_lab, dtau, o.method_tau);
  if (bad(intensity)) return fail(kFluxNonfinite);
  const double ashock = 1.0 - mu * beta_shock;
  const double lum = o.method_ne == PBAG_NE_USE_NPRIME
                         ? intensity * r * r * (dr / ashock)
                         : intensity * q.ne / (2. * cgs::pi_ * (1. - cos(q.theta) / q.ncells)) / Gamma / ashock;
  if (bad(lum)) return fail(kFluxNonfinite);
  flux[t] = lum;
}

}  // namespace

}  // namespace pbag

using namespace pbag;

extern "C" int pbag_flux_dens(pbag_ctx* ctx, const pbag_flux_opts* opts, int nbw, const int64_t* offsets,
                              const double* d_j_all, const double* d_a_all, const double* d_r_all, int nq,
                              const pbag_flux_query* d_q, double* d_flux, pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || !opts || nbw < 0 || nq < 0 || !offsets) return PBAG_ERR_ARG;
  if (opts->shock_vel < PBAG_VEL_SAME_AS_BW || opts->shock_vel > PBAG_VEL_SHOCK ||
      opts->method_ne < PBAG_NE_USE_NPRIME || opts->method_ne > PBAG_NE_USE_NE ||
      opts->method_tau < PBAG_TAU_APPROX || opts->method_tau > PBAG_TAU_SHARP)
    return PBAG_ERR_ARG;
  if (nq == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  if (!d_j_all || !d_a_all || !d_r_all || !d_q || !d_flux || nbw == 0) return PBAG_ERR_ARG;
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  // the queries' blastwave and row indices are checked on the host
  std::vector<pbag_flux_query> hq((size_t)nq);
  if (cudaMemcpy(hq.data(), d_q, (size_t)nq * sizeof(pbag_flux_query), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PBAG_ERR_CUDA;
  for (int i = 0; i < nq; ++i) {
    const pbag_flux_query& q = hq[(size_t)i];
    if (q.bw < 0 || q.bw >= nbw) return PBAG_ERR_ARG;
    const int64_t n = offsets[q.bw + 1] - offsets[q.bw];
    if (q.ia < 0 || q.ib < 0 || q.ia >= n || q.ib >= n) return PBAG_ERR_ARG;
  }
  int64_t* d_off = nullptr;
  unsigned long long* d_first = nullptr;
  cudaError_t e = cudaMalloc(&d_off, (size_t)(nbw + 1) * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&d_first, sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_off, offsets, (size_t)(nbw + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_first, 0xff, sizeof(unsigned long long), v.stream);
  if (e == cudaSuccess) {
    k_flux_dens<<<(nq + kFluxThreads - 1) / kFluxThreads, kFluxThreads, 0, v.stream>>>(
        *opts, v.F, v.dg.nu, d_off, d_j_all, d_a_all, d_r_all, nq, d_q, d_flux, d_first);
    e = cudaGetLastError();
  }
  unsigned long long first = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  cudaFree(d_off);
  cudaFree(d_first);
  if (e != cudaSuccess) return PBAG_ERR_CUDA;
  if (first != ~0ull) {
    const int idx = (int)(first >> 4), code = (int)(first & 15ull) == 1 ? PBAG_ERR_RANGE : PBAG_ERR_NONFINITE;
    if (st) {
      st->code = code;
      st->bw = hq[(size_t)idx].bw;
      st->step = idx;
    }
    return code;
  }
  if (st) st->code = PBAG_OK;
  return PBAG_OK;
}
