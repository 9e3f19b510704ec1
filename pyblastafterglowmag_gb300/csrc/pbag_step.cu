// pbag_step.cu - per-blastwave kernels of one comoving-radiation step.
//
//   k_evolve_radiate : evaluateElectronDistributionNumericMixed (microphysics.h:359-489)
//                      or initializeElectronDistribution (microphysics.h:347-357),
//                      then the synchrotron part of computeRadiationNumericMixed
//                      (microphysics.h:498-506): kernel, j_syn, SSA, N_e, SSC weights.
//   k_finalize       : the rest of computeRadiationNumericMixed (microphysics.h:516-599)
//                      and storeDenseOutput (:602-633): photon field, totals,
//                      normalisation, intensity, history rows.
// The SSC contraction between them lives in pbag_ssc.cu.
//
// One CTA of 128 threads (4 warps, one per SM sub-partition) owns one
// blastwave. The Chang-Cooper substeps run as a systolic pipeline: thread t
// owns c = ceil(G/128) consecutive gamma bins and processes substep m at tick
// m + (T-1-t), one tick after the thread above it produced the bin it needs.
// The recurrence stays in FP64.
#include <cuda_runtime.h>

#include "pbag_device.cuh"
#include "pbag_kernels.h"

namespace pbag {

using namespace cgs;

namespace {

__device__ __forceinline__ bool bad_value(double v) {  // !isfinite(v) || v < 0
  return !(v >= 0.) || !(v <= 1.7976931348623157e308);
}

// Record the first error of a blastwave (later ones are ignored).
__device__ void set_error(const DevState& S, int b, int code, int step, int site) {
  if (atomicCAS(&S.err[4 * b], 0, code) == 0) {
    S.err[4 * b + 1] = step;
    S.err[4 * b + 2] = site;
  }
}

// microphysics.h:228-280: coefficient of the analytic broken power law,
// K_f (fast cooling, gm > gc) or K_s (slow cooling).
__device__ double power_law_norm(double gm, double gc, double gM, double p, double n_inj) {
  if (gm > gc)
    return n_inj / (pow(gm, 1. - p) * (1. / gc - 1. / gm) + 1. / p * (pow(gm, -p) - pow(gM, -p)));
  return n_inj / ((1. / (1. - p)) * (pow(gc, 1. - p) - pow(gm, 1. - p)) - gc / p * (pow(gM, -p) - pow(gc, -p)));
}

// Entry of the analytic distribution at gamma g; false when the reference
// leaves the entry untouched (neither branch applies).
__device__ bool power_law_at(double g, double gm, double gc, double gM, double p, double K, double& v) {
  if (gm > gc) {
    if ((gc <= g) && (g < gm)) {
      v = K * pow(gm, 1. - p) * pow(g, -2.);
      return true;
    }
    if ((gm < g) && (g <= gM)) {
      v = K * pow(g, -p - 1.);
      return true;
    }
  } else {
    if ((gm <= g) && (g < gc)) {
      v = K * pow(g, -p);
      return true;
    }
    if ((gc <= g) && (g <= gM)) {
      v = K * gc * pow(g, -p - 1.);
      return true;
    }
  }
  return false;
}

template <typename T>
__device__ T block_sum(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  T r = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += red[i];
  return r;
}

template <typename T>
__device__ T block_max(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  T r = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = max(r, red[i]);
  return r;
}

}  // namespace

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kStepThreads)
k_evolve_radiate(DevGrid g, DevState S, const pbag_step_rec* __restrict__ recs, const int64_t* __restrict__ off,
                 const pbag_shock_params* __restrict__ prm, int step) {
  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int G = g.G, F = g.F;
  __shared__ double sh_f[PBAG_MAX_BINS];   // heating term, then N(gamma)
  __shared__ double sh_u[PBAG_MAX_BINS];   // seed-photon weights (FP64)
  __shared__ double sh_v[PBAG_MAX_BINS];   // SSA weights
  __shared__ float sh_w[PBAG_MAX_BINS];    // synchrotron weights (FP32, scaled)
  __shared__ double red_d[kStepThreads / 32];
  __shared__ double xfer[2][kStepThreads / 32];
  __shared__ int sh_bad;

  int flags = S.flags[b];
  const int64_t r0 = off[b], len = off[b + 1] - off[b];
  bool active = S.err[4 * b] == 0 && step < len;
  pbag_step_rec r;
  if (active) {
    r = recs[r0 + step];
    active = r.mode != PBAG_SKIP;
  }
  if (tid == 0) sh_bad = 0;
  __syncthreads();  // every thread has read flags before thread 0 rewrites them
  if (tid == 0) S.flags[b] = flags & ~kFlagActive;
  if (!active) return;
  const pbag_shock_params P = prm[b];
  double* f = S.f + (size_t)b * G;
  double* scal = S.scal + (size_t)b * kScal;

#define PBAG_FAIL(code)                                 \
  do {                                                  \
    if (tid == 0) set_error(S, b, (code), step, __LINE__); \
    return;                                             \
  } while (0)

  double dr_comov, vol;
  int nsub_taken = 0;
  if (!(flags & kFlagInit)) {
    // ---- initializeElectronDistribution (microphysics.h:347-357)
    dr_comov = r.dr;
    vol = r.m_p1 / r.rho_p1;
    const double K = power_law_norm(r.gamma_min, r.gamma_c, r.gamma_max, P.p, r.m_p1 / m_p);
    bool bad = false;
    for (int i = tid; i < G; i += kStepThreads) {
      double v;
      double fi = power_law_at(g.e[i], r.gamma_min, r.gamma_c, r.gamma_max, P.p, K, v) ? v : f[i];
      if (bad_value(fi)) bad = true;
      if (i < G - 1) fi *= r.accel_frac;
      f[i] = fi;
    }
    if (bad) atomicOr(&sh_bad, 1);
    __syncthreads();
    if (sh_bad) PBAG_FAIL(PBAG_ERR_NONFINITE);
    flags |= kFlagInit;
  } else {
    // ---- evaluateElectronDistributionNumericMixed (microphysics.h:359-489)
    if ((r.B <= 0) || (r.gamma_min < 1.) || (r.gamma_max <= 1.) || (r.gamma_min >= r.gamma_max) ||
        (r.accel_frac > 1.))
      PBAG_FAIL(PBAG_ERR_PARAM);
    dr_comov = r.dr;
    const double gm = r.gamma_min, gM = r.gamma_max, gc = r.gamma_c, p = P.p;
    const double K = power_law_norm(gm, gc, gM, p, r.m_p1 / m_p);
    const double dt = r.tc_p1 - r.tc;
    const double volume = r.m / r.rho;
    const double volume_p1 = r.m_p1 / r.rho_p1;
    const double dlnVdt = P.adi_on ? 1. / dt * (1. - volume / volume_p1) : 0.;
    const bool analytic = P.ele_method == PBAG_ELE_MIX || gm <= 2;
    // the analytic distribution is always evaluated (microphysics.h:389-390)
    // and the reference exits if an assigned entry is not finite or negative
    bool bad = false;
    for (int i = tid; i < G; i += kStepThreads) {
      double v = 0.;
      const bool set = power_law_at(g.e[i], gm, gc, gM, p, K, v);
      if (set && bad_value(v)) bad = true;
      if (analytic) f[i] = set ? v : 0.;
    }
    if (bad) atomicOr(&sh_bad, 1);
    __syncthreads();
    if (sh_bad) PBAG_FAIL(PBAG_ERR_NONFINITE);
    if ((!isfinite(dlnVdt)) || (dlnVdt < 0)) PBAG_FAIL(PBAG_ERR_DLNVDT);
    // substep count (microphysics.h:412-435)
    const double dts = sigma_T * gM * r.B * r.B / (6. * M_PI * m_e * c_light);
    const double dta = (gM * gM - 1.) / (3. * gM * gM) * dlnVdt;
    double delta_t = g.dlog_gam / (dts + dta);
    int n_sub;
    const int max_sub = P.max_substeps;
    if (delta_t >= dt / 1.) {
      delta_t = dt / 1.;
      n_sub = 1;
    } else if (delta_t < dt / (double)max_sub) {
      delta_t = dt / (double)max_sub;
      n_sub = max_sub;
    } else {
      n_sub = (int)(dt / delta_t);
    }
    vol = volume;
    if (!analytic) {
      nsub_taken = n_sub;
      const double Nsrc = (r.m_p1 - r.m) / m_p / dt;
      const double index = -p;
      const double norm = (1 + index) / (pow(gM, index + 1) - pow(gm, index + 1));
      const bool ssc = P.ssc_on && g.K32 != nullptr;
      // seed-photon weights n_k (nu_{k+1}-nu_k)/nu_k of the previous step
      if (ssc) {
        const double* n = S.n + (size_t)b * F;
        for (int k = tid; k < F; k += kStepThreads) sh_u[k] = n[k] / g.nu[k] * (g.nu[k + 1] - g.nu[k]);
      }
      __syncthreads();
      // heating / cooling terms at the half grid (numeric_model.h:753-801);
      // constant over the substeps, so evaluated once per step
      const double c_syn = sigma_T / (6. * M_PI * m_e * c_light);
      const double c_ssc = 3. / 4. * h_pl * sigma_T / m_e / c_light;
      double* gsyn = S.gdot + (size_t)b * 3 * G;
      double* gadi = gsyn + G;
      double* gssc = gadi + G;
      bool hbad = false;
      for (int i = tid; i < G - 1; i += kStepThreads) {
        const double ga = g.half[i];
        const double vs = c_syn * r.B * r.B * ga * ga;
        const double va = dlnVdt * (ga * ga - 1.) / (3. * ga);
        double vc = gssc[i];
        if (ssc) {
          const double* kr = g.Kint + (size_t)i * F;
          double res = 0;
          for (int k = 0; k < F - 1; k++) res = fma(sh_u[k], kr[k], res);
          vc = c_ssc * res / ga / ga;
          gssc[i] = vc;
        }
        gsyn[i] = vs;
        gadi[i] = va;
        const double H = vs + va + vc;
        if (!isfinite(H)) hbad = true;
        sh_f[i] = H;
      }
      if (tid == 0) sh_f[G - 1] = 0.;  // heating_term[G-1] is never set (numeric_model.h:761)
      if (hbad) atomicOr(&sh_bad, 1);
      __syncthreads();
      if (sh_bad) PBAG_FAIL(PBAG_ERR_NONFINITE);
      // tridiagonal coefficients (numeric_model.h:539-675 with dispersion = 0,
      // delta_j = 0): a = 0, b_k = 1 + dt H_{k-1}/dgb_k (b_0 = b_{G-1} = 1),
      // c_k = -dt H_k/dgb_k (c_{G-1} = 0). Each substep is the back
      // substitution f_k = (f_k + Q_k dt)/b_k - (c_k/b_k) f_{k+1}
      // (numeric_model.h:19-43, 682-708).
      const int c = (G + kStepThreads - 1) / kStepThreads;
      const int T = (G + c - 1) / c;  // threads that own bins
      double fr[kMaxPerThread], ib[kMaxPerThread], qb[kMaxPerThread], bt[kMaxPerThread];
#pragma unroll
      for (int q = 0; q < kMaxPerThread; ++q) {
        const int j = tid * c + q;
        fr[q] = ib[q] = qb[q] = bt[q] = 0.;
        if (q < c && j < G) {
          const double odgb = 1.0 / g.dgb[j];
          double braw, craw;
          if (j == 0) {
            braw = -odgb * ((0. + 0.) + 0. * 0. - 0. * sh_f[0]);
            craw = odgb * (1. * sh_f[0] + 0.);
          } else if (j == G - 1) {
            braw = -odgb * ((0. + 0.) + 1. * sh_f[G - 1] - 0.);
            craw = 0.;
          } else {
            braw = -odgb * ((0. + 0.) + 1. * sh_f[j - 1] - 0. * sh_f[j]);
            craw = odgb * (1. * sh_f[j] + 0.);
          }
          const double bb = (1. - braw * delta_t) + 0. * delta_t;
          const double cc = craw * -delta_t;
          const double Q = ((g.e[j] > gm) && (g.e[j] <= gM)) ? Nsrc * norm * pow(g.e[j], index) : 0.;
          ib[q] = 1. / bb;
          bt[q] = -(cc / bb);
          qb[q] = (Q * delta_t) / bb;
          fr[q] = f[j];
        }
      }
      // systolic substeps: thread t handles substep m = tau - (T-1-t)
      const int lane = tid & 31, warp = tid >> 5;
      if (tid < 2 * (kStepThreads / 32)) (&xfer[0][0])[tid] = 0.;
      __syncthreads();
      double low = 0.;
      bool sbad = false;
      const int ticks = n_sub + T - 1;
      for (int tau = 0; tau < ticks; ++tau) {
        double up = __shfl_down_sync(0xffffffffu, low, 1);
        if (lane == 31) up = warp + 1 < kStepThreads / 32 ? xfer[tau & 1][warp + 1] : 0.;
        const int m = tau - (T - 1 - tid);
        if (tid < T && m >= 0 && m < n_sub) {
          double fn = up;
#pragma unroll
          for (int q = kMaxPerThread - 1; q >= 0; --q) {
            if (q < c) {
              sbad |= bad_value(fr[q]);  // solve() checks f before each substep (numeric_model.h:688)
              const double a = fma(fr[q], ib[q], qb[q]);
              fr[q] = fma(bt[q], fn, a);
              fn = fr[q];
            }
          }
          low = fr[0];
        }
        if (lane == 0) xfer[(tau + 1) & 1][warp] = low;
        __syncthreads();
      }
      if (sbad) atomicOr(&sh_bad, 1);
#pragma unroll
      for (int q = 0; q < kMaxPerThread; ++q) {
        const int j = tid * c + q;
        if (q < c && j < G) f[j] = fr[q];
      }
      __syncthreads();
      if (sh_bad) PBAG_FAIL(PBAG_ERR_NONFINITE);
    }
  }
  __syncthreads();

  // ---- computeRadiationNumericMixed, synchrotron part (microphysics.h:498-506)
  const double B = r.B;
  if (B < 0) PBAG_FAIL(PBAG_ERR_PARAM);  // evalSynKernel (kernels.h:529-532)
  for (int i = tid; i < G; i += kStepThreads) sh_f[i] = f[i];
  __syncthreads();
  // N_e (microphysics.h:556-558) and the weights f_j (e_{j+1}-e_j)
  double ne = 0., wmax = 0.;
  for (int i = tid; i < G - 1; i += kStepThreads) {
    const double w = sh_f[i] * g.de[i];
    ne += w;
    wmax = fmax(wmax, w);
  }
  ne = block_sum(ne, red_d);
  wmax = block_max(wmax, red_d);
  const double sw = pow2_scale(wmax);
  // SSA: dfde = d(f/gamma^2)/dgamma, stateful (base_state.h:482-501, numeric_model.h:193-196)
  double* dfde = S.dfde + (size_t)b * G;
  if (P.ssa_on) {
    for (int i = tid; i < G; i += kStepThreads) {
      const double t = sh_f[i] / g.e[i] / g.e[i];
      if (t > 0) {
        double d;
        if (i == 0) {
          const double t1 = sh_f[1] / g.e[1] / g.e[1], t2 = sh_f[2] / g.e[2] / g.e[2];
          d = -1.5 * t + 2. * t1 - 0.5 * t2;
        } else if (i == G - 1) {
          const double t1 = sh_f[G - 2] / g.e[G - 2] / g.e[G - 2], t2 = sh_f[G - 3] / g.e[G - 3] / g.e[G - 3];
          d = 1.5 * t - 2. * t1 + 0.5 * t2;
        } else {
          const double tp = sh_f[i + 1] / g.e[i + 1] / g.e[i + 1], tm = sh_f[i - 1] / g.e[i - 1] / g.e[i - 1];
          d = 0.5 * (tp - tm) / (g.e[i] - g.e[i - 1]);
        }
        dfde[i] = d;
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < G; i += kStepThreads) {
    sh_w[i] = i < G - 1 ? (float)(sh_f[i] * g.de[i] * sw) : 0.f;
    sh_v[i] = (P.ssa_on && i < G - 1) ? g.e[i] * g.e[i] * (g.e[i + 1] - g.e[i]) * dfde[i] : 0.;
  }
  __syncthreads();
  // kernel prefactor (kernels.h:427 CSYN, :471 Dermer09) and nu / nu_crit
  const bool dermer = P.syn_method == PBAG_SYN_DER09;
  const double pref = dermer ? sqrt3 * pow(q_e, 3.) * B / (m_e * c_light * c_light) : sqrt3 * pow(q_e, 3.) * B / mec2;
  const double inv_ncrit = (4. * M_PI * m_e * c_light) / (3. * q_e * B);  // 1/nu_crit(B, 1) (kernels.h:194-197)
  const double inv_nlar = (2. * pi_ * m_e * c_light) / (3. * q_e * B);    // 1/nu_larmor(B) (kernels.h:199-202)
  const int jcyc = dermer ? 0 : g.n_cyc;  // bins with gamma <= 2 use the cyclotron branch (CSYN only)
  double* jsyn = S.jsyn + (size_t)b * F;
  double* asyn = S.asyn + (size_t)b * F;
  bool jbad = false;
  for (int k = tid; k < F; k += kStepThreads) {
    const double nu = g.nu[k];
    const float a_k = (float)(nu * inv_ncrit);
    const float xl = (float)(nu * inv_nlar);
    float acc = 0.f;
    double acca = 0.;
    for (int j = 0; j < G - 1; ++j) {
      float R;
      if (j >= jcyc) {
        R = aharonian_R32(a_k * g.ginv2[j]);
      } else {  // cyclotron branch of cycSynch (kernels.h:428-435)
        const float psq = g.psq32[j];
        R = (2.f * psq) / (1.f + 3.f * psq) * expf((2.f * (1.f - xl)) / (1.f + 3.f * psq));
      }
      acc = fmaf(R, sh_w[j], acc);
      if (P.ssa_on) acca = fma((double)R, sh_v[j], acca);
    }
    const double js = k < F - 1 ? pref * ((double)acc / sw) : 0.;  // j_syn[F-1] = 0 (numeric_model.h:157)
    if (!isfinite(js) || js < 0.) jbad = true;
    jsyn[k] = js;
    if (P.ssa_on) {
      double a = pref * acca;
      a *= -1. / (8. * M_PI * m_e * nu * nu);
      a = fabs(a);
      if (!isfinite(a)) a = 1e99;
      asyn[k] = a;
    } else {
      asyn[k] = 0.;
    }
  }
  if (jbad) atomicOr(&sh_bad, 1);
  // SSC electron weights W_j = f_j (e_{j+1}-e_j) 3/4 sigma_T c / e_j^2 (numeric_model.h:271-277)
  if (P.ssc_on && g.K32 != nullptr) {
    double wm = 0.;
    for (int j = tid; j < G - 1; j += kStepThreads)
      wm = fmax(wm, sh_f[j] * g.de[j] * (3. / 4. * sigma_T * c_light / (g.e[j] * g.e[j])));
    wm = block_max(wm, red_d);
    const double s = pow2_scale(wm);
    float* W = S.W32 + (size_t)b * g.Gp;
    for (int j = tid; j < g.Gp; j += kStepThreads)
      W[j] = j < G - 1 ? (float)(sh_f[j] * g.de[j] * (3. / 4. * sigma_T * c_light / (g.e[j] * g.e[j])) * s) : 0.f;
    if (tid == 0) scal[kScalSW] = 1. / s;
  }
  __syncthreads();
  if (sh_bad) PBAG_FAIL(PBAG_ERR_NONFINITE);
  if (ne <= 0) PBAG_FAIL(PBAG_ERR_NELE);  // microphysics.h:560-563
  if (tid == 0) {
    scal[kScalDr] = dr_comov;
    scal[kScalVol] = vol;
    scal[kScalNele] = ne;
    scal[kScalAcc] = r.accel_frac;
    scal[kScalNp] = r.n_prime;
    scal[kScalNsub] = (double)nsub_taken;
    S.flags[b] = flags | kFlagActive;
  }
#undef PBAG_FAIL
}

// ---------------------------------------------------------------------------
__device__ __forceinline__ double intensity_approx(double em, double dtau) {  // microphysics.h:11-58, iAPPROX
  if (dtau == 0) return em;
  const double u = 1. / 2. + exp(-dtau) / dtau - (1 - exp(-dtau)) / (dtau * dtau);
  return dtau > 1.e-3 ? em * (3. * u / dtau) : em;
}

__global__ void __launch_bounds__(kStepThreads)
k_finalize(DevGrid g, DevState S, const int64_t* __restrict__ off, const pbag_shock_params* __restrict__ prm,
           int step, pbag_outputs out) {
  const int b = blockIdx.x, tid = threadIdx.x;
  const int G = g.G, F = g.F;
  __shared__ double red_d[kStepThreads / 32];
  const int flags = S.flags[b];
  if (!(flags & kFlagActive)) return;
  const pbag_shock_params P = prm[b];
  const double* scal = S.scal + (size_t)b * kScal;
  const double dr = scal[kScalDr], vol = scal[kScalVol], ne = scal[kScalNele];
  const double acc = scal[kScalAcc], np = scal[kScalNp];
  const bool num = P.ele_method == PBAG_ELE_NUMERIC;
  const bool ssc = P.ssc_on && g.K32 != nullptr;
  const bool dense_syn = out.syn_j_all || out.syn_a_all || out.syn_i_all;
  const size_t row = (size_t)(off[b] + step);
  double* n = S.n + (size_t)b * F;
  const double* jsyn = S.jsyn + (size_t)b * F;
  const double* asyn = S.asyn + (size_t)b * F;
  const double* jssc = S.jssc + (size_t)b * F;
  // new photon density (microphysics.h:516-523)
  const double Tesc = dr / c_light;
  const double fac = Tesc / vol;
  bool bad = false, seen = false;
  double umax = 0.;
  for (int k = tid; k < F; k += kStepThreads) {
    const double nu = g.nu[k];
    double nk = jsyn[k] * fac / (h_pl * nu);
    if (num && ssc) nk += jssc[k] * fac / (h_pl * nu);
    n[k] = nk;
    umax = fmax(umax, nk / nu * (g.nu[k + 1] - nu));
    // totals and normalisation (microphysics.h:540-586)
    double tj = jsyn[k];
    if (num && ssc) tj += jssc[k];
    double ta = asyn[k];
    ta = ta / ne * acc * np;
    const double dtau = ta * dr;
    const double ti = intensity_approx(tj * acc, dtau);
    tj = tj * acc / ne;
    if (!isfinite(tj) || tj < 0.) bad = true;
    if (out.j_all) out.j_all[row * F + k] = tj;
    if (out.a_all) out.a_all[row * F + k] = ta;
    if (out.f_all) out.f_all[row * F + k] = nk;
    if (out.i_all) out.i_all[row * F + k] = ti;
    // storeDenseOutput (microphysics.h:602-633)
    if (dense_syn) {
      const double sj = jsyn[k] * acc;
      const double sa = asyn[k] / ne * acc * np;
      if (out.syn_j_all) out.syn_j_all[row * F + k] = sj;
      if (out.syn_a_all) out.syn_a_all[row * F + k] = sa;
      if (out.syn_i_all) out.syn_i_all[row * F + k] = intensity_approx(sj, sa * dr);
      if (sj != 0.) seen = true;
    }
    if (ssc) {
      const double cj = jssc[k] * acc;
      if (out.ssc_j_all) out.ssc_j_all[row * F + k] = cj;
      if (out.ssc_i_all) out.ssc_i_all[row * F + k] = cj;  // ssc.a = 0 without pair production
    }
  }
  if (out.ele_f_all || out.gdot_syn_all || out.gdot_adi_all || out.gdot_ssc_all) {
    const double* f = S.f + (size_t)b * G;
    const double* gd = S.gdot + (size_t)b * 3 * G;
    for (int i = tid; i < G; i += kStepThreads) {
      if (out.ele_f_all) out.ele_f_all[row * G + i] = f[i];
      if (out.gdot_syn_all) out.gdot_syn_all[row * G + i] = gd[i];
      if (out.gdot_adi_all) out.gdot_adi_all[row * G + i] = gd[G + i];
      if (out.gdot_ssc_all) out.gdot_ssc_all[row * G + i] = gd[2 * G + i];
    }
  }
  // seed-photon weights of this step for the next step's SSC contraction
  umax = block_max(umax, red_d);
  const double su = pow2_scale(umax);
  if (ssc) {
    float* U = S.U32 + (size_t)b * F;
    for (int k = tid; k < F; k += kStepThreads) U[k] = (float)(n[k] / g.nu[k] * (g.nu[k + 1] - g.nu[k]) * su);
  }
  const int any_bad = __syncthreads_or(bad ? 1 : 0);
  const int any_seen = __syncthreads_or(seen ? 1 : 0);
  if (tid == 0) {
    int fl = flags;
    if (any_seen) fl |= kFlagSynSeen;
    if (ssc) {
      S.scal[(size_t)b * kScal + kScalSU] = 1. / su;
      fl |= kFlagUValid;
    }
    S.flags[b] = fl;
    if (any_bad)
      set_error(S, b, PBAG_ERR_NONFINITE, step, __LINE__);
    else if (dense_syn && !(fl & kFlagSynSeen) && step > 0)
      set_error(S, b, PBAG_ERR_NONFINITE, step, __LINE__);  // microphysics.h:627-631
  }
}

// ---------------------------------------------------------------------------
cudaError_t launch_evolve_radiate(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const int64_t* off,
                                  const pbag_shock_params* prm, int nbw, int step, cudaStream_t st) {
  k_evolve_radiate<<<nbw, kStepThreads, 0, st>>>(g, S, recs, off, prm, step);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DevGrid& g, const DevState& S, const int64_t* off, const pbag_shock_params* prm,
                            int nbw, int step, const pbag_outputs& out, cudaStream_t st) {
  k_finalize<<<nbw, kStepThreads, 0, st>>>(g, S, off, prm, step, out);
  return cudaGetLastError();
}

}  // namespace pbag
