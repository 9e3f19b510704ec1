// pbag_step.cu - the kernels of one comoving-radiation step.
//
// Once per batch:
//   k_first_valid : first valid record of every blastwave (its init step)
//   k_powp        : e_i^-p per blastwave (injection index p is per blastwave)
//   k_prep        : every per-record scalar of evaluateElectronDistributionNumericMixed
//                   (microphysics.h:359-489) and initializeElectronDistribution
//                   (:347-357) that depends on the record alone, all records in
//                   parallel: power-law normalisation and bin ranges, dlnV/dt,
//                   substep count and length, injection amplitude, synchrotron
//                   prefactors, and the exit conditions those lines check.
// Every step (one launch each over all blastwaves):
//   k_evolve      : the state-dependent part of the evolution - analytic
//                   distribution, or cooling terms (numeric_model.h:753-801) and
//                   the Chang-Cooper substeps (:539-708) - then N_e and the FP32
//                   weights of the synchrotron, SSA and SSC sums.
//   k_rad_ssc     : the O(F G) synchrotron and SSA sums (numeric_model.h:148-238)
//                   and the O(F^2 G) SSC contraction (pbag_ssc.cu), in one launch.
//   k_finalize    : photon field, totals, normalisation, intensity and history
//                   rows (microphysics.h:516-633).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "pbag_device.cuh"
#include "pbag_kernels.h"
#include "pbag_ssc.cuh"

namespace pbag {

using namespace cgs;

namespace {

// Block-wide max of a non-negative int (exponent fields), on the integer pipe.
__device__ int block_max_int(int v, int* red) {
  v = __reduce_max_sync(0xffffffffu, v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  int r = red[0];
  for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = max(r, red[i]);
  return r;
}

// (float)(x * scale_from_exp(E)) without FP64 arithmetic: the same single
// rounding of x's significand (f64_mant), the power of two added to the
// exponent; 0 below the FP32 normal range
__device__ __forceinline__ float f32_scaled(double x, int E) {
  int e;
  const float m = f64_mant(x, e);
  return f32_ldexp(m, (E <= 26 || E >= 2019) ? e : e + 1022 - E);
}

// Record the first error of a blastwave (later ones are ignored).
__device__ void set_error(const DevState& S, int b, int code, int step, int site) {
  if (atomicCAS(&S.err[4 * b], 0, code) == 0) {
    S.err[4 * b + 1] = step;
    S.err[4 * b + 2] = site;
  }
}

// first index with e[i] >= x (lower bound) / e[i] > x (upper bound)
__device__ int lower_bound_e(const double* e, int G, double x) {
  int lo = 0, hi = G;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (e[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ int upper_bound_e(const double* e, int G, double x) {
  int lo = 0, hi = G;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (e[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo;
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

// Error-free transformation a + b = s + e (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

}  // namespace

// ---------------------------------------------------------------------------
// One CTA per blastwave: its threads test kFirstValidThreads consecutive
// records at a time (independent loads, not one dependent chain per
// blastwave - a history that is never valid would otherwise cost one load
// latency per record).
__global__ void __launch_bounds__(kFirstValidThreads) k_first_valid(const pbag_step_rec* __restrict__ recs,
                                                                    const int64_t* __restrict__ off, int nbw,
                                                                    int64_t* __restrict__ first) {
  const int b = blockIdx.x;
  if (b >= nbw) return;
  const int64_t beg = off[b], end = off[b + 1];
  for (int64_t r0 = beg; r0 < end; r0 += kFirstValidThreads) {
    const int64_t r = r0 + threadIdx.x;
    const bool hit = r < end && recs[r].mode != PBAG_SKIP;
    if (__syncthreads_or(hit)) {
      __shared__ int lo;
      if (threadIdx.x == 0) lo = kFirstValidThreads;
      __syncthreads();
      if (hit) atomicMin(&lo, (int)threadIdx.x);
      __syncthreads();
      if (threadIdx.x == 0) first[b] = r0 + lo;
      return;
    }
  }
  if (threadIdx.x == 0) first[b] = end;  // the blastwave is never valid
}

__global__ void k_powp(DevGrid g, const pbag_shock_params* __restrict__ prm, int nbw, double* __restrict__ powp) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nbw * g.G) return;
  const int b = (int)(idx / g.G), i = (int)(idx - (int64_t)b * g.G);
  powp[idx] = pow(g.e[i], -prm[b].p);
}

// Value of the analytic distribution (microphysics.h:237-278) at bin i, given
// that i lies in branch a (first) or b (second).
__device__ __forceinline__ double pl_branch_a(const GridTab& T, const StepScal& s, const double* pp, int i) {
  return (s.flags & kRecFast) ? s.K * s.c_fast * T.gt(kTabInvE2)[i] : s.K * pp[i];
}
__device__ __forceinline__ double pl_branch_b(const GridTab& T, const StepScal& s, const double* pp, int i,
                                              double Kb) {
  return Kb * pp[i] * T.gt(kTabInvE)[i];
}

__global__ void k_prep(DevGrid g, const pbag_step_rec* __restrict__ recs, const int64_t* __restrict__ off,
                       const pbag_shock_params* __restrict__ prm, int nbw, int64_t nrec,
                       const int64_t* __restrict__ first, const double* __restrict__ powp,
                       StepScal* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  int lo = 0, hi = nbw;  // blastwave owning record r: last b with off[b] <= r
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= r) lo = mid; else hi = mid;
  }
  const int b = lo;
  const pbag_step_rec q = recs[r];
  StepScal s = {};
  if (q.mode == PBAG_SKIP) {
    out[r] = s;
    return;
  }
  const pbag_shock_params P = prm[b];
  const int G = g.G;
  const double* pp = powp + (size_t)b * G;
  s.flags = kRecValid;
  const bool init = r == first[b];
  if (init) s.flags |= kRecInit;
  const double gm = q.gamma_min, gc = q.gamma_c, gM = q.gamma_max, p = P.p;
  // powerLawElectronDistributionAnalytic (microphysics.h:228-280), n_inj = m/m_p
  const double n_inj = q.m_p1 / m_p;
  const bool fast = gm > gc;
  double Kb;
  if (fast) {
    s.flags |= kRecFast;
    s.K = n_inj / (pow(gm, 1. - p) * (1. / gc - 1. / gm) + 1. / p * (pow(gm, -p) - pow(gM, -p)));
    s.c_fast = pow(gm, 1. - p);
    s.ia0 = lower_bound_e(g.e, G, gc);  // gc <= gamma < gm
    s.ia1 = lower_bound_e(g.e, G, gm);
    s.ib0 = upper_bound_e(g.e, G, gm);  // gm < gamma <= gM
    s.ib1 = upper_bound_e(g.e, G, gM);
    Kb = s.K;
  } else {
    s.K = n_inj / ((1. / (1. - p)) * (pow(gc, 1. - p) - pow(gm, 1. - p)) - gc / p * (pow(gM, -p) - pow(gc, -p)));
    s.c_fast = 0.;
    s.ia0 = lower_bound_e(g.e, G, gm);  // gm <= gamma < gc
    s.ia1 = lower_bound_e(g.e, G, gc);
    s.ib0 = lower_bound_e(g.e, G, gc);  // gc <= gamma <= gM
    s.ib1 = upper_bound_e(g.e, G, gM);
    Kb = s.K * gc;
  }
  if (s.ia1 < s.ia0) s.ia1 = s.ia0;
  if (s.ib1 < s.ib0) s.ib1 = s.ib0;
  // the reference exits when an assigned entry is not finite or negative; the
  // entries of each branch decrease with gamma, so its first entry decides
  const GridTab T{g.etab, g.Ge, g.Fe};
  bool pl_bad = (s.ia1 > s.ia0 && bad_value(pl_branch_a(T, s, pp, s.ia0))) ||
                (s.ib1 > s.ib0 && bad_value(pl_branch_b(T, s, pp, s.ib0, Kb)));
  // synchrotron kernel constants (kernels.h:194-202, 427, 471)
  const double B = q.B;
  // Dermer09 and Bessel divide by m_e c c, CSYN and GSL by mec2 (kernels.h:342, 410, 427, 471)
  const bool mcc = P.syn_method == PBAG_SYN_DER09 || P.syn_method == PBAG_SYN_BESSEL;
  s.pref = mcc ? sqrt3 * pow(q_e, 3.) * B / (m_e * c_light * c_light) : sqrt3 * pow(q_e, 3.) * B / mec2;
  s.inv_ncrit = (float)((4. * M_PI * m_e * c_light) / (3. * q_e * B));
  s.inv_nlar = (float)((2. * pi_ * m_e * c_light) / (3. * q_e * B));
  s.dr = q.dr;
  // the shift of the blastwave's synchrotron kernel against the tensor-core
  // bank: ln x = k dnu - s - 2 j dlng, s = ln nu_crit1(B) - ln nu_0 - ln xs
  bool bank_oor = false;
  if (g.synbank && B > 0) {
    const double lxs = P.syn_method == PBAG_SYN_GSL ? g.sb_lnxs_gsl : 0.;
    s.syn_shift = (log((3. * q_e * B) / (4. * M_PI * m_e * c_light)) - g.sb_lnnu0 - lxs) * g.sb_ih;
    const double n = floor(s.syn_shift);
    bank_oor = !(n - 1. >= (double)g.sb_nlo && n + 2. <= (double)g.sb_nhi);
  }
  if (init) {
    s.vol = q.m_p1 / q.rho_p1;
    s.fac = s.dr / c_light / s.vol;
    if (bank_oor) {  // field outside the bank: the caller reruns the batch on CUDA cores
      s.err = PBAG_ERR_UNSUPPORTED;
      s.site = kSiteSynBank;
    } else if (pl_bad) {
      s.err = PBAG_ERR_NONFINITE;
      s.site = __LINE__;
    } else if (B < 0) {  // evalSynKernel (kernels.h:529-532)
      s.err = PBAG_ERR_PARAM;
      s.site = __LINE__;
    }
    out[r] = s;
    return;
  }
  // evaluateElectronDistributionNumericMixed (microphysics.h:372-435)
  if ((B <= 0) || (gm < 1.) || (gM <= 1.) || (gm >= gM) || (q.accel_frac > 1.)) {
    s.err = PBAG_ERR_PARAM;
    s.site = __LINE__;
    out[r] = s;
    return;
  }
  if (pl_bad) {
    s.err = PBAG_ERR_NONFINITE;
    s.site = __LINE__;
    out[r] = s;
    return;
  }
  if (bank_oor) {
    s.err = PBAG_ERR_UNSUPPORTED;
    s.site = kSiteSynBank;
    out[r] = s;
    return;
  }
  const double dt = q.tc_p1 - q.tc;
  const double volume = q.m / q.rho;
  const double volume_p1 = q.m_p1 / q.rho_p1;
  const double dlnVdt = P.adi_on ? 1. / dt * (1. - volume / volume_p1) : 0.;
  if ((!isfinite(dlnVdt)) || (dlnVdt < 0)) {
    s.err = PBAG_ERR_DLNVDT;
    s.site = __LINE__;
    out[r] = s;
    return;
  }
  s.dlnVdt = dlnVdt;
  const double dts = sigma_T * gM * B * B / (6. * M_PI * m_e * c_light);
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
  s.vol = volume;
  s.fac = s.dr / c_light / s.vol;
  if (P.ele_method == PBAG_ELE_MIX || gm <= 2) {
    s.n_sub = 0;  // analytic distribution replaces the evolution (microphysics.h:446-448)
  } else {
    s.n_sub = n_sub;
    s.dt_sub = delta_t;
    const double Nsrc = (q.m_p1 - q.m) / m_p / dt;
    const double index = -p;
    const double norm = (1 + index) / (pow(gM, index + 1) - pow(gm, index + 1));
    s.Ns = Nsrc * norm;
    s.iq0 = upper_bound_e(g.e, G, gm);  // gm < gamma <= gM (numeric_model.h:720)
    s.iq1 = upper_bound_e(g.e, G, gM);
    if (s.iq1 < s.iq0) s.iq1 = s.iq0;
  }
  out[r] = s;
}

template <int FQ>
__device__ int finalize_bw(const DevGrid& g, const GridTab& T, const DevState& S, int64_t r0,
                           const pbag_shock_params& P, int b, int step, const pbag_outputs& out, int flags, int err,
                           float* sh_v, double* sh_usv, int* sh_state, float* sh_pp);

// ---------------------------------------------------------------------------
// Chang-Cooper substeps (numeric_model.h:19-43, 682-708) of one blastwave-step.
// With dispersion 0 the system is upper bidiagonal and each substep is
//   f_j <- a_j + beta_j f_{j+1},  a_j = f_j / b_j + Q_j dt / b_j,  beta_j = -c_j / b_j,
// with a, b, c the same in every substep of a step. Thread t owns bins
// t*C .. t*C+C-1 in registers (fr, ib = 1/b, qb = Q dt / b, bt = beta).
// Both solvers below return whether a value checked before a substep was
// negative or not finite (solve() checks f first, numeric_model.h:688).

// Parallel suffix scan over the threads: the composition of the affine maps
// x -> A_t + P_t x of all threads to the right gives every thread the value of
// its right neighbour's first bin; the products P (the betas) are the same in
// every substep and are formed once. Cost per substep: C + 5 + (warps) + C
// dependent FMAs, so it wins for few substeps.
template <int C>
__device__ bool cc_scan(double (&fr)[C], const double (&ib)[C], const double (&qb)[C], const double (&bt)[C],
                        int n_sub, double (*xs)[kStepWarps], double* pw0) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double P = 1.;
#pragma unroll
  for (int q = 0; q < C; ++q) P *= bt[q];
  double pk[5];
  double Pc = P;
#pragma unroll
  for (int lev = 0; lev < 5; ++lev) {
    const int d = 1 << lev;
    const double Po = __shfl_down_sync(0xffffffffu, Pc, d);
    pk[lev] = Pc;
    if (lane + d < 32) Pc *= Po;
  }
  // Pc: product of the betas from this thread to the end of its warp
  double Pwn = __shfl_down_sync(0xffffffffu, Pc, 1);
  if (lane == 31) Pwn = 1.;
  if (lane == 0) pw0[warp] = Pc;
  __syncthreads();
  double pwr[kStepWarps];
#pragma unroll
  for (int v = 0; v < kStepWarps; ++v) pwr[v] = pw0[v];
  bool bad = false;
  for (int m = 0; m < n_sub; ++m) {
    double a[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      bad |= bad_value(fr[q]);
      a[q] = fma(fr[q], ib[q], qb[q]);
    }
    double A = a[C - 1];
#pragma unroll
    for (int q = C - 2; q >= 0; --q) A = fma(bt[q], A, a[q]);
    double Sx = A;
#pragma unroll
    for (int lev = 0; lev < 5; ++lev) {
      const int d = 1 << lev;
      const double So = __shfl_down_sync(0xffffffffu, Sx, d);
      if (lane + d < 32) Sx = fma(pk[lev], So, Sx);
    }
    double Sn = __shfl_down_sync(0xffffffffu, Sx, 1);
    if (lane == 31) Sn = 0.;
    if (lane == 0) xs[m & 1][warp] = Sx;
    __syncthreads();
    // value of the first bin of the next warp
    double carry = 0.;
#pragma unroll
    for (int v = kStepWarps - 1; v > 0; --v)
      if (v > warp) carry = fma(pwr[v], carry, xs[m & 1][v]);
    double fn = fma(Pwn, carry, Sn);  // first bin of the right neighbour
#pragma unroll
    for (int q = C - 1; q >= 0; --q) {
      fr[q] = fma(bt[q], fn, a[q]);
      fn = fr[q];
    }
  }
  return bad;
}

// ---- double-float: an FP32 pair (hi + lo, ~48-bit significand) ------------
// On this part an FP64 warp instruction occupies its sub-partition's FP64 unit
// for 64 cycles, so the substep recurrence runs in pairs of FP32 values instead
// (Dekker's products with FMA, Knuth's two-sum; every operand of the
// recurrence is non-negative, so no cancellation), scaled per blastwave by a
// power of two into the FP32 range.
struct dfl {
  float hi, lo;
};

// x 2^s as a pair, from the bits of x (no FP64 arithmetic): hi = the leading
// 24 bits, lo = the remaining 29 rounded to 24; 0 below the FP32 normal range,
// inf above it
__device__ __forceinline__ dfl dfl_from(double x, int s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long m = b & 0xfffffffffffffull;
  if (ex == 0) return {__uint_as_float(sign), 0.f};
  if (ex == 0x7ff) return {__uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u)), 0.f};
  const int e = ex - 1023 + s;  // exponent of the scaled value
  if (e + 127 >= 255) return {__uint_as_float(sign | 0x7f800000u), 0.f};
  if (e + 127 <= 0) return {__uint_as_float(sign), 0.f};
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29));
  const unsigned r = (unsigned)(m & 0x1fffffffull);
  float lo = r ? f32_ldexp((float)r, e - 52) : 0.f;
  if (sign) lo = -lo;
  const float h2 = hi + lo;  // normalise: |lo| <= ulp(hi) / 2
  return {h2, lo - (h2 - hi)};
}
// (hi + lo) 2^-s in FP64: the two parts built from their bits, one FP64 add
__device__ __forceinline__ double dfl_to(dfl a, int s) { return f64_from_mant(a.hi, -s) + f64_from_mant(a.lo, -s); }
__device__ __forceinline__ dfl dfl_mul(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  const float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
  const float hi = p + e;
  return {hi, e - (hi - p)};
}
// a b + c
__device__ __forceinline__ dfl dfl_fma(dfl a, dfl b, dfl c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
  const float s = p + c.hi;
  const float v = s - p;
  e += ((p - (s - v)) + (c.hi - v)) + c.lo;
  const float hi = s + e;
  return {hi, e - (hi - s)};
}
__device__ __forceinline__ bool dfl_bad(dfl a) {  // negative, inf or NaN (as bad_value)
  const unsigned u = __float_as_uint(a.hi);
  return (u & 0x7f800000u) == 0x7f800000u || (u > 0x80000000u);
}
__device__ __forceinline__ dfl dfl_shfl_down(dfl a, int d) {
  return {__shfl_down_sync(0xffffffffu, a.hi, d), __shfl_down_sync(0xffffffffu, a.lo, d)};
}

// cc_scan in double-float: the same recurrence, scan tree and order of
// operations, with the state and source scaled by 2^s (s from the block's
// largest exponent of f and Q dt / b, so that the values stay far inside the
// FP32 range for the substeps of this path). Returns false
// (and leaves fr untouched) when a coefficient or product leaves the FP32
// range: the caller then runs the FP64 scan. *bad as cc_scan's result.
template <int C>
__device__ bool cc_scan_df(double (&fr)[C], const double (&ib)[C], const double (&qb)[C], const double (&bt)[C],
                           int n_sub, double (*xs)[kStepWarps], double* pw0, int* red, bool* bad_out) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  bool bad = false;
  int E = 0;
#pragma unroll
  for (int q = 0; q < C; ++q) {
    bad |= bad_value(fr[q]);  // the check before the first substep, on the FP64 values
    E = max(E, max(exp_field(fr[q]), exp_field(qb[q])));
  }
  E = block_max_int(E, red);
  const int s = 1023 - E - 8;  // largest scaled input ~2^-8
  dfl f[C], ibd[C], qbd[C], btd[C];
  bool ok = true;
#pragma unroll
  for (int q = 0; q < C; ++q) {
    f[q] = dfl_from(fr[q], s);
    ibd[q] = dfl_from(ib[q], 0);
    qbd[q] = dfl_from(qb[q], s);
    btd[q] = dfl_from(bt[q], 0);
  }
  dfl P = {1.f, 0.f};
#pragma unroll
  for (int q = 0; q < C; ++q) P = dfl_mul(P, btd[q]);
  dfl pk[5];
  dfl Pc = P;
#pragma unroll
  for (int lev = 0; lev < 5; ++lev) {
    const int d = 1 << lev;
    const dfl Po = dfl_shfl_down(Pc, d);
    pk[lev] = Pc;
    if (lane + d < 32) Pc = dfl_mul(Pc, Po);
  }
  dfl Pwn = dfl_shfl_down(Pc, 1);
  if (lane == 31) Pwn = {1.f, 0.f};
  // every coefficient and product in range (finite; a product may underflow to 0)
#pragma unroll
  for (int q = 0; q < C; ++q)
    ok &= isfinite(ibd[q].hi) && isfinite(qbd[q].hi) && isfinite(btd[q].hi) && isfinite(f[q].hi) && !bad_value(fr[q]);
#pragma unroll
  for (int lev = 0; lev < 5; ++lev) ok &= isfinite(pk[lev].hi);
  ok &= isfinite(Pc.hi) && isfinite(Pwn.hi);
  dfl* pw = reinterpret_cast<dfl*>(pw0);
  if (lane == 0) pw[warp] = Pc;
  if (!__syncthreads_and(ok ? 1 : 0)) return false;
  dfl pwr[kStepWarps];
#pragma unroll
  for (int v = 0; v < kStepWarps; ++v) pwr[v] = pw[v];
  bool okc = true;
#pragma unroll
  for (int v = 0; v < kStepWarps; ++v) okc &= isfinite(pwr[v].hi);
  // a barrier also before a fallback: the FP64 scan rewrites pw0
  if (!__syncthreads_and(okc ? 1 : 0)) return false;
  dfl (*xd)[kStepWarps] = reinterpret_cast<dfl(*)[kStepWarps]>(xs);
  for (int m = 0; m < n_sub; ++m) {
    dfl a[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      if (m > 0) bad |= dfl_bad(f[q]);
      a[q] = dfl_fma(f[q], ibd[q], qbd[q]);
    }
    dfl A = a[C - 1];
#pragma unroll
    for (int q = C - 2; q >= 0; --q) A = dfl_fma(btd[q], A, a[q]);
    dfl Sx = A;
#pragma unroll
    for (int lev = 0; lev < 5; ++lev) {
      const int d = 1 << lev;
      const dfl So = dfl_shfl_down(Sx, d);
      if (lane + d < 32) Sx = dfl_fma(pk[lev], So, Sx);
    }
    dfl Sn = dfl_shfl_down(Sx, 1);
    if (lane == 31) Sn = {0.f, 0.f};
    if (lane == 0) xd[m & 1][warp] = Sx;
    __syncthreads();
    dfl carry = {0.f, 0.f};
#pragma unroll
    for (int v = kStepWarps - 1; v > 0; --v)
      if (v > warp) carry = dfl_fma(pwr[v], carry, xd[m & 1][v]);
    dfl fn = dfl_fma(Pwn, carry, Sn);
#pragma unroll
    for (int q = C - 1; q >= 0; --q) {
      f[q] = dfl_fma(btd[q], fn, a[q]);
      fn = f[q];
    }
  }
#pragma unroll
  for (int q = 0; q < C; ++q) fr[q] = dfl_to(f[q], s);
  *bad_out = bad;
  return true;
}

// Systolic pipeline: thread t runs substep m at tick m + (T-1-t), taking the
// right neighbour's new first bin of the same substep from the tick before.
// n_sub + T - 1 ticks of C dependent FMAs: it wins for many substeps.
template <int C>
__device__ bool cc_systolic(double (&fr)[C], const double (&ib)[C], const double (&qb)[C], const double (&bt)[C],
                            int n_sub, int T, double (*xs)[kStepWarps]) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < 2 * kStepWarps) (&xs[0][0])[tid] = 0.;
  __syncthreads();
  double low = 0.;
  bool bad = false;
  const int ticks = n_sub + T - 1;
  for (int tau = 0; tau < ticks; ++tau) {
    double up = __shfl_down_sync(0xffffffffu, low, 1);
    if (lane == 31) up = warp + 1 < kStepWarps ? xs[tau & 1][warp + 1] : 0.;
    const int m = tau - (T - 1 - tid);
    if (tid < T && m >= 0 && m < n_sub) {
      double fn = up;
#pragma unroll
      for (int q = C - 1; q >= 0; --q) {
        bad |= bad_value(fr[q]);
        const double a = fma(fr[q], ib[q], qb[q]);
        fr[q] = fma(bt[q], fn, a);
        fn = fr[q];
      }
      low = fr[0];
    }
    if (lane == 0) xs[(tau + 1) & 1][warp] = low;
    __syncthreads();
  }
  return bad;
}

// cc_systolic in double-float, with cc_scan_df's power-of-two scaling and
// range checks. Each tick is C dependent pair FMAs on the FP32 pipe instead of
// FP64 ones (which hold a sub-partition's FP64 unit for 64 cycles each, and are
// shared by every CTA on the SM), so the pipeline stays latency-bound when
// several blastwaves run their long substep loops side by side. Returns false
// (fr untouched) when a coefficient or the state leaves the FP32 range; the
// caller then runs cc_systolic. *bad as cc_systolic's result.
template <int C>
__device__ bool cc_systolic_df(double (&fr)[C], const double (&ib)[C], const double (&qb)[C], const double (&bt)[C],
                               int n_sub, int T, double (*xs)[kStepWarps], int* red, bool* bad_out) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  bool bad = false;
  int E = 0;
#pragma unroll
  for (int q = 0; q < C; ++q) {
    bad |= bad_value(fr[q]);  // the check before the first substep, on the FP64 values
    E = max(E, max(exp_field(fr[q]), exp_field(qb[q])));
  }
  E = block_max_int(E, red);
  const int s = 1023 - E - 8;  // largest scaled input ~2^-8
  dfl f[C], ibd[C], qbd[C], btd[C];
  bool ok = true;
#pragma unroll
  for (int q = 0; q < C; ++q) {
    f[q] = dfl_from(fr[q], s);
    ibd[q] = dfl_from(ib[q], 0);
    qbd[q] = dfl_from(qb[q], s);
    btd[q] = dfl_from(bt[q], 0);
    ok &= isfinite(ibd[q].hi) && isfinite(qbd[q].hi) && isfinite(btd[q].hi) && isfinite(f[q].hi) && !bad_value(fr[q]);
  }
  if (!__syncthreads_and(ok ? 1 : 0)) return false;
  dfl(*xd)[kStepWarps] = reinterpret_cast<dfl(*)[kStepWarps]>(xs);
  if (tid < 2 * kStepWarps) (&xd[0][0])[tid] = dfl{0.f, 0.f};
  __syncthreads();
  dfl low = {0.f, 0.f};
  const int ticks = n_sub + T - 1;
  for (int tau = 0; tau < ticks; ++tau) {
    dfl up = dfl_shfl_down(low, 1);
    if (lane == 31) up = warp + 1 < kStepWarps ? xd[tau & 1][warp + 1] : dfl{0.f, 0.f};
    const int m = tau - (T - 1 - tid);
    if (tid < T && m >= 0 && m < n_sub) {
      dfl fn = up;
#pragma unroll
      for (int q = C - 1; q >= 0; --q) {
        if (m > 0) bad |= dfl_bad(f[q]);
        const dfl a = dfl_fma(f[q], ibd[q], qbd[q]);
        f[q] = dfl_fma(btd[q], fn, a);
        fn = f[q];
      }
      low = f[0];
    }
    if (lane == 0) xd[(tau + 1) & 1][warp] = low;
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < C; ++q) fr[q] = dfl_to(f[q], s);
  *bad_out = bad;
  return true;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// bounded wait on phase `parity` of an mbarrier
__device__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (it > 16) __nanosleep(32);
  }
  return false;
}

// bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) into
// shared memory, completing on `bar`, in pieces of at most 32 KiB
__device__ void bulk_to_smem(void* dst, const void* src, int bytes, uint32_t bar) {
  for (int o = 0; o < bytes; o += 32768) {
    const uint32_t n = (uint32_t)min(32768, bytes - o);
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(static_cast<unsigned char*>(dst) + o)),
        "l"(static_cast<const unsigned char*>(src) + o), "r"(n), "r"(bar)
        : "memory");
  }
}

// Dynamic shared memory of k_evolve: [staged KintT (kstage bytes)][tables
// (etab)][N(gamma) | f/gamma^2 | SSA weights (G doubles each)][seed-photon
// weights (F floats)].
__host__ __device__ inline size_t evolve_kint_bytes(int kstage) { return ((size_t)kstage + 127) / 128 * 128; }
__host__ __device__ inline size_t evolve_bytes(const DevGrid& g, int kstage) {
  return evolve_kint_bytes(kstage) + (size_t)g.etab_doubles * sizeof(double) + 3 * (size_t)g.G * sizeof(double) +
         (size_t)g.F * sizeof(float);
}

// Largest dynamic shared memory of k_evolve. The kernel-integral table is
// staged only for batches small enough to run with few CTAs per SM (larger
// batches keep more CTAs per SM instead) and only when it fits.
constexpr size_t kEvolveSmemMax = 220 * 1024;
constexpr int kStageMaxBw = 304;
inline int evolve_kint_stage(const DevGrid& g, int nbw) {
  if (g.kint_stage <= 0 || nbw > kStageMaxBw) return 0;
  return evolve_bytes(g, g.kint_stage) <= kEvolveSmemMax ? g.kint_stage : 0;
}

// ---------------------------------------------------------------------------
// One step of every blastwave, one CTA each, C gamma bins per thread in the solve,
// FQ frequencies per thread in the completion of the previous step.
// Every global load that does not depend on another is issued at the start
// (grid tables by one bulk copy into shared memory, the blastwave's state into
// registers), so that the step pays few dependent memory round trips.
template <int C, int FQ, int MINB>
__global__ void __launch_bounds__(kStepThreads, MINB)
k_evolve(DevGrid g, DevState S, const pbag_step_rec* __restrict__ recs, const StepScal* __restrict__ ss,
         const int64_t* __restrict__ off, const pbag_shock_params* __restrict__ prm, int step, pbag_outputs out,
         int kstage) {
  const int b = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = g.G, F = g.F;
  extern __shared__ __align__(128) unsigned char evo_smem[];
  float* sh_k = reinterpret_cast<float*>(evo_smem);  // staged KintT
  double* sh_tab = reinterpret_cast<double*>(evo_smem + evolve_kint_bytes(kstage));
  double* sh_f = sh_tab + g.etab_doubles;  // heating term, then N(gamma)
  double* sh_t = sh_f + G;                 // f / gamma^2; photon field of the previous step
  double* sh_vd = sh_t + G;                // SSA weights
  float* sh_v = reinterpret_cast<float*>(sh_vd + G);  // seed-photon weights of the SSC cooling GEMV
  __shared__ double red_d[kStepWarps];
  __shared__ int red_i[3][kStepWarps];
  __shared__ double xs[2][kStepWarps];
  __shared__ double pw0[kStepWarps];
  __shared__ __align__(8) uint64_t bars[2];  // tables, kernel integral
  __shared__ int sh_state[2];                // flags and error code after the previous step's completion
  __shared__ double sh_usv;                  // inverse scale of sh_v
  __shared__ float sh_pp[PBAG_MAX_BINS];     // scaled photon density of the pair-production sums
  const GridTab T{sh_tab, g.Ge, g.Fe};

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const int tb = g.etab_doubles * (int)sizeof(double);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&bars[0])), "r"(tb)
                 : "memory");
    bulk_to_smem(sh_tab, g.etab, tb, smem_addr(&bars[0]));
  }
  // independent loads of this blastwave: first what no kernel of the pass
  // writes (the slot map, records, step scalars, parameters, e^-p tables)
  const int bw = slot_bw(S, b);  // the caller's blastwave in this slot
  const int64_t r0 = off[bw], len = off[bw + 1] - r0;
  const pbag_shock_params P = prm[bw];
  double* f = S.f + (size_t)b * G;
  const double* pp = S.powp + (size_t)bw * G;
  double* dfde = S.dfde + (size_t)b * G;
  double fr[C], ppq[C], dpre[C];
#pragma unroll
  for (int q = 0; q < C; ++q) {
    const int j = tid * C + q;  // solve: contiguous bins per thread
    ppq[q] = j < G ? pp[j] : 0.;
  }
  const bool in_range = step < len;
  StepScal sc{};
  double accel = 0., B = 0., gamma_c = 0., n_prime = 0.;
  if (in_range) {
    sc = ss[r0 + step];
    const pbag_step_rec& r = recs[r0 + step];
    accel = r.accel_frac;
    B = r.B;
    gamma_c = r.gamma_c;
    n_prime = r.n_prime;
  }
  const bool ssc = P.ssc_on && g.KintT != nullptr;
  // the kernel-integral table streams into shared memory while the previous
  // step completes, when this step runs the Chang-Cooper substeps with SSC
  // (a blastwave stopped by an error returns before it reads the table)
  const bool staged = kstage > 0 && ssc && in_range && (sc.flags & kRecValid) && !sc.err &&
                      !(sc.flags & kRecInit) && sc.n_sub > 0;
  if (staged && tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&bars[1])), "r"(kstage)
                 : "memory");
    bulk_to_smem(sh_k, g.KintT, kstage, smem_addr(&bars[1]));
  }
  // then the state the previous step's kernels wrote, once they completed
  // (no early release of this step's radiation kernels: resident next to
  // these CTAs they slowed the pass)
  grid_dep_wait();
  const int flags0 = S.flags[b];
  const int err0 = S.err[4 * b];
#pragma unroll
  for (int q = 0; q < C; ++q) {
    const int j = tid * C + q;
    fr[q] = j < G ? f[j] : 0.;
    const int i = tid + q * kStepThreads;  // everything else: strided bins
    dpre[q] = (P.ssa_on && i < G) ? dfde[i] : 0.;
  }
  // gamma-grid history rows of the previous step, written once it completes
  const bool hist_g = step > 0 && (out.ele_f_all || out.gdot_syn_all || out.gdot_adi_all || out.gdot_ssc_all);
  double hf[C], hgs[C], hga[C], hgc[C];
#pragma unroll
  for (int q = 0; q < C; ++q) {
    const int i = tid + q * kStepThreads;
    const bool in = hist_g && i < G;
    const double* gd = S.gdot + (size_t)b * 3 * G;
    hf[q] = in ? f[i] : 0.;
    hgs[q] = in ? gd[i] : 0.;
    hga[q] = in ? gd[G + i] : 0.;
    hgc[q] = in ? gd[2 * G + i] : 0.;
  }
  __syncthreads();  // the barriers are initialised
  auto drain = [&]() {  // copies must land before the CTA exits
    if (tid == 0 && staged) mbar_wait_bounded(smem_addr(&bars[1]), 0);
  };
  if (__syncthreads_or(mbar_wait_bounded(smem_addr(&bars[0]), 0) ? 0 : 1)) {
    if (tid == 0) {
      set_error(S, b, PBAG_ERR_TIMEOUT, step, __LINE__);
      mbar_wait_bounded(smem_addr(&bars[0]), 0);
    }
    drain();
    return;
  }

  // the previous step's photon field, totals and history rows (same CTA shape);
  // its photon field and seed-photon weights stay in shared memory
  int flags = flags0, errc = err0;
  bool have_v = false;
  if (step > 0) {
    const int fin =
        finalize_bw<FQ>(g, T, S, r0, P, b, step - 1, out, flags0, err0, sh_v, &sh_usv, sh_state, sh_pp);
    if (fin) {
      __syncthreads();
      flags = sh_state[0];
      errc = sh_state[1];
      have_v = fin == 1 && errc == 0;
    }
    if (fin == 1 && hist_g) {
      const size_t row = (size_t)(r0 + step - 1);
#pragma unroll
      for (int q = 0; q < C; ++q) {
        const int i = tid + q * kStepThreads;
        if (i >= G) continue;
        if (out.ele_f_all) out.ele_f_all[row * G + i] = hf[q];
        if (out.gdot_syn_all) out.gdot_syn_all[row * G + i] = hgs[q];
        if (out.gdot_adi_all) out.gdot_adi_all[row * G + i] = hga[q];
        if (out.gdot_ssc_all) out.gdot_ssc_all[row * G + i] = hgc[q];
      }
    }
  }
  const bool active = errc == 0 && in_range && (sc.flags & kRecValid);
  if (tid == 0) S.flags[b] = flags & ~kFlagActive;
  if (!active) {
    drain();
    return;
  }

#define PBAG_FAIL(code, site)                            \
  do {                                                   \
    if (tid == 0) set_error(S, b, (code), step, (site)); \
    return;                                              \
  } while (0)

  if (sc.err) PBAG_FAIL(sc.err, sc.site);
  const double Kb = (sc.flags & kRecFast) ? sc.K : sc.K * gamma_c;

  if (sc.flags & kRecInit) {
    // ---- initializeElectronDistribution (microphysics.h:347-357): untouched
    // entries keep their value, then all but the last bin scale by accel_frac
    for (int i = tid; i < G; i += kStepThreads) {
      double v = f[i];
      if (i >= sc.ia0 && i < sc.ia1) v = pl_branch_a(T, sc, pp, i);
      else if (i >= sc.ib0 && i < sc.ib1) v = pl_branch_b(T, sc, pp, i, Kb);
      if (i < G - 1) v *= accel;
      f[i] = v;
      sh_f[i] = v;
    }
    flags |= kFlagInit;
  } else if (sc.n_sub == 0) {
    // ---- analytic distribution (microphysics.h:446-448)
    for (int i = tid; i < G; i += kStepThreads) {
      double v = 0.;
      if (i >= sc.ia0 && i < sc.ia1) v = pl_branch_a(T, sc, pp, i);
      else if (i >= sc.ib0 && i < sc.ib1) v = pl_branch_b(T, sc, pp, i, Kb);
      f[i] = v;
      sh_f[i] = v;
    }
  } else {
    // ---- Chang-Cooper evolution (microphysics.h:451-480)
    const double delta_t = sc.dt_sub;
    const int n_sub = sc.n_sub;
    double usv = 1.;
    if (ssc) {
      if (have_v) {
        usv = sh_usv;
      } else {  // the photon field of an earlier step, from global memory
        const double* n = S.n + (size_t)b * F;
        const double* dnu = T.ft(kTabDnuNu);
        const double* ksc = T.ft(kTabKscale);
        int vexp = 0;
        for (int k = tid; k < F - 1; k += kStepThreads) vexp = max(vexp, exp_field(n[k] * dnu[k] * ksc[k]));
        vexp = block_max_int(vexp, red_i[0]);
        const double sv = scale_from_exp(vexp);
        usv = unscale_from_exp(vexp);
        for (int k = tid; k < F; k += kStepThreads) sh_v[k] = k < F - 1 ? (float)(n[k] * dnu[k] * ksc[k] * sv) : 0.f;
        __syncthreads();
      }
    }
    const bool kint_smem = staged;
    if (kint_smem) {
      const int miss = __syncthreads_or(mbar_wait_bounded(smem_addr(&bars[1]), 0) ? 0 : 1);
      if (miss) {
        if (tid == 0) mbar_wait_bounded(smem_addr(&bars[1]), 0);
        PBAG_FAIL(PBAG_ERR_TIMEOUT, __LINE__);
      }
    }
    // heating / cooling terms at the half grid (numeric_model.h:753-801);
    // constant over the substeps, so evaluated once per step
    const double c_syn = sigma_T / (6. * M_PI * m_e * c_light) * B * B;
    const double c_ssc = 3. / 4. * h_pl * sigma_T / m_e / c_light * usv;
    double* gsyn = S.gdot + (size_t)b * 3 * G;
    double* gadi = gsyn + G;
    double* gssc = gadi + G;
    const int Gs = g.Gs;
    bool hbad = false;
    // SSC cooling GEMV of this thread's (at most two) bins together, two
    // partial sums per bin: four independent FMA chains instead of one
    float accA = 0.f, accB = 0.f;
    const bool gemv2 = ssc && G - 1 <= 2 * kStepThreads;
    if (gemv2 && tid < G - 1) {
      const int i0 = tid, i1 = tid + kStepThreads < G - 1 ? tid + kStepThreads : tid;
      const float* k0 = kint_smem ? sh_k + i0 : g.KintT + i0;
      const float* k1 = kint_smem ? sh_k + i1 : g.KintT + i1;
      float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
      int k = 0;
      if (kint_smem) {
#pragma unroll 4
        for (; k + 1 < F - 1; k += 2) {
          const float v0 = sh_v[k], v1 = sh_v[k + 1];
          a0 = fmaf(v0, k0[(size_t)k * Gs], a0);
          b0 = fmaf(v0, k1[(size_t)k * Gs], b0);
          a1 = fmaf(v1, k0[(size_t)(k + 1) * Gs], a1);
          b1 = fmaf(v1, k1[(size_t)(k + 1) * Gs], b1);
        }
        if (k < F - 1) {
          a0 = fmaf(sh_v[k], k0[(size_t)k * Gs], a0);
          b0 = fmaf(sh_v[k], k1[(size_t)k * Gs], b0);
        }
      } else {
#pragma unroll 8
        for (; k + 1 < F - 1; k += 2) {
          const float v0 = sh_v[k], v1 = sh_v[k + 1];
          a0 = fmaf(v0, __ldg(k0 + (size_t)k * Gs), a0);
          b0 = fmaf(v0, __ldg(k1 + (size_t)k * Gs), b0);
          a1 = fmaf(v1, __ldg(k0 + (size_t)(k + 1) * Gs), a1);
          b1 = fmaf(v1, __ldg(k1 + (size_t)(k + 1) * Gs), b1);
        }
        if (k < F - 1) {
          a0 = fmaf(sh_v[k], __ldg(k0 + (size_t)k * Gs), a0);
          b0 = fmaf(sh_v[k], __ldg(k1 + (size_t)k * Gs), b0);
        }
      }
      accA = a0 + a1;
      accB = b0 + b1;
    }
    for (int i = tid, m = 0; i < G - 1; i += kStepThreads, ++m) {
      const double vs = c_syn * T.gt(kTabHalf2)[i];
      const double va = sc.dlnVdt * T.gt(kTabHadi)[i];
      double vc = 0.;
      if (gemv2) {
        vc = c_ssc * (double)(m == 0 ? accA : accB) * T.gt(kTabIhalf2)[i];
        gssc[i] = vc;
      } else if (ssc) {
        float acc = 0.f;
        if (kint_smem) {
          const float* kc = sh_k + i;
#pragma unroll 8
          for (int k = 0; k < F - 1; k++) acc = fmaf(sh_v[k], kc[(size_t)k * Gs], acc);
        } else {
          const float* kc = g.KintT + i;
#pragma unroll 16
          for (int k = 0; k < F - 1; k++) acc = fmaf(sh_v[k], __ldg(kc + (size_t)k * Gs), acc);
        }
        vc = c_ssc * (double)acc * T.gt(kTabIhalf2)[i];
        gssc[i] = vc;
      } else {
        vc = gssc[i];  // stays as the last SSC step left it
      }
      gsyn[i] = vs;
      gadi[i] = va;
      const double H = vs + va + vc;
      if (not_finite(H)) hbad = true;
      sh_f[i] = H;
    }
    if (tid == 0) sh_f[G - 1] = 0.;  // heating_term[G-1] is never set (numeric_model.h:761)
    if (__syncthreads_or(hbad ? 1 : 0)) PBAG_FAIL(PBAG_ERR_NONFINITE, __LINE__);
    // pair production (addPPSource, numeric_model.h:727-733, with
    // computePPinjection :305-340): pairs from the photon density of the
    // previous radiating step join the source of every bin; the sums over the
    // photon grid in FP32 with the density scaled by a power of two
    double inj[C];
#pragma unroll
    for (int q = 0; q < C; ++q) inj[q] = 0.;
    if (ssc && P.pp_on) {
      const double* n = S.n + (size_t)b * F;
      int pexp = 0;
      for (int k = tid; k < F - 1; k += kStepThreads) pexp = max(pexp, exp_field(n[k]));
      pexp = block_max_int(pexp, red_i[0]);
      const double sp = scale_from_exp(pexp), usp = unscale_from_exp(pexp);
      for (int k = tid; k < F; k += kStepThreads) sh_pp[k] = k < F - 1 ? (float)(n[k] * sp) : 0.f;
      __syncthreads();
      const double ppfac = 4. * m_e * (c_light * c_light) / h_pl;
#pragma unroll
      for (int q = 0; q < C; ++q) {
        const int j = tid * C + q;
        if (j >= G) continue;
        float acc = 0.f;
        for (int k = 0; k < F - 1; ++k) acc = fmaf(sh_pp[k], __ldg(g.ppinjT + (size_t)k * Gs + j), acc);
        inj[q] = ppfac * n[g.ppidx[j]] * ((double)acc * usp) * sc.vol;
      }
    }
    // tridiagonal coefficients (numeric_model.h:539-675 with dispersion = 0,
    // delta_j = 0): a = 0, b_k = 1 + dt H_{k-1}/dgb_k (b_0 = b_{G-1} = 1),
    // c_k = -dt H_k/dgb_k (c_{G-1} = 0)
    double ib[C], qb[C], bt[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int j = tid * C + q;
      ib[q] = qb[q] = bt[q] = 0.;
      if (j < G) {
        const double odg = T.gt(kTabInvDgb)[j];
        const double Hb = (j > 0 && j < G - 1) ? sh_f[j - 1] : 0.;  // b_0 and b_{G-1} see no inflow
        const double Hf = j < G - 1 ? sh_f[j] : 0.;
        const double bb = 1. + (odg * Hb) * delta_t;
        const double cc = (odg * Hf) * -delta_t;
        const double Q = ((j >= sc.iq0 && j < sc.iq1) ? sc.Ns * ppq[q] : 0.) + inj[q];
        ib[q] = 1. / bb;
        bt[q] = -(cc * ib[q]);
        qb[q] = (Q * delta_t) * ib[q];
      }
    }
    const int Tn = (G + C - 1) / C;  // threads that own bins
    bool sbad = false;
    if (n_sub >= g.sys_min_sub) {
      if (g.scan_fp64 || !cc_systolic_df<C>(fr, ib, qb, bt, n_sub, Tn, xs, red_i[0], &sbad))
        sbad = cc_systolic<C>(fr, ib, qb, bt, n_sub, Tn, xs);
    } else if (g.scan_fp64 || !cc_scan_df<C>(fr, ib, qb, bt, n_sub, xs, pw0, red_i[0], &sbad))
      sbad = cc_scan<C>(fr, ib, qb, bt, n_sub, xs, pw0);
    __syncthreads();  // every heating value has been read: sh_f takes N(gamma)
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int j = tid * C + q;
      if (j < G) {
        f[j] = fr[q];
        sh_f[j] = fr[q];
      }
    }
    if (__syncthreads_or(sbad ? 1 : 0)) PBAG_FAIL(PBAG_ERR_NONFINITE, __LINE__);
  }
  __syncthreads();

  // ---- per-step weights of the radiation sums (microphysics.h:498-558):
  // N_e and the power-of-two scales in one block reduction
  const double* t_inv_e2 = T.gt(kTabInvE2);
  const double* t_de = T.gt(kTabDe);
  double ne = 0.;
  int wexp = 0, Wexp = 0;
  double wk[C], Wk[C];  // f_j dgamma_j and f_j dgamma_j / e_j^2 of this thread's bins (tid + 128 k)
#pragma unroll
  for (int k = 0; k < C; ++k) {
    const int i = tid + k * kStepThreads;
    wk[k] = Wk[k] = 0.;
    if (i < G) {
      const double fi = sh_f[i];
      sh_t[i] = fi * t_inv_e2[i];  // f / e / e (numeric_model.h:194-195)
      if (i < G - 1) {
        const double w = fi * t_de[i];
        wk[k] = w;
        Wk[k] = w * t_inv_e2[i];
        ne += w;  // N_e (microphysics.h:556-558)
        wexp = max(wexp, exp_field(w));
        Wexp = max(Wexp, exp_field(Wk[k]));
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ne += __shfl_down_sync(0xffffffffu, ne, o);
  wexp = __reduce_max_sync(0xffffffffu, wexp);
  Wexp = __reduce_max_sync(0xffffffffu, Wexp);
  if (lane == 0) {
    red_d[warp] = ne;
    red_i[1][warp] = wexp;
    red_i[2][warp] = Wexp;
  }
  __syncthreads();  // publishes sh_t and the partial results
  ne = 0.;
  wexp = Wexp = 0;
#pragma unroll
  for (int v = 0; v < kStepWarps; ++v) {
    ne += red_d[v];
    wexp = max(wexp, red_i[1][v]);
    Wexp = max(Wexp, red_i[2][v]);
  }
  float* w32 = S.w32 + (size_t)b * G;
  // weight rows of the tensor-core synchrotron sums: row 2 (b mod tbw) of
  // tile b / tbw, BF16 hi + lo (pbag_syn_tc.cu)
  uint16_t* Sb = S.Sbf ? S.Sbf + (size_t)(b / g.sb_tbw) * tc_tile_elems(2 * g.sb_tbw, g.Gp) : nullptr;
  const int srow = 2 * (b % max(g.sb_tbw, 1));
#pragma unroll
  for (int k = 0; k < C; ++k) {
    const int i = tid + k * kStepThreads;
    if (i < G) {
      const float w = f32_scaled(wk[k], wexp);  // wk = 0 for the last bin
      w32[i] = w;
      if (Sb) {
        const __nv_bfloat16 hi = __float2bfloat16_rn(w);
        Sb[tc_operand_offset(srow, i, 2 * g.sb_tbw, g.Gp, false)] = __bfloat16_as_ushort(hi);
        Sb[tc_operand_offset(srow, i, 2 * g.sb_tbw, g.Gp, true)] =
            __bfloat16_as_ushort(__float2bfloat16_rn(w - __bfloat162float(hi)));
      }
    }
  }
  // SSC electron weights W_j = f_j (e_{j+1}-e_j) 3/4 sigma_T c / e_j^2 (numeric_model.h:271-277)
  // (FP32 for the CUDA-core contraction, BF16 hi + lo tiles for the tensor cores)
  if (P.ssc_on && g.K32 != nullptr) {
    float* W = S.W32 + (size_t)b * g.Gp;
    uint16_t* A = S.Abf ? S.Abf + (size_t)(b / kTcCols) * tc_tile_elems(kTcCols, g.Gp) : nullptr;
    const int m = b % kTcCols;
    // Gp <= 128 C (G <= 128 C, Gp its multiple of 16): bin j = tid + 128 k
#pragma unroll
    for (int k = 0; k < C; ++k) {
      const int j = tid + k * kStepThreads;
      if (j >= g.Gp) continue;
      const float w = f32_scaled(Wk[k], Wexp);  // Wk = 0 from the last bin on
      W[j] = w;
      if (A) {
        const __nv_bfloat16 hi = __float2bfloat16_rn(w);
        const __nv_bfloat16 lo = __float2bfloat16_rn(w - __bfloat162float(hi));
        A[tc_operand_offset(m, j, kTcCols, g.Gp, false)] = __bfloat16_as_ushort(hi);
        A[tc_operand_offset(m, j, kTcCols, g.Gp, true)] = __bfloat16_as_ushort(lo);
      }
    }
  }
  // SSA weights: dfde = d(f/gamma^2)/dgamma, stateful (base_state.h:482-501)
  int vexp = 0;
  if (P.ssa_on) {
    const double* t_dxm = T.gt(kTabInvDxm);
    const double* t_e2de = T.gt(kTabE2de);
#pragma unroll
    for (int k = 0; k < C; ++k) {
      const int i = tid + k * kStepThreads;
      if (i < G) {
        const double t = sh_t[i];
        double d = dpre[k];
        if (positive(t)) {
          if (i == 0)
            d = -1.5 * t + 2. * sh_t[1] - 0.5 * sh_t[2];
          else if (i == G - 1)
            d = 1.5 * t - 2. * sh_t[G - 2] + 0.5 * sh_t[G - 3];
          else
            d = 0.5 * (sh_t[i + 1] - sh_t[i - 1]) * t_dxm[i];
          dfde[i] = d;
        }
        if (i < G - 1) {
          const double v = t_e2de[i] * d;  // e_j^2 (e_{j+1}-e_j) dfde_j (numeric_model.h:208)
          sh_vd[i] = v;
          vexp = max(vexp, exp_field(v));
        }
      }
    }
    vexp = __reduce_max_sync(0xffffffffu, vexp);
    if (lane == 0) red_i[0][warp] = vexp;
  }
  __syncthreads();  // publishes sh_vd and the SSA scale
  if (P.ssa_on) {
    vexp = 0;
#pragma unroll
    for (int v = 0; v < kStepWarps; ++v) vexp = max(vexp, red_i[0][v]);
    float* v32 = S.v32 + (size_t)b * G;
    for (int i = tid; i < G; i += kStepThreads) {
      const float v = i < G - 1 ? f32_scaled(sh_vd[i], vexp) : 0.f;
      v32[i] = v;
      if (Sb) {
        const __nv_bfloat16 hi = __float2bfloat16_rn(v);
        Sb[tc_operand_offset(srow + 1, i, 2 * g.sb_tbw, g.Gp, false)] = __bfloat16_as_ushort(hi);
        Sb[tc_operand_offset(srow + 1, i, 2 * g.sb_tbw, g.Gp, true)] =
            __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(hi)));
      }
    }
  }
  if (!positive(ne) && !is_nan(ne)) PBAG_FAIL(PBAG_ERR_NELE, __LINE__);  // n_ele <= 0 (microphysics.h:560-563)
  if (tid == 0) {
    double* scal = S.scal + (size_t)b * kScal;
    if (P.ssc_on && g.K32 != nullptr) scal[kScalSW] = 3. / 4. * sigma_T * c_light * unscale_from_exp(Wexp);
    scal[kScalDr] = sc.dr;
    scal[kScalVol] = sc.vol;
    scal[kScalNele] = ne;
    scal[kScalFac] = sc.fac;
    scal[kScalAcc] = accel;
    scal[kScalNp] = n_prime;
    scal[kScalNsub] = (double)sc.n_sub;
    scal[kScalSw] = unscale_from_exp(wexp);
    scal[kScalSv] = unscale_from_exp(vexp);
    scal[kScalPref] = sc.pref;
    scal[kScalB] = B;
    scal[kScalSynShift] = sc.syn_shift;
    float* rp = S.rad32 + (size_t)b * 4;
    rp[0] = sc.inv_ncrit;
    rp[1] = sc.inv_nlar;
    rp[2] = cbrtf(sc.inv_ncrit);
    rp[3] = 0.f;
    S.flags[b] = flags | kFlagActive;
  } else if (tid == 32) {  // the two divisions on other sub-partitions' FP64 units, next to thread 0's work
    S.scal[(size_t)b * kScal + kScalAccNe] = accel / ne;
  } else if (tid == 64) {
    S.scal[(size_t)b * kScal + kScalAnpNe] = accel * n_prime / ne;
  }
#undef PBAG_FAIL
}

// ---------------------------------------------------------------------------
// Synchrotron and SSA sums of one blastwave: each warp of the CTA takes R
// frequencies (k = base + r kRadFreqs + warp), its lanes split the gamma sum;
// the blastwave's setup is paid once for the R frequencies, and the gamma-bin
// tables and weights of the later frequencies come from L1. The synchrotron
// kernel values are generated in FP32 on the fly and never stored. The kernel
// has no FP64 instruction (each costs a warp 64 cycles of its SM
// sub-partition's FP64 unit on this part): the FP64 prefactors are applied by
// finalize_bw.
__device__ void radiate_block(const DevGrid& g, const DevState& S, const pbag_shock_params* prm, int b, int kblk,
                              int R) {
  const int tid = threadIdx.x;
  const int G = g.G, F = g.F;
  if (!(S.flags[b] & kFlagActive)) return;
  const pbag_shock_params* pb = prm + slot_bw(S, b);
  const bool ssa = pb->ssa_on != 0;
  const int method = pb->syn_method;
  // GSL and Bessel: the tabulated functions, no cyclotron branch
  const bool tab = method == PBAG_SYN_GSL || method == PBAG_SYN_BESSEL;
  const float* stab = g.syntab + (method == PBAG_SYN_BESSEL ? kSynTabN : 0);
  const float xs = method == PBAG_SYN_GSL ? g.gsl_xs : 1.f;
  const float4 rp = *reinterpret_cast<const float4*>(S.rad32 + (size_t)b * 4);
  const float incrit = rp.x, inlar = rp.y;
  const int kq = tid / kRadLanes, jl = tid % kRadLanes;
  const int jcyc = method == PBAG_SYN_CSYN ? g.n_cyc : 0;
  const float* w = S.w32 + (size_t)b * G;
  const float* v = S.v32 + (size_t)b * G;
  for (int r = 0; r < R; ++r) {
    const int k = kblk * (kRadFreqs * R) + r * kRadFreqs + kq;
    if (k >= F) break;  // warp-uniform
    const float nu = g.nu32[k];
    const float a_k = nu * incrit;          // x = a_k / e_j^2
    const float y_k = g.nu13[k] * rp.z;     // x^(1/3) = y_k e_j^(-2/3)
    const float xl = nu * inlar;
    const float la = tab ? __logf(a_k * xs) : 0.f, y13 = tab ? cbrtf(a_k * xs) : 0.f;
    float acc = 0.f, as = 0.f, ac = 0.f;  // synchrotron sum; SSA sum and its compensation
    for (int j = jl; j < G - 1; j += kRadLanes) {
      const float R_ =
          tab ? tabulated_R32(stab, g.syn_u0, g.syn_ih, g.syn_n, la + __ldg(g.lnginv2 + j), y13 * __ldg(g.ginv23 + j))
          : j >= jcyc ? aharonian_R32(a_k * __ldg(g.ginv2 + j), y_k * __ldg(g.ginv23 + j))
                      : cyclotron_R32(__ldg(g.psq32 + j), xl);
      acc = fmaf(R_, __ldg(w + j), acc);
      if (ssa) {  // Neumaier-compensated sum of the signed SSA terms
        const float x = R_ * __ldg(v + j);
        const float t = as + x;
        ac += fabsf(as) >= fabsf(x) ? (as - t) + x : (x - t) + as;
        as = t;
      }
    }
    // combine the kRadLanes partial sums of each frequency
#pragma unroll
    for (int o = 1; o < kRadLanes; o <<= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      const float os = __shfl_xor_sync(0xffffffffu, as, o);
      const float oc = __shfl_xor_sync(0xffffffffu, ac, o);
      float s_, e_;
      two_sum(as, os, s_, e_);
      as = s_;
      ac = ac + oc + e_;
    }
    if (jl == 0) {
      S.syn32[(size_t)b * F + k] = acc;
      S.ssa32[(size_t)b * F + k] = ssa ? make_float2(as, ac) : make_float2(0.f, 0.f);
    }
  }
}

// The same sums with the lane's gamma-bin inputs (JQ bins per lane, j = lane +
// 32 q, G - 1 <= 32 JQ) loaded once into registers and used for all R
// frequencies of the warp, and the synchrotron function (gamma > 2; every
// method) read from its value/slope table around the nearest point instead of
// evaluated: x = a_k / gamma_j^2 gives the table position from two logs, R(x) =
// g(ln x) x^(1/3) with x^(1/3) = a_k^(1/3) gamma_j^(-2/3) (relative error of
// the table ~1e-5). The cyclotron branch of CSYN (gamma <= 2) is evaluated.
// Every independent load is issued before the first use (one latency round).
template <int JQ, int RM>
__device__ void radiate_block_regs(const DevGrid& g, const DevState& S, const pbag_shock_params* prm, int b,
                                   int kblk, int R) {
  const int tid = threadIdx.x;
  const int G = g.G, F = g.F;
  const int kq = tid / kRadLanes, jl = tid % kRadLanes;
  const int flg = S.flags[b];
  const pbag_shock_params* pb = prm + slot_bw(S, b);
  const int ssa_on = pb->ssa_on, method = pb->syn_method;
  const float4 rp = *reinterpret_cast<const float4*>(S.rad32 + (size_t)b * 4);
  float nuv[RM], nu13v[RM], lnuv[RM];
#pragma unroll
  for (int r = 0; r < RM; ++r) {
    const int k = kblk * (kRadFreqs * R) + r * kRadFreqs + kq;
    const bool in = r < R && k < F;
    nuv[r] = in ? __ldg(g.nu32 + k) : 0.f;
    nu13v[r] = in ? __ldg(g.nu13 + k) : 0.f;
    lnuv[r] = in ? __ldg(g.lnnu + k) : 0.f;
  }
  const float* w = S.w32 + (size_t)b * G;
  const float* v = S.v32 + (size_t)b * G;
  const float ih = g.syn2_ih;
  float wv[JQ], vv[JQ], lgp[JQ], x13[JQ], ps[JQ];
#pragma unroll
  for (int q = 0; q < JQ; ++q) {
    const int j = jl + kRadLanes * q;
    const bool in = j < G - 1;
    wv[q] = in ? __ldg(w + j) : 0.f;
    vv[q] = in ? __ldg(v + j) : 0.f;
    lgp[q] = in ? __ldg(g.lnginv2 + j) * ih : 0.f;  // table position of ln(1/gamma^2)
    x13[q] = in ? __ldg(g.ginv23 + j) : 0.f;
    ps[q] = in ? __ldg(g.psq32 + j) : 0.f;
  }
  if (!(flg & kFlagActive)) return;
  const bool ssa = ssa_on != 0;
  const float2* tab =
      g.syntab2 + (method == PBAG_SYN_GSL ? 0 : method == PBAG_SYN_BESSEL ? kSynTab2N : 2 * kSynTab2N);
  const float xs = method == PBAG_SYN_GSL ? g.gsl_xs : 1.f;
  const float lxs = logf(xs) + logf(rp.x), cxs = cbrtf(xs);
  const float inlar = rp.y;
  const int jcyc = method == PBAG_SYN_CSYN ? g.n_cyc : 0;
  const int last = g.syn2_n - 1;
  constexpr float kRound = 12582912.f;  // 1.5 2^23: x + kRound rounds x to an integer in the mantissa
#pragma unroll
  for (int r = 0; r < RM; ++r) {
    const int k = kblk * (kRadFreqs * R) + r * kRadFreqs + kq;
    if (r >= R || k >= F) break;  // warp-uniform
    const float la = (lnuv[r] + lxs - g.syn2_u0) * ih;  // table position of ln a_k
    const float y13 = nu13v[r] * rp.z * cxs;            // a_k^(1/3)
    const float xl = nuv[r] * inlar;
    float acc = 0.f, as = 0.f, ac = 0.f;
#pragma unroll
    for (int q = 0; q < JQ; ++q) {
      const int j = jl + kRadLanes * q;
      if (j < G - 1) {
        float R_;
        // the cyclotron bins (jcyc <= 32) are all in register 0: the branch
        // exists in the first unrolled iteration only
        if (q > 0 || j >= jcyc) {
          const float p = la + lgp[q];
          const float rr = p + kRound;
          const int i = min(max(__float_as_int(rr) - __float_as_int(kRound), 0), last);
          const float f = p - (rr - kRound);
          const float2 t = __ldg(tab + i);
          R_ = fmaf(f, t.y, t.x) * (y13 * x13[q]);
        } else {
          R_ = cyclotron_R32(ps[q], xl);
        }
        acc = fmaf(R_, wv[q], acc);
        if (ssa) {
          const float x = R_ * vv[q];
          const float t = as + x;
          ac += fabsf(as) >= fabsf(x) ? (as - t) + x : (x - t) + as;
          as = t;
        }
      }
    }
#pragma unroll
    for (int o = 1; o < kRadLanes; o <<= 1) {
      acc += __shfl_xor_sync(0xffffffffu, acc, o);
      const float os = __shfl_xor_sync(0xffffffffu, as, o);
      const float oc = __shfl_xor_sync(0xffffffffu, ac, o);
      float s_, e_;
      two_sum(as, os, s_, e_);
      as = s_;
      ac = ac + oc + e_;
    }
    if (jl == 0) {
      S.syn32[(size_t)b * F + k] = acc;
      S.ssa32[(size_t)b * F + k] = ssa ? make_float2(as, ac) : make_float2(0.f, 0.f);
    }
  }
}

constexpr int kRadJq = 8;    // gamma bins per lane held in registers (G - 1 <= 256)
constexpr int kRadRMax = 2;  // frequencies per warp of the register path

template <int KPT>
__global__ void __launch_bounds__(kRadThreads)
k_rad_ssc(DevGrid g, DevState S, const pbag_shock_params* __restrict__ prm, int nbw, int rad_blocks, int R) {
  static_assert(kRadThreads == kSscThreads, "radiation and SSC tiles share the launch shape");
  grid_dep_wait();    // the step's evolve launch has completed
  grid_dep_launch();  // the next evolve launch may be scheduled
  const int blk = blockIdx.x;
  const int rc = (g.F + kRadFreqs * R - 1) / (kRadFreqs * R);
  if (blk < rad_blocks) {
    if (g.G - 1 <= kRadJq * kRadLanes && g.n_cyc <= kRadLanes && R <= kRadRMax)
      radiate_block_regs<kRadJq, kRadRMax>(g, S, prm, blk / rc, blk % rc, R);
    else
      radiate_block(g, S, prm, blk / rc, blk % rc, R);
  } else {
    ssc_block<KPT>(g, S, nbw, blk - rad_blocks);
  }
}

// ---------------------------------------------------------------------------
// microphysics.h:11-58, METHOD_TAU::iAPPROX; one reciprocal instead of three divisions
// computeIntensity's APPROX law (microphysics.h:11-45): em for dtau <= 1e-3,
// else em 3u/dtau with u = 1/2 + e/dtau - (1 - e)/dtau^2, e = exp(-dtau). The
// factor 3u/dtau lies in (0, 1] and is formed in FP32 from the bits of dtau
// (an FP64 exp and division would be ~45 FP64 instructions per frequency, each
// holding its sub-partition's FP64 unit 64 cycles): below dtau = 1 by its
// series 3 sum_{m>=3} (-1)^(m+1) (m-1)/m! dtau^(m-3) (the closed form cancels
// to ~dtau^3 there; the reference's FP64 form keeps ~1e-7 at dtau = 1e-3), above
// by the closed form (relative error < 1e-6 at dtau = 1). One FP64 product.
__device__ __forceinline__ double intensity_approx(double em, double dtau) {
  if (((__double2hiint(dtau) & 0x7fffffff) | __double2loint(dtau)) == 0) return em;  // dtau == 0
  if (!(dtau > 1.e-3)) return em;
  int ex;
  const float mt = f64_mant(dtau, ex);  // dtau = mt 2^ex, ex >= -10 here
  const float t = ex >= 127 ? 3.0e38f : f32_ldexp(mt, ex);
  float f;
  if (t < 1.f) {
    // coefficients 3 (-1)^(m+1) (m-1)/m!, m = 3 .. 14
    f = -4.4735908e-10f;
    f = fmaf(f, t, 5.7812558e-09f);
    f = fmaf(f, t, -6.8893298e-08f);
    f = fmaf(f, t, 7.5156325e-07f);
    f = fmaf(f, t, -7.4404762e-06f);
    f = fmaf(f, t, 6.6137566e-05f);
    f = fmaf(f, t, -5.2083333e-04f);
    f = fmaf(f, t, 3.5714286e-03f);
    f = fmaf(f, t, -2.0833333e-02f);
    f = fmaf(f, t, 0.1f);
    f = fmaf(f, t, -0.375f);
    f = fmaf(f, t, 1.f);
  } else {
    const float e = __expf(-t);
    const float r = 1.f / t;
    f = 3.f * (0.5f + e * r - (1.f - e) * (r * r)) * r;
  }
  return em * f64_from_mant(f, 0);
}

// The rest of computeRadiationNumericMixed for blastwave b at `step`, once its
// synchrotron and SSC sums are in place: synchrotron emissivity and SSA
// absorption, photon field, totals, the frequency-grid history rows, the
// seed-photon weights U of the step's SSC contraction and, when sh_v is given,
// the SSC cooling weights of the next step. A no-op returning false unless the
// blastwave radiated at `step` without error. The gamma-grid history rows
// (ele_f_all, gdot_*) are the caller's. Thread 0 leaves the blastwave's new
// flags and error code in sh_state; the caller synchronises before reading.
// Returns 0 (nothing to do), 1 (rows written) or 2 (a synchrotron value failed
// its check; nothing written). FQ frequencies per thread (F <= 128 FQ).
template <int FQ>
__device__ int finalize_bw(const DevGrid& g, const GridTab& T, const DevState& S, int64_t r0,
                            const pbag_shock_params& P, int b, int step, const pbag_outputs& out, int flags, int err,
                            float* sh_v, double* sh_usv, int* sh_state, float* sh_pp) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int F = g.F;
  __shared__ int red_f[3][kStepWarps];
  if (!(flags & kFlagActive) || err != 0) return 0;
  const double* scal = S.scal + (size_t)b * kScal;
  const bool num = P.ele_method == PBAG_ELE_NUMERIC;
  const bool ssc = P.ssc_on && g.K32 != nullptr;
  const bool dense_syn = out.syn_j_all || out.syn_a_all || out.syn_i_all;
  const size_t row = (size_t)(r0 + step);
  const float* syn32 = S.syn32 + (size_t)b * F;
  const float2* ssa32 = S.ssa32 + (size_t)b * F;
  const double* jssc = S.jssc + (size_t)b * F;
  // every load first
  const double dr = scal[kScalDr], acc = scal[kScalAcc];
  const double pref = scal[kScalPref], ssw = scal[kScalSw], ssv = scal[kScalSv];
  const int ew = exp_field(ssw) - 1023, ev = exp_field(ssv) - 1023;  // both are powers of two
  const double fac = scal[kScalFac], acc_ne = scal[kScalAccNe], anp_ne = scal[kScalAnpNe];
  float s32[FQ];
  float2 a32[FQ];
  double cs[FQ];
  if (S.Dsyn) {
    // tensor-core sums: cubic interpolation over the four bank nodes around the
    // blastwave's shift (pbag_syn_tc.cu), then CSYN's cyclotron bins on CUDA cores
    const double shd = scal[kScalSynShift];
    const double fl = floor(shd);
    const int n = (int)fl;
    float L[4];
    bank_weights((float)(shd - fl), L);
    const int tbw = g.sb_tbw, M = g.sb_M, Pb = g.sb_P;
    const float* Dt = S.Dsyn + ((size_t)(b / tbw) * Pb * 2 * tbw + 2 * (b % tbw)) * M;
    int base[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int na = n - 1 + a;
      const int qa = na >= 0 ? na / Pb : -((-na + Pb - 1) / Pb);
      base[a] = (na - qa * Pb) * 2 * tbw * M - qa - g.sb_mlo;  // + k: the row of output k
    }
    const bool cyc = P.syn_method == PBAG_SYN_CSYN && g.n_cyc > 0;
    const float inlar = S.rad32[(size_t)b * 4 + 1];
    const float* wv = S.w32 + (size_t)b * g.G;
    const float* vv = S.v32 + (size_t)b * g.G;
#pragma unroll
    for (int q = 0; q < FQ; ++q) {
      const int k = tid + q * kStepThreads;
      float sj = 0.f, sa = 0.f;
      if (k < F) {
        float dj[4], da[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float* d = Dt + base[a] + k;
          dj[a] = d[0];
          da[a] = P.ssa_on ? d[M] : 0.f;
        }
        sj = fmaxf(bank_interp(L, dj), 0.f);  // every synchrotron term is non-negative
        if (P.ssa_on) sa = bank_interp(L, da);
        if (cyc) {
          const float xl = g.nu32[k] * inlar;
          for (int j = 0; j < g.n_cyc; ++j) {
            const float R_ = cyclotron_R32(g.psq32[j], xl);
            sj = fmaf(R_, wv[j], sj);
            if (P.ssa_on) sa = fmaf(R_, vv[j], sa);
          }
        }
      }
      s32[q] = sj;
      a32[q] = make_float2(sa, 0.f);
      cs[q] = (k < F && ssc) ? jssc[k] : 0.;
    }
  } else {
#pragma unroll
    for (int q = 0; q < FQ; ++q) {
      const int k = tid + q * kStepThreads;
      const bool in = k < F;
      s32[q] = in ? syn32[k] : 0.f;
      a32[q] = (in && P.ssa_on) ? ssa32[k] : make_float2(0.f, 0.f);
      cs[q] = (in && ssc) ? jssc[k] : 0.;
    }
  }
  // synchrotron emissivity and SSA absorption from the FP32 sums
  // (numeric_model.h:148-238): the prefactor and the power-of-two scales
  double jsv[FQ], asv[FQ];
  bool jbad = false;
#pragma unroll
  for (int q = 0; q < FQ; ++q) {
    const int k = tid + q * kStepThreads;
    jsv[q] = asv[q] = 0.;
    if (k < F) {
      // (double)s * ssw with ssw a power of two, built from the bits (exactly the
      // same value without the FP64 conversion and product)
      const double js = k < F - 1 ? pref * f64_from_mant(s32[q], ew) : 0.;  // j_syn[F-1] = 0 (numeric_model.h:157)
      if (bad_value(js)) jbad = true;
      jsv[q] = js;
      if (P.ssa_on) {
        const double sa = f64_from_mant(a32[q].x, ev) + f64_from_mant(a32[q].y, ev);  // ((double)x + (double)y) ssv
        double a = fabs(pref * sa * T.ft(kTabSsaNu)[k]);  // :206-211
        if (not_finite(a)) a = 1e99;
        asv[q] = a;
      }
    }
  }
  if (__syncthreads_or(jbad ? 1 : 0)) {
    if (tid == 0) {
      set_error(S, b, PBAG_ERR_NONFINITE, step, __LINE__);
      if (sh_state) {
        sh_state[0] = flags;
        sh_state[1] = PBAG_ERR_NONFINITE;
      }
    }
    return 2;
  }
  // pair-production absorption (computePPabsorption, numeric_model.h:343-356)
  // from the previous photon density, before it is overwritten
  double* n = S.n + (size_t)b * F;
  const bool pp = ssc && P.pp_on;
  double ppa[FQ];
#pragma unroll
  for (int q = 0; q < FQ; ++q) ppa[q] = 0.;
  if (pp) {
    int pexp = 0;
    for (int k = tid; k < F - 1; k += kStepThreads) pexp = max(pexp, exp_field(n[k]));
    pexp = __reduce_max_sync(0xffffffffu, pexp);
    if (lane == 0) red_f[0][warp] = pexp;
    __syncthreads();
    pexp = 0;
#pragma unroll
    for (int v = 0; v < kStepWarps; ++v) pexp = max(pexp, red_f[0][v]);
    const double sp = scale_from_exp(pexp), usp = unscale_from_exp(pexp);
    for (int k = tid; k < F; k += kStepThreads) sh_pp[k] = k < F - 1 ? (float)(n[k] * sp) : 0.f;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < FQ; ++q) {
      const int k = tid + q * kStepThreads;
      if (k >= F) continue;
      float acc = 0.f;
      for (int j = 0; j < F - 1; ++j) acc = fmaf(sh_pp[j], __ldg(g.ppabsT + (size_t)j * F + k), acc);
      ppa[q] = (double)acc * usp;
    }
    __syncthreads();  // every thread has read the previous density
  }
  // new photon density (microphysics.h:516-523), totals and normalisation (:540-586)
  const double* inv_hnu = T.ft(kTabInvHnu);
  const double* dnu = T.ft(kTabDnuNu);
  const double* ksc = T.ft(kTabKscale);
  bool bad = false, seen = false;
  int uexp = 0, vexp = 0;
  double un[FQ], uk[FQ];  // u_k = n_k dnu_k and u_k kscale_k
#pragma unroll
  for (int q = 0; q < FQ; ++q) {
    const int k = tid + q * kStepThreads;
    un[q] = uk[q] = 0.;
    if (k >= F) continue;
    const double js = jsv[q], c = num ? cs[q] : 0.;
    const double nk = js * fac * inv_hnu[k] + c * fac * inv_hnu[k];
    n[k] = nk;
    const double u = nk * dnu[k];
    un[q] = u;
    uexp = max(uexp, exp_field(u));
    if (k < F - 1) {
      uk[q] = u * ksc[k];
      vexp = max(vexp, exp_field(uk[q]));
    }
    double tj0 = js + c;
    if (num && pp) {  // pair-production attenuation (microphysics.h:565-574)
      const double tau_pp = ppa[q] * dr;
      if (tau_pp > 0.) tj0 = tj0 * (-expm1(-tau_pp) / tau_pp);
    }
    const double ta = asv[q] * anp_ne;
    const double ti = intensity_approx(tj0 * acc, ta * dr);
    const double tj = tj0 * acc_ne;
    if (bad_value(tj)) bad = true;
    if (out.j_all) out.j_all[row * F + k] = tj;
    if (out.a_all) out.a_all[row * F + k] = ta;
    if (out.f_all) out.f_all[row * F + k] = nk;
    if (out.i_all) out.i_all[row * F + k] = ti;
    // storeDenseOutput (microphysics.h:602-633)
    if (dense_syn) {
      const double sj = js * acc;
      const double sa = asv[q] * anp_ne;
      if (out.syn_j_all) out.syn_j_all[row * F + k] = sj;
      if (out.syn_a_all) out.syn_a_all[row * F + k] = sa;
      if (out.syn_i_all) out.syn_i_all[row * F + k] = intensity_approx(sj, sa * dr);
      if (sj != 0.) seen = true;
    }
    if (ssc) {
      const double cj = cs[q] * acc;
      if (out.ssc_j_all) out.ssc_j_all[row * F + k] = cj;
      // ssc.a is the pair-production absorption (0 without it: I = j)
      if (out.ssc_i_all) out.ssc_i_all[row * F + k] = pp ? intensity_approx(cj, ppa[q] * anp_ne * dr) : cj;
    }
  }
  // one reduction: the scales of U and of the cooling weights, the checks
  uexp = __reduce_max_sync(0xffffffffu, uexp);
  vexp = __reduce_max_sync(0xffffffffu, vexp);
  const unsigned bits = __reduce_or_sync(0xffffffffu, (bad ? 1u : 0u) | (seen ? 2u : 0u));
  if (lane == 0) {
    red_f[0][warp] = uexp;
    red_f[1][warp] = vexp;
    red_f[2][warp] = (int)bits;
  }
  __syncthreads();
  uexp = vexp = 0;
  unsigned any = 0;
#pragma unroll
  for (int v = 0; v < kStepWarps; ++v) {
    uexp = max(uexp, red_f[0][v]);
    vexp = max(vexp, red_f[1][v]);
    any |= (unsigned)red_f[2][v];
  }
  if (ssc) {
    // seed-photon weights n_k (nu_{k+1}-nu_k)/nu_k of this step's SSC contraction,
    // and the cooling weights n_k dnu_k/nu_k kscale_k of the next step
    // (numeric_model.h:395-400), scaled to FP32 through their bits
    float* U = S.U32 + (size_t)b * F;
#pragma unroll
    for (int q = 0; q < FQ; ++q) {
      const int k = tid + q * kStepThreads;
      if (k >= F) continue;
      U[k] = f32_scaled(un[q], uexp);
      if (sh_v) sh_v[k] = k < F - 1 ? f32_scaled(uk[q], vexp) : 0.f;
    }
  }
  if (tid == 0) {
    int fl = flags;
    if (any & 2u) fl |= kFlagSynSeen;
    if (ssc) {
      S.scal[(size_t)b * kScal + kScalSU] = unscale_from_exp(uexp);
      fl |= kFlagUValid;
      if (sh_usv) *sh_usv = unscale_from_exp(vexp);
    }
    S.flags[b] = fl;
    int e = 0;
    if (any & 1u)
      e = PBAG_ERR_NONFINITE;
    else if (dense_syn && !(fl & kFlagSynSeen) && step > 0)
      e = PBAG_ERR_NONFINITE;  // microphysics.h:627-631
    if (e) set_error(S, b, e, step, __LINE__);
    if (sh_state) {
      sh_state[0] = fl;
      sh_state[1] = e;
    }
  }
  return 1;
}

// gamma-grid history rows of blastwave b at `step` (storeDenseOutput, microphysics.h:602-633)
__device__ void history_rows_g(const DevGrid& g, const DevState& S, size_t row, int b, const pbag_outputs& out) {
  if (!(out.ele_f_all || out.gdot_syn_all || out.gdot_adi_all || out.gdot_ssc_all)) return;
  const int G = g.G;
  const double* f = S.f + (size_t)b * G;
  const double* gd = S.gdot + (size_t)b * 3 * G;
  for (int i = threadIdx.x; i < G; i += kStepThreads) {
    if (out.ele_f_all) out.ele_f_all[row * G + i] = f[i];
    if (out.gdot_syn_all) out.gdot_syn_all[row * G + i] = gd[i];
    if (out.gdot_adi_all) out.gdot_adi_all[row * G + i] = gd[G + i];
    if (out.gdot_ssc_all) out.gdot_ssc_all[row * G + i] = gd[2 * G + i];
  }
}

__global__ void __launch_bounds__(kStepThreads)
k_finalize(DevGrid g, DevState S, const int64_t* __restrict__ off, const pbag_shock_params* __restrict__ prm,
           int step, pbag_outputs out) {
  const int b = blockIdx.x, bw = slot_bw(S, b);
  const int flags = S.flags[b], err = S.err[4 * b];
  const int64_t r0 = off[bw];
  if (step >= off[bw + 1] - r0) return;
  const pbag_shock_params P = prm[bw];
  const GridTab T{g.etab, g.Ge, g.Fe};
  __shared__ float sh_pp[PBAG_MAX_BINS];
  const int fq = (g.F + kStepThreads - 1) / kStepThreads;
  int fin;
  if (fq <= 1)
    fin = finalize_bw<1>(g, T, S, r0, P, b, step, out, flags, err, nullptr, nullptr, nullptr, sh_pp);
  else if (fq <= 2)
    fin = finalize_bw<2>(g, T, S, r0, P, b, step, out, flags, err, nullptr, nullptr, nullptr, sh_pp);
  else if (fq <= 4)
    fin = finalize_bw<4>(g, T, S, r0, P, b, step, out, flags, err, nullptr, nullptr, nullptr, sh_pp);
  else
    fin = finalize_bw<8>(g, T, S, r0, P, b, step, out, flags, err, nullptr, nullptr, nullptr, sh_pp);
  if (fin == 1) history_rows_g(g, S, (size_t)(r0 + step), b, out);
}

// ---------------------------------------------------------------------------
cudaError_t launch_prepare(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const int64_t* off,
                           const pbag_shock_params* prm, int nbw, int64_t nrec, int64_t* first, StepScal* ss,
                           cudaStream_t st) {
  if (nbw <= 0) return cudaSuccess;
  k_first_valid<<<nbw, kFirstValidThreads, 0, st>>>(recs, off, nbw, first);
  const int64_t npw = (int64_t)nbw * g.G;
  k_powp<<<(unsigned)((npw + 255) / 256), 256, 0, st>>>(g, prm, nbw, S.powp);
  if (nrec > 0)
    k_prep<<<(unsigned)((nrec + 127) / 128), 128, 0, st>>>(g, recs, off, prm, nbw, nrec, first, S.powp, ss);
  return cudaGetLastError();
}

cudaError_t launch_evolve(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const StepScal* ss,
                          const int64_t* off, const pbag_shock_params* prm, int nbw, int step,
                          const pbag_outputs& out, cudaStream_t st) {
  if (nbw <= 0) return cudaSuccess;
  const int kstage = evolve_kint_stage(g, nbw);
  const size_t smem = evolve_bytes(g, kstage);
  const int c = (g.G + kStepThreads - 1) / kStepThreads;
  const int fq = (g.F + kStepThreads - 1) / kStepThreads;
  cudaError_t e = cudaSuccess;
  auto go = [&](auto kern) {
    e = launch_step_kernel(kern, dim3(nbw), dim3(kStepThreads), smem, st, g, S, recs, ss, off, prm, step, out, kstage);
  };
  // large batches (the kernel-integral table not staged, small shared
  // memory): the register budget of four CTAs per SM, for more resident
  // blastwaves (no spills at 128 registers for grids up to 256 x 256); for
  // grids of at most 256 gamma and 128 nu also six or eight (80 / 64
  // registers, PBAG_EVOLVE_CTAS)
  if (kstage == 0 && nbw > kStageMaxBw && c <= 2 && fq <= 2) {
    if (c == 2 && fq == 1 && g.evolve_ctas >= 8)
      go(k_evolve<2, 1, 8>);
    else if (c == 2 && fq == 1 && g.evolve_ctas >= 6)
      go(k_evolve<2, 1, 6>);
    else if (c <= 1)
      fq <= 1 ? go(k_evolve<1, 1, 4>) : go(k_evolve<1, 2, 4>);
    else
      fq <= 1 ? go(k_evolve<2, 1, 4>) : go(k_evolve<2, 2, 4>);
    return e;
  }
#define PBAG_EVOLVE_FQ(CC)                 \
  if (fq <= 1) go(k_evolve<CC, 1, 1>);     \
  else if (fq <= 2) go(k_evolve<CC, 2, 1>); \
  else if (fq <= 4) go(k_evolve<CC, 4, 1>); \
  else go(k_evolve<CC, 8, 1>);
  if (c <= 1) {
    PBAG_EVOLVE_FQ(1)
  } else if (c <= 2) {
    PBAG_EVOLVE_FQ(2)
  } else if (c <= 4) {
    PBAG_EVOLVE_FQ(4)
  } else {
    PBAG_EVOLVE_FQ(8)
  }
#undef PBAG_EVOLVE_FQ
  return e;
}

cudaError_t launch_rad_ssc(const DevGrid& g, const DevState& S, const pbag_shock_params* prm, int nbw, bool ssc,
                           int step, cudaStream_t st) {
  (void)step;
  // frequencies per warp: each warp's per-blastwave setup and gamma-bin loads
  // serve R frequencies; with the register path R = 2 keeps a small batch's
  // CTAs (42 blastwaves x 128 frequencies: 672) resident in one wave next to
  // the SSC kernel while each warp's work stays short
  const int64_t pairs = (int64_t)nbw * g.F;
  const bool regs = g.G - 1 <= kRadJq * kRadLanes && g.n_cyc <= kRadLanes;
  const int R = !regs ? (pairs <= 40000 ? 1 : pairs <= 160000 ? 2 : pairs <= 640000 ? 4 : 8) : kRadRMax;
  const int rc = (g.F + kRadFreqs * R - 1) / (kRadFreqs * R);
  const int rad_blocks = nbw * rc;
  const int ssc_blocks = ssc ? ssc_block_count(g, nbw) : 0;
  const int total = rad_blocks + ssc_blocks;
  if (total <= 0) return cudaSuccess;
  const int kpt = (g.F + kSscThreads - 1) / kSscThreads;
  const size_t smem = ssc ? (size_t)ssc_smem_bytes(g) : 0;
  auto go = [&](auto kern) {
    return launch_step_kernel(kern, dim3(total), dim3(kRadThreads), smem, st, g, S, prm, nbw, rad_blocks, R);
  };
  if (kpt <= 1) return go(k_rad_ssc<1>);
  if (kpt <= 2) return go(k_rad_ssc<2>);
  if (kpt <= 4) return go(k_rad_ssc<4>);
  return go(k_rad_ssc<8>);
}

cudaError_t launch_finalize(const DevGrid& g, const DevState& S, const int64_t* off, const pbag_shock_params* prm,
                            int nbw, int step, const pbag_outputs& out, cudaStream_t st) {
  if (nbw <= 0) return cudaSuccess;
  k_finalize<<<nbw, kStepThreads, 0, st>>>(g, S, off, prm, step, out);
  return cudaGetLastError();
}

bool& pdl_scope() {
  thread_local bool on = false;
  return on;
}

size_t evolve_smem_max_bytes() { return kEvolveSmemMax; }

cudaError_t configure_kernels() {
  const int smem = ssc_smem_max_bytes();
  const int esmem = (int)evolve_smem_max_bytes();
  cudaError_t e = cudaSuccess;
  auto attr = [&](const void* k, int bytes) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  };
#define PBAG_EVOLVE_ATTR(CC)                                   \
  attr((const void*)k_evolve<CC, 1, 1>, esmem);                \
  attr((const void*)k_evolve<CC, 2, 1>, esmem);                \
  attr((const void*)k_evolve<CC, 4, 1>, esmem);                \
  attr((const void*)k_evolve<CC, 8, 1>, esmem);
  PBAG_EVOLVE_ATTR(1)
  PBAG_EVOLVE_ATTR(2)
  PBAG_EVOLVE_ATTR(4)
  PBAG_EVOLVE_ATTR(8)
#undef PBAG_EVOLVE_ATTR
  attr((const void*)k_evolve<1, 1, 4>, esmem);
  attr((const void*)k_evolve<1, 2, 4>, esmem);
  attr((const void*)k_evolve<2, 1, 4>, esmem);
  attr((const void*)k_evolve<2, 2, 4>, esmem);
  attr((const void*)k_evolve<2, 1, 6>, esmem);
  attr((const void*)k_evolve<2, 1, 8>, esmem);
  attr((const void*)k_rad_ssc<1>, smem);
  attr((const void*)k_rad_ssc<2>, smem);
  attr((const void*)k_rad_ssc<4>, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_rad_ssc<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

}  // namespace pbag
