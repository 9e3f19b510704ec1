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
__global__ void k_first_valid(const pbag_step_rec* __restrict__ recs, const int64_t* __restrict__ off, int nbw,
                              int64_t* __restrict__ first) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbw) return;
  int64_t r = off[b];
  const int64_t end = off[b + 1];
  while (r < end && recs[r].mode == PBAG_SKIP) ++r;
  first[b] = r;  // == end when the blastwave is never valid
}

__global__ void k_powp(DevGrid g, const pbag_shock_params* __restrict__ prm, int nbw, double* __restrict__ powp) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)nbw * g.G) return;
  const int b = (int)(idx / g.G), i = (int)(idx - (int64_t)b * g.G);
  powp[idx] = pow(g.e[i], -prm[b].p);
}

// Value of the analytic distribution (microphysics.h:237-278) at bin i, given
// that i lies in branch a (first) or b (second).
__device__ __forceinline__ double pl_branch_a(const DevGrid& g, const StepScal& s, const double* pp, int i) {
  return (s.flags & kRecFast) ? s.K * s.c_fast * g.inv_e2[i] : s.K * pp[i];
}
__device__ __forceinline__ double pl_branch_b(const DevGrid& g, const StepScal& s, const double* pp, int i,
                                              double Kb) {
  return Kb * pp[i] * g.inv_e[i];
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
  bool pl_bad = (s.ia1 > s.ia0 && bad_value(pl_branch_a(g, s, pp, s.ia0))) ||
                (s.ib1 > s.ib0 && bad_value(pl_branch_b(g, s, pp, s.ib0, Kb)));
  // synchrotron kernel constants (kernels.h:194-202, 427, 471)
  const double B = q.B;
  const bool dermer = P.syn_method == PBAG_SYN_DER09;
  s.pref = dermer ? sqrt3 * pow(q_e, 3.) * B / (m_e * c_light * c_light) : sqrt3 * pow(q_e, 3.) * B / mec2;
  s.inv_ncrit = (float)((4. * M_PI * m_e * c_light) / (3. * q_e * B));
  s.inv_nlar = (float)((2. * pi_ * m_e * c_light) / (3. * q_e * B));
  s.dr = q.dr;
  if (init) {
    s.vol = q.m_p1 / q.rho_p1;
    s.fac = s.dr / c_light / s.vol;
    if (pl_bad) {
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

__device__ void finalize_bw(const DevGrid& g, const DevState& S, const int64_t* __restrict__ off,
                            const pbag_shock_params* __restrict__ prm, int b, int step, const pbag_outputs& out);

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

// Dynamic shared memory of k_evolve: [staged KintT][N(gamma) | f/gamma^2 | SSA
// weights (G doubles each)][seed-photon weights (F floats)].
__host__ __device__ inline size_t evolve_stage_bytes(const DevGrid& g) { return ((size_t)g.kint_stage + 127) / 128 * 128; }
__host__ __device__ inline size_t evolve_bytes(const DevGrid& g) {
  return evolve_stage_bytes(g) + 3 * (size_t)g.G * sizeof(double) + (size_t)g.F * sizeof(float);
}

// ---------------------------------------------------------------------------
// One step of every blastwave, one CTA each, C gamma bins per thread in the solve.
template <int C>
__global__ void __launch_bounds__(kStepThreads)
k_evolve(DevGrid g, DevState S, const pbag_step_rec* __restrict__ recs, const StepScal* __restrict__ ss,
         const int64_t* __restrict__ off, const pbag_shock_params* __restrict__ prm, int step, pbag_outputs out) {
  const int b = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = g.G, F = g.F;
  // the previous step's photon field, totals and history rows (same CTA shape)
  if (step > 0) {
    finalize_bw(g, S, off, prm, b, step - 1, out);
    __syncthreads();  // its flag and error updates are visible below
  }
  extern __shared__ __align__(128) unsigned char evo_smem[];
  float* sh_k = reinterpret_cast<float*>(evo_smem);  // staged KintT
  double* sh_f = reinterpret_cast<double*>(evo_smem + evolve_stage_bytes(g));  // heating term, then N(gamma)
  double* sh_t = sh_f + G;                                                      // f / gamma^2
  double* sh_vd = sh_t + G;                                                     // SSA weights
  float* sh_v = reinterpret_cast<float*>(sh_vd + G);  // seed-photon weights of the SSC cooling GEMV
  __shared__ double red_d[kStepWarps];
  __shared__ int red_i[3][kStepWarps];
  __shared__ double xs[2][kStepWarps];
  __shared__ double pw0[kStepWarps];
  __shared__ __align__(8) uint64_t kbar;

  int flags = S.flags[b];
  const int64_t r0 = off[b], len = off[b + 1] - off[b];
  bool active = S.err[4 * b] == 0 && step < len;
  StepScal sc;
  if (active) {
    sc = ss[r0 + step];
    active = (sc.flags & kRecValid) != 0;
  }
  __syncthreads();  // every thread has read flags before thread 0 rewrites them
  if (tid == 0) S.flags[b] = flags & ~kFlagActive;
  if (!active) return;

#define PBAG_FAIL(code, site)                            \
  do {                                                   \
    if (tid == 0) set_error(S, b, (code), step, (site)); \
    return;                                              \
  } while (0)

  if (sc.err) PBAG_FAIL(sc.err, sc.site);
  const pbag_step_rec& r = recs[r0 + step];
  const double accel = r.accel_frac, B = r.B;
  const pbag_shock_params P = prm[b];
  double* f = S.f + (size_t)b * G;
  const double* pp = S.powp + (size_t)b * G;
  const double Kb = (sc.flags & kRecFast) ? sc.K : sc.K * r.gamma_c;
  // the stateful SSA derivative of the last step, needed at the end
  double* dfde = S.dfde + (size_t)b * G;
  double dpre[C];
#pragma unroll
  for (int k = 0; k < C; ++k) {
    const int i = tid + k * kStepThreads;
    dpre[k] = (P.ssa_on && i < G) ? dfde[i] : 0.;
  }

  if (sc.flags & kRecInit) {
    // ---- initializeElectronDistribution (microphysics.h:347-357): untouched
    // entries keep their value, then all but the last bin scale by accel_frac
    for (int i = tid; i < G; i += kStepThreads) {
      double v = f[i];
      if (i >= sc.ia0 && i < sc.ia1) v = pl_branch_a(g, sc, pp, i);
      else if (i >= sc.ib0 && i < sc.ib1) v = pl_branch_b(g, sc, pp, i, Kb);
      if (i < G - 1) v *= accel;
      f[i] = v;
      sh_f[i] = v;
    }
    flags |= kFlagInit;
  } else if (sc.n_sub == 0) {
    // ---- analytic distribution (microphysics.h:446-448)
    for (int i = tid; i < G; i += kStepThreads) {
      double v = 0.;
      if (i >= sc.ia0 && i < sc.ia1) v = pl_branch_a(g, sc, pp, i);
      else if (i >= sc.ib0 && i < sc.ib1) v = pl_branch_b(g, sc, pp, i, Kb);
      f[i] = v;
      sh_f[i] = v;
    }
  } else {
    // ---- Chang-Cooper evolution (microphysics.h:451-480)
    const bool ssc = P.ssc_on && g.KintT != nullptr;
    const bool staged = ssc && g.kint_stage > 0;
    if (staged && tid == 0) {
      // the kernel-integral table streams into shared memory while the
      // seed-photon weights are formed
      const uint32_t bar = smem_addr(&kbar);
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"((uint32_t)g.kint_stage)
                   : "memory");
      const unsigned char* src = reinterpret_cast<const unsigned char*>(g.KintT);
      for (int o = 0; o < g.kint_stage; o += 32768) {
        const uint32_t n = (uint32_t)min(32768, g.kint_stage - o);
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_addr(evo_smem + o)),
            "l"(src + o), "r"(n), "r"(bar)
            : "memory");
      }
    }
    const double delta_t = sc.dt_sub;
    const int n_sub = sc.n_sub;
    // this thread's bins j = tid*C + q: state and per-bin tables, loaded early
    double fr[C], ppq[C], odg[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int j = tid * C + q;
      const bool in = j < G;
      fr[q] = in ? f[j] : 0.;
      ppq[q] = in ? pp[j] : 0.;
      odg[q] = in ? g.inv_dgb[j] : 0.;
    }
    double sv = 1., usv = 1.;
    if (ssc) {  // seed-photon weights n_k dnu_k / nu_k, scaled by the kernel-integral columns
      const double* n = S.n + (size_t)b * F;
      int vexp = 0;
      for (int k = tid; k < F - 1; k += kStepThreads) {
        const double v = n[k] * g.dnu_nu[k] * g.kscale[k];
        sh_t[k] = v;  // (sh_t is free until the weights below)
        vexp = max(vexp, exp_field(v));
      }
      vexp = block_max_int(vexp, red_i[0]);
      sv = scale_from_exp(vexp);
      usv = unscale_from_exp(vexp);
      for (int k = tid; k < F; k += kStepThreads) sh_v[k] = k < F - 1 ? (float)(sh_t[k] * sv) : 0.f;
    }
    __syncthreads();
    if (staged) {
      const int miss = __syncthreads_or(mbar_wait_bounded(smem_addr(&kbar), 0) ? 0 : 1);
      if (miss) {
        if (tid == 0) {
          set_error(S, b, PBAG_ERR_TIMEOUT, step, __LINE__);
          mbar_wait_bounded(smem_addr(&kbar), 0);  // the copy must land before the CTA exits
        }
        return;
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
    for (int i = tid; i < G - 1; i += kStepThreads) {
      const double vs = c_syn * g.half2[i];
      const double va = sc.dlnVdt * g.hadi[i];
      double vc = gssc[i];
      if (ssc) {
        float acc = 0.f;
        if (staged) {
          const float* kc = sh_k + i;
#pragma unroll 8
          for (int k = 0; k < F - 1; k++) acc = fmaf(sh_v[k], kc[(size_t)k * Gs], acc);
        } else {
          const float* kc = g.KintT + i;
#pragma unroll 16
          for (int k = 0; k < F - 1; k++) acc = fmaf(sh_v[k], __ldg(kc + (size_t)k * Gs), acc);
        }
        vc = c_ssc * (double)acc * g.ihalf2[i];
        gssc[i] = vc;
      }
      gsyn[i] = vs;
      gadi[i] = va;
      const double H = vs + va + vc;
      if (not_finite(H)) hbad = true;
      sh_f[i] = H;
    }
    if (tid == 0) sh_f[G - 1] = 0.;  // heating_term[G-1] is never set (numeric_model.h:761)
    if (__syncthreads_or(hbad ? 1 : 0)) PBAG_FAIL(PBAG_ERR_NONFINITE, __LINE__);
    // tridiagonal coefficients (numeric_model.h:539-675 with dispersion = 0,
    // delta_j = 0): a = 0, b_k = 1 + dt H_{k-1}/dgb_k (b_0 = b_{G-1} = 1),
    // c_k = -dt H_k/dgb_k (c_{G-1} = 0)
    double ib[C], qb[C], bt[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      const int j = tid * C + q;
      ib[q] = qb[q] = bt[q] = 0.;
      if (j < G) {
        const double Hb = (j > 0 && j < G - 1) ? sh_f[j - 1] : 0.;  // b_0 and b_{G-1} see no inflow
        const double Hf = j < G - 1 ? sh_f[j] : 0.;
        const double bb = 1. + (odg[q] * Hb) * delta_t;
        const double cc = (odg[q] * Hf) * -delta_t;
        const double Q = (j >= sc.iq0 && j < sc.iq1) ? sc.Ns * ppq[q] : 0.;
        ib[q] = 1. / bb;
        bt[q] = -(cc * ib[q]);
        qb[q] = (Q * delta_t) * ib[q];
      }
    }
    const int T = (G + C - 1) / C;  // threads that own bins
    const bool sbad = n_sub < kScanMaxSub ? cc_scan<C>(fr, ib, qb, bt, n_sub, xs, pw0)
                                          : cc_systolic<C>(fr, ib, qb, bt, n_sub, T, xs);
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
  double ne = 0.;
  int wexp = 0, Wexp = 0;
#pragma unroll
  for (int k = 0; k < C; ++k) {
    const int i = tid + k * kStepThreads;
    if (i < G) {
      const double fi = sh_f[i];
      sh_t[i] = fi * g.inv_e2[i];  // f / e / e (numeric_model.h:194-195)
      if (i < G - 1) {
        const double w = fi * g.de[i];
        ne += w;  // N_e (microphysics.h:556-558)
        wexp = max(wexp, exp_field(w));
        Wexp = max(Wexp, exp_field(w * g.inv_e2[i]));
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
  const double sw = scale_from_exp(wexp);
  float* w32 = S.w32 + (size_t)b * G;
  for (int i = tid; i < G; i += kStepThreads) w32[i] = i < G - 1 ? (float)(sh_f[i] * g.de[i] * sw) : 0.f;
  // SSC electron weights W_j = f_j (e_{j+1}-e_j) 3/4 sigma_T c / e_j^2 (numeric_model.h:271-277)
  // (FP32 for the CUDA-core contraction, BF16 hi + lo tiles for the tensor cores)
  if (P.ssc_on && g.K32 != nullptr) {
    const double sW = scale_from_exp(Wexp);
    float* W = S.W32 + (size_t)b * g.Gp;
    uint16_t* A = S.Abf ? S.Abf + (size_t)(b / kTcCols) * tc_tile_elems(kTcCols, g.Gp) : nullptr;
    const int m = b % kTcCols;
    for (int j = tid; j < g.Gp; j += kStepThreads) {
      const float w = j < G - 1 ? (float)(sh_f[j] * g.de[j] * g.inv_e2[j] * sW) : 0.f;
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
            d = 0.5 * (sh_t[i + 1] - sh_t[i - 1]) * g.inv_dxm[i];
          dfde[i] = d;
        }
        if (i < G - 1) {
          const double v = g.e2de[i] * d;  // e_j^2 (e_{j+1}-e_j) dfde_j (numeric_model.h:208)
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
    const double svd = scale_from_exp(vexp);
    float* v32 = S.v32 + (size_t)b * G;
    for (int i = tid; i < G; i += kStepThreads) v32[i] = i < G - 1 ? (float)(sh_vd[i] * svd) : 0.f;
  }
  if (!positive(ne) && !is_nan(ne)) PBAG_FAIL(PBAG_ERR_NELE, __LINE__);  // n_ele <= 0 (microphysics.h:560-563)
  if (tid == 0) {
    double* scal = S.scal + (size_t)b * kScal;
    if (P.ssc_on && g.K32 != nullptr) scal[kScalSW] = 3. / 4. * sigma_T * c_light * unscale_from_exp(Wexp);
    scal[kScalDr] = sc.dr;
    scal[kScalVol] = sc.vol;
    scal[kScalNele] = ne;
    scal[kScalFac] = sc.fac;
    const double acc_ne = accel / ne;
    scal[kScalAccNe] = acc_ne;
    scal[kScalAnpNe] = accel * r.n_prime / ne;
    scal[kScalAcc] = accel;
    scal[kScalNp] = r.n_prime;
    scal[kScalNsub] = (double)sc.n_sub;
    scal[kScalSw] = unscale_from_exp(wexp);
    scal[kScalSv] = unscale_from_exp(vexp);
    scal[kScalPref] = sc.pref;
    float* rp = S.rad32 + (size_t)b * 4;
    rp[0] = sc.inv_ncrit;
    rp[1] = sc.inv_nlar;
    rp[2] = cbrtf(sc.inv_ncrit);
    rp[3] = 0.f;
    S.flags[b] = flags | kFlagActive;
  }
#undef PBAG_FAIL
}

// ---------------------------------------------------------------------------
// Synchrotron and SSA sums of one blastwave for kRadFreqs frequencies: one warp
// per frequency splits the gamma sum over its lanes; the synchrotron kernel
// values are generated in FP32 on the fly and never stored. The kernel has no
// FP64 instruction (each costs a warp 64 cycles of its SM sub-partition's
// FP64 unit on this part): the FP64 prefactors are applied by finalize_bw.
__device__ void radiate_block(const DevGrid& g, const DevState& S, const pbag_shock_params* prm, int b, int kblk) {
  const int tid = threadIdx.x;
  const int G = g.G, F = g.F;
  if (!(S.flags[b] & kFlagActive)) return;
  const bool ssa = prm[b].ssa_on != 0;
  const bool dermer = prm[b].syn_method == PBAG_SYN_DER09;
  const float4 rp = *reinterpret_cast<const float4*>(S.rad32 + (size_t)b * 4);
  const float incrit = rp.x, inlar = rp.y;
  const int kq = tid / kRadLanes, jl = tid % kRadLanes;
  const int k = kblk * kRadFreqs + kq;
  const int kk = k < F ? k : F - 1;
  const float nu = g.nu32[kk];
  const float a_k = nu * incrit;          // x = a_k / e_j^2
  const float y_k = g.nu13[kk] * rp.z;    // x^(1/3) = y_k e_j^(-2/3)
  const float xl = nu * inlar;
  const int jcyc = dermer ? 0 : g.n_cyc;
  const float* w = S.w32 + (size_t)b * G;
  const float* v = S.v32 + (size_t)b * G;
  float acc = 0.f, as = 0.f, ac = 0.f;  // synchrotron sum; SSA sum and its compensation
  for (int j = jl; j < G - 1; j += kRadLanes) {
    const float R = j >= jcyc ? aharonian_R32(a_k * __ldg(g.ginv2 + j), y_k * __ldg(g.ginv23 + j))
                              : cyclotron_R32(__ldg(g.psq32 + j), xl);
    acc = fmaf(R, __ldg(w + j), acc);
    if (ssa) {  // Neumaier-compensated sum of the signed SSA terms
      const float x = R * __ldg(v + j);
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
    float s, e;
    two_sum(as, os, s, e);
    as = s;
    ac = ac + oc + e;
  }
  if (jl == 0 && k < F) {
    S.syn32[(size_t)b * F + k] = acc;
    S.ssa32[(size_t)b * F + k] = ssa ? make_float2(as, ac) : make_float2(0.f, 0.f);
  }
}

template <int KPT>
__global__ void __launch_bounds__(kRadThreads)
k_rad_ssc(DevGrid g, DevState S, const pbag_shock_params* __restrict__ prm, int nbw, int rad_blocks, int step) {
  static_assert(kRadThreads == kSscThreads, "radiation and SSC tiles share the launch shape");
  (void)step;
  const int blk = blockIdx.x;
  const int rc = (g.F + kRadFreqs - 1) / kRadFreqs;
  if (blk < rad_blocks) {
    radiate_block(g, S, prm, blk / rc, blk % rc);
  } else {
    ssc_block<KPT>(g, S, nbw, blk - rad_blocks);
  }
}

// ---------------------------------------------------------------------------
// microphysics.h:11-58, METHOD_TAU::iAPPROX; one reciprocal instead of three divisions
__device__ __forceinline__ double intensity_approx(double em, double dtau) {
  if (((__double2hiint(dtau) & 0x7fffffff) | __double2loint(dtau)) == 0) return em;  // dtau == 0
  if (!(dtau > 1.e-3)) return em;
  const double e = exp(-dtau);
  const double r = 1. / dtau;
  const double u = 1. / 2. + e * r - (1 - e) * (r * r);
  return em * (3. * u * r);
}

// The rest of computeRadiationNumericMixed for blastwave b at `step`, once its
// synchrotron and SSC emissivities are in place; a no-op unless the
// blastwave radiated at that step. Runs at the start of the next step's
// k_evolve (same CTA shape), and as k_finalize after the last step.
__device__ void finalize_bw(const DevGrid& g, const DevState& S, const int64_t* __restrict__ off,
                            const pbag_shock_params* __restrict__ prm, int b, int step, const pbag_outputs& out) {
  const int tid = threadIdx.x;
  const int G = g.G, F = g.F;
  __shared__ int red_i[kStepThreads / 32];
  const int flags = S.flags[b];
  if (!(flags & kFlagActive) || S.err[4 * b] != 0) return;
  const pbag_shock_params P = prm[b];
  const double* scal = S.scal + (size_t)b * kScal;
  const double dr = scal[kScalDr], acc = scal[kScalAcc];
  const bool num = P.ele_method == PBAG_ELE_NUMERIC;
  const bool ssc = P.ssc_on && g.K32 != nullptr;
  const bool dense_syn = out.syn_j_all || out.syn_a_all || out.syn_i_all;
  const size_t row = (size_t)(off[b] + step);
  double* n = S.n + (size_t)b * F;
  const float* syn32 = S.syn32 + (size_t)b * F;
  const float2* ssa32 = S.ssa32 + (size_t)b * F;
  const double* jssc = S.jssc + (size_t)b * F;
  // synchrotron emissivity and SSA absorption from the FP32 sums
  // (numeric_model.h:148-238): the prefactor and the power-of-two scales
  const double pref = scal[kScalPref], ssw = scal[kScalSw], ssv = scal[kScalSv];
  double jsv[kFinalPerThread], asv[kFinalPerThread];
  bool jbad = false;
#pragma unroll
  for (int q = 0; q < kFinalPerThread; ++q) {
    const int k = tid + q * kStepThreads;
    jsv[q] = asv[q] = 0.;
    if (k < F) {
      const double js = k < F - 1 ? pref * ((double)syn32[k] * ssw) : 0.;  // j_syn[F-1] = 0 (numeric_model.h:157)
      if (bad_value(js)) jbad = true;
      jsv[q] = js;
      if (P.ssa_on) {
        const float2 sa = ssa32[k];
        double a = fabs(pref * (((double)sa.x + (double)sa.y) * ssv) * g.ssa_nu[k]);  // numeric_model.h:206-211
        if (not_finite(a)) a = 1e99;
        asv[q] = a;
      }
    }
  }
  if (__syncthreads_or(jbad ? 1 : 0)) {
    if (tid == 0) set_error(S, b, PBAG_ERR_NONFINITE, step, __LINE__);
    return;
  }
  // new photon density (microphysics.h:516-523)
  const double fac = scal[kScalFac];
  const double acc_ne = scal[kScalAccNe], anp_ne = scal[kScalAnpNe];
  bool bad = false, seen = false;
  int uexp = 0;
#pragma unroll
  for (int q = 0; q < kFinalPerThread; ++q) {
    const int k = tid + q * kStepThreads;
    if (k >= F) continue;
    const double js = jsv[q], cs = (num && ssc) ? jssc[k] : 0.;
    const double nk = js * fac * g.inv_hnu[k] + cs * fac * g.inv_hnu[k];
    n[k] = nk;
    uexp = max(uexp, exp_field(nk * g.dnu_nu[k]));
    // totals and normalisation (microphysics.h:540-586)
    const double tj0 = js + cs;
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
  // seed-photon weights n_k (nu_{k+1}-nu_k)/nu_k for the next step's SSC contraction
  uexp = block_max_int(uexp, red_i);
  const double su = scale_from_exp(uexp);
  if (ssc) {
    float* U = S.U32 + (size_t)b * F;
    for (int k = tid; k < F; k += kStepThreads) U[k] = (float)(n[k] * g.dnu_nu[k] * su);
  }
  const int any_bad = __syncthreads_or(bad ? 1 : 0);
  const int any_seen = __syncthreads_or(seen ? 1 : 0);
  if (tid == 0) {
    int fl = flags;
    if (any_seen) fl |= kFlagSynSeen;
    if (ssc) {
      S.scal[(size_t)b * kScal + kScalSU] = unscale_from_exp(uexp);
      fl |= kFlagUValid;
    }
    S.flags[b] = fl;
    if (any_bad)
      set_error(S, b, PBAG_ERR_NONFINITE, step, __LINE__);
    else if (dense_syn && !(fl & kFlagSynSeen) && step > 0)
      set_error(S, b, PBAG_ERR_NONFINITE, step, __LINE__);  // microphysics.h:627-631
  }
}

__global__ void __launch_bounds__(kStepThreads)
k_finalize(DevGrid g, DevState S, const int64_t* __restrict__ off, const pbag_shock_params* __restrict__ prm,
           int step, pbag_outputs out) {
  finalize_bw(g, S, off, prm, blockIdx.x, step, out);
}

// ---------------------------------------------------------------------------
cudaError_t launch_prepare(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const int64_t* off,
                           const pbag_shock_params* prm, int nbw, int64_t nrec, int64_t* first, StepScal* ss,
                           cudaStream_t st) {
  if (nbw <= 0) return cudaSuccess;
  k_first_valid<<<(nbw + 127) / 128, 128, 0, st>>>(recs, off, nbw, first);
  const int64_t npw = (int64_t)nbw * g.G;
  k_powp<<<(unsigned)((npw + 255) / 256), 256, 0, st>>>(g, prm, nbw, S.powp);
  if (nrec > 0)
    k_prep<<<(unsigned)((nrec + 127) / 128), 128, 0, st>>>(g, recs, off, prm, nbw, nrec, first, S.powp, ss);
  return cudaGetLastError();
}

cudaError_t launch_evolve(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const StepScal* ss,
                          const int64_t* off, const pbag_shock_params* prm, int nbw, int step,
                          const pbag_outputs& out, cudaStream_t st) {
  const size_t smem = evolve_bytes(g);
  const int c = (g.G + kStepThreads - 1) / kStepThreads;
  if (c <= 1)
    k_evolve<1><<<nbw, kStepThreads, smem, st>>>(g, S, recs, ss, off, prm, step, out);
  else if (c <= 2)
    k_evolve<2><<<nbw, kStepThreads, smem, st>>>(g, S, recs, ss, off, prm, step, out);
  else if (c <= 4)
    k_evolve<4><<<nbw, kStepThreads, smem, st>>>(g, S, recs, ss, off, prm, step, out);
  else
    k_evolve<8><<<nbw, kStepThreads, smem, st>>>(g, S, recs, ss, off, prm, step, out);
  return cudaGetLastError();
}

cudaError_t launch_rad_ssc(const DevGrid& g, const DevState& S, const pbag_shock_params* prm, int nbw, bool ssc,
                           int step, cudaStream_t st) {
  const int rc = (g.F + kRadFreqs - 1) / kRadFreqs;
  const int rad_blocks = nbw * rc;
  const int ssc_blocks = ssc ? ssc_block_count(g, nbw) : 0;
  const int total = rad_blocks + ssc_blocks;
  if (total <= 0) return cudaSuccess;
  const int kpt = (g.F + kSscThreads - 1) / kSscThreads;
  const size_t smem = ssc ? (size_t)ssc_smem_bytes(g) : 0;
  if (kpt <= 1)
    k_rad_ssc<1><<<total, kRadThreads, smem, st>>>(g, S, prm, nbw, rad_blocks, step);
  else if (kpt <= 2)
    k_rad_ssc<2><<<total, kRadThreads, smem, st>>>(g, S, prm, nbw, rad_blocks, step);
  else if (kpt <= 4)
    k_rad_ssc<4><<<total, kRadThreads, smem, st>>>(g, S, prm, nbw, rad_blocks, step);
  else
    k_rad_ssc<8><<<total, kRadThreads, smem, st>>>(g, S, prm, nbw, rad_blocks, step);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DevGrid& g, const DevState& S, const int64_t* off, const pbag_shock_params* prm,
                            int nbw, int step, const pbag_outputs& out, cudaStream_t st) {
  k_finalize<<<nbw, kStepThreads, 0, st>>>(g, S, off, prm, step, out);
  return cudaGetLastError();
}

size_t evolve_smem_bytes(const DevGrid& g) { return evolve_bytes(g); }
size_t evolve_smem_max_bytes() {
  return ((size_t)kKintStageMax + 127) / 128 * 128 + 3 * (size_t)PBAG_MAX_BINS * sizeof(double) +
         (size_t)PBAG_MAX_BINS * sizeof(float);
}

cudaError_t configure_kernels() {
  const int smem = ssc_smem_max_bytes();
  const int esmem = (int)evolve_smem_max_bytes();
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_evolve<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, esmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_evolve<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, esmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_evolve<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, esmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_evolve<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, esmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_rad_ssc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_rad_ssc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(k_rad_ssc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(k_rad_ssc<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

}  // namespace pbag
