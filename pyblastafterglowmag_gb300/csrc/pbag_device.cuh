// pbag_device.cuh - device-side data layout and helpers shared by the step
// kernels. Paths in comments are relative to the reference's src/ directory.
#ifndef PBAG_DEVICE_CUH
#define PBAG_DEVICE_CUH

#include <cstdint>

#include "pbag.h"
#include "pbag_internal.h"
#include "pbag_const.h"

namespace pbag {

constexpr int kStepThreads = 128;     // threads per blastwave in the evolve / finalize kernels
constexpr int kMaxPerThread = (PBAG_MAX_BINS + kStepThreads - 1) / kStepThreads;  // gamma bins per thread
constexpr int kRadThreads = 128;      // threads of one radiation CTA
constexpr int kRadLanes = 32;         // threads per frequency in a radiation CTA (one warp)
constexpr int kRadFreqs = kRadThreads / kRadLanes;  // frequencies per radiation CTA
constexpr int kStepWarps = kStepThreads / 32;
constexpr int kFinalPerThread = (PBAG_MAX_BINS + kStepThreads - 1) / kStepThreads;  // frequencies per thread in finalize
constexpr int kKintStageMax = 112 * 1024;  // largest SSC kernel-integral table staged in shared memory
constexpr int kScanMaxSub = 32;       // below this many substeps the solve is a parallel scan, else systolic
constexpr int kFirstValidThreads = 256;  // records one k_first_valid CTA tests at a time
constexpr int kKernelClasses = 3;     // evolve, ssc (+radiation), finalize (pbag_kernel_class)
constexpr int kClassEvolve = PBAG_K_EVOLVE, kClassSsc = PBAG_K_SSC, kClassFinalize = PBAG_K_FINALIZE;
constexpr int kSiteSynBank = 900001;  // status site: a field outside the synchrotron bank's range

// Read-only tables of one grid (one CommonTables entry), device pointers.
// Products and reciprocals the reference recomputes every step are tabulated
// once in FP64 so that the per-step kernels use multiplications only.
struct DevGrid {
  int G, F, Gp;          // Gp: G rounded up to a multiple of 16 (padded SSC operand)
  int n_cyc;             // number of bins with e[j] <= 2 (cyclotron branch of cycSynch)
  int scan_fp64;         // Chang-Cooper substeps in FP64 only (PBAG_SCAN_FP64=1), else double-float first
  int sys_min_sub;       // substep count from which the solve is the systolic pipeline (PBAG_SYSTOLIC_MIN)
  int evolve_ctas;       // evolve CTAs per SM for large batches: 4, 6 or 8 (PBAG_EVOLVE_CTAS)
  double dlog_gam;       // (e[1]-e[0])/e[0] (microphysics.h:413)
  const double* e;       // [G]   gamma grid e[i] = step^i
  const double* inv_e;   // [G]   1/e
  const double* inv_e2;  // [G]   1/e^2 (f/e/e of computeSSA, numeric_model.h:195)
  const double* de;      // [G-1] e[j+1]-e[j]
  const double* e2de;    // [G-1] e_j^2 (e_{j+1}-e_j) (numeric_model.h:208)
  const double* inv_dxm; // [G]   1/(e_i - e_{i-1}) (base_state.h:492), 0 at i=0
  const double* half2;   // [G-1] half grid squared (numeric_model.h:374)
  const double* hadi;    // [G-1] (half^2-1)/(3 half) (numeric_model.h:383)
  const double* ihalf2;  // [G-1] 1/half^2 (numeric_model.h:400)
  const double* inv_dgb; // [G]   1/delta_grid_bar (numeric_model.h:556)
  const float* ginv2;    // [G]   1/e[j]^2 (FP32, synchrotron argument)
  const float* psq32;    // [G]   e[j]^2 - 1 in FP32 (cyclotron branch)
  const float* lnginv2;  // [G]   ln(1/e[j]^2): argument of the tabulated synchrotron functions
  const float* syntab;   // [3][kSynTabN] g(u) of the GSL, Bessel and Aharonian functions (pbag_syntab.cpp)
  const float* lnnu;     // [F]   ln nu
  float syn_u0, syn_ih;  // first u of syntab and the inverse spacing
  int syn_n;             // points of each table (zero after them)
  const float2* syntab2; // [3][kSynTab2N] value / slope pairs of the same functions (batch sums)
  float syn2_u0, syn2_ih;
  int syn2_n;
  float gsl_xs;          // the GSL method's argument over nu / nu_crit (kernels.h:282-285)
  // pair production (numeric_model.h:295-356): FP32 tables of the rate kernel
  const float* ppinjT;   // [F][Gs] R(nu1_i, nu_k) (nu_{k+1} - nu_k), k < F-1 (nu1_i = 2 e_i m_e c^2 / h)
  const int* ppidx;      // [G]     photon bin of nu1_i (computePPinjection's idx)
  const float* ppabsT;   // [F][F]  R(nu_i, nu_k) (nu_{k+1} - nu_k) / c at [k][i], k < F-1
  const float* ginv23;   // [G]   e[j]^(-2/3): cube root of the 1/e^2 factor of the synchrotron argument
  const double* nu;      // [F+1] frequency grid, nu[F] = next logspace point
  const float* nu13;     // [F]   cube root of nu
  const float* nu32;     // [F]   nu in FP32
  const double* dnu_nu;  // [F]   (nu[k+1]-nu[k])/nu[k]
  const double* inv_hnu; // [F]   1/(h nu) (microphysics.h:520)
  const double* hnu;     // [F]   h nu (output scale of the SSC contraction)
  const double* ssa_nu;  // [F]   -1/(8 pi m_e nu^2) (numeric_model.h:211)
  int Gs;                // G rounded up to a multiple of 4 (row stride of KintT)
  int kint_stage;        // bytes of KintT the evolve kernel stages in shared memory (0: read from L2)
  const float* KintT;    // [F][Gs] SSC kernel integral / kscale[k] (kernels.h:79-91), k-major
  const double* kscale;  // [F]   power-of-two column scales of KintT
  const float* K32;      // [F][Gp][F] SSC kernel (i, j, k) in FP32, j >= G zero
  const uint16_t* Bt;    // SSC kernel as BF16 hi/lo tensor-core operand slabs (pbag_ssc_tc.cu), or null
  const double* etab;    // the FP64 tables of the evolve kernel in one block (GridTab), staged by one bulk copy
  int Ge, Fe;            // G and F rounded up to even (sub-table strides of etab)
  int etab_doubles;      // size of etab: kTabG * Ge + kTabF * Fe
  // grid factors as FP32 mantissa in [1, 2) times a power of two (f64_mant),
  // for products with FP64 state values computed without FP64 arithmetic:
  // tables kM32De (dgamma), kM32DeIe2 (dgamma / gamma^2), kM32DnuNu (dnu / nu)
  int Tm;                // table stride: max(G, F)
  const float* tmant;    // [3][Tm]
  const int* texp;       // [3][Tm]
  // synchrotron kernel bank of the tensor-core radiation sums (pbag_syn_tc.cu),
  // for the method class of the running batch; null: CUDA-core sums
  const uint16_t* synbank;  // [P][M/128] BF16 hi/lo operand slabs of 128 rows x Gp
  int sb_P, sb_M, sb_mlo;   // sub-shifts, bank rows, index of the first row
  int sb_tbw;               // blastwaves per weight tile (2 weight rows each)
  int sb_nlo, sb_nhi;       // shift nodes the bank covers (s / h)
  double sb_ih;             // 1 / h = P / dnu
  double sb_lnnu0;          // ln nu_0
  double sb_lnxs_gsl;       // ln of the GSL method's argument scale (gsl_xs)
};
enum : int { kM32De = 0, kM32DeIe2, kM32DnuNu, kM32 };

// Layout of DevGrid::etab: G tables at t * Ge, then F tables at kTabG * Ge + u * Fe.
enum : int {
  kTabInvE = 0, kTabInvE2, kTabDe, kTabE2de, kTabInvDxm, kTabHalf2, kTabHadi, kTabIhalf2, kTabInvDgb, kTabG
};
enum : int { kTabDnuNu = 0, kTabInvHnu, kTabKscale, kTabSsaNu, kTabF };
struct GridTab {
  const double* p;  // etab in global or shared memory
  int Ge, Fe;
  __host__ __device__ const double* gt(int t) const { return p + t * Ge; }
  __host__ __device__ const double* ft(int u) const { return p + kTabG * Ge + u * Fe; }
};

// Per-record scalars of one step, computed once for the whole batch by
// k_prep (the reference recomputes them inside each step).
struct StepScal {
  double K;          // power-law normalisation K_s / K_f (microphysics.h:237-263)
  double c_fast;     // gamma_min^(1-p) (fast-cooling lower branch)
  double Ns;         // N_inj * norm: source amplitude (numeric_model.h:718-721)
  double dt_sub;     // substep length (microphysics.h:416-431)
  double dlnVdt;     // (microphysics.h:405)
  double dr, vol;    // dr_comov and source.vol of this step
  double fac;        // (dr/c)/vol: photon-field factor (microphysics.h:517-518)
  double pref;       // synchrotron prefactor sqrt(3) q^3 B / (m_e c^2) (kernels.h:427,471)
  float inv_ncrit;   // 1 / nu_crit(B, gamma=1) (kernels.h:194-197)
  float inv_nlar;    // 1 / nu_larmor(B) (kernels.h:199-202)
  int n_sub;         // Chang-Cooper substeps; 0 = analytic distribution this step
  int flags;         // kRec* bits
  int err, site;     // error the record alone triggers (0 = none) and its check site
  int ia0, ia1;      // first branch of the analytic distribution: bins [ia0, ia1)
  int ib0, ib1;      // second branch: bins [ib0, ib1)
  int iq0, iq1;      // injection (source) bins [iq0, iq1)
  double syn_shift;  // (ln nu_crit1(B) - ln nu_0 - ln xs) / h: the bank shift of the synchrotron kernel
};

enum : int {
  kRecValid = 1,     // the blastwave is valid at this step
  kRecInit = 2,      // first valid step: initializeElectronDistribution
  kRecFast = 4,      // fast-cooling branch (gamma_min > gamma_c)
};

// Per-blastwave state that lives across steps (structure of arrays).
struct DevState {
  double* f;       // [nbw][G]   N(gamma) (ele.f)
  double* dfde;    // [nbw][G]   d(f/gamma^2)/dgamma, stateful (base_state.h:482-536)
  double* powp;    // [nbw][G]   e^-p of the blastwave's injection index
  double* gdot;    // [nbw][3][G] gam_dot_syn, _adi, _ssc (last substep)
  double* n;       // [nbw][F]   photon density total_rad.f of the previous step
  float* syn32;    // [nbw][F]   FP32 synchrotron sum of this step (scaled by the w32 scale)
  float2* ssa32;   // [nbw][F]   FP32 SSA sum and its compensation (scaled by the v32 scale)
  float* rad32;    // [nbw][4]   FP32 scalars of the radiation kernel: 1/nu_crit(B,1), 1/nu_larmor(B), cbrt(1/nu_crit)
  double* jssc;    // [nbw][F]   SSC emissivity of this step
  float* W32;      // [nbw][Gp]  SSC electron weights, scaled to FP32
  uint16_t* Abf;   // [ceil(nbw/256)][2*256*Gp] the same weights as BF16 hi/lo tensor-core operand tiles
  float* U32;      // [nbw][F]   SSC seed-photon weights, scaled to FP32
  float* w32;      // [nbw][G]   synchrotron weights f_j (e_{j+1}-e_j), scaled
  float* v32;      // [nbw][G]   SSA weights e_j^2 (e_{j+1}-e_j) dfde_j, scaled
  double* scal;    // [nbw][kScal] per-step scalars handed between kernels
  int* flags;      // [nbw]      kFlag* bits
  int* err;        // [nbw][4]   first error: code, step index, check site, unused
  // tensor-core radiation sums (null: CUDA-core sums): the synchrotron and SSA
  // weights as BF16 hi/lo operand tiles of sb_tbw blastwaves (rows 2b: w,
  // 2b+1: v), and the bank products D [tile][P][2 sb_tbw][sb_M]
  uint16_t* Sbf;
  float* Dsyn;
  // slot -> the caller's blastwave (null: the same index). Every array above
  // is indexed by slot, except powp, which follows the caller's blastwave
  // like the offsets, the parameters and the step records. A batch of uneven
  // histories runs in slots ordered by decreasing length, so that the
  // blastwaves still running at a step are a prefix of the slots and each
  // step's launches cover only that prefix.
  const int* slot_bw;
};

__device__ __forceinline__ int slot_bw(const DevState& S, int slot) { return S.slot_bw ? S.slot_bw[slot] : slot; }

// Programmatic dependent launch (griddepcontrol). A kernel launched with
// programmatic stream serialization may be scheduled before the kernels it
// depends on have finished: grid_dep_wait() returns once they have completed
// and their memory operations are visible to this grid (at once for a kernel
// launched without the attribute), so a kernel touches nothing those kernels
// read or write before it. grid_dep_launch() lets the kernels that depend on
// this one be scheduled (they still wait for its completion).
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

enum : int {
  kScalDr = 0,     // dr_comov of this step
  kScalVol = 1,    // source.vol of this step
  kScalNele = 2,   // total electron number
  kScalSW = 3,     // scale of W32 (true value = W32 * sW)
  kScalSU = 4,     // scale of U32
  kScalAcc = 5,    // accel_frac of this step
  kScalNp = 6,     // n_prime of this step
  kScalNsub = 7,   // substeps taken (diagnostic)
  kScalSw = 8,     // scale of w32
  kScalSv = 9,     // scale of v32
  kScalPref = 10,  // synchrotron prefactor of this step
  kScalB = 11,       // magnetic field of this step
  kScalSynShift = 12,  // bank shift s / h of the synchrotron kernel (tensor-core sums)
  kScalFac = 13,     // photon escape factor (dr/c)/vol (microphysics.h:517-518)
  kScalAccNe = 14,   // accel_frac / N_e
  kScalAnpNe = 15,   // accel_frac n' / N_e
  kScal = 16
};

enum : int {
  kFlagInit = 1,     // distribution initialised (is_distribution_initialized)
  kFlagActive = 2,   // blastwave radiates at the current step
  kFlagSynSeen = 4,  // a non-zero synchrotron emissivity was produced (dense check)
  kFlagUValid = 8    // U32/sU hold the previous step's photon field
};

// ---- tensor-core operand layout (pbag_ssc_tc.cu) ----------------------------
// A K-major operand of `rows` rows (output columns k of one SSC kernel slab, or
// the blastwaves of one tile) and Gp columns (gamma, a multiple of 16), with
// elements of esize bytes (2: BF16, 4: TF32), is stored in chunks of
// kTcChunk16 16-byte columns; chunk c (kc = its number of 16-byte columns)
// holds the hi part, then the lo part, each as rows/8 x kc core matrices of 8
// rows x 16 bytes, row-group major. The first n rows of a part are therefore
// its first n/8 row groups, contiguous.
constexpr int kTcCols = 256;   // blastwaves per tensor-core tile (MMA N at most)
constexpr int kTcChunk16 = 4;  // 16-byte K columns per chunk
constexpr int kTcChunk = kTcChunk16 * 8;  // BF16 K columns per chunk
__host__ __device__ inline size_t tc_operand_byte_offset(int row, int col, int rows, int Gp, int esize, bool lo) {
  const int epc = 16 / esize;  // elements per 16-byte column
  const int c = col / (kTcChunk16 * epc), kl = col % (kTcChunk16 * epc);
  const int left = Gp / epc - c * kTcChunk16;
  const int kc = left < kTcChunk16 ? left : kTcChunk16;
  return (size_t)2 * rows * kTcChunk16 * 16 * c + (lo ? (size_t)rows * kc * 16 : 0) +
         (size_t)((row >> 3) * kc + kl / epc) * 128 + (row & 7) * 16 + (kl % epc) * esize;
}
__host__ __device__ inline size_t tc_operand_offset(int row, int col, int rows, int Gp, bool lo) {
  return tc_operand_byte_offset(row, col, rows, Gp, 2, lo) / 2;
}
__host__ __device__ inline size_t tc_tile_bytes(int rows, int Gp, int esize) { return (size_t)2 * rows * Gp * esize; }
__host__ __device__ inline size_t tc_tile_elems(int rows, int Gp) { return (size_t)2 * rows * Gp; }

// Power of two close to 1/max|x| (exact rescaling); 1 when max is 0, not
// finite, or so small that the inverse would overflow.
__host__ __device__ inline double pow2_scale(double maxabs) {
  if (!(maxabs > 1.e-300) || !(maxabs < 1.e300)) return 1.;
  int ex;
  frexp(maxabs, &ex);
  return ldexp(1., -ex);
}

// ---- FP64 predicates and scales on the integer pipe -------------------------
// FP64 compares, max/min, frexp/ldexp and divisions cost hundreds of cycles
// per warp instruction on this part; these helpers read the bit pattern.

// !isfinite(v) || v < 0, as the reference's checks (-0.0 passes)
__device__ __forceinline__ bool bad_value(double v) {
  const int hi = __double2hiint(v);
  if ((hi & 0x7ff00000) == 0x7ff00000) return true;  // inf or NaN
  return hi < 0 && ((hi & 0x7fffffff) | __double2loint(v)) != 0;
}
// v > 0 for a non-NaN v
__device__ __forceinline__ bool positive(double v) {
  const int hi = __double2hiint(v);
  if ((hi & 0x7ff00000) == 0x7ff00000 && (((hi & 0xfffff) | __double2loint(v)) != 0)) return false;  // NaN
  return hi > 0 || (hi == 0 && __double2loint(v) != 0);
}
// !isfinite(v)
__device__ __forceinline__ bool not_finite(double v) { return (__double2hiint(v) & 0x7ff00000) == 0x7ff00000; }
// isnan(v)
__device__ __forceinline__ bool is_nan(double v) {
  const int hi = __double2hiint(v);
  return (hi & 0x7ff00000) == 0x7ff00000 && (((hi & 0xfffff) | __double2loint(v)) != 0);
}
// biased exponent field of |v| (0 for zero and subnormals)
__device__ __forceinline__ int exp_field(double v) { return (__double2hiint(v) >> 20) & 0x7ff; }
// pow2_scale(max) given the biased exponent E of max: 2^-(E-1022), or 1 outside
// the range where the scaled values and the inverse stay normal
__device__ __forceinline__ double scale_from_exp(int E) {
  return (E <= 26 || E >= 2019) ? 1. : __hiloint2double((2045 - E) << 20, 0);
}
// ---- FP64 values through FP32 and integer arithmetic -----------------------
// FP64 arithmetic is slow on this GPU; products of FP64 state values with grid
// factors that only need FP32 accuracy (tensor-core operands, FP32 sums) are
// formed as mantissa x power of two.
constexpr int kExpZero = -100000;  // exponent of a zero (or FP64-subnormal) value
// x = m 2^e with |m| in [1, 2) rounded to FP32 (nearest even); zero and FP64
// subnormals give m = 0, e = kExpZero; inf / NaN give m = inf / NaN, e = 0
__device__ __forceinline__ float f64_mant(double x, int& e) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long m = b & 0xfffffffffffffull;
  if (ex == 0) {
    e = kExpZero;
    return 0.f;
  }
  if (ex == 0x7ff) {
    e = 0;
    return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
  }
  unsigned long long r = m >> 29;
  const unsigned long long rem = m & 0x1fffffffull;
  if (rem > 0x10000000ull || (rem == 0x10000000ull && (r & 1ull))) ++r;
  e = ex - 1023;
  if (r == (1ull << 23)) {
    r = 0;
    ++e;
  }
  return __uint_as_float(sign | (127u << 23) | (unsigned)r);
}
// the product of two mantissas (|m| in [1, 2) each) renormalised to [1, 2),
// its exponent added to e
__device__ __forceinline__ float mant_mul(float a, float b, int& e) {
  float p = a * b;
  if (fabsf(p) >= 2.f) {
    p *= 0.5f;
    ++e;
  }
  return p;
}
// m 2^e as FP32 for |m| < 4 (or 0, inf, NaN: unchanged); below the FP32 normal
// range: zero
__device__ __forceinline__ float f32_ldexp(float m, int e) {
  const unsigned u = __float_as_uint(m);
  const int ex = (int)((u >> 23) & 0xff);
  if (ex == 0 || ex == 0xff) return m;
  const int ne = ex + e;
  if (ne <= 0) return __uint_as_float(u & 0x80000000u);
  if (ne >= 255) return __uint_as_float((u & 0x80000000u) | 0x7f800000u);
  return __uint_as_float((u & 0x807fffffu) | ((unsigned)ne << 23));
}
// m 2^e as FP64 built from the bits (m an FP32 value, finite or not), without
// FP64 arithmetic; zero below the FP64 normal range
__device__ __forceinline__ double f64_from_mant(float m, int e) {
  const unsigned u = __float_as_uint(m);
  const int ex = (int)((u >> 23) & 0xff);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (ex == 0) return __longlong_as_double((long long)sign);
  if (ex == 0xff)
    return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull |
                                            ((unsigned long long)(u & 0x7fffffu) << 29)));
  const int ne = ex - 127 + e + 1023;
  if (ne <= 0) return __longlong_as_double((long long)sign);
  if (ne >= 2047) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull));
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)ne << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// 2^e in FP64, e clamped to the normal range
__device__ __forceinline__ double f64_pow2(int e) {
  e = e < -1022 ? -1022 : e > 1023 ? 1023 : e;
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// the exact inverse of scale_from_exp(E)
__device__ __forceinline__ double unscale_from_exp(int E) {
  return (E <= 26 || E >= 2019) ? 1. : __hiloint2double((E + 1) << 20, 0);
}

// ---- the synchrotron kernel bank's interpolation (pbag_syn_tc.cu) ---------
// Cubic Lagrange weights at the nodes -1, 0, 1, 2 for 0 <= r < 1.
__device__ __forceinline__ void bank_weights(float r, float (&L)[4]) {
  L[0] = -r * (r - 1.f) * (r - 2.f) * (1.f / 6.f);
  L[1] = (r + 1.f) * (r - 1.f) * (r - 2.f) * 0.5f;
  L[2] = -(r + 1.f) * r * (r - 2.f) * 0.5f;
  L[3] = (r + 1.f) * r * (r - 1.f) * (1.f / 6.f);
}
// The interpolated sum from the four node values d: in log space when all
// four have one sign (exact on the exponential tails of the synchrotron
// function, where neighbouring nodes differ by orders of magnitude and a
// linear-space cubic would swing negative), else in linear space.
__device__ __forceinline__ float bank_interp(const float (&L)[4], const float (&d)[4]) {
  const bool pos = d[0] > 0.f && d[1] > 0.f && d[2] > 0.f && d[3] > 0.f;
  const bool neg = d[0] < 0.f && d[1] < 0.f && d[2] < 0.f && d[3] < 0.f;
  if (pos || neg) {
    float lg = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a) lg = fmaf(L[a], logf(fabsf(d[a])), lg);
    const float v = expf(lg);
    return pos ? v : -v;
  }
  float v = 0.f;
#pragma unroll
  for (int a = 0; a < 4; ++a) v = fmaf(L[a], d[a], v);
  return v;
}

// ---- synchrotron kernel functions in FP32 (kernels.h) ---------------------
// All return the dimensionless shape R; the caller multiplies by the FP64
// prefactor sqrt(3) q^3 B / (m_e c^2) of kernels.h:427,434,471.

// Aharonian+2010 eq. D7 fit (kernels.h:420-427), x = nu / nu_crit, y = x^(1/3)
// (the caller forms y as a product of tabulated cube roots). Beyond x = 150
// the factor exp(-x) is below the smallest FP32 subnormal, so the value is 0
// (this also keeps x^(4/3) from overflowing for huge x).
__device__ __forceinline__ float aharonian_R32(float x, float y) {
  if (!(x <= 150.f)) return x > 150.f ? 0.f : x;  // NaN propagates
  float y2 = y * y;
  float y4 = y2 * y2;
  float num = fmaf(0.347f, y4, fmaf(2.21f, y2, 1.f));
  float den = fmaf(0.217f, y4, fmaf(1.353f, y2, 1.f));
  return 1.808f * y * rsqrtf(fmaf(3.4f, y2, 1.f)) * __fdividef(num, den) * expf(-x);
}

// Tabulated synchrotron function (GSL or Bessel method): R(x) = g(ln x)
// x^(1/3), g interpolated linearly in u = ln x; lx = ln x, x13 = x^(1/3).
__device__ __forceinline__ float tabulated_R32(const float* __restrict__ tab, float u0, float ih, int n, float lx,
                                               float x13) {
  if (!(lx == lx)) return lx;  // NaN propagates
  const float p = (lx - u0) * ih;
  if (p >= (float)(n - 1)) return 0.f;
  if (p <= 0.f) return __ldg(tab) * x13;
  const int i = (int)p;
  const float f = p - (float)i, a = __ldg(tab + i), b = __ldg(tab + i + 1);
  return fmaf(f, b - a, a) * x13;
}

// Cyclotron branch of cycSynch (kernels.h:428-435) for gamma <= 2.
__device__ __forceinline__ float cyclotron_R32(float psq, float xl) {
  return (2.f * psq) / (1.f + 3.f * psq) * expf((2.f * (1.f - xl)) / (1.f + 3.f * psq));
}

}  // namespace pbag

#endif
