// pbag_contract.cu - emissivity contractions of a batch of comoving states.
//
// pbag_contract evaluates, for n given states (N(gamma), B, seed photon density),
// the synchrotron emissivity of computeSynSpectrum (numeric_model.h:148-184)
// and the SSC emissivity of computeSSCSpectrum (numeric_model.h:247-285) with
// the same device code the step uses: the FP32 synchrotron sums of the
// radiation kernel, and the SSC contraction on CUDA cores (FP32) or on the
// tensor cores in BF16, split BF16 or TF32 with FP32 accumulation. It is the
// contraction microbenchmark and a building block for callers that evolve
// N(gamma) themselves.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_kernels.h"

using namespace pbag;

namespace {

using namespace cgs;

constexpr int kPrepWarps = 8;  // states per CTA of the preparation kernel (a warp each)
constexpr int kSynBatchMin = 512;  // batches from this size on take the tabulated synchrotron sums
// synchrotron constants per unit field (kernels.h:194-202, 427, 471): the
// prefactors sqrt(3) q^3 / (m_e c^2) (CSYN) and sqrt(3) q^3 / (m_e c c)
// (Dermer09), and in FP32 4 pi m_e c / (3 q) and 2 pi m_e c / (3 q)
constexpr double kSqrt3 = 1.7320508075688772;
constexpr double kPrefCsyn = kSqrt3 * q_e * q_e * q_e / mec2;
constexpr double kPrefDer = kSqrt3 * q_e * q_e * q_e / (m_e * c_light * c_light);
constexpr float kIncrit32 = (float)((4. * M_PI * m_e * c_light) / (3. * q_e));
constexpr float kNuL32 = (float)((2. * pi_ * m_e * c_light) / (3. * q_e));

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// One warp per state: the scaled FP32 weights of the synchrotron sum and of
// the SSC contraction (and its tensor-core operand tile), the seed-photon
// weights, the per-state scalars. The same formulas as the evolve kernel's
// epilogue and the step completion (microphysics.h:498-558,
// numeric_model.h:271-277). The products of the FP64 state values with the
// grid factors are formed as FP32 mantissa times power of two (f64_mant):
// every weight keeps FP32 accuracy, each row is scaled by a power of two to a
// largest value in [1, 2), and the scale goes to the per-state scalars.
// WPL: electron bins per lane (Gp <= 32 WPL); the mantissas and exponents of
// N(gamma) stay in registers, the SSC row is staged in shared memory for the
// tile's 16-byte rows of eight consecutive bins.
template <int WPL>
__global__ void __launch_bounds__(32 * kPrepWarps)
k_contract_prep(DevGrid g, int n, const double* __restrict__ f, const double* __restrict__ Bf,
                const double* __restrict__ nph, int syn_method, int mode, int want_syn, int want_ssc, DevState S,
                unsigned char* __restrict__ Wt, pbag_shock_params* __restrict__ prm) {
  __shared__ __align__(16) float srow_all[kPrepWarps][32 * WPL];
  const int lane = threadIdx.x & 31;
  const int s = blockIdx.x * kPrepWarps + (threadIdx.x >> 5);
  if (s >= n) return;
  float* srow = srow_all[threadIdx.x >> 5];
  const int G = g.G, F = g.F;
  const double* fs = f + (size_t)s * G;
  const float* m_de = g.tmant + (size_t)kM32De * g.Tm;
  const int* e_de = g.texp + (size_t)kM32De * g.Tm;
  const float* m_w = g.tmant + (size_t)kM32DeIe2 * g.Tm;
  const int* e_w = g.texp + (size_t)kM32DeIe2 * g.Tm;
  // N(gamma) as mantissa and exponent (bin lane + 32 q), and the largest
  // exponents of f_j dgamma_j and f_j dgamma_j / gamma_j^2
  float mf[WPL];
  int ef[WPL];
  int wexp = kExpZero, Wexp = kExpZero;
#pragma unroll
  for (int q = 0; q < WPL; ++q) {
    const int j = lane + 32 * q;
    mf[q] = 0.f;
    ef[q] = kExpZero;
    if (j < G - 1) {
      mf[q] = f64_mant(__ldg(fs + j), ef[q]);
      if (mf[q] != 0.f) {
        int e1 = ef[q] + __ldg(e_de + j), e2 = ef[q] + __ldg(e_w + j);
        mant_mul(mf[q], __ldg(m_de + j), e1);
        mant_mul(mf[q], __ldg(m_w + j), e2);
        wexp = max(wexp, e1);
        Wexp = max(Wexp, e2);
      }
    }
  }
  wexp = __reduce_max_sync(0xffffffffu, wexp);
  Wexp = __reduce_max_sync(0xffffffffu, Wexp);
  if (wexp == kExpZero) wexp = 0;
  if (Wexp == kExpZero) Wexp = 0;
  double* scal = S.scal + (size_t)s * kScal;
  if (want_syn) {
    float* w32 = S.w32 + (size_t)s * G;
    // the tensor-core synchrotron sums (pbag_syn_tc.cu): one BF16 hi / lo
    // weight row per state, tiles of 2 sb_tbw states
    const int tb1 = 2 * g.sb_tbw;
    uint16_t* Sb = S.Sbf ? S.Sbf + (size_t)(s / tb1) * tc_tile_elems(tb1, g.Gp) : nullptr;
#pragma unroll
    for (int q = 0; q < WPL; ++q) {
      const int j = lane + 32 * q;
      if (j < G) {
        float w = 0.f;
        if (j < G - 1) {
          int e = ef[q] + __ldg(e_de + j);
          w = f32_ldexp(mant_mul(mf[q], __ldg(m_de + j), e), e - wexp);
        }
        w32[j] = w;
        if (Sb) {
          const __nv_bfloat16 hi = __float2bfloat16_rn(w);
          Sb[tc_operand_offset(s % tb1, j, tb1, g.Gp, false)] = __bfloat16_as_ushort(hi);
          Sb[tc_operand_offset(s % tb1, j, tb1, g.Gp, true)] =
              __bfloat16_as_ushort(__float2bfloat16_rn(w - __bfloat162float(hi)));
        }
      }
    }
  }
  if (want_ssc) {
    const int Gp = g.Gp;
    const int m = s % kTcCols;
    unsigned char* tile = Wt ? Wt + (size_t)(s / kTcCols) * tc_tile_bytes(kTcCols, Gp, mode == kTcTf32 ? 4 : 2)
                             : nullptr;
    // the SSC weights of the row: to the FP32 rows (CUDA-core contraction) or
    // through shared memory to the tensor-core tile
    float* W = S.W32 + (size_t)s * Gp;
#pragma unroll
    for (int q = 0; q < WPL; ++q) {
      const int j = lane + 32 * q;
      if (j < Gp) {
        float w = 0.f;
        if (j < G - 1) {
          int e = ef[q] + __ldg(e_w + j);
          w = f32_ldexp(mant_mul(mf[q], __ldg(m_w + j), e), e - Wexp);
        }
        if (tile)
          srow[j] = w;
        else
          W[j] = w;
      }
    }
    __syncwarp();
    if (tile && mode == kTcTf32) {
      for (int j = lane; j < Gp; j += 32)
        *reinterpret_cast<float*>(tile + tc_operand_byte_offset(m, j, kTcCols, Gp, 4, false)) = tf32_rna(srow[j]);
    } else if (tile) {
      // eight consecutive K columns of a row are one 16-byte row of a core
      // matrix: hi and lo parts written as 16-byte words
      for (int q = lane; q < Gp / 8; q += 32) {
        const float4 a = *reinterpret_cast<const float4*>(srow + 8 * q);
        const float4 b = *reinterpret_cast<const float4*>(srow + 8 * q + 4);
        const float wv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float w0 = wv[2 * e], w1 = wv[2 * e + 1];
          const __nv_bfloat16 h0 = __float2bfloat16_rn(w0), h1 = __float2bfloat16_rn(w1);
          const __nv_bfloat16 l0 = __float2bfloat16_rn(w0 - __bfloat162float(h0));
          const __nv_bfloat16 l1 = __float2bfloat16_rn(w1 - __bfloat162float(h1));
          hi[e] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
          lo[e] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        }
        *reinterpret_cast<uint4*>(tile + tc_operand_byte_offset(m, 8 * q, kTcCols, Gp, 2, false)) =
            make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(tile + tc_operand_byte_offset(m, 8 * q, kTcCols, Gp, 2, true)) =
            make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
    }
    // seed-photon weights n_k (nu_{k+1}-nu_k)/nu_k (microphysics.h:516-523 feeds them to numeric_model.h:271)
    const double* ns = nph + (size_t)s * F;
    const float* m_u = g.tmant + (size_t)kM32DnuNu * g.Tm;
    const int* e_u = g.texp + (size_t)kM32DnuNu * g.Tm;
    int uexp = kExpZero;
    for (int k = lane; k < F; k += 32) {
      int e;
      const float mn = f64_mant(ns[k], e);
      e += e_u[k];
      mant_mul(mn, m_u[k], e);
      if (mn != 0.f) uexp = max(uexp, e);
    }
    uexp = __reduce_max_sync(0xffffffffu, uexp);
    if (uexp == kExpZero) uexp = 0;
    float* U = S.U32 + (size_t)s * F;
    for (int k = lane; k < F; k += 32) {
      int e;
      const float mn = f64_mant(ns[k], e);
      e += e_u[k];
      U[k] = f32_ldexp(mant_mul(mn, m_u[k], e), e - uexp);
    }
    if (lane == 0) {
      scal[kScalSW] = 3. / 4. * sigma_T * c_light * f64_pow2(Wexp);
      scal[kScalSU] = f64_pow2(uexp);
    }
  }
  if (lane == 0) {
    // synchrotron kernel constants (kernels.h:194-202, 427, 471)
    const double B = want_syn ? Bf[s] : 1.;
    const bool mcc = syn_method == PBAG_SYN_DER09 || syn_method == PBAG_SYN_BESSEL;
    scal[kScalPref] = (mcc ? kPrefDer : kPrefCsyn) * B;
    scal[kScalSw] = f64_pow2(wexp);
    const float Bf32 = (float)B;
    const float incrit = kIncrit32 / Bf32;
    float* rp = S.rad32 + (size_t)s * 4;
    rp[0] = incrit;
    rp[1] = kNuL32 / Bf32;
    rp[2] = cbrtf(incrit);
    rp[3] = 0.f;
    S.flags[s] = kFlagActive;
    for (int q = 0; q < 4; ++q) S.err[4 * s + q] = 0;
    if (want_syn && S.Sbf) {  // the state's shift against the synchrotron bank
      const double lxs = syn_method == PBAG_SYN_GSL ? g.sb_lnxs_gsl : 0.;
      const double sh = (log((3. * q_e * B) / (4. * M_PI * m_e * c_light)) - g.sb_lnnu0 - lxs) * g.sb_ih;
      scal[kScalSynShift] = sh;
      const double nn = floor(sh);
      if (!(B > 0) || !(nn - 1. >= (double)g.sb_nlo && nn + 2. <= (double)g.sb_nhi)) {
        S.err[4 * s] = PBAG_ERR_UNSUPPORTED;
        S.err[4 * s + 2] = kSiteSynBank;
      }
    }
    pbag_shock_params p{};
    p.syn_method = syn_method;
    p.ssc_on = want_ssc;
    prm[s] = p;
  }
}

template <typename... A>
void launch_prep(int Gp, int blocks, cudaStream_t st, A... args) {
  if (Gp <= 32 * 8)
    k_contract_prep<8><<<blocks, 32 * kPrepWarps, 0, st>>>(args...);
  else
    k_contract_prep<32><<<blocks, 32 * kPrepWarps, 0, st>>>(args...);
}

// Synchrotron sums of a large batch (computeSynSpectrum, numeric_model.h:
// 148-184, kernel values of kernels.h:414-538): one warp per (state, 8
// frequencies), lanes over gamma; the synchrotron function is interpolated
// from its FP64-built table (g(u) = R(e^u) e^(-u/3) on a uniform grid in
// u = ln x, staged in shared memory once per persistent CTA) instead of
// evaluating the fit per term: x = a_k / gamma^2 gives u = ln a_k + ln(1 /
// gamma^2) from two tables, and x^(1/3) = a_k^(1/3) gamma^(-2/3). The
// cyclotron branch of CSYN (gamma <= 2) is evaluated directly.
constexpr int kSbWarps = 8;  // warps of a CTA
constexpr int kSbF = 8;      // frequencies of a warp's work item
constexpr int kSbBlocksPerSm = 3;
inline size_t syn_batch_smem(int G) { return (size_t)kSynTab2N * 8 + (size_t)2 * G * 4; }

__global__ void __launch_bounds__(32 * kSbWarps)
k_syn_batch(DevGrid g, DevState S, int method, int items) {
  extern __shared__ float2 sb_smem[];
  float2* tab = sb_smem;  // value / slope pairs
  float* lng = reinterpret_cast<float*>(tab + kSynTab2N);
  float* g23 = lng + g.G;
  __shared__ float cst[kSbWarps][3][kSbF];  // per warp item: ln a_k, a_k^(1/3), nu_k / nu_L
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = g.G, F = g.F;
  const float2* src =
      g.syntab2 + (method == PBAG_SYN_GSL ? 0 : method == PBAG_SYN_BESSEL ? kSynTab2N : 2 * kSynTab2N);
  for (int i = tid; i < kSynTab2N; i += blockDim.x) tab[i] = src[i];
  const float ih = g.syn2_ih, u0 = g.syn2_u0;
  for (int j = tid; j < G; j += blockDim.x) {
    lng[j] = g.lnginv2[j] * ih;  // table positions
    g23[j] = g.ginv23[j];
  }
  __syncthreads();
  const float xs = method == PBAG_SYN_GSL ? g.gsl_xs : 1.f;
  const float lxs = logf(xs), cxs = cbrtf(xs);
  const int jcyc = method == PBAG_SYN_CSYN ? g.n_cyc : 0;
  const int last = g.syn2_n - 1;
  const int nfb = (F + kSbF - 1) / kSbF;
  constexpr float kRound = 12582912.f;  // 1.5 2^23: x + kRound rounds x to an integer in the mantissa
  for (int item = blockIdx.x * kSbWarps + warp; item < items; item += gridDim.x * kSbWarps) {
    const int b = item / nfb, k0 = (item % nfb) * kSbF;
    const float4 rp = *reinterpret_cast<const float4*>(S.rad32 + (size_t)b * 4);  // incrit, inlar, cbrt(incrit)
    if (lane < kSbF) {
      const int k = min(k0 + lane, F - 1);
      cst[warp][0][lane] = (g.lnnu[k] + logf(rp.x) + lxs - u0) * ih;  // table position of ln a_k
      cst[warp][1][lane] = g.nu13[k] * rp.z * cxs;
      cst[warp][2][lane] = g.nu32[k] * rp.y;
    }
    __syncwarp();
    float acc[kSbF], la[kSbF], y13[kSbF], xl[kSbF];
#pragma unroll
    for (int q = 0; q < kSbF; ++q) {
      acc[q] = 0.f;
      la[q] = cst[warp][0][q];
      y13[q] = cst[warp][1][q];
      xl[q] = cst[warp][2][q];
    }
    const float* w = S.w32 + (size_t)b * G;
    for (int j = lane; j < G - 1; j += 32) {
      const float wj = __ldg(w + j);
      if (j < jcyc) {
        const float psq = __ldg(g.psq32 + j);
#pragma unroll
        for (int q = 0; q < kSbF; ++q) acc[q] = fmaf(cyclotron_R32(psq, xl[q]), wj, acc[q]);
      } else {
        const float lg = lng[j], gw = g23[j] * wj;
#pragma unroll
        for (int q = 0; q < kSbF; ++q) {
          // nearest table point i (clamped: below the table the first, flat
          // point; from the last point on zero) and the offset from it
          const float p = la[q] + lg;
          const float r = p + kRound;
          const int i = min(max(__float_as_int(r) - __float_as_int(kRound), 0), last);
          const float f = p - (r - kRound);  // offset from the nearest point (unused where clamped: slope 0)
          const float2 t = tab[i];
          acc[q] = fmaf(fmaf(f, t.y, t.x) * y13[q], gw, acc[q]);
        }
      }
    }
    float mine = 0.f;
#pragma unroll
    for (int q = 0; q < kSbF; ++q) {
      float v = acc[q];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == q) mine = v;
    }
    if (lane < kSbF && k0 + lane < F) S.syn32[(size_t)b * F + k0 + lane] = mine;
    __syncwarp();  // the item's constants are read before the next item writes them
  }
}

cudaError_t launch_syn_batch(const DevGrid& g, const DevState& S, int n, int method, cudaStream_t st) {
  static int sms = 0;
  static bool attr = false;
  if (!attr) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(k_syn_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)syn_batch_smem(PBAG_MAX_BINS));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int items = n * ((g.F + kSbF - 1) / kSbF);
  const int blocks = std::max(1, std::min((items + kSbWarps - 1) / kSbWarps, kSbBlocksPerSm * std::max(sms, 1)));
  k_syn_batch<<<blocks, 32 * kSbWarps, syn_batch_smem(g.G), st>>>(g, S, method, items);
  return cudaGetLastError();
}

// j_syn from the FP32 sums: prefactor and scale (numeric_model.h:148-184);
// j_syn[F-1] = 0. A negative or non-finite value is the reference's exit.
// With the tensor-core sums (S.Dsyn): the cubic interpolation over the
// state's four bank nodes (pbag_syn_tc.cu) plus CSYN's cyclotron bins.
__global__ void k_contract_syn_out(int n, int F, DevGrid g, DevState S, int syn_method, double* __restrict__ jsyn) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * F) return;
  const int s = (int)(idx / F), k = (int)(idx - (int64_t)s * F);
  const double* scal = S.scal + (size_t)s * kScal;
  float sum;
  if (S.Dsyn) {
    const double shd = scal[kScalSynShift];
    const double fl = floor(shd);
    const int nn = (int)fl;
    float L[4], d[4];
    bank_weights((float)(shd - fl), L);
    const int tb1 = 2 * g.sb_tbw, M = g.sb_M, Pb = g.sb_P;
    const float* Dt = S.Dsyn + ((size_t)(s / tb1) * Pb * tb1 + s % tb1) * M;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int na = nn - 1 + a;
      const int qa = na >= 0 ? na / Pb : -((-na + Pb - 1) / Pb);
      d[a] = Dt[(size_t)(na - qa * Pb) * tb1 * M + k - qa - g.sb_mlo];
    }
    sum = fmaxf(bank_interp(L, d), 0.f);
    if (syn_method == PBAG_SYN_CSYN) {
      const float xl = g.nu32[k] * S.rad32[(size_t)s * 4 + 1];
      for (int j = 0; j < g.n_cyc; ++j) sum = fmaf(cyclotron_R32(g.psq32[j], xl), S.w32[(size_t)s * g.G + j], sum);
    }
  } else {
    sum = S.syn32[idx];
  }
  const double js = k < F - 1 ? scal[kScalPref] * ((double)sum * scal[kScalSw]) : 0.;
  jsyn[idx] = js;
  if (bad_value(js) && atomicCAS(&S.err[4 * s], 0, PBAG_ERR_NONFINITE) == 0) S.err[4 * s + 2] = __LINE__;
}

// The first failing state (smallest index with an error code): every state
// checked in parallel, the minimum index kept in out[3] (set to a value >= n
// before), then code, index and site into out[0..2].
__global__ void k_contract_fail_scan(const int* __restrict__ err, int n, int* __restrict__ out) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    if (err[4 * s] != 0) atomicMin(&out[3], s);
}
__global__ void k_contract_fail_pick(const int* __restrict__ err, int n, int* __restrict__ out) {
  const int s = out[3];
  const bool any = s >= 0 && s < n;  // an index outside [0, n): no state failed
  out[0] = any ? err[4 * s] : PBAG_OK;
  out[1] = any ? s : -1;
  out[2] = any ? err[4 * s + 2] : 0;
}

// Per-context workspace of pbag_contract, grown on demand.
struct ContractWs : CtxExtension {
  int device = 0;
  int cap = 0;
  int cap_mode = -1;
  DevState S{};
  unsigned char* Wt = nullptr;
  pbag_shock_params* prm = nullptr;
  int* fail = nullptr;
  float* bt32 = nullptr;  // kernel slabs as TF32 operands, built on first use
  std::vector<void*> mem;
  ~ContractWs() override {
    cudaSetDevice(device);
    for (void* p : mem) cudaFree(p);
    cudaFree(bt32);
  }
  template <typename T>
  cudaError_t take(T** p, size_t count) {
    *p = nullptr;
    if (!count) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e == cudaSuccess) mem.push_back(*p);
    return e;
  }
  cudaError_t reserve(int n, int mode, const CtxView& v) {
    if (n <= cap && mode == cap_mode) return cudaSuccess;
    for (void* p : mem) cudaFree(p);
    mem.clear();
    S = DevState{};
    cap = 0;
    const size_t c = (size_t)std::max(n, 64);
    const size_t rows = (c + kTcCols - 1) / kTcCols * kTcCols;  // whole tensor-core tiles
    cudaError_t e;
    if ((e = take(&S.w32, c * v.G)) != cudaSuccess) return e;
    S.v32 = S.w32;  // no SSA here
    if ((e = take(&S.W32, c * v.Gp)) != cudaSuccess) return e;
    if ((e = take(&S.U32, rows * v.F)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(S.U32, 0, rows * v.F * sizeof(float), v.stream)) != cudaSuccess) return e;
    if ((e = take(&S.syn32, c * v.F)) != cudaSuccess) return e;
    if ((e = take(&S.ssa32, c * v.F)) != cudaSuccess) return e;
    if ((e = take(&S.rad32, c * 4)) != cudaSuccess) return e;
    if ((e = take(&S.scal, c * kScal)) != cudaSuccess) return e;
    if ((e = take(&S.flags, c)) != cudaSuccess) return e;
    if ((e = take(&S.err, c * 4)) != cudaSuccess) return e;
    if ((e = take(&prm, c)) != cudaSuccess) return e;
    if ((e = take(&fail, 4)) != cudaSuccess) return e;
    const size_t wt = rows / kTcCols * tc_tile_bytes(kTcCols, v.Gp, mode == kTcTf32 ? 4 : 2);
    if ((e = take(&Wt, wt)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(Wt, 0, wt, v.stream)) != cudaSuccess) return e;
    if (v.dg.sb_tbw > 0) {  // the tensor-core synchrotron sums: one weight row per state
      const int tb1 = 2 * v.dg.sb_tbw;
      const size_t tiles = (c + tb1 - 1) / tb1;
      if ((e = take(&S.Sbf, tiles * tc_tile_elems(tb1, v.Gp))) != cudaSuccess) return e;
      if ((e = cudaMemsetAsync(S.Sbf, 0, tiles * tc_tile_elems(tb1, v.Gp) * 2, v.stream)) != cudaSuccess) return e;
      if ((e = take(&S.Dsyn, tiles * (size_t)v.dg.sb_P * tb1 * v.dg.sb_M)) != cudaSuccess) return e;
    }
    cap = (int)c;
    cap_mode = mode;
    return cudaSuccess;
  }
};

int cuda_status(cudaError_t e) { return e == cudaErrorMemoryAllocation ? PBAG_ERR_NOMEM : PBAG_ERR_CUDA; }

}  // namespace

namespace pbag {
// The contraction workspace of the context, reserved for n states, and the
// split-BF16 operands (W tiles, U32, scales) of the states f / nph: the first
// part of pbag_contract, shared with the surrogate.
int contract_prepare(pbag_ctx* ctx, const CtxView& v, int n, const double* d_f, const double* d_nph, DevState* S,
                     const void** Wt) {
  auto* ws = static_cast<ContractWs*>(ctx_get_extension(ctx, kExtContract));
  if (!ws) {
    ws = new ContractWs();
    ws->device = v.device;
    ctx_set_extension(ctx, kExtContract, ws);
  }
  cudaError_t e = ws->reserve(n, kTcSplit, v);
  if (e != cudaSuccess) return cuda_status(e);
  *S = ws->S;
  *Wt = ws->Wt;
  launch_prep(v.dg.Gp, (n + kPrepWarps - 1) / kPrepWarps, v.stream, v.dg, n, d_f, (const double*)nullptr, d_nph,
              (int)PBAG_SYN_CSYN, (int)kTcSplit, 0, 1, ws->S, ws->Wt, ws->prm);
  return cudaGetLastError() == cudaSuccess ? PBAG_OK : PBAG_ERR_CUDA;
}
}  // namespace pbag

namespace {
int contract_run(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph, int syn_method,
                 int precision, double* d_jsyn, double* d_jssc, pbag_status* st, bool bank_ok);
}

extern "C" int pbag_contract(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph,
                             int syn_method, int precision, double* d_jsyn, double* d_jssc, pbag_status* st) {
  pbag_status ls{};
  int rc = contract_run(ctx, n, d_f, d_B, d_nph, syn_method, precision, d_jsyn, d_jssc, &ls, true);
  // a field outside the synchrotron bank's range: the CUDA-core sums instead
  if (rc == PBAG_ERR_UNSUPPORTED && ls.site == kSiteSynBank)
    rc = contract_run(ctx, n, d_f, d_B, d_nph, syn_method, precision, d_jsyn, d_jssc, &ls, false);
  if (st) *st = ls;
  return rc;
}

namespace {
int contract_run(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph, int syn_method,
                 int precision, double* d_jsyn, double* d_jssc, pbag_status* st, bool bank_ok) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || n < 0) return PBAG_ERR_ARG;
  if (n > 0 && (!d_f || (d_jsyn && !d_B) || (d_jssc && !d_nph))) return PBAG_ERR_ARG;
  if (syn_method < PBAG_SYN_CSYN || syn_method > PBAG_SYN_BESSEL) return PBAG_ERR_ARG;
  if (precision < PBAG_PREC_FP32 || precision > PBAG_PREC_TF32) return PBAG_ERR_ARG;
  const bool tc = precision != PBAG_PREC_FP32;
  if (d_jssc && !v.ssc) return PBAG_ERR_ARG;  // the context was created without SSC tables
  if (d_jssc && tc && !v.dg.Bt) return PBAG_ERR_UNSUPPORTED;
  const int mode = precision == PBAG_PREC_TF32 ? kTcTf32 : precision == PBAG_PREC_BF16 ? kTcBf16 : kTcSplit;
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (n == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  auto* ws = static_cast<ContractWs*>(ctx_get_extension(ctx, kExtContract));
  if (!ws) {
    ws = new ContractWs();
    ws->device = v.device;
    ctx_set_extension(ctx, kExtContract, ws);
  }
  cudaError_t e = ws->reserve(n, tc && d_jssc ? mode : -1, v);
  if (e != cudaSuccess) return cuda_status(e);
  if (d_jssc && tc && mode == kTcTf32 && !ws->bt32) {
    // TF32 kernel slabs from the FP32 kernel tensor of the context
    std::vector<float> K32((size_t)v.F * v.Gp * v.F), Bt32;
    if (cudaMemcpy(K32.data(), v.dg.K32, K32.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
      return PBAG_ERR_CUDA;
    build_ssc_tc_operand_tf32(K32, v.F, v.Gp, Bt32);
    if ((e = cudaMalloc(&ws->bt32, Bt32.size() * sizeof(float))) != cudaSuccess) return cuda_status(e);
    if (cudaMemcpy(ws->bt32, Bt32.data(), Bt32.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
      return PBAG_ERR_CUDA;
  }
  cudaStream_t s = v.stream;
  DevState S = ws->S;
  S.jssc = d_jssc;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  // synchrotron sums of large batches on the tensor cores when the grid allows
  const bool fp32_ssc = d_jssc && !tc;
  DevGrid gg = v.dg;
  const bool bank = bank_ok && d_jsyn && !fp32_ssc && n >= kSynBatchMin && S.Sbf &&
                    ctx_syn_bank(ctx, syn_method, &gg);
  if (!bank) {
    S.Sbf = nullptr;
    S.Dsyn = nullptr;
  }
  launch_prep(v.dg.Gp, (n + kPrepWarps - 1) / kPrepWarps, s, gg, n, d_f, d_B, d_nph, syn_method, mode,
              d_jsyn ? 1 : 0, d_jssc ? 1 : 0, S, tc && d_jssc ? ws->Wt : (unsigned char*)nullptr, ws->prm);
  ok(cudaGetLastError());
  // synchrotron sums (and the CUDA-core SSC contraction in FP32)
  if (bank)
    ok(launch_syn_tc(gg, S, n, s, 1));  // the bank GEMM, interpolated in k_contract_syn_out
  else if (d_jsyn && !fp32_ssc && n >= kSynBatchMin)
    ok(launch_syn_batch(v.dg, S, n, syn_method, s));  // large batches: the tabulated function
  else if (d_jsyn || fp32_ssc)
    ok(launch_rad_ssc(v.dg, S, ws->prm, n, fp32_ssc, 0, s));
  if (d_jssc && tc)
    ok(launch_ssc_tc_mode(mode, v.F, v.Gp, ws->Wt, mode == kTcTf32 ? (const void*)ws->bt32 : (const void*)v.dg.Bt, n,
                          S.flags, S.U32, S.scal, v.dg.hnu, v.F, v.F, d_jssc, S.err, s));
  if (d_jsyn) {
    const int64_t tot = (int64_t)n * v.F;
    k_contract_syn_out<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, v.F, gg, S, syn_method, d_jsyn);
    ok(cudaGetLastError());
  }
  ok(cudaMemsetAsync(ws->fail + 3, 0x7f, sizeof(int), s));  // 0x7f7f7f7f: above any state index
  k_contract_fail_scan<<<(unsigned)std::min((n + 255) / 256, 1184), 256, 0, s>>>(S.err, n, ws->fail);
  k_contract_fail_pick<<<1, 1, 0, s>>>(S.err, n, ws->fail);
  ok(cudaGetLastError());
  int fail[3] = {0, -1, 0};
  ok(cudaMemcpyAsync(fail, ws->fail, sizeof(fail), cudaMemcpyDeviceToHost, s));
  ok(cudaStreamSynchronize(s));
  if (e != cudaSuccess) return cuda_status(e);
  if (st) {
    st->code = fail[0];
    st->bw = fail[1];
    st->step = fail[0] ? 0 : -1;
    st->site = fail[2];
  }
  return fail[0];
}
}  // namespace
