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

constexpr int kPrepThreads = 128;

__device__ int block_max_exp(int v, int* red) {
  v = __reduce_max_sync(0xffffffffu, v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  int r = 0;
  for (int i = 0; i < kPrepThreads / 32; ++i) r = max(r, red[i]);
  return r;
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// One CTA per state: the scaled FP32 weights of the synchrotron sum and of the
// SSC contraction (and its tensor-core operand tile), the seed-photon weights,
// the per-state scalars. The same formulas as the evolve kernel's epilogue and
// the step completion (microphysics.h:498-558, numeric_model.h:271-277).
__global__ void __launch_bounds__(kPrepThreads)
k_contract_prep(DevGrid g, int n, const double* __restrict__ f, const double* __restrict__ Bf,
                const double* __restrict__ nph, int syn_method, int mode, int want_syn, int want_ssc, DevState S,
                unsigned char* __restrict__ Wt, pbag_shock_params* __restrict__ prm) {
  const int s = blockIdx.x, tid = threadIdx.x;
  const int G = g.G, F = g.F;
  __shared__ int red[kPrepThreads / 32];
  const GridTab T{g.etab, g.Ge, g.Fe};
  const double* fs = f + (size_t)s * G;
  const double* t_de = T.gt(kTabDe);
  const double* t_ie2 = T.gt(kTabInvE2);
  int wexp = 0, Wexp = 0;
  for (int j = tid; j < G - 1; j += kPrepThreads) {
    const double w = fs[j] * t_de[j];
    wexp = max(wexp, exp_field(w));
    Wexp = max(Wexp, exp_field(w * t_ie2[j]));
  }
  wexp = block_max_exp(wexp, red);
  Wexp = block_max_exp(Wexp, red);
  double* scal = S.scal + (size_t)s * kScal;
  if (want_syn) {
    const double sw = scale_from_exp(wexp);
    float* w32 = S.w32 + (size_t)s * G;
    for (int j = tid; j < G; j += kPrepThreads) w32[j] = j < G - 1 ? (float)(fs[j] * t_de[j] * sw) : 0.f;
  }
  if (want_ssc) {
    const double sW = scale_from_exp(Wexp);
    float* W = S.W32 + (size_t)s * g.Gp;
    const int m = s % kTcCols;
    unsigned char* tile = Wt ? Wt + (size_t)(s / kTcCols) * tc_tile_bytes(kTcCols, g.Gp, mode == kTcTf32 ? 4 : 2)
                             : nullptr;
    for (int j = tid; j < g.Gp; j += kPrepThreads) {
      const float w = j < G - 1 ? (float)(fs[j] * t_de[j] * t_ie2[j] * sW) : 0.f;
      W[j] = w;
      if (tile && mode == kTcTf32) {
        *reinterpret_cast<float*>(tile + tc_operand_byte_offset(m, j, kTcCols, g.Gp, 4, false)) = tf32_rna(w);
      } else if (tile) {
        const __nv_bfloat16 hi = __float2bfloat16_rn(w);
        const __nv_bfloat16 lo = __float2bfloat16_rn(w - __bfloat162float(hi));
        *reinterpret_cast<uint16_t*>(tile + tc_operand_byte_offset(m, j, kTcCols, g.Gp, 2, false)) =
            __bfloat16_as_ushort(hi);
        *reinterpret_cast<uint16_t*>(tile + tc_operand_byte_offset(m, j, kTcCols, g.Gp, 2, true)) =
            __bfloat16_as_ushort(lo);
      }
    }
    // seed-photon weights n_k (nu_{k+1}-nu_k)/nu_k (microphysics.h:516-523 feeds them to numeric_model.h:271)
    const double* ns = nph + (size_t)s * F;
    const double* dnu = T.ft(kTabDnuNu);
    int uexp = 0;
    for (int k = tid; k < F; k += kPrepThreads) uexp = max(uexp, exp_field(ns[k] * dnu[k]));
    uexp = block_max_exp(uexp, red);
    const double su = scale_from_exp(uexp);
    float* U = S.U32 + (size_t)s * F;
    for (int k = tid; k < F; k += kPrepThreads) U[k] = (float)(ns[k] * dnu[k] * su);
    if (tid == 0) {
      scal[kScalSW] = 3. / 4. * sigma_T * c_light * unscale_from_exp(Wexp);
      scal[kScalSU] = unscale_from_exp(uexp);
    }
  }
  if (tid == 0) {
    // synchrotron kernel constants (kernels.h:194-202, 427, 471)
    const double B = want_syn ? Bf[s] : 1.;
    const bool dermer = syn_method == PBAG_SYN_DER09;
    const double sqrt3 = 1.7320508075688772;
    scal[kScalPref] = dermer ? sqrt3 * pow(q_e, 3.) * B / (m_e * c_light * c_light) : sqrt3 * pow(q_e, 3.) * B / mec2;
    scal[kScalSw] = unscale_from_exp(wexp);
    const float incrit = (float)((4. * M_PI * m_e * c_light) / (3. * q_e * B));
    float* rp = S.rad32 + (size_t)s * 4;
    rp[0] = incrit;
    rp[1] = (float)((2. * pi_ * m_e * c_light) / (3. * q_e * B));
    rp[2] = cbrtf(incrit);
    rp[3] = 0.f;
    S.flags[s] = kFlagActive;
    for (int q = 0; q < 4; ++q) S.err[4 * s + q] = 0;
    pbag_shock_params p{};
    p.syn_method = syn_method;
    p.ssc_on = want_ssc;
    prm[s] = p;
  }
}

// j_syn from the FP32 sums: prefactor and scale (numeric_model.h:148-184);
// j_syn[F-1] = 0. A negative or non-finite value is the reference's exit.
__global__ void k_contract_syn_out(int n, int F, DevState S, double* __restrict__ jsyn) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * F) return;
  const int s = (int)(idx / F), k = (int)(idx - (int64_t)s * F);
  const double* scal = S.scal + (size_t)s * kScal;
  const double js = k < F - 1 ? scal[kScalPref] * ((double)S.syn32[idx] * scal[kScalSw]) : 0.;
  jsyn[idx] = js;
  if (bad_value(js) && atomicCAS(&S.err[4 * s], 0, PBAG_ERR_NONFINITE) == 0) S.err[4 * s + 2] = __LINE__;
}

__global__ void k_contract_first_failure(const int* __restrict__ err, int n, int* __restrict__ out) {
  __shared__ int best[256];
  int b = INT_MAX;
  for (int s = threadIdx.x; s < n; s += blockDim.x)
    if (err[4 * s] != 0) b = min(b, s);
  best[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) best[threadIdx.x] = min(best[threadIdx.x], best[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int s = best[0];
    out[0] = s == INT_MAX ? PBAG_OK : err[4 * s];
    out[1] = s == INT_MAX ? -1 : s;
    out[2] = s == INT_MAX ? 0 : err[4 * s + 2];
  }
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
  k_contract_prep<<<n, kPrepThreads, 0, v.stream>>>(v.dg, n, d_f, nullptr, d_nph, PBAG_SYN_CSYN, kTcSplit, 0, 1,
                                                     ws->S, ws->Wt, ws->prm);
  return cudaGetLastError() == cudaSuccess ? PBAG_OK : PBAG_ERR_CUDA;
}
}  // namespace pbag

extern "C" int pbag_contract(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph,
                             int syn_method, int precision, double* d_jsyn, double* d_jssc, pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || n < 0) return PBAG_ERR_ARG;
  if (n > 0 && (!d_f || (d_jsyn && !d_B) || (d_jssc && !d_nph))) return PBAG_ERR_ARG;
  if (syn_method != PBAG_SYN_CSYN && syn_method != PBAG_SYN_DER09) return PBAG_ERR_UNSUPPORTED;
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
  k_contract_prep<<<n, kPrepThreads, 0, s>>>(v.dg, n, d_f, d_B, d_nph, syn_method, mode, d_jsyn ? 1 : 0,
                                              d_jssc ? 1 : 0, S, tc && d_jssc ? ws->Wt : nullptr, ws->prm);
  ok(cudaGetLastError());
  // synchrotron sums (and the CUDA-core SSC contraction in FP32)
  const bool fp32_ssc = d_jssc && !tc;
  if (d_jsyn || fp32_ssc) ok(launch_rad_ssc(v.dg, S, ws->prm, n, fp32_ssc, 0, s));
  if (d_jssc && tc)
    ok(launch_ssc_tc_mode(mode, v.F, v.Gp, ws->Wt, mode == kTcTf32 ? (const void*)ws->bt32 : (const void*)v.dg.Bt, n,
                          S.flags, S.U32, S.scal, v.dg.hnu, v.F, v.F, d_jssc, S.err, s));
  if (d_jsyn) {
    const int64_t tot = (int64_t)n * v.F;
    k_contract_syn_out<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(n, v.F, S, d_jsyn);
    ok(cudaGetLastError());
  }
  k_contract_first_failure<<<1, 256, 0, s>>>(S.err, n, ws->fail);
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
