// pbag_surrogate.cu - learned SSC emissivity with an exact error check.
//
// The SSC spectrum of a state (computeSSCSpectrum, numeric_model.h:247-285)
// is j_i = h nu_i sum_jk K[i][j][k] W_j U_k. Over a band of frequencies, its
// power P_b = sum_{i in b} j_i dnu_i and the power-weighted moments Q_b, R_b
// of x_i = ln nu_i - c_b (first and second) are the same bilinear form with
// the kernel slabs summed over the band: 3 x 16 exact projections, 48 instead
// of F slabs on the tensor cores (the same contraction kernel). In each band a
// baseline shape s_i ~ exp(beta x_i) matches P_b and Q_b exactly; an MLP
// (pbag_mlp, hidden layers of 256) predicts the log10 correction to it from
// the state (B, moments and shape of N(gamma), shape of the seed photon field,
// shape of the band powers, band tilts); the spectrum is scaled to the exact
// band powers. The mismatch of the predicted and exact Q and R is the
// per-state error estimate; states above the tolerance are recomputed exactly.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_kernels.h"

namespace pbag {

cudaError_t mlp_forward(pbag_mlp* net, int n, const float* X, float* Y, cudaStream_t st);
int mlp_in_dim(const pbag_mlp* net);
int mlp_out_dim(const pbag_mlp* net);
int mlp_layers(const pbag_mlp* net);
cudaError_t mlp_reserve(pbag_mlp* net, int n);

namespace {

constexpr int kNb = PBAG_SUR_BANDS;
constexpr int kNproj = PBAG_SUR_PROJ;
constexpr int kNin = PBAG_SUR_IN;
constexpr int kFeatThreads = 128;
constexpr float kFloor = -30.f;  // log10 floor of the shape features

uint16_t bf16_round(float x) {  // round to nearest even (finite inputs)
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float bf16_float(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

struct Surrogate : CtxExtension {
  int device = 0;
  int F = 0, G = 0, Gp = 0, per = 0;  // per: frequencies per band
  uint16_t* Kp = nullptr;             // projection slabs, split-BF16 operand layout (rows F)
  double* oscale = nullptr;           // [kNproj] output scales
  double* lnrel = nullptr;            // [F] ln nu_i - (centre of ln nu of its band)
  double* invdnu = nullptr;           // [F] 1 / (nu_{i+1} - nu_i)
  double* hw = nullptr;               // [kNb] half width of each band in ln nu
  float* mean = nullptr;              // [kNin] feature standardisation
  float* stdv = nullptr;
  pbag_mlp* net = nullptr;            // not owned
  float tol = 0.01f;
  int64_t generation = 0;             // bumped by every pbag_surrogate_configure
  int cap = 0;
  float* X = nullptr;                 // [cap][kNin]
  double* proj = nullptr;             // [cap][kNproj]
  float* Y = nullptr;                 // [cap][F]
  float* err = nullptr;               // [cap]
  int* fb = nullptr;                  // [cap] fallback flags (kFlagActive)
  int* nfb = nullptr;                 // fallback count
  ~Surrogate() override {
    cudaSetDevice(device);
    for (void* p : {(void*)Kp, (void*)oscale, (void*)lnrel, (void*)invdnu, (void*)hw, (void*)mean, (void*)stdv, (void*)X,
                    (void*)proj, (void*)Y, (void*)err, (void*)fb, (void*)nfb})
      cudaFree(p);
  }
  cudaError_t reserve(int n) {
    if (n <= cap) return cudaSuccess;
    for (void* p : {(void*)X, (void*)proj, (void*)Y, (void*)err, (void*)fb}) cudaFree(p);
    X = nullptr;
    proj = nullptr;
    Y = nullptr;
    err = nullptr;
    fb = nullptr;
    cap = 0;
    const size_t c = (size_t)std::max(n, 64);
    cudaError_t e;
    if ((e = cudaMalloc(&X, c * kNin * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&proj, c * kNproj * sizeof(double))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&Y, c * F * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&err, c * sizeof(float))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&fb, c * sizeof(int))) != cudaSuccess) return e;
    cap = (int)c;
    return cudaSuccess;
  }
};

// Projection slabs from the FP32 kernel tensor K32[i][j][k] (rows k of a
// slab, K-dim j), FP64 accumulation over the band, power-of-two scaled, split
// BF16; band centres and half widths in ln nu.
int build_projections(const CtxView& v, Surrogate* s) {
  const int F = v.F, Gp = v.Gp;
  std::vector<float> K32((size_t)F * Gp * F);
  std::vector<double> nu(F + 1);
  if (cudaMemcpy(K32.data(), v.dg.K32, K32.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(nu.data(), v.dg.nu, nu.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PBAG_ERR_CUDA;
  s->per = F / kNb;
  std::vector<uint16_t> Kp((size_t)kNproj * tc_tile_elems(F, Gp), 0);
  std::vector<double> osc(kNproj), lnrel(F), invdnu(F), hw(kNb);
  for (int i = 0; i < F; ++i) invdnu[i] = 1. / (nu[i + 1] - nu[i]);
  std::vector<double> slab((size_t)F * Gp);
  for (int b = 0; b < kNb; ++b) {
    const int i0 = b * s->per, i1 = i0 + s->per;
    double c = 0.;
    for (int i = i0; i < i1; ++i) c += std::log(nu[i]);
    c /= s->per;
    for (int i = i0; i < i1; ++i) lnrel[i] = std::log(nu[i]) - c;
    hw[b] = 0.5 * (std::log(nu[i1 - 1]) - std::log(nu[i0])) + 1e-300;
    for (int q = 0; q < 3; ++q) {
      std::fill(slab.begin(), slab.end(), 0.);
      double mx = 0.;
      for (int k = 0; k < F; ++k)
        for (int j = 0; j < Gp; ++j) {
          double acc = 0.;
          for (int i = i0; i < i1; ++i) {
            const double x = std::log(nu[i]) - c;
            const double wgt = nu[i] * (nu[i + 1] - nu[i]) * (q == 0 ? 1. : q == 1 ? x : x * x);
            acc += wgt * (double)K32[((size_t)i * Gp + j) * F + k];
          }
          slab[(size_t)k * Gp + j] = acc;
          mx = std::max(mx, std::fabs(acc));
        }
      // scaled so that the largest entry is ~2^96: the small kernel entries
      // that carry the spectrum's high-frequency tail stay far from the FP32 /
      // BF16 subnormal range, and the FP32 accumulations (<= 2^9 terms of
      // operands <= 1 each) stay far below overflow
      int ex = 0;
      if (mx > 0.) std::frexp(mx, &ex);
      const double sc = std::ldexp(1., 96 - ex);
      const int o = q * kNb + b;
      osc[o] = cgs::h_pl / sc;
      uint16_t* T = Kp.data() + (size_t)o * tc_tile_elems(F, Gp);
      for (int k = 0; k < F; ++k)
        for (int j = 0; j < Gp; ++j) {
          const float x = (float)(slab[(size_t)k * Gp + j] * sc);
          const uint16_t h = bf16_round(x);
          T[tc_operand_offset(k, j, F, Gp, false)] = h;
          T[tc_operand_offset(k, j, F, Gp, true)] = bf16_round(x - bf16_float(h));
        }
    }
  }
  cudaError_t e = cudaSuccess;
  auto up = [&](auto** dst, const auto& h) {
    if (e == cudaSuccess) e = cudaMalloc(dst, h.size() * sizeof(h[0]));
    if (e == cudaSuccess) e = cudaMemcpy(*dst, h.data(), h.size() * sizeof(h[0]), cudaMemcpyHostToDevice);
  };
  up(&s->Kp, Kp);
  up(&s->oscale, osc);
  up(&s->lnrel, lnrel);
  up(&s->invdnu, invdnu);
  up(&s->hw, hw);
  return e == cudaSuccess ? PBAG_OK : PBAG_ERR_CUDA;
}

// Baseline shape of one band: log10 shares s_i ~ exp(beta x_i) (normalised
// over the band's `per` frequencies) whose mean of x equals mu (Newton on
// beta; mu clamped just inside the band).
__device__ void tilt_log10_shares(const double* __restrict__ x, int per, double mu, float* out) {
  float xl[64];
  float lo = 1e30f, hi = -1e30f;
  for (int i = 0; i < per; ++i) {
    xl[i] = (float)x[i];
    lo = fminf(lo, xl[i]);
    hi = fmaxf(hi, xl[i]);
  }
  const float span = hi - lo;
  float m = fminf(fmaxf((float)mu, lo + 0.01f * span), hi - 0.01f * span);
  float beta = 0.f;
  for (int it = 0; it < 40; ++it) {
    float z = 0.f, s1 = 0.f, s2 = 0.f;
    const float ref = beta >= 0.f ? hi : lo;
    for (int i = 0; i < per; ++i) {
      const float w = __expf(beta * (xl[i] - ref));
      z += w;
      s1 += w * xl[i];
      s2 += w * xl[i] * xl[i];
    }
    const float mean = s1 / z, var = fmaxf(s2 / z - mean * mean, 1e-12f);
    beta -= (mean - m) / var;
    beta = fminf(fmaxf(beta, -400.f / span), 400.f / span);
  }
  const float ref = beta >= 0.f ? hi : lo;
  float z = 0.f;
  for (int i = 0; i < per; ++i) z += __expf(beta * (xl[i] - ref));
  const float lz = logf(z);
  for (int i = 0; i < per; ++i) out[i] = (beta * (xl[i] - ref) - lz) * 0.43429448f;
}

__device__ float block_max_f(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float r = red[0];
  for (int i = 1; i < kFeatThreads / 32; ++i) r = fmaxf(r, red[i]);
  return r;
}
__device__ float block_sum_f(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float r = 0.f;
  for (int i = 0; i < kFeatThreads / 32; ++i) r += red[i];
  return r;
}

// Feature vector of each state (one CTA per state). f, nph: rows of N(gamma)
// and of the seed photon density (strides fs, ns); B: field (stride bs); proj:
// the exact band projections. Standardised when mean/stdv are given.
__global__ void __launch_bounds__(kFeatThreads)
k_sur_features(DevGrid g, int n, const double* __restrict__ f, int fs, const double* __restrict__ nph, int ns,
               const double* __restrict__ Bv, int bs, const double* __restrict__ proj, const double* __restrict__ hw,
               const double* __restrict__ lnrel, int per, const float* __restrict__ mean,
               const float* __restrict__ stdv, float* __restrict__ X, float* __restrict__ base) {
  const int s = blockIdx.x, tid = threadIdx.x;
  const int G = g.G, F = g.F;
  __shared__ float red[kFeatThreads / 32];
  __shared__ float feat[kNin];
  const GridTab T{g.etab, g.Ge, g.Fe};
  const double* fr = f + (size_t)s * fs;
  const double* nr = nph + (size_t)s * ns;
  for (int d = tid; d < kNin; d += kFeatThreads) feat[d] = 0.f;
  // electron weights w_j = f_j dgamma_j, scaled by a power of two into FP32
  int ex = 0;
  for (int j = tid; j < G - 1; j += kFeatThreads) ex = max(ex, exp_field(fr[j] * T.gt(kTabDe)[j]));
  ex = __reduce_max_sync(0xffffffffu, ex);
  __shared__ int redi[kFeatThreads / 32];
  if ((tid & 31) == 0) redi[tid >> 5] = ex;
  __syncthreads();
  ex = max(max(redi[0], redi[1]), max(redi[2], redi[3]));
  const double sw = scale_from_exp(ex);
  float m0 = 0.f, m1 = 0.f;
  for (int j = tid; j < G - 1; j += kFeatThreads) {
    const float w = (float)(fr[j] * T.gt(kTabDe)[j] * sw);
    const float lg = logf((float)(1. / T.gt(kTabInvE)[j]));
    m0 += w;
    m1 += w * lg;
  }
  m0 = block_sum_f(m0, red);
  m1 = block_sum_f(m1, red);
  const float mu = m0 > 0.f ? m1 / m0 : 0.f;
  float c2 = 0.f, c3 = 0.f, c4 = 0.f, wmax = 0.f;
  for (int j = tid; j < G - 1; j += kFeatThreads) {
    const float w = (float)(fr[j] * T.gt(kTabDe)[j] * sw);
    const float d = logf((float)(1. / T.gt(kTabInvE)[j])) - mu;
    c2 += w * d * d;
    c3 += w * d * d * d;
    c4 += w * d * d * d * d;
    wmax = fmaxf(wmax, w);
  }
  c2 = block_sum_f(c2, red);
  c3 = block_sum_f(c3, red);
  c4 = block_sum_f(c4, red);
  wmax = block_max_f(wmax, red);
  if (tid == 0) {
    const float var = m0 > 0.f ? c2 / m0 : 0.f;
    const float sd = sqrtf(fmaxf(var, 1e-30f));
    feat[0] = log10f(fmaxf((float)Bv[(size_t)s * bs], 1e-30f));
    feat[1] = m0 > 0.f ? log10f(m0) - (float)log10(sw) : kFloor;  // log10 of the unscaled N_e
    feat[2] = mu;
    feat[3] = log10f(sd);
    feat[4] = m0 > 0.f ? c3 / m0 / (sd * sd * sd) : 0.f;
    feat[5] = m0 > 0.f ? c4 / m0 / (var * var + 1e-30f) : 0.f;
  }
  // electron shape on 24 bins
  for (int q = tid; q < 24; q += kFeatThreads) {
    const int j = (int)lrintf(q * (float)(G - 2) / 23.f);
    const float w = (float)(fr[j] * T.gt(kTabDe)[j] * sw);
    feat[102 + q] = wmax > 0.f ? fmaxf(log10f(fmaxf(w / wmax, 1e-30f)), kFloor) : kFloor;
  }
  // seed photon shape on 64 frequencies: u_k = n_k dnu_k / nu_k
  int ue = 0;
  for (int k = tid; k < F; k += kFeatThreads) ue = max(ue, exp_field(nr[k] * T.ft(kTabDnuNu)[k]));
  ue = __reduce_max_sync(0xffffffffu, ue);
  __syncthreads();
  if ((tid & 31) == 0) redi[tid >> 5] = ue;
  __syncthreads();
  ue = max(max(redi[0], redi[1]), max(redi[2], redi[3]));
  const double su = scale_from_exp(ue);
  float umax = 0.f;
  for (int k = tid; k < F; k += kFeatThreads) umax = fmaxf(umax, (float)(nr[k] * T.ft(kTabDnuNu)[k] * su));
  umax = block_max_f(umax, red);
  for (int q = tid; q < 64; q += kFeatThreads) {
    const int k = q * F / 64;
    const float u = (float)(nr[k] * T.ft(kTabDnuNu)[k] * su);
    feat[6 + q] = umax > 0.f ? fmaxf(log10f(fmaxf(u / umax, 1e-30f)), kFloor) : kFloor;
  }
  // band power shape
  if (tid < 32) {
    const double P = tid < kNb ? proj[(size_t)s * kNproj + tid] : 0.;
    double pm = P;
    for (int o = 16; o > 0; o >>= 1) pm = fmax(pm, __shfl_xor_sync(0xffffffffu, pm, o));
    if (tid < kNb) {
      feat[70 + tid] = pm > 0. ? fmaxf(log10f((float)fmax(P / pm, 1e-30)), kFloor) : kFloor;
      // tilt of the band: mean of x over its half width
      const double Q = proj[(size_t)s * kNproj + kNb + tid];
      feat[86 + tid] = P > 0. ? fminf(fmaxf((float)(Q / P / hw[tid]), -1.f), 1.f) : 0.f;
    }
  }
  // baseline log10 shares of every frequency in its band (for the training targets)
  if (base && tid < kNb) {
    const double P = proj[(size_t)s * kNproj + tid], Q = proj[(size_t)s * kNproj + kNb + tid];
    tilt_log10_shares(lnrel + tid * per, per, P > 0. ? Q / P : 0., base + (size_t)s * F + tid * per);
  }
  __syncthreads();
  for (int d = tid; d < kNin; d += kFeatThreads) {
    float x = feat[d];
    if (!(x == x) || isinf(x)) x = kFloor;
    if (mean) x = (x - mean[d]) / stdv[d];
    X[(size_t)s * kNin + d] = x;
  }
}

// Spectrum from the baseline band shapes plus the predicted log10 correction,
// scaled to the exact band powers; error estimate from the band moments Q and
// R; fallback flags.
__global__ void __launch_bounds__(kFeatThreads)
k_sur_reconstruct(int F, int n, const int* __restrict__ flags, const float* __restrict__ Y,
                  const double* __restrict__ proj, const double* __restrict__ lnrel, const double* __restrict__ invdnu,
                  const double* __restrict__ hw, float tol, int per, double* __restrict__ out, float* __restrict__ err,
                  int* __restrict__ fb, int* __restrict__ nfb) {
  const int s = blockIdx.x, tid = threadIdx.x;
  __shared__ float fr[1024];
  __shared__ double bscale[kNb], be[kNb];
  const bool live = !flags || (flags[s] & kFlagActive);
  const double* P = proj + (size_t)s * kNproj;
  if (tid < kNb) {
    const double Pb = P[tid], Qb = P[kNb + tid];
    tilt_log10_shares(lnrel + tid * per, per, Pb > 0. ? Qb / Pb : 0., fr + tid * per);
  }
  __syncthreads();
  for (int i = tid; i < F; i += kFeatThreads)
    fr[i] = exp10f(fminf(fmaxf(fr[i] + Y[(size_t)s * F + i], -30.f), 10.f));
  __syncthreads();
  if (tid < kNb) {
    const int b = tid, i0 = b * per;
    float sum = 0.f;
    double m1 = 0., m2 = 0.;
    for (int i = i0; i < i0 + per; ++i) {
      sum += fr[i];
      m1 += (double)fr[i] * lnrel[i];
      m2 += (double)fr[i] * lnrel[i] * lnrel[i];
    }
    const double Pb = P[b], Qb = P[kNb + b], Rb = P[2 * kNb + b];
    const bool ok = Pb > 0. && sum > 0.f;
    const double isum = ok ? 1. / (double)sum : 0.;
    bscale[b] = ok ? Pb * isum : 0.;
    be[b] = ok ? fabs(Pb * m1 * isum - Qb) / (Pb * hw[b]) + fabs(Pb * m2 * isum - Rb) / (Pb * hw[b] * hw[b]) : 0.;
  }
  __syncthreads();
  if (live)
    for (int i = tid; i < F; i += kFeatThreads) out[(size_t)s * F + i] = bscale[i / per] * (double)fr[i] * invdnu[i];
  if (tid == 0) {
    double ptot = 0., e = 0.;
    for (int b = 0; b < kNb; ++b) ptot += fmax(P[b], 0.);
    for (int b = 0; b < kNb; ++b) e += ptot > 0. ? fmax(P[b], 0.) / ptot * be[b] : 0.;
    const bool finite = e == e && !isinf(e);
    err[s] = finite ? (float)e : 1e30f;
    const bool back = live && (!finite || e > tol);
    fb[s] = back ? kFlagActive : 0;
    if (back) atomicAdd(nfb, 1);
  }
}

int status_of(cudaError_t e) { return e == cudaErrorMemoryAllocation ? PBAG_ERR_NOMEM : PBAG_ERR_CUDA; }

}  // namespace

// The surrogate tail shared by the batch entry point and the step: exact
// projections, features, MLP, reconstruction with error estimate, exact
// fallback. Operands: W tiles Wt, U32, scal (SW, SU) of nrows rows; f / nph /
// B rows for the features; rows with flags & kFlagActive are written to out.
cudaError_t surrogate_run(pbag_ctx* ctx, const CtxView& v, int nrows, const void* Wt, const int* flags,
                          const float* U32, const double* scal, const double* f, int fs, const double* nph, int ns,
                          const double* Bv, int bs, double* out, int* errs, cudaStream_t st) {
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  if (!sg || !sg->net) return cudaErrorInvalidValue;
  cudaError_t e = sg->reserve(nrows);
  if (e != cudaSuccess) return e;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ok(launch_ssc_tc_mode(kTcSplit, v.F, v.Gp, Wt, sg->Kp, nrows, flags, U32, scal, sg->oscale, kNproj, kNproj,
                        sg->proj, errs, st));
  k_sur_features<<<nrows, kFeatThreads, 0, st>>>(v.dg, nrows, f, fs, nph, ns, Bv, bs, sg->proj, sg->hw, sg->lnrel,
                                                  sg->per, sg->mean, sg->stdv, sg->X, nullptr);
  ok(cudaGetLastError());
  ok(mlp_forward(sg->net, nrows, sg->X, sg->Y, st));
  ok(cudaMemsetAsync(sg->nfb, 0, sizeof(int), st));
  k_sur_reconstruct<<<nrows, kFeatThreads, 0, st>>>(v.F, nrows, flags, sg->Y, sg->proj, sg->lnrel, sg->invdnu,
                                                     sg->hw, sg->tol, sg->per, out, sg->err, sg->fb, sg->nfb);
  ok(cudaGetLastError());
  // the states whose error estimate is above the tolerance, exactly
  ok(launch_ssc_tc_mode(kTcSplit, v.F, v.Gp, Wt, v.dg.Bt, nrows, sg->fb, U32, scal, v.dg.hnu, v.F, v.F, out, errs,
                        st));
  return e;
}

bool surrogate_ready(pbag_ctx* ctx) {
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  return sg && sg->net;
}

// every buffer of the surrogate path for n rows (before a graph capture)
cudaError_t surrogate_reserve(pbag_ctx* ctx, int n) {
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  if (!sg || !sg->net) return cudaErrorInvalidValue;
  cudaError_t e = sg->reserve(n);
  return e == cudaSuccess ? mlp_reserve(sg->net, n) : e;
}

int64_t surrogate_generation(pbag_ctx* ctx) {
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  return sg ? sg->generation : 0;
}

int surrogate_launches(const pbag_ctx* ctx) {
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(const_cast<pbag_ctx*>(ctx), kExtSurrogate));
  // projections, features, the MLP layers, reconstruction, exact fallback
  return sg && sg->net ? 4 + mlp_layers(sg->net) : 0;
}

}  // namespace pbag

using namespace pbag;

extern "C" {

int pbag_surrogate_configure(pbag_ctx* ctx, pbag_mlp* net, const float* mean, const float* stdv, float tol) {
  CtxView v;
  if (!ctx_view(ctx, &v)) return PBAG_ERR_ARG;
  if (!v.ssc || !v.dg.Bt || v.F % kNb != 0 || v.F > 1024) return PBAG_ERR_UNSUPPORTED;
  if (net && (mlp_in_dim(net) != kNin || mlp_out_dim(net) != v.F)) return PBAG_ERR_ARG;
  if (!(tol >= 0.f)) return PBAG_ERR_ARG;
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  if (!sg) {
    sg = new Surrogate();
    sg->device = v.device;
    sg->F = v.F;
    sg->G = v.G;
    sg->Gp = v.Gp;
    int rc = build_projections(v, sg);
    cudaError_t e = cudaMalloc(&sg->nfb, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&sg->mean, kNin * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&sg->stdv, kNin * sizeof(float));
    if (rc != PBAG_OK || e != cudaSuccess) {
      delete sg;
      return rc != PBAG_OK ? rc : status_of(e);
    }
    std::vector<float> z(kNin, 0.f), o(kNin, 1.f);
    cudaMemcpy(sg->mean, z.data(), kNin * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(sg->stdv, o.data(), kNin * sizeof(float), cudaMemcpyHostToDevice);
    ctx_set_extension(ctx, kExtSurrogate, sg);
  }
  sg->net = net;
  sg->tol = tol;
  sg->generation += 1;
  if (mean && cudaMemcpy(sg->mean, mean, kNin * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return PBAG_ERR_CUDA;
  if (stdv && cudaMemcpy(sg->stdv, stdv, kNin * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return PBAG_ERR_CUDA;
  return PBAG_OK;
}

int pbag_surrogate_features(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph,
                            float* d_x, double* d_proj, float* d_base, pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || n < 0) return PBAG_ERR_ARG;
  if (n > 0 && (!d_f || !d_B || !d_nph || (!d_x && !d_proj && !d_base))) return PBAG_ERR_ARG;
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  if (!sg) return PBAG_ERR_ARG;  // pbag_surrogate_configure first
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (n == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  DevState S{};
  const void* Wt = nullptr;
  int rc = contract_prepare(ctx, v, n, d_f, d_nph, &S, &Wt);
  if (rc != PBAG_OK) return rc;
  cudaError_t e = sg->reserve(n);
  double* proj = d_proj ? d_proj : sg->proj;
  if (e == cudaSuccess)
    e = launch_ssc_tc_mode(kTcSplit, v.F, v.Gp, Wt, sg->Kp, n, S.flags, S.U32, S.scal, sg->oscale, kNproj, kNproj,
                           proj, S.err, v.stream);
  if (e == cudaSuccess && (d_x || d_base)) {
    k_sur_features<<<n, kFeatThreads, 0, v.stream>>>(v.dg, n, d_f, v.G, d_nph, v.F, d_B, 1, proj, sg->hw, sg->lnrel,
                                                      sg->per, nullptr, nullptr, d_x ? d_x : sg->X, d_base);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return status_of(e);
  if (st) st->code = PBAG_OK;
  return PBAG_OK;
}

int pbag_surrogate_contract(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph,
                            double* d_jssc, float* d_err, int* n_fallback, pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || n < 0) return PBAG_ERR_ARG;
  if (n > 0 && (!d_f || !d_B || !d_nph || !d_jssc)) return PBAG_ERR_ARG;
  if (!surrogate_ready(ctx)) return PBAG_ERR_ARG;  // pbag_surrogate_configure with a network first
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (n_fallback) *n_fallback = 0;
  if (n == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  DevState S{};
  const void* Wt = nullptr;
  int rc = contract_prepare(ctx, v, n, d_f, d_nph, &S, &Wt);
  if (rc != PBAG_OK) return rc;
  cudaError_t e = surrogate_run(ctx, v, n, Wt, S.flags, S.U32, S.scal, d_f, v.G, d_nph, v.F, d_B, 1, d_jssc, S.err,
                                v.stream);
  auto* sg = static_cast<Surrogate*>(ctx_get_extension(ctx, kExtSurrogate));
  int nfb = 0;
  if (e == cudaSuccess && d_err) e = cudaMemcpyAsync(d_err, sg->err, n * sizeof(float), cudaMemcpyDeviceToDevice, v.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nfb, sg->nfb, sizeof(int), cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return status_of(e);
  if (n_fallback) *n_fallback = nfb;
  if (st) st->code = PBAG_OK;
  return PBAG_OK;
}

}  // extern "C"
