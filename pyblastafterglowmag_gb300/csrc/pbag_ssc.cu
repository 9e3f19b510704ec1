// pbag_ssc.cu - synchrotron self-Compton emissivity of a batch of blastwaves.
//
// computeSSCSpectrum (numeric_model.h:247-285) is, per blastwave b and output
// frequency i,
//   j_ssc[b][i] = h nu_i sum_j W[b][j] sum_k K[i][j][k] U[b][k],
//   W[b][j] = f_j (e_{j+1}-e_j) 3/4 sigma_T c / e_j^2   (j < G-1),
//   U[b][k] = n_k (nu_{k+1}-nu_k) / nu_k                (photon field of the previous step),
// with K the Blumenthal-Gould kernel of kernels.h:96-117. All factors are
// non-negative, so W and U are rescaled per blastwave by powers of two into
// FP32 range and the contraction accumulates in FP32; the scales are applied
// back in FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <thread>
#include <vector>

#include "pbag_kernels.h"

namespace pbag {

using namespace cgs;

namespace {

// kernels.h:96-117 (sscNava): isotropic Compton kernel, Nava et al. form.
double ssc_nava(double nu, double gam, double nu_tilde) {
  const double en = nu * h_by_mec2;
  const double en_t = nu_tilde * h_by_mec2;
  double K = 0.;
  if (en_t / (4. * gam * gam) < en && en <= en_t) {
    K = (en / en_t) - (1. / (4. * gam * gam));
  } else if (en_t < en && en < (4. * gam * gam * en_t / (1. + 4. * gam * en_t))) {
    const double q = en / (4. * gam * en_t * (gam - en));
    K = 2. * q * std::log(q) + (1. + 2. * q) * (1. - q) +
        .5 * (1. - q) * std::pow(4. * gam * en_t * q, 2.) / (1. + 4. * gam * en_t * q);
  }
  return K;
}

constexpr int kSscThreads = 128;
constexpr int kSscTile = 16;  // blastwaves per CTA

template <int KPT>
__global__ void __launch_bounds__(kSscThreads)
k_ssc_contract(DevGrid g, DevState S, int nbw) {
  const int i = blockIdx.x;  // output frequency
  const int b0 = blockIdx.y * kSscTile;
  const int tid = threadIdx.x;
  const int F = g.F, Gp = g.Gp;
  extern __shared__ float Ws[];  // [kSscTile][Gp]
  __shared__ float red[kSscTile][kSscThreads / 32];
  __shared__ int live[kSscTile];
  if (tid < kSscTile) {
    const int b = b0 + tid;
    live[tid] = b < nbw && (S.flags[b] & kFlagActive) ? 1 : 0;
  }
  __syncthreads();
  for (int idx = tid; idx < kSscTile * Gp; idx += kSscThreads) {
    const int bt = idx / Gp, j = idx - bt * Gp;
    Ws[idx] = live[bt] ? S.W32[(size_t)(b0 + bt) * Gp + j] : 0.f;
  }
  __syncthreads();
  float acc[kSscTile][KPT];
#pragma unroll
  for (int bt = 0; bt < kSscTile; ++bt)
#pragma unroll
    for (int q = 0; q < KPT; ++q) acc[bt][q] = 0.f;
  const float* Ki = g.K32 + (size_t)i * Gp * F;
  for (int j = 0; j < Gp; ++j) {
    float kv[KPT];
#pragma unroll
    for (int q = 0; q < KPT; ++q) {
      const int k = tid + q * kSscThreads;
      kv[q] = k < F ? __ldg(Ki + (size_t)j * F + k) : 0.f;
    }
#pragma unroll
    for (int bt = 0; bt < kSscTile; ++bt) {
      const float w = Ws[bt * Gp + j];
#pragma unroll
      for (int q = 0; q < KPT; ++q) acc[bt][q] = fmaf(w, kv[q], acc[bt][q]);
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int bt = 0; bt < kSscTile; ++bt) {
    float s = 0.f;
    const int b = b0 + bt;
    if (live[bt]) {
#pragma unroll
      for (int q = 0; q < KPT; ++q) {
        const int k = tid + q * kSscThreads;
        if (k < F) s = fmaf(acc[bt][q], S.U32[(size_t)b * F + k], s);
      }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[bt][warp] = s;
  }
  __syncthreads();
  if (tid < kSscTile && live[tid]) {
    const int b = b0 + tid;
    float s = 0.f;
    for (int w = 0; w < kSscThreads / 32; ++w) s += red[tid][w];
    const double* sc = S.scal + (size_t)b * kScal;
    S.jssc[(size_t)b * F + i] = h_pl * g.nu[i] * sc[kScalSW] * sc[kScalSU] * (double)s;
  }
}

template <int KPT>
cudaError_t launch_kpt(const DevGrid& g, const DevState& S, int nbw, cudaStream_t st) {
  const size_t smem = (size_t)kSscTile * g.Gp * sizeof(float);
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_ssc_contract<KPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSscTile * PBAG_MAX_BINS * (int)sizeof(float));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid(g.F, (nbw + kSscTile - 1) / kSscTile);
  k_ssc_contract<KPT><<<grid, kSscThreads, smem, st>>>(g, S, nbw);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_ssc_contract(const DevGrid& g, const DevState& S, int nbw, cudaStream_t st) {
  if (nbw <= 0) return cudaSuccess;
  const int kpt = (g.F + kSscThreads - 1) / kSscThreads;
  if (kpt <= 1) return launch_kpt<1>(g, S, nbw, st);
  if (kpt <= 2) return launch_kpt<2>(g, S, nbw, st);
  if (kpt <= 4) return launch_kpt<4>(g, S, nbw, st);
  return launch_kpt<8>(g, S, nbw, st);
}

void build_ssc_tables(const double* gam, int G, const double* freq, int F, int Gp, std::vector<double>& Kint,
                      std::vector<float>& K32) {
  std::vector<double> K((size_t)F * G * F);
  const unsigned hw = std::thread::hardware_concurrency();
  const int nth = (int)std::max(1u, std::min(hw, 16u));
  auto fill = [&](int t) {
    for (int i = t; i < F; i += nth)
      for (int j = 0; j < G; j++)
        for (int k = 0; k < F; k++) K[((size_t)i * G + j) * F + k] = ssc_nava(freq[i], gam[j], freq[k]);
  };
  std::vector<std::thread> th;
  for (int t = 0; t < nth; ++t) th.emplace_back(fill, t);
  for (auto& t : th) t.join();
  // kernels.h:79-91: integral over the scattered frequency
  Kint.assign((size_t)G * F, 0.);
  for (int j = 0; j < G; j++)
    for (int k = 0; k < F; k++) {
      double res = 0;
      for (int i = 0; i < F - 1; i++) res += K[((size_t)i * G + j) * F + k] * freq[i + 1] * (freq[i + 1] - freq[i]);
      Kint[(size_t)j * F + k] = res;
    }
  K32.assign((size_t)F * Gp * F, 0.f);
  for (int i = 0; i < F; i++)
    for (int j = 0; j < G; j++)
      for (int k = 0; k < F; k++) K32[((size_t)i * Gp + j) * F + k] = (float)K[((size_t)i * G + j) * F + k];
}

}  // namespace pbag
