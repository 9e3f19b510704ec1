// pbag_ssc.cuh - CUDA-core SSC contraction tile (device code, included by the
// step kernels).
//
// computeSSCSpectrum (numeric_model.h:247-285) is, per blastwave b and output
// frequency i,
//   j_ssc[b][i] = h nu_i sum_j W[b][j] sum_k K[i][j][k] U[b][k],
//   W[b][j] = f_j (e_{j+1}-e_j) 3/4 sigma_T c / e_j^2   (j < G-1),
//   U[b][k] = n_k (nu_{k+1}-nu_k) / nu_k                (photon field of the previous step),
// with K the Blumenthal-Gould kernel of kernels.h:96-117. All factors are
// non-negative, so W and U are rescaled per blastwave by powers of two into
// FP32 range and the contraction accumulates in FP32; the scales are applied
// back in FP64. One tile = one output frequency i for kSscTile blastwaves;
// thread t owns frequencies k = t, t+128, ... of the inner sum.
#ifndef PBAG_SSC_CUH
#define PBAG_SSC_CUH

#include "pbag_device.cuh"

namespace pbag {

constexpr int kSscThreads = 128;
constexpr int kSscTile = 16;  // blastwaves per tile
constexpr int kSscUnroll = 8; // gamma bins loaded ahead (Gp is a multiple of 16)

__host__ __device__ inline int ssc_block_count(const DevGrid& g, int nbw) {
  return g.F * ((nbw + kSscTile - 1) / kSscTile);
}
__host__ __device__ inline int ssc_smem_bytes(const DevGrid& g) { return kSscTile * g.Gp * (int)sizeof(float); }
__host__ __device__ inline int ssc_smem_max_bytes() {
  return kSscTile * ((PBAG_MAX_BINS + 15) / 16 * 16) * (int)sizeof(float);
}

template <int KPT>
__device__ void ssc_block(const DevGrid& g, const DevState& S, int nbw, int tile) {
  const int tid = threadIdx.x;
  const int F = g.F, Gp = g.Gp;
  const int i = tile % F;
  const int b0 = (tile / F) * kSscTile;
  extern __shared__ float Ws[];  // [kSscTile][Gp]
  __shared__ float red[kSscTile][kSscThreads / 32];
  __shared__ int live[kSscTile];
  if (tid < kSscTile) {
    const int b = b0 + tid;
    live[tid] = b < nbw && (S.flags[b] & kFlagActive) ? 1 : 0;
  }
  __syncthreads();
  int any = 0;
  for (int t = 0; t < kSscTile; ++t) any |= live[t];
  if (!any) return;
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
  for (int j0 = 0; j0 < Gp; j0 += kSscUnroll) {
    float kv[kSscUnroll][KPT];
#pragma unroll
    for (int u = 0; u < kSscUnroll; ++u)
#pragma unroll
      for (int q = 0; q < KPT; ++q) {
        const int k = tid + q * kSscThreads;
        kv[u][q] = k < F ? __ldg(Ki + (size_t)(j0 + u) * F + k) : 0.f;
      }
#pragma unroll
    for (int u = 0; u < kSscUnroll; ++u)
#pragma unroll
      for (int bt = 0; bt < kSscTile; ++bt) {
        const float w = Ws[bt * Gp + j0 + u];
#pragma unroll
        for (int q = 0; q < KPT; ++q) acc[bt][q] = fmaf(w, kv[u][q], acc[bt][q]);
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
    S.jssc[(size_t)b * F + i] = cgs::h_pl * g.nu[i] * sc[kScalSW] * sc[kScalSU] * (double)s;
  }
}

}  // namespace pbag

#endif
