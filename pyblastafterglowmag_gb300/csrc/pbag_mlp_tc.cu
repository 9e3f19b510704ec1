// pbag_mlp_tc.cu - BF16 inference of the library's MLP (pbag_mlp) on the
// 5th-generation tensor cores, all layers fused in one kernel.
//
// One CTA runs 128 rows (states) through every layer. The activations of the
// current layer stay in shared memory as the A operand (BF16, K-major core
// matrices); the weights W_l [out][in] are laid out once (mlp_tc_pack) as the B
// operand and stream through a ring of stages by bulk copy, layer after layer,
// so the next layer's weights arrive while the epilogue of this one runs. The
// accumulator D [128 rows][out] is in tensor memory (FP32). One thread issues
// copies and MMAs; eight warps run the epilogue (tcgen05.ld, + bias, SiLU,
// round to BF16, written back in place as the next layer's A operand; the last
// layer adds its bias and stores FP32 rows). Layer l+1 starts when every
// epilogue thread has arrived on an mbarrier after its writes (with a proxy
// fence, so the tensor cores see them) and its tensor-memory reads.
//
// Supported shapes: in-dimension of every layer a multiple of 32, out-dimension
// a multiple of 32 up to 256, up to kMtMaxLayers layers. Every wait is bounded:
// on a timeout the CTA records PBAG_ERR_TIMEOUT, waits (bounded) for its copies
// and MMAs, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pbag.h"
#include "pbag_kernels.h"
#include "pbag_tc.cuh"

namespace pbag {

namespace {

using tc::smem_u32;

constexpr int kMtRows = 128;
constexpr int kMtEpiWarps = 8;
constexpr int kMtThreads = 32 * (kMtEpiWarps + 1);
// two CTAs per SM (shared memory 2 x 112 KiB, tensor memory 2 x 256 columns):
// the MMAs and copies of one overlap the epilogue of the other
constexpr int kMtCtasPerSm = 2;
constexpr int kMtStages = 3;
constexpr int kMtKc = 32;                                     // K columns of a stage: a multiple of this
constexpr int kMtKcMax = 32;                                  // ... up to this
constexpr uint32_t kMtStageBytes = kMtMaxOut * kMtKcMax * 2;  // 16 KiB
constexpr uint32_t kMtActBytes = kMtRows * kMtMaxOut * 2;     // 64 KiB
constexpr size_t kMtSmem = 128 + kMtActBytes + (size_t)kMtStages * kMtStageBytes;
static_assert(kMtCtasPerSm * (kMtSmem + 1024 + 256) <= 233472, "two CTAs per SM");

// byte offset of element (row r, column k) of a K-major operand with `rows`
// rows: core matrix (r/8, k/8) at (k/8)*rows*16 + (r/8)*128
__host__ __device__ __forceinline__ uint32_t mt_offset(int r, int k, int rows) {
  return (uint32_t)(k >> 3) * rows * 16 + (uint32_t)(r >> 3) * 128 + (uint32_t)(r & 7) * 16 + (uint32_t)(k & 7) * 2;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

__global__ void __launch_bounds__(kMtThreads, kMtCtasPerSm)
k_mlp_tc(MlpTcArgs a, int n, const float* __restrict__ X, float* __restrict__ Y, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ uint64_t bars[2 * kMtStages + 2];  // full[S], empty[S], acc full, activations ready
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int fail;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  unsigned char* act = base;
  unsigned char* ring = base + kMtActBytes;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kMtRows;
  const uint32_t accf = smem_u32(&bars[2 * kMtStages]), actr = smem_u32(&bars[2 * kMtStages + 1]);
  if (tid == 0) {
    fail = 0;
    for (int s = 0; s < 2 * kMtStages; ++s) tc::mbar_init(smem_u32(&bars[s]), 1);
    tc::mbar_init(accf, 1);
    tc::mbar_init(actr, 32 * kMtEpiWarps);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)kMtMaxOut));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == kMtEpiWarps) {
    if (lane == 0) {
      // copies and MMAs
      // K columns per stage of layer l: 64 where the in-dimension allows
      auto kcl = [&](int l) { return a.dims[l] % kMtKcMax == 0 ? kMtKcMax : kMtKc; };
      int total = 0;
      for (int l = 0; l < a.L; ++l) total += a.dims[l] / kcl(l);
      int ll = 0, lc = 0;  // next chunk to copy: layer, chunk
      auto load_next = [&](int st) {
        const int N = a.dims[ll + 1];
        const int kc = kcl(ll);
        const uint32_t bytes = (uint32_t)N * kc * 2;
        const uint32_t bar = smem_u32(&bars[st]);
        tc::mbar_expect_tx(bar, bytes);
        tc::bulk_g2s(smem_u32(ring + (size_t)st * kMtStageBytes),
                     a.W[ll] + (size_t)lc * N * kc, bytes, bar);
        if (++lc == a.dims[ll] / kc) {
          lc = 0;
          ++ll;
        }
      };
      int loaded = 0;
      for (; loaded < kMtStages && loaded < total; ++loaded) load_next(loaded);
      int g = 0;  // next chunk to consume
      bool ok = true;
      for (int l = 0; l < a.L && ok; ++l) {
        if (!tc::mbar_wait(actr, (uint32_t)l & 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int N = a.dims[l + 1], kc = kcl(l), nc = a.dims[l] / kc;
        const uint32_t idesc = tc::idesc_mma(kMtRows, N, false);
        for (int c = 0; c < nc; ++c) {
          const int st = g % kMtStages;
          if (!tc::mbar_wait(smem_u32(&bars[st]), (uint32_t)(g / kMtStages) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sb = smem_u32(ring + (size_t)st * kMtStageBytes);
          for (int s = 0; s < kc / 16; ++s) {
            const uint64_t ad = tc::smem_desc(smem_u32(act) + (uint32_t)((kc / 8) * c + 2 * s) * kMtRows * 16,
                                              kMtRows * 16, 128);
            const uint64_t bd = tc::smem_desc(sb + (uint32_t)(2 * s) * N * 16, (uint32_t)N * 16, 128);
            tc::mma_issue<false>(tmem, ad, bd, idesc, (c > 0 || s > 0) ? 1u : 0u);
          }
          tc::mma_commit(smem_u32(&bars[kMtStages + st]));
          // refill the stage of the previous chunk once its MMAs are done
          if (g >= 1 && loaded < total) {
            const int pg = g - 1, pst = pg % kMtStages;
            if (!tc::mbar_wait(smem_u32(&bars[kMtStages + pst]), (uint32_t)(pg / kMtStages) & 1)) {
              ok = false;
              ++g;
              break;
            }
            load_next(pst);
            ++loaded;
          }
          ++g;
        }
        if (ok) tc::mma_commit(accf);
      }
      if (!ok) {
        fail = 1;
        atomicCAS(err, 0, PBAG_ERR_TIMEOUT);
        // copies and MMAs in flight: one more bounded wait each
        for (int c = g; c < loaded; ++c) tc::mbar_wait(smem_u32(&bars[c % kMtStages]), (uint32_t)(c / kMtStages) & 1);
        if (g > 0)
          tc::mbar_wait(smem_u32(&bars[kMtStages + (g - 1) % kMtStages]), (uint32_t)((g - 1) / kMtStages) & 1);
      }
    }
  } else {
    // the input rows, rounded to BF16, as the first A operand
    const int K0 = a.dims[0];
    for (int u = tid; u < kMtRows * (K0 / 8); u += 32 * kMtEpiWarps) {
      const int r = u % kMtRows, k8 = u / kMtRows;
      uint4 w = make_uint4(0u, 0u, 0u, 0u);
      if (row0 + r < n) {
        const float4* src = reinterpret_cast<const float4*>(X + (size_t)(row0 + r) * K0 + 8 * k8);
        const float4 x0 = __ldg(src), x1 = __ldg(src + 1);
        w = make_uint4(pack_bf16(x0.x, x0.y), pack_bf16(x0.z, x0.w), pack_bf16(x1.x, x1.y), pack_bf16(x1.z, x1.w));
      }
      *reinterpret_cast<uint4*>(act + mt_offset(r, 8 * k8, kMtRows)) = w;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc::mbar_arrive(actr);
    const int q = warp & 3, h = warp >> 2;
    const int r = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    for (int l = 0; l < a.L; ++l) {
      bool ready = false;
      for (int t = 0; t < 64 && !ready && !fail; ++t) ready = tc::mbar_wait(accf, (uint32_t)l & 1, 1 << 15);
      if (!ready) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int N = a.dims[l + 1], half = N / 2;
      const float* bias = a.b[l];
      const bool last = l == a.L - 1;
      for (int col0 = h * half; col0 < (h + 1) * half; col0 += 16) {
        uint32_t v[16];
        tc::tmem_ld16(tl + (uint32_t)col0, v);
        float y[16];
        const float4* b4 = reinterpret_cast<const float4*>(bias + col0);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float4 bb = __ldg(b4 + c);
          y[4 * c] = __uint_as_float(v[4 * c]) + bb.x;
          y[4 * c + 1] = __uint_as_float(v[4 * c + 1]) + bb.y;
          y[4 * c + 2] = __uint_as_float(v[4 * c + 2]) + bb.z;
          y[4 * c + 3] = __uint_as_float(v[4 * c + 3]) + bb.w;
        }
        if (last) {
          if (row0 + r < n) {
            float4* dst = reinterpret_cast<float4*>(Y + (size_t)(row0 + r) * N + col0);
#pragma unroll
            for (int c = 0; c < 4; ++c) dst[c] = make_float4(y[4 * c], y[4 * c + 1], y[4 * c + 2], y[4 * c + 3]);
          }
        } else {
#pragma unroll
          for (int c = 0; c < 16; ++c) y[c] = __fdividef(y[c], 1.f + __expf(-y[c]));  // SiLU (0 where exp overflows)
#pragma unroll
          for (int k8 = 0; k8 < 2; ++k8) {
            const uint4 w = make_uint4(pack_bf16(y[8 * k8], y[8 * k8 + 1]), pack_bf16(y[8 * k8 + 2], y[8 * k8 + 3]),
                                       pack_bf16(y[8 * k8 + 4], y[8 * k8 + 5]),
                                       pack_bf16(y[8 * k8 + 6], y[8 * k8 + 7]));
            *reinterpret_cast<uint4*>(act + mt_offset(r, col0 + 8 * k8, kMtRows)) = w;
          }
        }
      }
      if (!last) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        tc::mbar_arrive(actr);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kMtMaxOut));
  }
}

// FP32 W [N][K] (row-major) into the B-operand layout
__global__ void k_mlp_tc_pack(int N, int K, const float* __restrict__ W, uint16_t* __restrict__ out) {
  const int64_t tot = (int64_t)N * K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int nn = (int)(e / K), k = (int)(e % K);
    __nv_bfloat16 b = __float2bfloat16_rn(W[e]);
    out[mt_offset(nn, k, N) / 2] = *reinterpret_cast<uint16_t*>(&b);
  }
}

}  // namespace

bool mlp_tc_supported(const int* dims, int L) {
  if (L < 1 || L > kMtMaxLayers) return false;
  for (int l = 0; l < L; ++l) {
    if (dims[l] % kMtKc != 0 || dims[l] > kMtMaxOut) return false;
    if (dims[l + 1] % 32 != 0 || dims[l + 1] > kMtMaxOut) return false;
  }
  return true;
}

size_t mlp_tc_layer_elems(int N, int K) { return (size_t)N * K; }

cudaError_t mlp_tc_pack(int N, int K, const float* W, uint16_t* out, cudaStream_t st) {
  const int64_t tot = (int64_t)N * K;
  const int blocks = (int)std::min<int64_t>((tot + 255) / 256, 1024);
  k_mlp_tc_pack<<<blocks, 256, 0, st>>>(N, K, W, out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_tc(const MlpTcArgs& a, int n, const float* X, float* Y, int* err, cudaStream_t st) {
  static bool attr = false;  // set on the first call, which may launch nothing (before any graph capture)
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMtSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (n <= 0) return cudaSuccess;
  k_mlp_tc<<<(n + kMtRows - 1) / kMtRows, kMtThreads, kMtSmem, st>>>(a, n, X, Y, err);
  return cudaGetLastError();
}

}  // namespace pbag
