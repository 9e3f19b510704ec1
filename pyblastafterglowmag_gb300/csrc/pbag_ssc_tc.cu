// pbag_ssc_tc.cu - SSC contraction on the 5th-generation tensor cores.
//
// computeSSCSpectrum (numeric_model.h:247-285) for a batch of blastwaves is,
// for each output frequency i, the GEMM
//   T_i[b][k] = sum_j W[b][j] K[i][j][k]        (M = blastwaves, N = k, K-dim = j)
// followed by j_ssc[b][i] = h nu_i sW_b sU_b sum_k T_i[b][k] U[b][k].
// One CTA owns one output frequency i and 128 blastwaves: the accumulator
// D[128][N = F] lives in tensor memory, tcgen05.mma is issued by one thread
// with operands in shared memory (BF16, K-major, no swizzle), the K operand
// slabs arrive by bulk copy (cp.async.bulk, completion on an mbarrier) into a
// ring of stages so that copies, operand conversion and MMAs overlap, and the
// epilogue reads D back with tcgen05.ld and reduces it against U in FP32.
//
// Precision: W and K are split into BF16 hi + lo parts and the three products
// hi*hi + hi*lo + lo*hi are accumulated in FP32 (relative error ~1e-5 on
// these non-negative sums); the plain-BF16 variant issues hi*hi only.
// Every wait is bounded: on a timeout the CTA records PBAG_ERR_TIMEOUT for its
// blastwaves, waits (bounded) for its copies and MMAs, frees its tensor
// memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "pbag_kernels.h"

namespace pbag {

namespace {

constexpr int kTcThreads = 128;
constexpr int kTcM = 128;        // blastwaves per tile (TMEM lanes)
constexpr int kChunkK8 = 8;      // 16-byte K columns per chunk (64 BF16 values of j)
constexpr int kWaitLimit = 1 << 21;

template <int N>
struct TcShape {
  static constexpr int kStages = N <= 128 ? 3 : 2;
  static constexpr uint32_t kABytes = kTcM * kChunkK8 * 16;  // one part (hi or lo) of an A chunk
  static constexpr uint32_t kBBytes = N * kChunkK8 * 16;     // one part of a B chunk
  static constexpr uint32_t kStageBytes = 2 * kABytes + 2 * kBBytes;
  static constexpr size_t kSmem = 1024 + (size_t)kStages * kStageBytes + 8 * 2 * kStages + 16;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor: K-major, no swizzle. lbo = byte
// stride between core matrices along K, sbo = along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this architecture
  return d;               // base offset 0, relative LBO, no swizzle
}

// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (it > 32) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void store_split(uint4* hi, uint4* lo, const float* w, bool split) {
  __nv_bfloat16 h[8], l[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    h[q] = __float2bfloat16_rn(w[q]);
    l[q] = split ? __float2bfloat16_rn(w[q] - __bfloat162float(h[q])) : __float2bfloat16_rn(0.f);
  }
  std::memcpy(hi, h, 16);
  std::memcpy(lo, l, 16);
}

// One tile: output frequency i = blockIdx.x, blastwaves 128*blockIdx.y ...
template <int N, bool kSplit>
__global__ void __launch_bounds__(kTcThreads)
k_ssc_tc(const float* __restrict__ W32, int Gp, int nrows, const int* __restrict__ flags,
         const uint16_t* __restrict__ Bt, const float* __restrict__ U32, const double* __restrict__ scal,
         int scal_stride, int sw_idx, int su_idx, const double* __restrict__ nu, double* __restrict__ out,
         int* __restrict__ err) {
  using Sh = TcShape<N>;
  constexpr int S = Sh::kStages;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i = blockIdx.x;
  const int row0 = blockIdx.y * kTcM;
  const int F = N;
  // shared layout: S stages of [A_hi | A_lo | B_hi | B_lo], then barriers and the tmem slot
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + (size_t)S * Sh::kStageBytes);  // tma[S], mma[S]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S);
  __shared__ int live[kTcM];
  __shared__ int fail;

  for (int m = tid; m < kTcM; m += kTcThreads) {
    const int r = row0 + m;
    live[m] = (r < nrows && (!flags || (flags[r] & kFlagActive))) ? 1 : 0;
  }
  if (tid == 0) {
    fail = 0;
    for (int s = 0; s < 2 * S; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  int any = 0;
  for (int m = 0; m < kTcM; ++m) any |= live[m];

  const int nk8 = Gp / 8;
  const int nchunks = (nk8 + kChunkK8 - 1) / kChunkK8;
  const uint16_t* Bi = Bt + (size_t)i * 2 * N * Gp;
  constexpr uint32_t idesc = idesc_bf16(kTcM, N);

  auto stage_ptr = [&](int st) { return base + (size_t)st * Sh::kStageBytes; };
  // K operand slab of chunk c into stage st: one bulk copy (hi then lo)
  auto load_B = [&](int c, int st) {
    const int kc8 = min(kChunkK8, nk8 - c * kChunkK8);
    const uint32_t bytes = 2u * (uint32_t)N * kc8 * 16;
    const uint32_t bar = smem_u32(&bars[st]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(stage_ptr(st) + 2 * Sh::kABytes)),
        "l"(Bi + (size_t)2 * N * 64 * c), "r"(bytes), "r"(bar)
        : "memory");
  };
  // W operand of chunk c into stage st: FP32 -> BF16 hi/lo in the core-matrix layout
  auto load_A = [&](int c, int st) {
    const int kc8 = min(kChunkK8, nk8 - c * kChunkK8);
    unsigned char* A_hi = stage_ptr(st);
    unsigned char* A_lo = A_hi + Sh::kABytes;
    for (int p = tid; p < kTcM * kc8; p += kTcThreads) {
      const int m = p % kTcM, k8 = p / kTcM;
      float w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (live[m]) {
        const float4* src = reinterpret_cast<const float4*>(W32 + (size_t)(row0 + m) * Gp + (c * kChunkK8 + k8) * 8);
        const float4 a = __ldg(src), b = __ldg(src + 1);
        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
        w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
      }
      const uint32_t off = (uint32_t)(((m >> 3) * kc8 + k8) * 128 + (m & 7) * 16);
      store_split(reinterpret_cast<uint4*>(A_hi + off), reinterpret_cast<uint4*>(A_lo + off), w, kSplit);
    }
  };

  bool ok = any != 0;
  if (ok) {
    const int pre = min(S, nchunks);
    if (tid == 0)
      for (int c = 0; c < pre; ++c) load_B(c, c);
    for (int c = 0; c < pre; ++c) load_A(c, c);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    for (int c = 0; c < nchunks; ++c) {
      const int st = c % S;
      const uint32_t use = (uint32_t)(c / S);  // how often this stage was filled before
      if (c >= S) {
        // refill the stage once the MMAs of chunk c - S have read it
        if (!mbar_wait(smem_u32(&bars[S + st]), (use - 1) & 1)) fail = 1;
        __syncthreads();
        if (fail) break;
        if (tid == 0) load_B(c, st);
        load_A(c, st);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
      }
      if (tid == 0) {
        if (!mbar_wait(smem_u32(&bars[st]), use & 1)) {
          fail = 1;
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const int kc8 = min(kChunkK8, nk8 - c * kChunkK8);
          const uint32_t sbo = (uint32_t)kc8 * 128;
          const uint32_t a_hi = smem_u32(stage_ptr(st)), a_lo = a_hi + Sh::kABytes;
          const uint32_t b_hi = a_lo + Sh::kABytes, b_lo = b_hi + (uint32_t)N * kc8 * 16;
          for (int s = 0; s < kc8 / 2; ++s) {
            const uint32_t ko = (uint32_t)s * 256;  // two 16-byte K columns per MMA (K = 16)
            mma_bf16(tmem, smem_desc(a_hi + ko, 128, sbo), smem_desc(b_hi + ko, 128, sbo), idesc,
                     (c > 0 || s > 0) ? 1u : 0u);
            if (kSplit) {
              mma_bf16(tmem, smem_desc(a_hi + ko, 128, sbo), smem_desc(b_lo + ko, 128, sbo), idesc, 1);
              mma_bf16(tmem, smem_desc(a_lo + ko, 128, sbo), smem_desc(b_hi + ko, 128, sbo), idesc, 1);
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           smem_u32(&bars[S + st]))
                       : "memory");
        }
      }
      __syncthreads();
      if (fail) break;
    }
    // the last commit completes after every earlier MMA of this thread
    if (!fail) {
      const int c = nchunks - 1;
      if (!mbar_wait(smem_u32(&bars[S + c % S]), (uint32_t)(c / S) & 1)) fail = 1;
    }
    __syncthreads();
    ok = fail == 0;
    if (!ok && tid == 0) {
      // a bounded wait ran out: record it and give in-flight work one more bounded wait
      for (int s = 0; s < 2 * S; ++s) mbar_wait(smem_u32(&bars[s]), 0);
      for (int m = 0; m < kTcM; ++m)
        if (live[m]) atomicCAS(&err[4 * (row0 + m)], 0, PBAG_ERR_TIMEOUT);
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // epilogue: row m = 32*warp + lane of the accumulator
    const int m = warp * 32 + lane;
    const int r = row0 + m;
    const bool mine = live[m] != 0;
    const float* Ur = U32 + (size_t)(mine ? r : 0) * F;
    float acc = 0.f;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int col = 0; col < N; col += 16) {
      uint32_t v[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr + (uint32_t)col));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (mine) {
        const float4* u4 = reinterpret_cast<const float4*>(Ur + col);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 u = __ldg(u4 + q);
          acc = fmaf(__uint_as_float(v[4 * q + 0]), u.x, acc);
          acc = fmaf(__uint_as_float(v[4 * q + 1]), u.y, acc);
          acc = fmaf(__uint_as_float(v[4 * q + 2]), u.z, acc);
          acc = fmaf(__uint_as_float(v[4 * q + 3]), u.w, acc);
        }
      }
    }
    if (mine) {
      const double* sc = scal + (size_t)r * scal_stride;
      out[(size_t)r * F + i] = cgs::h_pl * nu[i] * sc[sw_idx] * sc[su_idx] * (double)acc;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(N));
  }
}

template <int N, bool kSplit>
cudaError_t launch_tc(const float* W32, int Gp, int nrows, const int* flags, const uint16_t* Bt, const float* U32,
                      const double* scal, int scal_stride, int sw_idx, int su_idx, const double* nu, double* out,
                      int* err, int F, cudaStream_t st) {
  const size_t smem = TcShape<N>::kSmem;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_ssc_tc<N, kSplit>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid(F, (nrows + kTcM - 1) / kTcM);
  k_ssc_tc<N, kSplit><<<grid, kTcThreads, smem, st>>>(W32, Gp, nrows, flags, Bt, U32, scal, scal_stride, sw_idx,
                                                       su_idx, nu, out, err);
  return cudaGetLastError();
}

uint16_t bf16_bits(float x) {  // round to nearest even (finite inputs)
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float bf16_value(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

}  // namespace

bool ssc_tc_supported(int F) { return F == 128 || F == 256; }

void build_ssc_tc_operand(const std::vector<float>& K32, int F, int Gp, std::vector<uint16_t>& Bt) {
  const int N = F;
  const int nk8 = Gp / 8;
  Bt.assign((size_t)F * 2 * N * Gp, 0);
  for (int i = 0; i < F; ++i) {
    uint16_t* Bi = Bt.data() + (size_t)i * 2 * N * Gp;
    for (int c = 0; c * kChunkK8 < nk8; ++c) {
      const int kc8 = std::min(kChunkK8, nk8 - c * kChunkK8);
      uint16_t* hi = Bi + (size_t)2 * N * 64 * c;
      uint16_t* lo = hi + (size_t)N * kc8 * 8;
      for (int n = 0; n < N; ++n)
        for (int kl = 0; kl < kc8 * 8; ++kl) {
          const int j = c * 64 + kl;
          const float v = K32[((size_t)i * Gp + j) * F + n];  // K[i][j][k = n]
          const uint16_t h = bf16_bits(v);
          const uint16_t l = bf16_bits(v - bf16_value(h));
          const size_t e = (size_t)((n >> 3) * kc8 + (kl >> 3)) * 64 + (n & 7) * 8 + (kl & 7);
          hi[e] = h;
          lo[e] = l;
        }
    }
  }
}

cudaError_t launch_ssc_tc(const DevGrid& g, const DevState& S, const uint16_t* Bt, int nbw, bool split,
                          cudaStream_t st) {
  if (nbw <= 0) return cudaSuccess;
  if (g.F == 128)
    return split ? launch_tc<128, true>(S.W32, g.Gp, nbw, S.flags, Bt, S.U32, S.scal, kScal, kScalSW, kScalSU, g.nu,
                                        S.jssc, S.err, g.F, st)
                 : launch_tc<128, false>(S.W32, g.Gp, nbw, S.flags, Bt, S.U32, S.scal, kScal, kScalSW, kScalSU, g.nu,
                                         S.jssc, S.err, g.F, st);
  if (g.F == 256)
    return split ? launch_tc<256, true>(S.W32, g.Gp, nbw, S.flags, Bt, S.U32, S.scal, kScal, kScalSW, kScalSU, g.nu,
                                        S.jssc, S.err, g.F, st)
                 : launch_tc<256, false>(S.W32, g.Gp, nbw, S.flags, Bt, S.U32, S.scal, kScal, kScalSW, kScalSU, g.nu,
                                         S.jssc, S.err, g.F, st);
  return cudaErrorInvalidValue;
}

}  // namespace pbag
