// pbag_ssc_tc.cu - SSC contraction on the 5th-generation tensor cores.
//
// computeSSCSpectrum (numeric_model.h:247-285) for a batch of blastwaves is,
// for each output frequency i, the GEMM
//   D_i[k][b] = sum_j K[i][j][k] W[b][j]      (M = k, N = blastwaves b, K-dim = j)
// followed by j_ssc[b][i] = h nu_i sW_b sU_b sum_k D_i[k][b] U[b][k].
// One CTA owns one output frequency i and a tile of up to 256 blastwaves: the
// accumulator (128 rows k per half of the frequency grid, N = blastwave
// columns) lives in tensor memory, tcgen05.mma is issued by one thread with
// both operands in shared memory (BF16, K-major, no swizzle). The operands are
// stored in global memory already in that layout (tc_operand_offset): the
// kernel slabs once per grid, the weights W by the evolve kernel of the step.
// They arrive by bulk copy (cp.async.bulk, completion on an mbarrier) into a
// ring of stages so that copies and MMAs overlap. The epilogue reads D back
// with tcgen05.ld (thread = row k), multiplies by U, and sums over k through
// shared memory (thread = blastwave).
//
// Blastwaves on N rather than M: a small batch (42 blastwaves) costs an MMA of
// N = 48 columns instead of 128 mostly empty rows.
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
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "pbag.h"
#include "pbag_kernels.h"
#include "pbag_tc.cuh"

namespace pbag {

namespace {

using tc::idesc_mma;
using tc::mbar_wait;
using tc::mma_issue;
using tc::smem_desc;
using tc::smem_u32;

constexpr int kTcThreads = 128;
constexpr int kTcK = 128;          // accumulator rows (output columns k) per half of the frequency grid
constexpr int kTcMaxStages = 8;    // ring of chunk stages (all chunks of a small problem at once)
constexpr int kK8 = kTcChunk16;   // 16-byte K columns of a full chunk
constexpr int kPStride = kTcK + 1;  // row stride (floats) of the epilogue's product table
constexpr size_t kTcDynMax = 231424;       // dynamic shared memory of a CTA (227 KiB less the static part)
constexpr size_t kTcFixed = 1024 + 256;   // alignment slack, barriers and the tensor-memory slot
constexpr size_t kTcUSmemMax = 64 * 1024; // largest U tile staged whole in shared memory
constexpr int kTcURing = 2;               // otherwise: ring of U column blocks (16 blastwaves each)
constexpr int kRowsMin = 2048;            // batches from this size on run with blastwaves on the rows

// Dynamic shared memory of one launch: [body: ring of stages of [A hi | A lo (F
// rows each) | B hi | B lo (N rows each)], reused by the product table][U: the
// whole tile (N x F floats) when it fits, else a ring of kTcURing blocks of 16
// rows][barriers].
__host__ __device__ constexpr uint32_t tc_a_region(int F) { return 2u * F * kK8 * 16; }
__host__ __device__ constexpr uint32_t tc_stage_bytes(int F, int N) { return tc_a_region(F) + 2u * N * kK8 * 16; }
struct TcPlan {
  int S;            // stages
  uint32_t body;    // bytes of the stage ring / product table
  uint32_t ubytes;  // bytes of the whole U tile in shared memory (0: the ring instead)
  uint32_t uring;   // bytes of the U block ring (0 when the whole tile is staged)
  size_t smem;      // dynamic shared memory
};
inline TcPlan tc_plan(int F, int N, int Gp) {
  TcPlan p;
  const int nchunks = (Gp / 8 + kK8 - 1) / kK8;
  const uint32_t stage = tc_stage_bytes(F, N);
  const size_t ub = (size_t)N * F * sizeof(float);
  p.ubytes = ub <= kTcUSmemMax ? (uint32_t)ub : 0u;
  p.uring = p.ubytes ? 0u : (uint32_t)(kTcURing * 16 * F * sizeof(float));
  const size_t room = kTcDynMax - kTcFixed - p.ubytes - p.uring;
  p.S = std::max(2, std::min({nchunks, kTcMaxStages, (int)(room / stage)}));
  p.body = std::max<uint32_t>((uint32_t)p.S * stage, (uint32_t)(N * kPStride * sizeof(float)));
  p.body = (p.body + 1023) / 1024 * 1024;
  p.smem = 1024 + (size_t)p.body + p.ubytes + p.uring + 16 * kTcMaxStages + 16;
  return p;
}

__device__ __forceinline__ void cp_async4(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(static_cast<uint32_t>(
                   __cvta_generic_to_shared(dst))),
               "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}

// One CTA: output frequency i = blockIdx.x, blastwaves kTcCols*blockIdx.y + [0, N).
// Thread 0 streams the chunks of the kernel slab (A, F rows) and of the weight
// tile (B, N rows) through a ring of S stages and issues the MMAs; all threads
// run the epilogue. H = F / 128 accumulator halves; MODE is kTcBf16, kTcSplit
// (three MMAs per K step) or kTcTf32 (4-byte operands, kind::tf32). Every load
// that does not depend on another is issued first, the copies before the
// tensor-memory allocation.
template <int H, int MODE>
__global__ void __launch_bounds__(kTcThreads, 1)
k_ssc_tc(const unsigned char* __restrict__ Wt, const unsigned char* __restrict__ Kt, int Gp, int nrows, int N, int S,
         uint32_t body, uint32_t ubytes, uint32_t uring, const int* __restrict__ flags, const float* __restrict__ U32,
         const double* __restrict__ scal, const double* __restrict__ oscale, int ostride, double* __restrict__ out,
         int* __restrict__ err, const int* __restrict__ nlive, const int* __restrict__ rowmap) {
  constexpr int F = kTcK * H;
  constexpr bool kSplit = MODE == kTcSplit;
  constexpr bool kTf32 = MODE == kTcTf32;
  constexpr int kEs = kTf32 ? 4 : 2;  // operand element size
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int i = blockIdx.x;
  const int row0 = blockIdx.y * kTcCols;
  grid_dep_wait();  // the weights, flags and row counts of the step's evolve launch
  grid_dep_launch();
  if (nlive && row0 >= *nlive) return;  // a tile beyond the rows counted on the device
  const uint32_t stage_bytes = tc_stage_bytes(F, N);
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  float* Us = reinterpret_cast<float*>(base + body);                           // U tile [N][F] or ring [2][16][F]
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + body + ubytes + uring);  // full[S], empty[S], U
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kTcMaxStages + 1);
  __shared__ int fail;
  auto stage_ptr = [&](int st) { return base + (size_t)st * stage_bytes; };

  const int nk8 = Gp * kEs / 16;  // 16-byte K columns
  const int nchunks = (nk8 + kK8 - 1) / kK8;
  const unsigned char* Ai = Kt + (size_t)i * tc_tile_bytes(F, Gp, kEs);                  // kernel slab of frequency i
  const unsigned char* Bw = Wt + (size_t)blockIdx.y * tc_tile_bytes(kTcCols, Gp, kEs);  // weight tile
  auto load = [&](int c, int st) {
    const int kc8 = min(kK8, nk8 - c * kK8);
    const uint32_t ab = (kSplit ? 2u : 1u) * F * kc8 * 16;  // hi (+ lo), contiguous
    const uint32_t bp = (uint32_t)N * kc8 * 16;              // first N rows of one part
    const uint32_t bar = smem_u32(&bars[st]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"(ab + (kSplit ? 2u : 1u) * bp)
                 : "memory");
    const unsigned char* bsrc = Bw + (size_t)2 * kTcCols * kK8 * 16 * c;
    unsigned char* bdst = stage_ptr(st) + tc_a_region(F);
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(stage_ptr(st))),
        "l"(Ai + (size_t)2 * F * kK8 * 16 * c), "r"(ab), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(bdst)),
        "l"(bsrc), "r"(bp), "r"(bar)
        : "memory");
    if (kSplit)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_u32(bdst + bp)),
          "l"(bsrc + (size_t)kTcCols * kc8 * 16), "r"(bp), "r"(bar)
          : "memory");
  };
  const int pre = min(S, nchunks);
  const uint32_t ubar = smem_u32(&bars[2 * kTcMaxStages]);
  if (tid == 0) {
    fail = 0;
    for (int s = 0; s < 2 * S; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int c = 0; c < pre; ++c) load(c, c);
    if (ubytes) {  // the tile's seed-photon weights, rows as in global memory
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ubar), "r"(ubytes) : "memory");
      const unsigned char* usrc = reinterpret_cast<const unsigned char*>(U32 + (size_t)row0 * F);
      for (uint32_t o = 0; o < ubytes; o += 32768u)
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(reinterpret_cast<unsigned char*>(Us) + o)),
            "l"(usrc + o), "r"(min(32768u, ubytes - o)), "r"(ubar)
            : "memory");
    }
  }
  // the blastwaves this thread finishes (columns tid and tid + 128) and their FP64 factors
  bool live[2];
  double fac[2];
  const double hnu = oscale[i];  // h nu_i for the SSC spectrum
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int col = tid + q * kTcThreads, r = row0 + col;
    const bool in = col < N && r < nrows;
    const int fl = in ? flags[r] : 0;
    const double sw = in ? scal[(size_t)r * kScal + kScalSW] : 0.;
    const double su = in ? scal[(size_t)r * kScal + kScalSU] : 0.;
    live[q] = (fl & kFlagActive) != 0;
    fac[q] = hnu * sw * su;
  }
  // without a staged U tile: this thread's U[b][k] (k = tid + 128 h) of 16
  // columns at a time, copied asynchronously into its own slots of a ring
  // (each thread reads only what it copied, so no barrier is needed)
  const int nb = N / 16;
  auto u_block = [&](int cb) {
    float* slot = Us + (size_t)(cb % kTcURing) * 16 * F;
#pragma unroll
    for (int h = 0; h < H; ++h)
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int r = row0 + cb * 16 + c;
        cp_async4(slot + c * F + tid + kTcK * h, U32 + (size_t)(r < nrows ? r : 0) * F + tid + kTcK * h, r < nrows);
      }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  if (!ubytes)
    for (int cb = 0; cb < kTcURing && cb < nb; ++cb) u_block(cb);

  uint32_t ncols = 32;
  while (ncols < (uint32_t)(H * N)) ncols <<= 1;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  const int any = __syncthreads_or((live[0] || live[1]) ? 1 : 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (tid == 0) {
    int loaded = pre;  // chunks whose copies were issued
    int next = 0;      // next chunk to consume
    bool ok = true;
    if (any) {
      const uint32_t idesc = idesc_mma(kTcK, N, kTf32);
      for (; next < nchunks; ++next) {
        const int c = next, st = c % S;
        if (!mbar_wait(smem_u32(&bars[st]), (uint32_t)(c / S) & 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int kc8 = min(kK8, nk8 - c * kK8);
        const uint32_t sbo = (uint32_t)kc8 * 128;
        const uint32_t a_hi = smem_u32(stage_ptr(st)), a_lo = a_hi + (uint32_t)F * kc8 * 16;
        const uint32_t b_hi = a_hi + tc_a_region(F), b_lo = b_hi + (uint32_t)N * kc8 * 16;
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const uint32_t ah = (uint32_t)h * kTcK * kc8 * 16;  // rows k of half h: row groups 16h ...
          const uint32_t d = tmem + (uint32_t)(h * N);
          for (int s2 = 0; s2 < kc8 / 2; ++s2) {
            const uint32_t ko = (uint32_t)s2 * 256;  // two 16-byte K columns per MMA (K = 16 BF16 or 8 TF32)
            mma_issue<kTf32>(d, smem_desc(a_hi + ah + ko, 128, sbo), smem_desc(b_hi + ko, 128, sbo), idesc,
                             (c > 0 || s2 > 0) ? 1u : 0u);
            if (kSplit) {
              mma_issue<kTf32>(d, smem_desc(a_hi + ah + ko, 128, sbo), smem_desc(b_lo + ko, 128, sbo), idesc, 1);
              mma_issue<kTf32>(d, smem_desc(a_lo + ah + ko, 128, sbo), smem_desc(b_hi + ko, 128, sbo), idesc, 1);
            }
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&bars[S + st]))
                     : "memory");
        // refill the stage of the previous chunk once its MMAs are done (they
        // complete while this chunk's MMAs run)
        if (c >= 1 && loaded < nchunks) {
          const int pc = c - 1, pst = pc % S;
          if (!mbar_wait(smem_u32(&bars[S + pst]), (uint32_t)(pc / S) & 1)) {
            ok = false;
            ++next;
            break;
          }
          load(loaded, pst);
          ++loaded;
        }
      }
      if (ok) {
        // the last commit completes after every earlier MMA of this thread
        const int c = nchunks - 1;
        ok = mbar_wait(smem_u32(&bars[S + c % S]), (uint32_t)(c / S) & 1);
      }
    }
    if (ubytes && !mbar_wait(ubar, 0)) ok = false;
    if (!any || !ok) {
      // nothing to compute, or a bounded wait ran out: the copies and MMAs in
      // flight get one more bounded wait each before the CTA exits
      for (int c = next; c < loaded; ++c) mbar_wait(smem_u32(&bars[c % S]), (uint32_t)(c / S) & 1);
      if (next > 0) mbar_wait(smem_u32(&bars[S + (next - 1) % S]), (uint32_t)((next - 1) / S) & 1);
      if (ubytes) mbar_wait(ubar, 0);
    }
    if (!ok) {
      fail = 1;
      for (int col = 0; col < N; ++col) {
        const int r = row0 + col;
        if (r < nrows && (flags[r] & kFlagActive)) atomicCAS(&err[4 * (rowmap ? rowmap[r] : r)], 0, PBAG_ERR_TIMEOUT);
      }
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (any && !fail) {
    // products D[k][b] U[b][k] of this thread's rows k, into a [b][k] table in
    // the (now idle) stage memory
    float* P = reinterpret_cast<float*>(base);
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    for (int cb = 0; cb < nb; ++cb) {
      float u[H][16];
      if (ubytes) {
#pragma unroll
        for (int h = 0; h < H; ++h)
#pragma unroll
          for (int c = 0; c < 16; ++c) u[h][c] = Us[(size_t)(cb * 16 + c) * F + tid + kTcK * h];
      } else {
        if (cb + 1 < nb)
          asm volatile("cp.async.wait_group 1;" ::: "memory");
        else
          asm volatile("cp.async.wait_group 0;" ::: "memory");
        const float* slot = Us + (size_t)(cb % kTcURing) * 16 * F;
#pragma unroll
        for (int h = 0; h < H; ++h)
#pragma unroll
          for (int c = 0; c < 16; ++c) u[h][c] = slot[c * F + tid + kTcK * h];
        if (cb + kTcURing < nb) u_block(cb + kTcURing);
      }
      float p[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) p[c] = 0.f;
#pragma unroll
      for (int h = 0; h < H; ++h) {
        uint32_t v[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(tl + (uint32_t)(h * N + cb * 16)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int c = 0; c < 16; ++c) p[c] = fmaf(__uint_as_float(v[c]), u[h][c], p[c]);
      }
#pragma unroll
      for (int c = 0; c < 16; ++c) P[(size_t)(cb * 16 + c) * kPStride + tid] = p[c];
    }
    __syncthreads();
    // sum over k for blastwaves tid and tid + 128 (four partial sums)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (!live[q]) continue;
      const int col = tid + q * kTcThreads;
      const float* row = P + (size_t)col * kPStride;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 8
      for (int k = 0; k < kTcK; k += 4) {
        a0 += row[k];
        a1 += row[k + 1];
        a2 += row[k + 2];
        a3 += row[k + 3];
      }
      const int orow = rowmap ? rowmap[row0 + col] : row0 + col;
      out[(size_t)orow * ostride + i] = fac[q] * (double)((a0 + a1) + (a2 + a3));
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");  // no copy may land after the CTA exits
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
  }
}

// Small batches (N <= kSmallN blastwaves, F = 128, BF16 operands): the whole
// kernel slab of output i arrives in ONE bulk copy and the N weight rows and
// U rows by 16-byte asynchronous copies of all threads, so a CTA waits for one
// copy latency instead of one per chunk and operand part; then all MMAs, and
// the epilogue of k_ssc_tc. Shared memory: [slab: chunks of (hi | lo) F rows,
// reused by the product table][W: chunks of (hi | lo) N rows][U: N x F][barrier].
constexpr int kSmallN = 64;
static_assert(2 * kSmallN <= kTcThreads, "one W row part per thread in k_ssc_tc_small");
__host__ __device__ constexpr size_t small_slab_bytes(int Gp) { return (size_t)2 * kTcK * Gp * 2; }
__host__ __device__ constexpr size_t small_w_bytes(int N, int Gp) { return (size_t)2 * N * Gp * 2; }
inline size_t small_smem(int N, int Gp) {
  return 1024 + small_slab_bytes(Gp) + small_w_bytes(N, Gp) + (size_t)N * kTcK * 4 + 64;
}

template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 1)
k_ssc_tc_small(const unsigned char* __restrict__ Wt, const unsigned char* __restrict__ Kt, int Gp, int nrows, int N,
               const int* __restrict__ flags, const float* __restrict__ U32, const double* __restrict__ scal,
               const double* __restrict__ oscale, int ostride, double* __restrict__ out, int* __restrict__ err,
               const int* __restrict__ nlive, const int* __restrict__ rowmap) {
  constexpr int F = kTcK;
  constexpr bool kSplit = MODE == kTcSplit;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t abar;
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;
  __shared__ double sh_fac[kSmallN];  // per column: output factor
  __shared__ int sh_live[kSmallN];    // per column: a live row
  const int tid = threadIdx.x, warp = tid >> 5;
  const int i = blockIdx.x;
  const int row0 = blockIdx.y * kTcCols;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* As = base;
  unsigned char* Bs = base + small_slab_bytes(Gp);
  float* Us = reinterpret_cast<float*>(Bs + small_w_bytes(N, Gp));
  const int nk8 = Gp / 8, nchunks = (nk8 + kK8 - 1) / kK8;
  // the kernel slab (written once per context) streams in while the step's
  // evolve launch finishes; everything else is read after it completed
  if (tid == 0) {
    fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&abar)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const uint32_t bytes = (uint32_t)small_slab_bytes(Gp);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&abar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(As)),
        "l"(Kt + (size_t)i * tc_tile_bytes(F, Gp, 2)), "r"(bytes), "r"(smem_u32(&abar))
        : "memory");
  }
  grid_dep_wait();
  grid_dep_launch();  // the next evolve launch may be scheduled
  if (nlive && row0 >= *nlive) {  // a tile beyond the rows counted on the device: the copy lands first
    if (tid == 0) mbar_wait(smem_u32(&abar), 0);
    return;
  }
  // W rows [row0, row0 + N) of both parts of every chunk, and the U rows
  const unsigned char* Wtile = Wt + (size_t)blockIdx.y * tc_tile_bytes(kTcCols, Gp, 2);
  // thread (row r, part) of the first 2N threads copies its 16-byte unit of
  // every K column (2N <= kTcThreads): no division by the runtime N
  if (tid < 2 * N) {
    const int part = tid & 1, r = tid >> 1;
    for (int k16 = 0; k16 < nk8; ++k16) {
      const int c = k16 / kK8, kk = k16 - c * kK8, kc = min(kK8, nk8 - c * kK8);
      const size_t within = (size_t)((r >> 3) * kc + kk) * 128 + (size_t)(r & 7) * 16;
      const unsigned char* src =
          Wtile + (size_t)2 * kTcCols * kK8 * 16 * c + (size_t)part * kTcCols * kc * 16 + within;
      const uint32_t dst = smem_u32(Bs + (size_t)2 * N * kK8 * 16 * c + (size_t)part * N * kc * 16 + within);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    }
  }
  for (int u = tid; u < N * F / 4; u += kTcThreads) {
    const int r = u / (F / 4), k4 = u % (F / 4);
    const int gr = row0 + r < nrows ? row0 + r : row0;  // rows beyond the batch: any finite row
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(Us + (size_t)r * F + 4 * k4)),
                 "l"(U32 + (size_t)gr * F + 4 * k4)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  bool live[2];
  double fac[2];
  const double hnu = oscale[i];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int col = tid + q * kTcThreads, r = row0 + col;
    const bool in = col < N && r < nrows;
    live[q] = in && (flags[r] & kFlagActive);
    fac[q] = in ? hnu * scal[(size_t)r * kScal + kScalSW] * scal[(size_t)r * kScal + kScalSU] : 0.;
    if (col < N) {  // published by the barriers below
      sh_fac[col] = fac[q];
      sh_live[col] = live[q] ? 1 : 0;
    }
  }
  uint32_t ncols = 32;
  while (ncols < (uint32_t)N) ncols <<= 1;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  const int any = __syncthreads_or((live[0] || live[1]) ? 1 : 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    bool ok = mbar_wait(smem_u32(&abar), 0);
    if (ok && any) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t idesc = idesc_mma(kTcK, N, false);
      for (int c = 0; c < nchunks; ++c) {
        const int kc = min(kK8, nk8 - c * kK8);
        const uint32_t sbo = (uint32_t)kc * 128;
        const uint32_t a_hi = smem_u32(As + (size_t)2 * F * kK8 * 16 * c), a_lo = a_hi + (uint32_t)F * kc * 16;
        const uint32_t b_hi = smem_u32(Bs + (size_t)2 * N * kK8 * 16 * c), b_lo = b_hi + (uint32_t)N * kc * 16;
        for (int s2 = 0; s2 < kc / 2; ++s2) {
          const uint32_t ko = (uint32_t)s2 * 256;
          mma_issue<false>(tmem, smem_desc(a_hi + ko, 128, sbo), smem_desc(b_hi + ko, 128, sbo), idesc,
                           (c > 0 || s2 > 0) ? 1u : 0u);
          if (kSplit) {
            mma_issue<false>(tmem, smem_desc(a_hi + ko, 128, sbo), smem_desc(b_lo + ko, 128, sbo), idesc, 1u);
            mma_issue<false>(tmem, smem_desc(a_lo + ko, 128, sbo), smem_desc(b_hi + ko, 128, sbo), idesc, 1u);
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&mbar))
                   : "memory");
      ok = mbar_wait(smem_u32(&mbar), 0);
    }
    if (!ok) {
      fail = 1;
      for (int col = 0; col < N; ++col) {
        const int r = row0 + col;
        if (r < nrows && (flags[r] & kFlagActive)) atomicCAS(&err[4 * (rowmap ? rowmap[r] : r)], 0, PBAG_ERR_TIMEOUT);
      }
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (any && !fail) {
    // products D[k][b] U[b][k] of this thread's row k, into a [b][k] table in
    // the (now idle) slab memory; then the sum over k of each blastwave
    float* P = reinterpret_cast<float*>(base);
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    for (int cb = 0; cb < N / 16; ++cb) {
      uint32_t v[16];
      tc::tmem_ld16(tl + (uint32_t)(cb * 16), v);
#pragma unroll
      for (int c = 0; c < 16; ++c)
        P[(size_t)(cb * 16 + c) * kPStride + tid] = __uint_as_float(v[c]) * Us[(size_t)(cb * 16 + c) * F + tid];
    }
    __syncthreads();
    // sum over k of each column by a pair of neighbouring threads (half of k
    // each, the second half in a rotated order so the pair reads distinct banks)
    {
      const int col = tid >> 1, half = tid & 1;
      const bool in = col < N && sh_live[col] != 0;
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
      if (in) {
        const float* row = P + (size_t)col * kPStride + (kTcK / 2) * half;
#pragma unroll 4
        for (int kk = 0; kk < kTcK / 2; kk += 4) {
          const int k = (kk + 16 * half) & (kTcK / 2 - 1);
          a0 += row[k];
          a1 += row[k + 1];
          a2 += row[k + 2];
          a3 += row[k + 3];
        }
      }
      float v = (a0 + a1) + (a2 + a3);
      v += __shfl_xor_sync(0xffffffffu, v, 1);
      if (in && half == 0) {
        const int orow = rowmap ? rowmap[row0 + col] : row0 + col;
        out[(size_t)orow * ostride + i] = sh_fac[col] * (double)v;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
  }
}

template <int MODE>
cudaError_t launch_tc_small(const unsigned char* Wt, const unsigned char* Kt, int Gp, int nrows, const int* flags,
                            const float* U32, const double* scal, const double* oscale, int nout, int ostride,
                            double* out, int* err, TcRows rows, cudaStream_t st) {
  const int N = (nrows + 15) / 16 * 16;
  if (N > kSmallN || small_smem(N, Gp) > kTcDynMax) return cudaErrorInvalidConfiguration;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_ssc_tc_small<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kTcDynMax);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  return launch_step_kernel(k_ssc_tc_small<MODE>, dim3(nout, 1), dim3(kTcThreads), small_smem(N, Gp), st, Wt, Kt,
                            Gp, nrows, N, flags, U32, scal, oscale, ostride, out, err, rows.nlive, rows.rowmap);
}

template <int H, int MODE>
cudaError_t launch_tc(const unsigned char* Wt, const unsigned char* Kt, int Gp, int nrows, const int* flags,
                      const float* U32, const double* scal, const double* oscale, int nout, int ostride, double* out,
                      int* err, TcRows rows, cudaStream_t st) {
  constexpr int F = kTcK * H;
  const int N = std::min(kTcCols, (nrows + 15) / 16 * 16);
  const TcPlan plan = tc_plan(F, N, Gp * (MODE == kTcTf32 ? 2 : 1));
  if (plan.smem > kTcDynMax) return cudaErrorInvalidConfiguration;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_ssc_tc<H, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kTcDynMax);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid(nout, (nrows + kTcCols - 1) / kTcCols);
  return launch_step_kernel(k_ssc_tc<H, MODE>, grid, dim3(kTcThreads), plan.smem, st, Wt, Kt, Gp, nrows, N, plan.S,
                            plan.body, plan.ubytes, plan.uring, flags, U32, scal, oscale, ostride, out, err,
                            rows.nlive, rows.rowmap);
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
  Bt.assign((size_t)F * tc_tile_elems(N, Gp), 0);
  for (int i = 0; i < F; ++i) {
    uint16_t* Bi = Bt.data() + (size_t)i * tc_tile_elems(N, Gp);
    for (int n = 0; n < N; ++n)
      for (int j = 0; j < Gp; ++j) {
        const float v = K32[((size_t)i * Gp + j) * F + n];  // K[i][j][k = n]
        const uint16_t h = bf16_bits(v);
        Bi[tc_operand_offset(n, j, N, Gp, false)] = h;
        Bi[tc_operand_offset(n, j, N, Gp, true)] = bf16_bits(v - bf16_value(h));
      }
  }
}

float tf32_round(float x) {  // round to nearest even at TF32 precision (finite inputs)
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u += 0xFFFu + ((u >> 13) & 1u);
  u &= ~0x1FFFu;
  float y;
  std::memcpy(&y, &u, 4);
  return y;
}

void build_ssc_tc_operand_tf32(const std::vector<float>& K32, int F, int Gp, std::vector<float>& Bt32) {
  const int N = F;
  Bt32.assign(tc_tile_bytes(N, Gp, 4) / 4 * F, 0.f);
  for (int i = 0; i < F; ++i) {
    float* Bi = Bt32.data() + tc_tile_bytes(N, Gp, 4) / 4 * i;
    for (int n = 0; n < N; ++n)
      for (int j = 0; j < Gp; ++j)
        Bi[tc_operand_byte_offset(n, j, N, Gp, 4, false) / 4] = tf32_round(K32[((size_t)i * Gp + j) * F + n]);
  }
}

namespace {

// ---- autotuner --------------------------------------------------------------
// A choice of kernel for one contraction shape: the slab-per-CTA kernel, or
// the blastwave-row kernel with its chunks per stage and CTA target.
struct TcChoice {
  int kind = 0;  // 0: slab per CTA, 1: blastwaves on rows, 2: slab per CTA for small batches
  RowsCfg cfg;
  float ms = -1.f;  // measured time (-1: default, not measured)
};
struct TcKey {
  int mode, F, Gp, nout, octave;
  bool operator<(const TcKey& o) const {
    return std::tie(mode, F, Gp, nout, octave) < std::tie(o.mode, o.F, o.Gp, o.nout, o.octave);
  }
};
std::mutex g_tune_mu;
std::map<TcKey, TcChoice> g_tune;
bool g_tune_on = [] {
  const char* e = std::getenv("PBAG_AUTOTUNE");
  return !(e && e[0] == '0');
}();

int octave(int n) {
  int o = 0;
  while ((1 << (o + 1)) <= n) ++o;
  return o;
}

cudaError_t launch_slab(int mode, int F, int Gp, const void* Wt, const void* Kt, int nrows, const int* flags,
                        const float* U32, const double* scal, const double* oscale, int nout, int ostride, double* out,
                        int* err, TcRows rows, cudaStream_t st) {
  const auto* w = static_cast<const unsigned char*>(Wt);
  const auto* k = static_cast<const unsigned char*>(Kt);
#define PBAG_TC_CASE(HH, MM) \
  return launch_tc<HH, MM>(w, k, Gp, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows, st)
  if (F == 128) {
    if (mode == kTcSplit) PBAG_TC_CASE(1, kTcSplit);
    if (mode == kTcBf16) PBAG_TC_CASE(1, kTcBf16);
    if (mode == kTcTf32) PBAG_TC_CASE(1, kTcTf32);
  }
  if (F == 256) {
    if (mode == kTcSplit) PBAG_TC_CASE(2, kTcSplit);
    if (mode == kTcBf16) PBAG_TC_CASE(2, kTcBf16);
    if (mode == kTcTf32) PBAG_TC_CASE(2, kTcTf32);
  }
#undef PBAG_TC_CASE
  return cudaErrorInvalidValue;
}

}  // namespace

void ssc_tune_enable(bool on) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_on = on;
}

int ssc_tune_report(char* buf, int len) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::string r;
  for (const auto& kv : g_tune) {
    char line[200];
    std::snprintf(line, sizeof line, "mode=%d F=%d Gp=%d nout=%d rows~2^%d -> %s cps=%d ctas=%d lsu=%d %.3f ms\n",
                  kv.first.mode, kv.first.F, kv.first.Gp, kv.first.nout, kv.first.octave,
                  kv.second.kind == 1 ? "rows" : kv.second.kind == 2 ? "slab-small" : "slab", kv.second.cfg.cps, kv.second.cfg.ctas, kv.second.cfg.lsu,
                  kv.second.ms);
    r += line;
  }
  if (buf && len > 0) {
    std::strncpy(buf, r.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)r.size();
}

cudaError_t launch_ssc_tc_mode(int mode, int F, int Gp, const void* Wt, const void* Kt, int nrows,
                               const int* flags, const float* U32, const double* scal, const double* oscale, int nout,
                               int ostride, double* out, int* err, cudaStream_t st, TcRows rows) {
  if (nrows <= 0) return cudaSuccess;
  if (!Wt || !Kt || Gp % 16 != 0) return cudaErrorInvalidValue;
  const bool rows_ok = ssc_rows_supported(F, Gp, mode);
  const bool small_ok = F == kTcK && nrows <= kSmallN && (mode == kTcSplit || mode == kTcBf16);
  auto run = [&](const TcChoice& c) {
    const auto* w = static_cast<const unsigned char*>(Wt);
    const auto* k = static_cast<const unsigned char*>(Kt);
    if (c.kind == 2)
      return mode == kTcSplit
                 ? launch_tc_small<kTcSplit>(w, k, Gp, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows,
                                             st)
                 : launch_tc_small<kTcBf16>(w, k, Gp, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows,
                                            st);
    return c.kind ? launch_ssc_rows(mode, Gp, Wt, Kt, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows,
                                    c.cfg, st)
                  : launch_slab(mode, F, Gp, Wt, Kt, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows,
                                st);
  };
  // an explicit kernel choice (environment PBAG_TC_KERNEL = slab | rows |
  // slab-small) overrides the tuner where that kernel takes the shape
  if (const char* force = std::getenv("PBAG_TC_KERNEL")) {
    TcChoice c;
    c.kind = !std::strcmp(force, "rows") && rows_ok ? 1 : !std::strcmp(force, "slab-small") && small_ok ? 2 : 0;
    if (c.kind || !std::strcmp(force, "slab")) return run(c);
  }
  const TcKey key{mode, F, Gp, nout, octave(nrows)};
  TcChoice choice;
  bool known = false, tune = false;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      choice = it->second;
      known = true;
    }
    tune = g_tune_on;
  }
  if (!known) {
    choice.kind = nrows >= kRowsMin && rows_ok ? 1 : 0;  // the default without measurements
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    // candidates are timed only on rows whose output the caller discards or
    // overwrites anyway (each launch writes the same values), never inside a
    // graph capture, and never with a device-side row count (its rows are not
    // known here)
    if (tune && !rows.nlive && cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
      std::vector<TcChoice> cand;
      cand.push_back(TcChoice{});
      if (small_ok) {
        TcChoice c;
        c.kind = 2;
        cand.push_back(c);
      }
      if (rows_ok)
        for (int lsu : {0, 1})
          for (int cps : {1, 2, 3})
            for (int ctas : {2 * 152, 4 * 152, 8 * 152}) {
              TcChoice c;
              c.kind = 1;
              c.cfg.cps = cps;
              c.cfg.ctas = ctas;
              c.cfg.lsu = lsu;
              cand.push_back(c);
            }
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
        float best = 1e30f;
        for (TcChoice& c : cand) {
          if (run(c) != cudaSuccess) continue;  // warm-up (a shape the kernel refuses is skipped)
          cudaEventRecord(e0, st);
          run(c);
          cudaEventRecord(e1, st);
          float ms = 0.f;
          if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) continue;
          c.ms = ms;
          if (ms < best) {
            best = ms;
            choice = c;
          }
        }
      }
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      cudaGetLastError();
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[key] = choice;
    }
  }
  return run(choice);
}

cudaError_t launch_ssc_tc(const DevGrid& g, const DevState& S, const uint16_t* Bt, int nbw, bool split,
                          cudaStream_t st) {
  if (!S.Abf || !Bt) return cudaErrorInvalidValue;
  return launch_ssc_tc_mode(split ? kTcSplit : kTcBf16, g.F, g.Gp, S.Abf, Bt, nbw, S.flags, S.U32, S.scal, g.hnu,
                            g.F, g.F, S.jssc, S.err, st);
}

}  // namespace pbag

extern "C" {

int pbag_autotune(int enable) {
  pbag::ssc_tune_enable(enable != 0);
  return PBAG_OK;
}

int pbag_autotune_report(char* buf, int len) { return pbag::ssc_tune_report(buf, len); }

}  // extern "C"
