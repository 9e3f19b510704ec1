// pbag_ssc_rows.cu - the SSC contraction of large batches with blastwaves on
// the accumulator rows.
//
// computeSSCSpectrum (numeric_model.h:247-285) for state b and output slab o
// is j[b][o] = s_o sW_b sU_b sum_k U[b][k] D_o[b][k], D_o[b][k] = sum_j
// W[b][j] K_o[k][j]. Here the GEMM is oriented M = blastwaves (128 per CTA,
// one per tensor-memory lane), N = k (F = 128 columns), K-dim = j: the sum over
// k then runs inside each epilogue thread over its own accumulator row, with
// that blastwave's U row held in registers. One CTA keeps its 128 weight rows
// W (the A operand: hi and lo BF16 parts, hi only in plain BF16) resident in
// shared memory and streams the kernel slabs of a group of outputs o through
// as deep a ring of stages as the rest of shared memory holds; the
// accumulator is double-buffered in tensor memory, so the epilogue of output o
// overlaps the MMAs of output o+1. Warp roles: four epilogue warps, one MMA
// warp (one thread issues), one copy warp (one thread issues).
//
// Compared with the slab-per-CTA kernel (pbag_ssc_tc.cu), W and U are read
// once per CTA instead of once per output, and the per-CTA fixed costs are
// paid once per group of outputs; for small batches that kernel keeps every SM
// busy with one output each and stays the choice.
//
// Every wait is bounded: on a timeout the CTA records PBAG_ERR_TIMEOUT for its
// blastwaves, waits (bounded) for its copies and MMAs, frees its tensor memory
// and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pbag.h"
#include "pbag_kernels.h"
#include "pbag_tc.cuh"

namespace pbag {

namespace {

using tc::smem_u32;

constexpr int kRwRows = 128;                 // blastwaves per CTA
constexpr int kRwF = 128;                    // frequency grid (MMA N)
constexpr int kRwEpiWarps = 4;
constexpr int kRwThreads = 32 * (kRwEpiWarps + 2);
constexpr int kRwK8 = kTcChunk16;            // 16-byte K columns of a full chunk
// bytes of a full chunk (4 16-byte K columns) of the A rows: hi + lo parts
// (split BF16) or the hi part alone (plain BF16)
__host__ __device__ constexpr uint32_t rw_a_chunk(bool split) { return (split ? 2u : 1u) * kRwRows * kRwK8 * 16; }
// A stage of the slab ring holds cps consecutive chunks of one output, copied
// as one bulk copy (a chunk is its hi part, then its lo part, so consecutive
// chunks are contiguous); plain BF16 with one chunk per stage copies the hi
// part alone.
constexpr uint32_t kRwChunkBytes = 2u * kRwF * kRwK8 * 16;
__host__ __device__ constexpr uint32_t rw_stage(bool split, int cps) {
  return (!split && cps == 1) ? kRwChunkBytes / 2 : (uint32_t)cps * kRwChunkBytes;
}
constexpr size_t kRwDynMax = 231424;
constexpr int kRwMaxStages = 14;
constexpr int kRwLsuDepth = 3;  // stages of 16-byte copies in flight per copy warp

struct RwPlan {
  int S, cps;
  size_t smem;
};
inline RwPlan rw_plan(int Gp, bool split, int cps) {
  const int nchunks = (Gp / 8 + kRwK8 - 1) / kRwK8;
  cps = std::max(1, std::min(cps, nchunks));
  const size_t fixed = 1024 + (size_t)nchunks * rw_a_chunk(split);
  const size_t st = rw_stage(split, cps);
  RwPlan p;
  p.cps = cps;
  p.S = fixed + 2 * st > kRwDynMax ? 0 : (int)std::min<size_t>(kRwMaxStages, (kRwDynMax - fixed) / st);
  p.smem = fixed + (size_t)p.S * st;
  return p;
}

template <int MODE>
__global__ void __launch_bounds__(kRwThreads, 1)
k_ssc_rows(const unsigned char* __restrict__ Wt, const unsigned char* __restrict__ Kt, int Gp, int nrows, int gsz,
           int nout, int S, int cps, int lsu, const int* __restrict__ flags, const float* __restrict__ U32,
           const double* __restrict__ scal, const double* __restrict__ oscale, int ostride, double* __restrict__ out,
           int* __restrict__ err, const int* __restrict__ nlive, const int* __restrict__ rowmap) {
  constexpr bool kSplit = MODE == kTcSplit;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t bars[2 * kRwMaxStages + 6];  // full[S], empty[S], A, tfull[2], tempty[2], done
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kRwRows;
  grid_dep_wait();  // the weights, flags and row counts of the step's evolve launch
  grid_dep_launch();
  if (nlive && row0 >= *nlive) return;  // a tile beyond the rows counted on the device
  const int o0 = blockIdx.y * gsz, no = min(gsz, nout - o0);
  if (no <= 0) return;
  const int nk8 = Gp / 8, nchunks = (nk8 + kRwK8 - 1) / kRwK8;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t kAChunk = rw_a_chunk(kSplit);
  const uint32_t kStage = rw_stage(kSplit, cps);
  const bool hi_only = !kSplit && cps == 1;  // stage holds hi parts only
  const int nst = (nchunks + cps - 1) / cps;  // stages per output
  unsigned char* As = base;  // [chunk][hi | lo] of the 128 rows
  unsigned char* ring = base + (size_t)nchunks * kAChunk;
  const uint32_t abar = smem_u32(&bars[2 * kRwMaxStages]);
  const uint32_t tfull0 = smem_u32(&bars[2 * kRwMaxStages + 1]), tempty0 = smem_u32(&bars[2 * kRwMaxStages + 3]);
  const uint32_t done = smem_u32(&bars[2 * kRwMaxStages + 5]);
  auto full = [&](int s) { return smem_u32(&bars[s]); };
  auto empty = [&](int s) { return smem_u32(&bars[kRwMaxStages + s]); };
  if (tid == 0) {
    fail = 0;
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(full(s), 1);
      tc::mbar_init(empty(s), 1);
    }
    tc::mbar_init(abar, 1);
    for (int d = 0; d < 2; ++d) {
      tc::mbar_init(tfull0 + 8 * d, 1);
      tc::mbar_init(tempty0 + 8 * d, 32 * kRwEpiWarps);
    }
    tc::mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)(2 * kRwF)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const int total = no * nst;  // slab stages to stream
  // the CTAs of a wave start at different outputs, so that they do not all
  // request the same slab lines from the same L2 slices at once
  const int rot = (int)((blockIdx.x * 37u) % (unsigned)no);
  auto out_of = [&](int ol) { return o0 + (ol + rot) % no; };

  if (warp == kRwEpiWarps + 1) {
    // copies: the CTA's weight rows once, then the slab chunks of its outputs
    if (lane == 0) {
      const int tile = row0 / kTcCols, h = (row0 % kTcCols) / kRwRows;
      const unsigned char* Wtile = Wt + (size_t)tile * tc_tile_bytes(kTcCols, Gp, 2);
      uint32_t abytes = 0;
      for (int c = 0; c < nchunks; ++c) abytes += (kSplit ? 2u : 1u) * kRwRows * min(kRwK8, nk8 - c * kRwK8) * 16;
      tc::mbar_expect_tx(abar, abytes);
      for (int c = 0; c < nchunks; ++c) {
        const uint32_t kc = (uint32_t)min(kRwK8, nk8 - c * kRwK8), part = kRwRows * kc * 16;
        const unsigned char* src = Wtile + (size_t)2 * kTcCols * kRwK8 * 16 * c + (size_t)h * part;
        tc::bulk_g2s(smem_u32(As + (size_t)c * kAChunk), src, part, abar);
        if (kSplit)
          tc::bulk_g2s(smem_u32(As + (size_t)c * kAChunk + part), src + (size_t)kTcCols * kc * 16, part, abar);
      }
    }
    // the slab stages: source, bytes
    auto stage_src = [&](int g, uint32_t& bytes) {
      const int ol = g / nst, c0 = (g % nst) * cps, c1 = min(c0 + cps, nchunks);
      bytes = 0;
      for (int c = c0; c < c1; ++c) bytes += (hi_only ? 1u : 2u) * kRwF * min(kRwK8, nk8 - c * kRwK8) * 16;
      return Kt + (size_t)out_of(ol) * tc_tile_bytes(kRwF, Gp, 2) + (size_t)kRwChunkBytes * c0;
    };
    if (!lsu) {
      // one bulk copy per stage, issued by one thread
      if (lane == 0) {
        int g = 0;
        for (; g < total && !fail; ++g) {
          const int s = g % S;
          if (g >= S && !tc::mbar_wait_spin(empty(s), (uint32_t)(g / S - 1) & 1)) {
            fail = 1;
            break;
          }
          uint32_t bytes;
          const unsigned char* src = stage_src(g, bytes);
          tc::mbar_expect_tx(full(s), bytes);
          tc::bulk_g2s(smem_u32(ring + (size_t)s * kStage), src, bytes, full(s));
        }
        // copies still in flight complete before the CTA exits (bounded waits)
        for (int q = max(0, g - S); q < g; ++q) tc::mbar_wait(full(q % S), (uint32_t)(q / S) & 1);
      }
    } else {
      // 16-byte asynchronous copies by the whole warp, kRwLsuDepth stages in
      // flight; a stage is signalled (proxy fence, then one arrival) once its
      // copies have landed
      int g = 0, q = 0;
      auto signal = [&](int qq) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(full(qq % S));
      };
      for (; g < total; ++g) {
        const int s = g % S;
        int stop = 0;
        if (lane == 0) stop = fail || (g >= S && !tc::mbar_wait_spin(empty(s), (uint32_t)(g / S - 1) & 1));
        stop = __shfl_sync(0xffffffffu, stop, 0);
        if (stop) {
          if (lane == 0) fail = 1;
          break;
        }
        uint32_t bytes;
        const unsigned char* src = stage_src(g, bytes);
        const uint32_t dst = smem_u32(ring + (size_t)s * kStage);
        for (uint32_t off = (uint32_t)lane * 16; off < bytes; off += 32 * 16)
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + off), "l"(src + off) : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (g - q + 1 > kRwLsuDepth) {
          asm volatile("cp.async.wait_group %0;" ::"n"(kRwLsuDepth) : "memory");
          signal(q++);
        }
      }
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      if (g == total)
        while (q < g) signal(q++);
    }
    if (lane == 0) tc::mbar_wait(abar, 0);
  } else if (warp == kRwEpiWarps) {
    // MMAs
    if (lane == 0) {
      bool ok = tc::mbar_wait(abar, 0);
      const uint32_t idesc = tc::idesc_mma(kRwRows, kRwF, false);
      int g = 0;
      for (int ol = 0; ol < no && ok; ++ol) {
        const int d = ol & 1;
        if (ol >= 2 && !tc::mbar_wait_spin(tempty0 + 8 * d, (uint32_t)(ol / 2 - 1) & 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dt = tmem + (uint32_t)(d * kRwF);
        for (int q = 0; q < nst; ++q, ++g) {
          const int s = g % S;
          if (!tc::mbar_wait_spin(full(s), (uint32_t)(g / S) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          for (int c = q * cps; c < min(q * cps + cps, nchunks); ++c) {
            const uint32_t kc = (uint32_t)min(kRwK8, nk8 - c * kRwK8), sbo = kc * 128;
            const uint32_t a_hi = smem_u32(As + (size_t)c * kAChunk), a_lo = a_hi + kRwRows * kc * 16;
            const uint32_t b_hi = smem_u32(ring + (size_t)s * kStage + (size_t)(c - q * cps) * kRwChunkBytes);
            const uint32_t b_lo = b_hi + kRwF * kc * 16;
            for (uint32_t s2 = 0; s2 < kc / 2; ++s2) {
              const uint32_t ko = s2 * 256;  // two 16-byte K columns (K = 16) per MMA
              tc::mma_issue<false>(dt, tc::smem_desc(a_hi + ko, 128, sbo), tc::smem_desc(b_hi + ko, 128, sbo), idesc,
                                   (c > 0 || s2 > 0) ? 1u : 0u);
              if (kSplit) {
                tc::mma_issue<false>(dt, tc::smem_desc(a_hi + ko, 128, sbo), tc::smem_desc(b_lo + ko, 128, sbo),
                                     idesc, 1u);
                tc::mma_issue<false>(dt, tc::smem_desc(a_lo + ko, 128, sbo), tc::smem_desc(b_hi + ko, 128, sbo),
                                     idesc, 1u);
              }
            }
          }
          tc::mma_commit(empty(s));
        }
        if (ok) tc::mma_commit(tfull0 + 8 * d);
      }
      if (!ok) fail = 1;
      // every MMA issued is complete before the CTA exits
      tc::mma_commit(done);
      tc::mbar_wait(done, 0);
    }
  } else {
    // epilogue: thread = blastwave row
    const int q = warp, b = 32 * q + lane, r = row0 + b;
    float u[kRwF];  // this blastwave's U row
#pragma unroll
    for (int k4 = 0; k4 < kRwF / 4; ++k4) {
      float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < nrows) x = __ldg(reinterpret_cast<const float4*>(U32 + (size_t)r * kRwF) + k4);
      u[4 * k4] = x.x;
      u[4 * k4 + 1] = x.y;
      u[4 * k4 + 2] = x.z;
      u[4 * k4 + 3] = x.w;
    }
    const bool live = r < nrows && (flags[r] & kFlagActive);
    const double fac = live ? scal[(size_t)r * kScal + kScalSW] * scal[(size_t)r * kScal + kScalSU] : 0.;
    const int orow = live ? (rowmap ? rowmap[r] : r) : 0;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    bool ok = true;
    for (int ol = 0; ol < no; ++ol) {
      const int d = ol & 1;
      bool ready = false;
      for (int t = 0; t < 64 && !ready && !fail; ++t) ready = tc::mbar_wait_spin(tfull0 + 8 * d, (uint32_t)(ol / 2) & 1, 1 << 16);
      if (!ready) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
      // the row in two halves of four loads each, one wait per half
#pragma unroll
      for (int hb = 0; hb < kRwF / 64; ++hb) {
        uint32_t v[4][16];
#pragma unroll
        for (int x = 0; x < 4; ++x) tc::tmem_ld16_nowait(tl + (uint32_t)(d * kRwF + hb * 64 + x * 16), v[x]);
#pragma unroll
        for (int x = 0; x < 4; ++x) tc::tmem_wait_ld(v[x]);
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int i = 0; i < 16; i += 4) {
            const int k = hb * 64 + x * 16 + i;
            a0 = fmaf(__uint_as_float(v[x][i]), u[k], a0);
            a1 = fmaf(__uint_as_float(v[x][i + 1]), u[k + 1], a1);
            a2 = fmaf(__uint_as_float(v[x][i + 2]), u[k + 2], a2);
            a3 = fmaf(__uint_as_float(v[x][i + 3]), u[k + 3], a3);
          }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      tc::mbar_arrive(tempty0 + 8 * d);
      const int o = out_of(ol);
      if (live) out[(size_t)orow * ostride + o] = oscale[o] * fac * (double)((a0 + a1) + (a2 + a3));
    }
    if (!ok) {
      fail = 1;
      if (r < nrows && (flags[r] & kFlagActive)) atomicCAS(&err[4 * (rowmap ? rowmap[r] : r)], 0, PBAG_ERR_TIMEOUT);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (fail && warp < kRwEpiWarps) {
    const int r = row0 + 32 * warp + lane;
    if (r < nrows && (flags[r] & kFlagActive)) atomicCAS(&err[4 * (rowmap ? rowmap[r] : r)], 0, PBAG_ERR_TIMEOUT);
  }
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * kRwF)));
  }
}

template <int MODE>
cudaError_t launch_rows(const unsigned char* Wt, const unsigned char* Kt, int Gp, int nrows, const int* flags,
                        const float* U32, const double* scal, const double* oscale, int nout, int ostride, double* out,
                        int* err, TcRows rows, RowsCfg cfg, cudaStream_t st) {
  // three chunks per stage is the default (bulk copies cost a roughly fixed
  // latency each, so fewer and larger ones win over a deeper ring); the
  // autotuner of launch_ssc_tc_mode measures the alternatives
  RwPlan plan = rw_plan(Gp, MODE == kTcSplit, cfg.cps > 0 ? cfg.cps : 3);
  if (plan.S < 2) plan = rw_plan(Gp, MODE == kTcSplit, 1);
  // the warp-copy path keeps kRwLsuDepth stages in flight and needs one more to refill
  if (cfg.lsu && plan.S < kRwLsuDepth + 1) return cudaErrorInvalidConfiguration;
  if (plan.S < 2) return cudaErrorInvalidConfiguration;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_ssc_rows<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kRwDynMax);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  // groups of outputs: enough CTAs to fill the GPU several times over, at
  // least 8 outputs per CTA
  const int tiles = (nrows + kRwRows - 1) / kRwRows;
  const int target = cfg.ctas > 0 ? cfg.ctas : 4 * 152;
  int groups = std::max(1, std::min((target + tiles - 1) / tiles, nout / 8));
  const int gsz = (nout + groups - 1) / groups;
  groups = (nout + gsz - 1) / gsz;
  dim3 grid(tiles, groups);
  return launch_step_kernel(k_ssc_rows<MODE>, grid, dim3(kRwThreads), plan.smem, st, Wt, Kt, Gp, nrows, gsz, nout,
                            plan.S, plan.cps, cfg.lsu, flags, U32, scal, oscale, ostride, out, err, rows.nlive,
                            rows.rowmap);
}

}  // namespace

bool ssc_rows_supported(int F, int Gp, int mode) {
  return F == kRwF && (mode == kTcBf16 || mode == kTcSplit) && Gp % 16 == 0 &&
         rw_plan(Gp, mode == kTcSplit, 1).S >= 2;
}

cudaError_t launch_ssc_rows(int mode, int Gp, const void* Wt, const void* Kt, int nrows, const int* flags,
                            const float* U32, const double* scal, const double* oscale, int nout, int ostride,
                            double* out, int* err, TcRows rows, RowsCfg cfg, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const auto* w = static_cast<const unsigned char*>(Wt);
  const auto* k = static_cast<const unsigned char*>(Kt);
  if (mode == kTcSplit)
    return launch_rows<kTcSplit>(w, k, Gp, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows, cfg, st);
  if (mode == kTcBf16)
    return launch_rows<kTcBf16>(w, k, Gp, nrows, flags, U32, scal, oscale, nout, ostride, out, err, rows, cfg, st);
  return cudaErrorInvalidValue;
}

}  // namespace pbag
