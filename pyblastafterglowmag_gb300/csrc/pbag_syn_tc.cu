// pbag_syn_tc.cu - the synchrotron and SSA sums of the step on the tensor
// cores: computeSynSpectrum and computeSSA (numeric_model.h:148-238) with the
// kernel of SynKernel::evalSynKernel (kernels.h:528-538).
//
// The kernel K[k][j] = pref(B) R(x), x = nu_k xs / (nu_crit1(B) gamma_j^2),
// depends on the blastwave's field B, so as written it is no shared matrix.
// On the logarithmic grids it is one after a shift: ln nu_k = ln nu_0 + k dnu
// and ln gamma_j = j dlng give
//   ln x = k dnu - s - 2 j dlng,   s = ln nu_crit1(B) - ln nu_0 - ln xs.
// A bank of P matrices at sub-shifts p h (h = dnu / P),
//   K_p[m][j] = R(exp(m dnu - p h - 2 j dlng)),
// covers every s: with s / h = n + r (n integer, 0 <= r < 1), node n_a =
// n - 1 + a (a = 0..3) is q_a P + p_a, i.e. the shift q_a dnu + p_a h, whose
// kernel row for output k is row k - q_a of K_{p_a}. The blastwave's kernel
// is the cubic Lagrange interpolation over the four nodes, taken on the node
// sums D_p = K_p w (a plain GEMM of the fixed bank against the weights of
// every blastwave; N = 2 per blastwave: the synchrotron weights w and the SSA
// weights v):
//   sum_j K[k][j] w_j = pref interp_a(L_a(r), D_{p_a}[k - q_a]).
// The interpolation runs in log space where the four node values share a
// sign: on the exponential tail of the synchrotron function neighbouring
// nodes differ by orders of magnitude and a linear-space cubic swings
// negative there, while the log-space one stays within ~1e-5 of every entry
// (per-entry relative error, down to entries 1e-30 below the row's largest).
// Interpolation error ~1e-7 relative L2 with P = 8; split-BF16 operands with
// FP32 accumulation add ~3e-6 (synchrotron) and ~7e-6 (SSA, signed terms). CSYN's cyclotron bins (gamma <= 2) depend on nu / nu_Larmor
// and gamma separately: they stay out of the bank (zero columns) and the step
// completion adds them on CUDA cores.
//
// k_syn_tc: one CTA per (sub-shift p, 128-row tile of the bank, tile of
// blastwaves); the bank slab arrives by one bulk copy, the weight rows by one
// bulk copy per chunk and part, the MMAs (M = 128 rows m, N = weight rows, K =
// gamma) accumulate in tensor memory, the epilogue stores D_p as FP32 with the
// bank row fastest (thread = row), so the step completion reads contiguous
// rows. Every wait is bounded.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "pbag.h"
#include "pbag_internal.h"
#include "pbag_kernels.h"
#include "pbag_tc.cuh"

namespace pbag {

namespace {

using tc::idesc_mma;
using tc::mbar_wait;
using tc::mma_issue;
using tc::smem_desc;
using tc::smem_u32;

constexpr int kSbThreads = 128;
constexpr int kSbK8 = kTcChunk16;                // 16-byte K columns per operand chunk
constexpr size_t kSbDynMax = 231424;             // dynamic shared memory of a CTA
constexpr size_t kSbFixed = 1024 + 128;          // alignment slack and barriers

uint16_t bf16_bits_host(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float bf16_value_host(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float v;
  std::memcpy(&v, &u, 4);
  return v;
}

__device__ __forceinline__ size_t slab_bytes(int Gp) { return (size_t)2 * 128 * Gp * 2; }

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// rpb: weight rows per blastwave (2: synchrotron and SSA, 1: synchrotron
// only); tbw blastwaves per stored tile of rpb tbw rows. scal: the per-
// blastwave scalars (the bank shift at kScalSynShift), F: outputs per
// blastwave, mlo: index of the bank's first row.
template <bool kSplit>
__global__ void __launch_bounds__(kSbThreads, 1)
k_syn_tc(const unsigned char* __restrict__ bank, const unsigned char* __restrict__ Sbf, int Gp, int nbw, int tbw,
         int rpb, int Mt, int P, int F, int mlo, const int* __restrict__ flags, const double* __restrict__ scal,
         float* __restrict__ D, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t bars[2];  // copies, MMAs
  __shared__ uint32_t tmem_slot;
  __shared__ int fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int p = blockIdx.x / Mt, mt = blockIdx.x % Mt, tile = blockIdx.y;
  const int b0 = tile * tbw, nb = min(tbw, nbw - b0);
  const int rows_tile = rpb * tbw;          // weight rows of a stored tile
  const int N = (rpb * nb + 15) / 16 * 16;  // weight rows this CTA multiplies
  const int M = Mt * 128;
  // does an active blastwave of the tile read a row of this 128-row part of
  // the bank? Its shift s / h = n + r reads rows k - q - mlo, k < F, for the
  // nodes' q in [floor((n - 1) / P), floor((n + 2) / P)]
  bool mine = false;
  for (int b = tid; b < nb; b += kSbThreads) {
    if (!(flags[b0 + b] & kFlagActive)) continue;
    const int n = (int)floor(scal[(size_t)(b0 + b) * kScal + kScalSynShift]);
    const int lo = -floor_div(n + 2, P) - mlo, hi = F - 1 - floor_div(n - 1, P) - mlo;
    mine |= lo <= mt * 128 + 127 && hi >= mt * 128;
  }
  if (!__syncthreads_or(mine ? 1 : 0)) return;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* As = base;
  unsigned char* Bs = base + slab_bytes(Gp);
  const int nk8 = Gp / 8, nchunks = (nk8 + kSbK8 - 1) / kSbK8;
  if (tid == 0) {
    fail = 0;
    tc::mbar_init(smem_u32(&bars[0]), 1);
    tc::mbar_init(smem_u32(&bars[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const uint32_t abytes = (uint32_t)slab_bytes(Gp);
    const uint32_t bbytes = (uint32_t)(2u * N * Gp * 2u);
    tc::mbar_expect_tx(smem_u32(&bars[0]), abytes + bbytes);
    const unsigned char* A = bank + (size_t)(p * Mt + mt) * slab_bytes(Gp);
    for (uint32_t o = 0; o < abytes; o += 32768u)
      tc::bulk_g2s(smem_u32(As + o), A + o, min(32768u, abytes - o), smem_u32(&bars[0]));
    const unsigned char* W = Sbf + (size_t)tile * tc_tile_bytes(rows_tile, Gp, 2);
    for (int c = 0; c < nchunks; ++c) {
      const int kc = min(kSbK8, nk8 - c * kSbK8);
      for (int part = 0; part < 2; ++part)
        tc::bulk_g2s(smem_u32(Bs + (size_t)2 * N * kSbK8 * 16 * c + (size_t)part * N * kc * 16),
                     W + (size_t)2 * rows_tile * kSbK8 * 16 * c + (size_t)part * rows_tile * kc * 16,
                     (uint32_t)(N * kc * 16), smem_u32(&bars[0]));
    }
  }
  uint32_t ncols = 32;
  while (ncols < (uint32_t)N) ncols <<= 1;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    bool ok = mbar_wait(smem_u32(&bars[0]), 0);
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t idesc = idesc_mma(128, N, false);
      for (int c = 0; c < nchunks; ++c) {
        const int kc = min(kSbK8, nk8 - c * kSbK8);
        const uint32_t sbo = (uint32_t)kc * 128;
        const uint32_t a_hi = smem_u32(As + (size_t)2 * 128 * kSbK8 * 16 * c), a_lo = a_hi + 128u * kc * 16;
        const uint32_t b_hi = smem_u32(Bs + (size_t)2 * N * kSbK8 * 16 * c), b_lo = b_hi + (uint32_t)N * kc * 16;
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
      tc::mma_commit(smem_u32(&bars[1]));
      ok = mbar_wait(smem_u32(&bars[1]), 0);
    } else {
      mbar_wait(smem_u32(&bars[0]), 0);  // let the copies land before the CTA winds down
    }
    if (!ok) {
      fail = 1;
      for (int b = 0; b < nb; ++b)
        if (flags[b0 + b] & kFlagActive) atomicCAS(&err[4 * (b0 + b)], 0, PBAG_ERR_TIMEOUT);
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!fail) {
    // D_p rows m = mt 128 + tid, column col = weight row; stored [col][m]
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    float* Dt = D + ((size_t)tile * P + p) * (size_t)rows_tile * M + (size_t)mt * 128 + tid;
    for (int cb = 0; cb < N / 16; ++cb) {
      uint32_t v[16];
      tc::tmem_ld16(tl + (uint32_t)(cb * 16), v);
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int col = cb * 16 + c;
        if (col < rpb * nb) Dt[(size_t)col * M] = __uint_as_float(v[c]);
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

}  // namespace

// ---- host -----------------------------------------------------------------

int syn_tc_tile_bw(int Gp) {
  const size_t a = (size_t)2 * 128 * Gp * 2;
  if (a + kSbFixed >= kSbDynMax) return 0;
  const int t = (int)((kSbDynMax - kSbFixed - a) / ((size_t)8 * Gp)) & ~7;
  return std::min(t, 128);
}

bool syn_tc_supported(int G, int F) {
  const int Gp = (G + 15) / 16 * 16;
  return G >= 8 && F >= 8 && syn_tc_tile_bw(Gp) >= 8;
}

void syn_tc_geometry(double dnu, double nu0, double xs_gsl, int F, SynBankGeom* g) {
  g->P = kSynBankP;
  g->h = dnu / g->P;
  // the bank covers fields B in [kSynBankBmin, kSynBankBmax] for every method
  // (xs = 1, or the GSL method's scale): the shifts s / h there, with the
  // interpolation's reach of one node below and two above
  const double ncrit1 = 3. * cgs::q_e / (4. * M_PI * cgs::m_e * cgs::c_light);  // nu_crit1 / B
  const double s_lo = std::log(ncrit1 * kSynBankBmin) - std::log(nu0) - std::max(0., std::log(xs_gsl));
  const double s_hi = std::log(ncrit1 * kSynBankBmax) - std::log(nu0) - std::min(0., std::log(xs_gsl));
  g->n_lo = (int)std::floor(s_lo / g->h) - 1;
  g->n_hi = (int)std::floor(s_hi / g->h) + 2;
  const int q_lo = (int)std::floor((double)g->n_lo / g->P), q_hi = (int)std::floor((double)g->n_hi / g->P);
  g->mlo = -q_hi;
  g->M = (F + q_hi - q_lo + 127) / 128 * 128;
}

void build_syn_bank(int method, int jc, const double* gam, int G, int Gp, double dnu, const SynBankGeom& sg,
                    std::vector<uint16_t>& out) {
  const int Mt = sg.M / 128;
  const double dlng = std::log(gam[1] / gam[0]);
  out.assign((size_t)sg.P * Mt * tc_tile_elems(128, Gp), 0);
  std::vector<double> lg2(G);
  for (int j = 0; j < G; ++j) lg2[j] = 2. * j * dlng;
  for (int p = 0; p < sg.P; ++p)
    for (int mt = 0; mt < Mt; ++mt) {
      uint16_t* S = out.data() + (size_t)(p * Mt + mt) * tc_tile_elems(128, Gp);
      for (int r = 0; r < 128; ++r) {
        const int m = sg.mlo + mt * 128 + r;
        for (int j = jc; j < G - 1; ++j) {  // w_{G-1} = 0 (numeric_model.h:157)
          const double lx = m * dnu - p * sg.h - lg2[j];
          if (lx > std::log(kSynTabXmax)) continue;  // R < e^-120: zero
          const float v = (float)syn_shape(method, std::exp(lx));
          const uint16_t hi = bf16_bits_host(v);
          S[tc_operand_offset(r, j, 128, Gp, false)] = hi;
          S[tc_operand_offset(r, j, 128, Gp, true)] = bf16_bits_host(v - bf16_value_host(hi));
        }
      }
    }
}

cudaError_t launch_syn_tc(const DevGrid& g, const DevState& S, int nbw, cudaStream_t st, int rpb) {
  if (nbw <= 0) return cudaSuccess;
  const int tbw = g.sb_tbw * 2 / rpb, Mt = g.sb_M / 128;
  const int ntiles = (nbw + tbw - 1) / tbw;
  const int nmax = (rpb * std::min(tbw, nbw) + 15) / 16 * 16;
  const size_t smem = 1024 + (size_t)2 * 128 * g.Gp * 2 + (size_t)2 * nmax * g.Gp * 2 + 64;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_syn_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSbDynMax);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_syn_tc<true><<<dim3(g.sb_P * Mt, ntiles), kSbThreads, smem, st>>>(
      reinterpret_cast<const unsigned char*>(g.synbank), reinterpret_cast<const unsigned char*>(S.Sbf), g.Gp, nbw,
      tbw, rpb, Mt, g.sb_P, g.F, g.sb_mlo, S.flags, S.scal, S.Dsyn, S.err);
  return cudaGetLastError();
}

}  // namespace pbag
