// pbag_limits.cu - the per-step shock scalars of a whole batch on the GPU
// (updateSockProperties + computeEleSpectrumLimits, microphysics_base.h:
// 575-966, for every recorded state of every blastwave), for callers that know
// the whole history up front (post-processing mode) and keep it on the device.
//
// The reference calls computeEleSpectrumLimits once per burster time on one
// object, so the members it leaves carry from call to call. Almost all of one
// call's result depends on that call's state alone: B, gamma_min, gamma_max,
// gamma_c, Theta and z_cool are recomputed by every call that passes
// checkParams (the constant gamma_max / gamma_c methods keep their initial
// values, capped the same way every time), while accel_frac keeps its earlier
// value unless the non-relativistic branch assigns it, and a refused call
// changes nothing. So k_limits_states evaluates every state in parallel (one
// thread each, the FP64 arithmetic of pbag_limits.cuh), and k_limits_carry
// resolves the two carries per blastwave with one warp: each state takes its
// fields from the last accepted state at or before it, and accel_frac from the
// last state that assigned it (the initial members where there is none). The
// one case whose arithmetic reads an earlier call's result - the bisection of
// gammaMinFunc at p = 1 or 2, whose branches use the member gamma_min - runs
// state after state in one thread per blastwave instead (k_limits_serial).
//
// Results agree with the host prep to rounding: the device pow / log differ
// from the host's in the last bits, so a bisection step can (rarely) go the
// other way at a midpoint where gammaMinFunc is within rounding of zero.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_limits.cuh"

namespace pbag {
namespace {

constexpr int kLimThreads = 128;
enum : unsigned char { kLimValid = 1, kLimAccel = 2 };

__device__ __forceinline__ int owner_of(const int64_t* __restrict__ off, int nbw, int64_t r) {
  int lo = 0, hi = nbw;  // last b with off[b] <= r
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= r) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void load_state(LimState& s, const double* st) {
  s.gamma_min = st[0], s.gamma_max = st[1], s.gamma_c = st[2], s.accel_frac = st[3];
  s.B = st[4], s.Theta = st[5], s.z_cool = st[6];
}

// the first failure of a blastwave: lowest state index, then its code
__device__ __forceinline__ void note_failure(unsigned long long* fail, int b, int64_t step, int code) {
  atomicMin(fail + b, ((unsigned long long)step << 8) | (unsigned long long)(unsigned char)(-code));
}

__device__ __forceinline__ bool serial_case(const pbag_limits_opts& o) {
  return o.method_gamma_min == 1 && (o.p == 1. || o.p == 2.);
}

__global__ void __launch_bounds__(kLimThreads)
k_limits_states(const pbag_limits_opts* __restrict__ opts, int nbw, const int64_t* __restrict__ off, int64_t n,
                const pbag_shock_state* __restrict__ in, const double* __restrict__ state0,
                const double* __restrict__ gam, int G, pbag_limits* __restrict__ out, unsigned char* __restrict__ bits,
                unsigned long long* __restrict__ fail) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int b = owner_of(off, nbw, r);
  const pbag_limits_opts o = opts[b];
  if (serial_case(o)) return;
  LimState s{};
  s.o = &o;
  load_state(s, state0 + (size_t)7 * b);
  int valid = 0, aset = 0;
  const int rc = lim_one(s, in[r], gam[0], gam[G - 1], &valid, &aset);
  if (rc != PBAG_OK) note_failure(fail, b, r - off[b], rc);
  lim_store(s, valid, out[r]);
  bits[r] = (unsigned char)((valid ? kLimValid : 0) | (valid && aset ? kLimAccel : 0));
}

// one warp per blastwave: the carries of consecutive states
__global__ void __launch_bounds__(kLimThreads)
k_limits_carry(const pbag_limits_opts* __restrict__ opts, int nbw, const int64_t* __restrict__ off,
               double* __restrict__ state, pbag_limits* __restrict__ out, const unsigned char* __restrict__ bits) {
  const int b = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nbw || serial_case(opts[b])) return;
  const int64_t r0 = off[b], r1 = off[b + 1];
  double* st = state + (size_t)7 * b;
  // the members before the first state, as an accepted state's fields
  pbag_limits init{};
  init.B = st[4], init.gamma_min = st[0], init.gamma_max = st[1], init.gamma_c = st[2];
  init.accel_frac = st[3], init.Theta = st[5], init.z_cool = st[6];
  int64_t cv = -1, ca = -1;  // last accepted state / last accel_frac assignment so far (-1: the initial members)
  for (int64_t base = r0; base < r1; base += 32) {
    const int64_t r = base + lane;
    const bool in = r < r1;
    const unsigned char bb = in ? bits[r] : 0;
    const unsigned mv = __ballot_sync(0xffffffffu, bb & kLimValid);
    const unsigned ma = __ballot_sync(0xffffffffu, bb & kLimAccel);
    const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
    const unsigned lv = mv & upto, la = ma & upto;
    const int64_t iv = lv ? base + (31 - __clz(lv)) : cv;
    const int64_t ia = la ? base + (31 - __clz(la)) : ca;
    pbag_limits v = iv >= 0 ? out[iv] : init;
    v.accel_frac = ia >= 0 ? out[ia].accel_frac : init.accel_frac;
    v.valid = (bb & kLimValid) ? 1 : 0;
    __syncwarp();  // every lane has read its sources before any lane writes
    if (in) out[r] = v;
    __syncwarp();
    if (mv) cv = base + (31 - __clz(mv));
    if (ma) ca = base + (31 - __clz(ma));
  }
  if (lane == 0 && r1 > r0) {
    const pbag_limits& last = out[r1 - 1];
    st[0] = last.gamma_min, st[1] = last.gamma_max, st[2] = last.gamma_c, st[3] = last.accel_frac;
    st[4] = last.B, st[5] = last.Theta, st[6] = last.z_cool;
  }
}

// one thread per blastwave, call after call (the bisection at p = 1 or 2)
__global__ void __launch_bounds__(kLimThreads)
k_limits_serial(const pbag_limits_opts* __restrict__ opts, int nbw, const int64_t* __restrict__ off,
                const pbag_shock_state* __restrict__ in, double* __restrict__ state, const double* __restrict__ gam,
                int G, pbag_limits* __restrict__ out, unsigned long long* __restrict__ fail) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbw) return;
  const pbag_limits_opts o = opts[b];
  if (!serial_case(o)) return;
  LimState s{};
  s.o = &o;
  double* st = state + (size_t)7 * b;
  load_state(s, st);
  for (int64_t r = off[b]; r < off[b + 1]; ++r) {
    int valid = 0, aset = 0;
    const int rc = lim_one(s, in[r], gam[0], gam[G - 1], &valid, &aset);
    if (rc != PBAG_OK) {
      note_failure(fail, b, r - off[b], rc);
      return;
    }
    lim_store(s, valid, out[r]);
  }
  st[0] = s.gamma_min, st[1] = s.gamma_max, st[2] = s.gamma_c, st[3] = s.accel_frac;
  st[4] = s.B, st[5] = s.Theta, st[6] = s.z_cool;
}

__global__ void k_fill_u64(unsigned long long* p, int n, unsigned long long v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

}  // namespace
}  // namespace pbag

using namespace pbag;

extern "C" int pbag_shock_limits_device(pbag_ctx* ctx, int nbw, const int64_t* off,
                                        const pbag_limits_opts* d_opts, const pbag_shock_state* d_in,
                                        double* d_state, pbag_limits* d_out, pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || nbw < 0 || !off || (nbw > 0 && (!d_opts || !d_state))) return PBAG_ERR_ARG;
  if (off[0] != 0) return PBAG_ERR_ARG;
  for (int b = 0; b < nbw; ++b)
    if (off[b + 1] < off[b]) return PBAG_ERR_ARG;
  const int64_t n = nbw > 0 ? off[nbw] : 0;
  if (n > ((int64_t)1 << 40) || (n > 0 && (!d_in || !d_out))) return PBAG_ERR_ARG;
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (nbw == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  cudaStream_t s = v.stream;
  int64_t* d_off = nullptr;
  unsigned char* d_bits = nullptr;
  unsigned long long* d_fail = nullptr;
  cudaError_t e = cudaMalloc(&d_off, sizeof(int64_t) * (nbw + 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_bits, (size_t)(n > 0 ? n : 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_fail, sizeof(unsigned long long) * nbw);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_off, off, sizeof(int64_t) * (nbw + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_fill_u64<<<(nbw + 255) / 256, 256, 0, s>>>(d_fail, nbw, ~0ull);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && n > 0) {
    k_limits_states<<<(unsigned)((n + kLimThreads - 1) / kLimThreads), kLimThreads, 0, s>>>(
        d_opts, nbw, d_off, n, d_in, d_state, v.dg.e, v.G, d_out, d_bits, d_fail);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_limits_carry<<<(nbw * 32 + kLimThreads - 1) / kLimThreads, kLimThreads, 0, s>>>(d_opts, nbw, d_off, d_state,
                                                                                         d_out, d_bits);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_limits_serial<<<(nbw + kLimThreads - 1) / kLimThreads, kLimThreads, 0, s>>>(d_opts, nbw, d_off, d_in, d_state,
                                                                                    v.dg.e, v.G, d_out, d_fail);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> fail((size_t)nbw, ~0ull);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(fail.data(), d_fail, sizeof(unsigned long long) * nbw, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d_off);
  cudaFree(d_bits);
  cudaFree(d_fail);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? PBAG_ERR_NOMEM : PBAG_ERR_CUDA;
  ctx_set_launches(ctx, n > 0 ? 4 : 3);
  // the reference stops at its first failing call: the earliest step, then blastwave
  int code = PBAG_OK, fb = -1;
  int64_t fs = -1;
  for (int b = 0; b < nbw; ++b) {
    if (fail[b] == ~0ull) continue;
    const int64_t step = (int64_t)(fail[b] >> 8);
    if (fs < 0 || step < fs) {
      fs = step;
      fb = b;
      code = -(int)(fail[b] & 0xff);
    }
  }
  if (st) {
    st->code = code;
    st->bw = fb;
    st->step = (int)fs;
  }
  return code;
}
