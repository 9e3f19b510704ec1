// pbag_noalloc.cu - a variant of the batch step that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the moment they run the step: hosts
// that hand out device memory only through their own pool, or latency-critical
// loops where an allocation (and the implicit device synchronisation it may
// cause) is not acceptable. For them, pbag_run_batch_noalloc evolves a batch as
// pbag_run_batch_device does - same preparation, evolve and radiation kernels,
// results within the same tolerance - but keeps every intermediate buffer
// (per-blastwave state, per-record scalars, offsets, error records) in one
// file-scope __device__ array of fixed size instead of memory the context
// allocates on demand. Its SSC contraction is always the FP32 CUDA-core one
// (the tensor-core operand tiles would need more scratch), whatever
// pbag_set_ssc_path chose for the context. The call is synchronous: it reads
// the parameters back to validate them and waits for the batch to finish.
//
// That array is part of the loaded module: every GPU that loads the library
// holds its PBAG_NOALLOC_SCRATCH_BYTES until the process exits. All calls
// share it and it keeps the previous call's contents, so each call clears the
// parts that must start at zero, and calls that overlap on the GPU (from two
// host threads, or on two streams) race on it.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_kernels.h"

using namespace pbag;

namespace {

// The scratch itself. Host code only sees a host-side stand-in under this
// name; the device address comes from cudaGetSymbolAddress (below).
static __device__ __align__(256) unsigned char g_scratch[PBAG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_dev[kMaxDevices] = {};  // device address of g_scratch, per device

// Once per device, with that device current: look up the address of the
// scratch array (no allocation; the module already holds it).
int scratch_address(int device, unsigned char** p) {
  if (device < 0 || device >= kMaxDevices) return PBAG_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_dev[device]) {
    void* addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_scratch) != cudaSuccess || !addr) return PBAG_ERR_CUDA;
    g_scratch_dev[device] = addr;
  }
  *p = static_cast<unsigned char*>(g_scratch_dev[device]);
  return PBAG_OK;
}

// Bump carving of the scratch into 256-byte aligned pieces.
struct Carver {
  unsigned char* base;
  size_t used = 0;
  template <typename T>
  T* take(size_t n) {
    T* p = reinterpret_cast<T*>(base + used);
    used += (n * sizeof(T) + 255) / 256 * 256;
    return p;
  }
};

size_t scratch_need(int nbw, size_t nrec, int G, int F, int Gp) {
  Carver c{nullptr};
  const size_t n = (size_t)nbw;
  c.take<int64_t>(n + 1);
  c.take<int64_t>(n);
  for (int k = 0; k < 3; ++k) c.take<double>(n * G);  // f, dfde, powp
  c.take<double>(n * 3 * G);                          // gdot
  c.take<double>(n * F);                              // n
  c.take<float>(n * F);                               // syn32
  c.take<float2>(n * F);                              // ssa32
  c.take<float>(n * 4);                               // rad32
  c.take<double>(n * F);                              // jssc
  c.take<float>(n * Gp);                              // W32
  c.take<float>(n * F);                               // U32
  c.take<float>(n * G);                               // w32
  c.take<float>(n * G);                               // v32
  c.take<double>(n * kScal);
  c.take<int>(n);
  c.take<int>(n * 4);
  c.take<int>(4);  // first failure
  c.take<StepScal>(nrec);
  return c.used;
}

// First failure in time order, then blastwave order, into out[4].
__global__ void k_first_failure(const int* __restrict__ err, int nbw, int* __restrict__ out) {
  __shared__ long long best[256];
  long long key = LLONG_MAX;
  for (int b = threadIdx.x; b < nbw; b += blockDim.x)
    if (err[4 * b] != 0) {
      const long long k = ((long long)err[4 * b + 1] << 32) | (unsigned)b;
      key = k < key ? k : key;
    }
  best[threadIdx.x] = key;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && best[threadIdx.x + s] < best[threadIdx.x]) best[threadIdx.x] = best[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const long long k = best[0];
    if (k == LLONG_MAX) {
      out[0] = PBAG_OK;
      out[1] = -1;
      out[2] = -1;
      out[3] = 0;
    } else {
      const int b = (int)(k & 0xffffffffLL);
      out[0] = err[4 * b];
      out[1] = b;
      out[2] = err[4 * b + 1];
      out[3] = err[4 * b + 2];
    }
  }
}

int check_params_host(const CtxView& v, const pbag_shock_params* d_prm, int nbw) {
  pbag_shock_params chunk[64];  // validated in fixed-size pieces: no host allocation either
  for (int b0 = 0; b0 < nbw; b0 += 64) {
    const int n = nbw - b0 < 64 ? nbw - b0 : 64;
    if (cudaMemcpy(chunk, d_prm + b0, n * sizeof(pbag_shock_params), cudaMemcpyDeviceToHost) != cudaSuccess)
      return PBAG_ERR_CUDA;
    for (int k = 0; k < n; ++k) {
      const pbag_shock_params& p = chunk[k];
      if (p.pp_on && !p.ssc_on) return PBAG_ERR_PARAM;  // "PP requires SSC" (microphysics_base.h:394-397)
      if (p.syn_method < PBAG_SYN_CSYN || p.syn_method > PBAG_SYN_BESSEL) return PBAG_ERR_ARG;
      if (p.ele_method != PBAG_ELE_NUMERIC && p.ele_method != PBAG_ELE_MIX) return PBAG_ERR_ARG;
      if (p.max_substeps < 1 || !(p.p > 0.) || !std::isfinite(p.p)) return PBAG_ERR_ARG;
      if (p.ssc_on && !v.ssc) return PBAG_ERR_ARG;
    }
  }
  return PBAG_OK;
}

}  // namespace

extern "C" int pbag_run_batch_noalloc(pbag_ctx* ctx, const pbag_shock_params* d_prm, int nbw, const int64_t* off,
                                      const pbag_step_rec* d_recs, const pbag_outputs* d_out, pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
  CtxView v;
  if (!ctx_view(ctx, &v) || !d_out || !off || nbw < 0 || (nbw > 0 && (!d_prm || !d_recs))) return PBAG_ERR_ARG;
  if (off[0] != 0) return PBAG_ERR_ARG;
  if (nbw > 0 && off[nbw] > ((int64_t)1 << 40)) return PBAG_ERR_ARG;  // keeps scratch_need free of overflow
  int64_t max_len = 0;
  for (int b = 0; b < nbw; ++b) {
    if (off[b + 1] < off[b] || off[b + 1] - off[b] > ((int64_t)1 << 30)) return PBAG_ERR_ARG;
    max_len = off[b + 1] - off[b] > max_len ? off[b + 1] - off[b] : max_len;
  }
  const size_t nrec = (size_t)off[nbw];
  // the batch must fit the fixed scratch; report the need in KiB otherwise
  const size_t need = scratch_need(nbw, nrec, v.G, v.F, v.Gp);
  if (need > (size_t)PBAG_NOALLOC_SCRATCH_BYTES) {
    if (st) st->site = (int)((need + 1023) / 1024);
    return PBAG_ERR_ARG;
  }
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  unsigned char* base = nullptr;
  int rc = scratch_address(v.device, &base);
  if (rc != PBAG_OK) return rc;
  if ((rc = check_params_host(v, d_prm, nbw)) != PBAG_OK) {
    if (st) st->code = rc;
    return rc;
  }
  // carve the scratch (same order as scratch_need)
  Carver cv{base};
  DevState S{};
  const size_t n = (size_t)nbw;
  int64_t* d_off = cv.take<int64_t>(n + 1);
  int64_t* d_first = cv.take<int64_t>(n);
  S.f = cv.take<double>(n * v.G);
  S.dfde = cv.take<double>(n * v.G);
  S.powp = cv.take<double>(n * v.G);
  S.gdot = cv.take<double>(n * 3 * v.G);
  S.n = cv.take<double>(n * v.F);
  S.syn32 = cv.take<float>(n * v.F);
  S.ssa32 = cv.take<float2>(n * v.F);
  S.rad32 = cv.take<float>(n * 4);
  S.jssc = cv.take<double>(n * v.F);
  S.W32 = cv.take<float>(n * v.Gp);
  S.U32 = cv.take<float>(n * v.F);
  S.w32 = cv.take<float>(n * v.G);
  S.v32 = cv.take<float>(n * v.G);
  S.scal = cv.take<double>(n * kScal);
  S.flags = cv.take<int>(n);
  S.err = cv.take<int>(n * 4);
  int* d_fail = cv.take<int>(4);
  StepScal* d_ss = cv.take<StepScal>(nrec);
  cudaStream_t s = v.stream;
  // the scratch keeps the previous call's contents: clear what must start at zero
  auto z = [&](void* p, size_t bytes) { return bytes ? cudaMemsetAsync(p, 0, bytes, s) : cudaSuccess; };
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ok(cudaMemcpyAsync(d_off, off, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  ok(z(S.f, n * v.G * sizeof(double)));
  ok(z(S.dfde, n * v.G * sizeof(double)));
  ok(z(S.gdot, n * 3 * v.G * sizeof(double)));
  ok(z(S.n, n * v.F * sizeof(double)));
  ok(z(S.jssc, n * v.F * sizeof(double)));
  ok(z(S.U32, n * v.F * sizeof(float)));
  ok(z(S.W32, n * v.Gp * sizeof(float)));
  ok(z(S.scal, n * kScal * sizeof(double)));
  ok(z(S.flags, n * sizeof(int)));
  ok(z(S.err, n * 4 * sizeof(int)));
  // skipped steps keep zero output rows
  double* const* outp = reinterpret_cast<double* const*>(d_out);
  for (int fi = 0; fi < 13; ++fi)
    if (outp[fi] && nrec) ok(z(outp[fi], nrec * ((fi >= 4 && fi < 8) ? (size_t)v.G : (size_t)v.F) * sizeof(double)));
  if (e != cudaSuccess) return PBAG_ERR_CUDA;
  if (nbw > 0) {
    ok(launch_prepare(v.dg, S, d_recs, d_off, d_prm, nbw, (int64_t)nrec, d_first, d_ss, s));
    for (int64_t step = 0; step < max_len && e == cudaSuccess; ++step) {
      ok(launch_evolve(v.dg, S, d_recs, d_ss, d_off, d_prm, nbw, (int)step, *d_out, s));
      ok(launch_rad_ssc(v.dg, S, d_prm, nbw, v.ssc, (int)step, s));
    }
    if (max_len > 0) ok(launch_finalize(v.dg, S, d_off, d_prm, nbw, (int)(max_len - 1), *d_out, s));
  }
  int fail[4] = {PBAG_OK, -1, -1, 0};
  if (nbw > 0) {
    k_first_failure<<<1, 256, 0, s>>>(S.err, nbw, d_fail);
    ok(cudaGetLastError());
    ok(cudaMemcpyAsync(fail, d_fail, sizeof(fail), cudaMemcpyDeviceToHost, s));
  }
  ok(cudaStreamSynchronize(s));
  if (e != cudaSuccess) return PBAG_ERR_CUDA;
  // kernels of this call: preparation (3, or 2 without records), evolve and
  // radiation per step, the completion of the last step, the failure scan
  ctx_set_launches(ctx, nbw > 0 ? (nrec > 0 ? 3 : 2) + 2 * max_len + (max_len > 0 ? 1 : 0) + 1 : 0);
  if (st) {
    st->code = fail[0];
    st->bw = fail[1];
    st->step = fail[2];
    st->site = fail[3];
  }
  return fail[0];
}
