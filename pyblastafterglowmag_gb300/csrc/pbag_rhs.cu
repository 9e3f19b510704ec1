// pbag_rhs.cu - the blastwave ODE right-hand side for many blastwaves at once:
// one thread per blastwave state, the restatement of pbag_rhs.cuh (the
// reference's rhs_fs / rhs_fsrs and the pieces they call). pbag_bw_rhs runs
// the same code on the host.
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "pbag_ctx_view.h"
#include "pbag_rhs.cuh"

namespace pbag {
namespace {

constexpr int kRhsThreads = 128;

// The first failure by blastwave index: (b << 16) | (site << 2) | code class.
__global__ void __launch_bounds__(kRhsThreads) k_bw_rhs(int n, const pbag_bw_rhs_pars* __restrict__ pars,
                                                         pbag_bw_rhs_state* __restrict__ state, double* __restrict__ dydt,
                                                         unsigned long long* __restrict__ first) {
  const int b = blockIdx.x * kRhsThreads + threadIdx.x;
  if (b >= n) return;
  const pbag_bw_rhs_pars P = pars[b];
  pbag_bw_rhs_state S = state[b];
  double out[PBAG_Y_N];
  double* o = dydt + (size_t)b * PBAG_Y_N;
#pragma unroll
  for (int k = 0; k < PBAG_Y_N; ++k) out[k] = o[k];
  int site = 0;
  const int rc = rhs::rhs_one(P, S, out, &site);
  if (rc != PBAG_OK) {
    const unsigned long long cls = rc == PBAG_ERR_PARAM ? 1ull : rc == PBAG_ERR_UNSUPPORTED ? 2ull : 0ull;
    atomicMin(first, ((unsigned long long)b << 16) | ((unsigned long long)(site & 0x3fff) << 2) | cls);
    return;
  }
#pragma unroll
  for (int k = 0; k < PBAG_Y_N; ++k) o[k] = out[k];
  state[b] = S;
}

int code_of(unsigned long long cls) {
  return cls == 1ull ? PBAG_ERR_PARAM : cls == 2ull ? PBAG_ERR_UNSUPPORTED : PBAG_ERR_NONFINITE;
}

void status_arg(pbag_status* st) {
  if (st) {
    st->code = PBAG_ERR_ARG;
    st->bw = st->step = -1;
    st->site = 0;
  }
}

}  // namespace
}  // namespace pbag

using namespace pbag;

extern "C" int pbag_bw_rhs(int n, const pbag_bw_rhs_pars* pars, pbag_bw_rhs_state* state, double* dydt,
                           pbag_status* st) {
  status_arg(st);
  if (n < 0 || (n > 0 && (!pars || !state || !dydt))) return PBAG_ERR_ARG;
  for (int b = 0; b < n; ++b) {
    double* o = dydt + (size_t)b * PBAG_Y_N;
    int site = 0;
    const int rc = rhs::rhs_one(pars[b], state[b], o, &site);
    if (rc != PBAG_OK) {
      if (st) {
        st->code = rc;
        st->bw = b;
        st->site = site;
      }
      return rc;
    }
  }
  if (st) st->code = PBAG_OK;
  return PBAG_OK;
}

extern "C" int pbag_bw_rhs_device(pbag_ctx* ctx, int n, const pbag_bw_rhs_pars* d_pars, pbag_bw_rhs_state* d_state,
                                  double* d_dydt, pbag_status* st) {
  status_arg(st);
  CtxView v;
  if (!ctx_view(ctx, &v) || n < 0) return PBAG_ERR_ARG;
  if (n == 0) {
    if (st) st->code = PBAG_OK;
    return PBAG_OK;
  }
  if (!d_pars || !d_state || !d_dydt) return PBAG_ERR_ARG;
  if (cudaSetDevice(v.device) != cudaSuccess) return PBAG_ERR_CUDA;
  unsigned long long* d_first = nullptr;
  cudaError_t e = cudaMalloc(&d_first, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_first, 0xff, sizeof(unsigned long long), v.stream);
  if (e == cudaSuccess) {
    k_bw_rhs<<<(unsigned)((n + kRhsThreads - 1) / kRhsThreads), kRhsThreads, 0, v.stream>>>(n, d_pars, d_state,
                                                                                             d_dydt, d_first);
    e = cudaGetLastError();
  }
  unsigned long long first = ~0ull;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  cudaFree(d_first);
  ctx_set_launches(ctx, 1);
  if (e != cudaSuccess) return PBAG_ERR_CUDA;
  if (first != ~0ull) {
    const int code = code_of(first & 3ull);
    if (st) {
      st->code = code;
      st->bw = (int)(first >> 16);
      st->site = (int)((first >> 2) & 0x3fff);
    }
    return code;
  }
  if (st) st->code = PBAG_OK;
  return PBAG_OK;
}
