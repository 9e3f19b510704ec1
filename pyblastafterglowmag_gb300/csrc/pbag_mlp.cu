// pbag_mlp.cu - a small multilayer perceptron with its own training and
// inference kernels (FP32 on CUDA cores), for the SSC surrogate.
//
// Layers d_0 -> d_1 -> ... -> d_L; hidden activation SiLU, linear output.
// Parameters are one FP32 array: for each layer l, W_l [d_{l+1}][d_l]
// (row-major) followed by b_l [d_{l+1}]. Training minimises the masked mean
// squared error with Adam.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_kernels.h"

namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16;  // GEMM tile
constexpr int kGemmThreads = 256;            // 16 x 16 threads, 4 x 4 outputs each

enum : int { kEpiStore = 0, kEpiBias = 1, kEpiBiasSilu = 2 };

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + __expf(-z)); }

// C[M][N] = op(A)[M][K] op(B)[K][N]; A is [M][K] (lda) or, transposed, [K][M];
// B is [K][N] (ldb) or, transposed, [N][K]. Epilogues: plain store; + bias[n];
// + bias[n] and SiLU into H (C keeps the pre-activation).
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(kGemmThreads)
k_sgemm(int M, int N, int K, const float* __restrict__ A, int lda, const float* __restrict__ B, int ldb,
        float* __restrict__ C, int ldc, const float* __restrict__ bias, float* __restrict__ H) {
  __shared__ float As[kBK][kBM + 4];
  __shared__ float Bs[kBK][kBN + 4];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kBK) {
    // 64 x 16 elements of each operand, 4 per thread
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + q * kGemmThreads;
      int mm, kk;
      if (TA) {  // consecutive threads along m (contiguous in a transposed A)
        mm = e % kBM;
        kk = e / kBM;
      } else {   // consecutive threads along k
        kk = e % kBK;
        mm = e / kBK;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < K) v = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      As[kk][mm] = v;
      int nn, kb;
      if (TB) {
        kb = e % kBK;
        nn = e / kBK;
      } else {
        nn = e % kBN;
        kb = e / kBN;
      }
      const int gn = n0 + nn, gkb = k0 + kb;
      float w = 0.f;
      if (gn < N && gkb < K) w = TB ? B[(size_t)gn * ldb + gkb] : B[(size_t)gkb * ldb + gn];
      Bs[kb][nn] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (EPI != kEpiStore) v += bias[gn];
      C[(size_t)gm * ldc + gn] = v;
      if (EPI == kEpiBiasSilu) H[(size_t)gm * ldc + gn] = v * sigmoidf_(v);
    }
  }
}

template <bool TA, bool TB, int EPI>
cudaError_t sgemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                  const float* bias, float* H, cudaStream_t st) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM);
  k_sgemm<TA, TB, EPI><<<grid, kGemmThreads, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, H);
  return cudaGetLastError();
}

// masked squared error: dY = 2 m (Y - T) / count, loss partial sums per block
__global__ void k_mse(int n, int d, const float* __restrict__ Y, const float* __restrict__ T,
                      const float* __restrict__ mask, float inv_count, float* __restrict__ dY,
                      float* __restrict__ loss) {
  __shared__ float red[256];
  float s = 0.f;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (int64_t)n * d;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const float m = mask ? mask[idx] : 1.f;
    const float e = (Y[idx] - T[idx]) * m;
    dY[idx] = 2.f * e * inv_count;
    s += e * e;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] * inv_count);
}

// dZ = dH * silu'(Z)
__global__ void k_silu_back(int64_t count, const float* __restrict__ Z, float* __restrict__ dZ) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= count) return;
  const float z = Z[idx];
  const float s = sigmoidf_(z);
  dZ[idx] *= s * (1.f + z * (1.f - s));
}

// db[j] = sum over rows of dZ[:, j]
__global__ void k_colsum(int n, int d, const float* __restrict__ dZ, float* __restrict__ db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  float s = 0.f;
  for (int r = 0; r < n; ++r) s += dZ[(size_t)r * d + j];
  db[j] = s;
}

__global__ void k_adam(int64_t count, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= count) return;
  const float gi = g[idx];
  const float mi = b1 * m[idx] + (1.f - b1) * gi;
  const float vi = b2 * v[idx] + (1.f - b2) * gi * gi;
  m[idx] = mi;
  v[idx] = vi;
  p[idx] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

}  // namespace

struct pbag_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<int> dims;
  std::vector<size_t> woff, boff;  // offsets of W_l and b_l in the parameter array
  size_t nparams = 0;
  float* p = nullptr;  // parameters
  float* g = nullptr;  // gradients
  float* m = nullptr;  // Adam moments
  float* v = nullptr;
  int64_t t = 0;       // Adam step
  int64_t pgen = 0;    // bumped whenever the parameters change
  // BF16 copy of the weights in the tensor-core operand layout (inference)
  uint16_t* wtc = nullptr;
  int64_t tcgen = -1;  // pgen the copy was made from
  int* tcerr = nullptr;
  // activations of the last forward pass: Z_l (pre-activation) and H_l per layer
  int cap = 0;
  std::vector<float*> Z, Hs, dH;
  float* loss = nullptr;
  ~pbag_mlp() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    cudaFree(p);
    cudaFree(g);
    cudaFree(m);
    cudaFree(v);
    cudaFree(loss);
    cudaFree(wtc);
    cudaFree(tcerr);
    for (float* x : Z) cudaFree(x);
    for (float* x : Hs) cudaFree(x);
    for (float* x : dH) cudaFree(x);
    if (stream) cudaStreamDestroy(stream);
  }
  int L() const { return (int)dims.size() - 1; }
  cudaError_t reserve(int n) {
    if (n <= cap) return cudaSuccess;
    for (float* x : Z) cudaFree(x);
    for (float* x : Hs) cudaFree(x);
    for (float* x : dH) cudaFree(x);
    Z.assign(L() + 1, nullptr);
    Hs.assign(L() + 1, nullptr);
    dH.assign(L() + 1, nullptr);
    cap = 0;
    for (int l = 1; l <= L(); ++l) {
      const size_t bytes = (size_t)n * dims[l] * sizeof(float);
      cudaError_t e;
      if ((e = cudaMalloc(&Z[l], bytes)) != cudaSuccess) return e;
      if ((e = cudaMalloc(&Hs[l], bytes)) != cudaSuccess) return e;
      if ((e = cudaMalloc(&dH[l], bytes)) != cudaSuccess) return e;
    }
    cap = n;
    return cudaSuccess;
  }
  // forward pass of n rows of X [n][d_0] into Y [n][d_L] (Y may be the
  // internal output buffer); keeps Z and H for a backward pass
  cudaError_t forward(int n, const float* X, float* Y) {
    cudaError_t e = cudaSuccess;
    const float* Hin = X;
    for (int l = 0; l < L(); ++l) {
      const int din = dims[l], dout = dims[l + 1];
      const float* W = p + woff[l];
      const float* b = p + boff[l];
      const bool last = l == L() - 1;
      float* out = last && Y ? Y : Z[l + 1];
      if (last)
        e = sgemm<false, true, kEpiBias>(n, dout, din, Hin, din, W, din, out, dout, b, nullptr, stream);
      else
        e = sgemm<false, true, kEpiBiasSilu>(n, dout, din, Hin, din, W, din, Z[l + 1], dout, b, Hs[l + 1], stream);
      if (e != cudaSuccess) return e;
      Hin = Hs[l + 1];
    }
    return e;
  }
  // gradients of the masked MSE of the last forward pass (output in Yout)
  cudaError_t backward(int n, const float* X, const float* Yout, const float* T, const float* mask, float count) {
    cudaError_t e;
    const int dL = dims[L()];
    if ((e = cudaMemsetAsync(loss, 0, sizeof(float), stream)) != cudaSuccess) return e;
    const int64_t tot = (int64_t)n * dL;
    const int blocks = (int)std::min<int64_t>((tot + 255) / 256, 1024);
    k_mse<<<blocks, 256, 0, stream>>>(n, dL, Yout, T, mask, 1.f / count, dH[L()], loss);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int l = L() - 1; l >= 0; --l) {
      const int din = dims[l], dout = dims[l + 1];
      float* dZ = dH[l + 1];  // holds dL/dH_{l+1}; becomes dL/dZ_{l+1} in place
      if (l < L() - 1) {
        const int64_t c = (int64_t)n * dout;
        k_silu_back<<<(unsigned)((c + 255) / 256), 256, 0, stream>>>(c, Z[l + 1], dZ);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
      }
      const float* Hin = l == 0 ? X : Hs[l];
      // dW_l [dout][din] = dZ^T [dout][n] . H_l [n][din]
      if ((e = sgemm<true, false, kEpiStore>(dout, din, n, dZ, dout, Hin, din, g + woff[l], din, nullptr, nullptr,
                                             stream)) != cudaSuccess)
        return e;
      k_colsum<<<(dout + 127) / 128, 128, 0, stream>>>(n, dout, dZ, g + boff[l]);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      if (l > 0) {
        // dH_l [n][din] = dZ [n][dout] . W_l [dout][din]
        if ((e = sgemm<false, false, kEpiStore>(n, din, dout, dZ, dout, p + woff[l], din, dH[l], din, nullptr,
                                                nullptr, stream)) != cudaSuccess)
          return e;
      }
    }
    return cudaSuccess;
  }
};

namespace pbag {
// BF16 tensor-core inference: lays the weights out again when they changed
cudaError_t mlp_infer(pbag_mlp* net, int n, const float* X, float* Y, cudaStream_t st) {
  const int L = net->L();
  if (!mlp_tc_supported(net->dims.data(), L)) return cudaErrorNotSupported;
  cudaError_t e = cudaSuccess;
  size_t tot = 0;
  for (int l = 0; l < L; ++l) tot += (size_t)net->dims[l + 1] * net->dims[l];
  if (!net->wtc) {
    if ((e = cudaMalloc(&net->wtc, tot * sizeof(uint16_t))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&net->tcerr, sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMemset(net->tcerr, 0, sizeof(int))) != cudaSuccess) return e;
  }
  MlpTcArgs a{};
  a.L = L;
  size_t off = 0;
  for (int l = 0; l <= L; ++l) a.dims[l] = net->dims[l];
  for (int l = 0; l < L; ++l) {
    if (net->tcgen != net->pgen)
      if ((e = mlp_tc_pack(net->dims[l + 1], net->dims[l], net->p + net->woff[l], net->wtc + off, st)) != cudaSuccess)
        return e;
    a.W[l] = net->wtc + off;
    a.b[l] = net->p + net->boff[l];
    off += (size_t)net->dims[l + 1] * net->dims[l];
  }
  net->tcgen = net->pgen;
  return launch_mlp_tc(a, n, X, Y, net->tcerr, st);
}
int* mlp_infer_error(pbag_mlp* net) { return net->tcerr; }
// used by the surrogate step path (pbag_surrogate.cu)
cudaError_t mlp_forward(pbag_mlp* net, int n, const float* X, float* Y, cudaStream_t st) {
  cudaStream_t keep = net->stream;
  net->stream = st;
  cudaError_t e = net->reserve(n);
  if (e == cudaSuccess) e = net->forward(n, X, Y);
  net->stream = keep;
  return e;
}
int mlp_in_dim(const pbag_mlp* net) { return net->dims.front(); }
int mlp_out_dim(const pbag_mlp* net) { return net->dims.back(); }
int mlp_layers(const pbag_mlp* net) { return net->L(); }
cudaError_t mlp_reserve(pbag_mlp* net, int n) { return net->reserve(n); }
}  // namespace pbag

namespace {
int status_of(cudaError_t e) { return e == cudaErrorMemoryAllocation ? PBAG_ERR_NOMEM : PBAG_ERR_CUDA; }
}  // namespace

extern "C" {

int pbag_mlp_create(int device, const int* dims, int nlayers, pbag_mlp** out) {
  if (!out || !dims || nlayers < 1 || nlayers > 16) return PBAG_ERR_ARG;
  *out = nullptr;
  for (int l = 0; l <= nlayers; ++l)
    if (dims[l] < 1 || dims[l] > 4096) return PBAG_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PBAG_ERR_CUDA;
  auto* net = new pbag_mlp();
  net->device = device;
  net->dims.assign(dims, dims + nlayers + 1);
  for (int l = 0; l < nlayers; ++l) {
    net->woff.push_back(net->nparams);
    net->nparams += (size_t)dims[l + 1] * dims[l];
    net->boff.push_back(net->nparams);
    net->nparams += (size_t)dims[l + 1];
  }
  cudaError_t e = cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking);
  const size_t bytes = net->nparams * sizeof(float);
  for (float** q : {&net->p, &net->g, &net->m, &net->v})
    if (e == cudaSuccess) e = cudaMalloc(q, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&net->loss, sizeof(float));
  for (float* q : {net->p, net->g, net->m, net->v})
    if (e == cudaSuccess) e = cudaMemset(q, 0, bytes);
  if (e != cudaSuccess) {
    delete net;
    return status_of(e);
  }
  *out = net;
  return PBAG_OK;
}

void pbag_mlp_destroy(pbag_mlp* net) { delete net; }

int64_t pbag_mlp_param_count(const pbag_mlp* net) { return net ? (int64_t)net->nparams : -1; }

int pbag_mlp_set_params(pbag_mlp* net, const float* host) {
  if (!net || !host) return PBAG_ERR_ARG;
  if (cudaSetDevice(net->device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (cudaMemcpy(net->p, host, net->nparams * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return PBAG_ERR_CUDA;
  cudaMemset(net->m, 0, net->nparams * sizeof(float));
  cudaMemset(net->v, 0, net->nparams * sizeof(float));
  net->t = 0;
  net->pgen += 1;
  return PBAG_OK;
}

int pbag_mlp_get_params(const pbag_mlp* net, float* host, float* host_grad) {
  if (!net) return PBAG_ERR_ARG;
  if (cudaSetDevice(net->device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (cudaStreamSynchronize(net->stream) != cudaSuccess) return PBAG_ERR_CUDA;
  if (host && cudaMemcpy(host, net->p, net->nparams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PBAG_ERR_CUDA;
  if (host_grad &&
      cudaMemcpy(host_grad, net->g, net->nparams * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return PBAG_ERR_CUDA;
  return PBAG_OK;
}

int pbag_mlp_forward(pbag_mlp* net, int n, const float* d_x, float* d_y) {
  if (!net || n < 0 || (n > 0 && (!d_x || !d_y))) return PBAG_ERR_ARG;
  if (n == 0) return PBAG_OK;
  if (cudaSetDevice(net->device) != cudaSuccess) return PBAG_ERR_CUDA;
  cudaError_t e = net->reserve(n);
  if (e == cudaSuccess) e = net->forward(n, d_x, d_y);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
  return e == cudaSuccess ? PBAG_OK : status_of(e);
}

int pbag_mlp_infer(pbag_mlp* net, int n, const float* d_x, float* d_y) {
  if (!net || n < 0 || (n > 0 && (!d_x || !d_y))) return PBAG_ERR_ARG;
  if (!pbag::mlp_tc_supported(net->dims.data(), net->L())) return PBAG_ERR_UNSUPPORTED;
  if (n == 0) return PBAG_OK;
  if (cudaSetDevice(net->device) != cudaSuccess) return PBAG_ERR_CUDA;
  cudaError_t e = pbag::mlp_infer(net, n, d_x, d_y, net->stream);
  int code = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&code, net->tcerr, sizeof(int), cudaMemcpyDeviceToHost, net->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
  if (e != cudaSuccess) return status_of(e);
  if (code != 0) {
    cudaMemset(net->tcerr, 0, sizeof(int));
    return code;
  }
  return PBAG_OK;
}

int pbag_mlp_train_step(pbag_mlp* net, int n, const float* d_x, const float* d_t, const float* d_mask, float lr,
                        int update, float* loss) {
  if (!net || n <= 0 || !d_x || !d_t) return PBAG_ERR_ARG;
  if (cudaSetDevice(net->device) != cudaSuccess) return PBAG_ERR_CUDA;
  cudaError_t e = net->reserve(n);
  float* Y = net->Z[net->L()];
  if (e == cudaSuccess) e = net->forward(n, d_x, Y);
  if (e == cudaSuccess) e = net->backward(n, d_x, Y, d_t, d_mask, (float)n * net->dims.back());
  if (e == cudaSuccess && update) {
    net->t += 1;
    net->pgen += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f / (1.f - std::pow(b1, (float)net->t));
    const float c2 = 1.f / (1.f - std::pow(b2, (float)net->t));
    const int64_t c = (int64_t)net->nparams;
    k_adam<<<(unsigned)((c + 255) / 256), 256, 0, net->stream>>>(c, net->p, net->g, net->m, net->v, lr, b1, b2,
                                                                  1e-8f, c1, c2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, net->loss, sizeof(float), cudaMemcpyDeviceToHost, net->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(net->stream);
  return e == cudaSuccess ? PBAG_OK : status_of(e);
}

}  // extern "C"
