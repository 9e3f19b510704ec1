// pbag_kernels.h - host-callable launchers of the device kernels (internal).
#ifndef PBAG_KERNELS_H
#define PBAG_KERNELS_H

#include <cuda_runtime.h>

#include <vector>

#include "pbag_device.cuh"

namespace pbag {

// Launches of the step loop's kernels (k_evolve, k_rad_ssc and the three SSC
// contractions). While pdl_scope() is set - around each evolve launch of the
// capture of a batch's step loop into a CUDA graph - they carry programmatic
// stream serialization, so that the kernel is resident and has loaded its
// constant tables when the kernels before it end; otherwise they are plain
// launches. Every kernel launched here calls grid_dep_wait() before it
// touches memory that the kernels before it in the stream read or write, and
// the radiation kernels release their dependents (grid_dep_launch) right
// after it. The flag is per host thread, like the capture.
bool& pdl_scope();
template <typename... P, typename... A>
inline cudaError_t launch_step_kernel(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                      A&&... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = pdl_scope() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, static_cast<A&&>(args)...);
}

// once per batch: init steps, e^-p tables, per-record scalars
cudaError_t launch_prepare(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const int64_t* off,
                           const pbag_shock_params* prm, int nbw, int64_t nrec, int64_t* first, StepScal* ss,
                           cudaStream_t st);
// every step: k_evolve(step) first completes step-1 (photon field, totals,
// history rows); after the last step launch_finalize completes it
cudaError_t launch_evolve(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const StepScal* ss,
                          const int64_t* off, const pbag_shock_params* prm, int nbw, int step,
                          const pbag_outputs& out, cudaStream_t st);
cudaError_t launch_rad_ssc(const DevGrid& g, const DevState& S, const pbag_shock_params* prm, int nbw, bool ssc,
                           int step, cudaStream_t st);
cudaError_t launch_finalize(const DevGrid& g, const DevState& S, const int64_t* off, const pbag_shock_params* prm,
                            int nbw, int step, const pbag_outputs& out, cudaStream_t st);
// kernel attributes (dynamic shared memory limits); call once per device
cudaError_t configure_kernels();

// tensor-core synchrotron / SSA sums (pbag_syn_tc.cu): a bank of the
// synchrotron kernel at kSynBankP sub-shifts of the frequency step, covering
// fields B in [kSynBankBmin, kSynBankBmax] G
constexpr int kSynBankP = 8;
constexpr double kSynBankBmin = 1e-12, kSynBankBmax = 1e12;
struct SynBankGeom {
  int P, M, mlo, n_lo, n_hi;
  double h;
};
bool syn_tc_supported(int G, int F);
int syn_tc_tile_bw(int Gp);
void syn_tc_geometry(double dnu, double nu0, double xs_gsl, int F, SynBankGeom* g);
// the bank of one synchrotron method (bins j < jc left out: CSYN's cyclotron bins)
void build_syn_bank(int method, int jc, const double* gam, int G, int Gp, double dnu, const SynBankGeom& sg,
                    std::vector<uint16_t>& out);
// rpb: weight rows per blastwave (2: synchrotron and SSA weights, the step's
// tiles of sb_tbw blastwaves; 1: synchrotron only, tiles of 2 sb_tbw states)
cudaError_t launch_syn_tc(const DevGrid& g, const DevState& S, int nbw, cudaStream_t st, int rpb = 2);

// tensor-core SSC contraction (pbag_ssc_tc.cu), for F = 128 or 256
bool ssc_tc_supported(int F);
void build_ssc_tc_operand(const std::vector<float>& K32, int F, int Gp, std::vector<uint16_t>& Bt);
cudaError_t launch_ssc_tc(const DevGrid& g, const DevState& S, const uint16_t* Bt, int nbw, bool split,
                          cudaStream_t st);
// the same contraction on explicit operands: mode kTcBf16 / kTcSplit (BF16
// tiles) or kTcTf32 (FP32 tiles in the 4-byte layout), Wt the weight tiles,
// Kt the kernel slabs
enum : int { kTcBf16 = 0, kTcSplit = 1, kTcTf32 = 2 };
// nout slabs (grid x), output o of row r at out[r ostride + o] scaled by oscale[o].
// rows.nlive (device): tiles from that row on exit at once; rows.rowmap
// (device): row r writes its output and error to row rowmap[r].
struct TcRows {
  const int* nlive = nullptr;
  const int* rowmap = nullptr;
};
cudaError_t launch_ssc_tc_mode(int mode, int F, int Gp, const void* Wt, const void* Kt, int nrows,
                               const int* flags, const float* U32, const double* scal, const double* oscale, int nout,
                               int ostride, double* out, int* err, cudaStream_t st, TcRows rows = TcRows{});
// the same contraction with blastwaves on the accumulator rows (pbag_ssc_rows.cu;
// F = 128, BF16 or split BF16), chosen by launch_ssc_tc_mode for large batches
// cps: slab chunks per ring stage, ctas: CTAs the output groups aim at (0:
// defaults), lsu: slab stages by 16-byte asynchronous copies of a whole warp
// instead of one bulk copy
struct RowsCfg {
  int cps = 0;
  int ctas = 0;
  int lsu = 0;
};
bool ssc_rows_supported(int F, int Gp, int mode);
cudaError_t launch_ssc_rows(int mode, int Gp, const void* Wt, const void* Kt, int nrows, const int* flags,
                            const float* U32, const double* scal, const double* oscale, int nout, int ostride,
                            double* out, int* err, TcRows rows, RowsCfg cfg, cudaStream_t st);
// The contraction autotuner (pbag_ssc_tc.cu): per (mode, F, Gp, outputs,
// batch-size octave) the kernel and its shape measured fastest on the first
// launch outside a graph capture; on by default (ssc_tune_enable).
void ssc_tune_enable(bool on);
int ssc_tune_report(char* buf, int len);
// K slabs as TF32 operands (FP32 values rounded to TF32, 4-byte layout, lo parts zero)
void build_ssc_tc_operand_tf32(const std::vector<float>& K32, int F, int Gp, std::vector<float>& Bt32);

// SSC kernel tables on the host (kernels.h:49-117): KintT[F][Gs] = Kint[j][k] /
// kscale[k] stored k-major (row k, column j < G, zero beyond) with power-of-two
// column scales, and K32[F][Gp][F] (i, j, k) in FP32, j >= G zero-padded.
void build_ssc_tables(const double* gam, int G, const double* freq, int F, int Gp, int Gs, std::vector<float>& KintT,
                      std::vector<double>& kscale, std::vector<float>& K32);
// the largest dynamic shared memory of k_evolve for any grid
size_t evolve_smem_max_bytes();

// BF16 MLP inference on the tensor cores (pbag_mlp_tc.cu): layer l maps
// dims[l] -> dims[l+1] with weights W[l] in the B-operand layout written by
// mlp_tc_pack and FP32 biases b[l]; SiLU between layers.
constexpr int kMtMaxOut = 256;
constexpr int kMtMaxLayers = 8;
struct MlpTcArgs {
  int L;
  int dims[kMtMaxLayers + 1];
  const uint16_t* W[kMtMaxLayers];
  const float* b[kMtMaxLayers];
};
bool mlp_tc_supported(const int* dims, int L);
cudaError_t mlp_tc_pack(int N, int K, const float* W, uint16_t* out, cudaStream_t st);
cudaError_t launch_mlp_tc(const MlpTcArgs& a, int n, const float* X, float* Y, int* err, cudaStream_t st);

}  // namespace pbag

#endif
