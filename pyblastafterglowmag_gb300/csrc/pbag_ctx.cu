// pbag_ctx.cu - the C ABI entry points that own device memory and run a batch.
//
// A pbag_ctx is the device-side counterpart of one CommonTables entry of the
// reference (microphysics/common.h:93-117): one electron grid, one photon grid
// and the SSC kernel tables, shared read-only by every blastwave of a batch.
// pbag_run_batch evolves the whole history of every blastwave of the batch:
// one preparation pass over all records, then, step index by step index,
//   k_evolve -> k_rad_ssc -> k_finalize
// over all blastwaves on one stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "pbag.h"
#include "pbag_ctx_view.h"
#include "pbag_internal.h"
#include "pbag_kernels.h"

using namespace pbag;

namespace {

__global__ void k_fill_flags(int* __restrict__ flags, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = v;
}

template <typename T>
cudaError_t dev_alloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) return cudaSuccess;
  return cudaMalloc((void**)p, n * sizeof(T));
}

template <typename T>
cudaError_t upload(T** p, const T* h, size_t n, cudaStream_t st) {
  cudaError_t e = dev_alloc(p, n);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, st);
}

int cuda_code(cudaError_t e) { return e == cudaErrorMemoryAllocation ? PBAG_ERR_NOMEM : PBAG_ERR_CUDA; }

constexpr int kOutputs = 13;  // pointers in pbag_outputs
inline bool output_on_gamma(int fi) { return fi >= 4 && fi < 8; }

// Everything a captured step loop depends on: replaying the graph is only
// valid while all of it is unchanged.
struct GraphKey {
  int nbw;
  int64_t max_len;
  size_t nrec;
  const void* recs;
  const void* prm;
  const void* state;
  const void* ss;
  bool ssc;
  int ssc_path;
  int64_t sur_gen;
  const void* synbank;
  const void* out[kOutputs];
  std::vector<int64_t> lens;  // history length of every blastwave (the step launches' extents)
  bool operator==(const GraphKey& o) const {
    if (lens != o.lens) return false;
    if (nbw != o.nbw || max_len != o.max_len || nrec != o.nrec || recs != o.recs || prm != o.prm ||
        state != o.state || ss != o.ss || ssc != o.ssc || ssc_path != o.ssc_path || sur_gen != o.sur_gen ||
        synbank != o.synbank)
      return false;
    for (int k = 0; k < kOutputs; ++k)
      if (out[k] != o.out[k]) return false;
    return true;
  }
};

}  // namespace

struct pbag_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  pbag_grid_desc desc{};
  int G = 0, F = 0, Gp = 0;
  bool ssc = false;
  int ssc_path = PBAG_SSC_AUTO;
  std::vector<double> gam, freq;
  DevGrid dg{};
  std::vector<void*> grid_mem;

  // which SSC contraction runs: tensor cores when the grid allows it, unless
  // the caller pinned a path
  bool ssc_on_tensor_cores() const {
    return ssc && dg.Bt && (ssc_path == PBAG_SSC_AUTO || ssc_path == PBAG_SSC_TC_SPLIT_BF16 ||
                            ssc_path == PBAG_SSC_TC_BF16 || ssc_path == PBAG_SSC_SURROGATE);
  }
  // kernels of one step's SSC contraction on the side stream
  int ssc_side_launches() const { return ssc_path == PBAG_SSC_SURROGATE ? surrogate_launches(this) : 1; }

  // radiation sums + SSC contraction of one step; the tensor-core contraction
  // runs on a second stream next to the synchrotron sums (both read only what
  // k_evolve wrote) and joins the main stream before the next step
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaError_t launch_radiation(const DevGrid& gg, const DevState& SS, const pbag_shock_params* d_prm, int nbw, int s) {
    if (nbw <= 0) return cudaSuccess;
    const bool syn_tc = SS.Dsyn != nullptr;  // synchrotron / SSA sums on the tensor cores
    if (!ssc_on_tensor_cores())
      return syn_tc ? launch_syn_tc(gg, SS, nbw, stream) : launch_rad_ssc(gg, SS, d_prm, nbw, ssc, s, stream);
    cudaError_t e;
    if ((e = cudaEventRecord(ev_fork, stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(side, ev_fork, 0)) != cudaSuccess) return e;
    if (ssc_path == PBAG_SSC_SURROGATE) {
      CtxView v;
      ctx_view(this, &v);
      if ((e = surrogate_run(this, v, nbw, S.Abf, S.flags, S.U32, S.scal, S.f, G, S.n, F, S.scal + kScalB, kScal,
                             S.jssc, S.err, side)) != cudaSuccess)
        return e;
    } else if ((e = launch_ssc_tc(dg, S, dg.Bt, nbw, ssc_path != PBAG_SSC_TC_BF16, side)) != cudaSuccess) {
      return e;
    }
    if ((e = cudaEventRecord(ev_join, side)) != cudaSuccess) return e;
    if ((e = syn_tc ? launch_syn_tc(gg, SS, nbw, stream) : launch_rad_ssc(gg, SS, d_prm, nbw, false, s, stream)) !=
        cudaSuccess)
      return e;
    return cudaStreamWaitEvent(stream, ev_join, 0);
  }
  // the tensor-core synchrotron sums: bank geometry (set at creation when the
  // grid allows them), the banks of the four method classes (built on first
  // use), the switch PBAG_SYN_TC=0 (CUDA-core sums)
  bool sb_ok = false;
  SynBankGeom sb{};
  double sb_lnnu0 = 0., sb_lnxs = 0., sb_dnu = 0.;
  const uint16_t* sb_bank[4] = {};
  // PBAG_SYN_TC=0: always the CUDA-core sums; =1: the tensor-core sums
  // whenever the grid allows; unset: the tensor-core sums for batches of at
  // least kSynTcMinBw blastwaves. A small batch's CUDA-core sums run next to
  // the SSC contraction and cost the step nothing, while the bank's
  // interpolation lengthens the step completion on the critical path; a large
  // batch's CUDA-core sums are issue-bound and the GEMM wins (measured: 42
  // blastwaves 1.25 M -> 1.10 M blastwave-steps/s, 2 370 blastwaves 3.43 M ->
  // 3.98 M).
  static constexpr int kSynTcMinBw = 128;
  bool syn_tc_enabled(int nbw = 1 << 30) const {
    const char* v = std::getenv("PBAG_SYN_TC");
    if (!sb_ok || (v && v[0] == '0')) return false;
    return (v && v[0] == '1') || nbw >= kSynTcMinBw;
  }
  // bank of the method class of syn_method: CSYN (cyclotron bins apart), Dermer09, GSL, Bessel
  static int syn_class(int syn_method) {
    return syn_method == PBAG_SYN_CSYN ? 0 : syn_method == PBAG_SYN_DER09 ? 1 : syn_method == PBAG_SYN_GSL ? 2 : 3;
  }
  cudaError_t syn_bank(int cls, const uint16_t** out) {
    if (!sb_bank[cls]) {
      std::vector<uint16_t> bank;
      const int method = cls == 0 ? PBAG_SYN_CSYN : cls == 1 ? PBAG_SYN_DER09 : cls == 2 ? PBAG_SYN_GSL : PBAG_SYN_BESSEL;
      build_syn_bank(method, cls == 0 ? dg.n_cyc : 0, gam.data(), G, Gp, sb_dnu, sb, bank);
      const uint16_t* p = nullptr;
      cudaError_t e = grid_upload(&p, bank);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // the host vector goes out of scope
      if (e != cudaSuccess) return e;
      sb_bank[cls] = p;
    }
    *out = sb_bank[cls];
    return cudaSuccess;
  }
  // batch buffers, grown on demand
  int cap_bw = 0;
  size_t cap_rec = 0;
  pbag_step_rec* d_recs = nullptr;  // records (host-buffer entry point)
  StepScal* d_ss = nullptr;         // per-record scalars
  int64_t* d_off = nullptr;
  int64_t* d_first = nullptr;
  int* d_slot = nullptr;  // slot -> blastwave of the running batch (uneven histories)
  std::vector<int> slot_of;  // blastwave -> slot of the last batch (empty: the same index)
  pbag_shock_params* d_prm = nullptr;
  DevState S{};
  std::vector<void*> state_mem;
  double* d_out = nullptr;  // output histories (host-buffer entry point)
  size_t cap_out = 0;
  int64_t launches = 0;
  int n_sm = 0;  // SMs of the device
  // optional per-kernel-class timing with CUDA events on the launch stream
  bool timing = false;
  std::vector<cudaEvent_t> ev;  // 2 events per timed launch
  std::vector<int> ev_class;    // kernel class of each event pair
  double class_ms[kKernelClasses] = {0, 0, 0};
  int64_t class_launches[kKernelClasses] = {0, 0, 0};
  // captured step loop of the last batch shape
  cudaGraphExec_t graph_exec = nullptr;
  GraphKey graph_key{};
  // workspaces of other entry points (pbag_contract)
  CtxExtension* ext[kExtSlots] = {};

  ~pbag_ctx() {
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (CtxExtension*& x : ext) {
      delete x;
      x = nullptr;
    }
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (side) cudaStreamSynchronize(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    for (void* p : grid_mem) cudaFree(p);
    free_state();
    cudaFree(d_recs);
    cudaFree(d_ss);
    cudaFree(d_out);
    if (stream) cudaStreamDestroy(stream);
  }

  void free_state() {
    for (void* p : state_mem) cudaFree(p);
    state_mem.clear();
    S.Abf = nullptr;
    S.Sbf = nullptr;
    S.Dsyn = nullptr;
    cap_bw = 0;
    d_off = nullptr;
    d_first = nullptr;
    d_slot = nullptr;
    d_prm = nullptr;
  }

  template <typename T>
  cudaError_t grid_upload(const T** dst, const std::vector<T>& h) {
    T* p = nullptr;
    cudaError_t e = upload(&p, h.data(), h.size(), stream);
    if (e == cudaSuccess) grid_mem.push_back(p);
    *dst = p;
    return e;
  }

  template <typename T>
  cudaError_t state_alloc(T** dst, size_t n) {
    cudaError_t e = dev_alloc(dst, n);
    if (e == cudaSuccess) state_mem.push_back(*dst);
    return e;
  }

  cudaError_t reserve_bw(int nbw) {
    if (nbw <= cap_bw && cap_bw > 0) return cudaSuccess;
    free_state();
    const size_t cap = (size_t)std::max(nbw, 64);
    cudaError_t e;
    if ((e = state_alloc(&d_off, cap + 1)) != cudaSuccess) return e;
    if ((e = state_alloc(&d_first, cap)) != cudaSuccess) return e;
    if ((e = state_alloc(&d_slot, cap)) != cudaSuccess) return e;
    if ((e = state_alloc(&d_prm, cap)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.f, cap * G)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.dfde, cap * G)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.powp, cap * G)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.gdot, cap * 3 * G)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.n, cap * F)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.syn32, cap * F)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.ssa32, cap * F)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.rad32, cap * 4)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.jssc, cap * F)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.W32, cap * Gp)) != cudaSuccess) return e;
    if (dg.Bt && (e = state_alloc(&S.Abf, (cap + kTcCols - 1) / kTcCols * tc_tile_elems(kTcCols, Gp))) != cudaSuccess)
      return e;
    // whole tensor-core tiles of rows: the SSC kernel copies U a tile at a time
    const size_t urows = dg.Bt ? (cap + kTcCols - 1) / kTcCols * kTcCols : cap;
    if ((e = state_alloc(&S.U32, urows * F)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(S.U32, 0, urows * F * sizeof(float), stream)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.w32, cap * G)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.v32, cap * G)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.scal, cap * kScal)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.flags, cap)) != cudaSuccess) return e;
    if ((e = state_alloc(&S.err, cap * 4)) != cudaSuccess) return e;
    if (sb_ok) {
      const size_t tiles = (cap + dg.sb_tbw - 1) / dg.sb_tbw;
      if ((e = state_alloc(&S.Sbf, tiles * tc_tile_elems(2 * dg.sb_tbw, Gp))) != cudaSuccess) return e;
      if ((e = state_alloc(&S.Dsyn, tiles * (size_t)sb.P * 2 * dg.sb_tbw * sb.M)) != cudaSuccess) return e;
    }
    cap_bw = (int)cap;
    return cudaSuccess;
  }

  cudaError_t reserve_rec(size_t nrec, bool host_records) {
    if (nrec > cap_rec) {
      cudaFree(d_recs);
      cudaFree(d_ss);
      d_recs = nullptr;
      d_ss = nullptr;
      cap_rec = 0;
      cudaError_t e;
      if ((e = dev_alloc(&d_ss, nrec)) != cudaSuccess) return e;
      if ((e = dev_alloc(&d_recs, nrec)) != cudaSuccess) return e;
      cap_rec = nrec;
    }
    (void)host_records;
    return cudaSuccess;
  }

  cudaError_t reset_state(int nbw) {
    cudaError_t e;
    const size_t n = (size_t)nbw;
    auto z = [&](void* p, size_t bytes) {
      return bytes ? cudaMemsetAsync(p, 0, bytes, stream) : cudaSuccess;
    };
    if ((e = z(S.f, n * G * sizeof(double))) != cudaSuccess) return e;
    if ((e = z(S.dfde, n * G * sizeof(double))) != cudaSuccess) return e;
    if ((e = z(S.gdot, n * 3 * G * sizeof(double))) != cudaSuccess) return e;
    if ((e = z(S.n, n * F * sizeof(double))) != cudaSuccess) return e;
    if ((e = z(S.jssc, n * F * sizeof(double))) != cudaSuccess) return e;
    if ((e = z(S.U32, n * F * sizeof(float))) != cudaSuccess) return e;
    if ((e = z(S.W32, n * Gp * sizeof(float))) != cudaSuccess) return e;
    if (S.Abf && (e = z(S.Abf, (n + kTcCols - 1) / kTcCols * tc_tile_elems(kTcCols, Gp) * sizeof(uint16_t))) !=
                     cudaSuccess)
      return e;
    if ((e = z(S.scal, n * kScal * sizeof(double))) != cudaSuccess) return e;
    if ((e = z(S.flags, n * sizeof(int))) != cudaSuccess) return e;
    if (S.Sbf && (e = z(S.Sbf, (n + dg.sb_tbw - 1) / dg.sb_tbw * tc_tile_elems(2 * dg.sb_tbw, Gp) *
                                   sizeof(uint16_t))) != cudaSuccess)
      return e;
    return z(S.err, n * 4 * sizeof(int));
  }
};

namespace {

// programmatic dependent launch of the captured step loop (PBAG_PDL=0: off)
bool pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("PBAG_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

int check_batch(const pbag_ctx* c, const pbag_shock_params* prm_host, int nbw, const int64_t* off) {
  if (nbw < 0 || !off) return PBAG_ERR_ARG;
  if (off[0] != 0) return PBAG_ERR_ARG;
  for (int b = 0; b < nbw; ++b)
    if (off[b + 1] < off[b]) return PBAG_ERR_ARG;
  if (nbw > 0 && off[nbw] > (int64_t)1 << 40) return PBAG_ERR_ARG;
  for (int b = 0; b < nbw; ++b)
    if (off[b + 1] - off[b] > (int64_t)1 << 30) return PBAG_ERR_ARG;
  if (prm_host) {
    for (int b = 0; b < nbw; ++b) {
      const pbag_shock_params& p = prm_host[b];
      if (p.pp_on && !p.ssc_on) return PBAG_ERR_PARAM;  // "PP requires SSC" (microphysics_base.h:394-397)
      if (p.syn_method < PBAG_SYN_CSYN || p.syn_method > PBAG_SYN_BESSEL) return PBAG_ERR_ARG;
      if (p.ele_method != PBAG_ELE_NUMERIC && p.ele_method != PBAG_ELE_MIX) return PBAG_ERR_ARG;
      if (p.max_substeps < 1 || !(p.p > 0.) || !std::isfinite(p.p)) return PBAG_ERR_ARG;
      if (p.ssc_on && !c->ssc) return PBAG_ERR_ARG;
    }
  }
  return PBAG_OK;
}

// Runs every step of the batch; all pointers are device pointers except off_h.
// syn_cls >= 0: the synchrotron / SSA sums on the tensor cores with the bank of
// that method class.
int run_device_once(pbag_ctx* c, const pbag_shock_params* d_prm, int nbw, const int64_t* off_h,
                    const pbag_step_rec* d_recs, const pbag_outputs& d_out, pbag_status* st, int syn_cls) {
  cudaError_t e = c->reserve_bw(nbw);
  if (e != cudaSuccess) return cuda_code(e);
  // this run's grid tables and state: the bank and its buffers only on the tensor-core path
  DevGrid gg = c->dg;
  DevState SS = c->S;
  if (syn_cls >= 0) {
    if ((e = c->syn_bank(syn_cls, &gg.synbank)) != cudaSuccess) return cuda_code(e);
  } else {
    SS.Sbf = nullptr;
    SS.Dsyn = nullptr;
  }
  const size_t nrec = (size_t)off_h[nbw];
  if ((e = c->reserve_rec(nrec, false)) != cudaSuccess) return cuda_code(e);
  if ((e = cudaMemcpyAsync(c->d_off, off_h, sizeof(int64_t) * (nbw + 1), cudaMemcpyHostToDevice, c->stream)) !=
      cudaSuccess)
    return PBAG_ERR_CUDA;
  if ((e = c->reset_state(nbw)) != cudaSuccess) return PBAG_ERR_CUDA;
  // zero rows: skipped steps keep zero output rows
  const double* const* outp = reinterpret_cast<const double* const*>(&d_out);
  for (int fi = 0; fi < kOutputs; ++fi) {
    if (!outp[fi] || !nrec) continue;
    const size_t n = output_on_gamma(fi) ? (size_t)c->G : (size_t)c->F;
    if (cudaMemsetAsync((void*)outp[fi], 0, nrec * n * sizeof(double), c->stream) != cudaSuccess)
      return PBAG_ERR_CUDA;
  }
  int64_t max_len = 0;
  for (int b = 0; b < nbw; ++b) max_len = std::max<int64_t>(max_len, off_h[b + 1] - off_h[b]);
  // Slots: the blastwaves of a batch of uneven histories run in slots ordered
  // by decreasing length, so that those still running at step s are the
  // first n(s) slots and each step launches over them only (finished
  // blastwaves get no CTA and no contraction row). A batch of equal lengths
  // keeps slot = blastwave.
  std::vector<int64_t> lens((size_t)nbw);
  for (int b = 0; b < nbw; ++b) lens[b] = off_h[b + 1] - off_h[b];
  bool uneven = false;
  for (int b = 1; b < nbw && !uneven; ++b) uneven = lens[b] != lens[0];
  std::vector<int64_t> slot_len = lens;  // history length by slot, decreasing when uneven
  if (uneven) {
    std::vector<int> slot((size_t)nbw);
    for (int b = 0; b < nbw; ++b) slot[b] = b;
    std::stable_sort(slot.begin(), slot.end(), [&](int a, int b) { return lens[a] > lens[b]; });
    for (int k = 0; k < nbw; ++k) slot_len[k] = lens[slot[k]];
    if (cudaMemcpyAsync(c->d_slot, slot.data(), sizeof(int) * nbw, cudaMemcpyHostToDevice, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)  // the host vector goes out of scope
      return PBAG_ERR_CUDA;
    SS.slot_bw = c->d_slot;
    c->slot_of.assign((size_t)nbw, 0);
    for (int k = 0; k < nbw; ++k) c->slot_of[slot[k]] = k;
  } else {
    c->slot_of.clear();
  }
  // slots whose history is longer than x steps
  auto longer = [&](int64_t x) -> int {
    if (!uneven) return nbw > 0 && slot_len[0] > x ? nbw : 0;
    return (int)(std::partition_point(slot_len.begin(), slot_len.end(), [&](int64_t v) { return v > x; }) -
                 slot_len.begin());
  };
  // step s: evolve completes step s-1 of every slot that ran it and runs step
  // s; the radiation covers the slots that run step s
  auto n_evolve = [&](int64_t s) { return longer(s > 0 ? s - 1 : 0); };
  auto n_radiate = [&](int64_t s) { return longer(s); };
  c->launches = 0;
  if (c->ssc_path == PBAG_SSC_SURROGATE && nbw > 0 && (e = surrogate_reserve(c, nbw)) != cudaSuccess)
    return cuda_code(e);
  if (nbw > 0) {
    if ((e = launch_prepare(gg, SS, d_recs, c->d_off, d_prm, nbw, (int64_t)nrec, c->d_first, c->d_ss,
                            c->stream)) != cudaSuccess)
      return PBAG_ERR_CUDA;
    c->launches += nrec > 0 ? 3 : 2;
  }
  size_t nev = 0;
  auto mark = [&](int cls, bool start) -> bool {
    if (!c->timing) return true;
    if (nev >= c->ev.size()) {
      cudaEvent_t x;
      if (cudaEventCreate(&x) != cudaSuccess) return false;
      c->ev.push_back(x);
      c->ev_class.push_back(0);
    }
    if (start) c->ev_class[nev / 2] = cls;
    return cudaEventRecord(c->ev[nev++], c->stream) == cudaSuccess;
  };
  // Without timing, the step loop (3 launches per step index) is captured once
  // into a CUDA graph per batch shape and buffer set, and replayed.
  if (!c->timing && max_len > 0) {
    GraphKey key{nbw, max_len, nrec, d_recs, d_prm, c->S.f, c->d_ss, c->ssc, c->ssc_path, surrogate_generation(c),
                 gg.synbank, {}};
    std::memcpy(key.out, &d_out, sizeof(d_out));
    key.lens = lens;
    if (!c->graph_exec || !(key == c->graph_key)) {
      if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
      c->graph_exec = nullptr;
      cudaGraph_t graph = nullptr;
      // the contraction autotuner measures outside the capture: SSC launches
      // on this batch's buffers with every row active, one per size class of
      // the steps' row counts (the flags are saved and restored; the step
      // writes the contraction's outputs before it reads them)
      if (nbw > 0 && c->ssc_on_tensor_cores() && c->ssc_path != PBAG_SSC_SURROGATE) {
        int* saved = nullptr;
        if (cudaMalloc(&saved, (size_t)nbw * sizeof(int)) == cudaSuccess) {
          cudaError_t te = cudaMemcpyAsync(saved, c->S.flags, (size_t)nbw * sizeof(int), cudaMemcpyDeviceToDevice,
                                           c->stream);
          if (te == cudaSuccess) {
            k_fill_flags<<<(nbw + 255) / 256, 256, 0, c->stream>>>(c->S.flags, nbw, kFlagActive);
            te = cudaGetLastError();
          }
          int last_octave = -1;
          for (int64_t s = 0; s < max_len && te == cudaSuccess; ++s) {
            const int n = n_radiate(s);  // decreasing in s
            int o = 0;
            while ((2 << o) <= n) ++o;
            if (n <= 0 || o == last_octave) continue;
            last_octave = o;
            te = launch_ssc_tc(c->dg, c->S, c->dg.Bt, n, c->ssc_path != PBAG_SSC_TC_BF16, c->stream);
          }
          cudaMemcpyAsync(c->S.flags, saved, (size_t)nbw * sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
          const cudaError_t se = cudaStreamSynchronize(c->stream);
          cudaFree(saved);
          if (te != cudaSuccess || se != cudaSuccess) return PBAG_ERR_CUDA;
        }
      }
      if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return PBAG_ERR_CUDA;
      cudaError_t ce = cudaSuccess;
      // each evolve launch of at most one CTA per SM a programmatic dependent
      // of the previous step's radiation kernels, which let it be scheduled
      // as soon as they start: its CTAs are resident, with the grid and
      // kernel-integral tables loaded, when the radiation ends (20.7 against
      // 21.7 ms for the 1 000 steps of the 21-layer jet). Larger launches
      // would hold the SMs' room that the radiation CTAs still need. The
      // radiation kernels keep plain edges: made programmatic dependents of
      // evolve too, the jet's pass took 25-27 ms, wherever evolve released
      // them. PBAG_PDL=0: plain edges throughout.
      for (int64_t s = 0; s < max_len && ce == cudaSuccess; ++s) {
        pdl_scope() = pdl_enabled() && n_evolve(s) <= c->n_sm;
        ce = launch_evolve(gg, SS, d_recs, c->d_ss, c->d_off, d_prm, n_evolve(s), (int)s, d_out, c->stream);
        pdl_scope() = false;
        if (ce == cudaSuccess) ce = c->launch_radiation(gg, SS, d_prm, n_radiate(s), (int)s);
      }
      if (ce == cudaSuccess)
        ce = launch_finalize(gg, SS, c->d_off, d_prm, longer(max_len - 1), (int)(max_len - 1), d_out, c->stream);
      cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
      if (ce != cudaSuccess || ee != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        return PBAG_ERR_CUDA;
      }
      ee = cudaGraphInstantiate(&c->graph_exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ee != cudaSuccess) {
        c->graph_exec = nullptr;
        return PBAG_ERR_CUDA;
      }
      c->graph_key = key;
    }
    if (cudaGraphLaunch(c->graph_exec, c->stream) != cudaSuccess) return PBAG_ERR_CUDA;
    c->launches += (c->ssc_on_tensor_cores() ? 2 + c->ssc_side_launches() : 2) * max_len + 1;
    max_len = 0;  // the loop below has nothing left to launch
  }
  for (int64_t s = 0; s < max_len; ++s) {
    if (!mark(kClassEvolve, true)) return PBAG_ERR_CUDA;
    if ((e = launch_evolve(gg, SS, d_recs, c->d_ss, c->d_off, d_prm, n_evolve(s), (int)s, d_out, c->stream)) !=
        cudaSuccess)
      return PBAG_ERR_CUDA;
    if (!mark(kClassEvolve, false)) return PBAG_ERR_CUDA;
    if (!mark(kClassSsc, true)) return PBAG_ERR_CUDA;
    if ((e = c->launch_radiation(gg, SS, d_prm, n_radiate(s), (int)s)) != cudaSuccess) return PBAG_ERR_CUDA;
    if (!mark(kClassSsc, false)) return PBAG_ERR_CUDA;
    c->launches += c->ssc_on_tensor_cores() ? 3 : 2;
    if (s == max_len - 1) {
      if (!mark(kClassFinalize, true)) return PBAG_ERR_CUDA;
      if ((e = launch_finalize(gg, SS, c->d_off, d_prm, longer(s), (int)s, d_out, c->stream)) != cudaSuccess)
        return PBAG_ERR_CUDA;
      if (!mark(kClassFinalize, false)) return PBAG_ERR_CUDA;
      c->launches += 1;
    }
  }
  std::vector<int> err((size_t)nbw * 4);
  if (nbw > 0 && cudaMemcpyAsync(err.data(), c->S.err, err.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                 c->stream) != cudaSuccess)
    return PBAG_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PBAG_ERR_CUDA;
  for (size_t k = 0; k + 1 < nev; k += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]) != cudaSuccess) return PBAG_ERR_CUDA;
    c->class_ms[c->ev_class[k / 2]] += ms;
    c->class_launches[c->ev_class[k / 2]] += 1;
  }
  // the reference stops at the first failure in time order (then blastwave order)
  int code = PBAG_OK, fb = -1, fs = -1, site = 0;
  for (int b = 0; b < nbw; ++b) {
    const size_t k = 4 * (size_t)(c->slot_of.empty() ? b : c->slot_of[b]);  // the blastwave's slot
    if (err[k] != 0 && (fs < 0 || err[k + 1] < fs)) {
      code = err[k];
      fb = b;
      fs = err[k + 1];
      site = err[k + 2];
    }
  }
  if (st) {
    st->code = code;
    st->bw = fb;
    st->step = fs;
    st->site = site;
  }
  return code;
}

// The synchrotron / SSA sums run on the tensor cores when the grid and the
// batch allow it (every blastwave of one synchrotron method class, the SSC
// contraction on the tensor cores or off); a field outside the bank's range
// reruns the batch with the CUDA-core sums. hprm: the shock parameters on the host.
int run_device(pbag_ctx* c, const pbag_shock_params* hprm, const pbag_shock_params* d_prm, int nbw,
               const int64_t* off_h, const pbag_step_rec* d_recs, const pbag_outputs& d_out, pbag_status* st) {
  int cls = -1;
  if (c->syn_tc_enabled(nbw) && nbw > 0) {
    bool any_ssc = false;
    cls = pbag_ctx::syn_class(hprm[0].syn_method);
    for (int b = 0; b < nbw; ++b) {
      any_ssc = any_ssc || hprm[b].ssc_on;
      if (pbag_ctx::syn_class(hprm[b].syn_method) != cls) cls = -1;
    }
    if (cls >= 0 && any_ssc && !c->ssc_on_tensor_cores()) cls = -1;  // the CUDA-core SSC kernel sums both
  }
  pbag_status ls{};
  int rc = run_device_once(c, d_prm, nbw, off_h, d_recs, d_out, &ls, cls);
  if (cls >= 0 && rc == PBAG_ERR_UNSUPPORTED && ls.site == kSiteSynBank)
    rc = run_device_once(c, d_prm, nbw, off_h, d_recs, d_out, &ls, -1);
  if (st) *st = ls;
  return rc;
}

void reset_status(pbag_status* st) {
  if (!st) return;
  st->code = PBAG_ERR_ARG;
  st->bw = st->step = -1;
  st->site = 0;
}

}  // namespace

extern "C" {

int pbag_create(const pbag_grid_desc* g, int device, int ssc_tables, pbag_ctx** out) {
  if (!out) return PBAG_ERR_ARG;
  *out = nullptr;
  if (!g || g->ngam < PBAG_MIN_BINS || g->ngam > PBAG_MAX_BINS || g->nfreq < PBAG_MIN_BINS ||
      g->nfreq > PBAG_MAX_BINS || !(g->gam2 > 1.) || !(g->freq1 > 0.) || !(g->freq2 > g->freq1))
    return PBAG_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PBAG_ERR_CUDA;
  if (configure_kernels() != cudaSuccess) return PBAG_ERR_CUDA;
  pbag_ctx* c = new (std::nothrow) pbag_ctx();
  if (!c) return PBAG_ERR_NOMEM;
  c->device = device;
  c->desc = *g;
  c->G = g->ngam;
  c->F = g->nfreq;
  c->Gp = (c->G + 15) / 16 * 16;
  c->ssc = ssc_tables != 0;
  if (cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    delete c;
    return PBAG_ERR_CUDA;
  }
  const int G = c->G, F = c->F;
  c->gam.assign(G, 0.);
  c->freq.assign(F + 1, 0.);
  build_grids(g, c->gam.data(), c->freq.data());
  const std::vector<double>& e = c->gam;
  const std::vector<double>& nu = c->freq;
  // derived tables (base_state.h:229-250 and the per-step products of
  // numeric_model.h / microphysics.h, tabulated once)
  const double step = std::exp(std::log(g->gam2) / (double)G);
  std::vector<double> inv_e(G), inv_e2(G), de(G - 1), e2de(G - 1), inv_dxm(G, 0.), half2(G - 1), hadi(G - 1),
      ihalf2(G - 1), dg(G + 1), inv_dgb(G), dnu(F), inv_hnu(F), ssa_nu(F);
  std::vector<float> ginv2(G), psq(G), ginv23(G), nu13(F), nu32(F);
  for (int i = 0; i < G; ++i) {
    inv_e[i] = 1. / e[i];
    inv_e2[i] = 1. / e[i] / e[i];
    if (i > 0) inv_dxm[i] = 1. / (e[i] - e[i - 1]);
  }
  for (int i = 0; i < G - 1; ++i) {
    de[i] = e[i + 1] - e[i];
    e2de[i] = e[i] * e[i] * (e[i + 1] - e[i]);
    const double h = .5 * e[i] * (step + 1.0);
    half2[i] = h * h;
    hadi[i] = (h * h - 1.) / (3. * h);
    ihalf2[i] = 1. / h / h;
    dg[i + 1] = e[i + 1] - e[i];
  }
  dg[0] = e[0] * (1 - 1.0 / step);
  dg[G] = e[G - 1] * (step - 1);
  for (int i = 0; i < G; ++i) inv_dgb[i] = 1.0 / ((dg[i] + dg[i + 1]) / 2.);
  int n_cyc = 0;
  for (int i = 0; i < G; ++i) {
    ginv2[i] = (float)(1. / (e[i] * e[i]));
    psq[i] = (float)(e[i] * e[i] - 1.);
    ginv23[i] = (float)std::pow(e[i], -2. / 3.);
    if (e[i] <= 2.) n_cyc = i + 1;
  }
  for (int k = 0; k < F; ++k) {
    dnu[k] = (nu[k + 1] - nu[k]) / nu[k];
    nu13[k] = (float)std::cbrt(nu[k]);
    nu32[k] = (float)nu[k];
    inv_hnu[k] = 1. / (cgs::h_pl * nu[k]);
    ssa_nu[k] = -1. / (8. * M_PI * cgs::m_e * nu[k] * nu[k]);
  }
  DevGrid& d = c->dg;
  d.G = G;
  d.F = F;
  d.Gp = c->Gp;
  d.n_cyc = n_cyc;
  {
    const char* sf = std::getenv("PBAG_SCAN_FP64");
    d.scan_fp64 = (sf && sf[0] == '1') ? 1 : 0;
    const char* sm = std::getenv("PBAG_SYSTOLIC_MIN");
    const int v = sm ? std::atoi(sm) : 0;
    d.sys_min_sub = v >= 2 ? v : kScanMaxSub;
    const char* ec = std::getenv("PBAG_EVOLVE_CTAS");
    d.evolve_ctas = ec ? std::atoi(ec) : 4;
  }
  d.dlog_gam = (e[1] - e[0]) / e[0];
  cudaError_t err = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (err == cudaSuccess) err = x;
  };
  ok(c->grid_upload(&d.e, e));
  ok(c->grid_upload(&d.inv_e, inv_e));
  ok(c->grid_upload(&d.inv_e2, inv_e2));
  ok(c->grid_upload(&d.de, de));
  ok(c->grid_upload(&d.e2de, e2de));
  ok(c->grid_upload(&d.inv_dxm, inv_dxm));
  ok(c->grid_upload(&d.half2, half2));
  ok(c->grid_upload(&d.hadi, hadi));
  ok(c->grid_upload(&d.ihalf2, ihalf2));
  ok(c->grid_upload(&d.inv_dgb, inv_dgb));
  ok(c->grid_upload(&d.ginv2, ginv2));
  ok(c->grid_upload(&d.psq32, psq));
  ok(c->grid_upload(&d.ginv23, ginv23));
  {
    // pair-production rate kernel R (numeric_model.h:295-303) on the grids
    auto ppR = [](double nu, double nu_t) {
      const double x = nu * nu_t;
      const double l = cgs::h_pl / cgs::m_e / cgs::c_light / cgs::c_light;
      const double v = x * l * l;
      return v - 1 > 0 ? 0.652 * cgs::c_light * cgs::sigma_T * (v * v - 1) * std::log(v) / (v * v * v) : 0.;
    };
    const int Gs = (G + 3) / 4 * 4;  // the row stride of KintT (d.Gs)
    std::vector<float> inj((size_t)F * Gs, 0.f), ab((size_t)F * F, 0.f);
    std::vector<int> idx(G, F - 1);
    const double c4 = cgs::c_light * cgs::c_light * cgs::c_light * cgs::c_light;
    for (int i = 0; i < G; ++i) {
      const double nu1 = 2. * e[i] * cgs::m_e * cgs::c_light * cgs::c_light / cgs::h_pl;
      for (int k = 0; k < F - 1; ++k)
        if ((nu[k] < nu1) && (nu[k + 1] >= nu1)) {
          idx[i] = k;
          break;
        }
      for (int k = 0; k < F - 1; ++k) {
        if (nu[k] * nu1 * cgs::h_pl * cgs::h_pl / cgs::m_e / cgs::m_e / c4 < 1.) continue;
        inj[(size_t)k * Gs + i] = (float)(ppR(nu1, nu[k]) * (nu[k + 1] - nu[k]));
      }
    }
    for (int i = 0; i < F; ++i)
      for (int k = 0; k < F - 1; ++k) ab[(size_t)k * F + i] = (float)(ppR(nu[i], nu[k]) * (nu[k + 1] - nu[k]) / cgs::c_light);
    ok(c->grid_upload(&d.ppinjT, inj));
    ok(c->grid_upload(&d.ppidx, idx));
    ok(c->grid_upload(&d.ppabsT, ab));
  }
  {
    // tabulated synchrotron functions of the GSL and Bessel methods
    std::vector<float> lg(G);
    for (int i = 0; i < G; ++i) lg[i] = (float)(-2. * std::log(e[i]));
    ok(c->grid_upload(&d.lnginv2, lg));
    double u0 = 0., h = 0.;
    int tn = 0;
    syn_table_grid(std::log(e[1] / e[0]), &u0, &h, &tn);
    std::vector<float> st = syn_table(PBAG_SYN_GSL, u0, h, tn), sb = syn_table(PBAG_SYN_BESSEL, u0, h, tn),
                       sa = syn_table(PBAG_SYN_CSYN, u0, h, tn);
    st.insert(st.end(), sb.begin(), sb.end());
    st.insert(st.end(), sa.begin(), sa.end());
    std::vector<float> lnu(F);
    for (int k = 0; k < F; ++k) lnu[k] = (float)std::log(nu[k]);
    ok(c->grid_upload(&d.lnnu, lnu));
    ok(c->grid_upload(&d.syntab, st));
    d.syn_u0 = (float)u0;
    d.syn_ih = (float)(1. / h);
    d.syn_n = tn;
    // value / slope pairs for the batch sums (a coarser grid, matched the same way)
    double u2 = 0., h2 = 0.;
    int n2 = 0;
    syn_table_grid(std::log(e[1] / e[0]), &u2, &h2, &n2, kSynTab2N);
    std::vector<float> t2;
    for (int m : {PBAG_SYN_GSL, PBAG_SYN_BESSEL, PBAG_SYN_CSYN}) {
      const std::vector<float> t = syn_table2(m, u2, h2, n2);
      t2.insert(t2.end(), t.begin(), t.end());
    }
    const float* t2p = nullptr;
    ok(c->grid_upload(&t2p, t2));
    d.syntab2 = reinterpret_cast<const float2*>(t2p);
    d.syn2_u0 = (float)u2;
    d.syn2_ih = (float)(1. / h2);
    d.syn2_n = n2;
    // GSL: x = (h nu / m_e c^2) / (1.5 B gamma^2 / 4.14e13) against nu / nu_crit = nu 4 pi m_e c / (3 q B gamma^2)
    d.gsl_xs = (float)(cgs::h_by_mec2 * 4.14e13 / 1.5 / (4. * M_PI * cgs::m_e * cgs::c_light / (3. * cgs::q_e)));
    // the tensor-core synchrotron sums (pbag_syn_tc.cu): the bank's geometry;
    // the banks themselves are built on first use, per method class
    if (syn_tc_supported(G, F)) {
      const double xs = cgs::h_by_mec2 * 4.14e13 / 1.5 / (4. * M_PI * cgs::m_e * cgs::c_light / (3. * cgs::q_e));
      c->sb_dnu = std::log(nu[1] / nu[0]);
      syn_tc_geometry(c->sb_dnu, nu[0], xs, F, &c->sb);
      d.sb_P = c->sb.P;
      d.sb_M = c->sb.M;
      d.sb_mlo = c->sb.mlo;
      d.sb_nlo = c->sb.n_lo;
      d.sb_nhi = c->sb.n_hi;
      d.sb_ih = 1. / c->sb.h;
      d.sb_lnnu0 = std::log(nu[0]);
      d.sb_lnxs_gsl = std::log(xs);
      d.sb_tbw = syn_tc_tile_bw(c->Gp);
      c->sb_ok = true;
    }
  }
  ok(c->grid_upload(&d.nu13, nu13));
  ok(c->grid_upload(&d.nu32, nu32));
  ok(c->grid_upload(&d.nu, nu));
  ok(c->grid_upload(&d.dnu_nu, dnu));
  ok(c->grid_upload(&d.inv_hnu, inv_hnu));
  {
    std::vector<double> hnu(F);
    for (int k = 0; k < F; ++k) hnu[k] = cgs::h_pl * nu[k];
    ok(c->grid_upload(&d.hnu, hnu));
  }
  ok(c->grid_upload(&d.ssa_nu, ssa_nu));
  {
    // mantissa / exponent tables (f64_mant) of dgamma, dgamma/gamma^2, dnu/nu
    d.Tm = std::max(G, F);
    std::vector<float> tm((size_t)kM32 * d.Tm, 0.f);
    std::vector<int> te((size_t)kM32 * d.Tm, kExpZero);
    auto put = [&](int t, int i, double x) {
      if (x == 0.) return;
      int ex = 0;
      const double fr = std::frexp(x, &ex);  // x = fr 2^ex, |fr| in [0.5, 1)
      float m = (float)(2. * fr);
      int e2 = ex - 1;
      if (std::fabs(m) >= 2.f) {
        m *= 0.5f;
        ++e2;
      }
      tm[(size_t)t * d.Tm + i] = m;
      te[(size_t)t * d.Tm + i] = e2;
    };
    for (int j = 0; j < G - 1; ++j) {
      put(kM32De, j, de[j]);
      put(kM32DeIe2, j, de[j] * inv_e2[j]);
    }
    for (int k = 0; k < F; ++k) put(kM32DnuNu, k, dnu[k]);
    ok(c->grid_upload(&d.tmant, tm));
    ok(c->grid_upload(&d.texp, te));
  }
  // the evolve kernel's tables in one block (GridTab layout)
  d.Ge = (G + 1) / 2 * 2;
  d.Fe = (F + 1) / 2 * 2;
  d.etab_doubles = kTabG * d.Ge + kTabF * d.Fe;
  std::vector<double> etab((size_t)d.etab_doubles, 0.);
  {
    const std::vector<double>* gsrc[kTabG] = {&inv_e, &inv_e2, &de, &e2de, &inv_dxm, &half2, &hadi, &ihalf2, &inv_dgb};
    for (int t = 0; t < kTabG; ++t) std::copy(gsrc[t]->begin(), gsrc[t]->end(), etab.begin() + (size_t)t * d.Ge);
    const size_t fb = (size_t)kTabG * d.Ge;
    std::copy(dnu.begin(), dnu.end(), etab.begin() + fb + (size_t)kTabDnuNu * d.Fe);
    std::copy(inv_hnu.begin(), inv_hnu.end(), etab.begin() + fb + (size_t)kTabInvHnu * d.Fe);
    std::fill(etab.begin() + fb + (size_t)kTabKscale * d.Fe, etab.begin() + fb + (size_t)kTabKscale * d.Fe + F, 1.);
    std::copy(ssa_nu.begin(), ssa_nu.end(), etab.begin() + fb + (size_t)kTabSsaNu * d.Fe);
  }
  d.Gs = (G + 3) / 4 * 4;
  d.kint_stage = 0;
  d.KintT = nullptr;
  d.kscale = nullptr;
  d.K32 = nullptr;
  d.Bt = nullptr;
  if (c->ssc) {
    std::vector<float> KintT, K32;
    std::vector<double> kscale;
    std::vector<uint16_t> Bt;
    build_ssc_tables(e.data(), G, nu.data(), F, c->Gp, d.Gs, KintT, kscale, K32);
    ok(c->grid_upload(&d.KintT, KintT));
    const size_t kbytes = KintT.size() * sizeof(float);
    d.kint_stage = kbytes <= kKintStageMax ? (int)kbytes : 0;
    ok(c->grid_upload(&d.kscale, kscale));
    std::copy(kscale.begin(), kscale.end(), etab.begin() + (size_t)kTabG * d.Ge + (size_t)kTabKscale * d.Fe);
    ok(c->grid_upload(&d.K32, K32));
    if (ssc_tc_supported(F)) {
      build_ssc_tc_operand(K32, F, c->Gp, Bt);
      ok(c->grid_upload(&d.Bt, Bt));
    }
    ok(cudaStreamSynchronize(c->stream));  // the host vectors go out of scope
  }
  ok(c->grid_upload(&d.etab, etab));
  ok(cudaStreamSynchronize(c->stream));
  if (err != cudaSuccess) {
    const int code = cuda_code(err);
    delete c;
    return code;
  }
  *out = c;
  return PBAG_OK;
}

void pbag_destroy(pbag_ctx* c) { delete c; }

int pbag_run_batch(pbag_ctx* c, const pbag_shock_params* prm, int nbw, const int64_t* off,
                   const pbag_step_rec* recs, const pbag_outputs* out, pbag_status* st) {
  reset_status(st);
  if (!c || !out || (nbw > 0 && (!prm || !recs))) return PBAG_ERR_ARG;
  int rc = check_batch(c, prm, nbw, off);
  if (rc != PBAG_OK) {
    if (st) st->code = rc;
    return rc;
  }
  if (cudaSetDevice(c->device) != cudaSuccess) return PBAG_ERR_CUDA;
  const size_t nrec = (size_t)off[nbw];
  cudaError_t e = c->reserve_bw(nbw);
  if (e != cudaSuccess) return cuda_code(e);
  if ((e = c->reserve_rec(nrec, true)) != cudaSuccess) return cuda_code(e);
  // device output buffers for the requested histories
  const double* const* outp = reinterpret_cast<const double* const*>(out);
  size_t need = 0;
  for (int fi = 0; fi < kOutputs; ++fi)
    if (outp[fi]) need += nrec * (output_on_gamma(fi) ? (size_t)c->G : (size_t)c->F);
  if (need > c->cap_out) {
    cudaFree(c->d_out);
    c->d_out = nullptr;
    c->cap_out = 0;
    if ((e = dev_alloc(&c->d_out, need)) != cudaSuccess) return cuda_code(e);
    c->cap_out = need;
  }
  pbag_outputs dout{};
  double** dp = reinterpret_cast<double**>(&dout);
  size_t pos = 0;
  for (int fi = 0; fi < kOutputs; ++fi) {
    if (!outp[fi]) continue;
    dp[fi] = c->d_out + pos;
    pos += nrec * (output_on_gamma(fi) ? (size_t)c->G : (size_t)c->F);
  }
  if (nrec && cudaMemcpyAsync(c->d_recs, recs, nrec * sizeof(pbag_step_rec), cudaMemcpyHostToDevice, c->stream) !=
                  cudaSuccess)
    return PBAG_ERR_CUDA;
  if (nbw && cudaMemcpyAsync(c->d_prm, prm, nbw * sizeof(pbag_shock_params), cudaMemcpyHostToDevice, c->stream) !=
                 cudaSuccess)
    return PBAG_ERR_CUDA;
  rc = run_device(c, prm, c->d_prm, nbw, off, c->d_recs, dout, st);
  if (rc == PBAG_ERR_CUDA || rc == PBAG_ERR_NOMEM) return rc;
  // copy the histories back even on a physics error (rows before the failure are valid)
  for (int fi = 0; fi < kOutputs; ++fi) {
    if (!outp[fi]) continue;
    const size_t n = nrec * (output_on_gamma(fi) ? (size_t)c->G : (size_t)c->F);
    if (n && cudaMemcpyAsync((void*)outp[fi], dp[fi], n * sizeof(double), cudaMemcpyDeviceToHost, c->stream) !=
                 cudaSuccess)
      return PBAG_ERR_CUDA;
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PBAG_ERR_CUDA;
  return rc;
}

int pbag_run_batch_device(pbag_ctx* c, const pbag_shock_params* d_prm, int nbw, const int64_t* off,
                          const pbag_step_rec* d_recs, const pbag_outputs* d_out, pbag_status* st, void* stream) {
  reset_status(st);
  if (!c || !d_out || (nbw > 0 && (!d_prm || !d_recs))) return PBAG_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return PBAG_ERR_CUDA;
  // the inputs may come from work still running on the caller's stream
  if (stream && cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess) return PBAG_ERR_CUDA;
  std::vector<pbag_shock_params> hp((size_t)std::max(nbw, 0));
  if (nbw > 0 && cudaMemcpy(hp.data(), d_prm, hp.size() * sizeof(pbag_shock_params), cudaMemcpyDeviceToHost) !=
                     cudaSuccess)
    return PBAG_ERR_CUDA;
  int rc = check_batch(c, hp.data(), nbw, off);
  if (rc != PBAG_OK) {
    if (st) st->code = rc;
    return rc;
  }
  return run_device(c, hp.data(), d_prm, nbw, off, d_recs, *d_out, st);
}

int64_t pbag_last_launch_count(const pbag_ctx* c) { return c ? c->launches : -1; }

int pbag_set_ssc_path(pbag_ctx* c, int path) {
  if (!c || path < PBAG_SSC_AUTO || path > PBAG_SSC_SURROGATE) return PBAG_ERR_ARG;
  if ((path == PBAG_SSC_TC_SPLIT_BF16 || path == PBAG_SSC_TC_BF16) && !c->dg.Bt) return PBAG_ERR_UNSUPPORTED;
  if (path == PBAG_SSC_SURROGATE && !surrogate_ready(c)) return PBAG_ERR_ARG;  // pbag_surrogate_configure first
  c->ssc_path = path;
  return PBAG_OK;
}

int pbag_set_timing(pbag_ctx* c, int enable) {
  if (!c) return PBAG_ERR_ARG;
  c->timing = enable != 0;
  for (int k = 0; k < kKernelClasses; ++k) {
    c->class_ms[k] = 0.;
    c->class_launches[k] = 0;
  }
  return PBAG_OK;
}

int pbag_get_timing(const pbag_ctx* c, double* ms, int64_t* launches) {
  if (!c || !ms || !launches) return PBAG_ERR_ARG;
  for (int k = 0; k < kKernelClasses; ++k) {
    ms[k] = c->class_ms[k];
    launches[k] = c->class_launches[k];
  }
  return PBAG_OK;
}

}  // extern "C"

namespace pbag {

CtxExtension* ctx_get_extension(pbag_ctx* c, int slot) {
  return c && slot >= 0 && slot < kExtSlots ? c->ext[slot] : nullptr;
}
void ctx_set_extension(pbag_ctx* c, int slot, CtxExtension* x) {
  if (!c || slot < 0 || slot >= kExtSlots) return;
  delete c->ext[slot];
  c->ext[slot] = x;
}

void ctx_set_launches(pbag_ctx* c, int64_t n) {
  if (c) c->launches = n;
}

bool ctx_syn_bank(pbag_ctx* c, int syn_method, DevGrid* g) {
  if (!c || !g || !c->syn_tc_enabled()) return false;
  return c->syn_bank(pbag_ctx::syn_class(syn_method), &g->synbank) == cudaSuccess;
}

bool ctx_view(const pbag_ctx* c, CtxView* v) {
  if (!c || !v) return false;
  v->device = c->device;
  v->stream = c->stream;
  v->dg = c->dg;
  v->ssc = c->ssc;
  v->G = c->G;
  v->F = c->F;
  v->Gp = c->Gp;
  return true;
}

}  // namespace pbag
