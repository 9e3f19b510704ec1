// pbag_ctx_view.h - read-only view of a context for entry points that live in
// other translation units (internal).
#ifndef PBAG_CTX_VIEW_H
#define PBAG_CTX_VIEW_H

#include <cuda_runtime.h>

#include "pbag_device.cuh"

namespace pbag {

struct CtxView {
  int device;
  cudaStream_t stream;
  DevGrid dg;
  bool ssc;
  int G, F, Gp;
};

// Fills *v from c; false when c is null.
bool ctx_view(const pbag_ctx* c, CtxView* v);
// The kernel count pbag_last_launch_count reports for c's last run.
void ctx_set_launches(pbag_ctx* c, int64_t n);
// The tensor-core synchrotron bank of syn_method into g->synbank (built on
// first use); false when the context's grid or the environment rules it out.
bool ctx_syn_bank(pbag_ctx* c, int syn_method, DevGrid* g);

// A per-context workspace owned by an entry point of another translation
// unit: created on first use, destroyed with the context.
struct CtxExtension {
  virtual ~CtxExtension() = default;
};
enum : int { kExtContract = 0, kExtSurrogate = 1, kExtSlots = 2 };
CtxExtension* ctx_get_extension(pbag_ctx* c, int slot);
void ctx_set_extension(pbag_ctx* c, int slot, CtxExtension* ext);

// pbag_surrogate.cu: the surrogate SSC contraction of nrows rows (see there)
cudaError_t surrogate_run(pbag_ctx* ctx, const CtxView& v, int nrows, const void* Wt, const int* flags,
                          const float* U32, const double* scal, const double* f, int fs, const double* nph, int ns,
                          const double* Bv, int bs, double* out, int* errs, cudaStream_t st,
                          bool host_count = false);
bool surrogate_ready(pbag_ctx* ctx);
cudaError_t surrogate_reserve(pbag_ctx* ctx, int n);
int64_t surrogate_generation(pbag_ctx* ctx);
int surrogate_launches(const pbag_ctx* ctx);

// pbag_contract.cu: reserve the contraction workspace for n states and build
// their split-BF16 operands (W tiles, U32, scales) into S / Wt
int contract_prepare(pbag_ctx* ctx, const CtxView& v, int n, const double* d_f, const double* d_nph, DevState* S,
                     const void** Wt);

}  // namespace pbag

#endif
