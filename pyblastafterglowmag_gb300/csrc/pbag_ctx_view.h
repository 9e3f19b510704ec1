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

// A per-context workspace owned by an entry point of another translation
// unit: created on first use, destroyed with the context.
struct CtxExtension {
  virtual ~CtxExtension() = default;
};
enum : int { kExtContract = 0, kExtSlots = 2 };
CtxExtension* ctx_get_extension(pbag_ctx* c, int slot);
void ctx_set_extension(pbag_ctx* c, int slot, CtxExtension* ext);

}  // namespace pbag

#endif
