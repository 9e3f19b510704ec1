// pbag_internal.h - declarations shared between the host and device
// translation units of libpbag (not part of the C ABI).
#ifndef PBAG_INTERNAL_H
#define PBAG_INTERNAL_H

#include "pbag.h"

namespace pbag {

// Electron grid gam[G] and photon grid freq[F+1] (see pbag_build_grids).
void build_grids(const pbag_grid_desc* g, double* gam, double* freq);

}  // namespace pbag

#endif
