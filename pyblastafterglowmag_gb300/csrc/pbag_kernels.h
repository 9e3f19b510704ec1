// pbag_kernels.h - host-callable launchers of the device kernels (internal).
#ifndef PBAG_KERNELS_H
#define PBAG_KERNELS_H

#include <cuda_runtime.h>

#include <vector>

#include "pbag_device.cuh"

namespace pbag {

cudaError_t launch_evolve_radiate(const DevGrid& g, const DevState& S, const pbag_step_rec* recs, const int64_t* off,
                                  const pbag_shock_params* prm, int nbw, int step, cudaStream_t st);
cudaError_t launch_finalize(const DevGrid& g, const DevState& S, const int64_t* off, const pbag_shock_params* prm,
                            int nbw, int step, const pbag_outputs& out, cudaStream_t st);
cudaError_t launch_ssc_contract(const DevGrid& g, const DevState& S, int nbw, cudaStream_t st);

// SSC kernel tables on the host (kernels.h:49-117): Kint[G][F] in FP64 and
// K32[F][Gp][F] (i, j, k) in FP32, j >= G zero-padded.
void build_ssc_tables(const double* gam, int G, const double* freq, int F, int Gp, std::vector<double>& Kint,
                      std::vector<float>& K32);

}  // namespace pbag

#endif
