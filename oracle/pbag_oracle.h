/*
 * pbag_oracle.h - CPU restatement (FP64) of the reference's comoving-radiation
 * step, used ONLY as the checker in tests, in smoke() and as the CPU-baseline
 * leg of bench.py. The product path never links or calls it.
 *
 * Every function follows the reference source cited beside it
 * (paths relative to the reference project's src/ directory).
 */
#ifndef PBAG_ORACLE_H
#define PBAG_ORACLE_H

#include "pbag.h"

#ifdef __cplusplus
extern "C" {
#endif

/* grids: gam[G] (base_state.h:217-253), freq[F+1] (utils.h MakeLogspaceVec;
 * freq[F] is the next logspace point, the value the oracle defines for the
 * one-past-the-end read in numeric_model.h:269-272). */
int orc_build_grids(const pbag_grid_desc* g, double* gam, double* freq);

/* single synchrotron kernel value K(nu; gamma, B) (kernels.h:211-522) */
double orc_syn_func(int method, double B, double nu, double gam);
/* single SSC kernel value (kernels.h:96-117) */
double orc_ssc_func(double nu, double gam, double nu_tilde);

/* SSC kernel tensor K[i][j][k] (may be NULL) and Kint[j][k] (kernels.h:49-94) */
int orc_ssc_kernel(const double* gam, int G, const double* freq, int F, double* K, double* Kint);

/* Emissivity contractions of n comoving states on the grid g: jsyn[s][k]
 * (computeSynSpectrum, numeric_model.h:148-184, kernel at field B[s]) and
 * jssc[s][i] (computeSSCSpectrum, numeric_model.h:247-285, seed photon
 * density nph[s]) from the electron spectra f[s][G]. jsyn or jssc may be
 * NULL. threads > 1 runs states concurrently. */
int orc_contract(const pbag_grid_desc* g, int n, const double* f, const double* B, const double* nph, int syn_method,
                 double* jsyn, double* jssc, int threads);

/* fluxDens / computeFluxDensity (microphysics.h:799-867, 1185-1217) for nq
 * queries over the histories of a batch; on a failure the failing query's
 * index in *fail_index and the status code. */
int orc_flux_dens(const pbag_grid_desc* g, const pbag_flux_opts* o, const int64_t* offsets, const double* j_all,
                  const double* a_all, const double* r_all, int nq, const pbag_flux_query* qs, double* flux,
                  int* fail_index);

/* Per-step shock scalars of one blastwave object over n consecutive calls of
 * updateSockProperties + computeEleSpectrumLimits (microphysics_base.h:575-605,
 * 642-652, 736-966; Bisect rootfinders.h:17-58), with the same arguments and
 * the same persistent-state convention as pbag_shock_limits (pbag.h). */
int orc_shock_limits(const pbag_limits_opts* o, const double* gam, int ngam, int n, const pbag_shock_state* in,
                     double* state, pbag_limits* out);

/* Flags for orc_run. */
enum {
  ORC_HOIST_HEATING = 1,  /* compute the (substep-invariant) cooling terms once per
                             step instead of once per substep as the reference does;
                             results are bitwise identical, only faster            */
  ORC_INNER_OMP = 2       /* parallelise the inner nu loops with inner_threads, like
                             the reference's num_threads(4) pragmas                 */
};

/* Full histories of nbw blastwaves (see pbag.h for the record and output
 * layouts). outer_threads > 1 runs blastwaves concurrently (one per thread,
 * private state). Returns PBAG_OK or the first error; st (may be NULL)
 * receives the failing blastwave/step. */
int orc_run(const pbag_grid_desc* g, const pbag_shock_params* prm, int nbw, const int64_t* offsets,
            const pbag_step_rec* recs, pbag_outputs* out, int flags, int outer_threads,
            int inner_threads, pbag_status* st);

/* Adaptive EATS light curve of nl layers (pbag_eats_flux_a's inputs on the
 * host): flux[q] in mJy for every query; histories j_all / a_all of the
 * blastwaves the layers name (offsets as for orc_run). Returns PBAG_OK or the
 * first failure (*fail_index = its query). */
int orc_eats_flux(const pbag_grid_desc* g, const pbag_eats_opts* o, int nl, const pbag_eats_layer* layers, int nr,
                  const double* dyn, const int64_t* offsets, const double* j_all, const double* a_all, int nq,
                  const pbag_eats_query* qs, double* flux, int* fail_index);

#ifdef __cplusplus
}
#endif
#endif
