/*
 * pbag.h - C ABI of the GB300 comoving-radiation step for PyBlastAfterglowMag.
 *
 * One "blastwave" is one (layer, shock) pair: one ElectronAndRadiation object
 * in the reference (src/microphysics/microphysics.h:60). One "step" of a
 * blastwave is the pair of calls the reference's blastwave driver makes at one
 * burster-frame time index (src/blastwave/blastwave_radiation.h:1109-1182):
 *   initializeElectronDistribution      (microphysics.h:347)   on the first valid step, or
 *   evaluateElectronDistributionNumericMixed (microphysics.h:359) on later ones,
 * followed by
 *   computeRadiationNumericMixed(it)     (microphysics.h:492).
 *
 * A caller records one pbag_step_rec per (blastwave, time index) - the scalar
 * arguments of those calls plus the members that computeEleSpectrumLimits()
 * (microphysics_base.h:642) set just before them - and hands the whole history
 * of a batch of blastwaves to pbag_run_batch(), which evolves all of them on
 * one GPU and fills the same time-major "*_all" arrays the reference fills
 * (base_state.h:200-211, 288-296).
 *
 * All functions return PBAG_OK (0) or a negative pbag_status code; they never
 * throw and never exit the process. Pointers are plain host or device pointers
 * as each function documents; sizes are element counts.
 */
#ifndef PBAG_H
#define PBAG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBAG_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum pbag_status_code {
  PBAG_OK = 0,
  PBAG_ERR_ARG = -1,        /* bad argument (null pointer, size out of range) */
  PBAG_ERR_CUDA = -2,       /* a CUDA runtime call failed                      */
  PBAG_ERR_NONFINITE = -3,  /* NaN / negative value where the reference exits  */
  PBAG_ERR_NELE = -4,       /* total electron number <= 0 (microphysics.h:560) */
  PBAG_ERR_PARAM = -5,      /* B<=0, gamma_min<1, ... (microphysics.h:372)     */
  PBAG_ERR_DLNVDT = -6,     /* dlnV/dt negative or not finite (microphysics.h:406) */
  PBAG_ERR_UNSUPPORTED = -7,/* option the GPU path does not implement          */
  PBAG_ERR_TIMEOUT = -8,    /* a bounded device-side wait ran out              */
  PBAG_ERR_NOMEM = -9,      /* device allocation failed                        */
  PBAG_ERR_RANGE = -10,     /* frequency outside the grid (microphysics.h:1190-1201) */
  PBAG_ERR_EVALS = -11      /* EATS quadrature past 1e7 integrand evaluations (eats.h:536-541) */
};

/* ---- options (same meaning as the reference's parfile options) ----------- */
enum pbag_mode {            /* what the blastwave driver does at this step      */
  PBAG_SKIP = 0,            /* blastwave not valid at this step: no call        */
  PBAG_INIT = 1,            /* valid step; the driver's first valid step calls   */
  PBAG_EVOLVE = 2           /* initializeElectronDistribution, later ones call    */
                            /* evaluateElectronDistributionNumericMixed; both are */
                            /* followed by computeRadiationNumericMixed. INIT and */
                            /* EVOLVE are equivalent: like the driver, the step   */
                            /* initialises iff no earlier step of this blastwave  */
                            /* was valid (blastwave_radiation.h:1160-1175).       */
};
enum pbag_syn_method {      /* method_synchrotron_{fs,rs} (microphysics_base.h:304-349) */
  PBAG_SYN_CSYN = 0,        /* "CSYN": SynKernel::cycSynch (kernels.h:414), the default */
  PBAG_SYN_DER09 = 1,       /* "Dermer09": SynKernel::synchDermer (kernels.h:451)      */
  PBAG_SYN_GSL = 2,         /* "GSL": SynKernel::synchGSL (kernels.h:211)              */
  PBAG_SYN_BESSEL = 3       /* "Bessel": SynKernel::synchBessel (kernels.h:396)        */
};
enum pbag_ele_method {      /* method_ele_{fs,rs} (microphysics_base.h:254-276) */
  PBAG_ELE_NUMERIC = 1,     /* "numeric": Chang-Cooper evolution                */
  PBAG_ELE_MIX = 2          /* "mix": analytic N(gamma), numeric radiation      */
};

/* Grid description: the electron grid is rebuilt as e[i] = step^i with
 * step = exp(ln(gam2)/ngam) (base_state.h:217-253); the photon grid is
 * logspace(log10 freq1, log10 freq2, nfreq) built by repeated multiplication
 * (utils.h MakeLogspaceVec), shared by synchrotron, SSC and total spectra. */
typedef struct pbag_grid_desc {
  int32_t ngam;             /* G, 8..1024                                       */
  int32_t nfreq;            /* F, 8..1024                                       */
  double gam1, gam2;        /* gam1_{fs,rs}, gam2_{fs,rs}                       */
  double freq1, freq2;      /* freq1_{fs,rs}, freq2_{fs,rs} [Hz]                */
} pbag_grid_desc;

/* Per-blastwave options and parameters read by the numeric step. */
typedef struct pbag_shock_params {
  double p;                 /* p_{fs,rs}: injection index                       */
  double eps_e;             /* eps_e_{fs,rs} (diagnostics only)                 */
  int32_t max_substeps;     /* max_substeps_{fs,rs} (default 1000)              */
  int32_t ele_method;       /* pbag_ele_method                                  */
  int32_t syn_method;       /* pbag_syn_method                                  */
  int32_t ssa_on;           /* use_ssa_{fs,rs}                                  */
  int32_t ssc_on;           /* method_ssc_{fs,rs} == "numeric"                  */
  int32_t adi_on;           /* num_ele_use_adi_loss_{fs,rs} (default yes)       */
  int32_t pp_on;            /* method_pp_{fs,rs} "numeric": pair source, absorption and attenuation (needs ssc_on) */
  int32_t reserved;
} pbag_shock_params;

/* One step record: the arguments of the reference's per-step calls plus the
 * members computeEleSpectrumLimits() set before them.
 *  EVOLVE: evaluateElectronDistributionNumericMixed(tc, tc_p1, m, m_p1, rho, rho_p1,
 *          r, rp1, dr, dr_p1, u_p, u_p_p1)   (r, rp1 are unused by the reference)
 *  INIT:   initializeElectronDistribution(tc_p1, m_p1, rho_p1, u_p_p1, dr)        */
typedef struct pbag_step_rec {
  int32_t mode;             /* pbag_mode                                        */
  int32_t reserved;
  double tc, tc_p1;         /* comoving time at it-1, it [s]                    */
  double m, m_p1;           /* swept-up mass at it-1, it [g]                    */
  double rho, rho_p1;       /* comoving density at it-1, it [g/cm^3]            */
  double dr, dr_p1;         /* comoving shock thickness at it-1, it [cm]        */
  double u_p, u_p_p1;       /* comoving energy density at it-1, it [erg/cm^3]   */
  double B;                 /* comoving magnetic field [G]                      */
  double gamma_min, gamma_max, gamma_c, accel_frac, n_prime;
} pbag_step_rec;

/* Output histories. Row r of every array belongs to record r (rows of one
 * blastwave are consecutive, in step order); F = nfreq, G = ngam doubles per
 * row. Any pointer may be NULL: that history is not produced. Skipped steps
 * produce zero rows, as the reference's zero-initialised vectors do. */
typedef struct pbag_outputs {
  double* j_all;            /* total_rad.j_all  [nrec x F] emissivity per electron */
  double* a_all;            /* total_rad.a_all  [nrec x F] absorption             */
  double* f_all;            /* total_rad.f_all  [nrec x F] photon density         */
  double* i_all;            /* total_rad.i_all  [nrec x F] intensity              */
  double* ele_f_all;        /* ele.f_all        [nrec x G]  (save_spec)           */
  double* gdot_syn_all;     /* ele.gam_dot_syn_all [nrec x G]                     */
  double* gdot_adi_all;     /* ele.gam_dot_adi_all [nrec x G]                     */
  double* gdot_ssc_all;     /* ele.gam_dot_ssc_all [nrec x G]                     */
  double* syn_j_all;        /* syn.j_all        [nrec x F]                        */
  double* syn_a_all;        /* syn.a_all        [nrec x F]                        */
  double* syn_i_all;        /* syn.i_all        [nrec x F]                        */
  double* ssc_j_all;        /* ssc.j_all        [nrec x F]                        */
  double* ssc_i_all;        /* ssc.i_all        [nrec x F]                        */
} pbag_outputs;

/* First failure, in the reference's order of checks. */
typedef struct pbag_status {
  int32_t code;             /* pbag_status_code                                 */
  int32_t bw;               /* blastwave index of the first failure, or -1      */
  int32_t step;             /* step index within that blastwave, or -1          */
  int32_t site;             /* diagnostics: source line of the failing device check */
} pbag_status;

/* ---- per-step shock scalars (host) --------------------------------------
 * Options of ElectronAndRadiaionBase::computeEleSpectrumLimits
 * (microphysics_base.h:642-966); the enum values follow the parfile strings. */
typedef struct pbag_limits_opts {
  double p, eps_e, eps_b, eps_t;     /* p_, eps_e_, eps_b_, eps_t_{fs,rs}          */
  double beta_min;                   /* beta_min_{fs,rs} (default 1e-5)            */
  double mu, mu_e;                   /* 0.62, 1.18 (microphysics_base.h:103-104)   */
  int32_t method_B;                  /* 0 "useU_b", 1 "useMAG21", 2 "useGammaSh"    */
  int32_t method_gamma_min;          /* 0 "useU_e", 1 "useNumeric", 2 "useBeta",   */
                                     /* 3 "useGamma", 4 "useTheta"                  */
  int32_t method_gamma_c;            /* 0 "useTe", 1 "useTcomov", 2 "useConst"      */
  int32_t method_gamma_max;          /* 0 "useB", 1 "useConst"                      */
  int32_t method_nonrel;             /* 0 "none", 1 "use_gamma_min", 2 "use_Ayache", 3 "use_Sironi" */
  int32_t ele_analytic;              /* 1 if method_ele is "analytic" (no grid caps) */
} pbag_limits_opts;

/* Arguments of updateSockProperties (microphysics_base.h:575). */
typedef struct pbag_shock_state {
  double e_prime, Gamma, GammaSh, t_e, t_b, tcomov, n_prime, n_protons;
} pbag_shock_state;

/* Members after computeEleSpectrumLimits; valid = 0 when checkParams()
 * rejected the state (beta_shock < beta_min) and nothing was recomputed. */
typedef struct pbag_limits {
  double B, gamma_min, gamma_max, gamma_c, accel_frac, Theta, z_cool;
  int32_t valid, reserved;
} pbag_limits;

#define PBAG_MIN_BINS 8
#define PBAG_MAX_BINS 1024

int pbag_abi_version(void);
/* sizeof of the ABI structs, in the order grid_desc, shock_params, step_rec,
 * outputs, status, limits_opts, shock_state, limits, flux_opts, flux_query
 * (0..9); for binding checks. */
size_t pbag_sizeof(int which);
const char* pbag_status_string(int code);

/* Electron grid gam[ngam] and photon grid freq[nfreq + 1] of one grid
 * description (host pointers). freq[nfreq] is the next logspace point: the
 * value used where the reference reads one past the end of its frequency
 * vector (numeric_model.h:269-272).
 * Replaces: Electrons::allocate + build_grid_chang_cooper (base_state.h:184-253)
 * and Photons::allocate (base_state.h:270-285). */
int pbag_build_grids(const pbag_grid_desc* g, double* gam, double* freq);

/* Per-step shock scalars for n consecutive calls on ONE blastwave object.
 * state[7] carries the members that persist between calls (gamma_min,
 * gamma_max, gamma_c, accel_frac, B, Theta, z_cool); initialise it to
 * {-1, gamma_max_param, gamma_c_param (or -1), 1, -1, -1, -1} as setBasePars
 * leaves them. gam is the electron grid (its first and last points cap
 * gamma_min and gamma_max). Host pointers.
 * Replaces: updateSockProperties + computeEleSpectrumLimits
 * (microphysics_base.h:575-605, 642-652, 808-966). */
int pbag_shock_limits(const pbag_limits_opts* o, const double* gam, int ngam, int n,
                      const pbag_shock_state* in, double* state, pbag_limits* out);

/* ---- the GPU step ---------------------------------------------------------- */

typedef struct pbag_ctx pbag_ctx;  /* opaque device context */

/* Per-step shock scalars of a whole batch on the GPU, for callers that hold
 * the histories on the device (the post-processing mode, where every state of
 * a blastwave is known before its electrons are evolved): pbag_shock_limits
 * for every blastwave at once, on the electron grid of ctx. Blastwave b owns
 * the states off[b] .. off[b+1]-1 (host array of nbw+1, as for pbag_run_batch)
 * and has options d_opts[b]; row b of d_state [nbw][7] carries its members as
 * the state argument of pbag_shock_limits does (initialise it the same way; on
 * return it holds the members after the last state); d_out receives one
 * pbag_limits per state. Device pointers; synchronous. Results equal the host
 * prep's to rounding (device pow and log differ in the last bits, which can
 * move the useNumeric bisection by one of its 0.1 % steps where gammaMinFunc
 * is within rounding of zero at a midpoint). On a failure st names the
 * blastwave and step of the earliest failing state; later results of that
 * blastwave are not meaningful.
 * Replaces: updateSockProperties + computeEleSpectrumLimits
 * (microphysics_base.h:575-605, 642-652, 808-966) over whole histories. */
int pbag_shock_limits_device(pbag_ctx* ctx, int nbw, const int64_t* off, const pbag_limits_opts* d_opts,
                             const pbag_shock_state* d_in, double* d_state, pbag_limits* d_out, pbag_status* st);

/* Create a device context for one grid (one CommonTables entry of the
 * reference, microphysics/common.h:93-117) on CUDA device `device`. When
 * ssc_tables != 0 the SSC kernel K[i][j][k] (kernels.h:49-117) and its
 * integral are built on the host and uploaded once; blastwaves with ssc_on
 * need it. Replaces: the CommonTables grids and kernels and
 * ElectronAndRadiation::allocateForNumericSpectra (microphysics.h:282-345). */
int pbag_create(const pbag_grid_desc* g, int device, int ssc_tables, pbag_ctx** out);
void pbag_destroy(pbag_ctx* ctx);

/* Evolve nbw blastwaves over their whole histories and fill the requested
 * output histories. Blastwave b owns records off[b] .. off[b+1]-1 (off has
 * nbw+1 entries, off[0] = 0, non-decreasing), one per burster-time index in
 * order; its state starts as a freshly allocated ElectronAndRadiation. All
 * pointers are HOST pointers; the call copies inputs to the device, runs, and
 * copies outputs back before returning. On a physics error the rows computed
 * before the failing step are still returned and st names the first failure
 * in time order, the step at which the reference would have exited.
 * Replaces, per blastwave and step: initializeElectronDistribution
 * (microphysics.h:347), evaluateElectronDistributionNumericMixed (:359),
 * computeRadiationNumericMixed (:492) and storeDenseOutput (:602). */
int pbag_run_batch(pbag_ctx* ctx, const pbag_shock_params* prm, int nbw, const int64_t* off,
                   const pbag_step_rec* recs, const pbag_outputs* out, pbag_status* st);

/* Same as pbag_run_batch with prm, recs and every output pointer in DEVICE
 * memory of the context's device (off stays a host array). stream (a
 * cudaStream_t, may be NULL) is the caller's stream whose work produces the
 * inputs: the call waits for it before it reads them. The batch runs on the
 * context's own stream; the call returns after it has finished there. */
int pbag_run_batch_device(pbag_ctx* ctx, const pbag_shock_params* d_prm, int nbw, const int64_t* off,
                          const pbag_step_rec* d_recs, const pbag_outputs* d_out, pbag_status* st,
                          void* stream);

/* Allocation-free variant of pbag_run_batch_device. No counterpart in the
 * reference: it exists for callers that cannot allocate device memory while
 * they run the step - hosts that hand out device memory only from their own
 * pool, latency-critical loops that must not pay an allocation or the device
 * synchronisation one can cause - and keeps every intermediate buffer in one
 * fixed __device__ array of PBAG_NOALLOC_SCRATCH_BYTES inside the library
 * instead of memory the context allocates. It calls no cudaMalloc/cudaFree;
 * inputs and outputs are the caller's device buffers exactly as for
 * pbag_run_batch_device, on a context created beforehand (pbag_create
 * allocates the grid tables). It runs the same preparation, evolve and
 * radiation kernels, except that its SSC contraction is always the FP32
 * CUDA-core one (whatever pbag_set_ssc_path chose); results agree with
 * pbag_run_batch_device within the plain-path tolerance. The call is
 * synchronous: it reads the shock parameters back to validate them and
 * returns after the batch has finished.
 * Limit: the batch needs about 17 KiB per blastwave of 201 x 128 bins plus
 * 128 B per record (all rounded to 256 B blocks); a larger batch returns
 * PBAG_ERR_ARG with st->site set to the KiB it would need.
 * The first call on a device looks up the array's device address (once per
 * device). Every call shares the array and it keeps the last call's contents
 * (the call clears what must start at zero): calls that overlap on the GPU
 * race, so issue them one at a time. Every GPU that loads the library holds
 * the array until exit. */
#define PBAG_NOALLOC_SCRATCH_BYTES (16u << 20)
int pbag_run_batch_noalloc(pbag_ctx* ctx, const pbag_shock_params* d_prm, int nbw, const int64_t* off,
                           const pbag_step_rec* d_recs, const pbag_outputs* d_out, pbag_status* st);

/* Number of kernels the last run (pbag_run_batch, pbag_run_batch_device or
 * pbag_run_batch_noalloc) launched (diagnostics). */
int64_t pbag_last_launch_count(const pbag_ctx* ctx);

/* How the SSC spectrum (numeric_model.h:247-285) is contracted. AUTO uses
 * the tensor cores with split-BF16 operands (FP32 accumulation, relative
 * error ~1e-5) when nfreq is 128 or 256, and FP32 CUDA cores otherwise.
 * TC_BF16 (one BF16 product, ~1e-3) exists for precision studies only. */
enum pbag_ssc_path {
  PBAG_SSC_AUTO = 0,
  PBAG_SSC_CUDA_FP32 = 1,
  PBAG_SSC_TC_SPLIT_BF16 = 2,
  PBAG_SSC_TC_BF16 = 3,
  PBAG_SSC_SURROGATE = 4    /* learned band shapes + exact fallback (pbag_surrogate_configure) */
};
int pbag_set_ssc_path(pbag_ctx* ctx, int path);

/* Kernel classes of a step, in launch order. */
enum pbag_kernel_class {
  PBAG_K_EVOLVE = 0,        /* Chang-Cooper evolution + synchrotron/SSA emissivity */
  PBAG_K_SSC = 1,           /* batched SSC contraction                          */
  PBAG_K_FINALIZE = 2       /* photon field, totals, normalisation, histories   */
};
/* Enable (1) or disable (0) CUDA-event timing of every kernel launch on the
 * context's stream; resets the accumulated totals. pbag_get_timing returns,
 * per class, the summed device time in ms and the number of timed launches
 * since the last reset (arrays of 3). Diagnostics only. */
int pbag_set_timing(pbag_ctx* ctx, int enable);
int pbag_get_timing(const pbag_ctx* ctx, double* ms, int64_t* launches);

/* Emissivity contractions of n comoving states, without the Chang-Cooper
 * evolution (the contraction microbenchmark, and a building block for callers
 * that hold N(gamma) themselves). For state s, with the electron spectrum
 * f[s][G] on the context's gamma grid, the field B[s] and the seed photon
 * density nph[s][F] (total_rad.f of the previous step):
 *   jsyn[s][k]: computeSynSpectrum (numeric_model.h:148-184) with the kernel of
 *               SynKernel::evalSynKernel (kernels.h:528-538) at B[s];
 *   jssc[s][i]: computeSSCSpectrum(nph[s]) (numeric_model.h:247-285).
 * The synchrotron sums run in FP32 on CUDA cores; `precision` selects the SSC
 * contraction. Device pointers on the context's device, row-major [n][F] /
 * [n][G]; jsyn or jssc may be NULL (then B or nph may be too). Needs a context
 * created with ssc_tables = 1 for jssc; the tensor-core precisions need
 * nfreq = 128 or 256 (else PBAG_ERR_UNSUPPORTED). Synchronous. A negative or
 * non-finite j_syn value (the reference's exit in computeSynSpectrum) returns
 * PBAG_ERR_NONFINITE with st->bw = the first failing state. */
enum pbag_precision {
  PBAG_PREC_FP32 = 0,        /* CUDA cores, FP32 with power-of-two scaling       */
  PBAG_PREC_BF16 = 1,        /* tensor cores, BF16 operands, FP32 accumulation   */
  PBAG_PREC_SPLIT_BF16 = 2,  /* tensor cores, hi+lo BF16 (3 products), FP32 acc. */
  PBAG_PREC_TF32 = 3         /* tensor cores, TF32 operands, FP32 accumulation   */
};
int pbag_contract(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph, int syn_method,
                  int precision, double* d_jsyn, double* d_jssc, pbag_status* st);

/* ---- SSC surrogate -------------------------------------------------------
 * A multilayer perceptron with its own FP32 training and inference kernels:
 * layers dims[0] -> ... -> dims[nlayers], SiLU between layers, linear output.
 * Parameters: one FP32 array, per layer W_l [dims[l+1]][dims[l]] (row-major)
 * then b_l [dims[l+1]]. Device pointers for the data; synchronous. */
typedef struct pbag_mlp pbag_mlp;
int pbag_mlp_create(int device, const int* dims, int nlayers, pbag_mlp** out);
void pbag_mlp_destroy(pbag_mlp* net);
int64_t pbag_mlp_param_count(const pbag_mlp* net);
int pbag_mlp_set_params(pbag_mlp* net, const float* host_params);
/* host_params and/or host_grad (gradients of the last train step) may be NULL */
int pbag_mlp_get_params(const pbag_mlp* net, float* host_params, float* host_grad);
int pbag_mlp_forward(pbag_mlp* net, int n, const float* d_x, float* d_y);
/* Inference on the tensor cores: weights and activations rounded to BF16, FP32
 * accumulation, all layers in one kernel (every in-dimension a multiple of 32,
 * every out-dimension a multiple of 32 up to 256, at most 8 layers; otherwise
 * PBAG_ERR_UNSUPPORTED). The weights are laid out again after they change. */
int pbag_mlp_infer(pbag_mlp* net, int n, const float* d_x, float* d_y);
/* One step on n rows: forward, loss = sum(mask (y - t)^2) / (n dims[L]) (mask
 * may be NULL), gradients, and (update != 0) an Adam update with rate lr.
 * *loss (host, may be NULL) receives the loss. */
int pbag_mlp_train_step(pbag_mlp* net, int n, const float* d_x, const float* d_t, const float* d_mask, float lr,
                        int update, float* loss);

/* ---- EATS flux density from the histories (fluxDens) ---------------------
 * The observer-frame flux density contribution of EATS cells from a batch's
 * total_rad.j_all / a_all histories: ElectronAndRadiation::fluxDens
 * (microphysics.h:1185-1217) - frequency index (findIndex), bilinear
 * interpolation of j and a in (frequency, radius) between the history rows ia
 * and ib of the cell's blastwave - followed by computeFluxDensity
 * (microphysics.h:799-867): Doppler factor, lab-frame emissivity and
 * absorption, shell thickness (Johannesson 2006, eq. 33), optical depth along
 * the line of sight, intensity (computeIntensity, microphysics.h:11-58) and
 * luminosity. One query per cell; queries are independent. FP64. */
enum pbag_shock_vel { PBAG_VEL_SAME_AS_BW = 0, PBAG_VEL_SHOCK = 1 };             /* "method_vel"  */
enum pbag_method_ne { PBAG_NE_USE_NPRIME = 0, PBAG_NE_USE_NE = 1 };             /* "method_ne"   */
enum pbag_method_tau { PBAG_TAU_APPROX = 0, PBAG_TAU_THICK = 1, PBAG_TAU_SMOOTH = 2,
                       PBAG_TAU_SHARP = 3 };                                     /* "method_tau"  */
typedef struct pbag_flux_opts {
  int32_t shock_vel, method_ne, method_tau, pad;
} pbag_flux_opts;
/* the arguments of fluxDens, in its order (rsh and dr as fluxDens names them;
 * computeFluxDensity recomputes dr from ne, r, theta, ncells, Gamma, n_prime) */
typedef struct pbag_flux_query {
  int32_t bw;               /* blastwave of the batch                            */
  int32_t ia, ib;           /* history rows (time indices) bracketing r          */
  int32_t pad;
  double theta, ncells, freq, Gamma, GammaSh, acc_fac, mu, r, rsh, dr, n_prime, ne;
} pbag_flux_query;
/* d_j_all, d_a_all: the batch's histories [nrec][nfreq] (offsets[] as for
 * pbag_run_batch, host array of nbw+1); d_r_all: radius of every record
 * [nrec]; d_q: nq queries; d_flux: nq results. Device pointers; synchronous.
 * A query whose frequency is outside (freq[0], freq[F-1]) gives
 * PBAG_ERR_RANGE, a negative or non-finite intensity or luminosity
 * PBAG_ERR_NONFINITE, both with bw = its blastwave and step = its index. */
int pbag_flux_dens(pbag_ctx* ctx, const pbag_flux_opts* opts, int nbw, const int64_t* offsets,
                   const double* d_j_all, const double* d_a_all, const double* d_r_all, int nq,
                   const pbag_flux_query* d_q, double* d_flux, pbag_status* st);

/* ---- adaptive EATS light curve (method_eats = "adaptive") -----------------
 * The observed flux density of a jet layer at (t_obs, nu_obs), integrated
 * over the equal-arrival-time surface: EATS::evalFluxDensA (eats.h:820-850)
 * with atol 0 as evalLightCurve passes it for a fresh layer (eats.h:808-818),
 * integrate_theta_phi (eats.h:587-700): phi in [0, pi] outside, 1 - cos(theta)
 * from the layer's lower cone edge to the jet edge of that phi (find_jet_edge,
 * eats.h:103-173) inside, each by CADRE (quadratures.h:1613-2113, adaptive
 * Romberg with trapezoid error control) or TRAP_FIXED (quadratures.h:939-951);
 * the integrand (eats.h:175-232) interpolates the layer's dynamics at the
 * emission time of that direction and calls fluxDens on the layer's forward
 * and reverse shock histories (fluxDensAdaptiveWithComov,
 * blastwave_radiation.h:75-150); the counter jet (obsAngleCJ) adds a second
 * integral. Output in mJy. One query = one (layer, t_obs, nu_obs). FP64. */
enum pbag_eats_quad { PBAG_QUAD_CADRE = 0, PBAG_QUAD_TRAP_FIXED = 1 };          /* "method_quad" */
/* the dynamics a layer's EATS reads, per time index (BW::Q of blastwave_pars.h:211-229) */
enum pbag_eats_q {
  PBAG_EQ_TBURST = 0, PBAG_EQ_R, PBAG_EQ_THETA, PBAG_EQ_GAMMA, PBAG_EQ_BETA, PBAG_EQ_GAMMA_FSH,
  PBAG_EQ_THICKNESS, PBAG_EQ_M2, PBAG_EQ_RHO2, PBAG_EQ_RSH, PBAG_EQ_ACC_FRAC, PBAG_EQ_CTHETA,
  PBAG_EQ_GAMMA_RSH, PBAG_EQ_THICKNESS_RS, PBAG_EQ_M3, PBAG_EQ_RHO3, PBAG_EQ_RRSH, PBAG_EQ_ACC_FRAC_RS,
  PBAG_EQ_N
};
typedef struct pbag_eats_opts {
  double theta_obs, z, d_l;      /* observer angle [rad], redshift, luminosity distance [cm] */
  double rtol_theta, rtol_phi;   /* "rtol_theta", "rtol_phi" */
  int32_t nmax_theta, nmax_phi;  /* "nmax_theta", "nmax_phi": evaluation limits */
  int32_t method_quad;           /* pbag_eats_quad */
  int32_t counter_jet;           /* "counter_jet": 1 adds the counter jet */
  pbag_flux_opts flux;           /* method_vel / method_ne / method_tau of the layer's shocks */
} pbag_eats_opts;
typedef struct pbag_eats_layer {
  int32_t i_end_r;               /* time indices of the layer's dynamics in use (m_i_end_r) */
  int32_t bw_fs, bw_rs;          /* blastwaves whose histories are the layer's forward / reverse
                                    shock (bw_rs < 0: no reverse-shock radiation) */
  int32_t pad;
  double theta_c_l, theta_c_h;   /* the layer's cone (setEatsPars, eats.h:721-731) */
  double ncells;                 /* cells of the layer (fluxDens' ncells) */
} pbag_eats_layer;
typedef struct pbag_eats_query {
  int32_t layer, pad;
  double t_obs, nu_obs;
} pbag_eats_query;
/* nl layers; d_dyn [nl][PBAG_EQ_N][nr] (device): the dynamics of layer l at
 * d_dyn + (l * PBAG_EQ_N + q) * nr; h_layers (host) [nl]; offsets (host,
 * nbw + 1) and d_j_all / d_a_all [nrec][nfreq] (device): the histories of the
 * batch that evolved the layers' shocks (blastwave b's row i is its time
 * index i); d_q [nq], d_flux [nq] (device). Synchronous. Failures where the
 * reference exits: PBAG_ERR_RANGE (a comoving frequency outside the grid),
 * PBAG_ERR_NONFINITE (a negative or non-finite intensity, luminosity or
 * interpolated dynamics value), PBAG_ERR_EVALS (more than 1e7 integrand
 * evaluations, eats.h:536-541), PBAG_ERR_NOMEM (an integration needed more
 * intervals than the workspace holds: nmax + 8 per level), each with st->step
 * = the first failing query and st->bw = its layer. */
int pbag_eats_flux_a(pbag_ctx* ctx, const pbag_eats_opts* opts, int nl, const pbag_eats_layer* h_layers, int nr,
                     const double* d_dyn, int nbw, const int64_t* offsets, const double* d_j_all,
                     const double* d_a_all, int nq, const pbag_eats_query* d_q, double* d_flux, pbag_status* st);

/* ---- the blastwave ODE right-hand side ----------------------------------- */

/* Evolution equations of a blastwave: forward shock (BlastWave::rhs_fs,
 * blastwave/blastwave.h:1515-1768) or forward and reverse shock
 * (BlastWave::rhs_fsrs, :1771-2118), selected by BW_TYPES iFS / iFSRS. */
enum pbag_bw_type { PBAG_BW_FS = 0, PBAG_BW_FSRS = 1 };
/* The ODE state of one blastwave, SOL::QS order (blastwave_pars.h:308-310). */
enum pbag_bw_q {
  PBAG_Y_R, PBAG_Y_RSH, PBAG_Y_TT, PBAG_Y_TCOMOV, PBAG_Y_GAMMA, PBAG_Y_EINT2, PBAG_Y_EINT3, PBAG_Y_THETA,
  PBAG_Y_RRSH, PBAG_Y_ERAD2, PBAG_Y_ERAD3, PBAG_Y_ESH2, PBAG_Y_ESH3, PBAG_Y_EAD2, PBAG_Y_EAD3, PBAG_Y_M2,
  PBAG_Y_M3, PBAG_Y_DELTAR4, PBAG_Y_N
};
enum pbag_eos { PBAG_EOS_PEER12 = 0, PBAG_EOS_NAVA13 = 1 };                 /* "method_eos"    */
enum pbag_spread { PBAG_SPREAD_NULL = 0, PBAG_SPREAD_ADI = 1, PBAG_SPREAD_AA = 2,
                   PBAG_SPREAD_AFGPY = 3, PBAG_SPREAD_OUR = 4 };           /* "method_spread" */
enum pbag_limit_spread { PBAG_LIMIT_SPREAD_NONE = 0, PBAG_LIMIT_SPREAD_GAMMA0_FRAC = 1,
                         PBAG_LIMIT_SPREAD_GAMMA_VAL = 2, PBAG_LIMIT_SPREAD_RD = 3 }; /* "method_limit_spread" */
enum pbag_dmdr { PBAG_DMDR_USING_A = 0, PBAG_DMDR_USING_DTHDR = 1, PBAG_DMDR_NONE = 2 }; /* "method_dmdr" */
enum pbag_dgdr { PBAG_DGDR_OUR = 0, PBAG_DGDR_PEER = 1 };                    /* "method_dgdr"   */

/* One shock's ElectronAndRadiation as its radiative-loss term reads it
 * (computeRadiationLoss, microphysics.h:749-791; computePtot :204-219). */
typedef struct pbag_bw_mphys {
  int32_t method_B;          /* as pbag_limits_opts: 0 useU_b, 1 useMAG21, 2 useGammaSh         */
  int32_t method_gamma_max;  /* as pbag_limits_opts: 0 useB, 1 useConst                         */
  int32_t method_nonrel;     /* 0 none, 1 useGm, 2 useAyache, 3 use_Sironi (method_nonrel_dist)  */
  int32_t method_up;         /* 0 useEint2, 1 useGamma (method_Up_{fs,rs})                      */
  int32_t ele_analytic;      /* method_ele = analytic: no clamps to the electron grid            */
  int32_t pad;
  double eps_e, eps_b, eps_t, p, mu, mu_e, beta_min;
  double gam_lo, gam_hi;     /* first and last point of the electron grid                        */
} pbag_bw_mphys;

/* The constant parameters of one blastwave (BW::Pars, blastwave_pars.h:13-203,
 * and the RhoISM / LatSpread / EOSadi objects it owns). */
typedef struct pbag_bw_rhs_pars {
  int32_t type;                /* pbag_bw_type                                          */
  int32_t method_dmdr, method_dgdr, method_limit_spread, method_spread, method_eos;
  int32_t adiab_loss, adiab_loss_rs, exponential_rho4;
  int32_t ilayer, nlayers;     /* the layer and the number of layers (EjectaID2::ctheta) */
  int32_t pad;
  double Gamma0, beta0, M0, mom0, ncells, theta_a, theta_max, Rd;
  double frac_mom0_spread;     /* fraction_of_mom0_when_spread_start                    */
  double mom_spread;           /* value_of_mom_when_spread_start                        */
  double spread_aa, spread_theta_max, spread_theta_c, spread_theta_w, spread_theta_b0; /* LatSpread */
  double eps_rad_fs, eps_rad_rs; /* epsilon_e_rad_{fs,rs}; < 0: from the loss term       */
  double tprompt, rs_Gamma0_frac_no_exceed;
  double n_ism, A0, s, R_ej, R_ism;  /* RhoISM: uniform for n_ism > 0, else the step profile */
  pbag_bw_mphys fs, rs;
} pbag_bw_rhs_pars;

/* What one evaluation reads besides the constants: the state Y, the flags the
 * reference keeps in BW::Pars, and the members of the shocks'
 * ElectronAndRadiation objects that the loss term reads (tcomov) and carries
 * from call to call (gamma_max with method_gamma_max = const, accel_frac when
 * gamma_min >= 2); the evaluation updates the carried members. */
typedef struct pbag_bw_rhs_state {
  double x;                          /* burster time of the evaluation                 */
  double Y[PBAG_Y_N];
  int32_t end_spreading, shut_off;   /* BW::Pars end_spreading, shutOff                */
  int32_t first_step;                /* BW::Pars prev_idx_x == 0                       */
  int32_t pad;
  double fs_tcomov, fs_gamma_max, fs_accel_frac;
  double rs_tcomov, rs_gamma_max, rs_accel_frac;
} pbag_bw_rhs_state;

/* dY/dt of n blastwave states (one ODE right-hand side each, as the
 * reference's RHS_comb calls rhs_dispatcher per blastwave,
 * model_evolve.h:1587-1624): pars[b], state[b] (carried members updated in
 * place) -> dydt[b][PBAG_Y_N]. rhs_fs writes R, Rsh, tt, tcomov, Gamma, Eint2,
 * theta, Erad2, Esh2, Ead2, M2; rhs_fsrs also Rsh_rs, Eint3, Erad3, Esh3,
 * Ead3, M3, deltaR4; entries a function does not write are left as they are.
 * pbag_bw_rhs runs on the host, pbag_bw_rhs_device on the GPU (one thread per
 * blastwave; device pointers; synchronous). Where the reference exits: the
 * first failing blastwave in st->bw, PBAG_ERR_NONFINITE or PBAG_ERR_PARAM,
 * st->site the condition (pbag_rhs.cuh Site). */
int pbag_bw_rhs(int n, const pbag_bw_rhs_pars* pars, pbag_bw_rhs_state* state, double* dydt, pbag_status* st);
int pbag_bw_rhs_device(pbag_ctx* ctx, int n, const pbag_bw_rhs_pars* d_pars, pbag_bw_rhs_state* d_state,
                       double* d_dydt, pbag_status* st);

/* Contraction autotuner: the first tensor-core SSC contraction of a shape
 * (precision, grid, outputs, batch size to a factor of two) launched outside
 * a graph capture times the candidate kernels and shapes (slab per CTA, or
 * blastwaves on rows with 1-3 slab chunks per copy and 2-8 CTAs per SM) on
 * its own data and keeps the fastest for that shape, process-wide. On by
 * default (environment PBAG_AUTOTUNE=0: off); pbag_autotune(0/1) switches it.
 * pbag_autotune_report writes one line per tuned shape into buf (len bytes,
 * NUL-terminated) and returns the full report's length. */
int pbag_autotune(int enable);
int pbag_autotune_report(char* buf, int len);

/* The SSC surrogate of a context. Exact projections of the SSC spectrum on
 * the tensor cores (BF16): over PBAG_SUR_BANDS bands of nfreq/PBAG_SUR_BANDS
 * frequencies the band power P and the power-weighted first and second moments
 * Q, R of x = ln nu - (band centre), and the spectrum itself at
 * PBAG_SUR_CHECKS check frequencies (two per band). In each band a baseline
 * shape exp(beta x + gamma x^2) matches P, Q and R; an MLP with PBAG_SUR_IN
 * inputs and nfreq outputs (BF16 on the tensor cores) predicts the log10
 * correction to it; the spectrum is scaled to the exact band powers. Error
 * estimate per state: est_scale times the relative L2 distance between the
 * predicted and the exact spectrum at the check frequencies. States whose
 * estimate exceeds tol are recomputed exactly (split BF16).
 * pbag_surrogate_configure: net (may be NULL until trained; not owned; dims
 *   PBAG_SUR_IN -> ... -> nfreq; call again after the network changes: the
 *   BF16 weights are laid out then), feature means and standard deviations
 *   (host, PBAG_SUR_IN each, NULL: 0 and 1), est_scale (> 0), tol. Needs
 *   ssc_tables and nfreq 128/256. With a network set,
 *   pbag_set_ssc_path(ctx, PBAG_SSC_SURROGATE) makes the step use it.
 * pbag_surrogate_features: unstandardised features [n][PBAG_SUR_IN], the exact
 *   projections [n][PBAG_SUR_PROJ] (P of every band, then Q, then R, then the
 *   check frequencies, whose indices pbag_surrogate_checks gives) and the
 *   baseline log10 share of each frequency in its band's power [n][nfreq] of n
 *   states (f [n][G], B [n], nph [n][F]); any output may be NULL.
 * pbag_surrogate_contract: j_ssc [n][F] of n states through the surrogate,
 *   the scaled error estimate of each state (d_err, may be NULL) and the number
 *   of states recomputed exactly. */
#define PBAG_SUR_BANDS 16
#define PBAG_SUR_CHECKS 32
#define PBAG_SUR_PROJ (3 * PBAG_SUR_BANDS + PBAG_SUR_CHECKS)
#define PBAG_SUR_IN 128
int pbag_surrogate_configure(pbag_ctx* ctx, pbag_mlp* net, const float* mean, const float* stdv, float est_scale,
                             float tol);
/* the frequency index of each check projection (host array of PBAG_SUR_CHECKS) */
int pbag_surrogate_checks(pbag_ctx* ctx, int* idx);
int pbag_surrogate_features(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph,
                            float* d_x, double* d_proj, float* d_base, pbag_status* st);
int pbag_surrogate_contract(pbag_ctx* ctx, int n, const double* d_f, const double* d_B, const double* d_nph,
                            double* d_jssc, float* d_err, int* n_fallback, pbag_status* st);

#ifdef __cplusplus
}
#endif
#endif /* PBAG_H */
