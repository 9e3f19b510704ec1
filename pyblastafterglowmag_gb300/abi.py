"""ctypes mirror of include/pbag.h (structs, enums, status codes).

The layouts here must match the C header field for field; tests check the
sizes against the values the compiled library reports.
"""
import ctypes as C

import numpy as np

PBAG_OK = 0
PBAG_ERR_ARG = -1
PBAG_ERR_CUDA = -2
PBAG_ERR_NONFINITE = -3
PBAG_ERR_NELE = -4
PBAG_ERR_PARAM = -5
PBAG_ERR_DLNVDT = -6
PBAG_ERR_UNSUPPORTED = -7
PBAG_ERR_TIMEOUT = -8
PBAG_ERR_NOMEM = -9
PBAG_ERR_RANGE = -10
PBAG_ERR_EVALS = -11

STATUS_NAMES = {
    PBAG_OK: "ok",
    PBAG_ERR_ARG: "bad argument",
    PBAG_ERR_CUDA: "CUDA error",
    PBAG_ERR_NONFINITE: "non-finite or negative value",
    PBAG_ERR_NELE: "total electron number <= 0",
    PBAG_ERR_PARAM: "invalid shock parameters",
    PBAG_ERR_DLNVDT: "invalid dlnV/dt",
    PBAG_ERR_UNSUPPORTED: "unsupported option",
    PBAG_ERR_TIMEOUT: "device wait timed out",
    PBAG_ERR_RANGE: "frequency outside the grid",
    PBAG_ERR_NOMEM: "device allocation failed",
    PBAG_ERR_EVALS: "EATS quadrature past 1e7 integrand evaluations",
}

PBAG_SKIP, PBAG_INIT, PBAG_EVOLVE = 0, 1, 2
PBAG_SYN_CSYN, PBAG_SYN_DER09, PBAG_SYN_GSL, PBAG_SYN_BESSEL = 0, 1, 2, 3
PBAG_ELE_NUMERIC, PBAG_ELE_MIX = 1, 2
PBAG_SSC_AUTO, PBAG_SSC_CUDA_FP32, PBAG_SSC_TC_SPLIT_BF16, PBAG_SSC_TC_BF16, PBAG_SSC_SURROGATE = 0, 1, 2, 3, 4
PBAG_PREC_FP32, PBAG_PREC_BF16, PBAG_PREC_SPLIT_BF16, PBAG_PREC_TF32 = 0, 1, 2, 3
PRECISION_NAMES = {PBAG_PREC_FP32: "fp32", PBAG_PREC_BF16: "bf16", PBAG_PREC_SPLIT_BF16: "split-bf16",
                   PBAG_PREC_TF32: "tf32"}


class GridDesc(C.Structure):
    _fields_ = [("ngam", C.c_int32), ("nfreq", C.c_int32),
                ("gam1", C.c_double), ("gam2", C.c_double),
                ("freq1", C.c_double), ("freq2", C.c_double)]


class ShockParams(C.Structure):
    _fields_ = [("p", C.c_double), ("eps_e", C.c_double),
                ("max_substeps", C.c_int32), ("ele_method", C.c_int32),
                ("syn_method", C.c_int32), ("ssa_on", C.c_int32),
                ("ssc_on", C.c_int32), ("adi_on", C.c_int32),
                ("pp_on", C.c_int32), ("reserved", C.c_int32)]


SHOCK_PARAMS_DTYPE = np.dtype([("p", np.float64), ("eps_e", np.float64),
                               ("max_substeps", np.int32), ("ele_method", np.int32),
                               ("syn_method", np.int32), ("ssa_on", np.int32),
                               ("ssc_on", np.int32), ("adi_on", np.int32),
                               ("pp_on", np.int32), ("reserved", np.int32)], align=True)
assert SHOCK_PARAMS_DTYPE.itemsize == C.sizeof(ShockParams)


class LimitsOpts(C.Structure):
    _fields_ = [("p", C.c_double), ("eps_e", C.c_double), ("eps_b", C.c_double),
                ("eps_t", C.c_double), ("beta_min", C.c_double), ("mu", C.c_double),
                ("mu_e", C.c_double), ("method_B", C.c_int32),
                ("method_gamma_min", C.c_int32), ("method_gamma_c", C.c_int32),
                ("method_gamma_max", C.c_int32), ("method_nonrel", C.c_int32),
                ("ele_analytic", C.c_int32)]


SHOCK_STATE_DTYPE = np.dtype([(f, np.float64) for f in
                              ["e_prime", "Gamma", "GammaSh", "t_e", "t_b", "tcomov",
                               "n_prime", "n_protons"]])
LIMITS_DTYPE = np.dtype([(f, np.float64) for f in
                         ["B", "gamma_min", "gamma_max", "gamma_c", "accel_frac", "Theta",
                          "z_cool"]] + [("valid", np.int32), ("reserved", np.int32)])

REC_FIELDS = ["tc", "tc_p1", "m", "m_p1", "rho", "rho_p1", "dr", "dr_p1",
              "u_p", "u_p_p1", "B", "gamma_min", "gamma_max", "gamma_c",
              "accel_frac", "n_prime"]


class StepRec(C.Structure):
    _fields_ = [("mode", C.c_int32), ("reserved", C.c_int32)] + \
        [(f, C.c_double) for f in REC_FIELDS]


# numpy view of an array of StepRec
STEP_DTYPE = np.dtype([("mode", np.int32), ("reserved", np.int32)] +
                      [(f, np.float64) for f in REC_FIELDS], align=True)
assert STEP_DTYPE.itemsize == C.sizeof(StepRec)

OUTPUT_FIELDS = ["j_all", "a_all", "f_all", "i_all",
                 "ele_f_all", "gdot_syn_all", "gdot_adi_all", "gdot_ssc_all",
                 "syn_j_all", "syn_a_all", "syn_i_all", "ssc_j_all", "ssc_i_all"]
# which outputs have G (electron grid) columns rather than F
OUTPUT_ON_GAMMA = {"ele_f_all", "gdot_syn_all", "gdot_adi_all", "gdot_ssc_all"}


class Outputs(C.Structure):
    _fields_ = [(f, C.POINTER(C.c_double)) for f in OUTPUT_FIELDS]


class Status(C.Structure):
    _fields_ = [("code", C.c_int32), ("bw", C.c_int32),
                ("step", C.c_int32), ("site", C.c_int32)]


def dptr(a):
    """POINTER(c_double) for a contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_outputs(arrays):
    """Outputs struct from a dict name -> float64 array (missing -> NULL)."""
    out = Outputs()
    for f in OUTPUT_FIELDS:
        a = arrays.get(f)
        setattr(out, f, dptr(a) if a is not None else C.POINTER(C.c_double)())
    return out


# ---- EATS flux density (pbag_flux_dens) ---------------------------------------
PBAG_VEL_SAME_AS_BW, PBAG_VEL_SHOCK = 0, 1
PBAG_NE_USE_NPRIME, PBAG_NE_USE_NE = 0, 1
PBAG_TAU_APPROX, PBAG_TAU_THICK, PBAG_TAU_SMOOTH, PBAG_TAU_SHARP = 0, 1, 2, 3


class FluxOpts(C.Structure):
    _fields_ = [("shock_vel", C.c_int32), ("method_ne", C.c_int32), ("method_tau", C.c_int32),
                ("pad", C.c_int32)]


FLUX_QUERY_DTYPE = np.dtype([("bw", np.int32), ("ia", np.int32), ("ib", np.int32), ("pad", np.int32)] +
                            [(f, np.float64) for f in ("theta", "ncells", "freq", "Gamma", "GammaSh", "acc_fac",
                                                        "mu", "r", "rsh", "dr", "n_prime", "ne")])


# ---- adaptive EATS light curve (pbag_eats_flux_a) ------------------------------
PBAG_QUAD_CADRE, PBAG_QUAD_TRAP_FIXED = 0, 1
# the dynamics of a layer, in the order of enum pbag_eats_q
EATS_Q = ("tburst", "R", "theta", "Gamma", "beta", "GammaFsh", "thickness", "M2", "rho2", "Rsh", "acc_frac",
          "ctheta", "GammaRsh", "thickness_rs", "M3", "rho3", "Rrsh", "acc_frac_rs")
PBAG_EQ_N = len(EATS_Q)


class EatsOpts(C.Structure):
    _fields_ = [("theta_obs", C.c_double), ("z", C.c_double), ("d_l", C.c_double),
                ("rtol_theta", C.c_double), ("rtol_phi", C.c_double),
                ("nmax_theta", C.c_int32), ("nmax_phi", C.c_int32),
                ("method_quad", C.c_int32), ("counter_jet", C.c_int32),
                ("flux", FluxOpts)]


EATS_LAYER_DTYPE = np.dtype([("i_end_r", np.int32), ("bw_fs", np.int32), ("bw_rs", np.int32), ("pad", np.int32),
                             ("theta_c_l", np.float64), ("theta_c_h", np.float64), ("ncells", np.float64)])
EATS_QUERY_DTYPE = np.dtype([("layer", np.int32), ("pad", np.int32), ("t_obs", np.float64), ("nu_obs", np.float64)])


# ---- the blastwave ODE right-hand side (pbag_bw_rhs) ----------------------
PBAG_BW_FS, PBAG_BW_FSRS = 0, 1
BW_Q = ("R", "Rsh", "tt", "tcomov", "Gamma", "Eint2", "Eint3", "theta", "Rsh_rs", "Erad2", "Erad3", "Esh2",
        "Esh3", "Ead2", "Ead3", "M2", "M3", "deltaR4")
PBAG_Y_N = len(BW_Q)
# the entries rhs_fs / rhs_fsrs write (blastwave.h:1757-1767, 2092-2111)
BW_Q_FS = ("R", "Rsh", "tt", "tcomov", "Gamma", "Eint2", "theta", "Erad2", "Esh2", "Ead2", "M2")
BW_Q_FSRS = BW_Q
PBAG_EOS_PEER12, PBAG_EOS_NAVA13 = 0, 1
PBAG_SPREAD_NULL, PBAG_SPREAD_ADI, PBAG_SPREAD_AA, PBAG_SPREAD_AFGPY, PBAG_SPREAD_OUR = 0, 1, 2, 3, 4
BW_MPHYS_DTYPE = np.dtype([(f, np.int32) for f in ("method_B", "method_gamma_max", "method_nonrel", "method_up",
                                                  "ele_analytic", "pad")] +
                          [(f, np.float64) for f in ("eps_e", "eps_b", "eps_t", "p", "mu", "mu_e", "beta_min",
                                                     "gam_lo", "gam_hi")])
BW_RHS_PARS_DTYPE = np.dtype(
    [(f, np.int32) for f in ("type", "method_dmdr", "method_dgdr", "method_limit_spread", "method_spread",
                             "method_eos", "adiab_loss", "adiab_loss_rs", "exponential_rho4", "ilayer", "nlayers",
                             "pad")] +
    [(f, np.float64) for f in ("Gamma0", "beta0", "M0", "mom0", "ncells", "theta_a", "theta_max", "Rd",
                               "frac_mom0_spread", "mom_spread", "spread_aa", "spread_theta_max", "spread_theta_c",
                               "spread_theta_w", "spread_theta_b0", "eps_rad_fs", "eps_rad_rs", "tprompt",
                               "rs_Gamma0_frac_no_exceed", "n_ism", "A0", "s", "R_ej", "R_ism")] +
    [("fs", BW_MPHYS_DTYPE), ("rs", BW_MPHYS_DTYPE)])
BW_RHS_STATE_DTYPE = np.dtype(
    [("x", np.float64), ("Y", np.float64, (PBAG_Y_N,))] +
    [(f, np.int32) for f in ("end_spreading", "shut_off", "first_step", "pad")] +
    [(f, np.float64) for f in ("fs_tcomov", "fs_gamma_max", "fs_accel_frac", "rs_tcomov", "rs_gamma_max",
                               "rs_accel_frac")])
