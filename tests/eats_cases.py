"""Seeded cases of the adaptive EATS light curve shared by the CPU and GPU
tests: a jet's step records and layer dynamics (the thin-shell model of
histories.py), the oracle's comoving histories of those records, the EATS
options and the (layer, t_obs, nu_obs) queries."""
import os

import numpy as np

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300 import histories as H

NTH = os.cpu_count() or 1

# name: (structure, layers, theta_obs, quadrature, counter jet, frequencies)
CASES = {
    "tophat_on_axis": ("tophat", 1, 0.0, abi.PBAG_QUAD_CADRE, 1, (1e15,)),
    "tophat_off_axis": ("tophat", 1, 0.3, abi.PBAG_QUAD_CADRE, 1, (1e15, 2.4e17)),
    "gaussian_fsrs": ("gaussian", 3, 0.36, abi.PBAG_QUAD_CADRE, 1, (1e15, 2.4e17)),
    "gaussian_trap_no_cj": ("gaussian", 3, 0.05, abi.PBAG_QUAD_TRAP_FIXED, 0, (1e15,)),
}
T_OBS = np.logspace(np.log10(3e3), np.log10(1e9), 12)


def config(name):
    struct, nl, *_ = CASES[name]
    if struct == "tophat":
        cfg = H.config_tophat_fs()
    else:
        cfg = H.config_gaussian_ssc()
        cfg.nlayers = nl
    return cfg


def opts(name):
    _, _, th, quad, cj, _ = CASES[name]
    o = abi.EatsOpts()
    o.theta_obs, o.z, o.d_l = th, 0.0, 3.09e26
    o.rtol_theta = o.rtol_phi = 1e-6
    o.nmax_theta = o.nmax_phi = 1000 if quad == abi.PBAG_QUAD_CADRE else 64
    o.method_quad = quad
    o.counter_jet = cj
    o.flux.shock_vel, o.flux.method_ne, o.flux.method_tau = abi.PBAG_VEL_SHOCK, abi.PBAG_NE_USE_NE, abi.PBAG_TAU_APPROX
    return o


def queries(name, nlayers):
    freqs = CASES[name][5]
    q = np.zeros(nlayers * len(T_OBS) * len(freqs), dtype=abi.EATS_QUERY_DTYPE)
    k = 0
    for l in range(nlayers):
        for t in T_OBS:
            for nu in freqs:
                q[k] = (l, 0, t, nu)
                k += 1
    return q


def inputs(name, tables, oracle):
    """(grid, opts, layers, dyn, offsets, recs, prm, j_all, a_all, queries):
    tables builds the records (the library or the oracle), the oracle evolves
    them."""
    cfg = config(name)
    recs, off, prm, grid = H.make_batch(tables, cfg)
    rc, where, h = oracle.run(grid, recs, off, prm, outputs=("j_all", "a_all"), outer_threads=NTH)
    assert rc == 0, (rc, where)
    layers, dyn = H.eats_inputs(cfg, recs, off)
    return grid, opts(name), layers, dyn, off, recs, prm, h["j_all"], h["a_all"], queries(name, len(layers))
