"""ctypes wrappers for the oracle libraries (test infrastructure only).

* ``Oracle`` wraps oracle/_build/libpbag_oracle.so, the FP64 restatement of
  the reference's comoving-radiation step (built on any machine by
  ``make -C oracle port``).
* ``Reference`` wraps oracle/_ref/libpbaref.so, the reference's own
  src/microphysics headers compiled in place (``make -C oracle ref``; only
  where the reference sources exist).
* ``ReferenceEats`` wraps oracle/_ref/libpbaref_eats.so, the reference's EATS
  integrator compiled in place with its blastwave headers (same target).

Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from pyblastafterglowmag_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libpbag_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpbaref.so")
REF_EATS_SO = os.path.join(HERE, "_ref", "libpbaref_eats.so")
REF_RUN_SO = os.path.join(HERE, "_ref", "libpbaref_run.so")
# the reference project's src/ directory: PBAG_REF_SRC, else a checkout named
# "reference" next to this repository
REF_SRC = os.environ.get("PBAG_REF_SRC") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "src")

ORC_HOIST_HEATING = 1
ORC_INNER_OMP = 2


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def build_reference():
    """Build oracle/_ref/libpbaref.so when the reference sources are present."""
    if not os.path.isdir(os.path.join(REF_SRC, "microphysics")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={REF_SRC}"], check=True)
    return True


def _alloc_outputs(grid, nrec, outputs):
    arrays = {}
    for f in outputs:
        n = grid.ngam if f in abi.OUTPUT_ON_GAMMA else grid.nfreq
        arrays[f] = np.zeros((nrec, n))
    return arrays


class Oracle:
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        lib = C.CDLL(path)
        P = C.POINTER
        lib.orc_build_grids.argtypes = [P(abi.GridDesc), P(C.c_double), P(C.c_double)]
        lib.orc_syn_func.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
        lib.orc_syn_func.restype = C.c_double
        lib.orc_ssc_func.argtypes = [C.c_double, C.c_double, C.c_double]
        lib.orc_ssc_func.restype = C.c_double
        lib.orc_ssc_kernel.argtypes = [P(C.c_double), C.c_int, P(C.c_double), C.c_int,
                                       P(C.c_double), P(C.c_double)]
        lib.orc_run.argtypes = [P(abi.GridDesc), C.c_void_p, C.c_int, P(C.c_int64), C.c_void_p,
                                P(abi.Outputs), C.c_int, C.c_int, C.c_int, P(abi.Status)]
        lib.orc_contract.argtypes = [P(abi.GridDesc), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                     C.c_void_p, C.c_void_p, C.c_int]
        lib.orc_flux_dens.argtypes = [P(abi.GridDesc), P(abi.FluxOpts), P(C.c_int64), P(C.c_double), P(C.c_double),
                                      P(C.c_double), C.c_int, C.c_void_p, P(C.c_double), P(C.c_int)]
        lib.orc_shock_limits.argtypes = [P(abi.LimitsOpts), P(C.c_double), C.c_int, C.c_int, C.c_void_p,
                                         P(C.c_double), C.c_void_p]
        lib.orc_eats_flux.argtypes = [P(abi.GridDesc), P(abi.EatsOpts), C.c_int, C.c_void_p, C.c_int,
                                      P(C.c_double), P(C.c_int64), P(C.c_double), P(C.c_double), C.c_int,
                                      C.c_void_p, P(C.c_double), P(C.c_int)]
        self.lib = lib

    def eats_flux(self, grid, opts, layers, dyn, offsets, j_all, a_all, queries):
        """orc_eats_flux: (status, failing query, flux[nq] in mJy)."""
        layers = np.ascontiguousarray(layers, dtype=abi.EATS_LAYER_DTYPE)
        dyn = np.ascontiguousarray(dyn, dtype=np.float64)
        q = np.ascontiguousarray(queries, dtype=abi.EATS_QUERY_DTYPE)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        flux = np.zeros(len(q))
        fail = C.c_int(-1)
        rc = self.lib.orc_eats_flux(C.byref(grid), C.byref(opts), len(layers), layers.ctypes.data, dyn.shape[-1],
                                    abi.dptr(dyn), off.ctypes.data_as(C.POINTER(C.c_int64)),
                                    abi.dptr(np.ascontiguousarray(j_all)), abi.dptr(np.ascontiguousarray(a_all)),
                                    len(q), q.ctypes.data, abi.dptr(flux), C.byref(fail))
        return rc, fail.value, flux

    def shock_limits(self, opts, gam, states, state=None):
        """orc_shock_limits over a sequence of shock states of one blastwave
        (the same arguments and results as the library's shock_limits), so that
        histories.make_batch(Oracle(), cfg) builds step records without the
        product library."""
        states = np.ascontiguousarray(states, dtype=abi.SHOCK_STATE_DTYPE)
        out = np.zeros(len(states), dtype=abi.LIMITS_DTYPE)
        if state is None:
            state = np.array([-1.0, 1e7, -1.0, 1.0, -1.0, -1.0, -1.0])
        gam = np.ascontiguousarray(gam, dtype=np.float64)
        rc = self.lib.orc_shock_limits(C.byref(opts), abi.dptr(gam), len(gam), len(states), states.ctypes.data,
                                       abi.dptr(state), out.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"orc_shock_limits failed: {rc}")
        return out

    def grids(self, grid):
        gam = np.zeros(grid.ngam)
        freq = np.zeros(grid.nfreq + 1)
        self.lib.orc_build_grids(C.byref(grid), abi.dptr(gam), abi.dptr(freq))
        return gam, freq

    def syn_kernel(self, method, B, gam, freq):
        out = np.zeros((len(freq), len(gam)))
        for k, nu in enumerate(freq):
            for j, g in enumerate(gam):
                out[k, j] = self.lib.orc_syn_func(method, B, nu, g)
        return out

    def ssc_kernel(self, gam, freq_ext, full=True):
        """K[F][G][F] (or None) and Kint[G][F]; freq_ext has F+1 points."""
        G, F = len(gam), len(freq_ext) - 1
        K = np.zeros((F, G, F)) if full else None
        Kint = np.zeros((G, F))
        self.lib.orc_ssc_kernel(abi.dptr(np.ascontiguousarray(gam)), G,
                                abi.dptr(np.ascontiguousarray(freq_ext)), F,
                                abi.dptr(K) if full else None, abi.dptr(Kint))
        return K, Kint

    def contract(self, grid, f, B=None, nph=None, syn_method=abi.PBAG_SYN_CSYN, syn=True, ssc=True, threads=1):
        """FP64 j_syn and j_ssc [n][F] of n states (orc_contract)."""
        f = np.ascontiguousarray(f, dtype=np.float64)
        n = f.shape[0]
        jsyn = np.zeros((n, grid.nfreq)) if syn else None
        jssc = np.zeros((n, grid.nfreq)) if ssc else None
        Bv = np.ascontiguousarray(B, dtype=np.float64) if B is not None else None
        nv = np.ascontiguousarray(nph, dtype=np.float64) if nph is not None else None
        rc = self.lib.orc_contract(C.byref(grid), n, f.ctypes.data,
                                   Bv.ctypes.data if Bv is not None else None,
                                   nv.ctypes.data if nv is not None else None, int(syn_method),
                                   jsyn.ctypes.data if syn else None, jssc.ctypes.data if ssc else None,
                                   int(threads))
        if rc != 0:
            raise RuntimeError(f"orc_contract failed: {rc}")
        return jsyn, jssc

    def run(self, grid, recs, offsets, params, outputs=("j_all", "a_all", "f_all", "i_all"),
            flags=ORC_HOIST_HEATING, outer_threads=1, inner_threads=1):
        recs = np.ascontiguousarray(recs, dtype=abi.STEP_DTYPE)
        params = np.ascontiguousarray(params, dtype=abi.SHOCK_PARAMS_DTYPE)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        arrays = _alloc_outputs(grid, int(offsets[-1]), outputs)
        out = abi.make_outputs(arrays)
        st = abi.Status()
        rc = self.lib.orc_run(C.byref(grid), params.ctypes.data, len(params),
                              offsets.ctypes.data_as(C.POINTER(C.c_int64)), recs.ctypes.data,
                              C.byref(out), flags, outer_threads, inner_threads, C.byref(st))
        return rc, (st.bw, st.step), arrays


    def flux_dens(self, grid, opts, offsets, j_all, a_all, r_all, queries):
        """orc_flux_dens: (status, failing query index, flux[nq])."""
        q = np.ascontiguousarray(queries, dtype=abi.FLUX_QUERY_DTYPE)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        flux = np.zeros(len(q))
        fail = C.c_int(-1)
        rc = self.lib.orc_flux_dens(C.byref(grid), C.byref(opts), off.ctypes.data_as(C.POINTER(C.c_int64)),
                                    abi.dptr(np.ascontiguousarray(j_all)), abi.dptr(np.ascontiguousarray(a_all)),
                                    abi.dptr(np.ascontiguousarray(r_all)), len(q), q.ctypes.data,
                                    abi.dptr(flux), C.byref(fail))
        return rc, fail.value, flux


class Reference:
    def __init__(self, path=REF_SO):
        if not os.path.exists(path) and not build_reference():
            raise FileNotFoundError("reference sources not available")
        lib = C.CDLL(path)
        P = C.POINTER
        lib.ref_grids.argtypes = [P(abi.GridDesc), P(C.c_double), P(C.c_double), P(C.c_double)]
        lib.ref_syn_kernel.argtypes = [C.c_int, C.c_double, P(C.c_double), C.c_int, P(C.c_double),
                                       C.c_int, P(C.c_double)]
        lib.ref_ssc_kernel.argtypes = [P(C.c_double), C.c_int, P(C.c_double), C.c_int, P(C.c_double),
                                       P(C.c_double)]
        lib.ref_ele_limits.argtypes = [P(abi.GridDesc)] + [C.c_double] * 4 + [C.c_int] * 5 + \
            [C.c_double, C.c_double, C.c_int, P(C.c_double), P(C.c_double)]
        lib.ref_run.argtypes = [P(abi.GridDesc), C.c_void_p, C.c_int, P(C.c_int64), C.c_void_p,
                                P(abi.Outputs)]
        lib.ref_flux_dens.argtypes = [P(abi.GridDesc), P(abi.FluxOpts), C.c_int, P(C.c_double), P(C.c_double),
                                      P(C.c_double), C.c_int, C.c_void_p, P(C.c_double)]
        self.lib = lib

    def grids(self, grid):
        gam = np.zeros(grid.ngam)
        freq = np.zeros(grid.nfreq)
        extra = C.c_double()
        self.lib.ref_grids(C.byref(grid), abi.dptr(gam), abi.dptr(freq), C.byref(extra))
        return gam, np.concatenate([freq, [extra.value]])

    def syn_kernel(self, method, B, gam, freq):
        gam = np.ascontiguousarray(gam)
        freq = np.ascontiguousarray(freq)
        out = np.zeros((len(freq), len(gam)))
        self.lib.ref_syn_kernel(method, B, abi.dptr(gam), len(gam), abi.dptr(freq), len(freq),
                                abi.dptr(out))
        return out

    def ssc_kernel(self, gam, freq, full=True):
        gam = np.ascontiguousarray(gam)
        freq = np.ascontiguousarray(freq)
        G, F = len(gam), len(freq)
        K = np.zeros((F, G, F)) if full else None
        Kint = np.zeros((G, F))
        self.lib.ref_ssc_kernel(abi.dptr(gam), G, abi.dptr(freq), F,
                                abi.dptr(K) if full else None, abi.dptr(Kint))
        return K, Kint

    def ele_limits(self, grid, opts, states, gamma_max_const=1e7, gamma_c_const=1e5):
        """ref_ele_limits with a LimitsOpts; returns [n][8] (B, gm, gM, gc,
        accel, Theta, z_cool, valid)."""
        states = np.ascontiguousarray(states, dtype=abi.SHOCK_STATE_DTYPE)
        inp = states.view(np.float64).reshape(len(states), 8).copy()
        out = np.zeros((len(states), 8))
        self.lib.ref_ele_limits(C.byref(grid), opts.p, opts.eps_e, opts.eps_b, opts.eps_t,
                                opts.method_gamma_min, opts.method_gamma_c, opts.method_gamma_max,
                                opts.method_B, opts.method_nonrel, gamma_max_const, gamma_c_const,
                                len(states), abi.dptr(inp), abi.dptr(out))
        return out

    def contract(self, grid, f, B=None, nph=None, syn_method=abi.PBAG_SYN_CSYN, syn=True, ssc=True, threads=1):
        """FP64 j_syn and j_ssc [n][F] of n states (orc_contract)."""
        f = np.ascontiguousarray(f, dtype=np.float64)
        n = f.shape[0]
        jsyn = np.zeros((n, grid.nfreq)) if syn else None
        jssc = np.zeros((n, grid.nfreq)) if ssc else None
        Bv = np.ascontiguousarray(B, dtype=np.float64) if B is not None else None
        nv = np.ascontiguousarray(nph, dtype=np.float64) if nph is not None else None
        rc = self.lib.orc_contract(C.byref(grid), n, f.ctypes.data,
                                   Bv.ctypes.data if Bv is not None else None,
                                   nv.ctypes.data if nv is not None else None, int(syn_method),
                                   jsyn.ctypes.data if syn else None, jssc.ctypes.data if ssc else None,
                                   int(threads))
        if rc != 0:
            raise RuntimeError(f"orc_contract failed: {rc}")
        return jsyn, jssc

    def flux_dens(self, grid, opts, j_all, a_all, r_arr, queries):
        """ElectronAndRadiation::fluxDens itself on queries of one blastwave
        (histories [nr][F], radii [nr]); only queries the reference does not
        exit on."""
        q = np.ascontiguousarray(queries, dtype=abi.FLUX_QUERY_DTYPE)
        flux = np.zeros(len(q))
        j = np.ascontiguousarray(j_all, dtype=np.float64)
        a = np.ascontiguousarray(a_all, dtype=np.float64)
        r = np.ascontiguousarray(r_arr, dtype=np.float64)
        self.lib.ref_flux_dens(C.byref(grid), C.byref(opts), len(r), abi.dptr(j), abi.dptr(a), abi.dptr(r), len(q),
                               q.ctypes.data, abi.dptr(flux))
        return flux

    def run(self, grid, recs, offsets, params, outputs=("j_all", "a_all", "f_all", "i_all")):
        recs = np.ascontiguousarray(recs, dtype=abi.STEP_DTYPE)
        params = np.ascontiguousarray(params, dtype=abi.SHOCK_PARAMS_DTYPE)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        arrays = _alloc_outputs(grid, int(offsets[-1]), outputs)
        out = abi.make_outputs(arrays)
        self.lib.ref_run(C.byref(grid), params.ctypes.data, len(params),
                         offsets.ctypes.data_as(C.POINTER(C.c_int64)), recs.ctypes.data,
                         C.byref(out))
        return arrays


class ReferenceEats:
    """The reference's EATS::evalFluxDensA on one layer at a time."""

    def __init__(self, path=REF_EATS_SO):
        if not os.path.exists(path) and not build_reference():
            raise FileNotFoundError("reference sources not available")
        lib = C.CDLL(path)
        P = C.POINTER
        lib.ref_eats_flux.argtypes = [P(abi.GridDesc), P(abi.EatsOpts), C.c_void_p, C.c_int, P(C.c_double),
                                      P(C.c_double), P(C.c_double), P(C.c_double), P(C.c_double), C.c_int,
                                      P(C.c_double), P(C.c_double), P(C.c_double)]
        self.lib = lib

    def eats_flux(self, grid, opts, layers, dyn, offsets, j_all, a_all, queries):
        """flux[nq] in mJy, layer by layer (the same inputs as Oracle.eats_flux)."""
        q = np.ascontiguousarray(queries, dtype=abi.EATS_QUERY_DTYPE)
        flux = np.zeros(len(q))
        nr = dyn.shape[-1]
        for l in np.unique(q["layer"]):
            L = np.ascontiguousarray(layers[l:l + 1], dtype=abi.EATS_LAYER_DTYPE)
            sel = np.flatnonzero(q["layer"] == l)
            rows = lambda b: (offsets[b], offsets[b] + nr)
            bf, br = int(L["bw_fs"][0]), int(L["bw_rs"][0])
            jf = np.ascontiguousarray(j_all[slice(*rows(bf))])
            af = np.ascontiguousarray(a_all[slice(*rows(bf))])
            jr = np.ascontiguousarray(j_all[slice(*rows(br))]) if br >= 0 else None
            ar = np.ascontiguousarray(a_all[slice(*rows(br))]) if br >= 0 else None
            t = np.ascontiguousarray(q["t_obs"][sel])
            nu = np.ascontiguousarray(q["nu_obs"][sel])
            out = np.zeros(len(sel))
            self.lib.ref_eats_flux(C.byref(grid), C.byref(opts), L.ctypes.data, nr,
                                   abi.dptr(np.ascontiguousarray(dyn[l])), abi.dptr(jf), abi.dptr(af),
                                   abi.dptr(jr), abi.dptr(ar), len(sel), abi.dptr(t), abi.dptr(nu), abi.dptr(out))
            flux[sel] = out
        return flux
