"""Loader for the in-tree libpbag.so (the C-ABI library of include/pbag.h).

The library is built in place by pyblastafterglowmag_gb300.build (called by
__graft_entry__.build()). There is no fallback: if the shared object is
missing, every entry point raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpbag.so")

_lib = None


class PbagError(RuntimeError):
    def __init__(self, code, what, bw=-1, step=-1, site=0):
        self.code, self.bw, self.step, self.site = code, bw, step, site
        name = abi.STATUS_NAMES.get(code, str(code))
        where = f" (blastwave {bw}, step {step}, check {site})" if bw >= 0 else ""
        super().__init__(f"{what}: {name} [{code}]{where}")


def _check(rc, what, st=None):
    if rc != abi.PBAG_OK:
        if st is not None:
            raise PbagError(rc, what, st.bw, st.step, st.site)
        raise PbagError(rc, what)


P_I64 = C.POINTER(C.c_int64)


def load():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    lib.pbag_abi_version.restype = C.c_int
    lib.pbag_sizeof.argtypes = [C.c_int]
    lib.pbag_sizeof.restype = C.c_size_t
    lib.pbag_status_string.argtypes = [C.c_int]
    lib.pbag_status_string.restype = C.c_char_p
    lib.pbag_build_grids.argtypes = [P(abi.GridDesc), P(C.c_double), P(C.c_double)]
    lib.pbag_shock_limits.argtypes = [P(abi.LimitsOpts), P(C.c_double), C.c_int, C.c_int,
                                      C.c_void_p, P(C.c_double), C.c_void_p]
    lib.pbag_create.argtypes = [P(abi.GridDesc), C.c_int, C.c_int, P(C.c_void_p)]
    lib.pbag_destroy.argtypes = [C.c_void_p]
    lib.pbag_run_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int, P(C.c_int64), C.c_void_p,
                                   P(abi.Outputs), P(abi.Status)]
    lib.pbag_run_batch_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int, P(C.c_int64),
                                          C.c_void_p, P(abi.Outputs), P(abi.Status), C.c_void_p]
    lib.pbag_last_launch_count.argtypes = [C.c_void_p]
    lib.pbag_last_launch_count.restype = C.c_int64
    lib.pbag_set_timing.argtypes = [C.c_void_p, C.c_int]
    lib.pbag_set_ssc_path.argtypes = [C.c_void_p, C.c_int]
    lib.pbag_contract.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                  C.c_void_p, C.c_void_p, P(abi.Status)]
    lib.pbag_get_timing.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int64)]
    if lib.pbag_abi_version() != 1:
        raise RuntimeError("libpbag ABI version mismatch")
    sizes = [C.sizeof(abi.GridDesc), C.sizeof(abi.ShockParams), C.sizeof(abi.StepRec),
             C.sizeof(abi.Outputs), C.sizeof(abi.Status), C.sizeof(abi.LimitsOpts),
             abi.SHOCK_STATE_DTYPE.itemsize, abi.LIMITS_DTYPE.itemsize]
    for i, s in enumerate(sizes):
        if lib.pbag_sizeof(i) != s:
            raise RuntimeError(f"libpbag struct {i} size {lib.pbag_sizeof(i)} != binding {s}")
    _lib = lib
    return lib


def grids(grid):
    """(gam[G], freq[F+1]) for a GridDesc."""
    lib = load()
    gam = np.zeros(grid.ngam)
    freq = np.zeros(grid.nfreq + 1)
    _check(lib.pbag_build_grids(C.byref(grid), abi.dptr(gam), abi.dptr(freq)), "pbag_build_grids")
    return gam, freq


def flux_dens(ctx, opts, offsets, d_j_all, d_a_all, d_r_all, nq, d_q, d_flux):
    """pbag_flux_dens: EATS flux densities of nq queries (device addresses;
    offsets a host int64 array of nbw+1)."""
    lib = load()
    lib.pbag_flux_dens.argtypes = [C.c_void_p, C.POINTER(abi.FluxOpts), C.c_int, C.POINTER(C.c_int64),
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                   C.POINTER(abi.Status)]
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    st = abi.Status()
    _check(lib.pbag_flux_dens(ctx.handle, C.byref(opts), len(off) - 1, off.ctypes.data_as(C.POINTER(C.c_int64)),
                              C.c_void_p(d_j_all), C.c_void_p(d_a_all), C.c_void_p(d_r_all), int(nq),
                              C.c_void_p(d_q), C.c_void_p(d_flux), C.byref(st)), "pbag_flux_dens", st)


def eats_flux_a(ctx, opts, layers, d_dyn, nr, offsets, d_j_all, d_a_all, nq, d_q, d_flux):
    """pbag_eats_flux_a: the adaptive EATS flux density [mJy] of nq (layer,
    t_obs, nu_obs) queries. layers: host EATS_LAYER_DTYPE array; d_dyn
    [nlayers][PBAG_EQ_N][nr], d_j_all / d_a_all, d_q, d_flux: device
    addresses; offsets: host int64 array of nbw+1."""
    lib = load()
    lib.pbag_eats_flux_a.argtypes = [C.c_void_p, C.POINTER(abi.EatsOpts), C.c_int, C.c_void_p, C.c_int,
                                     C.c_void_p, C.c_int, C.POINTER(C.c_int64), C.c_void_p, C.c_void_p, C.c_int,
                                     C.c_void_p, C.c_void_p, C.POINTER(abi.Status)]
    layers = np.ascontiguousarray(layers, dtype=abi.EATS_LAYER_DTYPE)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    st = abi.Status()
    _check(lib.pbag_eats_flux_a(ctx.handle, C.byref(opts), len(layers), layers.ctypes.data, int(nr),
                                C.c_void_p(d_dyn), len(off) - 1, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                C.c_void_p(d_j_all), C.c_void_p(d_a_all), int(nq), C.c_void_p(d_q),
                                C.c_void_p(d_flux), C.byref(st)), "pbag_eats_flux_a", st)


def autotune(enable=True):
    """Switch the contraction autotuner (pbag_autotune) on or off."""
    lib = load()
    lib.pbag_autotune.argtypes = [C.c_int]
    _check(lib.pbag_autotune(int(bool(enable))), "pbag_autotune")


def autotune_report():
    """The tuned contraction shapes, one line each (pbag_autotune_report)."""
    lib = load()
    lib.pbag_autotune_report.argtypes = [C.c_char_p, C.c_int]
    n = lib.pbag_autotune_report(None, 0)
    buf = C.create_string_buffer(n + 1)
    lib.pbag_autotune_report(buf, n + 1)
    return buf.value.decode()


def shock_limits(opts, gam, states, state=None):
    """pbag_shock_limits over a sequence of shock states of one blastwave.

    states: SHOCK_STATE_DTYPE array; returns a LIMITS_DTYPE array. state (7
    floats, modified in place) carries the persistent members; by default it
    starts as setBasePars leaves them."""
    lib = load()
    states = np.ascontiguousarray(states, dtype=abi.SHOCK_STATE_DTYPE)
    out = np.zeros(len(states), dtype=abi.LIMITS_DTYPE)
    if state is None:
        state = np.array([-1.0, 1e7, -1.0, 1.0, -1.0, -1.0, -1.0])
    gam = np.ascontiguousarray(gam, dtype=np.float64)
    _check(lib.pbag_shock_limits(C.byref(opts), abi.dptr(gam), len(gam), len(states),
                                 states.ctypes.data, abi.dptr(state), out.ctypes.data),
           "pbag_shock_limits")
    return out


def shock_limits_device(ctx, off, d_opts, d_in, d_state, d_out):
    """pbag_shock_limits_device: the shock scalars of every state of nbw
    blastwaves on the GPU (device addresses; off a host int64 array of
    nbw+1). Returns the pbag_status."""
    lib = load()
    lib.pbag_shock_limits_device.argtypes = [C.c_void_p, C.c_int, P_I64, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.POINTER(abi.Status)]
    off = np.ascontiguousarray(off, dtype=np.int64)
    st = abi.Status()
    rc = lib.pbag_shock_limits_device(ctx.handle, len(off) - 1, off.ctypes.data_as(P_I64), C.c_void_p(d_opts),
                                      C.c_void_p(d_in), C.c_void_p(d_state), C.c_void_p(d_out), C.byref(st))
    if rc != 0:
        raise PbagError(rc, "pbag_shock_limits_device", st.bw, st.step, st.site)
    return st


def bw_rhs(pars, state, dydt=None):
    """pbag_bw_rhs on the host: dY/dt of the blastwave states (pars
    BW_RHS_PARS_DTYPE, state BW_RHS_STATE_DTYPE, one each per blastwave).
    Returns (dydt [n][PBAG_Y_N], state after the evaluation: the carried
    microphysics members updated). dydt: the values of the entries the
    blastwave's function does not write (zeros by default)."""
    lib = load()
    lib.pbag_bw_rhs.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(abi.Status)]
    pars = np.ascontiguousarray(pars, dtype=abi.BW_RHS_PARS_DTYPE)
    state = np.array(state, dtype=abi.BW_RHS_STATE_DTYPE, copy=True)
    out = np.zeros((len(pars), abi.PBAG_Y_N)) if dydt is None else np.array(dydt, dtype=np.float64, copy=True)
    st = abi.Status()
    rc = lib.pbag_bw_rhs(len(pars), pars.ctypes.data, state.ctypes.data, out.ctypes.data, C.byref(st))
    if rc != 0:
        raise PbagError(rc, "pbag_bw_rhs", st.bw, st.step, st.site)
    return out, state


def bw_rhs_device(ctx, n, d_pars, d_state, d_dydt):
    """pbag_bw_rhs_device (device addresses); returns the pbag_status."""
    lib = load()
    lib.pbag_bw_rhs_device.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(abi.Status)]
    st = abi.Status()
    rc = lib.pbag_bw_rhs_device(ctx.handle, int(n), C.c_void_p(d_pars), C.c_void_p(d_state), C.c_void_p(d_dydt),
                                C.byref(st))
    if rc != 0:
        raise PbagError(rc, "pbag_bw_rhs_device", st.bw, st.step, st.site)
    return st


class Context:
    """One device context: one grid (a CommonTables entry) on one GPU."""

    def __init__(self, grid, device=0, ssc=True):
        lib = load()
        self.grid = grid
        self._h = C.c_void_p()
        _check(lib.pbag_create(C.byref(grid), int(device), int(bool(ssc)), C.byref(self._h)),
               "pbag_create")

    def close(self):
        if self._h:
            load().pbag_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def last_launch_count(self):
        return int(load().pbag_last_launch_count(self._h))

    def contract_device(self, n, d_f, d_B, d_nph, syn_method, precision, d_jsyn, d_jssc):
        """pbag_contract on device addresses (int, or 0 for NULL): f [n][G],
        B [n], nph [n][F] in; jsyn, jssc [n][F] out."""
        st = abi.Status()
        rc = load().pbag_contract(self._h, int(n), C.c_void_p(d_f or None), C.c_void_p(d_B or None),
                                  C.c_void_p(d_nph or None), int(syn_method), int(precision),
                                  C.c_void_p(d_jsyn or None), C.c_void_p(d_jssc or None), C.byref(st))
        _check(rc, "pbag_contract", st)

    def set_ssc_path(self, path):
        """abi.PBAG_SSC_AUTO / _CUDA_FP32 / _TC_SPLIT_BF16 / _TC_BF16."""
        _check(load().pbag_set_ssc_path(self._h, int(path)), "pbag_set_ssc_path")

    def set_timing(self, enable):
        _check(load().pbag_set_timing(self._h, int(bool(enable))), "pbag_set_timing")

    def timing(self):
        """{class: (ms, launches)} for evolve, ssc, finalize since set_timing."""
        ms = (C.c_double * 3)()
        n = (C.c_int64 * 3)()
        _check(load().pbag_get_timing(self._h, ms, n), "pbag_get_timing")
        return {name: (ms[i], n[i]) for i, name in enumerate(("evolve", "ssc", "finalize"))}

    def run_device(self, d_params, nbw, offsets, d_recs, d_outputs):
        """pbag_run_batch_device: d_params / d_recs are device addresses (int),
        d_outputs a dict name -> device address; offsets a host int64 array."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        out = abi.Outputs()
        for f in abi.OUTPUT_FIELDS:
            a = d_outputs.get(f)
            setattr(out, f, C.cast(C.c_void_p(a), C.POINTER(C.c_double)) if a else C.POINTER(C.c_double)())
        st = abi.Status()
        rc = load().pbag_run_batch_device(self._h, C.c_void_p(d_params), int(nbw),
                                          offsets.ctypes.data_as(C.POINTER(C.c_int64)),
                                          C.c_void_p(d_recs), C.byref(out), C.byref(st), None)
        _check(rc, "pbag_run_batch_device", st)

    def run(self, recs, offsets, params, outputs=("j_all", "a_all", "f_all", "i_all")):
        """pbag_run_batch with host buffers; returns dict name -> array."""
        lib = load()
        recs = np.ascontiguousarray(recs, dtype=abi.STEP_DTYPE)
        params = np.ascontiguousarray(params, dtype=abi.SHOCK_PARAMS_DTYPE)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        nrec = int(offsets[-1])
        arrays = {}
        for f in outputs:
            n = self.grid.ngam if f in abi.OUTPUT_ON_GAMMA else self.grid.nfreq
            arrays[f] = np.zeros((nrec, n))
        out = abi.make_outputs(arrays)
        st = abi.Status()
        rc = lib.pbag_run_batch(self._h, params.ctypes.data, len(params),
                                offsets.ctypes.data_as(C.POINTER(C.c_int64)), recs.ctypes.data,
                                C.byref(out), C.byref(st))
        _check(rc, "pbag_run_batch", st)
        return arrays
