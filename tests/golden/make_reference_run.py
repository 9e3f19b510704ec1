"""Run the REFERENCE's own program and record what its blastwave driver feeds
to the comoving-radiation step and what the step returns.

Runs here, where the reference sources are present. oracle/Makefile compiles
the reference's src/main.cpp in place (oracle/ref_run.cpp, with the HDF5
stand-in of oracle/shim keeping its inputs and outputs in memory). This
script builds the run's parfile and its jet initial data with the
reference's own Python front end (PyBlastAfterglowMag.parfile_tools and
.id_analytic, imported from the reference sources; h5py and matplotlib, which
those modules import but these functions do not use, are replaced by empty
modules), runs the program in a child process and stores, per case:

  * the options of the run (grids, microphysics parameters);
  * every layer's dynamics as its ODE driver saved them (saveEjectaBWsDynamics):
    the histories the driver passes to ElectronAndRadiation at every burster
    time (blastwave_radiation.h:976-1198);
  * the comoving spectra its step produced (computeSaveEjectaSpectrum:
    total_j / total_a of the forward and reverse shocks), all rows for the
    top-hat, every 10th time index of the first layers' shocks for the jet;
  * its light curve (computeSaveEjectaLightCurve, adaptive EATS: CADRE,
    counter jet, rtol 1e-6, nmax 1000 - the parfile defaults) per layer;
  * sampled evaluations of its ODE right-hand side (rhs_fs / rhs_fsrs through
    the integrator's RHS_comb): every layer's inputs - state, parameters,
    flags, the microphysics members its radiative-loss term reads - and
    outputs, in the layout of pbag_bw_rhs, at calls spread over the run.

    python tests/golden/make_reference_run.py [tophat|gaussian ...]
"""
import copy
import ctypes as C
import importlib
import os
import struct
import sys
import tempfile
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402
from pyblastafterglowmag_gb300 import abi  # noqa: E402

# dynamics quantities kept (BW::VARNAMES of blastwave_pars.h)
DYN = ("tburst", "tt", "tcomov", "R", "Rsh", "Gamma", "beta", "GammaFsh", "U_p", "rho2", "M2", "thickness",
       "theta", "ctheta", "accel_frac", "B", "gamma_min", "gamma_max", "nprime",
       "GammaRsh", "U_p3", "rho3", "M3", "thichness_rs", "Rsh_rs", "accel_frac_rs")


def reference_tools():
    """The reference's Python front end modules that write parfiles and jet
    initial data."""
    if "h5py" not in sys.modules:
        h5 = types.ModuleType("h5py")
        h5.File = object
        sys.modules["h5py"] = h5
    for m in ("matplotlib", "matplotlib.pyplot"):
        sys.modules.setdefault(m, types.ModuleType(m))
    pkg = types.ModuleType("PyBlastAfterglowMag")
    pkg.__path__ = [os.path.join(pyoracle.REF_SRC, os.pardir, "package", "src", "PyBlastAfterglowMag")]
    sys.modules.setdefault("PyBlastAfterglowMag", pkg)
    return (importlib.import_module("PyBlastAfterglowMag.parfile_tools"),
            importlib.import_module("PyBlastAfterglowMag.id_analytic"))


RHS_EVERY = 97  # the harness samples every 97th right-hand-side call

CASES = {
    # one top-hat layer, forward shock, synchrotron only (151 gamma, 96 nu)
    "tophat": dict(
        main=dict(d_l=3.09e26, z=0.0, n_ism=1e-2, theta_obs=0.0, rtol=5e-7, lc_freqs="array 1e15",
                  lc_times="array logspace 3e3 1e10 32", tb0=3e2, tb1=1e14, ntb=1000),
        struct=dict(struct="tophat", Eiso_c=1e52, Gamma0c=300., M0c=-1., theta_c=0.1, theta_w=0.1),
        grb=dict(eps_e_fs=0.1, eps_b_fs=1e-3, p_fs=2.2, gam1_fs=1., gam2_fs=1e8, ngam_fs=151, freq1_fs=1e8,
                 freq2_fs=1e29, nfreq_fs=96, method_ele_fs="numeric", method_synchrotron_fs="CSYN"),
        keep_layers=1, every=1, rhs_calls=600),
    # the 21-layer Gaussian jet, forward and reverse shocks, synchrotron + SSC + SSA (201 gamma, 128 nu)
    "gaussian": dict(
        main=dict(d_l=3.09e26, z=0.0, n_ism=10 ** -1.6, theta_obs=np.deg2rad(20.8), rtol=5e-7,
                  lc_freqs="array 1e15", lc_times="array logspace 3e3 1e10 16", tb0=3e2, tb1=1e14, ntb=1000),
        struct=dict(struct="gaussian", Eiso_c=10 ** 54.1, Gamma0c=300., M0c=-1., theta_c=np.deg2rad(3.5),
                    theta_w=np.deg2rad(25.), n_layers_a=21),
        grb=dict(eps_e_fs=10 ** -3.42, eps_b_fs=10 ** -4.02, p_fs=2.1, eps_e_rs=10 ** -3.42, eps_b_rs=10 ** -4.02,
                 p_rs=2.1, gam1_fs=1., gam2_fs=1e9, ngam_fs=201, freq1_fs=1e8, freq2_fs=1e29, nfreq_fs=128,
                 gam1_rs=1., gam2_rs=1e9, ngam_rs=201, freq1_rs=1e8, freq2_rs=1e29, nfreq_rs=128,
                 do_rs="yes", bw_type="fsrs", do_rs_radiation="yes",
                 method_ele_fs="numeric", method_synchrotron_fs="CSYN", method_ssc_fs="numeric", use_ssa_fs="yes",
                 method_ele_rs="numeric", method_synchrotron_rs="CSYN", method_ssc_rs="numeric", use_ssa_rs="yes"),
        keep_layers=6, every=10, rhs_calls=100),
}


# one sampled evaluation of a blastwave's ODE right-hand side (oracle/ref_run.cpp)
RHS_SAMPLE_DTYPE = np.dtype([("call", np.int32), ("layer", np.int32), ("pars", abi.BW_RHS_PARS_DTYPE),
                             ("before", abi.BW_RHS_STATE_DTYPE), ("after", abi.BW_RHS_STATE_DTYPE),
                             ("dydt", np.float64, (abi.PBAG_Y_N,))], align=True)


def read_store(path):
    """What the program wrote, from the harness's write-through log
    (oracle/shim/H5Cpp.h): datasets {key: array}, attributes {key: value} and
    the sampled right-hand-side evaluations (RHS_SAMPLE_DTYPE)."""
    d, a, rhs = {}, {}, []
    with open(path, "rb") as f:
        buf = f.read()
    i = 0

    def take(n):
        nonlocal i
        b = buf[i:i + n]
        i += n
        return b

    while i < len(buf):
        tag = take(1)
        if tag == b"R":
            (sz,) = struct.unpack("<Q", take(8))
            assert sz == RHS_SAMPLE_DTYPE.itemsize, (sz, RHS_SAMPLE_DTYPE.itemsize)
            rhs.append(take(sz))
            continue
        (kl,) = struct.unpack("<I", take(4))
        k = take(kl).decode()
        if tag == b"A":
            a[k] = struct.unpack("<d", take(8))[0]
        elif tag == b"D":
            (r,) = struct.unpack("<I", take(4))
            dims = struct.unpack("<%dQ" % r, take(8 * r))
            (n,) = struct.unpack("<Q", take(8))
            v = np.frombuffer(take(8 * n), dtype=np.float64).copy()
            d[k] = v.reshape(dims) if r > 1 else v
        else:
            raise ValueError(f"bad record tag {tag!r} at {i - 1}")
    rhs = np.frombuffer(b"".join(rhs), dtype=RHS_SAMPLE_DTYPE).copy()
    return d, a, rhs


def run_case(name):
    pft, ida = reference_tools()
    case = CASES[name]
    lib = C.CDLL(pyoracle.REF_RUN_SO)
    lib.ref_h5_put.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_int]
    lib.ref_h5_put_attr.argtypes = [C.c_char_p, C.c_char_p, C.c_double]
    lib.ref_run.argtypes = [C.c_char_p] * 4
    lib.ref_rhs_record.argtypes = [C.c_long, C.c_long]
    lib.ref_rhs_record.restype = C.c_int
    assert lib.ref_rhs_record(RHS_EVERY, 200000) == 0
    wd = tempfile.mkdtemp() + "/"
    # the jet's initial data as the front end writes id_a.h5 (the adaptive EATS discretisation)
    st = copy.deepcopy(case["struct"])
    js = ida.JetStruct(n_layers_pw=81, n_layers_a=st.pop("n_layers_a", 1))
    idd, idp = js.get_1D_id(pars=st, type="adaptive")
    fid = (wd + "id_a.h5").encode()
    nl = len(np.atleast_1d(idd["mom"]))
    for k in ("entr", "press", "eps", "temp"):  # read by the loader; zero for a jet
        idd.setdefault(k, np.zeros(nl))
    for k, v in idd.items():
        a = np.ascontiguousarray(np.atleast_1d(v), dtype=np.float64)
        dims = np.array([len(a)], dtype=np.uint64)
        lib.ref_h5_put(fid, k.encode(), a.ctypes.data, dims.ctypes.data, 1)
    for k, v in idp.items():
        if isinstance(v, (int, float, np.floating)):
            lib.ref_h5_put_attr(fid, k.encode(), float(v))
    open(wd + "id_a.h5", "w").close()
    grb = dict(case["grb"], fname_ejecta_id="id_a.h5", method_eats="adaptive", ebl_tbl_fpath="none",
               save_dynamics="yes", save_spec="yes", do_lc="yes", do_skymap="no")
    pft.create_parfile(working_dir=wd, P={"main": dict(case["main"]), "grb": grb})
    t = time.time()
    rc = lib.ref_run(wd.encode(), b"parfile.par", b"err", (wd + "store.bin").encode())
    print(f"{name}: reference program exit {rc} after {time.time() - t:.1f} s")
    d, attrs, rhs = read_store(wd + "store.bin")
    out = {"grid": np.array([case["grb"]["ngam_fs"], case["grb"]["nfreq_fs"], case["grb"]["gam1_fs"],
                             case["grb"]["gam2_fs"], case["grb"]["freq1_fs"], case["grb"]["freq2_fs"]]),
           "layers": np.array(nl)}
    for k in ("eps_e_fs", "eps_b_fs", "p_fs", "eps_e_rs", "eps_b_rs", "p_rs", "n_ism", "theta_obs", "d_l", "z"):
        src = case["main"] if k in case["main"] else case["grb"]
        if k in src:
            out["par_" + k] = np.array(float(src[k]))
    out["id_theta_wing"] = np.array(float(idp["theta_wing"]))  # the layers' angular extent (_init_a_grid)
    out["opt_rs"] = np.array(int(case["grb"].get("do_rs", "no") == "yes"))
    out["opt_ssc"] = np.array(int(case["grb"].get("method_ssc_fs", "none") == "numeric"))
    out["opt_ssa"] = np.array(int(case["grb"].get("use_ssa_fs", "no") == "yes"))
    for il in range(nl):
        g = f"{wd}dyn.h5//shell=0 layer={il}/"
        for q in DYN:
            if g + q in d:
                out[f"dyn{il}_{q}"] = d[g + q]
    every, keep = case["every"], case["keep_layers"]
    for il in range(min(nl, keep)):
        g = f"{wd}spec.h5//shell=0 layer={il}/"
        for q in ("total_j_fs", "total_a_fs", "total_j_rs", "total_a_rs"):
            if g + q in d:
                F = case["grb"]["nfreq_fs"]
                out[f"spec{il}_{q}"] = d[g + q].reshape(-1, F)[::every]
    out["spec_every"] = np.array(every)
    out["lc_times"] = d[wd + "lc.h5//times"]
    out["lc_freqs"] = d[wd + "lc.h5//freqs"]
    for il in range(nl):
        out[f"lc{il}"] = d[f"{wd}lc.h5//shell=0 layer={il}/fluxdens"]
    # the sampled ODE right-hand-side evaluations: every layer at case["rhs_calls"]
    # sampled calls spread over the run
    calls = np.unique(rhs["call"])
    keep = calls[np.linspace(0, len(calls) - 1, min(case["rhs_calls"], len(calls))).astype(int)]
    rhs = rhs[np.isin(rhs["call"], keep)]
    for k in ("call", "layer", "pars", "before", "after", "dydt"):
        out["rhs_" + k] = rhs[k]
    path = os.path.join(HERE, f"refdrv_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"refdrv_{name}.npz: {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    pyoracle.build_reference()
    for name in sys.argv[1:] or list(CASES):
        run_case(name)
