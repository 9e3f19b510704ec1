"""Host-side parts of libpbag (no GPU needed): the library loads, exports
every entry point include/pbag.h declares with matching struct layouts, and
its grid builder and per-step shock-scalar prep match the reference."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi, histories as H
import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(pbag_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(lib):
    so = lib.load()
    names = declared_functions()
    assert "pbag_run_batch" in names and "pbag_create" in names
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_struct_layouts(lib):
    so = lib.load()
    assert so.pbag_abi_version() == 1
    assert so.pbag_sizeof(2) == abi.STEP_DTYPE.itemsize == 136
    assert so.pbag_sizeof(8) == C.sizeof(abi.FluxOpts) == 16
    assert so.pbag_sizeof(9) == abi.FLUX_QUERY_DTYPE.itemsize == 112


def test_grids_match_reference_fixture(lib):
    d = np.load(os.path.join(GOLD, "grids.npz"))
    for tag in ("tophat", "gauss"):
        a = d[f"{tag}_grid"]
        gam, freq = lib.grids(abi.GridDesc(int(a[0]), int(a[1]), *map(float, a[2:])))
        np.testing.assert_array_equal(gam, d[f"{tag}_gam"])
        np.testing.assert_array_equal(freq, d[f"{tag}_freq"])


def test_bad_grid_rejected(lib):
    with pytest.raises(lib.PbagError):
        lib.grids(abi.GridDesc(4, 128, 1.0, 1e9, 1e8, 1e29))
    with pytest.raises(lib.PbagError):
        lib.grids(abi.GridDesc(64, 64, 1.0, 1e9, 1e29, 1e8))


def test_shock_limits_match_reference_fixture(lib):
    d = np.load(os.path.join(GOLD, "shock_limits.npz"))
    a = d["grid"]
    gam, _ = lib.grids(abi.GridDesc(int(a[0]), int(a[1]), *map(float, a[2:])))
    for (gm, gc, gx, bm, nr, p), ref in zip(d["opts"], d["out"]):
        o = abi.LimitsOpts()
        o.p, o.eps_e, o.eps_b, o.eps_t = p, 0.1, 1e-3, 0.5
        o.beta_min, o.mu, o.mu_e = 1e-5, 0.62, 1.18
        o.method_B, o.method_gamma_min, o.method_gamma_c = int(bm), int(gm), int(gc)
        o.method_gamma_max, o.method_nonrel, o.ele_analytic = int(gx), int(nr), 0
        state = np.array([-1.0, 1e7, 1e5 if int(gc) == 2 else -1.0, 1.0, -1.0, -1.0, -1.0])
        got = lib.shock_limits(o, gam, d["states"], state=state)
        cols = ["B", "gamma_min", "gamma_max", "gamma_c", "accel_frac", "Theta", "z_cool"]
        g = np.stack([got[c] for c in cols] + [got["valid"].astype(float)], axis=1)
        np.testing.assert_allclose(g, ref, rtol=1e-13, atol=0, err_msg=str((gm, gc, gx, bm, nr, p)))


def test_shock_limits_live_reference(lib, reference):
    cfg = H.config_gaussian_ssc()
    g = cfg.grid()
    gam, _ = lib.grids(g)
    tb = np.logspace(np.log10(cfg.tb1), np.log10(cfg.tb2), 300)
    lo, hi, E, G0 = H.layer_table(cfg)
    d = H.layer_dynamics(E[0], G0[0], cfg.n_ism, tb, 0.01)
    st = H.fs_state(d)
    ss = np.zeros(len(tb), dtype=abi.SHOCK_STATE_DTYPE)
    ss["e_prime"], ss["Gamma"], ss["GammaSh"] = st["u_p"], st["Gamma"], st["GammaSh"]
    ss["t_e"], ss["t_b"], ss["tcomov"] = d["t_obs"], tb, d["tcomov"]
    ss["n_prime"], ss["n_protons"] = st["rho2"] / H.M_P, st["m2"] / H.M_P
    o = H.limits_opts(cfg.fs)
    got = lib.shock_limits(o, gam, ss)
    ref = reference.ele_limits(g, o, ss)
    cols = ["B", "gamma_min", "gamma_max", "gamma_c", "accel_frac", "Theta", "z_cool"]
    g2 = np.stack([got[c] for c in cols] + [got["valid"].astype(float)], axis=1)
    np.testing.assert_allclose(g2, ref, rtol=1e-13, atol=0)


def test_history_generator_is_seeded(lib):
    a = cases.uneven(lib, nsets=2, seed=3)
    b = cases.uneven(lib, nsets=2, seed=3)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_vectorised_dynamics_match_per_layer():
    cfg = H.config_gaussian_ssc()
    cfg.nlayers = 5
    tb = np.logspace(np.log10(cfg.tb1), np.log10(cfg.tb2), 200)
    lo, hi, E, G0 = H.layer_table(cfg)
    om = 2 * np.pi * (np.cos(lo) - np.cos(hi)) * 2
    many = H.layer_dynamics_many(E, G0, cfg.n_ism, tb, om, nsamp=800)
    for i in range(cfg.nlayers):
        one = H.layer_dynamics(E[i], G0[i], cfg.n_ism, tb, om[i], nsamp=800)
        for k in ("Gamma", "R", "m", "tcomov", "t_obs"):
            np.testing.assert_allclose(many[i][k], one[k], rtol=1e-10, atol=0)


def test_pooled_sweep_equals_serial(lib):
    a = H.sweep_batch(lib, 3, seed=11, min_steps=20, max_steps=60, max_layers=3)
    b = H.sweep_batch(lib, 3, seed=11, min_steps=20, max_steps=60, max_layers=3, workers=2)
    assert (a[0].tobytes() == b[0].tobytes()) and (a[1] == b[1]).all()


def test_oracle_shock_limits_match_reference_fixture(oracle):
    """The oracle's own restatement of computeEleSpectrumLimits against the
    values the reference produced, for every option set of the fixture."""
    d = np.load(os.path.join(GOLD, "shock_limits.npz"))
    a = d["grid"]
    gam, _ = oracle.grids(abi.GridDesc(int(a[0]), int(a[1]), *map(float, a[2:])))
    for (gm, gc, gx, bm, nr, p), ref in zip(d["opts"], d["out"]):
        o = abi.LimitsOpts()
        o.p, o.eps_e, o.eps_b, o.eps_t = p, 0.1, 1e-3, 0.5
        o.beta_min, o.mu, o.mu_e = 1e-5, 0.62, 1.18
        o.method_B, o.method_gamma_min, o.method_gamma_c = int(bm), int(gm), int(gc)
        o.method_gamma_max, o.method_nonrel, o.ele_analytic = int(gx), int(nr), 0
        state = np.array([-1.0, 1e7, 1e5 if int(gc) == 2 else -1.0, 1.0, -1.0, -1.0, -1.0])
        got = oracle.shock_limits(o, gam, d["states"], state=state)
        cols = ["B", "gamma_min", "gamma_max", "gamma_c", "accel_frac", "Theta", "z_cool"]
        g = np.stack([got[c] for c in cols] + [got["valid"].astype(float)], axis=1)
        np.testing.assert_allclose(g, ref, rtol=1e-13, atol=0, err_msg=str((gm, gc, gx, bm, nr, p)))


def test_oracle_built_records_equal_library_built_records(lib, oracle):
    """The benchmark's CPU arm builds the Gaussian jet's step records with the
    oracle alone; they are the same bytes the library's host code produces."""
    a = H.make_batch(lib, H.config_gaussian_ssc())
    b = H.make_batch(oracle, H.config_gaussian_ssc())
    assert a[0].tobytes() == b[0].tobytes()
    assert (a[1] == b[1]).all() and a[2].tobytes() == b[2].tobytes()
