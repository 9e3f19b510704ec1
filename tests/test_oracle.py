"""The oracle (FP64 CPU restatement) pinned against the reference: bit-exact
against the golden fixtures the reference's own code produced
(tests/golden/make_golden.py), and live against the compiled reference where
its sources exist."""
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
import cases

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name), allow_pickle=False)


def grid_of(a):
    return abi.GridDesc(int(a[0]), int(a[1]), *map(float, a[2:]))


def test_grids_exact(oracle):
    d = load("grids.npz")
    for tag in ("tophat", "gauss"):
        gam, freq = oracle.grids(grid_of(d[f"{tag}_grid"]))
        np.testing.assert_array_equal(gam, d[f"{tag}_gam"])
        np.testing.assert_array_equal(freq, d[f"{tag}_freq"])


@pytest.mark.parametrize("method,name", [(abi.PBAG_SYN_CSYN, "csyn"), (abi.PBAG_SYN_DER09, "der09"),
                                         (abi.PBAG_SYN_GSL, "gsl"), (abi.PBAG_SYN_BESSEL, "bessel")])
def test_syn_kernel_exact(oracle, method, name):
    d = load("syn_kernel.npz")
    for ib, B in enumerate(d["B"]):
        got = oracle.syn_kernel(method, float(B), d["gam"], d["freq"][:-1])
        np.testing.assert_array_equal(got, d[name][ib])


def test_ssc_kernel_exact(oracle):
    d = load("ssc_kernel.npz")
    K, Kint = oracle.ssc_kernel(d["gam"], d["freq"])
    np.testing.assert_array_equal(K, d["K"])
    np.testing.assert_array_equal(Kint, d["Kint"])


@pytest.mark.parametrize("name", ["run_tophat.npz", "run_gauss.npz"])
def test_histories_exact(oracle, name):
    d = load(name)
    rc, where, got = oracle.run(grid_of(d["grid"]), d["recs"], d["offsets"], d["params"],
                                outputs=cases.ALL_OUTPUTS)
    assert rc == 0, where
    for k in cases.ALL_OUTPUTS:
        np.testing.assert_array_equal(got[k], d[k], err_msg=k)


def test_hoisted_heating_is_bitwise_identical(oracle):
    d = load("run_gauss.npz")
    g = grid_of(d["grid"])
    _, _, a = oracle.run(g, d["recs"], d["offsets"], d["params"], flags=0)
    _, _, b = oracle.run(g, d["recs"], d["offsets"], d["params"], flags=1, outer_threads=4)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


def test_inner_threads_are_bitwise_identical(oracle):
    """The reference's own arrangement (blastwaves serial, inner loops on 4
    threads; the benchmark's as-is CPU figure) gives the serial results."""
    import pyoracle
    d = load("run_gauss.npz")
    g = grid_of(d["grid"])
    _, _, a = oracle.run(g, d["recs"], d["offsets"], d["params"], flags=0)
    rc, _, b = oracle.run(g, d["recs"], d["offsets"], d["params"], flags=pyoracle.ORC_INNER_OMP,
                          outer_threads=1, inner_threads=4)
    assert rc == 0
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


def test_live_reference_matches_oracle(lib, oracle, reference):
    for batch in (cases.tophat(lib, nsteps=120, ssa=True),
                  cases.tophat(lib, nsteps=80, syn_method=abi.PBAG_SYN_DER09, ele_method=abi.PBAG_ELE_MIX),
                  cases.gaussian(lib, nlayers=2, nsteps=50, ngam=64, nfreq=40),
                  cases.uneven(lib, nsets=2, seed=5)):
        recs, off, prm, grid = batch
        if np.any(prm["ssc_on"]) and not np.all(prm["ssc_on"]):
            continue  # the reference shares one SSC kernel object across blastwaves
        r = reference.run(grid, recs, off, prm, outputs=cases.ALL_OUTPUTS)
        rc, where, o = oracle.run(grid, recs, off, prm, outputs=cases.ALL_OUTPUTS, outer_threads=4)
        assert rc == 0, where
        for k in cases.ALL_OUTPUTS:
            np.testing.assert_array_equal(o[k], r[k], err_msg=k)


def test_live_reference_matches_oracle_with_pair_production(lib, oracle, reference):
    """Pair production (method_pp numeric: the pair source of numeric_model.h:
    727-733, the absorption of :343-356 and the attenuation of
    microphysics.h:565-574) with SSC and SSA, every history."""
    recs, off, prm, grid = cases.gaussian(lib, nlayers=2, nsteps=50, ngam=64, nfreq=40)
    prm = prm.copy()
    prm["pp_on"] = 1
    r = reference.run(grid, recs, off, prm, outputs=cases.ALL_OUTPUTS)
    rc, where, o = oracle.run(grid, recs, off, prm, outputs=cases.ALL_OUTPUTS, outer_threads=4)
    assert rc == 0, where
    for k in cases.ALL_OUTPUTS:
        np.testing.assert_array_equal(o[k], r[k], err_msg=k)
    # pair production changes the result
    prm0 = prm.copy()
    prm0["pp_on"] = 0
    _, _, base = oracle.run(grid, recs, off, prm0, outputs=("j_all",))
    assert not np.array_equal(base["j_all"], o["j_all"])


def test_oracle_reports_reference_exit_conditions(lib, oracle):
    """Conditions on which the reference calls exit(1) become status codes."""
    recs, off, prm, grid = cases.tophat(lib, nsteps=40)
    bad = recs.copy()
    bad["m_p1"][25] = bad["m"][25] * 0.5           # dlnV/dt < 0 (microphysics.h:406)
    rc, where, _ = oracle.run(grid, bad, off, prm)
    assert (rc, where) == (abi.PBAG_ERR_DLNVDT, (0, 25))
    bad = recs.copy()
    bad["B"][12] = -1.0                              # B <= 0 (microphysics.h:372)
    rc, where, _ = oracle.run(grid, bad, off, prm)
    assert (rc, where) == (abi.PBAG_ERR_PARAM, (0, 12))
    bad = recs.copy()
    bad["gamma_min"][30] = bad["gamma_max"][30] * 2  # gamma_min >= gamma_max
    rc, where, _ = oracle.run(grid, bad, off, prm)
    assert (rc, where) == (abi.PBAG_ERR_PARAM, (0, 30))
