"""The oracle's restatement of fluxDens / computeFluxDensity against the
reference's own ElectronAndRadiation::fluxDens (compiled from its sources in
this container; skipped where the reference is absent), for every option of
the shock velocity, the emitting-number method and the optical-depth method."""
import ctypes as C
import itertools
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
import cases
import flux_cases


def _reference():
    import pyoracle
    if not os.path.exists(pyoracle.REF_SO):
        if not pyoracle.build_reference():
            pytest.skip("reference sources not present")
    return pyoracle.Reference()


@pytest.mark.parametrize("vel,ne,tau", list(itertools.product((0, 1), (0, 1), (0, 1, 2, 3))))
def test_flux_dens_matches_reference(lib, oracle, vel, ne, tau):
    ref = _reference()
    recs, off, prm, grid = cases.tophat(lib, nsteps=60, ssa=True)
    rc, where, h = oracle.run(grid, recs, off, prm, outputs=("j_all", "a_all"))
    assert rc == 0
    _, freq = oracle.grids(grid)
    r_all = flux_cases.radii(off)
    q = flux_cases.queries(off, freq, r_all, h["j_all"], 300, seed=vel * 8 + ne * 4 + tau)
    opts = abi.FluxOpts(vel, ne, tau, 0)
    rc, fail, got = oracle.flux_dens(grid, opts, off, h["j_all"], h["a_all"], r_all, q)
    assert rc == 0 and fail == -1
    # one blastwave here: the reference object holds its histories
    want = ref.flux_dens(grid, opts, h["j_all"], h["a_all"], r_all, q)
    np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)
    assert (got > 0).any()


def test_flux_dens_frequency_outside_grid(lib, oracle):
    recs, off, prm, grid = cases.tophat(lib, nsteps=20)
    rc, where, h = oracle.run(grid, recs, off, prm, outputs=("j_all", "a_all"))
    _, freq = oracle.grids(grid)
    r_all = flux_cases.radii(off)
    q = flux_cases.queries(off, freq, r_all, h["j_all"], 5)
    q["freq"][3] = freq[grid.nfreq - 1] * 1.01
    rc, fail, _ = oracle.flux_dens(grid, abi.FluxOpts(1, 1, 0, 0), off, h["j_all"], h["a_all"], r_all, q)
    assert rc == abi.PBAG_ERR_RANGE and fail == 3
