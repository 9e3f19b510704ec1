"""The oracle's restatement of the adaptive EATS light curve against the
reference's own EATS::evalFluxDensA (compiled from its sources where they
exist) and against the golden light curves that reference produced
(tests/golden/eats_lc.npz, tests/golden/make_golden_eats.py)."""
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
import eats_cases

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def eats_inputs(oracle):
    return {name: eats_cases.inputs(name, oracle, oracle) for name in eats_cases.CASES}


@pytest.fixture(scope="module")
def reference_eats():
    import pyoracle
    try:
        return pyoracle.ReferenceEats()
    except (FileNotFoundError, OSError) as e:
        pytest.skip(f"reference sources not available: {e}")


@pytest.mark.parametrize("name", list(eats_cases.CASES))
def test_eats_oracle_matches_reference(oracle, reference_eats, eats_inputs, name):
    """Same inputs, same algorithm, same operation order: equal to the last bit."""
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs[name]
    ref = reference_eats.eats_flux(grid, o, layers, dyn, off, j, a, q)
    rc, fail, got = oracle.eats_flux(grid, o, layers, dyn, off, j, a, q)
    assert rc == 0, (rc, fail)
    assert np.all(ref > 0)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("name", list(eats_cases.CASES))
def test_eats_oracle_matches_golden(oracle, eats_inputs, name):
    """Against the reference's light curves: exact where the inputs were
    built with the same libm, within the adaptive tolerance otherwise."""
    gold = np.load(os.path.join(HERE, "golden", "eats_lc.npz"))[name]
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs[name]
    rc, fail, got = oracle.eats_flux(grid, o, layers, dyn, off, j, a, q)
    assert rc == 0, (rc, fail)
    rel = np.abs(got - gold) / gold
    assert rel.max() <= 1e-5, rel.max()


def test_eats_oracle_errors(oracle, eats_inputs):
    """An observer time outside the burster-time grid, and a comoving
    frequency below the photon grid, are where the reference exits."""
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs["tophat_on_axis"]
    bad = q.copy()
    bad["t_obs"][5] = dyn[0, abi.EATS_Q.index("tburst"), -1] * 2
    rc, fail, _ = oracle.eats_flux(grid, o, layers, dyn, off, j, a, bad)
    assert rc == abi.PBAG_ERR_RANGE and fail == 5
    bad = q.copy()
    bad["nu_obs"][3] = 1e6
    rc, fail, _ = oracle.eats_flux(grid, o, layers, dyn, off, j, a, bad)
    assert rc == abi.PBAG_ERR_RANGE and fail == 3
