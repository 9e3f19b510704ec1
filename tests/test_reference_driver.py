"""The oracle on the reference program's own inputs: step records rebuilt
from the dynamics the reference's blastwave driver saved must reproduce the
shock scalars the driver stored with them, the comoving spectra its
radiation step wrote (computeSaveEjectaSpectrum) and, through the oracle's
EATS, the light curve it wrote (computeSaveEjectaLightCurve). The recorded
runs are tests/golden/refdrv_*.npz; on CPU the Gaussian jet is checked on its
first layer (forward and reverse shock, synchrotron + SSC + SSA), the GPU
tests cover all of it."""
import os

import numpy as np
import pytest

from conftest import rel_l2_rows
import refdrv_cases

NTH = os.cpu_count() or 1


@pytest.fixture(scope="module")
def runs():
    return refdrv_cases.Runs()


@pytest.mark.parametrize("name", refdrv_cases.CASES)
def test_records_reproduce_saved_scalars(oracle, runs, name):
    """B, gamma_min and gamma_max of every step the driver ran, restated by
    the oracle's computeEleSpectrumLimits, equal what the driver saved."""
    run = runs[name]
    recs, off, prm = run.records(oracle)
    assert len(prm) == run.nlayers * (2 if run.rs else 1)
    for il in range(run.nlayers):
        b = run.blastwave(il, "fs")
        r = recs[off[b]:off[b + 1]]
        ran = r["mode"] != 0
        assert ran.sum() > 0.9 * len(r)
        for k in ("B", "gamma_min", "gamma_max"):
            np.testing.assert_array_equal(r[k][ran], run.dyn[il][k][ran], err_msg=f"layer {il} {k}")


def _oracle_spectra(oracle, run, layers):
    recs, off, prm = run.records(oracle, layers)
    rc, where, out = oracle.run(run.grid, recs, off, prm, outputs=("j_all", "a_all"), outer_threads=NTH)
    assert rc == 0, (rc, where)
    return off, out


def test_oracle_spectra_tophat(oracle, runs):
    """Every row of the top-hat's forward-shock spectrum, bit for bit."""
    run = runs["tophat"]
    off, out = _oracle_spectra(oracle, run, None)
    ref = run.spec[(0, "fs", "j")]
    np.testing.assert_array_equal(out["j_all"][off[0]:off[1]], ref)


def test_oracle_spectra_gaussian_first_layer(oracle, runs):
    """The Gaussian jet's core layer, forward and reverse shock, emissivity
    and absorption (SSA), every tenth time index."""
    run = runs["gaussian"]
    off, out = _oracle_spectra(oracle, run, 1)
    n = 0
    for shock in ("fs", "rs"):
        b = run.blastwave(0, shock)
        for q in ("j", "a"):
            ref = run.spec.get((0, shock, q))
            if ref is None:
                continue
            got = out[f"{q}_all"][off[b]:off[b + 1]][::run.every]
            rel, zm = rel_l2_rows(got, ref)
            assert zm == 0 and rel.max() <= 1e-12, (shock, q, rel.max(), zm)
            n += 1
    assert n == 4


def test_oracle_light_curve_tophat(oracle, runs):
    """The top-hat's light curve (32 observer times, counter jet, CADRE)
    from the oracle's spectra and EATS, bit for bit."""
    run = runs["tophat"]
    off, out = _oracle_spectra(oracle, run, None)
    layers, dyn, q = run.eats()
    rc, fail, flux = oracle.eats_flux(run.grid, run.eats_opts(), layers, dyn, off, out["j_all"], out["a_all"], q)
    assert rc == 0, (rc, fail)
    np.testing.assert_array_equal(flux, run.lc.ravel())
