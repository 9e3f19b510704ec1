"""The blastwave ODE right-hand side (pbag_bw_rhs on the host) against the
reference's own evaluations: the harness that runs the reference program
(oracle/ref_run.cpp) samples its integrator's right-hand-side calls and
records, per GRB blastwave, the inputs of rhs_fs / rhs_fsrs - state,
parameters, flags, the microphysics members its radiative-loss term reads -
and the derivatives it returned (tests/golden/refdrv_*.npz, rhs_*). The
forward shocks (rhs_fs) are compared bit for bit; the Gaussian jet's
forward + reverse shocks (rhs_fsrs) within 1e-10 relative: the reference
carries Gamma43 and the reverse-shock terms in x86 long double (64-bit
significands), the restatement Gamma43 in double-double (Gamma43 - 1 is
~1e-8 while the reverse shock starts), which leaves 1e-11 in Eint3 and Esh3
and ~1e-15 elsewhere. Plus the failure paths where the reference exits."""
import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300._lib import PbagError, bw_rhs
import refdrv_cases

# relative bar per written entry: exact for rhs_fs, 1e-10 for rhs_fsrs
TOL = {abi.PBAG_BW_FS: 0.0, abi.PBAG_BW_FSRS: 1e-10}


def rhs_samples(name):
    z = np.load(refdrv_cases.path(name))
    return z["rhs_pars"], z["rhs_before"], z["rhs_after"], z["rhs_dydt"]


def compare(P, A, D, got, after):
    """Max relative difference per (type, entry) over the entries each
    function writes, and of the carried members."""
    worst = {}
    for t, names in ((abi.PBAG_BW_FS, abi.BW_Q_FS), (abi.PBAG_BW_FSRS, abi.BW_Q_FSRS)):
        m = P["type"] == t
        if not m.any():
            continue
        for q in names:
            k = abi.BW_Q.index(q)
            r, g = D[m, k], got[m, k]
            den = np.abs(r)
            rel = np.where(den > 0, np.abs(g - r) / np.where(den > 0, den, 1.0), np.abs(g))
            worst[(t, q)] = float(rel.max())
    for f in ("fs_accel_frac", "fs_gamma_max", "rs_accel_frac", "rs_gamma_max"):
        d = np.abs(after[f] - A[f]) / np.maximum(np.abs(A[f]), 1e-300)
        worst[("carry", f)] = float(d.max())
    return worst


@pytest.mark.parametrize("name", refdrv_cases.CASES)
def test_rhs_matches_reference_evaluations(lib, name):
    P, B, A, D = rhs_samples(name)
    assert len(P) >= 500
    got, after = bw_rhs(P, B)
    worst = compare(P, A, D, got, after)
    for (t, q), w in worst.items():
        tol = TOL.get(t, 0.0) if t != "carry" else 0.0
        assert w <= tol, (name, t, q, w)
    if name == "gaussian":
        assert set(np.unique(P["type"])) == {abi.PBAG_BW_FS, abi.PBAG_BW_FSRS}


def test_rhs_failures(lib):
    """Where the reference exits: Gamma < 1 in rhs_fs (blastwave.h:1527),
    a negative swept-up mass, an invalid p in the loss term
    (microphysics_base.h:762-765), an unknown blastwave type; the first
    failing blastwave is reported."""
    P, B, A, D = rhs_samples("tophat")
    p, b = P[:4].copy(), B[:4].copy()
    bw_rhs(p, b)
    bad = b.copy()
    bad["Y"][2, abi.BW_Q.index("Gamma")] = 0.5
    bad["Y"][3, abi.BW_Q.index("M2")] = -1.0
    with pytest.raises(PbagError) as ei:
        bw_rhs(p, bad)
    assert ei.value.code == abi.PBAG_ERR_NONFINITE and ei.value.bw == 2 and ei.value.site == 1
    q = p.copy()
    q["fs"]["p"][1] = -1.0
    with pytest.raises(PbagError) as ei:
        bw_rhs(q, b)
    assert ei.value.code == abi.PBAG_ERR_PARAM and ei.value.bw == 1
    q = p.copy()
    q["type"][0] = 7
    with pytest.raises(PbagError) as ei:
        bw_rhs(q, b)
    assert ei.value.code == abi.PBAG_ERR_UNSUPPORTED and ei.value.bw == 0
