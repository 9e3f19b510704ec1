"""The GPU step against the FP64 oracle at the full sizes of the two
reference configurations, on every history (per-row relative L2 <= 1e-4,
rows the oracle leaves zero must be zero):

* the 21-layer Gaussian jet with forward and reverse shocks, synchrotron +
  SSA + SSC, 201 gamma x 128 nu, 1000 burster times - the benchmarked
  workload (42 blastwaves, 30 633 valid blastwave-steps; 2 697 of them run
  Chang-Cooper with 1 to 184 substeps);
* the top-hat forward shock, synchrotron only, 151 gamma x 96 nu, 1000
  burster times (543 Chang-Cooper steps, up to 26 substeps);

and windows of the jet that isolate the solver paths: 2-95 substeps per step
(the parallel scans, double-float and FP64) and 96 or more (the systolic
solve)."""
import os

import numpy as np
import pytest

import cases
from conftest import rel_l2_rows
from pyblastafterglowmag_gb300._lib import Context

pytestmark = pytest.mark.gpu
TOL = 1e-4
NTH = os.cpu_count() or 1


def _check(got, ref, outputs, tol=TOL):
    worst = {}
    for k in outputs:
        rel, zero_mismatch = rel_l2_rows(got[k], ref[k])
        worst[k] = float(rel.max())
        assert zero_mismatch == 0, f"{k}: {zero_mismatch} rows non-zero where the oracle is zero"
        assert rel.max() <= tol, f"{k}: max rel-L2 {rel.max():.3e} (p99 {np.percentile(rel, 99):.3e})"
    return worst


def _run_both(lib, oracle, batch, outputs=cases.ALL_OUTPUTS):
    recs, off, prm, grid = batch
    rc, where, ref = oracle.run(grid, recs, off, prm, outputs=outputs, outer_threads=NTH)
    assert rc == 0, (rc, where)
    ctx = Context(grid, device=0, ssc=bool(np.any(prm["ssc_on"])))
    got = ctx.run(recs, off, prm, outputs=outputs)
    ctx.close()
    return got, ref


def test_gaussian_jet_full_size(lib, oracle, cuda_device):
    batch = cases.gaussian_jet(lib)
    assert len(batch[1]) - 1 == 42 and int(batch[1][-1]) == 42000
    got, ref = _run_both(lib, oracle, batch)
    worst = _check(got, ref, cases.ALL_OUTPUTS)
    print("gaussian jet, worst rel-L2 per history:", {k: f"{v:.2e}" for k, v in worst.items()})


def test_tophat_full_size(lib, oracle, cuda_device):
    batch = cases.tophat_full(lib)
    assert int(batch[1][-1]) == 1000
    got, ref = _run_both(lib, oracle, batch)
    _check(got, ref, cases.ALL_OUTPUTS)


def test_jet_window_scan_substeps(lib, oracle, cuda_device):
    """Core and second layer, both shocks, steps 280-419: 242 steps with 2-95
    substeps (double-float scan), 36 with 96 or more."""
    got, ref = _run_both(lib, oracle, cases.jet_window(lib, (0, 1, 2, 3), 280, 140))
    _check(got, ref, cases.ALL_OUTPUTS)


def test_jet_window_systolic_substeps(lib, oracle, cuda_device):
    """Core and second layer forward shocks, steps 380-469: 118 steps with 96
    to 184 substeps (systolic solve)."""
    got, ref = _run_both(lib, oracle, cases.jet_window(lib, (0, 2), 380, 90))
    _check(got, ref, cases.ALL_OUTPUTS)


def test_gaussian_jet_full_size_tensor_core_sums(lib, oracle, cuda_device, monkeypatch):
    """The full jet with the synchrotron / SSA sums on the tensor cores (the
    kernel bank at 8 sub-shifts, log-space cubic interpolation), every history
    against the oracle."""
    monkeypatch.setenv("PBAG_SYN_TC", "1")
    got, ref = _run_both(lib, oracle, cases.gaussian_jet(lib))
    _check(got, ref, cases.ALL_OUTPUTS)
