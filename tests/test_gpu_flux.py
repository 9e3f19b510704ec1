"""pbag_flux_dens (EATS flux densities from the histories) against the
oracle, which the CPU suite pins to the reference's own fluxDens: every option
of the shock velocity, emitting-number and optical-depth methods, FP64 on both
sides; the out-of-grid frequency and bad-index errors."""
import itertools
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
import cases
import flux_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(lib, oracle):
    recs, off, prm, grid = cases.gaussian(lib, nlayers=2, nsteps=80)
    rc, where, h = oracle.run(grid, recs, off, prm, outputs=("j_all", "a_all"),
                              outer_threads=os.cpu_count() or 1)
    assert rc == 0
    _, freq = oracle.grids(grid)
    r_all = flux_cases.radii(off)
    return grid, off, freq, h["j_all"], h["a_all"], r_all


def _device(batch, q, cuda_device):
    import torch
    grid, off, freq, j, a, r = batch
    dev = torch.device("cuda", cuda_device)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in (("j", j), ("a", a), ("r", r))}
    t["q"] = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    t["out"] = torch.zeros(len(q), dtype=torch.float64, device=dev)
    return t


@pytest.mark.parametrize("vel,ne,tau", list(itertools.product((0, 1), (0, 1), (0, 1, 2, 3))))
def test_flux_dens_matches_oracle(lib, oracle, cuda_device, batch, vel, ne, tau):
    grid, off, freq, j, a, r = batch
    q = flux_cases.queries(off, freq, r, j, 2000, seed=100 + vel * 8 + ne * 4 + tau)
    opts = abi.FluxOpts(vel, ne, tau, 0)
    rc, fail, want = oracle.flux_dens(grid, opts, off, j, a, r, q)
    assert rc == 0
    ctx = lib.Context(grid, cuda_device, ssc=True)
    t = _device(batch, q, cuda_device)
    lib.flux_dens(ctx, opts, off, t["j"].data_ptr(), t["a"].data_ptr(), t["r"].data_ptr(), len(q),
                  t["q"].data_ptr(), t["out"].data_ptr())
    np.testing.assert_allclose(t["out"].cpu().numpy(), want, rtol=1e-12, atol=0)


def test_flux_dens_errors(lib, oracle, cuda_device, batch):
    grid, off, freq, j, a, r = batch
    q = flux_cases.queries(off, freq, r, j, 50, seed=7)
    q["freq"][17] = freq[0] * 0.5
    ctx = lib.Context(grid, cuda_device, ssc=True)
    t = _device(batch, q, cuda_device)
    with pytest.raises(lib.PbagError) as ei:
        lib.flux_dens(ctx, abi.FluxOpts(1, 1, 0, 0), off, t["j"].data_ptr(), t["a"].data_ptr(), t["r"].data_ptr(),
                      len(q), t["q"].data_ptr(), t["out"].data_ptr())
    assert ei.value.code == abi.PBAG_ERR_RANGE and ei.value.step == 17 and ei.value.bw == int(q["bw"][17])
    q2 = q.copy()
    q2["freq"][17] = q["freq"][16]
    q2["ib"][3] = 10 ** 6  # beyond the blastwave's history
    t = _device(batch, q2, cuda_device)
    with pytest.raises(lib.PbagError) as ei:
        lib.flux_dens(ctx, abi.FluxOpts(1, 1, 0, 0), off, t["j"].data_ptr(), t["a"].data_ptr(), t["r"].data_ptr(),
                      len(q2), t["q"].data_ptr(), t["out"].data_ptr())
    assert ei.value.code == abi.PBAG_ERR_ARG
