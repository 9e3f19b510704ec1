"""pbag_eats_flux_a (the adaptive EATS light curve on the GPU) against the
oracle, which the CPU suite pins to the reference's own EATS integrator:
the quadrature alone on the same histories, and the device-resident path -
the GPU step's histories left on the device and integrated there - against
the oracle's step and quadrature. The quadratures adapt to rtol 1e-6, so
results that differ in the last bits of an interpolated value may take
another subdivision: the bar is relative 1e-5 on the same histories."""
import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300._lib import Context, PbagError, eats_flux_a
import eats_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eats_inputs(lib, oracle):
    return {name: eats_cases.inputs(name, lib, oracle) for name in eats_cases.CASES}


def _gpu_eats(ctx, o, layers, dyn, off, d_j, d_a, q):
    import torch
    dev = torch.device("cuda", 0)
    d_dyn = torch.from_numpy(np.ascontiguousarray(dyn)).to(dev)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    d_f = torch.zeros(len(q), dtype=torch.float64, device=dev)
    eats_flux_a(ctx, o, layers, d_dyn.data_ptr(), dyn.shape[-1], off, d_j, d_a, len(q), d_q.data_ptr(),
                d_f.data_ptr())
    return d_f.cpu().numpy()


@pytest.mark.parametrize("name", list(eats_cases.CASES))
def test_eats_gpu_matches_oracle(oracle, cuda_device, eats_inputs, name):
    import torch
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs[name]
    rc, fail, ref = oracle.eats_flux(grid, o, layers, dyn, off, j, a, q)
    assert rc == 0, (rc, fail)
    ctx = Context(grid, device=0, ssc=bool(np.any(prm["ssc_on"])))
    dev = torch.device("cuda", 0)
    d_j = torch.from_numpy(np.ascontiguousarray(j)).to(dev)
    d_a = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    got = _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), q)
    ctx.close()
    rel = np.abs(got - ref) / ref
    assert rel.max() <= 1e-5, (rel.max(), np.argmax(rel))


def test_eats_device_resident(lib, oracle, cuda_device, eats_inputs):
    """The Gaussian jet's forward and reverse shocks: the GPU step writes its
    histories to device memory, the quadrature reads them there; against the
    oracle's step and quadrature (the step's own 1e-4 bar carried through)."""
    import torch
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs["gaussian_fsrs"]
    rc, fail, ref = oracle.eats_flux(grid, o, layers, dyn, off, j, a, q)
    assert rc == 0, (rc, fail)
    dev = torch.device("cuda", 0)
    ctx = Context(grid, device=0, ssc=True)
    nrec = int(off[-1])
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
    d_out = {k: torch.zeros((nrec, grid.nfreq), dtype=torch.float64, device=dev) for k in ("j_all", "a_all")}
    ctx.run_device(d_prm.data_ptr(), len(prm), off, d_recs.data_ptr(), {k: v.data_ptr() for k, v in d_out.items()})
    got = _gpu_eats(ctx, o, layers, dyn, off, d_out["j_all"].data_ptr(), d_out["a_all"].data_ptr(), q)
    ctx.close()
    rel = np.abs(got - ref) / ref
    assert rel.max() <= 1e-4, (rel.max(), np.argmax(rel))


@pytest.mark.parametrize("name", ["gaussian_fsrs", "gaussian_trap_no_cj"])
def test_eats_crew_matches_single_warp(oracle, cuda_device, eats_inputs, monkeypatch, name):
    """Four warps per item (the phi points of each outer step spread over
    them, the default) and one warp per item give the same light curve bit
    for bit: the same inner integrals, the outer sums in the same order."""
    import torch
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs[name]
    dev = torch.device("cuda", 0)
    ctx = Context(grid, device=0, ssc=True)
    d_j = torch.from_numpy(np.ascontiguousarray(j)).to(dev)
    d_a = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    monkeypatch.setenv("PBAG_EATS_WARPS", "1")
    one = _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), q)
    monkeypatch.setenv("PBAG_EATS_WARPS", "4")
    four = _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), q)
    ctx.close()
    np.testing.assert_array_equal(four, one)


@pytest.mark.parametrize("name", ["gaussian_fsrs", "tophat_off_axis"])
def test_eats_points_ahead_bit_identical(oracle, cuda_device, eats_inputs, monkeypatch, name):
    """The inner integral's points evaluated ahead on idle lanes (the
    default) and every point evaluated on request (PBAG_EATS_AHEAD=0) give
    the same light curve bit for bit: a point's value depends on its
    abscissa alone, and both form the abscissae the same way."""
    import torch
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs[name]
    assert o.method_quad == abi.PBAG_QUAD_CADRE
    dev = torch.device("cuda", 0)
    ctx = Context(grid, device=0, ssc=True)
    d_j = torch.from_numpy(np.ascontiguousarray(j)).to(dev)
    d_a = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    monkeypatch.setenv("PBAG_EATS_AHEAD", "0")
    on_request = _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), q)
    monkeypatch.delenv("PBAG_EATS_AHEAD")
    ahead = _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), q)
    ctx.close()
    assert np.all(ahead > 0)
    np.testing.assert_array_equal(ahead, on_request)


def test_eats_gpu_errors(oracle, cuda_device, eats_inputs):
    """Where the reference exits: an observer time outside the burster-time
    grid (PBAG_ERR_RANGE with the failing query), a query naming no layer
    (PBAG_ERR_ARG, checked before any launch)."""
    import torch
    grid, o, layers, dyn, off, recs, prm, j, a, q = eats_inputs["tophat_on_axis"]
    dev = torch.device("cuda", 0)
    ctx = Context(grid, device=0, ssc=False)
    d_j = torch.from_numpy(np.ascontiguousarray(j)).to(dev)
    d_a = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    bad = q.copy()
    bad["t_obs"][5] = dyn[0, abi.EATS_Q.index("tburst"), -1] * 2
    with pytest.raises(PbagError) as ei:
        _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), bad)
    assert ei.value.code == abi.PBAG_ERR_RANGE and ei.value.step == 5 and ei.value.bw == 0
    bad = q.copy()
    bad["layer"][2] = 7
    with pytest.raises(PbagError) as ei:
        _gpu_eats(ctx, o, layers, dyn, off, d_j.data_ptr(), d_a.data_ptr(), bad)
    assert ei.value.code == abi.PBAG_ERR_ARG
    ctx.close()
