"""The GPU step and the GPU light curve on the reference program's own
inputs, against what the reference program computed from them
(tests/golden/refdrv_*.npz, recorded by tests/golden/make_reference_run.py):
the step records come from the dynamics the reference's blastwave driver
saved, the library's pbag_run over all of them must give the comoving
spectra the reference wrote (relative L2 per row 1e-4, the step's bar
against the oracle), and pbag_eats_flux_a over the step's device-resident
histories the reference's light curve of every layer (relative 1e-4: the
step's bar carried through the adaptive quadrature). The top-hat is one
forward shock with synchrotron; the Gaussian jet is 21 layers of forward
and reverse shocks with synchrotron, SSC and SSA."""
import numpy as np
import pytest

from conftest import rel_l2_rows
from pyblastafterglowmag_gb300._lib import Context, eats_flux_a
import refdrv_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def runs():
    return refdrv_cases.Runs()


def _gpu_run(lib, run):
    """The step over every blastwave with its outputs left on the device;
    returns (ctx, offsets, d_out)."""
    import torch
    dev = torch.device("cuda", 0)
    recs, off, prm = run.records(lib)
    ctx = Context(run.grid, device=0, ssc=bool(np.any(prm["ssc_on"])))
    nrec = int(off[-1])
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
    d_out = {k: torch.zeros((nrec, run.grid.nfreq), dtype=torch.float64, device=dev) for k in ("j_all", "a_all")}
    ctx.run_device(d_prm.data_ptr(), len(prm), off, d_recs.data_ptr(), {k: v.data_ptr() for k, v in d_out.items()})
    torch.cuda.synchronize()
    return ctx, off, d_out


@pytest.mark.parametrize("name", refdrv_cases.CASES)
def test_gpu_step_matches_reference_program(lib, cuda_device, runs, name):
    run = runs[name]
    ctx, off, d_out = _gpu_run(lib, run)
    out = {k: v.cpu().numpy() for k, v in d_out.items()}
    ctx.close()
    assert run.spec
    for (il, shock, q), ref in run.spec.items():
        b = run.blastwave(il, shock)
        got = out[f"{q}_all"][off[b]:off[b + 1]][::run.every]
        rel, zm = rel_l2_rows(got, ref)
        assert zm == 0 and rel.max() <= 1e-4, (il, shock, q, rel.max(), zm)


@pytest.mark.parametrize("name", refdrv_cases.CASES)
def test_gpu_light_curve_matches_reference_program(lib, cuda_device, runs, name):
    import torch
    run = runs[name]
    ctx, off, d_out = _gpu_run(lib, run)
    layers, dyn, q = run.eats()
    dev = torch.device("cuda", 0)
    d_dyn = torch.from_numpy(np.ascontiguousarray(dyn)).to(dev)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    d_f = torch.zeros(len(q), dtype=torch.float64, device=dev)
    eats_flux_a(ctx, run.eats_opts(), layers, d_dyn.data_ptr(), dyn.shape[-1], off, d_out["j_all"].data_ptr(),
                d_out["a_all"].data_ptr(), len(q), d_q.data_ptr(), d_f.data_ptr())
    got = d_f.cpu().numpy()
    ctx.close()
    ref = run.lc.ravel()
    assert np.all(ref > 0)
    rel = np.abs(got - ref) / ref
    assert rel.max() <= 1e-4, (rel.max(), int(np.argmax(rel)))
