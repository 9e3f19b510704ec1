"""GPU path (libpbag through its C ABI) against the FP64 oracle on identical
seeded records. Tolerance: per-row relative L2 error <= 1e-4 for every
history (the plain-path bar), computed over rows where the oracle is non-zero;
rows the oracle leaves zero must be zero on the GPU too."""
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300._lib import Context, PbagError
import cases
from conftest import rel_l2_rows

pytestmark = pytest.mark.gpu
TOL = 1e-4
NTH = os.cpu_count() or 1


def _compare(lib, oracle, batch, outputs=cases.ALL_OUTPUTS, tol=TOL):
    recs, off, prm, grid = batch
    rc, where, ref = oracle.run(grid, recs, off, prm, outputs=outputs, outer_threads=NTH)
    assert rc == 0, (rc, where)
    ssc = bool(np.any(prm["ssc_on"]))
    ctx = Context(grid, device=0, ssc=ssc)
    got = ctx.run(recs, off, prm, outputs=outputs)
    assert ctx.last_launch_count() > 0
    worst = {}
    for k in outputs:
        rel, zero_mismatch = rel_l2_rows(got[k], ref[k])
        worst[k] = float(rel.max())
        assert zero_mismatch == 0, f"{k}: {zero_mismatch} rows non-zero where the oracle is zero"
        assert rel.max() <= tol, f"{k}: max rel-L2 {rel.max():.3e} (p99 {np.percentile(rel, 99):.3e})"
    ctx.close()
    return worst


def test_tophat_syn(lib, oracle, cuda_device):
    _compare(lib, oracle, cases.tophat(lib, nsteps=250))


def test_tophat_ssa(lib, oracle, cuda_device):
    _compare(lib, oracle, cases.tophat(lib, nsteps=250, ssa=True))


def test_tophat_dermer_mix(lib, oracle, cuda_device):
    _compare(lib, oracle, cases.tophat(lib, nsteps=120, ssa=True, syn_method=abi.PBAG_SYN_DER09,
                                       ele_method=abi.PBAG_ELE_MIX))


@pytest.mark.parametrize("method", [abi.PBAG_SYN_GSL, abi.PBAG_SYN_BESSEL])
def test_tophat_gsl_bessel(lib, oracle, cuda_device, method):
    """The GSL and Bessel synchrotron methods (tabulated in FP64 on the host,
    interpolated on the device) with SSA, against the oracle's direct FP64
    evaluation."""
    _compare(lib, oracle, cases.tophat(lib, nsteps=120, ssa=True, syn_method=method))


def test_gaussian_ssc(lib, oracle, cuda_device):
    _compare(lib, oracle, cases.gaussian(lib, nlayers=3, nsteps=120))


def test_gaussian_ssc_pair_production(lib, oracle, cuda_device):
    """method_pp numeric: the pair source of every electron bin, the pair
    absorption and the attenuation of the total emissivity, every history."""
    recs, off, prm, grid = cases.gaussian(lib, nlayers=3, nsteps=80)
    prm = prm.copy()
    prm["pp_on"] = 1
    _compare(lib, oracle, (recs, off, prm, grid))


def test_gaussian_ssc_small_batch_kernel(lib, oracle, cuda_device, monkeypatch):
    """The step with the small-batch slab kernel forced for its SSC contraction."""
    monkeypatch.setenv("PBAG_TC_KERNEL", "slab-small")
    _compare(lib, oracle, cases.gaussian(lib, nlayers=3, nsteps=60))


def test_gaussian_ssc_fp64_scan(lib, oracle, cuda_device, monkeypatch):
    """The Chang-Cooper substeps with the FP64 scan and systolic pipeline
    forced (the paths a step takes when its coefficients leave the FP32 range
    of the double-float ones), on a window of the jet whose Chang-Cooper steps
    take 2-125 substeps."""
    monkeypatch.setenv("PBAG_SCAN_FP64", "1")
    _compare(lib, oracle, cases.jet_window(lib, (0, 1, 2, 3), 280, 140))


def test_double_float_scan_matches_fp64_scan(lib, cuda_device, monkeypatch):
    """The double-float substeps against the FP64 ones on the same batch: the
    electron histories agree to far below the plain-path bar (the pairs carry
    ~48 significant bits); the emissivities, formed from FP32 weights of those
    histories, to within an FP32 rounding. The window's Chang-Cooper steps
    take 2-125 substeps (scan below 32, systolic pipeline from 32)."""
    recs, off, prm, grid = cases.jet_window(lib, (0, 1, 2, 3), 280, 140)
    outs = ("ele_f_all", "j_all")
    ctx = Context(grid, device=0, ssc=True)
    df = ctx.run(recs, off, prm, outputs=outs)
    ctx.close()
    monkeypatch.setenv("PBAG_SCAN_FP64", "1")
    ctx = Context(grid, device=0, ssc=True)
    f64 = ctx.run(recs, off, prm, outputs=outs)
    ctx.close()
    for k, tol in (("ele_f_all", 1e-9), ("j_all", 1e-6)):
        rel, zero_mismatch = rel_l2_rows(df[k], f64[k])
        assert zero_mismatch == 0, k
        assert rel.max() <= tol, (k, rel.max())


def test_double_float_systolic_matches_fp64_systolic(lib, cuda_device, monkeypatch):
    """The systolic pipeline in double-float against the FP64 one on the
    uneven batch, whose long steps take up to 1000 substeps: electron
    histories within 1e-9, emissivities within an FP32 rounding."""
    recs, off, prm, grid = cases.uneven(lib)
    outs = ("ele_f_all", "j_all")
    ctx = Context(grid, device=0, ssc=True)
    df = ctx.run(recs, off, prm, outputs=outs)
    ctx.close()
    monkeypatch.setenv("PBAG_SCAN_FP64", "1")
    ctx = Context(grid, device=0, ssc=True)
    f64 = ctx.run(recs, off, prm, outputs=outs)
    ctx.close()
    for k, tol in (("ele_f_all", 1e-9), ("j_all", 1e-6)):
        rel, zero_mismatch = rel_l2_rows(df[k], f64[k])
        assert zero_mismatch == 0, k
        assert rel.max() <= tol, (k, rel.max())


def test_systolic_from_two_substeps(lib, oracle, cuda_device, monkeypatch):
    """Every Chang-Cooper step with two or more substeps on the systolic
    pipeline (PBAG_SYSTOLIC_MIN=2): the jet window of 2-125 substeps per step,
    every history against the oracle."""
    monkeypatch.setenv("PBAG_SYSTOLIC_MIN", "2")
    _compare(lib, oracle, cases.jet_window(lib, (0, 1, 2, 3), 280, 140))


def test_gaussian_late_window(lib, oracle, cuda_device):
    _compare(lib, oracle, cases.gaussian_window(lib, start=380, nsteps=60))


def test_uneven_batch(lib, oracle, cuda_device):
    """Three seeded sweep jets with uneven histories (up to 1000 substeps per
    step; the blastwaves run in slots ordered by history length), every
    history."""
    _compare(lib, oracle, cases.uneven(lib))


def test_error_status_matches_oracle(lib, oracle, cuda_device):
    recs, off, prm, grid = cases.tophat(lib, nsteps=60)
    bad = recs.copy()
    bad["m_p1"][37] = bad["m"][37] * 0.5  # volume shrinks: dlnV/dt < 0 (microphysics.h:406-409)
    rc, where, _ = oracle.run(grid, bad, off, prm, outputs=cases.TOTALS)
    assert rc == abi.PBAG_ERR_DLNVDT and where == (0, 37)
    ctx = Context(grid, device=0, ssc=False)
    with pytest.raises(PbagError) as ei:
        ctx.run(bad, off, prm)
    assert ei.value.code == abi.PBAG_ERR_DLNVDT and (ei.value.bw, ei.value.step) == (0, 37)


def test_error_status_in_uneven_batch(lib, oracle, cuda_device):
    """An uneven batch runs its blastwaves in slots ordered by history length;
    the first failure is still reported as the caller's blastwave and step."""
    recs, off, prm, grid = cases.uneven(lib)
    lens = np.diff(off)
    b = int(np.argsort(lens)[len(lens) // 2])  # a blastwave of middle length
    valid = np.flatnonzero(recs["mode"][off[b]:off[b + 1]] != 0)
    s = int(valid[len(valid) // 2])
    bad = recs.copy()
    bad["m_p1"][off[b] + s] = bad["m"][off[b] + s] * 0.5  # dlnV/dt < 0 (microphysics.h:406-409)
    rc, where, _ = oracle.run(grid, bad, off, prm, outputs=cases.TOTALS)
    assert rc == abi.PBAG_ERR_DLNVDT
    ctx = Context(grid, device=0, ssc=True)
    with pytest.raises(PbagError) as ei:
        ctx.run(bad, off, prm)
    assert ei.value.code == rc and (ei.value.bw, ei.value.step) == where


def test_empty_and_zero_length(lib, oracle, cuda_device):
    recs, off, prm, grid = cases.tophat(lib, nsteps=30)
    ctx = Context(grid, device=0, ssc=False)
    got = ctx.run(recs[:0], np.zeros(1, dtype=np.int64), prm[:0])
    assert all(v.shape[0] == 0 for v in got.values())
    # a zero-length blastwave between two real ones
    recs2 = np.concatenate([recs, recs])
    off2 = np.array([0, 30, 30, 60], dtype=np.int64)
    prm2 = np.concatenate([prm, prm, prm])
    got = ctx.run(recs2, off2, prm2)
    rc, where, ref = oracle.run(grid, recs2, off2, prm2, outputs=cases.TOTALS)
    assert rc == 0
    for k in cases.TOTALS:
        rel, zm = rel_l2_rows(got[k], ref[k])
        assert zm == 0 and rel.max() <= TOL


def test_unsupported_options_rejected(lib, cuda_device):
    recs, off, prm, grid = cases.tophat(lib, nsteps=10)
    ctx = Context(grid, device=0, ssc=False)
    p = prm.copy()
    p["pp_on"] = 1  # pair production needs SSC (microphysics_base.h:394-397)
    with pytest.raises(PbagError) as ei:
        ctx.run(recs, off, p)
    assert ei.value.code == abi.PBAG_ERR_PARAM
    p = prm.copy()
    p["ssc_on"] = 1  # context built without SSC tables
    with pytest.raises(PbagError) as ei:
        ctx.run(recs, off, p)
    assert ei.value.code == abi.PBAG_ERR_ARG


@pytest.mark.parametrize("method", [abi.PBAG_SYN_CSYN, abi.PBAG_SYN_DER09, abi.PBAG_SYN_GSL, abi.PBAG_SYN_BESSEL])
def test_tensor_core_synchrotron_sums_match_cuda_core_sums(lib, cuda_device, monkeypatch, method):
    """The synchrotron and SSA sums as a GEMM against the shifted kernel bank
    (tensor cores, split BF16) against the CUDA-core sums on the same batch:
    the synchrotron and SSA histories agree to far below the plain-path bar."""
    recs, off, prm, grid = cases.tophat(lib, nsteps=120, ssa=True, syn_method=method)
    outs = ("syn_j_all", "syn_a_all", "j_all", "a_all")
    monkeypatch.setenv("PBAG_SYN_TC", "1")
    ctx = Context(grid, device=0, ssc=False)
    tc = ctx.run(recs, off, prm, outputs=outs)
    ctx.close()
    monkeypatch.setenv("PBAG_SYN_TC", "0")
    ctx = Context(grid, device=0, ssc=False)
    cc = ctx.run(recs, off, prm, outputs=outs)
    ctx.close()
    for k in outs:
        rel, zm = rel_l2_rows(tc[k], cc[k])
        assert zm == 0 and rel.max() <= 2e-5, (k, rel.max())


def test_field_outside_synchrotron_bank_falls_back(lib, oracle, cuda_device, monkeypatch):
    """A magnetic field outside the range the tensor-core bank covers
    (1e-12..1e12 G) sends the whole batch to the CUDA-core sums; the result
    still matches the oracle."""
    monkeypatch.setenv("PBAG_SYN_TC", "1")
    recs, off, prm, grid = cases.tophat(lib, nsteps=40, ssa=True)
    recs = recs.copy()
    recs["B"][20:] *= 1e-14
    _compare(lib, oracle, (recs, off, prm, grid), outputs=cases.TOTALS)


def test_uneven_batch_tensor_core_sums(lib, oracle, cuda_device, monkeypatch):
    """The uneven batch with the synchrotron / SSA sums on the tensor cores
    (the path large batches take), every history against the oracle."""
    monkeypatch.setenv("PBAG_SYN_TC", "1")
    _compare(lib, oracle, cases.uneven(lib))
