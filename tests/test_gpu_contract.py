"""pbag_contract (emissivity contractions of a batch of states) against the
FP64 oracle, for every SSC precision: FP32 CUDA cores and split-BF16 at the
plain path's bar (rel-L2 <= 1e-4 per state), TF32 and plain BF16 at theirs."""
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300 import contraction as CT
from conftest import rel_l2_rows

pytestmark = pytest.mark.gpu

TOL = {abi.PBAG_PREC_FP32: 1e-4, abi.PBAG_PREC_SPLIT_BF16: 1e-4, abi.PBAG_PREC_TF32: 5e-3,
       abi.PBAG_PREC_BF16: 2e-2}


def _case(oracle, ngam, nfreq, n, seed):
    g = CT.grid_desc(ngam=ngam, nfreq=nfreq)
    gam, freq = oracle.grids(g)
    f, B = CT.states(gam, n, seed=seed)
    threads = os.cpu_count() or 1
    jsyn, _ = oracle.contract(g, f, B=B, ssc=False, threads=threads)
    nph = CT.seed_photons(jsyn, freq)
    _, jssc = oracle.contract(g, f, B=B, nph=nph, syn=False, threads=threads)
    return g, f, B, nph, jsyn, jssc


@pytest.mark.parametrize("ngam,nfreq,n", [(256, 256, 300), (201, 128, 70)])
def test_contract_precisions(lib, oracle, cuda_device, ngam, nfreq, n):
    import torch
    g, f, B, nph, jsyn_o, jssc_o = _case(oracle, ngam, nfreq, n, seed=4)
    ctx = lib.Context(g, cuda_device, ssc=True)
    dev = torch.device("cuda", cuda_device)
    d_f = torch.from_numpy(f).to(dev)
    d_B = torch.from_numpy(B).to(dev)
    d_n = torch.from_numpy(nph).to(dev)
    for prec, tol in TOL.items():
        d_js = torch.zeros((n, nfreq), dtype=torch.float64, device=dev)
        d_jc = torch.zeros((n, nfreq), dtype=torch.float64, device=dev)
        ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN, prec,
                            d_js.data_ptr(), d_jc.data_ptr())
        js, jc = d_js.cpu().numpy(), d_jc.cpu().numpy()
        rel_s, zs = rel_l2_rows(js, jsyn_o)
        rel_c, zc = rel_l2_rows(jc, jssc_o)
        name = abi.PRECISION_NAMES[prec]
        assert zs == 0 and zc == 0, name
        assert rel_s.max() <= 1e-4, (name, rel_s.max())
        assert rel_c.max() <= tol, (name, rel_c.max(), np.percentile(rel_c, 99))


def test_contract_edge_cases(lib, oracle, cuda_device):
    import torch
    g, f, B, nph, jsyn_o, jssc_o = _case(oracle, 64, 128, 5, seed=9)
    ctx = lib.Context(g, cuda_device, ssc=True)
    dev = torch.device("cuda", cuda_device)
    # empty batch
    ctx.contract_device(0, 0, 0, 0, abi.PBAG_SYN_CSYN, abi.PBAG_PREC_SPLIT_BF16, 0, 0)
    # synchrotron only (no photon field), SSC only (no field)
    d_f = torch.from_numpy(f).to(dev)
    d_B = torch.from_numpy(B).to(dev)
    d_n = torch.from_numpy(nph).to(dev)
    d_js = torch.zeros((5, 128), dtype=torch.float64, device=dev)
    d_jc = torch.zeros((5, 128), dtype=torch.float64, device=dev)
    ctx.contract_device(5, d_f.data_ptr(), d_B.data_ptr(), 0, abi.PBAG_SYN_CSYN, abi.PBAG_PREC_FP32,
                        d_js.data_ptr(), 0)
    assert rel_l2_rows(d_js.cpu().numpy(), jsyn_o)[0].max() <= 1e-4
    ctx.contract_device(5, d_f.data_ptr(), 0, d_n.data_ptr(), abi.PBAG_SYN_CSYN, abi.PBAG_PREC_SPLIT_BF16,
                        0, d_jc.data_ptr())
    assert rel_l2_rows(d_jc.cpu().numpy(), jssc_o)[0].max() <= 1e-4
    # a non-finite state is the reference's exit in computeSynSpectrum
    f_bad = f.copy()
    f_bad[3, 10] = np.nan
    d_fb = torch.from_numpy(f_bad).to(dev)
    with pytest.raises(lib.PbagError) as ei:
        ctx.contract_device(5, d_fb.data_ptr(), d_B.data_ptr(), 0, abi.PBAG_SYN_CSYN, abi.PBAG_PREC_FP32,
                            d_js.data_ptr(), 0)
    assert ei.value.code == abi.PBAG_ERR_NONFINITE and ei.value.bw == 3
    # tensor-core precisions need nfreq 128 or 256
    g2 = CT.grid_desc(ngam=64, nfreq=96)
    ctx2 = lib.Context(g2, cuda_device, ssc=True)
    d_f2 = torch.zeros((2, 64), dtype=torch.float64, device=dev)
    d_n2 = torch.zeros((2, 96), dtype=torch.float64, device=dev)
    d_jc2 = torch.zeros((2, 96), dtype=torch.float64, device=dev)
    with pytest.raises(lib.PbagError) as ei:
        ctx2.contract_device(2, d_f2.data_ptr(), 0, d_n2.data_ptr(), abi.PBAG_SYN_CSYN, abi.PBAG_PREC_TF32,
                             0, d_jc2.data_ptr())
    assert ei.value.code == abi.PBAG_ERR_UNSUPPORTED


def test_large_batch_runs_with_blastwaves_on_rows(lib, oracle, cuda_device):
    """Large batches (nfreq 128) run the SSC contraction with blastwaves on the
    accumulator rows, the W rows resident and the slabs streamed (or the
    slab-per-CTA kernel, whichever the autotuner measured faster): the plain
    path's bar, and the same values as a smaller batch of the same states."""
    import torch
    n = 2300
    g, f, B, nph, _, jssc_o = _case(oracle, 201, 128, n, seed=12)
    ctx = lib.Context(g, cuda_device, ssc=True)
    dev = torch.device("cuda", cuda_device)
    d_f = torch.from_numpy(f).to(dev)
    d_B = torch.from_numpy(B).to(dev)
    d_n = torch.from_numpy(nph).to(dev)
    for prec, tol in ((abi.PBAG_PREC_SPLIT_BF16, 1e-4), (abi.PBAG_PREC_BF16, 2e-2)):
        d_jc = torch.zeros((n, 128), dtype=torch.float64, device=dev)
        ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN, prec, 0,
                            d_jc.data_ptr())
        jc = d_jc.cpu().numpy()
        rel, z = rel_l2_rows(jc, jssc_o)
        assert z == 0 and rel.max() <= tol, (abi.PRECISION_NAMES[prec], rel.max())
        # the first 2000 states alone: another shape, tuned on its own
        m = 2000
        d_small = torch.zeros((m, 128), dtype=torch.float64, device=dev)
        ctx.contract_device(m, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN, prec, 0,
                            d_small.data_ptr())
        rel2, _ = rel_l2_rows(jc[:m], d_small.cpu().numpy())
        assert rel2.max() <= 1e-5, (abi.PRECISION_NAMES[prec], rel2.max())


def test_autotuner_measures_and_keeps_a_choice(lib, oracle, cuda_device):
    """The first contraction of a shape times the candidate kernels on its own
    data and keeps the fastest; the result stays at the plain path's bar."""
    import torch
    n = 3000
    g, f, B, nph, _, jssc_o = _case(oracle, 201, 128, n, seed=13)
    ctx = lib.Context(g, cuda_device, ssc=True)
    dev = torch.device("cuda", cuda_device)
    d_f, d_B, d_n = (torch.from_numpy(a).to(dev) for a in (f, B, nph))
    d_jc = torch.zeros((n, 128), dtype=torch.float64, device=dev)
    lib.autotune(True)
    ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN,
                        abi.PBAG_PREC_SPLIT_BF16, 0, d_jc.data_ptr())
    report = lib.autotune_report()
    line = [ln for ln in report.splitlines() if "F=128" in ln and "nout=128" in ln and "2^11" in ln]
    assert line and " ms" in line[0], report
    assert float(line[0].split()[-2]) > 0.0, report  # a measured time, not the untuned default
    rel, z = rel_l2_rows(d_jc.cpu().numpy(), jssc_o)
    assert z == 0 and rel.max() <= 1e-4


@pytest.mark.parametrize("n", [50, 700])
@pytest.mark.parametrize("method", [abi.PBAG_SYN_CSYN, abi.PBAG_SYN_DER09, abi.PBAG_SYN_GSL, abi.PBAG_SYN_BESSEL])
def test_contract_synchrotron_methods(lib, oracle, cuda_device, method, n):
    """Every synchrotron method, on a small batch (the kernel values of each
    term) and on a large one (the tabulated functions, interpolated)."""
    import torch
    g = CT.grid_desc(ngam=201, nfreq=128)
    gam, freq = oracle.grids(g)
    f, B = CT.states(gam, n, seed=14)
    jsyn_o, _ = oracle.contract(g, f, B=B, ssc=False, syn_method=method, threads=os.cpu_count() or 1)
    ctx = lib.Context(g, cuda_device, ssc=False)
    dev = torch.device("cuda", cuda_device)
    d_f, d_B = torch.from_numpy(f).to(dev), torch.from_numpy(B).to(dev)
    d_js = torch.zeros((n, 128), dtype=torch.float64, device=dev)
    ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), 0, method, abi.PBAG_PREC_FP32, d_js.data_ptr(), 0)
    rel, z = rel_l2_rows(d_js.cpu().numpy(), jsyn_o)
    assert z == 0 and rel.max() <= 1e-4, (method, rel.max())


@pytest.mark.parametrize("kernel", ["slab", "slab-small", "rows"])
def test_every_contraction_kernel_on_a_small_batch(lib, oracle, cuda_device, monkeypatch, kernel):
    """Each kernel the autotuner chooses from, forced on the same small batch
    (40 states, 201 x 128), split and plain BF16, against the oracle."""
    import torch
    monkeypatch.setenv("PBAG_TC_KERNEL", kernel)
    n = 40
    g, f, B, nph, _, jssc_o = _case(oracle, 201, 128, n, seed=15)
    ctx = lib.Context(g, cuda_device, ssc=True)
    dev = torch.device("cuda", cuda_device)
    d_f, d_B, d_n = (torch.from_numpy(a).to(dev) for a in (f, B, nph))
    for prec, tol in ((abi.PBAG_PREC_SPLIT_BF16, 1e-4), (abi.PBAG_PREC_BF16, 2e-2)):
        d_jc = torch.zeros((n, 128), dtype=torch.float64, device=dev)
        ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), abi.PBAG_SYN_CSYN, prec, 0,
                            d_jc.data_ptr())
        rel, z = rel_l2_rows(d_jc.cpu().numpy(), jssc_o)
        assert z == 0 and rel.max() <= tol, (kernel, abi.PRECISION_NAMES[prec], rel.max())


def test_contract_synchrotron_bank_on_256_grid(lib, oracle, cuda_device):
    """The contraction microbenchmark's grid (256 gamma x 256 nu): the
    synchrotron sums of a large batch through the tensor-core kernel bank,
    against the FP64 oracle."""
    import torch
    n = 640
    g = CT.grid_desc(ngam=256, nfreq=256)
    gam, freq = oracle.grids(g)
    f, B = CT.states(gam, n, seed=16)
    jsyn_o, _ = oracle.contract(g, f, B=B, ssc=False, threads=os.cpu_count() or 1)
    ctx = lib.Context(g, cuda_device, ssc=False)
    dev = torch.device("cuda", cuda_device)
    d_f, d_B = torch.from_numpy(f).to(dev), torch.from_numpy(B).to(dev)
    d_js = torch.zeros((n, 256), dtype=torch.float64, device=dev)
    ctx.contract_device(n, d_f.data_ptr(), d_B.data_ptr(), 0, abi.PBAG_SYN_CSYN, abi.PBAG_PREC_FP32, d_js.data_ptr(), 0)
    rel, z = rel_l2_rows(d_js.cpu().numpy(), jsyn_o)
    assert z == 0 and rel.max() <= 1e-4, rel.max()
    ctx.close()
