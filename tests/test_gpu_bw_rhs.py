"""pbag_bw_rhs_device (one thread per blastwave state) against the reference's
own right-hand-side evaluations (tests/golden/refdrv_*.npz, see
test_bw_rhs.py) and against the host entry on the same inputs. The device's
FP64 pow, exp, sin and asin differ from the host library's in the last bits,
so the bar is relative 1e-10 per written entry (1e-9 for the reverse-shock
terms the reference carries in long double), and the carried microphysics
members must agree to the same bar."""
import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300._lib import Context, PbagError, bw_rhs, bw_rhs_device
import refdrv_cases
from test_bw_rhs import compare, rhs_samples

pytestmark = pytest.mark.gpu

TOL = {abi.PBAG_BW_FS: 1e-10, abi.PBAG_BW_FSRS: 1e-9, "carry": 1e-10}


def _device(ctx, P, B, D0=None):
    import torch
    dev = torch.device("cuda", 0)
    d_p = torch.from_numpy(np.ascontiguousarray(P).view(np.uint8).copy()).to(dev)
    d_s = torch.from_numpy(np.ascontiguousarray(B).view(np.uint8).copy()).to(dev)
    d_y = torch.zeros((len(P), abi.PBAG_Y_N), dtype=torch.float64, device=dev)
    if D0 is not None:
        d_y.copy_(torch.from_numpy(D0))
    bw_rhs_device(ctx, len(P), d_p.data_ptr(), d_s.data_ptr(), d_y.data_ptr())
    after = d_s.cpu().numpy().view(abi.BW_RHS_STATE_DTYPE).reshape(-1)
    return d_y.cpu().numpy(), after


@pytest.mark.parametrize("name", refdrv_cases.CASES)
def test_gpu_rhs_matches_reference_evaluations(lib, cuda_device, name):
    P, B, A, D = rhs_samples(name)
    ctx = Context(refdrv_cases.Runs()[name].grid, device=0, ssc=False)
    got, after = _device(ctx, P, B)
    ctx.close()
    for (t, q), w in compare(P, A, D, got, after).items():
        assert w <= TOL[t], (name, t, q, w)


def test_gpu_rhs_many_states_match_host(lib, cuda_device):
    """A large batch (the jet's samples repeated to 200 000 states, the
    blastwaves' states perturbed): device against host entry by entry."""
    P, B, A, D = rhs_samples("gaussian")
    rng = np.random.default_rng(7)
    idx = rng.integers(0, len(P), 200_000)
    P2, B2 = P[idx].copy(), B[idx].copy()
    for q in ("R", "Gamma", "Eint2", "M2"):
        k = abi.BW_Q.index(q)
        B2["Y"][:, k] *= 1.0 + 1e-3 * rng.standard_normal(len(idx))
    B2["Y"][:, abi.BW_Q.index("Gamma")] = np.maximum(B2["Y"][:, abi.BW_Q.index("Gamma")], 1.0 + 1e-6)
    ref, ref_after = bw_rhs(P2, B2)
    ctx = Context(refdrv_cases.Runs()["gaussian"].grid, device=0, ssc=False)
    got, after = _device(ctx, P2, B2)
    ctx.close()
    for (t, q), w in compare(P2, ref_after, ref, got, after).items():
        assert w <= TOL[t], (t, q, w)


def test_gpu_rhs_reports_first_failure(lib, cuda_device):
    P, B, A, D = rhs_samples("tophat")
    p, b = P[:300].copy(), B[:300].copy()
    b["Y"][[120, 250], abi.BW_Q.index("Gamma")] = 0.5
    ctx = Context(refdrv_cases.Runs()["tophat"].grid, device=0, ssc=False)
    with pytest.raises(PbagError) as ei:
        _device(ctx, p, b)
    ctx.close()
    assert ei.value.code == abi.PBAG_ERR_NONFINITE and ei.value.bw == 120 and ei.value.site == 1
