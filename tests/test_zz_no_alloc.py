"""pbag_run_batch_noalloc: the step for callers that cannot allocate device
memory while they run it (hosts that hand out device memory only from their
own pool, latency-critical loops). It keeps all intermediates in a fixed array
inside the library, so it must give the same histories as
pbag_run_batch_device on the same device buffers (within the plain-path
tolerance: its SSC contraction is the FP32 CUDA-core one), call after call,
and must reject a batch that does not fit.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300._lib import Context
import cases
from conftest import rel_l2_rows

pytestmark = pytest.mark.gpu
TOL = 1e-4  # the plain-path tolerance of the parity tests
OUTS = ("j_all", "a_all", "f_all", "i_all", "ele_f_all", "gdot_ssc_all", "syn_j_all", "syn_a_all", "ssc_j_all")


def _bind(so):
    so.pbag_run_batch_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int64), C.c_void_p,
                                          C.POINTER(abi.Outputs), C.POINTER(abi.Status)]
    so.pbag_run_batch_noalloc.restype = C.c_int
    return so.pbag_run_batch_noalloc


def _outputs(torch, grid, nrec, fill):
    bufs = {}
    for k in OUTS:
        n = grid.ngam if k in abi.OUTPUT_ON_GAMMA else grid.nfreq
        bufs[k] = torch.full((nrec, n), fill, dtype=torch.float64, device="cuda")
    out = abi.Outputs()
    for k in abi.OUTPUT_FIELDS:
        setattr(out, k, C.cast(C.c_void_p(bufs[k].data_ptr()), C.POINTER(C.c_double)) if k in bufs
                else C.POINTER(C.c_double)())
    return bufs, out


def test_noalloc_matches_device_entry_point_twice(lib, cuda_device):
    torch = pytest.importorskip("torch")
    so = lib.load()
    noalloc = _bind(so)
    recs, off, prm, grid = cases.gaussian(lib, nlayers=2, nsteps=80)
    ctx = Context(grid, device=0, ssc=True)
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    d_prm = torch.from_numpy(prm.view(np.uint8).copy()).cuda()
    off = np.ascontiguousarray(off, dtype=np.int64)
    nrec = int(off[-1])

    ref_bufs, _ = _outputs(torch, grid, nrec, 0.0)
    ctx.run_device(d_prm.data_ptr(), len(prm), off, d_recs.data_ptr(), {k: v.data_ptr() for k, v in ref_bufs.items()})
    ref = {k: v.cpu().numpy() for k, v in ref_bufs.items()}

    free_before = None
    for call in range(2):
        bufs, out = _outputs(torch, grid, nrec, float("nan"))  # every row must be written
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        st = abi.Status()
        rc = noalloc(ctx.handle, C.c_void_p(d_prm.data_ptr()), len(prm), off.ctypes.data_as(C.POINTER(C.c_int64)),
                     C.c_void_p(d_recs.data_ptr()), C.byref(out), C.byref(st))
        assert rc == abi.PBAG_OK, (rc, st.bw, st.step, st.site)
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "the call allocated device memory"
        # preparation (3), evolve + radiation per step, the last completion, the failure scan
        max_len = int((off[1:] - off[:-1]).max())
        assert ctx.last_launch_count() == 3 + 2 * max_len + 1 + 1
        got = {k: v.cpu().numpy() for k, v in bufs.items()}
        for k in OUTS:
            assert np.isfinite(got[k]).all(), k
            rel, zm = rel_l2_rows(got[k], ref[k])
            assert zm == 0 and rel.max() <= TOL, (call, k, rel.max())
    ctx.close()


def test_noalloc_rejects_batch_beyond_scratch(lib, cuda_device):
    torch = pytest.importorskip("torch")
    noalloc = _bind(lib.load())
    recs, off, prm, grid = cases.gaussian(lib, nlayers=1, nsteps=4)
    ctx = Context(grid, device=0, ssc=True)
    nbw = 4000  # ~17 KiB of state each: far beyond 16 MiB
    prm_big = np.repeat(prm[:1], nbw)
    d_prm = torch.from_numpy(prm_big.view(np.uint8).copy()).cuda()
    d_recs = torch.from_numpy(recs.view(np.uint8).copy()).cuda()
    off_big = np.zeros(nbw + 1, dtype=np.int64)  # empty histories
    _, out = _outputs(torch, grid, 1, 0.0)
    st = abi.Status()
    rc = noalloc(ctx.handle, C.c_void_p(d_prm.data_ptr()), nbw, off_big.ctypes.data_as(C.POINTER(C.c_int64)),
                 C.c_void_p(d_recs.data_ptr()), C.byref(out), C.byref(st))
    assert rc == abi.PBAG_ERR_ARG
    assert st.site * 1024 > (16 << 20)  # the KiB the batch would need
    ctx.close()
