"""The SSC contraction paths against the FP64 oracle: FP32 CUDA cores and the
tcgen05 tensor-core kernel with split-BF16 operands must both meet the plain
path's 1e-4 (per-row relative L2); plain BF16 operands are a precision study
and must stay within 1e-2. A batch of more than 128 blastwaves exercises
several tensor-core row tiles."""
import os

import numpy as np
import pytest

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300._lib import Context
import cases
from conftest import rel_l2_rows

pytestmark = pytest.mark.gpu
NTH = os.cpu_count() or 1
OUTS = ("j_all", "f_all", "ssc_j_all", "gdot_ssc_all", "ele_f_all")


def _check(got, ref, tol):
    worst = {}
    for k in OUTS:
        rel, zm = rel_l2_rows(got[k], ref[k])
        assert zm == 0, k
        worst[k] = float(rel.max())
        assert rel.max() <= tol, (k, rel.max())
    return worst


@pytest.mark.parametrize("path,tol", [(abi.PBAG_SSC_CUDA_FP32, 1e-4), (abi.PBAG_SSC_TC_SPLIT_BF16, 1e-4),
                                      (abi.PBAG_SSC_TC_BF16, 1e-2)])
def test_ssc_path_against_oracle(lib, oracle, cuda_device, path, tol):
    recs, off, prm, grid = cases.gaussian(lib, nlayers=2, nsteps=110)
    rc, where, ref = oracle.run(grid, recs, off, prm, outputs=OUTS, outer_threads=NTH)
    assert rc == 0, where
    ctx = Context(grid, device=0, ssc=True)
    ctx.set_ssc_path(path)
    _check(ctx.run(recs, off, prm, outputs=OUTS), ref, tol)
    ctx.close()


def test_tensor_core_many_row_tiles(lib, oracle, cuda_device):
    recs, off, prm, grid = cases.H.sweep_batch(lib, 4, seed=12, min_steps=12, max_steps=24, max_layers=41)
    assert len(prm) > 128
    rc, where, ref = oracle.run(grid, recs, off, prm, outputs=OUTS, outer_threads=NTH)
    assert rc == 0, where
    ctx = Context(grid, device=0, ssc=True)
    ctx.set_ssc_path(abi.PBAG_SSC_TC_SPLIT_BF16)
    _check(ctx.run(recs, off, prm, outputs=OUTS), ref, 1e-4)
    ctx.close()
