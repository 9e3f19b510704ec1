"""Programmatic dependent launch of the captured step loop (each evolve
launch scheduled while the previous step's radiation kernels run, reading
the blastwave state only after griddepcontrol.wait) changes when the
kernels run, never what they compute: the reference program's 21-layer
Gaussian jet (forward and reverse shocks, synchrotron, SSC, SSA; 42
blastwaves, one CTA per SM, so every evolve launch takes the programmatic
edge) gives bit-identical histories with PBAG_PDL=0 (plain graph edges) and
by default, on the first pass (graph capture) and on a replay. The switch is
read once per process, so each setting runs in its own."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import os, sys
import numpy as np
import torch
root = os.getcwd()
sys.path.insert(0, root)
sys.path.insert(0, os.path.join(root, "tests"))
from pyblastafterglowmag_gb300 import _lib
import refdrv_cases
run = refdrv_cases.Runs()["gaussian"]
recs, off, prm = run.records(_lib)
dev = torch.device("cuda", 0)
ctx = _lib.Context(run.grid, device=0, ssc=True)
d_recs = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
d_prm = torch.from_numpy(prm.view(np.uint8).copy()).to(dev)
keys = ("j_all", "a_all", "f_all", "i_all")
res = {}
for rep in range(2):
    d_out = {k: torch.zeros((int(off[-1]), run.grid.nfreq), dtype=torch.float64, device=dev) for k in keys}
    ctx.run_device(d_prm.data_ptr(), len(prm), off, d_recs.data_ptr(), {k: v.data_ptr() for k, v in d_out.items()})
    torch.cuda.synchronize()
    res.update({f"{k}_{rep}": v.cpu().numpy() for k, v in d_out.items()})
ctx.close()
np.savez(sys.argv[1], **res)
"""


def test_pdl_outputs_bit_identical(lib, cuda_device, tmp_path):
    outs = []
    for pdl in ("0", "1"):
        path = tmp_path / f"pdl{pdl}.npz"
        env = dict(os.environ, PBAG_PDL=pdl)
        r = subprocess.run([sys.executable, "-c", SCRIPT, str(path)], cwd=ROOT, env=env, capture_output=True,
                           text=True, timeout=900)
        assert r.returncode == 0, r.stderr[-3000:]
        outs.append(np.load(path))
    plain, pdl = outs
    assert set(plain.files) == set(pdl.files) and len(plain.files) == 8
    for k in plain.files:
        assert np.any(plain[k] != 0.), k
        assert np.array_equal(plain[k], pdl[k]), k
