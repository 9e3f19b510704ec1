"""Small seeded parity cases shared by the CPU and GPU tests."""
import numpy as np

from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300 import histories as H

ALL_OUTPUTS = tuple(abi.OUTPUT_FIELDS)
TOTALS = ("j_all", "a_all", "f_all", "i_all")


def tophat(lib, nsteps=200, ssa=False, syn_method=abi.PBAG_SYN_CSYN, ele_method=abi.PBAG_ELE_NUMERIC):
    cfg = H.config_tophat_fs()
    cfg.fs.ssa = ssa
    cfg.fs.syn_method = syn_method
    cfg.fs.ele_method = ele_method
    return H.make_batch(lib, cfg, nsteps=nsteps)


def gaussian(lib, nlayers=3, nsteps=120, ssa=True, ssc=True, ngam=201, nfreq=128):
    cfg = H.config_gaussian_ssc()
    cfg.nlayers = nlayers
    cfg.ngam, cfg.nfreq = ngam, nfreq
    for sh in (cfg.fs, cfg.rs):
        sh.ssa, sh.ssc = ssa, ssc
    return H.make_batch(lib, cfg, nsteps=nsteps)


def gaussian_window(lib, start, nsteps, nlayers=2):
    """Steps [start, start+nsteps) of the Gaussian jet, re-initialised at
    `start` (the later, non-relativistic and analytic-fallback regimes)."""
    recs, off, prm, grid = gaussian(lib, nlayers=nlayers, nsteps=start + nsteps)
    out, lens = [], []
    for b in range(len(prm)):
        r = recs[off[b] + start: off[b + 1]].copy()
        out.append(r)
        lens.append(len(r))
    offsets = np.zeros(len(lens) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(lens)
    return np.concatenate(out), offsets, prm, grid


def uneven(lib, nsets=3, seed=7):
    return H.sweep_batch(lib, nsets, seed=seed, min_steps=20, max_steps=90, max_layers=3)


_JET = {}


def gaussian_jet(lib):
    """The full 21-layer Gaussian jet: 42 blastwaves (forward + reverse
    shocks) x 1000 burster times, 201 gamma x 128 nu, synchrotron + SSA + SSC
    (the benchmarked workload). Built once per process."""
    if "jet" not in _JET:
        _JET["jet"] = H.make_batch(lib, H.config_gaussian_ssc())
    return _JET["jet"]


def tophat_full(lib):
    """One top-hat forward shock over all 1000 burster times, 151 gamma x 96
    nu, synchrotron only."""
    return H.make_batch(lib, H.config_tophat_fs())


def jet_window(lib, bws, start, nsteps):
    """Blastwaves `bws` of the full Gaussian jet, steps [start, start+nsteps),
    re-initialised at `start`. Steps 280-420 of the core layer's forward shock
    run the Chang-Cooper substeps with 2 to 95 substeps per step (the scan
    paths), steps 400-470 with 96 or more (the systolic path)."""
    recs, off, prm, grid = gaussian_jet(lib)
    out, lens = [], []
    for b in bws:
        r = recs[off[b] + start: min(off[b] + start + nsteps, off[b + 1])].copy()
        out.append(r)
        lens.append(len(r))
    offsets = np.zeros(len(lens) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(lens)
    return np.concatenate(out), offsets, prm[list(bws)].copy(), grid
