"""The FP64 contraction restatement (orc_contract) against the oracle's full
step, which is bit-exact against the reference: at every radiating step of a
blastwave, j_syn and j_ssc of (N(gamma) after the step, B of the step, photon
field of the previous radiating step) times accel_frac are the dense
syn_j_all / ssc_j_all rows (numeric_model.h:148-184, 247-285;
microphysics.h:602-633)."""
import numpy as np

import cases
from pyblastafterglowmag_gb300 import abi


def test_contract_matches_step(lib, oracle):
    recs, off, prm, grid = cases.gaussian(lib, nlayers=1, nsteps=80)
    rc, where, out = oracle.run(grid, recs, off, prm, outputs=cases.ALL_OUTPUTS)
    assert rc == 0, where
    checked = 0
    for b in range(len(prm)):
        nprev = np.zeros(grid.nfreq)
        for r in range(off[b], off[b + 1]):
            if recs["mode"][r] == 0 or not out["ele_f_all"][r].any():
                continue
            f = out["ele_f_all"][r][None, :]
            jsyn, jssc = oracle.contract(grid, f, B=[recs["B"][r]], nph=nprev[None, :],
                                         syn_method=int(prm["syn_method"][b]))
            acc = recs["accel_frac"][r]
            np.testing.assert_allclose(jsyn[0] * acc, out["syn_j_all"][r], rtol=1e-12, atol=0)
            np.testing.assert_allclose(jssc[0] * acc, out["ssc_j_all"][r], rtol=1e-12, atol=0)
            nprev = out["f_all"][r]
            checked += 1
    assert checked > 20


def test_contract_states_are_finite(oracle):
    from pyblastafterglowmag_gb300 import contraction as CT
    g = CT.grid_desc(ngam=64, nfreq=48)
    gam, freq = oracle.grids(g)
    f, B = CT.states(gam, 6)
    jsyn, _ = oracle.contract(g, f, B=B, ssc=False)
    assert np.isfinite(jsyn).all() and (jsyn >= 0).all() and (jsyn[:, :-1] > 0).any()
    nph = CT.seed_photons(jsyn, freq)
    _, jssc = oracle.contract(g, f, B=B, nph=nph, syn=False)
    assert np.isfinite(jssc).all() and (jssc >= 0).all() and (jssc > 0).any()
