"""The SSC surrogate: exact band projections against the FP64 oracle, a
trained network against the method without it (in each band the baseline shape
matched to the band's exact power and first moment), the error estimate and
exact fallback, and the surrogate inside the step (tolerance 0: every state
recomputed exactly, so the step's histories must match the oracle)."""
import os

import numpy as np
import pytest

import cases
from conftest import rel_l2_rows
from pyblastafterglowmag_gb300 import abi
from pyblastafterglowmag_gb300 import contraction as CT

pytestmark = pytest.mark.gpu


def test_band_projections_match_oracle(lib, oracle, cuda_device):
    import torch
    from pyblastafterglowmag_gb300 import surrogate as SG
    g = CT.grid_desc(ngam=201, nfreq=128)
    gam, freq = oracle.grids(g)
    f, B = CT.states(gam, 40, seed=6)
    threads = os.cpu_count() or 1
    jsyn, _ = oracle.contract(g, f, B=B, ssc=False, threads=threads)
    nph = CT.seed_photons(jsyn, freq)
    _, jssc = oracle.contract(g, f, B=B, nph=nph, syn=False, threads=threads)
    ctx = lib.Context(g, cuda_device, ssc=True)
    SG.configure(ctx)
    dev = torch.device("cuda", cuda_device)
    d_f, d_B, d_n = (torch.from_numpy(a).to(dev) for a in (f, B, nph))
    d_x = torch.zeros((40, SG.NIN), dtype=torch.float32, device=dev)
    d_p = torch.zeros((40, SG.NPROJ), dtype=torch.float64, device=dev)
    d_b = torch.zeros((40, 128), dtype=torch.float32, device=dev)
    SG.features(ctx, 40, d_f.data_ptr(), d_B.data_ptr(), d_n.data_ptr(), d_x.data_ptr(), d_p.data_ptr(), d_b.data_ptr())
    proj = d_p.cpu().numpy()
    per = 128 // SG.NB
    dnu = np.diff(freq)[:128]
    lnu = np.log(freq[:128])
    P = (jssc * dnu).reshape(40, SG.NB, per).sum(axis=2)
    c = lnu.reshape(SG.NB, per).mean(axis=1)
    x = lnu - np.repeat(c, per)
    Q = (jssc * dnu * x).reshape(40, SG.NB, per).sum(axis=2)
    R = (jssc * dnu * x * x).reshape(40, SG.NB, per).sum(axis=2)
    rel_p = np.abs(proj[:, :SG.NB] - P) / np.maximum(P, 1e-300)
    assert rel_p[P > 1e-6 * P.max(axis=1, keepdims=True)].max() <= 1e-4
    # log moments: against the band power times the band half width
    hw = 0.5 * (lnu.reshape(SG.NB, per)[:, -1] - lnu.reshape(SG.NB, per)[:, 0])
    big = P > 1e-6 * P.max(axis=1, keepdims=True)
    rel_q = np.abs(proj[:, SG.NB:2 * SG.NB] - Q) / np.maximum(P * hw, 1e-300)
    assert rel_q[big].max() <= 1e-4
    rel_r = np.abs(proj[:, 2 * SG.NB:] - R) / np.maximum(P * hw * hw, 1e-300)
    assert rel_r[big].max() <= 1e-4
    assert np.isfinite(d_x.cpu().numpy()).all()
    # the baseline shares of a band sum to one and match its exact first moment
    base = d_b.cpu().numpy().astype(np.float64).reshape(40, SG.NB, per)
    sh = 10.0 ** base
    np.testing.assert_allclose(sh.sum(axis=2), 1.0, rtol=1e-4)
    mu = (sh * x.reshape(SG.NB, per)[None]).sum(axis=2)
    inside = big & (np.abs(Q / np.maximum(P, 1e-300)) < 0.95 * hw[None, :])
    assert np.abs(mu - Q / np.maximum(P, 1e-300))[inside].max() <= 1e-3 * hw.max()


@pytest.fixture(scope="module")
def trained(lib, cuda_device):
    import torch
    from pyblastafterglowmag_gb300 import surrogate as SG
    from pyblastafterglowmag_gb300 import histories as H
    g = H.config_gaussian_ssc().grid()
    ctx = lib.Context(g, cuda_device, ssc=True)
    SG.configure(ctx)
    _, freq = lib.grids(g)
    f, B, nph = SG.sweep_states(ctx, g, nsets=6, seed=5, workers=os.cpu_count() or 1, device=cuda_device,
                                max_states=40000)
    n = f.shape[0]
    dev = f.device
    X = torch.zeros((n, SG.NIN), dtype=torch.float32, device=dev)
    proj = torch.zeros((n, SG.NPROJ), dtype=torch.float64, device=dev)
    base = torch.zeros((n, g.nfreq), dtype=torch.float32, device=dev)
    SG.features(ctx, n, f.data_ptr(), B.data_ptr(), nph.data_ptr(), X.data_ptr(), proj.data_ptr(), base.data_ptr())
    jex = SG.exact_ssc(ctx, f, B, nph)
    T, M = SG.make_targets(jex, proj, freq, base)
    ntr = int(0.85 * n)
    tr = SG.Trainer(g.nfreq, cuda_device, seed=0)
    Xs = tr.standardise(X.clone())
    tr.fit(Xs[:ntr], T[:ntr], M[:ntr], epochs=20, batch=1024, lr=2e-3)
    SG.configure(ctx, tr.net, tr.mean, tr.std, tol=1e30)
    va = slice(ntr, n)
    return dict(ctx=ctx, trainer=tr, f=f[va].contiguous(), B=B[va].contiguous(), nph=nph[va].contiguous(),
                jex=jex[va].contiguous(), proj=proj[va].contiguous(), base=base[va].contiguous(), freq=freq, grid=g)


def test_network_gains_over_band_baseline(trained):
    import torch
    from pyblastafterglowmag_gb300 import surrogate as SG
    d = trained
    n = d["f"].shape[0]
    j = torch.zeros_like(d["jex"])
    SG.contract(d["ctx"], n, d["f"].data_ptr(), d["B"].data_ptr(), d["nph"].data_ptr(), j.data_ptr())
    err_net = SG.rel_l2(j, d["jex"])
    err_base = SG.rel_l2(SG.band_baseline(d["proj"], d["freq"], d["base"]), d["jex"])
    med_net, med_base = float(err_net.median()), float(err_base.median())
    print(f"surrogate rel-L2 median {med_net:.4f} p90 {float(err_net.quantile(0.9)):.4f}; "
          f"baseline median {med_base:.4f}")
    assert med_net < 0.5 * med_base, (med_net, med_base)
    assert med_net < 0.06


def test_error_estimate_and_fallback(trained):
    import torch
    from pyblastafterglowmag_gb300 import surrogate as SG
    d = trained
    n = d["f"].shape[0]
    tol = 0.01
    SG.configure(d["ctx"], d["trainer"].net, d["trainer"].mean, d["trainer"].std, tol=tol)
    j = torch.zeros_like(d["jex"])
    est = torch.zeros(n, dtype=torch.float32, device=j.device)
    nfb = SG.contract(d["ctx"], n, d["f"].data_ptr(), d["B"].data_ptr(), d["nph"].data_ptr(), j.data_ptr(),
                      est.data_ptr())
    back = est > tol
    assert nfb == int(back.sum())
    err = SG.rel_l2(j, d["jex"])
    # recomputed states are exact
    assert float(err[back].max() if back.any() else 0.0) <= 1e-6
    SG.configure(d["ctx"], d["trainer"].net, d["trainer"].mean, d["trainer"].std, tol=1e30)


def test_step_with_surrogate_at_zero_tolerance_matches_oracle(lib, oracle, cuda_device, trained):
    from pyblastafterglowmag_gb300 import surrogate as SG
    recs, off, prm, grid = cases.gaussian(lib, nlayers=2, nsteps=80)
    ctx = lib.Context(grid, cuda_device, ssc=True)
    SG.configure(ctx, trained["trainer"].net, trained["trainer"].mean, trained["trainer"].std, tol=0.0)
    ctx.set_ssc_path(abi.PBAG_SSC_SURROGATE)
    out = ctx.run(recs, off, prm, outputs=cases.TOTALS)
    rc, where, ref = oracle.run(grid, recs, off, prm, outputs=cases.TOTALS)
    assert rc == 0
    for k in cases.TOTALS:
        rel, zero_mismatch = rel_l2_rows(out[k], ref[k])
        assert zero_mismatch == 0 and rel.max() <= 1e-4, (k, rel.max())
