"""Generate the golden fixtures of tests/golden/ from the REFERENCE's own code.

Runs here, where the reference sources are present: oracle/Makefile compiles
the reference's src/microphysics headers into oracle/_ref/libpbaref.so, and
this script drives them on seeded inputs and stores inputs and outputs
(float64, compressed npz). The GPU machine has no reference; its tests read these
files.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from pyblastafterglowmag_gb300 import _lib, abi, build  # noqa: E402
import pyoracle  # noqa: E402
import cases  # noqa: E402


def grid_arr(g):
    return np.array([g.ngam, g.nfreq, g.gam1, g.gam2, g.freq1, g.freq2])


def save(name, **kw):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **kw)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    build.build()
    ref = pyoracle.Reference()

    # grids of both jet configurations
    from pyblastafterglowmag_gb300 import histories as H
    out = {}
    for tag, cfg in (("tophat", H.config_tophat_fs()), ("gauss", H.config_gaussian_ssc())):
        g = cfg.grid()
        gam, freq = ref.grids(g)
        out[f"{tag}_grid"] = grid_arr(g)
        out[f"{tag}_gam"] = gam
        out[f"{tag}_freq"] = freq
    save("grids.npz", **out)

    # synchrotron kernel values, every method, a few fields, on a small grid
    g = abi.GridDesc(40, 24, 1.0, 1e9, 1e8, 1e29)
    gam, freq = ref.grids(g)
    out = {"grid": grid_arr(g), "gam": gam, "freq": freq, "B": np.array([1e-5, 3e-2, 1.0, 40.0])}
    for m, name in ((abi.PBAG_SYN_CSYN, "csyn"), (abi.PBAG_SYN_DER09, "der09"), (abi.PBAG_SYN_GSL, "gsl"),
                    (abi.PBAG_SYN_BESSEL, "bessel")):
        out[name] = np.stack([ref.syn_kernel(m, B, gam, freq[:-1]) for B in out["B"]])
    save("syn_kernel.npz", **out)

    # SSC kernel and its integral on a small grid
    g = abi.GridDesc(24, 16, 1.0, 1e9, 1e8, 1e29)
    gam, freq = ref.grids(g)
    K, Kint = ref.ssc_kernel(gam, freq[:-1])
    save("ssc_kernel.npz", grid=grid_arr(g), gam=gam, freq=freq, K=K, Kint=Kint)

    # per-step shock scalars for sequences of shock states and option sets
    rng = np.random.default_rng(11)
    n = 64
    st = np.zeros(n, dtype=abi.SHOCK_STATE_DTYPE)
    G = 10 ** rng.uniform(0.0005, 2.7, n)
    st["Gamma"] = G
    st["GammaSh"] = G * rng.uniform(0.9, 1.1, n).clip(min=1.0)
    st["n_prime"] = 10 ** rng.uniform(-4, 3, n)
    st["e_prime"] = (G - 1) * st["n_prime"] * 1.6726e-24 * 2.99792458e10 ** 2 * rng.uniform(0.5, 2, n)
    st["t_e"] = 10 ** rng.uniform(0, 8, n)
    st["t_b"] = st["t_e"] * 10
    st["tcomov"] = 10 ** rng.uniform(0, 9, n)
    st["n_protons"] = 10 ** rng.uniform(40, 52, n)
    g = abi.GridDesc(201, 128, 1.0, 1e9, 1e8, 1e29)
    combos = []
    for gm in (0, 1, 2, 3, 4):
        for nr in (0, 1, 2, 3):
            combos.append((gm, 0, 0, 0, nr, 2.3))
    combos += [(0, 1, 0, 0, 0, 2.2), (0, 0, 1, 1, 0, 2.5), (1, 0, 0, 2, 0, 2.0), (0, 0, 0, 0, 0, 2.05)]
    res, opts_arr = [], []
    for (gm, gc, gx, bm, nr, p) in combos:
        o = abi.LimitsOpts()
        o.p, o.eps_e, o.eps_b, o.eps_t = p, 0.1, 1e-3, 0.5
        o.beta_min, o.mu, o.mu_e = 1e-5, 0.62, 1.18
        o.method_B, o.method_gamma_min, o.method_gamma_c = bm, gm, gc
        o.method_gamma_max, o.method_nonrel, o.ele_analytic = gx, nr, 0
        res.append(ref.ele_limits(g, o, st))
        opts_arr.append([gm, gc, gx, bm, nr, p])
    save("shock_limits.npz", grid=grid_arr(g), states=st, opts=np.array(opts_arr), out=np.stack(res))

    # full histories: the top-hat (synchrotron) and a two-layer Gaussian (SSC + SSA)
    for name, batch, outputs in (
            ("run_tophat.npz", cases.tophat(_lib, nsteps=150, ssa=True), cases.ALL_OUTPUTS),
            ("run_gauss.npz", cases.gaussian(_lib, nlayers=2, nsteps=60, ngam=96, nfreq=64), cases.ALL_OUTPUTS)):
        recs, off, prm, grid = batch
        o = ref.run(grid, recs, off, prm, outputs=outputs)
        save(name, grid=grid_arr(grid), recs=recs, offsets=off, params=prm, **o)


if __name__ == "__main__":
    main()
