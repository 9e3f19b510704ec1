"""The drop-in ElectronAndRadiation (include/pbag_microphysics.hpp) driven
through the reference's own per-step call sequence by a C++ driver
(tests/cpp/microphysics_driver.cpp, which mirrors blastwave_radiation.h:
976-1182): it compiles with the host compiler on its own, the step records it
builds from the driver's calls are the bytes the batch generator builds, its
histories match the FP64 oracle at the plain-path tolerance, and its fluxDens
matches the oracle's restatement of fluxDens on those histories."""
import os
import subprocess

import numpy as np
import pytest

import cases
from conftest import rel_l2_rows
from pyblastafterglowmag_gb300 import abi, histories as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "microphysics_driver.cpp")
LIBDIR = os.path.join(ROOT, "pyblastafterglowmag_gb300")
ARRAYS = ("valid", "U_p", "Gamma", "GammaSh", "t_e", "t_b", "tcomov", "n_prime", "n_protons", "M2", "rho2", "R",
          "thickness", "dr")


# the fields of a record a step reads: an initialisation reads only the
# arguments of initializeElectronDistribution and the shock scalars
INIT_FIELDS = ("mode", "tc_p1", "m_p1", "rho_p1", "u_p_p1", "dr", "B", "gamma_min", "gamma_max", "gamma_c",
               "accel_frac", "n_prime")


def assert_same_records(got, ref):
    assert len(got) == len(ref)
    init = ref["mode"] == abi.PBAG_INIT
    evolve = ref["mode"] == abi.PBAG_EVOLVE
    assert (got["mode"] == ref["mode"]).all()  # skipped steps are read by nobody
    for k in abi.STEP_DTYPE.names:
        if k in ("mode", "reserved"):
            continue
        a, b = got[k], ref[k]
        rows = (init | evolve) if k in INIT_FIELDS else evolve
        assert a[rows].tobytes() == b[rows].tobytes(), k


def test_dropin_header_compiles():
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                    "-I" + os.path.join(ROOT, "include"), SRC], check=True)


def _driver_input(path, lib, cfg, nsteps, bws, queries):
    arrs = H.driver_arrays(lib, cfg, nsteps=nsteps)
    g = cfg.grid()
    sh = cfg.fs
    with open(path, "wb") as f:
        np.array([len(bws), nsteps], dtype=np.int32).tofile(f)
        np.array([g.ngam, g.nfreq, g.gam1, g.gam2, g.freq1, g.freq2], dtype=np.float64).tofile(f)
        np.array([sh.eps_e, sh.eps_b, sh.p, float(sh.ssa), float(sh.ssc), float(sh.max_substeps)]).tofile(f)
        for b in bws:
            is_rs, a = arrs[b]
            np.array([int(is_rs)], dtype=np.int32).tofile(f)
            for k in ARRAYS:
                np.ascontiguousarray(a[k], dtype=np.float64).tofile(f)
        np.array([len(queries)], dtype=np.int32).tofile(f)
        np.ascontiguousarray(queries, dtype=np.float64).tofile(f)
    return arrs


@pytest.mark.gpu
def test_dropin_follows_reference_call_sequence(lib, oracle, cuda_device, tmp_path):
    cfg = H.config_gaussian_ssc()
    nsteps = 1000
    bws = [0, 1, 2, 3]  # the two core layers, forward and reverse shocks (all solver paths)
    exe = tmp_path / "microphysics_driver"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-o", str(exe),
                    "-L" + LIBDIR, "-lpbag", "-Wl,-rpath," + LIBDIR], check=True)
    # fluxDens queries on the forward shock of the core layer: rows of valid
    # steps, frequencies inside the grid, the radius between the two rows
    recs, off, prm, grid = cases.gaussian_jet(lib)
    _, freq = lib.grids(grid)
    rng = np.random.default_rng(12)
    arrs = H.driver_arrays(lib, cfg, nsteps=nsteps)
    valid0 = np.nonzero(arrs[0][1]["valid"])[0]
    R0 = arrs[0][1]["R"]
    nq = 64
    q = np.zeros((nq, 16))
    ia = rng.choice(valid0[1:-2], nq)
    q[:, 0] = 0
    q[:, 1], q[:, 2] = ia, ia + 1
    q[:, 3] = 0.05                                          # theta
    q[:, 4] = 1.0                                           # ncells
    q[:, 5] = np.exp(rng.uniform(np.log(freq[2]), np.log(freq[grid.nfreq - 3]), nq))
    q[:, 6] = rng.uniform(1.5, 50.0, nq)                    # Gamma
    q[:, 7] = q[:, 6] * 1.2                                 # GammaSh
    q[:, 8] = 1.0
    q[:, 9] = rng.uniform(-0.9, 0.9, nq)                    # mu
    q[:, 10] = R0[ia] + rng.uniform(0, 1, nq) * (R0[ia + 1] - R0[ia])
    q[:, 13] = rng.uniform(1e-2, 10.0, nq)                  # n_prime
    q[:, 14] = rng.uniform(1e45, 1e50, nq)                  # ne
    _driver_input(tmp_path / "in.bin", lib, cfg, nsteps, bws, q)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(tmp_path / "out.bin", "rb").read()
    G, F = grid.ngam, grid.nfreq
    pos = 0
    got = {k: [] for k in abi.OUTPUT_FIELDS}
    got_recs = []
    for _ in bws:
        for k in abi.OUTPUT_FIELDS:
            n = nsteps * (G if k in abi.OUTPUT_ON_GAMMA else F)
            got[k].append(np.frombuffer(raw, dtype=np.float64, count=n, offset=pos).reshape(nsteps, -1))
            pos += 8 * n
        got_recs.append(np.frombuffer(raw, dtype=abi.STEP_DTYPE, count=nsteps, offset=pos))
        pos += abi.STEP_DTYPE.itemsize * nsteps
    flux = np.frombuffer(raw, dtype=np.float64, count=nq, offset=pos)
    # the records the drop-in built from the driver's calls are the batch generator's
    sub = np.concatenate([recs[off[b]:off[b + 1]] for b in bws])
    assert_same_records(np.concatenate(got_recs), sub)
    # histories against the oracle
    o = np.arange(len(bws) + 1, dtype=np.int64) * nsteps
    p = prm[bws].copy()
    rc, where, ref = oracle.run(grid, sub, o, p, outputs=cases.ALL_OUTPUTS, outer_threads=len(bws))
    assert rc == 0, (rc, where)
    for k in cases.ALL_OUTPUTS:
        g = np.concatenate(got[k])
        rel, zm = rel_l2_rows(g, ref[k])
        assert zm == 0 and rel.max() <= 1e-4, (k, rel.max())
    # fluxDens on the drop-in's own histories against the oracle's restatement
    qs = np.zeros(nq, dtype=abi.FLUX_QUERY_DTYPE)
    qs["bw"], qs["ia"], qs["ib"] = 0, q[:, 1].astype(np.int32), q[:, 2].astype(np.int32)
    for i, k in enumerate(("theta", "ncells", "freq", "Gamma", "GammaSh", "acc_fac", "mu", "r", "rsh", "dr",
                           "n_prime", "ne")):
        qs[k] = q[:, 3 + i]
    opts = abi.FluxOpts()
    opts.shock_vel, opts.method_ne, opts.method_tau = abi.PBAG_VEL_SAME_AS_BW, abi.PBAG_NE_USE_NE, abi.PBAG_TAU_SMOOTH
    R = np.ascontiguousarray(arrs[0][1]["R"])
    frc, fail, fref = oracle.flux_dens(grid, opts, np.array([0, nsteps], dtype=np.int64), got["j_all"][0],
                                       got["a_all"][0], R, qs)
    assert frc == 0, (frc, fail)
    np.testing.assert_allclose(flux, fref, rtol=1e-12, atol=0)


def test_dropin_records_equal_batch_records(lib, tmp_path):
    """Host side only: the records the drop-in builds from the driver's calls
    (shock scalars from its own computeEleSpectrumLimits) are byte for byte the
    batch generator's in every field a step reads, for every blastwave of the
    full jet. Without a GPU the
    closing flush fails, after the records have been written."""
    cfg = H.config_gaussian_ssc()
    nsteps = 1000
    bws = list(range(42))
    exe = tmp_path / "microphysics_driver"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-o", str(exe),
                    "-L" + LIBDIR, "-lpbag", "-Wl,-rpath," + LIBDIR], check=True)
    _driver_input(tmp_path / "in.bin", lib, cfg, nsteps, bws, np.zeros((0, 16)))
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode in (0, 1), r.stdout + r.stderr
    recs, off, prm, grid = cases.gaussian_jet(lib)
    G, F = grid.ngam, grid.nfreq
    per_bw = nsteps * 8 * (9 * F + 4 * G)
    raw = open(tmp_path / "out.bin", "rb").read()
    got = [np.frombuffer(raw, dtype=abi.STEP_DTYPE, count=nsteps, offset=b * (per_bw + 136 * nsteps) + per_bw)
           for b in bws]
    assert_same_records(np.concatenate(got), recs)
