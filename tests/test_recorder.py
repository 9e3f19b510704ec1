"""The C++ drop-in host layer (include/pbag_recorder.hpp): it compiles with
the host compiler, and replaying a batch's records through its per-step calls
gives the same histories as the batch entry point."""
import os
import subprocess

import numpy as np
import pytest

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "recorder_check.cpp")
LIBDIR = os.path.join(ROOT, "pyblastafterglowmag_gb300")


def test_recorder_header_compiles():
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"),
                    SRC], check=True)


@pytest.mark.gpu
def test_recorder_replay_matches_batch(lib, cuda_device, tmp_path):
    recs, off, prm, grid = cases.gaussian(lib, nlayers=2, nsteps=90)
    exe = tmp_path / "recorder_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-o", str(exe),
                    "-L" + LIBDIR, "-lpbag", "-Wl,-rpath," + LIBDIR], check=True)
    files = {}
    for name, arr in (("grid", np.frombuffer(bytes(grid), dtype=np.uint8)), ("params", prm), ("offsets", off),
                      ("records", recs)):
        p = tmp_path / f"{name}.bin"
        np.ascontiguousarray(arr).tofile(p)
        files[name] = str(p)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), files["grid"], files["params"], files["offsets"], files["records"], str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    # the spectrum writer's names (ejecta.h:354-455) for the vectors a caller gave
    names = [w.split(":")[0] for w in r.stdout.split("datasets", 1)[1].splitlines()[0].split()]
    assert names == ["syn_f_fs", "ssc_f_fs", "total_j_fs", "total_a_fs"], r.stdout
    got = np.fromfile(out, dtype=np.float64)
    ctx = lib.Context(grid, cuda_device, ssc=True)
    ref = ctx.run(recs, off, prm, outputs=("j_all", "a_all"))
    F = grid.nfreq
    expect = np.concatenate([np.concatenate([ref["j_all"][off[b]:off[b + 1]].ravel(),
                                             ref["a_all"][off[b]:off[b + 1]].ravel()]) for b in range(len(prm))])
    np.testing.assert_array_equal(got, expect)
