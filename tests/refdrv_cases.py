"""Runs of the reference's own program, recorded by
tests/golden/make_reference_run.py (refdrv_<case>.npz) and loaded by
histories.DriverRun: the dynamics its blastwave ODE driver saved, the
comoving spectra its radiation step produced from them and its adaptive-EATS
light curve, with the step records, EATS inputs and EATS options rebuilt from
them, so that the CPU and GPU tests compare what this library computes on the
reference's own inputs with what the reference computed."""
import os

from pyblastafterglowmag_gb300.histories import DriverRun

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("tophat", "gaussian")


def path(name):
    return os.path.join(GOLDEN, f"refdrv_{name}.npz")


class Runs(dict):
    """The recorded runs by name, each loaded on first use."""

    def __missing__(self, name):
        self[name] = DriverRun(path(name))
        return self[name]
