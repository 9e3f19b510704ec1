"""Generate tests/golden/eats_lc.npz from the REFERENCE's own EATS integrator.

Runs here, where the reference sources are present: oracle/Makefile compiles
the reference's eats.h with its blastwave headers into
oracle/_ref/libpbaref_eats.so, and this script drives EATS::evalFluxDensA on
the seeded cases of tests/eats_cases.py (histories from the oracle's step,
which the other fixtures pin to the reference) and stores the light curves.
The GPU machine has no reference; its tests rebuild the inputs and read these.

    python tests/golden/make_golden_eats.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pyoracle  # noqa: E402
import eats_cases  # noqa: E402


def main():
    orc = pyoracle.Oracle()
    ref = pyoracle.ReferenceEats()
    out = {}
    for name in eats_cases.CASES:
        grid, o, layers, dyn, off, recs, prm, j, a, q = eats_cases.inputs(name, orc, orc)
        out[name] = ref.eats_flux(grid, o, layers, dyn, off, j, a, q)
        print(name, len(q), "queries")
    path = os.path.join(HERE, "eats_lc.npz")
    np.savez_compressed(path, **out)
    print(f"eats_lc.npz: {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
