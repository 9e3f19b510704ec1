"""Seeded EATS queries over a batch's histories for the flux-density tests:
cells between two history rows of a blastwave, comoving frequencies inside
the grid, Lorentz factors, viewing cosines on both sides of the shock speed,
cell sizes and densities of the blastwave's range."""
import numpy as np

from pyblastafterglowmag_gb300 import abi


def radii(offsets, seed=0):
    """A monotonic radius history per blastwave (cm), one value per record."""
    rng = np.random.default_rng(seed)
    r = np.zeros(int(offsets[-1]))
    for b in range(len(offsets) - 1):
        n = int(offsets[b + 1] - offsets[b])
        r[offsets[b]:offsets[b + 1]] = np.cumsum(10 ** rng.uniform(14, 16, n)) + 1e15
    return r


def queries(offsets, freq, r_all, j_all, nq, seed=1):
    """nq queries on rows where the histories are non-zero."""
    rng = np.random.default_rng(seed)
    q = np.zeros(nq, dtype=abi.FLUX_QUERY_DTYPE)
    nb = len(offsets) - 1
    F = len(freq) - 1
    live = np.abs(j_all).sum(axis=1) > 0
    k = 0
    while k < nq:
        b = int(rng.integers(0, nb))
        n = int(offsets[b + 1] - offsets[b])
        if n < 2:
            continue
        ia = int(rng.integers(0, n - 1))
        if not (live[offsets[b] + ia] and live[offsets[b] + ia + 1]):
            continue
        r1, r2 = r_all[offsets[b] + ia], r_all[offsets[b] + ia + 1]
        G = 10 ** rng.uniform(0.05, 2.5)
        q[k] = (b, ia, ia + 1, 0, rng.uniform(0.01, 0.5), float(rng.integers(1, 40)),
                np.exp(rng.uniform(np.log(freq[0]) + 1e-6, np.log(freq[F - 1]) - 1e-6)), G, 1.4 * G,
                rng.uniform(0.1, 1.0), rng.uniform(-1, 1), rng.uniform(r1, r2), rng.uniform(r1, r2),
                rng.uniform(1e12, 1e15), 10 ** rng.uniform(-4, 2), 10 ** rng.uniform(45, 52))
        k += 1
    return q
