"""Seeded comoving states of the emissivity-contraction microbenchmark.

A batch of electron spectra on 256 log-spaced gamma in [1, 1e9] (the step's
gamma grid), each a power law with an exponential cutoff,
    f(gamma) = gamma^-p exp(-gamma / gamma_max),  p ~ U[2, 3],  log10 gamma_max ~ U[5, 8],
a field log10 B ~ U[-2, 1] G, and as seed photon density the synchrotron
spectrum of the same state, n_k = j_syn,k / (h nu_k) (times 1 s cm^-1: the SSC
emissivity is linear in n, so the normalisation is arbitrary). Frequencies:
256 log-spaced nu in [1e8, 1e29] Hz.
"""
import numpy as np

from . import abi

H_PL = 6.6260755e-27


def grid_desc(ngam=256, nfreq=256):
    return abi.GridDesc(ngam=ngam, nfreq=nfreq, gam1=1.0, gam2=1e9, freq1=1e8, freq2=1e29)


def states(gam, n, seed=4):
    """f [n][G] and B [n] of n seeded states on the gamma grid `gam`."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(2.0, 3.0, n)
    gmax = 10.0 ** rng.uniform(5.0, 8.0, n)
    B = 10.0 ** rng.uniform(-2.0, 1.0, n)
    f = gam[None, :] ** (-p[:, None]) * np.exp(-gam[None, :] / gmax[:, None])
    return f, B


def seed_photons(jsyn, freq):
    """Photon density n_k = j_syn,k / (h nu_k) of the states' own synchrotron spectra."""
    nu = np.asarray(freq)[: jsyn.shape[1]]
    return jsyn / (H_PL * nu[None, :])
