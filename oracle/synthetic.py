"""Seeded synthetic closed-shell systems (TEST INFRASTRUCTURE ONLY).

The reference has no synthetic generator; the shapes and distributions are the
ones its benchmark configurations name:

* orbital energies: occupied ~ U[-2.0, -0.3], virtual ~ U[0.1, 3.0] (Hartree),
  each sorted ascending, occupied first;
* density-fitting factors B^Q_pq = sigma * z / sqrt(naux), z ~ N(0, 1),
  sigma = 0.05 taken as the standard deviation, drawn for p <= q and mirrored
  (B_qp := B_pq).  The 1/sqrt(naux) normalisation keeps the integral scale
  independent of naux; without it (B ~ N(0, 0.05) summed over naux = 300)
  the o=10/v=90 system has E_MP2 ~ -664 Eh and the CCSD map diverges to NaN
  within six passes, while with it CCSD converges (E_corr ~ -7.25e-3 Eh);
* chemist-notation integrals (pq|rs) = sum_Q B^Q_pq B^Q_rs;
* Fock matrix = diag(orbital energies) (canonical; the reference only handles
  a diagonal Fock matrix correctly, ``ccsdt.cpp:400``).

Random numbers are counter-based: draw(key, i) = mix64(key + (i+1)*GOLDEN),
with mix64 the SplitMix64 output function (Steele, Lea & Flood, "Fast
splittable pseudorandom number generators", OOPSLA 2014).  A normal deviate
uses the Box-Muller transform on draws 2i and 2i+1.  The library's C++
generator (``ccsd_make_synthetic``) implements the same definition, so both
sides see the same inputs to within libm rounding.
"""
from __future__ import annotations

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
STREAM_MUL = np.uint64(0xD1B54A32D192ED03)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)

STREAM_OCC = 1
STREAM_VIR = 2
STREAM_B = 3

SIGMA_B = 0.05
OCC_RANGE = (-2.0, -0.3)
VIR_RANGE = (0.1, 3.0)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
    return z ^ (z >> np.uint64(31))


def stream_key(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        return mix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + np.uint64(stream) * STREAM_MUL)


def draws(key, idx):
    idx = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return mix64(key + (idx + np.uint64(1)) * GOLDEN)


def uniform(key, idx):
    """Uniform on [0, 1) with 53 random bits."""
    return (draws(key, idx) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def normal(key, idx):
    idx = np.asarray(idx, dtype=np.uint64)
    u1 = ((draws(key, 2 * idx) >> np.uint64(11)).astype(np.float64) + 1.0) * (2.0 ** -53)
    u2 = (draws(key, 2 * idx + np.uint64(1)) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def orbital_energies(nocc: int, nvir: int, seed: int) -> np.ndarray:
    ko, kv = stream_key(seed, STREAM_OCC), stream_key(seed, STREAM_VIR)
    eo = OCC_RANGE[0] + (OCC_RANGE[1] - OCC_RANGE[0]) * uniform(ko, np.arange(nocc))
    ev = VIR_RANGE[0] + (VIR_RANGE[1] - VIR_RANGE[0]) * uniform(kv, np.arange(nvir))
    return np.concatenate([np.sort(eo), np.sort(ev)])


def df_factors(n: int, naux: int, seed: int, sigma: float = SIGMA_B) -> np.ndarray:
    """B[Q, p, q], symmetric in (p, q)."""
    kb = stream_key(seed, STREAM_B)
    idx = np.arange(naux * n * n, dtype=np.uint64).reshape(naux, n, n)
    b = (sigma / np.sqrt(naux)) * normal(kb, idx)
    iu = np.triu_indices(n, 1)
    for q in range(naux):
        bq = b[q]
        bq[(iu[1], iu[0])] = bq[iu]
    return b


def eri_from_df(b: np.ndarray) -> np.ndarray:
    """Dense chemist-notation (pq|rs) = sum_Q B^Q_pq B^Q_rs."""
    naux, n, _ = b.shape
    m = b.reshape(naux, n * n)
    return (m.T @ m).reshape(n, n, n, n)


def make_system(nocc: int, nvir: int, naux: int, seed: int):
    """Return (fock[n,n], B[naux,n,n]) for one synthetic closed-shell system."""
    n = nocc + nvir
    eps = orbital_energies(nocc, nvir, seed)
    return np.diag(eps), df_factors(n, naux, seed)
