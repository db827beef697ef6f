"""CPU tests of the oracle: the closed-shell restatement against the
spin-orbital restatement of the reference equations, the committed golden
fixtures, and the properties the reference's amplitudes have."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import synthetic as syn
from oracle.ccsd_rhf import RHFCCSD
from oracle.ccsd_spinorb import SpinOrbitalCCSD

GOLDEN = json.loads((Path(__file__).parent / "golden" / "synthetic_oracle.json").read_text())


def _system(o, v, q, seed, sigma):
    fock = np.diag(syn.orbital_energies(o, v, seed))
    b = syn.df_factors(o + v, q, seed, sigma=sigma)
    return fock, b


@pytest.mark.parametrize("o,v,q,seed,sigma", [(2, 4, 10, 1, 0.3), (3, 6, 15, 9, 0.3),
                                              (4, 7, 25, 4, 0.2)])
def test_closed_shell_equals_spin_orbital_every_iterate(o, v, q, seed, sigma):
    fock, b = _system(o, v, q, seed, sigma)
    eri = syn.eri_from_df(b)
    so = SpinOrbitalCCSD(fock, eri, o).run(toler=1e-12, max_passes=10)
    cs = RHFCCSD(fock, o, eri=eri).run(toler=1e-12, max_passes=10)
    assert so["iter"] == cs["iter"]
    np.testing.assert_allclose(so["energies"], cs["energies"], rtol=0, atol=1e-13)
    # t(a alpha, b beta, i alpha, j beta) = t2[i, j, a, b]
    aa, ii = np.arange(v) * 2, np.arange(o) * 2
    t2ab = so["t2"][np.ix_(aa, aa + 1, ii, ii + 1)].transpose(2, 3, 0, 1)
    np.testing.assert_allclose(t2ab, cs["t2"], rtol=0, atol=1e-14)
    # same-spin block = t2[i,j,a,b] - t2[j,i,a,b]
    t2aa = so["t2"][np.ix_(aa, aa, ii, ii)].transpose(2, 3, 0, 1)
    np.testing.assert_allclose(t2aa, cs["t2"] - cs["t2"].transpose(1, 0, 2, 3), rtol=0, atol=1e-14)
    np.testing.assert_allclose(so["t1"][np.ix_(aa, ii)].T, cs["t1"], rtol=0, atol=1e-14)


def test_dense_and_df_blocks_agree():
    fock, b = _system(3, 8, 20, 17, 0.3)
    r1 = RHFCCSD(fock, 3, df=b).run(toler=1e-12, max_passes=6)
    r2 = RHFCCSD(fock, 3, eri=syn.eri_from_df(b)).run(toler=1e-12, max_passes=6)
    np.testing.assert_allclose(r1["energies"], r2["energies"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("key", [k for k, c in GOLDEN.items() if c["source"] == "oracle.ccsd_spinorb"])
def test_oracle_reproduces_golden(key):
    c = GOLDEN[key]
    fock, b = _system(c["nocc"], c["nvir"], c["naux"], c["seed"], c["sigma"])
    r = RHFCCSD(fock, c["nocc"], df=b).run(toler=c["tol"])
    assert r["iter"] == c["iter"]
    np.testing.assert_allclose(r["energies"], c["energies"], rtol=0, atol=1e-12)


def test_amplitude_symmetry_and_sign_flip_invariance():
    o, v = 3, 6
    fock, b = _system(o, v, 18, 21, 0.3)
    eri = syn.eri_from_df(b)
    r = RHFCCSD(fock, o, eri=eri).run(toler=1e-11)
    t2 = r["t2"]
    np.testing.assert_allclose(t2, t2.transpose(1, 0, 3, 2), atol=1e-15)
    # flipping the sign of orbitals leaves E invariant
    s = np.ones(o + v)
    s[[1, o + 2]] = -1.0
    eri_f = eri * s[:, None, None, None] * s[None, :, None, None] * s[None, None, :, None] * s[None, None, None, :]
    r2 = RHFCCSD(fock, o, eri=eri_f).run(toler=1e-11)
    assert abs(r["e_corr"] - r2["e_corr"]) < 1e-13
    so = s[:o][:, None, None, None] * s[:o][None, :, None, None] * s[o:][None, None, :, None] * s[o:][None, None, None, :]
    np.testing.assert_allclose(r2["t2"], t2 * so, atol=1e-14)


def test_reference_iteration_counter_and_stop_rule():
    """iter starts at 1 and is bumped once per update; the loop stops on
    |dE| < toler (ccsd_memory_optimized.cpp:513-556)."""
    fock, b = _system(2, 5, 12, 1, 0.3)
    r = RHFCCSD(fock, 2, df=b).run(toler=1e-8)
    e = r["energies"]
    assert r["iter"] == len(e)
    assert abs(e[-1] - e[-2]) < 1e-8
    assert all(abs(e[k] - e[k - 1]) >= 1e-8 for k in range(1, len(e) - 1))


def test_literal_sigma_diverges_normalised_converges():
    """B ~ N(0, 0.05) without the 1/sqrt(naux) normalisation drives the map to
    a huge MP2 energy (the recorded reason for the normalisation)."""
    o, v, q = 4, 30, 60
    eps = syn.orbital_energies(o, v, 3)
    b = syn.df_factors(o + v, q, 3) * np.sqrt(q)  # literal N(0, 0.05)
    cc = RHFCCSD(np.diag(eps), o, df=b)
    _, t2 = cc.mp2_guess()
    e_lit = cc.energy(np.zeros((o, v)), t2)
    r = RHFCCSD(np.diag(eps), o, df=syn.df_factors(o + v, q, 3)).run(toler=1e-10)
    assert abs(e_lit) > 50 * abs(r["e_corr"])
    assert r["iter"] < 20


@pytest.mark.parametrize("o,v,q,seed", [(3, 8, 20, 1), (4, 11, 30, 8), (1, 5, 10, 3), (2, 1, 6, 4), (1, 1, 4, 2)])
def test_cpu_update_equals_the_oracle_map(o, v, q, seed):
    """The timed CPU implementation (oracle.cpu_update: BLAS layouts, the pair
    forms of both ladders, Z and X on packs built from the DF factors) computes
    the closed-shell map of RHFCCSD.residual, at symmetric amplitudes, to
    rounding."""
    from oracle.ccsd_rhf import RHFCCSD
    from oracle.cpu_update import FullUpdate
    fock = np.diag(syn.orbital_energies(o, v, seed))
    b = syn.df_factors(o + v, q, seed, sigma=0.3)
    ref, fu = RHFCCSD(fock, o, df=b), FullUpdate(fock, o, b, diis_size=0)
    rng = np.random.default_rng(seed)
    t1 = 0.05 * rng.standard_normal((o, v))
    x = 0.05 * rng.standard_normal((o, o, v, v))
    t2 = x + x.transpose(1, 0, 3, 2)
    R1a, R2a = ref.residual(t1, t2)
    R1b, R2b = fu.residual(t1, t2)
    assert np.abs(R1a - R1b).max() < 1e-14 and np.abs(R2a - R2b).max() < 1e-14
    assert abs(ref.energy(t1, t2) - fu.energy(t1, t2)) < 1e-14
    # whole updates (plain Jacobi) follow the oracle's iterates
    r = ref.run(toler=1e-14, max_passes=4)
    for k in range(4):
        fu.step()
    assert abs(fu.energy(fu.t1, fu.t2) - r["e_corr"]) < 1e-13
