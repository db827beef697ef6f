"""Frozen core on the GPU engine (ccsd_problem.nfrozen; the reference's
Freeze_Core, Prepear_AOs(nr_freeze), ccsd_memory_optimized.cpp:2698-2709,
3520-3521). The reference's own frozen path is unfinished (its orbital count
reads the nuclear charges at electron indices, :5213-5219), so parity is held
to the definition: freezing the lowest k orbitals equals CCSD on the arrays with
those orbitals removed, and that equals the oracle on the same active space.

Tolerances: the full-array and sliced-array runs take the same contractions
over the same numbers, so energies agree to 1e-13 and amplitudes to 1e-13;
the oracle comparisons use the CCSD parity bound 1e-11."""
from pathlib import Path

import numpy as np
import pytest

import ccsd_parallel_gb300 as cg
from ccsd_parallel_gb300 import _abi
from oracle import synthetic as syn
from oracle.ccsd_rhf import RHFCCSD

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden"


def _h2o():
    d = np.load(GOLD / "h2o_631g_config_tol10.npz")
    return np.diag(d["eps"]), int(d["nocc"]), d["ao_eri"], d["mo_coeff"]


def _synthetic(o, v, naux, seed):
    eps = syn.orbital_energies(o, v, seed)
    return np.diag(eps), syn.df_factors(o + v, naux, seed, sigma=0.3)


@pytest.mark.parametrize("form", ["df", "eri", "ao", "so"])
@pytest.mark.parametrize("k", [1, 2])
def test_frozen_equals_sliced_inputs(form, k):
    """Every integral input form: nfrozen=k over the full arrays gives the
    iterates of the same solve over the arrays without the first k orbitals."""
    from oracle.ccsd_spinorb import spin_orbital_integrals
    o, v = 4, 9
    fock, b = _synthetic(o, v, 40, 31 + k)
    eri = syn.eri_from_df(b)
    act = slice(k, None)
    if form == "df":
        full, cut = dict(df=b), dict(df=np.ascontiguousarray(b[:, act, act]))
    elif form == "eri":
        full, cut = dict(eri=eri), dict(eri=np.ascontiguousarray(eri[act, act, act, act]))
    elif form == "ao":
        rng = np.random.default_rng(7)
        c = np.linalg.qr(rng.standard_normal((o + v, o + v)))[0]  # AO basis = rotated MOs
        ao = np.einsum("pqrs,ip,jq,kr,ls->ijkl", eri, c, c, c, c, optimize=True)
        full, cut = dict(ao_eri=ao, mo_coeff=c), dict(ao_eri=ao, mo_coeff=np.ascontiguousarray(c[:, act]))
    else:
        so = spin_orbital_integrals(eri)
        sact = slice(2 * k, None)
        full, cut = dict(so_eri=so), dict(so_eri=np.ascontiguousarray(so[sact, sact, sact, sact]))
    r_full = cg.solve(fock, o, nfrozen=k, energy_tol=1e-11, **full)
    r_cut = cg.solve(np.ascontiguousarray(fock[act, act]), o - k, energy_tol=1e-11, **cut)
    assert r_full["iterations"] == r_cut["iterations"]
    np.testing.assert_allclose(r_full["energies"], r_cut["energies"], rtol=0, atol=1e-13)
    assert r_full["t2"].shape == (o - k, o - k, v, v)
    np.testing.assert_allclose(r_full["t2"], r_cut["t2"], rtol=0, atol=1e-13)


def test_frozen_core_h2o_matches_oracle():
    """H2O 6-31G with the O 1s orbital frozen (one orbital, the reference's rule
    for Z = 8): the oracle on the active MO integrals, energy to 1e-11 with the
    same iteration counter; the all-electron energy is lower."""
    fock, nocc, ao, c = _h2o()
    assert cg.frozen_core_count([8.0, 1.0, 1.0]) == 1
    mo = np.einsum("pqrs,pi,qj,rk,sl->ijkl", ao, c, c, c, c, optimize=True)
    ref = RHFCCSD(fock[1:, 1:], nocc - 1, eri=mo[1:, 1:, 1:, 1:]).run(toler=1e-10)
    cc = cg.CCSD_Memory_optimized(fock, nocc, ao_eri=ao, mo_coeff=c, nfrozen=1, variant="ccsd")
    cc.CCSD(1e-10, False)
    assert cc.n_Electrons == 2 * (nocc - 1)
    assert cc.iter == ref["iter"]
    assert abs(cc.E_new - ref["e_corr"]) < 1e-11
    full = cg.solve(fock, nocc, ao_eri=ao, mo_coeff=c, energy_tol=1e-10)
    assert full["e_corr"] < cc.E_new


def test_frozen_core_gradient_is_the_embedded_active_gradient():
    """dE/d(inputs) with nfrozen=1: the active block equals the gradient of the
    sliced problem, every element touching only a frozen orbital is 0."""
    o, v, k = 3, 7, 1
    fock, b = _synthetic(o, v, 30, 41)
    act = slice(k, None)
    with cg.Solver(fock, o, df=b, nfrozen=k, energy_tol=1e-12) as s:
        s.solve()
        g = s.lambda_grad(tol=1e-12)
    with cg.Solver(np.ascontiguousarray(fock[act, act]), o - k, df=np.ascontiguousarray(b[:, act, act]),
                   energy_tol=1e-12) as s:
        s.solve()
        gc = s.lambda_grad(tol=1e-12)
    assert g["d_fock"].shape == fock.shape and g["d_df"].shape == b.shape
    np.testing.assert_allclose(g["d_fock"][act, act], gc["d_fock"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(g["d_df"][:, act, act], gc["d_df"], rtol=0, atol=1e-12)
    assert not g["d_fock"][:k].any() and not g["d_fock"][:, :k].any()
    assert not g["d_df"][:, :k].any() and not g["d_df"][:, :, :k].any()


def test_frozen_core_ccsdt_and_batched():
    """The triples methods and the batched solve see the same active space."""
    o, v, k = 3, 5, 1
    fock, b = _synthetic(o, v, 24, 43)
    act = slice(k, None)
    fc, bc = np.ascontiguousarray(fock[act, act]), np.ascontiguousarray(b[:, act, act])
    r = cg.solve(fock, o, df=b, nfrozen=k, method="ccsdt-1a", fixed_iterations=4)
    rc = cg.solve(fc, o - k, df=bc, method="ccsdt-1a", fixed_iterations=4)
    np.testing.assert_allclose(r["energies"], rc["energies"], rtol=0, atol=1e-13)
    f2, b2 = _synthetic(4, 6, 26, 44)
    res = cg.solve_batched([dict(fock=fock, nocc=o, df=b, nfrozen=k), dict(fock=f2, nocc=4, df=b2, nfrozen=2)],
                           energy_tol=1e-11)
    ref0 = cg.solve(fc, o - k, df=bc, energy_tol=1e-11)
    ref1 = cg.solve(np.ascontiguousarray(f2[2:, 2:]), 2, df=np.ascontiguousarray(b2[:, 2:, 2:]), energy_tol=1e-11)
    assert abs(res[0]["e_corr"] - ref0["e_corr"]) < 1e-12
    assert abs(res[1]["e_corr"] - ref1["e_corr"]) < 1e-12


def test_frozen_core_bad_counts_fail_loudly():
    fock, b = _synthetic(3, 5, 24, 45)
    for k in (-1, 3):  # negative, or every occupied orbital frozen (no active occupied)
        with pytest.raises(cg.CCSDError) as ei:
            cg.solve(fock, 3, df=b, nfrozen=k)
        assert ei.value.code == _abi.CCSD_ERR_INVALID_ARG
