"""GPU parity of the FP64 path against the oracle, through the C ABI.

Bar: every per-update energy within 1e-10 Eh of the oracle, the same
reference iteration counter at convergence, amplitudes within 1e-10."""
import json
from pathlib import Path

import numpy as np
import pytest

import ccsd_parallel_gb300 as cg
from oracle import synthetic as syn
from oracle.ccsd_rhf import RHFCCSD

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).parent / "golden" / "synthetic_oracle.json").read_text())
E_TOL = 1e-10


def _system(c):
    fock = np.diag(syn.orbital_energies(c["nocc"], c["nvir"], c["seed"]))
    b = syn.df_factors(c["nocc"] + c["nvir"], c["naux"], c["seed"], sigma=c["sigma"])
    return fock, b


@pytest.mark.parametrize("key", sorted(GOLDEN))
def test_fp64_matches_golden_every_update(key):
    c = GOLDEN[key]
    fock, b = _system(c)
    r = cg.solve(fock, c["nocc"], df=b, energy_tol=c["tol"])
    assert r["converged"]
    assert r["iterations"] + 1 == c["iter"]  # reference counter starts at 1
    np.testing.assert_allclose(r["energies"], c["energies"], rtol=0, atol=E_TOL)
    assert abs(r["e_corr"] - c["e_corr"]) < E_TOL
    assert abs(r["t1"].sum() - c["t1_sum"]) < 1e-10
    assert abs((r["t2"] ** 2).sum() - c["t2_sq"]) < 1e-10 * max(1.0, c["t2_sq"])


def test_library_generator_inputs_match_golden():
    c = GOLDEN["syn_o10_v90_q300_s2024_sig0.05"]
    fock, b = cg.make_synthetic(c["nocc"], c["nvir"], c["naux"], c["seed"])
    r = cg.solve(fock, c["nocc"], df=b, energy_tol=c["tol"])
    np.testing.assert_allclose(r["energies"], c["energies"], rtol=0, atol=E_TOL)


def test_amplitudes_match_oracle():
    fock, b = _system(dict(nocc=4, nvir=11, naux=30, seed=8, sigma=0.3))
    ref = RHFCCSD(fock, 4, df=b).run(toler=1e-11, max_passes=9)
    r = cg.solve(fock, 4, df=b, fixed_iterations=9)
    np.testing.assert_allclose(r["energies"], ref["energies"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["t1"], ref["t1"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["t2"], ref["t2"], rtol=0, atol=1e-12)
    assert np.abs(r["t2"] - r["t2"].transpose(1, 0, 3, 2)).max() < 1e-15


def test_integral_input_forms_agree():
    o, v = 3, 9
    fock, b = _system(dict(nocc=o, nvir=v, naux=25, seed=31, sigma=0.3))
    eri = syn.eri_from_df(b)
    r_df = cg.solve(fock, o, df=b, fixed_iterations=6)
    r_mo = cg.solve(fock, o, eri=eri, fixed_iterations=6)
    # AO form: eri = C^T ao C with a random orthogonal C
    rng = np.random.default_rng(0)
    cmat, _ = np.linalg.qr(rng.standard_normal((o + v, o + v)))
    ao = np.einsum("pqrs,mp,nq,lr,ks->mnlk", eri, cmat, cmat, cmat, cmat, optimize=True)
    r_ao = cg.solve(fock, o, ao_eri=ao, mo_coeff=cmat, fixed_iterations=6)
    np.testing.assert_allclose(r_mo["energies"], r_df["energies"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(r_ao["energies"], r_df["energies"], rtol=0, atol=1e-12)


def test_non_canonical_fock_matches_oracle():
    o, v = 3, 8
    fock, b = _system(dict(nocc=o, nvir=v, naux=20, seed=12, sigma=0.3))
    rng = np.random.default_rng(5)
    x = 0.01 * rng.standard_normal(fock.shape)
    fock = fock + x + x.T
    ref = RHFCCSD(fock, o, df=b).run(toler=1e-12, max_passes=8)
    r = cg.solve(fock, o, df=b, fixed_iterations=8)
    np.testing.assert_allclose(r["energies"], ref["energies"], rtol=0, atol=1e-12)


def test_diis_reaches_same_fixed_point_faster():
    c = GOLDEN["syn_o6_v24_q60_s7_sig0.3"]
    fock, b = _system(c)
    r = cg.solve(fock, c["nocc"], df=b, energy_tol=1e-11, residual_tol=1e-8, diis_size=6, diis_start=2)
    assert r["converged"]
    assert abs(r["e_corr"] - c["e_corr"]) < 1e-9
    assert r["iterations"] < c["iter"] - 1


def test_reference_mirror_class():
    """The mirror class iterates the reference class's own map by default and
    the CCSD equations with variant="ccsd"."""
    c = GOLDEN["syn_o3_v7_q20_s5_sig0.3"]
    fock, b = _system(c)
    cc = cg.CCSD_Memory_optimized(fock, c["nocc"], df=b, E_HF=-1.5, variant="ccsd")
    e = cc.CCSD(c["tol"], False)
    assert abs(e - (-1.5 + c["e_corr"])) < E_TOL
    assert cc.iter == c["iter"]
    assert cc.n_Electrons == 2 * c["nocc"] and cc.unocc_orb == 2 * c["nvir"]
    ref = RUNS["syn_o3_v7_q20_s5_sig0.3"]
    mo = cg.CCSD_Memory_optimized(fock, c["nocc"], df=b, E_HF=-1.5)
    e = mo.CCSD(10.0 ** ref["log10_tol"], False)
    assert abs(e - (-1.5 + ref["mo"]["e_corr"])) < E_TOL
    assert mo.iter == ref["mo"]["iter"]


GOLD = Path(__file__).parent / "golden"
H2O = sorted(GOLD.glob("h2o_*.npz"))
RUNS = json.loads((GOLD / "reference_runs.json").read_text())


@pytest.mark.parametrize("path", H2O, ids=[p.stem for p in H2O])
def test_h2o_from_ao_integrals_matches_reference(path):
    """The reference's RHF outputs (AO integrals, C, orbital energies) through
    the AO_DENSE input (h2o_631g_config_tol10 is config C1).  The mirror class
    (memory-optimised map, the default) equals CCSD_Memory_optimized::CCSD to
    1e-10 with its iteration counter; variant="ccsd" equals the reference's
    dense CCSD1 the same way.  The two reference codes differ by more than the
    bar on these molecules (1.9e-8 on C1), so each pin is discriminating."""
    d = np.load(path)
    tol = 10.0 ** float(d["log10_tol"])
    args = (np.diag(d["eps"]), int(d["nocc"]))
    kw = dict(ao_eri=d["ao_eri"], mo_coeff=d["mo_coeff"], E_HF=float(d["e_hf"]))
    cc = cg.CCSD_Memory_optimized(*args, **kw)
    e_total = cc.CCSD(tol, False)
    assert cc.iter == int(d["ref_iter"])
    assert abs(cc.E_new - float(d["ref_e_corr"])) < E_TOL
    assert abs(e_total - float(d["ref_e_total"])) < E_TOL
    c1 = cg.CCSD_Memory_optimized(*args, variant="ccsd", **kw)
    e_total = c1.CCSD(tol, False)
    assert c1.iter == int(d["ref_ccsd1_iter"])
    assert abs(c1.E_new - float(d["ref_ccsd1_e_corr"])) < E_TOL
    assert abs(e_total - (float(d["e_hf"]) + float(d["ref_ccsd1_e_corr"]))) < E_TOL
    assert abs(float(d["ref_e_corr"]) - float(d["ref_ccsd1_e_corr"])) > 10 * E_TOL


def test_h2o_known_answer():
    """-0.0501273 Eh after 20 iterations (ccsd_memory_optimized.cpp:2003)."""
    d = np.load(GOLD / "h2o_sto3g_incarsym_tol8.npz")
    r = cg.solve(np.diag(d["eps"]), 5, ao_eri=d["ao_eri"], mo_coeff=d["mo_coeff"], energy_tol=1e-8)
    assert r["iterations"] + 1 == 20
    assert round(float(r["e_corr"]), 7) == -0.0501273


@pytest.mark.parametrize("key", sorted(RUNS))
def test_synthetic_matches_reference_ccsd1(key):
    c = RUNS[key]
    fock, b = _system(c)
    r = cg.solve(fock, c["nocc"], df=b, energy_tol=10.0 ** c["log10_tol"])
    assert r["iterations"] + 1 == c["ccsd1"]["iter"]
    assert abs(r["e_corr"] - c["ccsd1"]["e_corr"]) < E_TOL


@pytest.mark.parametrize("key", sorted(RUNS))
def test_synthetic_matches_reference_memory_optimized(key):
    c = RUNS[key]
    fock, b = _system(c)
    r = cg.solve(fock, c["nocc"], df=b, energy_tol=10.0 ** c["log10_tol"], variant="memory_optimized")
    assert r["iterations"] + 1 == c["mo"]["iter"]
    assert abs(r["e_corr"] - c["mo"]["e_corr"]) < E_TOL


def test_memory_optimized_variant_follows_oracle_every_update():
    """Per-update energies and amplitudes of the memory-optimised map equal the
    oracle's variant to 1e-12 (FP64) and 1e-9 (split3), and the batched solve
    runs the same map."""
    fock, b = _system(dict(nocc=4, nvir=11, naux=30, seed=8, sigma=0.3))
    ref = RHFCCSD(fock, 4, df=b, variant="memory_optimized").run(toler=1e-11, max_passes=9)
    r = cg.solve(fock, 4, df=b, fixed_iterations=9, variant="memory_optimized")
    np.testing.assert_allclose(r["energies"], ref["energies"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["t2"], ref["t2"], rtol=0, atol=1e-12)
    rs = cg.solve(fock, 4, df=b, fixed_iterations=9, variant="memory_optimized", precision="split3")
    np.testing.assert_allclose(rs["energies"], ref["energies"], rtol=0, atol=1e-9)
    rb = cg.solve_batched([dict(fock=fock, nocc=4, df=b)] * 2, fixed_iterations=9, variant="memory_optimized")
    for x in rb:
        np.testing.assert_allclose(x["energies"], ref["energies"], rtol=0, atol=1e-12)


def test_variant_options_are_checked():
    fock, b = _system(dict(nocc=2, nvir=4, naux=8, seed=1, sigma=0.3))
    for bad in (dict(variant=2), dict(variant="memory_optimized", method="ccsdt-1a")):
        with pytest.raises(cg.CCSDError) as ei:
            cg.solve(fock, 2, df=b, **bad)
        assert ei.value.code == -1


def test_divergence_is_reported():
    fock, b = _system(dict(nocc=3, nvir=7, naux=20, seed=5, sigma=0.8))
    with pytest.raises(cg.CCSDError) as ei:
        cg.solve(fock, 3, df=b, max_iter=400)
    assert ei.value.code == -4


def test_bad_shape_is_rejected():
    fock, b = _system(dict(nocc=2, nvir=4, naux=5, seed=1, sigma=0.05))
    with pytest.raises(cg.CCSDError) as ei:
        cg.solve(fock, 0, df=b)
    assert ei.value.code == -1


@pytest.mark.parametrize("o,v", [(1, 1), (1, 4), (3, 1), (2, 2), (1, 17)])
def test_degenerate_shapes_match_oracle(o, v):
    """nocc = 1 or nvir = 1 leave the antisymmetric ladder half empty (no i > j or
    a > b pairs); single-system FP64 and split3 runs and the batched solve all
    follow the oracle."""
    from oracle.ccsd_rhf import RHFCCSD
    eps = syn.orbital_energies(o, v, 40 + o + v)
    fock = np.diag(eps)
    b = syn.df_factors(o + v, 3 * (o + v), 40 + o + v, sigma=0.3)
    ref = RHFCCSD(fock, o, df=b).run(toler=1e-11)
    for prec, tol in (("fp64", 1e-11), ("split3", 1e-9)):
        r = cg.solve(fock, o, df=b, energy_tol=1e-11, precision=prec)
        assert abs(r["e_corr"] - ref["e_corr"]) < tol, (prec, r["e_corr"], ref["e_corr"])
        np.testing.assert_allclose(r["t2"], ref["t2"], rtol=0, atol=100 * tol)
    rb = cg.solve_batched([dict(fock=fock, nocc=o, df=b)] * 2, energy_tol=1e-11)
    for x in rb:
        assert abs(x["e_corr"] - ref["e_corr"]) < 1e-11


def test_spin_orbital_input_matches_spatial_and_spin_orbital_oracle():
    """The reference's antisymmetrised spin-orbital integrals <PQ||RS> as input
    (CCSD_INTS_SO_ANTISYM): same iterates as the spatial input and as the
    spin-orbital oracle (the reference's CCSD1 equations)."""
    from oracle.ccsd_spinorb import SpinOrbitalCCSD, spin_orbital_integrals
    o, v = 2, 4
    eps = syn.orbital_energies(o, v, 8)
    eri = syn.eri_from_df(syn.df_factors(o + v, 14, 8, sigma=0.3))
    g = spin_orbital_integrals(eri)
    r_so = cg.solve(np.diag(eps), o, so_eri=g, energy_tol=1e-11)
    r_sp = cg.solve(np.diag(eps), o, eri=eri, energy_tol=1e-11)
    ref = SpinOrbitalCCSD(np.diag(eps), eri, o).run(toler=1e-11)
    assert r_so["iterations"] == r_sp["iterations"]
    np.testing.assert_allclose(r_so["energies"], r_sp["energies"], rtol=0, atol=1e-14)
    assert abs(r_so["e_corr"] - ref["e_corr"]) < 1e-10


def test_spin_orbital_input_rejects_open_shell_integrals():
    from oracle.ccsd_spinorb import spin_orbital_integrals
    o, v = 2, 3
    eri = syn.eri_from_df(syn.df_factors(o + v, 10, 9, sigma=0.3))
    g = spin_orbital_integrals(eri)
    g[0::2, 0::2, 0::2, 0::2] *= 1.1      # alpha-alpha block no longer (pr|qs) - (ps|qr)
    with pytest.raises(cg.CCSDError) as ei:
        cg.solve(np.diag(syn.orbital_energies(o, v, 9)), o, so_eri=g)
    assert ei.value.code == -1 and "closed-shell" in str(ei.value)


def test_restart_from_saved_amplitudes_continues_the_iteration():
    """A checkpoint: 3 updates, then a new solve started from their T1/T2
    (t1_start / t2_start) for 3 more gives the energies of 6 updates in a row
    (plain Jacobi, so no history is lost)."""
    fock, b = cg.make_synthetic(4, 16, 30, 5)
    full = cg.solve(fock, 4, df=b, fixed_iterations=6)
    first = cg.solve(fock, 4, df=b, fixed_iterations=3)
    second = cg.solve(fock, 4, df=b, fixed_iterations=3, t1_start=first["t1"], t2_start=first["t2"])
    np.testing.assert_allclose(second["energies"], full["energies"][3:], rtol=0, atol=1e-13)
    np.testing.assert_allclose(second["t2"], full["t2"], rtol=0, atol=1e-13)


def test_restart_arguments_are_checked():
    """A restart T2 of another system's shape is refused before the library
    copies from it; T1 without T2 is refused by the library."""
    fock, b = cg.make_synthetic(3, 8, 20, 5)
    first = cg.solve(fock, 3, df=b, fixed_iterations=2)
    with pytest.raises(cg.CCSDError) as ei:
        cg.solve(fock, 3, df=b, fixed_iterations=1, t2_start=first["t2"][:, :, :7, :7])
    assert ei.value.code == -1 and "shape" in str(ei.value)
    with pytest.raises(cg.CCSDError) as ei:
        cg.solve(fock, 3, df=b, fixed_iterations=1, t1_start=first["t1"])
    assert ei.value.code == -1 and "t2_start" in str(ei.value)


@pytest.mark.parametrize("precision", ["fp64", "split3"])
def test_graph_replay_equals_direct_issue(precision):
    """From its second update on a solve replays each update from a CUDA graph; with
    profile=1 it issues the same kernels directly.  Both follow the same iteration bit
    for bit: every per-update energy and the final amplitudes are equal."""
    fock, b = cg.make_synthetic(6, 48, 150, 31)
    kw = dict(df=b, precision=precision, fixed_iterations=8, diis_size=6, diis_start=2)
    with cg.Solver(fock, 6, **kw) as s:
        rg = s.solve()
    with cg.Solver(fock, 6, profile=True, **kw) as s:
        rd = s.solve()
    assert np.array_equal(rg["energies"], rd["energies"])
    assert np.array_equal(rg["t2"], rd["t2"]) and np.array_equal(rg["t1"], rd["t1"])
    assert rg["residual_norm"] == rd["residual_norm"]
