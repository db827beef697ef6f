"""GPU: the batched solve (ccsd_batch_* / ccsd_solve_batched) against the
single-system solve and the oracle.  Every system of a batch must follow its
own single-system iteration: same number of updates, energies within 1e-12,
amplitudes within 1e-10 (the grouped kernels sum in a different order)."""
import numpy as np
import pytest

import ccsd_parallel_gb300 as cg
from oracle import synthetic as syn
from oracle.ccsd_rhf import RHFCCSD

pytestmark = pytest.mark.gpu


def _c4_systems(count=64, seed=4):
    """Config: C4 batch, `count` synthetic systems with nocc in [4, 12] and nvir in
    [20, 80] (seeded sizes), naux = 3 (nocc + nvir) / 2, library generator."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        o = int(rng.integers(4, 13))
        v = int(rng.integers(20, 81))
        fock, b = cg.make_synthetic(o, v, 3 * (o + v) // 2, 1000 + k)
        out.append(dict(fock=fock, nocc=o, df=b))
    return out


def _compare(batch, singles, e_tol=1e-12, t_tol=1e-10):
    for k, (rb, rs) in enumerate(zip(batch, singles)):
        assert rb["iterations"] == rs["iterations"], k
        assert rb["converged"] == rs["converged"], k
        assert abs(rb["e_corr"] - rs["e_corr"]) < e_tol, (k, rb["e_corr"], rs["e_corr"])
        np.testing.assert_allclose(rb["energies"], rs["energies"], rtol=0, atol=e_tol)
        if rb["t2"] is not None:
            assert np.abs(rb["t1"] - rs["t1"]).max() < t_tol, k
            assert np.abs(rb["t2"] - rs["t2"]).max() < t_tol, k


def test_c4_batch_matches_single_solves():
    systems = _c4_systems()
    with cg.Batch(systems, energy_tol=1e-10) as b:
        batch = b.solve()
        rep = b.report()
    singles = [cg.solve(**s, energy_tol=1e-10) for s in systems]
    _compare(batch, singles)
    assert all(r["converged"] for r in batch)
    # uneven convergence: the batch really masks systems at different updates
    assert len({r["iterations"] for r in batch}) > 1
    # one grouped launch (plus a split-K reduce at most) per operation
    n_ops = len(rep["ops"])
    assert rep["systems"] == 64
    assert rep["launches_per_update"] <= 2 * n_ops + 16
    tiled = [op for op in rep["ops"] if op["kind"] == "contraction" and op["path"] == "tiled"]
    # every tiled contraction was timed or reuses the plan of an identical shape
    assert tiled and any(op["candidates"] > 1 for op in tiled)
    assert all(op["candidates"] > 1 or op["cached"] for op in tiled)


def test_batch_solve_twice_reuses_graphs():
    systems = _c4_systems(count=6, seed=11)
    with cg.Batch(systems) as b:
        r1 = b.solve(amplitudes=False)
        r2 = b.solve(amplitudes=False)
    for a, c in zip(r1, r2):
        assert a["iterations"] == c["iterations"]
        assert a["e_corr"] == c["e_corr"]


def test_batch_with_diis_matches_single_solves():
    systems = _c4_systems(count=8, seed=7)
    opts = dict(energy_tol=1e-10, diis_size=6)
    batch = cg.solve_batched(systems, **opts)
    singles = [cg.solve(**s, **opts) for s in systems]
    _compare(batch, singles, e_tol=1e-11, t_tol=1e-8)


def test_batch_mixed_inputs_and_fixed_iterations():
    o1, v1 = 3, 9
    eps = syn.orbital_energies(o1, v1, 2)
    b1 = syn.df_factors(o1 + v1, 20, 2, sigma=0.3)
    o2, v2 = 5, 11
    eps2 = syn.orbital_energies(o2, v2, 3)
    eri2 = syn.eri_from_df(syn.df_factors(o2 + v2, 30, 3, sigma=0.2))
    n3 = 10
    rng = np.random.default_rng(5)
    c3, _ = np.linalg.qr(rng.standard_normal((n3, n3)))
    eri3 = syn.eri_from_df(syn.df_factors(n3, 25, 4, sigma=0.2))
    ao3 = np.einsum("pqrs,mp,nq,lr,ks->mnlk", eri3, c3, c3, c3, c3, optimize=True)
    systems = [dict(fock=np.diag(eps), nocc=o1, df=b1),
               dict(fock=np.diag(eps2), nocc=o2, eri=eri2),
               dict(fock=np.diag(syn.orbital_energies(4, 6, 4)), nocc=4, ao_eri=ao3, mo_coeff=c3)]
    for opts in (dict(energy_tol=1e-11), dict(fixed_iterations=7)):
        batch = cg.solve_batched(systems, **opts)
        singles = [cg.solve(**s, **opts) for s in systems]
        _compare(batch, singles)
        if "fixed_iterations" in opts:
            assert all(r["iterations"] == 7 for r in batch)


def test_small_batch_matches_oracle():
    systems, ref = [], []
    for k, (o, v) in enumerate([(2, 6), (3, 8), (4, 12), (3, 5)]):
        fock = np.diag(syn.orbital_energies(o, v, 30 + k))
        b = syn.df_factors(o + v, 2 * (o + v), 30 + k, sigma=0.3)
        systems.append(dict(fock=fock, nocc=o, df=b))
        ref.append(RHFCCSD(fock, o, df=b).run(toler=1e-10))
    batch = cg.solve_batched(systems, energy_tol=1e-10)
    for rb, rr in zip(batch, ref):
        assert rb["iterations"] == len(rr["energies"]) - 1  # updates (the reference counter starts at 1)
        assert abs(rb["e_corr"] - rr["e_corr"]) < 1e-10


def test_divergent_system_reported_after_filling_the_rest():
    good = _c4_systems(count=2, seed=9)
    fock = np.diag(syn.orbital_energies(3, 7, 5))
    bad = syn.df_factors(10, 20, 5, sigma=0.8)
    systems = [good[0], dict(fock=fock, nocc=3, df=bad), good[1]]
    with pytest.raises(cg.CCSDError) as ei:
        cg.solve_batched(systems, max_iter=400)
    assert ei.value.code == -4
    assert "system 1" in str(ei.value)
    singles = [cg.solve(**s) for s in (good[0], good[1])]
    _compare([ei.value.results[0], ei.value.results[2]], singles)


def test_split_batch_runs_contractions_on_tensor_cores():
    """precision split3: the larger grouped contractions run as one grouped
    tcgen05 launch over packed split operands; every system follows its own
    split3 single-system solve (same updates, energies within 1e-9) and stays
    within 1e-8 of the FP64 batch."""
    rng = np.random.default_rng(13)
    systems = []
    for k in range(12):
        o, v = int(rng.integers(6, 13)), int(rng.integers(40, 81))
        fock, b = cg.make_synthetic(o, v, 3 * (o + v) // 2, 2000 + k)
        systems.append(dict(fock=fock, nocc=o, df=b))
    with cg.Batch(systems, precision="split3", energy_tol=1e-10) as bt:
        rb = bt.solve()
        rep = bt.report()
    split_ops = [op for op in rep["ops"] if op["kind"] == "contraction" and op["path"] == "split"]
    assert len(split_ops) >= 8, [op["site"] for op in split_ops]
    assert {"pp_ladder_sym", "ring1"} <= {op["site"] for op in split_ops}
    singles = [cg.solve(**s, precision="split3", energy_tol=1e-10) for s in systems]
    fp64 = cg.solve_batched(systems, energy_tol=1e-10)
    for k, (x, y, z) in enumerate(zip(rb, singles, fp64)):
        assert x["iterations"] == y["iterations"], k
        assert abs(x["e_corr"] - y["e_corr"]) < 1e-9, (k, x["e_corr"], y["e_corr"])
        assert abs(x["e_corr"] - z["e_corr"]) < 1e-8, (k, x["e_corr"], z["e_corr"])
        assert np.abs(x["t2"] - y["t2"]).max() < 1e-8
