"""GPU: ccsd_lambda_grad (Lambda equations + dE_corr/d(inputs)) through the C
ABI, against the host FP64 reference (torch autograd) and against central
finite differences (h = 1e-5, tolerance 1e-6) of the GPU energy itself."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import ccsd_parallel_gb300 as cg
from oracle import synthetic as syn
from oracle.ccsd_grad import lambda_grad as host_lambda_grad

pytestmark = pytest.mark.gpu


def read_positions(o, v, rng, k):
    n = o + v
    blocks = [((0, o), (o, n), (0, o), (o, n)), ((0, o), (0, o), (o, n), (o, n)), ((0, o), (o, n), (0, o), (0, o)),
              ((0, o), (0, o), (0, o), (0, o)), ((0, o), (o, n), (o, n), (o, n)), ((o, n), (o, n), (o, n), (o, n))]
    return [tuple(int(rng.integers(a, b)) for a, b in blocks[rng.integers(0, 6)]) for _ in range(k)]


def _system(o, v, q, seed, sigma, offdiag=0.0):
    eps = syn.orbital_energies(o, v, seed)
    eri = syn.eri_from_df(syn.df_factors(o + v, q, seed, sigma=sigma))
    fock = np.diag(eps)
    if offdiag:
        x = offdiag * np.random.default_rng(seed).standard_normal(fock.shape)
        fock = fock + x + x.T
    return fock, eri


def test_gpu_gradient_matches_host_reference():
    o, v = 4, 10
    fock, eri = _system(o, v, 20, 9, 0.3, offdiag=0.01)
    with cg.Solver(fock, o, eri=eri, energy_tol=1e-13) as s:
        r = s.solve()
        G = s.lambda_grad(tol=1e-12, lambdas=True)
    H = host_lambda_grad(fock, eri, o, r["t1"], r["t2"], tol=1e-12)
    np.testing.assert_allclose(G["lambda1"], H["lambda1"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(G["lambda2"], H["lambda2"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(G["d_fock"], H["d_fock"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(G["d_eri"], H["d_eri"], rtol=0, atol=1e-10)
    assert G["e_corr"] == pytest.approx(r["e_corr"], abs=1e-15)


def _fd_check(make, grad, positions, h=1e-5, tol=1e-6):
    worst = 0.0
    for key, idx in positions:
        ep = make(key, idx, +h)
        em = make(key, idx, -h)
        fd = (ep - em) / (2 * h)
        worst = max(worst, abs(fd - grad[key][idx]))
    print(f"finite-difference check: {len(positions)} entries, max |fd - grad| {worst:.3e}")
    assert worst < tol, worst
    return worst


def test_c3_gradient_against_finite_differences():
    """Config: synthetic nocc=8, nvir=60 (seeded DF generator, dense MO input),
    FP64; dE/dfock and dE/d(pq|rs) on 200 random read entries vs central FD."""
    o, v, q, seed = 8, 60, 200, 20
    fock, b = cg.make_synthetic(o, v, q, seed)
    eri = np.einsum("Qpq,Qrs->pqrs", b, b, optimize=True)
    with cg.Solver(fock, o, eri=eri, energy_tol=1e-13) as s:
        s.solve(amplitudes=False)
        G = s.lambda_grad(tol=1e-12)

    def energy(key, idx, dh):
        f, g = fock, eri
        if key == "d_fock":
            f = fock.copy()
            f[idx] += dh
        else:
            g = eri.copy()
            g[idx] += dh
        return cg.solve(f, o, eri=g, energy_tol=1e-13, amplitudes=False)["e_corr"]

    rng = np.random.default_rng(7)
    pos = [("d_eri", p) for p in read_positions(o, v, rng, 180)]
    n = o + v
    pos += [("d_fock", (int(rng.integers(0, n)),) * 2) for _ in range(10)]
    pos += [("d_fock", (int(rng.integers(0, o)), int(rng.integers(o, n)))) for _ in range(10)]
    _fd_check(energy, G, pos)


def test_df_and_ao_input_gradients_against_finite_differences():
    o, v, q = 3, 7, 16
    eps = syn.orbital_energies(o, v, 3)
    b = syn.df_factors(o + v, q, 3, sigma=0.3)
    fock = np.diag(eps)
    with cg.Solver(fock, o, df=b, energy_tol=1e-13) as s:
        s.solve(amplitudes=False)
        G = s.lambda_grad(tol=1e-12)
    rng = np.random.default_rng(3)
    pos = [("d_df", (int(rng.integers(0, q)), int(rng.integers(0, o + v)), int(rng.integers(0, o + v))))
           for _ in range(12)]

    def e_df(key, idx, dh):
        bb = b.copy()
        bb[idx] += dh
        return cg.solve(fock, o, df=bb, energy_tol=1e-13, amplitudes=False)["e_corr"]

    _fd_check(e_df, G, pos)

    eri = syn.eri_from_df(b)
    cmat, _ = np.linalg.qr(rng.standard_normal((o + v, o + v)))
    ao = np.einsum("pqrs,mp,nq,lr,ks->mnlk", eri, cmat, cmat, cmat, cmat, optimize=True)
    with cg.Solver(fock, o, ao_eri=ao, mo_coeff=cmat, energy_tol=1e-13) as s:
        s.solve(amplitudes=False)
        GA = s.lambda_grad(tol=1e-12)

    def e_ao(key, idx, dh):
        a, c = ao, cmat
        if key == "d_eri":
            a = ao.copy()
            a[idx] += dh
        else:
            c = cmat.copy()
            c[idx] += dh
        return cg.solve(fock, o, ao_eri=a, mo_coeff=c, energy_tol=1e-13, amplitudes=False)["e_corr"]

    n = o + v
    posa = [("d_eri", tuple(int(rng.integers(0, n)) for _ in range(4))) for _ in range(8)]
    posa += [("d_mo_coeff", (int(rng.integers(0, n)), int(rng.integers(0, n)))) for _ in range(8)]
    _fd_check(e_ao, GA, posa)


def test_gradient_requires_a_solve():
    fock, eri = _system(2, 4, 6, 1, 0.1)
    with cg.Solver(fock, 2, eri=eri) as s:
        with pytest.raises(cg.CCSDError) as ei:
            s.lambda_grad()
        assert ei.value.code == -1


def test_split_precision_gradient_close_to_fp64():
    """The split-precision engine runs the reverse sweep on the same tcgen05
    contractions; its gradient stays within 1e-8 of the FP64 gradient."""
    o, v, q, seed = 8, 60, 200, 21
    fock, b = cg.make_synthetic(o, v, q, seed)
    out = {}
    for prec in ("fp64", "split3"):
        with cg.Solver(fock, o, df=b, precision=prec, energy_tol=1e-12) as s:
            s.solve(amplitudes=False)
            out[prec] = s.lambda_grad(tol=1e-11, lambdas=True)
    for k in ("d_fock", "d_df", "lambda1", "lambda2"):
        d = np.abs(out["split3"][k] - out["fp64"][k]).max()
        print(f"split3 vs fp64 {k}: max |diff| {d:.3e}")
        assert d < 1e-8, (k, d)


def test_c5_df_gradient_against_finite_differences():
    """Config: the bench workload, synthetic nocc=24, nvir=300, naux=900, split3.
    dE/dB on four DF entries (two in the virtual-virtual block, whose ladder
    term is taken directly from Lambda without the v^4 adjoints) against
    central differences of split3 solves (h = 1e-4); within 1e-6."""
    o, v, q = 24, 300, 900
    fock, b = cg.make_synthetic(o, v, q, 2024)
    opts = dict(precision="split3", energy_tol=1e-11, diis_size=6, diis_start=2)
    with cg.Solver(fock, o, df=b, **opts) as s:
        s.solve(amplitudes=False)
        G = s.lambda_grad(tol=1e-9)
    n = o + v
    pos = [(17, o + 5, o + 200), (401, o + 123, o + 7), (3, 2, o + 50), (650, 1, 20)]
    h = 1e-4
    worst = 0.0
    for idx in pos:
        bp, bm = b.copy(), b.copy()
        bp[idx] += h
        bm[idx] -= h
        ep = cg.solve(fock, o, df=bp, amplitudes=False, **opts)["e_corr"]
        em = cg.solve(fock, o, df=bm, amplitudes=False, **opts)["e_corr"]
        worst = max(worst, abs((ep - em) / (2 * h) - G["d_df"][idx]))
    print(f"C5 finite-difference check: {len(pos)} DF entries, max |fd - grad| {worst:.3e}")
    assert worst < 1e-6


def test_spin_orbital_input_gradient():
    """dE/d<PQ||RS> for the spin-orbital input form: the alpha-beta block
    carries the spatial gradient, every other element has derivative 0 (the
    engine does not read it); central FD on alpha-beta entries (h = 1e-6, small
    enough for the input's closed-shell check)."""
    from oracle.ccsd_spinorb import spin_orbital_integrals
    o, v = 2, 4
    fock, eri = _system(o, v, 14, 8, 0.3)
    g = spin_orbital_integrals(eri)
    with cg.Solver(fock, o, so_eri=g, energy_tol=1e-13) as s:
        s.solve(amplitudes=False)
        G = s.lambda_grad(tol=1e-12)
    with cg.Solver(fock, o, eri=eri, energy_tol=1e-13) as s:
        s.solve(amplitudes=False)
        Gs = s.lambda_grad(tol=1e-12)
    n = o + v
    ab = G["d_eri"][0::2, 1::2, 0::2, 1::2].transpose(0, 2, 1, 3)   # [p][r][q][s] -> [p][q][r][s]
    np.testing.assert_allclose(ab, Gs["d_eri"], rtol=0, atol=1e-12)
    mask = np.ones_like(G["d_eri"], dtype=bool)
    mask[0::2, 1::2, 0::2, 1::2] = False
    assert np.abs(G["d_eri"][mask]).max() == 0.0
    h = 1e-6

    def e(idx, dh):
        gg = g.copy()
        gg[idx] += dh
        return cg.solve(fock, o, so_eri=gg, energy_tol=1e-13, amplitudes=False)["e_corr"]

    for idx in [(0, 1, 2, 3), (2 * 1, 2 * 3 + 1, 2 * 1, 2 * 3 + 1), (2 * 3, 2 * 0 + 1, 2 * 5, 2 * 2 + 1)]:
        fd = (e(idx, h) - e(idx, -h)) / (2 * h)
        assert abs(fd - G["d_eri"][idx]) < 1e-6, (idx, fd, G["d_eri"][idx])
