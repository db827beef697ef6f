"""FP64 restatement of the reference's Hartree-Fock steps
(Hartree_Fock_Solver::get_Energy, hartree_fock_solver.cpp:578-1229), TEST
INFRASTRUCTURE ONLY: what the GPU SCF (ccsd_rhf, ccsd_uhf) is compared with.

RHF (do_uhf = 0): canonical orthogonalisation X = U lambda^-1/2 of S (:686-690);
P = 0 at the start; F = h + J(P) - K(P)/2 (Make_Fock_Matrix :490-569); DIIS over
the last 3 Fock matrices with error F P S - S P F, from the second Fock matrix on,
extrapolating once 4 have been seen (DIIS :1252-1311); eigenpairs of X^T F X, C = X W
with c^T S c = 1 (Normalize :1230-1245); P = 2 C_occ C_occ^T (Calc_Density); stop
when |sum of occupied eps - previous| < tol or after 300 steps; E = sum h P +
1/2 sum F_prev P - 1/2 sum h P + E_nuc (Calc_Energy :482-488).

UHF (do_uhf = 1, :959-1025): F_up = h + J(P_up + P_down) - K(P_up), F_down likewise
(Unrestricted_Fock_Matrix :1359-1503), no DIIS, P_s = C_s,occ C_s,occ^T; stop when
|eps_up[0] - previous| + |eps_down[0] - previous| < tol; E as Unrestricted_Energy
(:1531-1537).  The reference starts from random densities (Initialize_UHF); here a
seeded generator gives the start.

J[i][j] = sum_kl (ij|kl) P[l][k], K[i][j] = sum_kl (il|kj) P[l][k], from the AO
integrals as a dense [n]^4 array (chemist notation).
"""
from __future__ import annotations

import numpy as np


def _orthogonaliser(S):
    lam, U = np.linalg.eigh(S)
    return U / np.sqrt(lam)


def _orbitals(X, S, F):
    eps, W = np.linalg.eigh(X.T @ F @ X)
    C = X @ W
    C = C / np.sqrt(np.einsum("ic,ij,jc->c", C, S, C))
    return eps, C


def rhf(S, h, eri, e_nuc: float, n_electrons: int, tol: float = 1e-10, limit: int = 300) -> dict:
    nocc = n_electrons // 2
    X = _orthogonaliser(S)
    n = S.shape[0]
    P = np.zeros((n, n))
    errs, focks = [], []
    hf_new, step = 0.0, 0
    while True:
        hf_old = hf_new
        F = h + np.einsum("ijkl,lk->ij", eri, P) - 0.5 * np.einsum("ilkj,lk->ij", eri, P)
        F_prev = F.copy()
        if step > 0:
            errs.append(F @ P @ S - S @ P @ F)
            focks.append(F.copy())
            if step > 3:
                errs.pop(0)
                focks.pop(0)
                B = -np.ones((4, 4))
                B[3, 3] = 0.0
                for i in range(3):
                    for j in range(3):
                        B[i, j] = np.sum(errs[i] * errs[j])
                c = np.linalg.solve(B, np.array([0.0, 0.0, 0.0, -1.0]))
                F = sum(c[i] * focks[i] for i in range(3))
        eps, C = _orbitals(X, S, F)
        P = 2.0 * C[:, :nocc] @ C[:, :nocc].T
        hf_new = eps[:nocc].sum()
        step += 1
        if abs(hf_new - hf_old) < tol or step > limit:
            break
    e1 = np.sum(h * P)
    return dict(e_hf=e1 + 0.5 * np.sum(F_prev * P) - 0.5 * e1 + e_nuc, eps=eps, C=C, iterations=step)


def uhf(S, h, eri, e_nuc: float, n_up: int, n_down: int, tol: float = 1e-10, limit: int = 300,
        seed: int = 0) -> dict:
    X = _orthogonaliser(S)
    n = S.shape[0]
    rng = np.random.default_rng(seed)
    Pu, Pd = rng.standard_normal((n, n)), rng.standard_normal((n, n))
    Pu, Pd = 0.5 * (Pu + Pu.T), 0.5 * (Pd + Pd.T)
    eu_old = ed_old = 0.0
    step = 0
    while True:
        J = np.einsum("ijkl,lk->ij", eri, Pu + Pd)
        Fu = h + J - np.einsum("ilkj,lk->ij", eri, Pu)
        Fd = h + J - np.einsum("ilkj,lk->ij", eri, Pd)
        eu, Cu = _orbitals(X, S, Fu)
        ed, Cd = _orbitals(X, S, Fd)
        Pu, Pd = Cu[:, :n_up] @ Cu[:, :n_up].T, Cd[:, :n_down] @ Cd[:, :n_down].T
        check = abs(eu[0] - eu_old) + abs(ed[0] - ed_old)
        eu_old, ed_old = eu[0], ed[0]
        step += 1
        if check < tol or step > limit:
            break
    e1 = np.sum((Pu + Pd) * h)
    e = e1 + 0.5 * np.sum(Fu * Pu) + 0.5 * np.sum(Fd * Pd) - 0.5 * e1 + e_nuc
    return dict(e_uhf=e, iterations=step)
