"""Host FP64 reference of the CCSD Lambda equations and dE_corr/d(inputs)
(TEST INFRASTRUCTURE ONLY).

The reference has no Lambda equations or gradients.  This restates the
closed-shell residual of oracle.ccsd_rhf in torch (FP64, CPU) and lets torch
autograd supply the vector-Jacobian products, independently of the engine's
hand-written adjoint tape:

    G(T; f, g) = R(T; f, g) - D(f) o T           (R: Jacobi numerator)
    Lambda = (dE/dT + (dR/dT)^T Lambda) / D      (Jacobi iteration)
    dE/dtheta = d/dtheta [ E(T; g) + Lambda^T G(T; f, g) ]  at fixed T, Lambda

with theta = (fock[n][n], eri[n][n][n][n]) as given, every element treated as
independent (the closed-shell equations read each block from fixed positions
of the dense tensor, exactly as the engine does).

Per-element derivatives depend on which of several equal-valued symmetric
copies a term reads.  The engine's particle-particle ladder works on
(ij,ab)-pairs and reads symmetrised inputs: the ladder of tau and
W[a][b][c][d] = (ac|bd) is sum_cd W_s[ab,cd] (P tau)[ij,cd] with
W_s = (W[abcd] + W[badc]) / 2 and (P tau)[ijcd] = (tau[ijcd] + tau[jidc]) / 2.
Both equal W and tau for symmetric integrals and amplitudes (energies and
amplitudes are unchanged); this restatement reads them the same way, so its
Lambda and per-element gradients are the engine's.  Sums of the gradient over
the 8 permutations of an integral do not depend on this choice.
"""
from __future__ import annotations

import numpy as np
import torch


def _blocks(eri, o):
    O, V = slice(0, o), slice(o, eri.shape[0])
    return dict(ovov=eri[O, V, O, V], oovv=eri[O, O, V, V], ovoo=eri[O, V, O, O], oooo=eri[O, O, O, O],
                ovvv=eri[O, V, V, V], vvvv=eri[V, V, V, V])


def numerators(t1, t2, fock, eri, o):
    """Jacobi numerators (R1, R2) of the closed-shell CCSD map (torch)."""
    E = torch.einsum
    B = _blocks(eri, o)
    ovov, oovv, ovoo, oooo, ovvv, vvvv = (B[k] for k in ("ovov", "oovv", "ovoo", "oooo", "ovvv", "vvvv"))
    f_oo, f_vv, fov = fock[:o, :o], fock[o:, o:], fock[:o, o:]
    eo, ev = torch.diagonal(fock)[:o], torch.diagonal(fock)[o:]
    tau = t2 + E("ia,jb->ijab", t1, t1)
    Lovov = 2.0 * ovov - ovov.permute(0, 3, 2, 1)
    Foo = f_oo + E("kcld,ilcd->ki", Lovov, tau)
    Fvv = f_vv - E("kcld,klad->ac", Lovov, tau)
    Fov = fov + E("kcld,ld->kc", Lovov, t1)
    Loo = Foo + E("kc,ic->ki", fov, t1) + 2.0 * E("lcki,lc->ki", ovoo, t1) - E("kcli,lc->ki", ovoo, t1)
    Lvv = Fvv - E("kc,ka->ac", fov, t1) + 2.0 * E("kdac,kd->ac", ovvv, t1) - E("kcad,kd->ac", ovvv, t1)
    Foo_p, Fvv_p = Foo - torch.diag(eo), Fvv - torch.diag(ev)
    Loo_p, Lvv_p = Loo - torch.diag(eo), Lvv - torch.diag(ev)
    R1 = (fov - 2.0 * E("kc,ka,ic->ia", fov, t1, t1) + E("ac,ic->ia", Fvv_p, t1) - E("ki,ka->ia", Foo_p, t1)
          + E("kc,kica->ia", Fov, 2.0 * t2 - t2.permute(1, 0, 2, 3)) + E("kc,ic,ka->ia", Fov, t1, t1)
          + 2.0 * E("kcia,kc->ia", ovov, t1) - E("kiac,kc->ia", oovv, t1)
          + E("kdac,ikcd->ia", 2.0 * ovvv - ovvv.permute(0, 3, 2, 1), tau)
          - E("lcki,klac->ia", 2.0 * ovoo - ovoo.permute(2, 1, 0, 3), tau))
    Woooo = (oooo.permute(0, 2, 1, 3) + E("lcki,jc->klij", ovoo, t1) + E("kclj,ic->klij", ovoo, t1)
             + E("kcld,ijcd->klij", ovov, tau))
    Wvoov = (ovov.permute(1, 0, 2, 3).permute(0, 2, 1, 3) + E("kcad,id->akic", ovvv, t1)
             - E("kcli,la->akic", ovoo, t1) - 0.5 * E("ldkc,ilda->akic", ovov, t2)
             - 0.5 * E("lckd,ilad->akic", ovov, t2) - E("ldkc,id,la->akic", ovov, t1, t1)
             + E("ldkc,ilad->akic", ovov, t2))
    Wvovo = (oovv.permute(2, 0, 3, 1) + E("kdac,id->akci", ovvv, t1) - E("lcki,la->akci", ovoo, t1)
             - 0.5 * E("lckd,ilda->akci", ovov, t2) - E("lckd,id,la->akci", ovov, t1, t1))

    def P(x):
        return x + x.permute(1, 0, 3, 2)

    tmpA = ovvv.permute(1, 2, 0, 3) - E("kibc,ka->abic", oovv, t1)
    X = E("abic,jc->ijab", tmpA, t1)
    tmpB = E("kcai,jc->akij", ovov.permute(0, 1, 3, 2), t1) + ovoo.permute(1, 3, 0, 2)
    Y = E("akij,kb->ijab", tmpB, t1)
    vvvv_s = 0.5 * (vvvv + vvvv.permute(2, 3, 0, 1))      # W_s in (ac|bd) order
    tau_s = 0.5 * (tau + tau.permute(1, 0, 3, 2))          # P tau
    R2 = ovov.permute(0, 2, 1, 3) + P(X - Y) + E("klij,klab->ijab", Woooo, tau) + E("acbd,ijcd->ijab", vvvv_s, tau_s)
    Z = E("kdac,ijcd->ijka", ovvv, tau)
    R2 = R2 - P(E("ijka,kb->ijab", Z, t1)) + P(E("ac,ijcb->ijab", Lvv_p, t2)) - P(E("ki,kjab->ijab", Loo_p, t2))
    R2 = R2 + P(E("akic,kjcb->ijab", 2.0 * Wvoov - Wvovo.permute(0, 1, 3, 2), t2))
    R2 = R2 - P(E("akic,kjbc->ijab", Wvoov, t2)) - P(E("bkci,kjac->ijab", Wvovo, t2))
    D1 = eo[:, None] - ev[None, :]
    D2 = D1[:, None, :, None] + D1[None, :, None, :]
    return R1, R2, D1, D2


def energy(t1, t2, eri, o):
    ovov = _blocks(eri, o)["ovov"]
    L = 2.0 * ovov - ovov.permute(0, 3, 2, 1)
    return torch.einsum("iajb,ijab->", L, t2 + torch.einsum("ia,jb->ijab", t1, t1))


def lambda_grad(fock: np.ndarray, eri: np.ndarray, nocc: int, t1: np.ndarray, t2: np.ndarray,
                tol: float = 1e-11, max_iter: int = 500):
    """Lambda amplitudes and dE/dfock, dE/deri at the converged (t1, t2)."""
    o = nocc
    f = torch.tensor(fock, dtype=torch.float64)
    g = torch.tensor(eri, dtype=torch.float64)
    T1 = torch.tensor(t1, dtype=torch.float64, requires_grad=True)
    T2 = torch.tensor(t2, dtype=torch.float64, requires_grad=True)
    e = energy(T1, T2, g, o)
    dE1, dE2 = torch.autograd.grad(e, (T1, T2))
    R1, R2, D1, D2 = numerators(T1, T2, f, g, o)
    l1, l2 = torch.zeros_like(dE1), torch.zeros_like(dE2)
    it = 0
    for it in range(1, max_iter + 1):
        j1, j2 = torch.autograd.grad((R1, R2), (T1, T2), grad_outputs=(l1, l2), retain_graph=True)
        n1, n2 = (dE1 + j1) / D1, (dE2 + j2) / D2
        d = torch.sqrt(((n1 - l1) ** 2).sum() + ((n2 - l2) ** 2).sum()).item()
        l1, l2 = n1, n2
        if d < tol:
            break
    fq = f.clone().requires_grad_(True)
    gq = g.clone().requires_grad_(True)
    R1, R2, D1, D2 = numerators(T1.detach(), T2.detach(), fq, gq, o)
    lag = (energy(T1.detach(), T2.detach(), gq, o) + (l1 * (R1 - D1 * T1.detach())).sum()
           + (l2 * (R2 - D2 * T2.detach())).sum())
    dfock, deri = torch.autograd.grad(lag, (fq, gq))
    return dict(lambda1=l1.numpy(), lambda2=l2.numpy(), d_fock=dfock.numpy(), d_eri=deri.numpy(), iterations=it)
