"""FP64 closed-shell (spin-adapted) CCSD restatement (TEST INFRASTRUCTURE ONLY).

This is the same Jacobi iteration map as the reference's spin-orbital CCSD
(``ccsdt.cpp:380-727`` with the driver of ``ccsd_memory_optimized.cpp:473-557``),
written over spatial orbitals for a closed-shell determinant.  The CCSD
residual projections are unique polynomials in (T1, T2), and both codes move
exactly the diagonal Fock terms into the denominators D_i^a = f_ii - f_aa and
D_ij^ab = f_ii + f_jj - f_aa - f_bb, so every iterate -- not only the fixed
point -- agrees with the spin-orbital form (t(ia jb, alpha beta) = t2[i,j,a,b]).
The residual is organised with Stanton-Gauss style spin-adapted
intermediates (published closed-shell CCSD; J. F. Stanton, J. Gauss,
J. D. Watts, R. J. Bartlett, J. Chem. Phys. 94, 4334 (1991), spin-adapted);
the particle-particle ladder contracts the bare (ac|bd) with tau and applies
the T1 dressing through one o^3 v^3 contraction, as the reference contracts
bare <ab||cd> with tau (``ccsd_memory_optimized.cpp:2093``).

Off-diagonal Fock blocks are treated exactly here; the reference adds
(1 - delta_ac) f_ac without t_i^c (``ccsdt.cpp:400``), so only a diagonal Fock
matrix is a parity case.  As in the reference driver the energy omits the
f_ia t_i^a term (``ccsd_memory_optimized.cpp:646``).

variant="memory_optimized" iterates the map of the reference's class
CCSD_Memory_optimized as written instead of the CCSD equations: its
Fill_t2_new contracts the occupied Fock intermediate transposed,
R_ij^ab += sum_k t_jk^ab F_ik - sum_k t_ik^ab F_jk, in all six spin cases
(``ccsd_memory_optimized.cpp:2085-2086, 2143-2144, 2193-2194, 2269-2270,
2324-2325, 2375-2376``: ``D2.row(i/2)`` where ``D2(k, i)`` holds F_ki), while
its T1 equation keeps F_ki (``:2444``).  In the closed-shell form this is
Loo'[i,k] in place of Loo'[k,i] in the T2 residual.

Index conventions: t1[i, a], t2[i, j, a, b] with t2[i,j,a,b] = t2[j,i,b,a];
integral blocks in chemist notation, e.g. ovov[i,a,j,b] = (ia|jb).
"""
from __future__ import annotations

import numpy as np

ES = dict(optimize=True)


class Blocks:
    """Spatial chemist-notation integral blocks for one closed-shell system.

    With ``with_vvvv=False`` (DF input only) the v^4 block is not formed; the
    particle-particle ladder is then available row by row through
    ``RHFCCSD.ladder_rows`` (used to time a bounded sample of the largest
    shapes on the CPU)."""

    def __init__(self, eri=None, nocc=None, df=None, with_vvvv=True):
        self.df = df
        if eri is not None:
            o = nocc
            n = eri.shape[0]
            O, V = slice(0, o), slice(o, n)
            self.ovov = np.ascontiguousarray(eri[O, V, O, V])
            self.oovv = np.ascontiguousarray(eri[O, O, V, V])
            self.ovoo = np.ascontiguousarray(eri[O, V, O, O])
            self.oooo = np.ascontiguousarray(eri[O, O, O, O])
            self.ovvv = np.ascontiguousarray(eri[O, V, V, V])
            self.vvvv = np.ascontiguousarray(eri[V, V, V, V])
        else:
            b = df
            o = nocc
            bo = b[:, :o, :o]
            bov = b[:, :o, o:]
            bvv = b[:, o:, o:]
            e = lambda x, y: np.einsum("Qpq,Qrs->pqrs", x, y, optimize=True)
            self.ovov = e(bov, bov)
            self.oovv = e(bo, bvv)
            self.ovoo = e(bov, bo)
            self.oooo = e(bo, bo)
            self.ovvv = e(bov, bvv)
            self.vvvv = e(bvv, bvv) if with_vvvv else None


class RHFCCSD:
    def __init__(self, fock: np.ndarray, nocc: int, eri=None, df=None, with_vvvv=True, variant="ccsd"):
        if variant not in ("ccsd", "memory_optimized"):
            raise ValueError("variant must be 'ccsd' or 'memory_optimized'")
        self.variant = variant
        self.o = nocc
        self.n = fock.shape[0]
        self.v = self.n - nocc
        o = nocc
        self.f_oo = fock[:o, :o].copy()
        self.f_vv = fock[o:, o:].copy()
        self.f_ov = fock[:o, o:].copy()
        self.eo = np.diag(fock)[:o].copy()
        self.ev = np.diag(fock)[o:].copy()
        self.d1 = self.eo[:, None] - self.ev[None, :]
        self.d2 = self.d1[:, None, :, None] + self.d1[None, :, None, :]
        self.B = Blocks(eri=eri, nocc=nocc, df=df, with_vvvv=with_vvvv)

    def ladder_rows(self, tau, a0: int, a1: int):
        """sum_cd (ac|bd) tau[i,j,c,d] for a in [a0, a1), building the needed
        (ac|bd) rows from the DF factors; returns [i, j, a - a0, b]."""
        o = self.o
        bvv = self.B.df[:, o:, o:]
        w = np.einsum("Qac,Qbd->acbd", bvv[:, a0:a1], bvv, optimize=True)
        return np.einsum("acbd,ijcd->ijab", w, tau, optimize=True)

    def tau(self, t1, t2):
        return t2 + np.einsum("ia,jb->ijab", t1, t1)

    def energy(self, t1, t2):
        ovov = self.B.ovov
        L = 2.0 * ovov - ovov.transpose(0, 3, 2, 1)  # 2(ia|jb) - (ib|ja)
        return np.einsum("iajb,ijab->", L, self.tau(t1, t2), **ES)

    def mp2_guess(self):
        t2 = self.B.ovov.transpose(0, 2, 1, 3) / self.d2
        return np.zeros((self.o, self.v)), t2

    def residual(self, t1, t2):
        """Return (R1, R2) with the diagonal Fock terms moved out, i.e. the
        Jacobi numerators: t1_new = R1 / D1, t2_new = R2 / D2."""
        B = self.B
        ovov, oovv, ovoo, oooo, ovvv, vvvv = B.ovov, B.oovv, B.ovoo, B.oooo, B.ovvv, B.vvvv
        fov = self.f_ov
        tau = self.tau(t1, t2)
        Lovov = 2.0 * ovov - ovov.transpose(0, 3, 2, 1)      # L[k,c,l,d] = 2(kc|ld)-(kd|lc)

        Foo = self.f_oo + np.einsum("kcld,ilcd->ki", Lovov, tau, **ES)
        Fvv = self.f_vv - np.einsum("kcld,klad->ac", Lovov, tau, **ES)
        Fov = fov + np.einsum("kcld,ld->kc", Lovov, t1, **ES)
        Loo = (Foo + np.einsum("kc,ic->ki", fov, t1, **ES)
               + 2.0 * np.einsum("lcki,lc->ki", ovoo, t1, **ES)
               - np.einsum("kcli,lc->ki", ovoo, t1, **ES))
        Lvv = (Fvv - np.einsum("kc,ka->ac", fov, t1, **ES)
               + 2.0 * np.einsum("kdac,kd->ac", ovvv, t1, **ES)
               - np.einsum("kcad,kd->ac", ovvv, t1, **ES))
        Foo_p = Foo - np.diag(self.eo)
        Fvv_p = Fvv - np.diag(self.ev)
        Loo_p = Loo - np.diag(self.eo)
        Lvv_p = Lvv - np.diag(self.ev)

        # ---- T1 ------------------------------------------------------------
        R1 = (fov.copy()
              - 2.0 * np.einsum("kc,ka,ic->ia", fov, t1, t1, **ES)
              + np.einsum("ac,ic->ia", Fvv_p, t1, **ES)
              - np.einsum("ki,ka->ia", Foo_p, t1, **ES)
              + np.einsum("kc,kica->ia", Fov, 2.0 * t2 - t2.transpose(1, 0, 2, 3), **ES)
              + np.einsum("kc,ic,ka->ia", Fov, t1, t1, **ES)
              + np.einsum("kcia,kc->ia", 2.0 * ovov, t1, **ES)
              - np.einsum("kiac,kc->ia", oovv, t1, **ES)
              + np.einsum("kdac,ikcd->ia", 2.0 * ovvv - ovvv.transpose(0, 3, 2, 1), tau, **ES)
              - np.einsum("lcki,klac->ia", 2.0 * ovoo - ovoo.transpose(2, 1, 0, 3), tau, **ES))

        # ---- intermediates for T2 -----------------------------------------
        Woooo = (oooo.transpose(0, 2, 1, 3)                        # (ki|lj) -> [k,l,i,j]
                 + np.einsum("lcki,jc->klij", ovoo, t1, **ES)
                 + np.einsum("kclj,ic->klij", ovoo, t1, **ES)
                 + np.einsum("kcld,ijcd->klij", ovov, tau, **ES))
        Wvoov = (ovov.transpose(1, 0, 2, 3)                         # (ai|kc) -> [a,i,k,c]
                 .transpose(0, 2, 1, 3)                             # -> [a,k,i,c]
                 + np.einsum("kcad,id->akic", ovvv, t1, **ES)
                 - np.einsum("kcli,la->akic", ovoo, t1, **ES)
                 - 0.5 * np.einsum("ldkc,ilda->akic", ovov, t2, **ES)
                 - 0.5 * np.einsum("lckd,ilad->akic", ovov, t2, **ES)
                 - np.einsum("ldkc,id,la->akic", ovov, t1, t1, **ES)
                 + np.einsum("ldkc,ilad->akic", ovov, t2, **ES))
        Wvovo = (oovv.transpose(2, 0, 3, 1)                         # (ki|ac) -> [a,k,c,i]
                 + np.einsum("kdac,id->akci", ovvv, t1, **ES)
                 - np.einsum("lcki,la->akci", ovoo, t1, **ES)
                 - 0.5 * np.einsum("lckd,ilda->akci", ovov, t2, **ES)
                 - np.einsum("lckd,id,la->akci", ovov, t1, t1, **ES))

        # ---- T2 ------------------------------------------------------------
        def P(x):
            return x + x.transpose(1, 0, 3, 2)

        tmpA = ovvv.transpose(1, 2, 0, 3) - np.einsum("kibc,ka->abic", oovv, t1, **ES)
        X = np.einsum("abic,jc->ijab", tmpA, t1, **ES)
        tmpB = np.einsum("kcai,jc->akij", ovov.transpose(0, 1, 3, 2), t1, **ES) + ovoo.transpose(1, 3, 0, 2)
        Y = np.einsum("akij,kb->ijab", tmpB, t1, **ES)
        R2 = ovov.transpose(0, 2, 1, 3).copy()                     # (ia|jb)
        R2 += P(X - Y)
        R2 += np.einsum("klij,klab->ijab", Woooo, tau, **ES)
        # particle-particle ladder with bare (ac|bd), then the T1 dressing
        if vvvv is not None:
            R2 += np.einsum("acbd,ijcd->ijab", vvvv, tau, **ES)
        elif not getattr(self, "skip_ladder", False):
            R2 += self.ladder_rows(tau, 0, self.v)
        Z = np.einsum("kdac,ijcd->ijka", ovvv, tau, **ES)           # sum_cd (ac|kd) tau_ij^cd
        R2 -= P(np.einsum("ijka,kb->ijab", Z, t1, **ES))
        R2 += P(np.einsum("ac,ijcb->ijab", Lvv_p, t2, **ES))
        if self.variant == "memory_optimized":  # F_ik, ccsd_memory_optimized.cpp:2085-2086
            R2 -= P(np.einsum("ik,kjab->ijab", Loo_p, t2, **ES))
        else:
            R2 -= P(np.einsum("ki,kjab->ijab", Loo_p, t2, **ES))
        R2 += P(np.einsum("akic,kjcb->ijab", 2.0 * Wvoov - Wvovo.transpose(0, 1, 3, 2), t2, **ES))
        R2 -= P(np.einsum("akic,kjbc->ijab", Wvoov, t2, **ES))
        R2 -= P(np.einsum("bkci,kjac->ijab", Wvovo, t2, **ES))
        return R1, R2

    def update(self, t1, t2):
        R1, R2 = self.residual(t1, t2)
        return R1 / self.d1, R2 / self.d2

    def run(self, toler: float = 1e-10, itermax: int = 1000, max_passes: int | None = None):
        """Same driver as the reference (see module docstring)."""
        t1, t2 = self.mp2_guess()
        e_new = self.energy(t1, t2)
        energies = [e_new]
        it = 1
        passes = 0
        while True:
            e_old = e_new
            t1, t2 = self.update(t1, t2)
            e_new = self.energy(t1, t2)
            it += 1
            passes += 1
            energies.append(e_new)
            if abs(e_new - e_old) < toler or it >= itermax:
                break
            if max_passes is not None and passes >= max_passes:
                break
        return dict(e_corr=e_new, energies=np.array(energies), iter=it, t1=t1, t2=t2)
