"""FP64 spin-orbital CCSD restatement of the reference (TEST INFRASTRUCTURE ONLY).

Equations: the reference's dense spin-orbital CCSD, ``CCSDT::Calc_Energy`` with
``Method_Nr == -1`` ("CCSD1", ``initializer.cpp:98-103``):

* antisymmetrised integrals <pq||rs> from spatial chemist (pq|rs), alpha/beta
  interleaved (spin-orbital p -> spatial p//2, spin p%2)    ``ccsdt.cpp:1466-1478``
* diagonal spin-orbital Fock fs(p,p) = eps(p//2)                ``ccsdt.cpp:1510-1516``
* F1/F2/F3 (D1 = F_me, D2 = F_mi, D3 = F_ae)                   ``ccsdt.cpp:2529-2600``
* W1 (W_mnij), W2, W3, W4 (W_mbej)                             ``ccsdt.cpp:2416-2526``
* T1 residual (only spin-allowed (a+i) even)                   ``ccsdt.cpp:380-444``
* T2 residual (a<b, i<j, (a+b+i+j) even, then the 4-fold
  antisymmetric copies)                                        ``ccsdt.cpp:625-727``
* tau = t2 + t1 t1 - t1 t1                                     ``ccsdt.cpp:2603-2620``
* MP2 initial T2, T1 = 0                                       ``ccsdt.cpp:172-192``
* CCSDT-1a (``Method_Nr == 1``): T3 from the bare integrals and T2
  (X1(b,c)(k,e) = <bc||ek>, X2(c,m)(j,k) = <mc||jk>)            ``ccsdt.cpp:1960-2042, 995-1290``
  T3 -> T1: + 1/4 <jk||bc> t_ijk^abc                            ``ccsdt.cpp:419-434``
  T3 -> T2: + 1/2 P(ab) <bk||cd> t_ijk^acd - 1/2 P(ij) <km||jc> t_ikm^abc
                                                                ``ccsdt.cpp:640-670``
  Each pass forms T1/T2 from the previous T3 and T3 from the previous T2
  (``ccsdt.cpp:255-271``); T3 starts at zero.
* CCSDT-1b (``Method_Nr == 2``): CCSDT-1a plus the T3 T1 term of T2
  (``ccsdt.cpp:676-700``):
  + 1/2 <kl||cd> [- t_ikj^acd t_l^b + t_ikj^bcd t_l^a - t_klj^adb t_i^c
                  + t_kli^adb t_j^c + 2 t_ijk^abc t_l^d]
* CCSDT-2 (``Method_Nr == 3``): CCSDT-1b with T2-dressed X1/X2 and the X12/X13
  terms of T3 (``triples``).
* CCSDT-3 (``Method_Nr == 4``): CCSDT-2 with T1 terms in X12/X13 and the X14/X15
  terms of T3 (``triples``).
* CCSDT-4 (``Method_Nr == 5``): CCSDT-3 with the X3/X4/X6 terms of the previous T3
  in T3 (``triples``).
* CCSDT (``Method_Nr == 6``): CCSDT-4 with T3 terms in X1/X2, dressed X3/X4/X6 and
  the X7/X8 terms (``triples``), including the reference's X3 loop as written.

variant="memory_optimized" (CCSD only) is the map of the reference's class
CCSD_Memory_optimized as written: its Fill_t2_new contracts the F_mi
intermediate transposed, + sum_k t_jk^ab F_ik - sum_k t_ik^ab F_jk, in all six
spin cases (``ccsd_memory_optimized.cpp:2085-2086, 2143-2144, 2193-2194,
2269-2270, 2324-2325, 2375-2376``: ``D2.row(i/2)`` with ``D2(k, i)`` = F_ki);
its T1 equation keeps F_ki (``:2444``).

Driver semantics follow ``CCSD_Memory_optimized::CCSD``
(``ccsd_memory_optimized.cpp:473-557``): E = 1/4 sum <ij||ab> tau_ij^ab with
the f_ia t_i^a term dropped (``:646``); ``iter`` starts at 1, each pass adds 1,
the loop stops when |E_new - E_old| < toler or iter >= 1000 (``:552-556``).

Arrays use the reference's index order: t1[a, i], t2[a, b, i, j],
g[p, q, r, s] = <pq||rs>, with virtual indices offset by O (= n_Electrons).
Only practical for a few dozen spin orbitals (dense N^4 integrals).
"""
from __future__ import annotations

import numpy as np

ES = dict(optimize=True)


def spin_orbital_integrals(eri: np.ndarray) -> np.ndarray:
    """<pq||rs> over 2n interleaved spin orbitals from chemist (pq|rs)
    (``ccsdt.cpp:1466-1478``: MOs(a,i)(b,j) = d(a,b)d(i,j)(ab|ij) - d(a,j)d(i,b)(aj|ib))."""
    n = eri.shape[0]
    N = 2 * n
    sp = np.arange(N) // 2
    spin = np.arange(N) % 2
    same = (spin[:, None] == spin[None, :]).astype(np.float64)
    # <pq|rs> = (pr|qs) delta(sp,sr) delta(sq,ss)
    pr_qs = eri[np.ix_(sp, sp, sp, sp)]  # [p, r, q, s] = (pr|qs)
    direct = pr_qs.transpose(0, 2, 1, 3) * same[:, None, :, None] * same[None, :, None, :]
    return direct - direct.transpose(0, 1, 3, 2)


def spin_orbital_fock(fock: np.ndarray) -> np.ndarray:
    """fs(p,p) = eps(p/2) (``ccsdt.cpp:1510-1516``); off-diagonal spatial
    elements are carried on same-spin pairs (the reference only ever fills
    the diagonal)."""
    n = fock.shape[0]
    N = 2 * n
    sp = np.arange(N) // 2
    spin = np.arange(N) % 2
    return fock[np.ix_(sp, sp)] * (spin[:, None] == spin[None, :])


class SpinOrbitalCCSD:
    def __init__(self, fock: np.ndarray, eri: np.ndarray, nocc: int, method: int = -1, x3_as_written: bool = True,
                 variant: str = "ccsd"):
        """fock: spatial n x n; eri: spatial chemist (pq|rs); nocc spatial;
        method: -1 = CCSD ("CCSD1"), 1 = CCSDT-1a, 2 = CCSDT-1b, 3 = CCSDT-2, 4 = CCSDT-3,
        5 = CCSDT-4, 6 = CCSDT (the reference's Method_Nr)."""
        if method not in (-1, 1, 2, 3, 4, 5, 6):
            raise ValueError("method must be -1 (CCSD1) or 1-6 (CCSDT-1a, -1b, -2, -3, -4, CCSDT)")
        if variant not in ("ccsd", "memory_optimized") or (variant != "ccsd" and method != -1):
            raise ValueError("variant must be 'ccsd', or 'memory_optimized' with method -1")
        self.variant = variant
        self.method = method
        # CCSDT's X3 tau term: the reference's loop (e fixed at the first virtual) or the
        # sum over all (d, e) that the equations state
        self.x3_as_written = x3_as_written
        self.fs = spin_orbital_fock(fock)
        self.g = spin_orbital_integrals(eri)
        self.O = 2 * nocc
        self.N = self.fs.shape[0]
        O, N = self.O, self.N
        self.V = N - O
        o, v = slice(0, O), slice(O, N)
        g = self.g
        self.goooo = g[o, o, o, o]
        self.gooov = g[o, o, o, v]
        self.goovo = g[o, o, v, o]
        self.goovv = g[o, o, v, v]
        self.govoo = g[o, v, o, o]
        self.govov = g[o, v, o, v]
        self.govvo = g[o, v, v, o]
        self.govvv = g[o, v, v, v]
        self.gvooo = g[v, o, o, o]
        self.gvovo = g[v, o, v, o]
        self.gvoov = g[v, o, o, v]
        self.gvovv = g[v, o, v, v]
        self.gvvoo = g[v, v, o, o]
        self.gvvvo = g[v, v, v, o]
        self.gvvvv = g[v, v, v, v]
        self.f_vo = self.fs[v, o]
        self.f_oo = self.fs[o, o]
        self.f_vv = self.fs[v, v]
        eo = np.diag(self.fs)[o]
        ev = np.diag(self.fs)[v]
        self.den = eo[None, :] - ev[:, None]  # den[a, i] = fs(i,i) - fs(a,a)
        ai = (np.arange(O, N)[:, None] + np.arange(O)[None, :]) % 2 == 0
        self.t1_mask = ai
        a_idx = np.arange(O, N)
        i_idx = np.arange(O)
        par = (a_idx[:, None, None, None] + a_idx[None, :, None, None]
               + i_idx[None, None, :, None] + i_idx[None, None, None, :]) % 2 == 0
        upper = (a_idx[:, None, None, None] < a_idx[None, :, None, None]) & \
                (i_idx[None, None, :, None] < i_idx[None, None, None, :])
        self.t2_write = par & upper

    # -- amplitudes ---------------------------------------------------------
    def mp2_guess(self):
        """t2(a,b)(i,j) = <ab||ij> / (den(a,i) + den(b,j)), t1 = 0."""
        d2 = self.den[:, None, :, None] + self.den[None, :, None, :]
        t2 = self.gvvoo / d2
        t2 = np.where(self.full_mask(), t2, 0.0)
        return np.zeros((self.V, self.O)), t2

    def full_mask(self):
        w = self.t2_write
        return w | w.transpose(1, 0, 2, 3) | w.transpose(0, 1, 3, 2) | w.transpose(1, 0, 3, 2)

    def tau(self, t1, t2):
        return t2 + np.einsum("ai,bj->abij", t1, t1) - np.einsum("aj,bi->abij", t1, t1)

    def energy(self, t1, t2):
        """1/4 sum <ij||ab> tau_ij^ab; the f_ia t_i^a term is dropped as in
        ``ccsd_memory_optimized.cpp:646``."""
        return 0.25 * np.einsum("ijab,abij->", self.goovv, self.tau(t1, t2))

    def triples(self, t2, t1=None, t3=None):
        """T3 from T2 (``ccsdt.cpp:995-1290``): t3[a,b,c,i,j,k] =
        [P(a/bc) P(k/ij) sum_e X1(b,c)(k,e) t2(a,e)(i,j) - P(c/ab) P(i/jk) sum_m X2(c,m)(j,k) t2(a,b)(i,m)
         (+ for CCSDT-2, Method_Nr 3: P(i/jk) P(abc) sum_e X12(a,b)(i,e) t2(e,c)(j,k)
                                    + P(a/bc) P(ijk) sum_m X13(a,m)(i,j) t2(b,c)(m,k))] / D3
        X1(b,c)(k,e) = <bc||ek> and X2(c,m)(j,k) = <mc||jk> for CCSDT-1a/1b; CCSDT-2
        dresses them with T2 (``ccsdt.cpp:1960-2040``):
          X1 += 1/2 sum_lm <lm||ek> t2(b,c)(l,m),  X2 += 1/2 sum_de t2(d,e)(j,k) <mc||de>
          X12(a,b)(i,d) = sum_le <lb||ed> t2(a,e)(i,l),  X13(a,l)(i,j) = -sum_md <ml||dj> t2(a,d)(i,m)
                                                                      ``ccsdt.cpp:2301-2390``
        CCSDT-3 (Method_Nr 4) adds T1 terms to X12/X13 and, with the antisymmetrisers
        of X1 and X2, P(c/ab) P(i/jk) sum_e X14(a,b)(i,e) t2(e,c)(j,k) and
        P(a/bc) P(k/ij) sum_m X15(a,m)(i,j) t2(b,c)(m,k)       ``ccsdt.cpp:1028-1070, 2043-2125``
          X14(a,b)(i,d) = sum_e <ab||ed> t1(e,i) + sum_elm <lm||ed> [t1(e,i) t1(a,l) t1(b,m)
                          - t1(e,l) t2(a,b)(i,m) + 1/2 t1(e,i) t2(a,b)(l,m)] + sum_lm <lm||id> t1(a,l) t1(b,m)
          X15(a,l)(i,j) = -sum_de <al||de> t1(d,i) t1(e,j) + sum_m <ml||ij> t1(a,m)
                          + 1/2 sum_mde <ml||de> t1(a,m) tau(d,e)(i,j)
        CCSDT-4 (Method_Nr 5) adds terms of the previous T3 (``ccsdt.cpp:1134-1180``) with the
        bare X3(i,j)(l,m) = 1/2 <ij||lm>, X4(a,b)(d,e) = 1/2 <ab||de>, X6(a,l)(i,d) = <al||id>
        (``ccsdt.cpp:2185-2300``):
          P(c/ab) sum_de X4(a,b)(d,e) t3(dec,ijk) + P(k/ij) sum_lm X3(i,j)(l,m) t3(abc,lmk)
          + P(i/jk) P(a/bc) sum_ld X6(a,l)(i,d) t3(dbc,ljk)
        CCSDT (Method_Nr 6) dresses X1, X2 with T3 and X3, X4, X6 with T1/T2, and adds
        P(a/bc) sum_d X8(a,d) t3(dbc,ijk) + P(i/jk) sum_m X7(i,m) t3(abc,mjk)
                                                        ``ccsdt.cpp:1183-1200, 1960-2040, 2128-2300``"""
        X1, X2 = self.gvvvo, self.govoo  # X1 at [b,c,e,k], X2 at [m,c,j,k]
        if self.method >= 3:
            X1 = X1 + 0.5 * np.einsum("lmek,bclm->bcek", self.goovo, t2, **ES)
            X2 = X2 + 0.5 * np.einsum("dejk,mcde->mcjk", t2, self.govvv, **ES)
        if self.method >= 6 and t3 is not None:  # ccsdt.cpp:1982-1988, 2020-2030
            X1 = X1 - 0.5 * np.einsum("lmde,beclmk->bcdk", self.goovv, t3, **ES)
            X2 = X2 + 0.5 * np.einsum("lmde,decjmk->lcjk", self.goovv, t3, **ES)
        A = np.einsum("bcek,aeij->abcijk", X1, t2, **ES)
        B = np.einsum("mcjk,abim->abcijk", X2, t2, **ES)
        if self.method >= 4:
            tau = self.tau(t1, t2)
            X14 = (np.einsum("abed,ei->abid", self.gvvvv, t1, **ES)
                   + np.einsum("lmed,ei,al,bm->abid", self.goovv, t1, t1, t1, **ES)
                   - np.einsum("lmed,el,abim->abid", self.goovv, t1, t2, **ES)
                   + 0.5 * np.einsum("lmed,ei,ablm->abid", self.goovv, t1, t2, **ES)
                   + np.einsum("lmid,al,bm->abid", self.gooov, t1, t1, **ES))
            X15 = (-np.einsum("alde,di,ej->alij", self.gvovv, t1, t1, **ES)
                   + np.einsum("mlij,am->alij", self.goooo, t1, **ES)
                   + 0.5 * np.einsum("mlde,am,deij->alij", self.goovv, t1, tau, **ES))
            A = A + np.einsum("amij,bcmk->abcijk", X15, t2, **ES)   # same antisymmetriser as the X1 term
            B = B - np.einsum("abie,ecjk->abcijk", X14, t2, **ES)   # same as the X2 term, opposite sign
        PA = A - A.transpose(1, 0, 2, 3, 4, 5) - A.transpose(2, 1, 0, 3, 4, 5)     # P(a/bc)
        PA = PA - PA.transpose(0, 1, 2, 5, 4, 3) - PA.transpose(0, 1, 2, 3, 5, 4)  # P(k/ij)
        PB = B - B.transpose(2, 1, 0, 3, 4, 5) - B.transpose(0, 2, 1, 3, 4, 5)     # P(c/ab)
        PB = PB - PB.transpose(0, 1, 2, 4, 3, 5) - PB.transpose(0, 1, 2, 5, 4, 3)  # P(i/jk)
        num = PA - PB
        if self.method >= 3:
            X12 = np.einsum("lbed,aeil->abid", self.govvv, t2, **ES)
            X13 = -np.einsum("mldj,adim->alij", self.goovo, t2, **ES)
            if self.method >= 4:  # ccsdt.cpp:2321-2333, 2365-2383
                X12 = (X12 - np.einsum("alid,bl->abid", self.gvoov, t1, **ES)
                       - np.einsum("lbed,ei,al->abid", self.govvv, t1, t1, **ES)
                       - np.einsum("lmed,bm,aeil->abid", self.goovv, t1, t2, **ES))
                X13 = (X13 + np.einsum("mldj,di,am->alij", self.goovo, t1, t1, **ES)
                       - np.einsum("mlde,adim,ej->alij", self.goovv, t2, t1, **ES)
                       - np.einsum("alid,dj->alij", self.gvoov, t1, **ES))
            Q = np.einsum("abie,ecjk->abcijk", X12, t2, **ES)
            # P(abc): all six orders of the virtual indices with their signs
            Q = (Q - Q.transpose(1, 0, 2, 3, 4, 5) - Q.transpose(2, 1, 0, 3, 4, 5) - Q.transpose(0, 2, 1, 3, 4, 5)
                 + Q.transpose(1, 2, 0, 3, 4, 5) + Q.transpose(2, 0, 1, 3, 4, 5))
            Q = Q - Q.transpose(0, 1, 2, 4, 3, 5) - Q.transpose(0, 1, 2, 5, 4, 3)  # P(i/jk)
            S = np.einsum("amij,bcmk->abcijk", X13, t2, **ES)
            S = S - S.transpose(1, 0, 2, 3, 4, 5) - S.transpose(2, 1, 0, 3, 4, 5)  # P(a/bc)
            # P(ijk): all six orders of the occupied indices with their signs
            S = (S - S.transpose(0, 1, 2, 4, 3, 5) - S.transpose(0, 1, 2, 5, 4, 3) - S.transpose(0, 1, 2, 3, 5, 4)
                 + S.transpose(0, 1, 2, 4, 5, 3) + S.transpose(0, 1, 2, 5, 3, 4))
            num = num + Q + S
        if self.method >= 5 and t3 is not None:
            X3, X4, X6 = 0.5 * self.goooo, 0.5 * self.gvvvv, self.gvoov
            if self.method >= 6:  # ccsdt.cpp:2128-2300
                tau = self.tau(t1, t2)
                # X3: the reference's tau loop runs "for (e = n_Electrons; d < Matrix_Size; d++)",
                # so e stays at the first virtual and d runs over all virtuals once
                x3tau = (np.einsum("lmd,dij->ijlm", self.goovv[:, :, :, 0], tau[:, 0], **ES) if self.x3_as_written
                         else np.einsum("lmde,deij->ijlm", self.goovv, tau, **ES))
                X3 = (X3 + 0.5 * x3tau
                      + np.einsum("lmdj,di->ijlm", self.goovo, t1, **ES)
                      - np.einsum("lmdi,dj->ijlm", self.goovo, t1, **ES))
                X4 = (X4 + 0.5 * np.einsum("lmde,ablm->abde", self.goovv, tau, **ES)
                      + np.einsum("lbde,al->abde", self.govvv, t1, **ES)
                      - np.einsum("lade,bl->abde", self.govvv, t1, **ES))
                X6 = (X6 + np.einsum("mled,aeim->alid", self.goovv, t2, **ES)
                      - np.einsum("mled,ei,am->alid", self.goovv, t1, t1, **ES)
                      + np.einsum("aled,ei->alid", self.gvovv, t1, **ES)
                      - np.einsum("mlid,am->alid", self.gooov, t1, **ES))
                X7 = (-0.5 * np.einsum("lmde,deli->im", self.goovv, tau, **ES)
                      - np.einsum("lmdi,dl->im", self.goovo, t1, **ES))
                X8 = (np.einsum("lade,dl->ae", self.govvv, t1, **ES)
                      - 0.5 * np.einsum("lmde,dalm->ae", self.goovv, tau, **ES)
                      - np.einsum("le,al->ae", self.fs[:self.O, self.O:], t1, **ES))
                W = np.einsum("ad,dbcijk->abcijk", X8, t3, **ES)
                num = num + W - W.transpose(1, 0, 2, 3, 4, 5) - W.transpose(2, 1, 0, 3, 4, 5)  # P(a/bc)
                W = np.einsum("im,abcmjk->abcijk", X7, t3, **ES)
                num = num + W - W.transpose(0, 1, 2, 4, 3, 5) - W.transpose(0, 1, 2, 5, 4, 3)  # P(i/jk)
            W = np.einsum("abde,decijk->abcijk", X4, t3, **ES)
            num = num + W - W.transpose(2, 1, 0, 3, 4, 5) - W.transpose(0, 2, 1, 3, 4, 5)      # P(c/ab)
            W = np.einsum("ijlm,abclmk->abcijk", X3, t3, **ES)
            num = num + W - W.transpose(0, 1, 2, 5, 4, 3) - W.transpose(0, 1, 2, 3, 5, 4)      # P(k/ij)
            W = np.einsum("alid,dbcljk->abcijk", X6, t3, **ES)
            W = W - W.transpose(1, 0, 2, 3, 4, 5) - W.transpose(2, 1, 0, 3, 4, 5)              # P(a/bc)
            num = num + W - W.transpose(0, 1, 2, 4, 3, 5) - W.transpose(0, 1, 2, 5, 4, 3)      # P(i/jk)
        d = self.den
        D3 = (d[:, None, None, :, None, None] + d[None, :, None, None, :, None] + d[None, None, :, None, None, :])
        return num / D3

    def update(self, t1, t2, t3=None):
        """One Jacobi pass: returns (t1_new, t2_new), or (t1_new, t2_new, t3_new)
        for CCSDT-1a (T1/T2 from the given t3, T3 from the given t2)."""
        fs_vo, f_oo, f_vv = self.f_vo, self.f_oo, self.f_vv
        O, V = self.O, self.V
        tau = self.tau(t1, t2)
        offd_oo = f_oo * (1.0 - np.eye(O))
        offd_vv = f_vv * (1.0 - np.eye(V))
        # F1 (D1[c,k])  ccsdt.cpp:2529-2546
        D1 = fs_vo + np.einsum("klcd,dl->ck", self.goovv, t1, **ES)
        # F2 (D2[k,i])  ccsdt.cpp:2549-2573
        D2 = (offd_oo + np.einsum("ci,ck->ki", t1, D1, **ES)
              + np.einsum("ickl,cl->ki", self.govoo, t1, **ES)
              + 0.5 * np.einsum("klcd,cdil->ki", self.goovv, t2, **ES))
        # F3 (D3[a,c])  ccsdt.cpp:2576-2600
        D3 = (offd_vv - np.einsum("ak,ck->ac", t1, D1, **ES)
              + np.einsum("akcd,dk->ac", self.gvovv, t1, **ES)
              - 0.5 * np.einsum("klcd,adkl->ac", self.goovv, t2, **ES))
        # W1[i,j,k,l]  ccsdt.cpp:2401-2424
        W1 = (self.goooo - np.einsum("jckl,ci->ijkl", self.govoo, t1, **ES)
              + np.einsum("ickl,cj->ijkl", self.govoo, t1, **ES)
              + 0.5 * np.einsum("klcd,cdij->ijkl", self.goovv, tau, **ES))
        # W2[a,k,i,j]  ccsdt.cpp:2427-2451
        W2 = (np.einsum("ijak->akij", self.goovo)
              + np.einsum("icak,cj->akij", self.govvo, t1, **ES)
              - np.einsum("jcak,ci->akij", self.govvo, t1, **ES)
              + 0.5 * np.einsum("akcd,cdij->akij", self.gvovv, tau, **ES))
        # W3[c,i,k,l]  ccsdt.cpp:2454-2473
        W3 = self.gvooo + np.einsum("cdkl,di->cikl", self.gvvoo, t1, **ES)
        # W4[a,k,i,c]  ccsdt.cpp:2476-2504
        W4 = (self.gvoov + np.einsum("kacd,di->akic", self.govvv, t1, **ES)
              - np.einsum("al,cikl->akic", t1, W3, **ES)
              + 0.5 * np.einsum("klcd,adil->akic", self.goovv, t2, **ES))
        # T1  ccsdt.cpp:383-441 (Method_Nr < 0 branch)
        R1 = (fs_vo - np.einsum("ak,ki->ai", t1, D2, **ES)
              + offd_vv.sum(axis=1)[:, None]  # sum_c (1-delta_ac) fs(a,c), no t1 (as in the reference)
              + np.einsum("cika,ck->ai", self.gvoov, t1, **ES)
              + np.einsum("acik,ck->ai", t2, D1, **ES)
              - 0.5 * np.einsum("cakl,cikl->ai", t2, W3, **ES)
              + 0.5 * np.einsum("kacd,cdki->ai", self.govvv, tau, **ES))
        if self.method >= 0 and t3 is not None:
            R1 = R1 + 0.25 * np.einsum("jkbc,abcijk->ai", self.goovv, t3, **ES)
        t1_new = np.where(self.t1_mask, R1 / self.den, 0.0)
        # T2  ccsdt.cpp:630-727 (Method_Nr < 0 branch)
        ring = np.einsum("bcjk,akic->abij", t2, W4, **ES)
        R2 = (np.einsum("ijab->abij", self.goovv)
              + 0.5 * np.einsum("abkl,ijkl->abij", tau, W1, **ES)
              - np.einsum("bk,akij->abij", t1, W2, **ES)
              + np.einsum("ak,bkij->abij", t1, W2, **ES)
              + np.einsum("abjk,ki->abij", t2, D2 if self.variant == "ccsd" else D2.T, **ES)
              - np.einsum("abik,kj->abij", t2, D2 if self.variant == "ccsd" else D2.T, **ES)
              + ring - ring.transpose(1, 0, 2, 3) - ring.transpose(0, 1, 3, 2)
              + ring.transpose(1, 0, 3, 2)
              - np.einsum("bcij,ac->abij", t2, D3, **ES)
              + np.einsum("acij,bc->abij", t2, D3, **ES)
              + np.einsum("abcj,ci->abij", self.gvvvo, t1, **ES)
              - np.einsum("abci,cj->abij", self.gvvvo, t1, **ES)
              + 0.5 * np.einsum("abcd,cdij->abij", self.gvvvv, tau, **ES))
        if self.method >= 0 and t3 is not None:
            R2 = (R2 + 0.5 * np.einsum("bkcd,acdijk->abij", self.gvovv, t3, **ES)
                  - 0.5 * np.einsum("akcd,bcdijk->abij", self.gvovv, t3, **ES)
                  - 0.5 * np.einsum("kmjc,abcikm->abij", self.gooov, t3, **ES)
                  + 0.5 * np.einsum("kmic,abcjkm->abij", self.gooov, t3, **ES))
        if self.method >= 2 and t3 is not None:  # ccsdt.cpp:676-700
            g = self.goovv
            R2 = R2 + 0.5 * (-np.einsum("klcd,acdikj,bl->abij", g, t3, t1, **ES)
                             + np.einsum("klcd,bcdikj,al->abij", g, t3, t1, **ES)
                             - np.einsum("klcd,adbklj,ci->abij", g, t3, t1, **ES)
                             + np.einsum("klcd,adbkli,cj->abij", g, t3, t1, **ES)
                             + 2.0 * np.einsum("klcd,abcijk,dl->abij", g, t3, t1, **ES))
        d2 = self.den[:, None, :, None] + self.den[None, :, None, :]
        val = np.where(self.t2_write, R2 / np.where(self.t2_write, d2, 1.0), 0.0)
        # symmetric copies (ccsdt.cpp:720-723)
        t2_new = val - val.transpose(1, 0, 2, 3) - val.transpose(0, 1, 3, 2) + val.transpose(1, 0, 3, 2)
        if self.method >= 0:
            return t1_new, t2_new, self.triples(t2, t1, t3)
        return t1_new, t2_new

    def closed_shell(self, t1, t2):
        """The spin-orbital t1, t2 a closed-shell engine works from: only the
        closed-shell amplitudes t1[i,a] = t1(2a,2i) and t2[i,j,a,b] =
        (t2(2a,2b+1,2i,2j+1) + t2(2b,2a+1,2j,2i+1)) / 2 (one amplitude for the pair
        t2[i,j,a,b] = t2[j,i,b,a]; the two differ only where the reference's X3 loop,
        ccsdt.cpp:2199-2206, breaks the alpha/beta symmetry) are kept, and expanded back as
        t1(A,I) = t1[I',A'] d(sA,sI),
        t2(A,B,I,J) = t2[I',J',A',B'] d(sA,sI) d(sB,sJ) - t2[J',I',A',B'] d(sA,sJ) d(sB,sI)."""
        t1s = np.zeros_like(t1)
        t1s[0::2, 0::2] = t1[0::2, 0::2]
        t1s[1::2, 1::2] = t1[0::2, 0::2]
        sp = t2[0::2, 1::2, 0::2, 1::2].transpose(2, 3, 0, 1)      # t2[i, j, a, b]
        sp = 0.5 * (sp + sp.transpose(1, 0, 3, 2))
        V, O = t2.shape[0], t2.shape[2]
        sa = np.arange(V) % 2
        si = np.arange(O) % 2
        A = np.arange(V) // 2
        I = np.arange(O) // 2
        direct = sp[I[None, None, :, None], I[None, None, None, :], A[:, None, None, None], A[None, :, None, None]]
        swapped = sp[I[None, None, None, :], I[None, None, :, None], A[:, None, None, None], A[None, :, None, None]]
        d1 = (sa[:, None, None, None] == si[None, None, :, None]) & (sa[None, :, None, None] == si[None, None, None, :])
        d2 = (sa[:, None, None, None] == si[None, None, None, :]) & (sa[None, :, None, None] == si[None, None, :, None])
        return t1s, np.where(d1, direct, 0.0) - np.where(d2, swapped, 0.0)

    def run(self, toler: float = 1e-10, itermax: int = 1000, max_passes: int | None = None,
            closed_shell: bool = False):
        """Reference driver loop. Returns dict with e_corr, energies (per
        ``iter``), iter (reference counter), t1, t2.  closed_shell: after every
        pass keep only the closed-shell amplitudes of T1/T2 (as a spin-adapted
        engine does, ``closed_shell()``), T3 as formed."""
        t1, t2 = self.mp2_guess()
        t3 = np.zeros((self.V,) * 3 + (self.O,) * 3) if self.method >= 0 else None
        e_new = self.energy(t1, t2)
        energies = [e_new]
        it = 1
        passes = 0
        while True:
            e_old = e_new
            if self.method >= 0:
                t1, t2, t3 = self.update(t1, t2, t3)
            else:
                t1, t2 = self.update(t1, t2)
            if closed_shell:
                t1, t2 = self.closed_shell(t1, t2)
            e_new = self.energy(t1, t2)
            it += 1
            passes += 1
            energies.append(e_new)
            if abs(e_new - e_old) < toler or it >= itermax:
                break
            if max_passes is not None and passes >= max_passes:
                break
        return dict(e_corr=e_new, energies=np.array(energies), iter=it, t1=t1, t2=t2, t3=t3)
