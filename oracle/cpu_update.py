"""Complete FP64 amplitude updates on the host cores (TEST INFRASTRUCTURE ONLY).

The timed CPU implementation of ``bench.py`` (its ``cpu_baseline`` object and
the ``--impl reference`` arm).  The reference's own CCSD keeps spin-orbital
arrays that cannot hold the nocc = 24 / nvir = 300 benchmark system (the v^4
spin-orbital block alone would be ~1 TB) and it cannot be compiled on the GPU
host (its sources are not there), so the timed implementation is this
repository's FP64 closed-shell restatement of the same map
(``oracle.ccsd_rhf.RHFCCSD.residual``, the Jacobi map of
``ccsd_memory_optimized.cpp:513-557`` over spatial orbitals), written for the
host's BLAS:

* every step is one whole update -- residual, denominators, DIIS extrapolation
  and energy -- with no term sampled or skipped;
* every o^3 v^3 and o^2 v^4 term is a matrix product on numpy's BLAS, all host
  threads; the contractions over a (c,d) or (k,l) pair of tau run in the same
  pair forms as the GPU engine with DF inputs, on tau+/tau- formed once per
  update: the particle-particle ladder (S+ = tau+ W+^T over c >= d, S- =
  tau- W-^T over c > d: a quarter of 2 o^2 v^4) with the hh ladder added to its
  halves, Z[i][j][k][a] = sum_cd (kd|ac) tau[ijcd] and X[k][l][i][j] =
  sum_cd (kc|ld) tau[ijcd] (half of their plain products);
* the integral blocks, W+/W- and the V+/V- and U+/U- packs of Z and X are built
  once, outside the timed steps, as the GPU engine builds them in ccsd_create.

``residual`` equals ``RHFCCSD.residual`` to rounding (tests/test_oracle.py).
"""
from __future__ import annotations

import os
import time

import numpy as np


def cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


class FullUpdate:
    """Closed-shell CCSD from a diagonal-or-not Fock matrix and DF factors
    B[Q][p][q]; t1[i,a], t2[i,j,a,b] as in ``oracle.ccsd_rhf``."""

    def __init__(self, fock: np.ndarray, nocc: int, df: np.ndarray, diis_size: int = 6, diis_start: int = 2):
        o = nocc
        n = fock.shape[0]
        v = n - o
        self.o, self.v = o, v
        self.f_oo = np.ascontiguousarray(fock[:o, :o])
        self.f_vv = np.ascontiguousarray(fock[o:, o:])
        self.f_ov = np.ascontiguousarray(fock[:o, o:])
        self.eo, self.ev = np.diag(fock)[:o].copy(), np.diag(fock)[o:].copy()
        self.d1 = self.eo[:, None] - self.ev[None, :]
        self.d2 = self.d1[:, None, :, None] + self.d1[None, :, None, :]
        naux = df.shape[0]
        bo = np.ascontiguousarray(df[:, :o, :o]).reshape(naux, o * o)
        bov = np.ascontiguousarray(df[:, :o, o:]).reshape(naux, o * v)
        bvv = np.ascontiguousarray(df[:, o:, o:])
        bvv2 = bvv.reshape(naux, v * v)
        self.ovov = (bov.T @ bov).reshape(o, v, o, v)
        self.oovv = (bo.T @ bvv2).reshape(o, o, v, v)
        self.ovoo = (bov.T @ bo).reshape(o, v, o, o)
        self.oooo = (bo.T @ bo).reshape(o, o, o, o)
        self.ovvv = (bov.T @ bvv2).reshape(o, v, v, v)
        ovov = self.ovov
        self.Lovov = 2.0 * ovov - ovov.transpose(0, 3, 2, 1)                    # [k,c,l,d]
        self.LovovT = np.ascontiguousarray(self.Lovov.transpose(0, 2, 1, 3))      # [k,l,c,d]
        self.LovovC = np.ascontiguousarray(self.Lovov.transpose(1, 0, 2, 3))      # [c,k,l,d]
        self.ovovT = np.ascontiguousarray(ovov.transpose(0, 2, 1, 3))             # [i,j,a,b] = (ia|jb)
        self.ovovX = np.ascontiguousarray(ovov.transpose(0, 3, 2, 1))             # [l,d,k,c] = (lc|kd)
        self.Lovoo = 2.0 * self.ovoo - self.ovoo.transpose(2, 1, 0, 3)           # [l,c,k,i]
        # (k,l,c) x i layout of Lovoo for sum_klc Lovoo[l,c,k,i] tau[k,l,a,c]
        self.LovooK = np.ascontiguousarray(self.Lovoo.transpose(2, 0, 1, 3)).reshape(o * o * v, o)
        self.ovooA = np.ascontiguousarray(self.ovoo.transpose(0, 1, 3, 2)).reshape(o * v * o, o)  # [(k,c,i), l]
        self.ovooB = np.ascontiguousarray(self.ovoo.transpose(1, 2, 3, 0)).reshape(v * o * o, o)  # [(c,k,i), l]
        ovvv = self.ovvv
        # [(k,c,d), a] = 2 (kd|ac) - (kc|ad)
        self.LovvvR = (2.0 * ovvv.transpose(0, 3, 1, 2) - ovvv.transpose(0, 1, 3, 2)).reshape(o * v * v, v)
        self._build_pairs(bvv)
        self.diis_size, self.diis_start = diis_size, diis_start
        self.t1 = np.zeros((o, v))
        self.t2 = self.ovovT / self.d2
        self.updates = 0
        self._hist = []

    # ---- particle-particle ladder in pair form --------------------------------
    def _build_pairs(self, bvv):
        """W+[ab,cd] = (ac|bd) + (ad|bc) (c > d), (ac|bc) (c = d) over a >= b, c >= d;
        W-[ab,cd] = (ac|bd) - (ad|bc) over a > b, c > d; rows built a at a time."""
        v = self.v
        naux = bvv.shape[0]
        tc, td = np.tril_indices(v)
        sc, sd = np.tril_indices(v, -1)
        Tv, Tmv = tc.size, sc.size
        self.Wp = np.empty((Tv, Tv))
        self.Wm = np.empty((Tmv, Tmv))
        diag = tc == td
        bflat = bvv.reshape(naux, v * v)
        for a in range(v):
            # G[b, c, d] = (ac|bd) for b <= a
            g = (bvv[:, a, :].T @ bflat[:, :(a + 1) * v]).reshape(v, a + 1, v).transpose(1, 0, 2)
            s = g + g.transpose(0, 2, 1)
            rows = s[:, tc, td]
            rows[:, diag] *= 0.5
            r0 = a * (a + 1) // 2
            self.Wp[r0:r0 + a + 1] = rows
            if a > 0:
                m0 = a * (a - 1) // 2
                self.Wm[m0:m0 + a] = (g[:a] - g[:a].transpose(0, 2, 1))[:, sc, sd]
        o = self.o
        self._otri = np.tril_indices(o)
        self._ostr = np.tril_indices(o, -1)
        # position of each strict pair i > j in the list of pairs i >= j (both row-major)
        self._ostr_in_tri = np.searchsorted(self._otri[0] * o + self._otri[1], self._ostr[0] * o + self._ostr[1])
        self._vtri = (tc, td)
        self._vstr = (sc, sd)
        # unpack maps: tri(max, min) / stri(max, min) and the sign of the antisymmetric half
        def maps(m):
            p = np.arange(m)
            hi, lo = np.maximum(p[:, None], p[None, :]), np.minimum(p[:, None], p[None, :])
            tri = hi * (hi + 1) // 2 + lo
            stri = np.where(hi > lo, hi * (hi - 1) // 2 + lo, 0)
            sgn = np.sign(p[:, None] - p[None, :]).astype(np.float64)
            return tri, stri, sgn
        self._otri_map, self._ostr_map, self._osgn = maps(o)
        self._vtri_map, self._vstr_map, self._vsgn = maps(v)
        # V+-[(k,a), cd pair] of Z (V[c,d] = (kd|ac)) and U+-[(k,l), cd pair] of X (U[c,d] = (kc|ld))
        # (V[(k,a)][c][d] = (kd|ac) = ovvv[k][d][a][c], packed k at a time from views of ovvv)
        self.Vzp = np.empty((o * v, v * (v + 1) // 2))
        self.Vzm = np.empty((o * v, v * (v - 1) // 2))
        for k in range(o):
            self.Vzp[k * v:(k + 1) * v], self.Vzm[k * v:(k + 1) * v] = self._row_packs(self.ovvv[k].transpose(1, 2, 0))
        self.Uxp, self.Uxm = self._row_packs(self.ovovT.reshape(o * o, v, v))

    @staticmethod
    def _row_packs(M, chunk: int = 256):
        """P+[r, tri(c,d)] = M[r,c,d] + M[r,d,c] (c > d), M[r,c,c] (c = d); P-[r, stri(c,d)] =
        M[r,c,d] - M[r,d,c]; rows a chunk at a time."""
        n, v = M.shape[0], M.shape[1]
        tc, td = np.tril_indices(v)
        sc, sd = np.tril_indices(v, -1)
        diag = tc == td
        P = np.empty((n, tc.size))
        Q = np.empty((n, sc.size))
        for r0 in range(0, n, chunk):
            m = M[r0:r0 + chunk]
            mt = m.transpose(0, 2, 1)
            p = (m + mt)[:, tc, td]
            p[:, diag] *= 0.5
            P[r0:r0 + chunk] = p
            Q[r0:r0 + chunk] = (m - mt)[:, sc, sd]
        return P, Q

    def _tau_pairs(self, tau):
        """tau+[ij pair, cd pair], tau-[strict ij pair, strict cd pair] over the four partners."""
        tsw = tau.transpose(0, 1, 3, 2)
        tji = tau.transpose(1, 0, 3, 2)
        oi, oj = self._otri
        tc, td = self._vtri
        sc, sd = self._vstr
        a, b = tau[oi, oj], tsw[oi, oj]                    # [ij pair, c, d]: tau[ijcd], tau[ijdc]
        c_, d_ = tji[oi, oj], tji.transpose(0, 1, 3, 2)[oi, oj]  # tau[jidc], tau[jicd]
        taup = (0.25 * (a + b + c_ + d_))[:, tc, td]
        taum = (0.25 * (a - b + c_ - d_))[self._ostr_in_tri][:, sc, sd]   # strict pairs i > j
        return taup, taum

    def _unpack_pairs(self, Ps, Pa):
        """P[(i,j), r] = Ps[tri(i,j), r] + sgn(i-j) Pa[stri(i,j), r]."""
        P = Ps[self._otri_map.ravel()]
        if Pa.size:
            P += self._osgn.ravel()[:, None] * Pa[self._ostr_map.ravel()]
        return P

    def ladder(self, taup, taum, Woooo):
        """sum_cd (ac|bd) tau[i,j,c,d] + sum_kl Woooo[k,l,i,j] tau[k,l,a,b] through the pair forms:
        the hh ladder adds W+ tau+ and W- tau- (W+- the (k,l) packs of Woooo[., ., i, j]) to the
        halves S+- before their one unpack."""
        o, v = self.o, self.v
        oi, oj = self._otri
        si, sj = self._ostr
        Wt = Woooo.transpose(2, 3, 0, 1)                   # [i, j, k, l]
        Whp = self._row_packs(np.ascontiguousarray(Wt[oi, oj]))[0]
        Sp = taup @ self.Wp.T + Whp @ taup                 # [ij pair, ab pair]
        R = Sp[:, self._vtri_map.ravel()].reshape(-1, v, v)[self._otri_map.ravel()].reshape(o, o, v, v)
        if taum.size and self._vstr[0].size:
            Whm = self._row_packs(np.ascontiguousarray(Wt[si, sj]))[1]
            Sm = taum @ self.Wm.T + Whm @ taum
            U = (Sm[:, self._vstr_map.ravel()].reshape(-1, v, v) * self._vsgn)[self._ostr_map.ravel()]
            R += U.reshape(o, o, v, v) * self._osgn[:, :, None, None]
        return R

    # ---- the residual numerators (diagonal Fock moved to the denominators) -----
    def residual(self, t1, t2):
        o, v = self.o, self.v
        ov = o * v
        ovov, oovv, ovoo, oooo, ovvv = self.ovov, self.oovv, self.ovoo, self.oooo, self.ovvv
        fov = self.f_ov
        tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
        # t2 as [(i,a),(l,d)]: t2[i,l,a,d] and t2[i,l,d,a]
        t2_iald = np.ascontiguousarray(t2.transpose(0, 2, 1, 3)).reshape(ov, ov)
        t2_ilda = np.ascontiguousarray(t2.transpose(0, 3, 1, 2)).reshape(ov, ov)

        Foo = self.f_oo + self.LovovT.reshape(o, -1) @ tau.reshape(o, -1).T
        Fvv = self.f_vv - np.ascontiguousarray(tau.transpose(2, 0, 1, 3)).reshape(v, -1) @ \
            self.LovovC.reshape(v, -1).T
        Fov = fov + (self.Lovov.reshape(ov, ov) @ t1.ravel()).reshape(o, v)
        Loo = Foo + fov @ t1.T + np.einsum("lcki,lc->ki", self.Lovoo, t1, optimize=True)
        # Lvv = Fvv - t1^T f + sum_kd (2 (kd|ac) - (kc|ad)) t1[k,d]
        Lvv = Fvv - t1.T @ fov + 2.0 * (t1.ravel() @ ovvv.reshape(ov, v * v)).reshape(v, v)
        for k in range(o):                                   # (kc|ad) t1[k,d] -> [c, a]
            Lvv -= (ovvv[k].reshape(v * v, v) @ t1[k]).reshape(v, v).T
        Foo_p = Foo - np.diag(self.eo)
        Fvv_p = Fvv - np.diag(self.ev)
        Loo_p = Loo - np.diag(self.eo)
        Lvv_p = Lvv - np.diag(self.ev)

        # ---- T1 --------------------------------------------------------------
        t2_kica = t2_iald.reshape(o, v, o, v)                # [k,c,i,a] = t2[k,i,c,a]
        R1 = (fov - 2.0 * (t1 @ fov.T) @ t1 + t1 @ Fvv_p.T - Foo_p.T @ t1
              + 2.0 * (Fov.ravel() @ t2_kica.reshape(ov, ov)).reshape(o, v)
              - (Fov.ravel() @ t2_kica.transpose(2, 1, 0, 3).reshape(ov, ov)).reshape(o, v)   # t2[i,k,c,a]
              + (t1 @ Fov.T) @ t1
              + 2.0 * (t1.ravel() @ ovov.reshape(ov, ov)).reshape(o, v)
              - np.einsum("kiac,kc->ia", oovv, t1, optimize=True))
        R1 += tau.reshape(o, o * v * v) @ self.LovvvR       # sum_kcd (2 (kd|ac) - (kc|ad)) tau[i,k,c,d]
        R1 -= (np.ascontiguousarray(tau.transpose(0, 1, 3, 2)).reshape(o * o * v, v).T @ self.LovooK).T

        # ---- intermediates ---------------------------------------------------
        taup, taum = self._tau_pairs(tau)
        X = self._unpack_pairs(taup @ self.Uxp.T, taum @ self.Uxm.T)               # [(i,j), (k,l)]
        Woooo = (oooo.transpose(0, 2, 1, 3) + np.einsum("lcki,jc->klij", ovoo, t1, optimize=True)
                 + np.einsum("kclj,ic->klij", ovoo, t1, optimize=True)
                 + X.T.reshape(o, o, o, o))
        # Wvoov and Wvovo stored as [(i,a), (k,c)] (W_akic, W_akci)
        t1t1 = (t1[:, None, None, :] * t1.T[None, :, :, None]).reshape(ov, ov)      # t1[i,d] t1[l,a]
        th1 = t2_iald - 0.5 * t2_ilda - t1t1
        th2 = 0.5 * t2_ilda + t1t1
        Wvoov = ovov.reshape(ov, ov).copy()                                         # (ia|kc) = (ai|kc)
        Wvoov += (ovvv.reshape(o * v * v, v) @ t1.T).reshape(o, v, v, o).transpose(3, 2, 0, 1).reshape(ov, ov)
        Wvoov -= (self.ovooA @ t1).reshape(o, v, o, v).transpose(2, 3, 0, 1).reshape(ov, ov)
        Wvoov += th1 @ ovov.reshape(ov, ov)
        Wvoov -= 0.5 * (t2_iald @ self.ovovX.reshape(ov, ov))
        Wvovo = oovv.transpose(1, 2, 0, 3).reshape(ov, ov).copy()                  # (ki|ac)
        W4 = Wvovo.reshape(o, v, o, v)
        for k in range(o):                                                         # sum_d (kd|ac) t1[i,d]
            W4[:, :, k, :] += (t1 @ ovvv[k].reshape(v, v * v)).reshape(o, v, v)
        Wvovo -= (self.ovooB @ t1).reshape(v, o, o, v).transpose(2, 3, 1, 0).reshape(ov, ov)
        Wvovo -= th2 @ self.ovovX.reshape(ov, ov)

        # ---- T2: R2 = (ia|jb) + Woooo tau + ladder + Rp + Rp^T (Rp^T[ijab] = Rp[jiba]) ----
        Rp = (ovvv.reshape(o * v * v, v) @ t1.T).reshape(o, v, v, o).transpose(0, 3, 1, 2).copy()  # (ia|bc) t1[j,c]
        Vk = (oovv.reshape(o * o * v, v) @ t1.T).reshape(o, o, v, o)               # [k,i,b,j]
        Rp -= (t1.T @ Vk.reshape(o, -1)).reshape(v, o, v, o).transpose(1, 3, 0, 2)
        tmpB = (np.einsum("kcia,jc->akij", ovov, t1, optimize=True) + ovoo.transpose(1, 3, 0, 2))   # [a,k,i,j]
        Rp -= np.einsum("akij,kb->ijab", tmpB, t1, optimize=True)
        Z = self._unpack_pairs(taup @ self.Vzp.T, taum @ self.Vzm.T)               # [(i,j), (k,a)]
        Rp -= (Z.reshape(o * o, o, v).transpose(0, 2, 1).reshape(o * o * v, o) @ t1).reshape(o, o, v, v)
        Rp += np.matmul(Lvv_p, t2)
        Rp -= (Loo_p.T @ t2.reshape(o, -1)).reshape(o, o, v, v)
        Wa = 2.0 * Wvoov - Wvovo
        ring = Wa @ t2_iald                                                         # t2_iald = t2[k,j,c,b]
        ring -= Wvoov @ t2_ilda                                                     # t2_ilda = t2[k,j,b,c]
        Rp += ring.reshape(o, v, o, v).transpose(0, 2, 1, 3)
        Rp -= (Wvovo @ t2_ilda).reshape(o, v, o, v).transpose(0, 2, 3, 1)
        R2 = self.ovovT + self.ladder(taup, taum, Woooo)
        R2 += Rp
        R2 += Rp.transpose(1, 0, 3, 2)
        return R1, R2

    def energy(self, t1, t2):
        tau = t2 + t1[:, None, :, None] * t1[None, :, None, :]
        L = 2.0 * self.ovovT - self.ovovT.transpose(0, 1, 3, 2)
        return float(np.vdot(L, tau))

    def _diis(self, t1, t2, t1_old, t2_old):
        """Pulay extrapolation over the last diis_size (T, T - T_old) pairs."""
        if not self.diis_size:
            return t1, t2
        self._hist.append((t1.copy(), t2.copy(), t1 - t1_old, t2 - t2_old))
        if len(self._hist) > self.diis_size:
            self._hist.pop(0)
        if self.updates < self.diis_start or len(self._hist) < 2:
            return t1, t2
        m = len(self._hist)
        B = -np.ones((m + 1, m + 1))
        B[m, m] = 0.0
        for i in range(m):
            for j in range(i, m):
                B[i, j] = B[j, i] = (np.vdot(self._hist[i][2], self._hist[j][2])
                                     + np.vdot(self._hist[i][3], self._hist[j][3]))
        rhs = np.zeros(m + 1)
        rhs[m] = -1.0
        try:
            c = np.linalg.solve(B, rhs)[:m]
        except np.linalg.LinAlgError:
            return t1, t2
        return (sum(ci * h[0] for ci, h in zip(c, self._hist)), sum(ci * h[1] for ci, h in zip(c, self._hist)))

    def step(self) -> dict:
        """One whole update; returns its wall-clock seconds and the new energy."""
        t0 = time.perf_counter()
        R1, R2 = self.residual(self.t1, self.t2)
        t1n, t2n = R1 / self.d1, R2 / self.d2
        self.updates += 1
        t1n, t2n = self._diis(t1n, t2n, self.t1, self.t2)
        self.t1, self.t2 = t1n, t2n
        e = self.energy(t1n, t2n)
        return dict(seconds=time.perf_counter() - t0, e_corr=e)
