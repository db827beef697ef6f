"""FP64 restatement of the reference's Gaussian integral engine
(hartree_integrals.cpp), TEST INFRASTRUCTURE ONLY: what the GPU integral
kernels (ccsd_ao_integrals) are compared with, never on the product path.

McMurchie-Davidson over contracted Cartesian Gaussians, as the reference does it:
  - Hermite expansion coefficients E_t^{ij} of a product of two 1-D Gaussians
    (Fill_E_ij, hartree_integrals.cpp:118-227);
  - overlap, <mu|nabla^2|nu> and sum_C Z_C <mu|1/r_C|nu> as the reference returns
    them (Overlap_Integral_Single :325-354, Kinetic_Energy_Single :398-459,
    Nuclei_Electron_Interaction_Single :512-555);
  - Hermite Coulomb integrals R_tuv (Set_R_ijk :23-94) with the Boys function
    evaluated as the reference does (Boys :643-693: a 100-term series for F_30
    below x = 50, the asymptotic form above, then downward recursion);
  - (mu nu|la si) = 2 pi^{5/2} / (p q sqrt(p+q)) sum E^{mu nu}_{tuv} (-1)^{t'+u'+v'}
    E^{la si}_{t'u'v'} R_{t+t',u+u',v+v'} (Electron_Electron_Interaction_Single
    :720-796), contracted with the normalised coefficients c (Normalize_small_c,
    hartree_fock_solver.cpp:236-462, applied by the caller).

The basis is the description the reference's Hartree_Integrals::Set_Input
receives (hartree_integrals.cpp:8-21): per basis function its atom, Cartesian
powers, primitive count, exponents and normalised coefficients.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Basis:
    Z: np.ndarray        # [natoms] nuclear charges
    R: np.ndarray        # [natoms, 3] bohr
    atom: np.ndarray     # [nbf] atom of each basis function
    powers: np.ndarray   # [nbf, 3] Cartesian powers (l, m, n)
    nprim: np.ndarray    # [nbf]
    alpha: np.ndarray    # [nbf, maxprim] exponents
    coef: np.ndarray     # [nbf, maxprim] normalised contraction coefficients

    @property
    def nbf(self) -> int:
        return int(self.atom.shape[0])

    @classmethod
    def from_dict(cls, d) -> "Basis":
        return cls(np.asarray(d["Z"], float), np.asarray(d["R"], float).reshape(-1, 3),
                   np.asarray(d["atom"], np.int64), np.asarray(d["powers"], np.int64).reshape(-1, 3),
                   np.asarray(d["nprim"], np.int64), np.asarray(d["alpha"], float), np.asarray(d["coef"], float))


BOYS_AS_WRITTEN = True


def boys(nmax: int, x: float, as_written: bool | None = None) -> np.ndarray:
    """F_0..F_nmax at x, the reference's way (hartree_integrals.cpp:643-693):
    F_30 from its series e^{-x} sum_{j<100} (2x)^j / ((61)(63)...(61+2j)) for
    x <= 50, else (59)!! / 2^31 sqrt(pi / x^61); then F_{i-1} = (2x F_i + e^{-x}) / (2i - 1).

    That asymptotic form needs x >> 30: just above x = 50 it is off by 1.2e-3
    (relative, every F_n), 1e-5 at x = 60, 1e-11 at x = 80.  as_written=False
    (default: the module's BOYS_AS_WRITTEN) takes x > 50 from F_0 = sqrt(pi/x)/2
    upward instead, F_{n+1} = (2n+1)/(2x) F_n, accurate to e^{-x} (the GPU engine's form)."""
    N = 30
    ex = math.exp(-x)
    if as_written is None:
        as_written = BOYS_AS_WRITTEN
    if x > 50 and not as_written:
        out = np.empty(nmax + 1)
        out[0] = 0.5 * math.sqrt(math.pi / x)
        for n in range(nmax):
            out[n + 1] = (2 * n + 1) / (2 * x) * out[n]
        return out
    if x > 50:
        dfac = 1.0
        i = 1.0
        while i < 2 * N - 1:
            i += 2
            dfac *= i
        try:
            xp = x ** (2 * N + 1)
        except OverflowError:  # the reference's pow() gives inf here, so F = 0
            xp = math.inf
        F = dfac / 2.0 ** (N + 1) * math.sqrt(math.pi / xp)
    else:
        F = 0.0
        for j in range(100):
            term = (2 * x) ** j
            M = 2 * N + 1
            while M < 2 * N + 2 + 2 * j:
                term /= M
                M += 2
            F += term
        F *= ex
    out = np.empty(N + 1)
    out[N] = F
    for i in range(N, 0, -1):
        out[i - 1] = (2 * x * out[i] + ex) / (2 * i - 1)
    return out[:nmax + 1]


def hermite_E(la: int, lb: int, a: float, b: float, A: float, B: float) -> np.ndarray:
    """E[i, j, t] for i <= la+2, j <= lb+2 (the reference fills two beyond, for
    the kinetic integrals), t <= i+j: E_0^{00} = exp(-ab/p X_AB^2),
    E_t^{i+1,j} = E_{t-1}^{ij}/(2p) + X_PA E_t^{ij} + (t+1) E_{t+1}^{ij} and the same in j
    with X_PB (hartree_integrals.cpp:160-210)."""
    p = a + b
    P = (a * A + b * B) / p
    XPA, XPB, XAB = P - A, P - B, A - B
    E = np.zeros((la + 3, lb + 3, la + lb + 7))
    E[0, 0, 0] = math.exp(-a * b * XAB * XAB / p)
    h = 0.5 / p
    for i in range(la + 2):
        for t in range(i + 2):
            E[i + 1, 0, t] = (E[i, 0, t - 1] * h if t else 0.0) + XPA * E[i, 0, t] + (t + 1) * E[i, 0, t + 1]
    for i in range(la + 3):
        for j in range(lb + 2):
            for t in range(i + j + 2):
                E[i, j + 1, t] = (E[i, j, t - 1] * h if t else 0.0) + XPB * E[i, j, t] + (t + 1) * E[i, j, t + 1]
    return E


def hermite_R(p: float, PC: np.ndarray, T: int, U: int, V: int) -> np.ndarray:
    """R^0_{tuv} for t <= T, u <= U, v <= V at exponent p and separation PC
    (Set_R_ijk, hartree_integrals.cpp:23-94): R^n_{000} = (-2p)^n F_n(p |PC|^2),
    R^n_{t+1,u,v} = t R^{n+1}_{t-1,u,v} + X_PC R^{n+1}_{t,u,v}, likewise in u, v."""
    L = T + U + V
    F = boys(L, p * float(PC @ PC))
    R = np.zeros((L + 2, T + 2, U + 2, V + 2))
    for n in range(L + 1):
        R[n, 0, 0, 0] = (-2 * p) ** n * F[n]
    for t in range(T):
        for n in range(L - t):
            R[n, t + 1, 0, 0] = PC[0] * R[n + 1, t, 0, 0] + (t * R[n + 1, t - 1, 0, 0] if t else 0.0)
    for t in range(T + 1):
        for u in range(U):
            for n in range(L - t - u):
                R[n, t, u + 1, 0] = PC[1] * R[n + 1, t, u, 0] + (u * R[n + 1, t, u - 1, 0] if u else 0.0)
    for t in range(T + 1):
        for u in range(U + 1):
            for v in range(V):
                for n in range(L - t - u - v):
                    R[n, t, u, v + 1] = PC[2] * R[n + 1, t, u, v] + (v * R[n + 1, t, u, v - 1] if v else 0.0)
    return R[0, :T + 1, :U + 1, :V + 1]


class Integrals:
    """All integrals of one basis (the reference's conventions)."""

    def __init__(self, basis: Basis):
        self.b = basis
        self._pairs = {}

    def _pair(self, i: int, j: int):
        """Primitive pairs of basis functions i, j: (p, P, c_i c_j, Ex, Ey, Ez) with
        E in the reference's [i, j, t] layout for this pair's powers."""
        key = (i, j)
        if key in self._pairs:
            return self._pairs[key]
        b = self.b
        A, B = b.R[b.atom[i]], b.R[b.atom[j]]
        li, lj = b.powers[i], b.powers[j]
        out = []
        for k in range(b.nprim[i]):
            for m in range(b.nprim[j]):
                a1, a2 = b.alpha[i, k], b.alpha[j, m]
                p = a1 + a2
                Es = [hermite_E(li[d], lj[d], a1, a2, A[d], B[d]) for d in range(3)]
                out.append((a1, a2, p, (a1 * A + a2 * B) / p, b.coef[i, k] * b.coef[j, m], Es))
        self._pairs[key] = out
        return out

    def overlap(self) -> np.ndarray:
        n = self.b.nbf
        S = np.zeros((n, n))
        for i in range(n):
            for j in range(i, n):
                li, lj = self.b.powers[i], self.b.powers[j]
                s = 0.0
                for a1, a2, p, P, cc, (Ex, Ey, Ez) in self._pair(i, j):
                    s += cc * (math.pi / p) ** 1.5 * Ex[li[0], lj[0], 0] * Ey[li[1], lj[1], 0] * Ez[li[2], lj[2], 0]
                S[i, j] = S[j, i] = s
        return S

    def laplacian(self) -> np.ndarray:
        """<mu|nabla^2|nu> (the reference's Kinetic_Energy; T = -1/2 of it)."""
        n = self.b.nbf
        K = np.zeros((n, n))
        for i in range(n):
            for j in range(i, n):
                li, lj = self.b.powers[i], self.b.powers[j]
                s = 0.0
                for a1, a2, p, P, cc, Es in self._pair(i, j):
                    e0 = [Es[d][li[d], lj[d], 0] for d in range(3)]
                    val = 0.0
                    for d in range(3):
                        D = lj[d]
                        jd = 4 * a2 * a2 * Es[d][li[d], D + 2, 0] - 2 * a2 * (2 * D + 1) * Es[d][li[d], D, 0]
                        if D > 1:
                            jd += D * (D - 1) * Es[d][li[d], D - 2, 0]
                        val += jd * e0[(d + 1) % 3] * e0[(d + 2) % 3]
                    s += cc * val * (math.pi / p) ** 1.5
                K[i, j] = K[j, i] = s
        return K

    def nuclear(self) -> np.ndarray:
        """sum_C Z_C <mu|1/r_C|nu> (the reference's Nuclei_Electron_Interaction;
        the attraction is minus this)."""
        n = self.b.nbf
        Vn = np.zeros((n, n))
        for i in range(n):
            for j in range(i, n):
                li, lj = self.b.powers[i], self.b.powers[j]
                s = 0.0
                for a1, a2, p, P, cc, (Ex, Ey, Ez) in self._pair(i, j):
                    T, U, W = li + lj
                    acc = 0.0
                    for C, Zc in zip(self.b.R, self.b.Z):
                        R = hermite_R(p, P - C, T, U, W)
                        ex = Ex[li[0], lj[0], :T + 1]
                        ey = Ey[li[1], lj[1], :U + 1]
                        ez = Ez[li[2], lj[2], :W + 1]
                        acc += Zc * np.einsum("t,u,v,tuv->", ex, ey, ez, R)
                    s += cc * acc * 2 * math.pi / p
                Vn[i, j] = Vn[j, i] = s
        return Vn

    def eri(self, i: int, j: int, k: int, l: int) -> float:
        """(ij|kl), chemist notation."""
        b = self.b
        li, lj, lk, ll = b.powers[i], b.powers[j], b.powers[k], b.powers[l]
        Lb, Lk = li + lj, lk + ll
        val = 0.0
        for _, _, p, P, c1, (Ex1, Ey1, Ez1) in self._pair(i, j):
            e1 = np.einsum("t,u,v->tuv", Ex1[li[0], lj[0], :Lb[0] + 1], Ey1[li[1], lj[1], :Lb[1] + 1],
                           Ez1[li[2], lj[2], :Lb[2] + 1])
            for _, _, q, Q, c2, (Ex2, Ey2, Ez2) in self._pair(k, l):
                e2 = np.einsum("t,u,v->tuv", Ex2[lk[0], ll[0], :Lk[0] + 1], Ey2[lk[1], ll[1], :Lk[1] + 1],
                               Ez2[lk[2], ll[2], :Lk[2] + 1])
                sgn = np.einsum("t,u,v->tuv", *[(-1.0) ** np.arange(Lk[d] + 1) for d in range(3)])
                R = hermite_R(p * q / (p + q), P - Q, *(Lb + Lk))
                s = 0.0
                for t in range(Lb[0] + 1):
                    for u in range(Lb[1] + 1):
                        for v in range(Lb[2] + 1):
                            if e1[t, u, v] == 0.0:
                                continue
                            s += e1[t, u, v] * np.sum(sgn * e2 * R[t:t + Lk[0] + 1, u:u + Lk[1] + 1, v:v + Lk[2] + 1])
                val += c1 * c2 * s * 2 * math.pi ** 2.5 / (p * q * math.sqrt(p + q))
        return val

    def eri_tensor(self) -> np.ndarray:
        """Every (ij|kl) from the unique quartets i >= j, k >= l, (ij) >= (kl)."""
        n = self.b.nbf
        G = np.zeros((n, n, n, n))
        for i in range(n):
            for j in range(i + 1):
                for k in range(i + 1):
                    for l in range(k + 1 if k < i else j + 1):
                        x = self.eri(i, j, k, l)
                        for a, b_, c, d in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k)):
                            G[a, b_, c, d] = G[c, d, a, b_] = x
        return G

    def nuclear_repulsion(self) -> float:
        """sum_{i<j} Z_i Z_j / |R_i - R_j| (Nuclei_Nuclei_Interaction :695-718)."""
        b = self.b
        e = 0.0
        for i in range(len(b.Z)):
            for j in range(i):
                e += b.Z[i] * b.Z[j] / float(np.linalg.norm(b.R[i] - b.R[j]))
        return e
