"""Gaussian94 basis text and INCAR text rebuilt from a golden fixture
(tests/golden/ints_*.npz): the raw contraction coefficients are the
reference's normalised ones divided by its primitive normalisation."""
from __future__ import annotations

import math

import numpy as np

SYMBOLS = {1: "H", 2: "He", 3: "Li", 4: "Be", 5: "B", 6: "C", 7: "N", 8: "O", 9: "F", 10: "Ne"}
NCOMP = {0: 1, 1: 3, 2: 6, 3: 10}
LETTER = {0: "S", 1: "P", 2: "D", 3: "F"}


def _odd_fact(k: int) -> float:
    r = 1.0
    for x in range(2 * k - 1, 1, -2):
        r *= x
    return r


def norm(a: float, p) -> float:
    L = int(sum(p))
    return (2 * a / math.pi) ** 0.75 * (4 * a) ** (L / 2) / math.sqrt(_odd_fact(p[0]) * _odd_fact(p[1]) * _odd_fact(p[2]))


def g94_from_fixture(d) -> str:
    out = []
    done = set()
    for a, z in enumerate(np.asarray(d["Z"]).astype(int)):
        if z in done:
            continue
        done.add(z)
        out.append(f"{SYMBOLS[z]}     0")
        idx = np.nonzero(np.asarray(d["atom"]) == a)[0]
        i = 0
        while i < len(idx):
            f = idx[i]
            p = d["powers"][f]
            L = int(p.sum())
            n = int(d["nprim"][f])
            out.append(f"{LETTER[L]}   {n}   1.00")
            for k in range(n):
                e = float(d["alpha"][f, k])
                out.append(f"  {e!r:>22}  {float(d['coef'][f, k]) / norm(e, p)!r:>24}")
            i += NCOMP[L]
        out.append("****")
    return "\n".join(out) + "\n"


def incar_text(d, method: str, log10_tol: float, extra: str = "", angstrom: bool = False) -> str:
    R = np.asarray(d["R"]) / (1.889725989 if angstrom else 1.0)
    lines = ["Basis_Set from-file", f"Method {method}", f"convergance_criteria {log10_tol}", "Freeze_Core false",
             "Relax_Pos false", f"use_angstrom {'true' if angstrom else 'false'}", "print_stuffies false", extra,
             "#ATOMS START"]
    for z, r in zip(np.asarray(d["Z"]).astype(int), R):
        lines.append(f"{SYMBOLS[z]} {float(r[0])!r} {float(r[1])!r} {float(r[2])!r}")
    lines.append("#ATOMS END")
    return "\n".join(lines) + "\n"
