"""Generate the golden fixtures under tests/golden/ from the oracle.

    python tests/golden/make_golden.py

For each seeded synthetic system (inputs regenerated from the seed by
``oracle.synthetic`` / the library generator) it stores the reference-driver
energy after every amplitude update, the reference iteration counter at
convergence and a few amplitude checksums:

* small systems: from the spin-orbital restatement of the reference
  equations (``oracle.ccsd_spinorb``), cross-checked against the closed-shell
  restatement (``oracle.ccsd_rhf``) before writing;
* the o=10/v=90/naux=300 system: closed-shell restatement only (the
  spin-orbital arrays do not fit).

Outputs of the reference's own compiled CCSD (``oracle/_ref``), when present,
are written by ``oracle/ref_build/make_ref_golden.py``.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import synthetic as syn  # noqa: E402
from oracle.ccsd_rhf import RHFCCSD  # noqa: E402
from oracle.ccsd_spinorb import SpinOrbitalCCSD  # noqa: E402

SMALL = [  # (nocc, nvir, naux, seed, sigma); sigma 0.05 is the default generator,
    # sigma 0.3 gives molecule-like correlation energies and 12-30 updates
    (2, 5, 12, 1, 0.05),
    (3, 7, 20, 5, 0.05),
    (4, 10, 30, 11, 0.05),
    (5, 14, 40, 3, 0.05),
    (2, 5, 12, 1, 0.3),
    (3, 7, 20, 5, 0.3),
    (4, 10, 30, 11, 0.3),
]
LARGE = [(10, 90, 300, 2024, 0.05), (6, 24, 60, 7, 0.3)]


def checksums(t1, t2):
    return dict(t1_sum=float(t1.sum()), t1_sq=float((t1 * t1).sum()), t2_sum=float(t2.sum()),
                t2_sq=float((t2 * t2).sum()), t2_first=float(t2.flat[1]),
                t2_max=float(np.abs(t2).max()))


def main():
    out = {}
    for (o, v, q, seed, sig) in SMALL:
        fock = np.diag(syn.orbital_energies(o, v, seed))
        b = syn.df_factors(o + v, q, seed, sigma=sig)
        eri = syn.eri_from_df(b)
        so = SpinOrbitalCCSD(fock, eri, o).run(toler=1e-10)
        cs = RHFCCSD(fock, o, eri=eri).run(toler=1e-10)
        assert so["iter"] == cs["iter"], (so["iter"], cs["iter"])
        assert np.abs(so["energies"] - cs["energies"]).max() < 1e-13
        key = f"syn_o{o}_v{v}_q{q}_s{seed}_sig{sig}"
        out[key] = dict(nocc=o, nvir=v, naux=q, seed=seed, sigma=sig, source="oracle.ccsd_spinorb",
                        tol=1e-10, iter=int(so["iter"]), e_corr=float(so["e_corr"]),
                        energies=[float(x) for x in so["energies"]], **checksums(cs["t1"], cs["t2"]))
        print(key, so["iter"], so["e_corr"])
    for (o, v, q, seed, sig) in LARGE:
        fock = np.diag(syn.orbital_energies(o, v, seed))
        b = syn.df_factors(o + v, q, seed, sigma=sig)
        cs = RHFCCSD(fock, o, df=b).run(toler=1e-10)
        key = f"syn_o{o}_v{v}_q{q}_s{seed}_sig{sig}"
        out[key] = dict(nocc=o, nvir=v, naux=q, seed=seed, sigma=sig, source="oracle.ccsd_rhf", tol=1e-10,
                        iter=int(cs["iter"]), e_corr=float(cs["e_corr"]),
                        energies=[float(x) for x in cs["energies"]], **checksums(cs["t1"], cs["t2"]))
        print(key, cs["iter"], cs["e_corr"])
    (HERE / "synthetic_oracle.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
