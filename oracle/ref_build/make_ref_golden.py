"""Golden fixtures from the reference's own code, compiled unchanged into
oracle/_ref/ by build_ref.py (TEST INFRASTRUCTURE ONLY; needs the reference
sources, so it runs in the development container, not on the GPU host).

    python -m oracle.ref_build.make_ref_golden            # CCSD fixtures
    python -m oracle.ref_build.make_ref_golden ccsdt-1a   # CCSDT-1a fixtures

Writes
* tests/golden/h2o_<basis>_<geometry>_tol<k>.npz: the RHF outputs the
  reference CCSD consumed (AO integrals, MO coefficients, orbital energies,
  E_HF) and the results (E_corr, iteration counter) of both reference CCSD
  codes ("ref_*" = CCSD_Memory_optimized, "ref_ccsd1_*" = CCSDT method -1);
* tests/golden/reference_runs.json: the reference's CCSD on the seeded
  synthetic systems of synthetic_oracle.json, from both of its CCSD codes:
  "mo" = CCSD_Memory_optimized::CCSD (the "CCSD" method) and
  "ccsd1" = CCSDT::Calc_Energy(toler, -1) (the dense spin-orbital "CCSD1");
* tests/golden/reference_ccsdt1a.json (with the ccsdt-1a argument): the
  reference's CCSDT-1a, CCSDT::Calc_Energy(toler, 1), on small seeded
  synthetic systems and on the H2O inputs of the .npz fixtures above.
"""
from __future__ import annotations

import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
GOLD = ROOT / "tests" / "golden"
REF = HERE.parent / "_ref"
sys.path.insert(0, str(ROOT))

from oracle import synthetic as syn  # noqa: E402

H2O = [  # (basis, geometry, log10 tolerance)
    ("STO-3G", "yz:1.079252,1.474611", -8),   # the reference's recorded known answer
    ("STO-3G", "yz:1.079252,1.474611", -10),
    ("6-31G", "config", -10),                 # O (0,0,0), H (+-1.4305, 1.1071, 0) bohr
]


def _parse(out: str):
    line = [l for l in out.splitlines() if l.startswith("iter")][-1].split()
    d = {line[k]: float(line[k + 1]) for k in range(0, len(line), 2)}
    d["iter"] = int(d["iter"])
    return d


def run_h2o(basis, geom, tol, mode="ccsd1"):
    with tempfile.TemporaryDirectory() as td:
        dump = Path(td) / "h2o.bin"
        out = subprocess.run([str(REF / "ref_h2o"), basis, geom, str(tol), str(dump), mode],
                             capture_output=True, text=True, check=True).stdout
        res = _parse(out)
        c1 = [l for l in out.splitlines() if l.startswith("ccsd1_iter")][-1].split()
        res["ccsd1_iter"], res["ccsd1_ecorr"] = int(c1[1]), float(c1[3])
        raw = dump.read_bytes()
    n, nocc = np.frombuffer(raw[:8], dtype=np.int32)
    f = np.frombuffer(raw[8:], dtype=np.float64)
    C = f[:n * n].reshape(n, n)
    eps = f[n * n:n * n + n]
    eri = f[n * n + n:n * n + n + n ** 4].reshape(n, n, n, n)
    ehf = f[-1]
    return res, int(n), int(nocc), C, eps, eri, ehf


def run_synthetic(o, v, q, seed, sigma, tol, mode):
    eps = syn.orbital_energies(o, v, seed)
    eri = syn.eri_from_df(syn.df_factors(o + v, q, seed, sigma=sigma))
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "in.bin"
        with open(p, "wb") as fh:
            np.array([o + v, o], dtype=np.int32).tofile(fh)
            eps.tofile(fh)
            np.ascontiguousarray(eri).tofile(fh)
        out = subprocess.run([str(REF / "ref_synthetic"), str(p), str(tol), mode], capture_output=True,
                             text=True, check=True).stdout
    return _parse(out)


def main():
    for basis, geom, tol in H2O:
        res, n, nocc, C, eps, eri, ehf = run_h2o(basis, geom, tol)
        tag = "incarsym" if geom.startswith("yz:1.079252") else geom
        name = f"h2o_{basis.lower().replace('-', '')}_{tag}_tol{-tol}.npz"
        np.savez_compressed(GOLD / name, basis=basis, geometry=geom, log10_tol=tol, nocc=nocc, mo_coeff=C,
                            eps=eps, ao_eri=eri, e_hf=ehf, ref_e_corr=res["ecorr"], ref_iter=res["iter"],
                            ref_e_total=res["etotal"], ref_ccsd1_e_corr=res["ccsd1_ecorr"],
                            ref_ccsd1_iter=res["ccsd1_iter"])
        print(name, res)
    runs = {}
    cases = json.loads((GOLD / "synthetic_oracle.json").read_text())
    for key, c in cases.items():
        if c["nocc"] > 4:
            continue  # the dense spin-orbital CCSD1 grows as N^8
        entry = dict(nocc=c["nocc"], nvir=c["nvir"], naux=c["naux"], seed=c["seed"], sigma=c["sigma"], log10_tol=-10)
        for mode in ("mo", "ccsd1"):
            r = run_synthetic(c["nocc"], c["nvir"], c["naux"], c["seed"], c["sigma"], -10, mode)
            entry[mode] = dict(iter=r["iter"], e_corr=r["ecorr"])
        runs[key] = entry
        print(key, entry)
    (GOLD / "reference_runs.json").write_text(json.dumps(runs, indent=1))


CCSDT1A_SYNTHETIC = [  # (nocc, nvir, naux, seed, sigma); sigma 0.2-0.3 gives visible triples
    (2, 4, 12, 5, 0.3), (3, 6, 20, 6, 0.3), (2, 8, 20, 7, 0.25), (4, 6, 24, 11, 0.2)]


CCSDT_METHODS = {"ccsdt-1a": (1, "reference_ccsdt1a.json"), "ccsdt-1b": (2, "reference_ccsdt1b.json"),
                 "ccsdt-2": (3, "reference_ccsdt2.json"), "ccsdt-3": (4, "reference_ccsdt3.json"),
                 "ccsdt-4": (5, "reference_ccsdt4.json"), "ccsdt": (6, "reference_ccsdt.json")}


def main_ccsdt(name="ccsdt-1a"):
    """The reference's CCSDT::Calc_Energy(toler, Method_Nr) on the synthetic
    systems and on H2O; Method_Nr 1 = CCSDT-1a, 2 = CCSDT-1b, 3 = CCSDT-2, 4 = CCSDT-3,
    5 = CCSDT-4, 6 = CCSDT."""
    method, out = CCSDT_METHODS[name]
    mode = f"ccsdt-{method}"
    runs = {"synthetic": {}, "h2o": {}}
    for o, v, q, seed, sigma in CCSDT1A_SYNTHETIC:
        r = run_synthetic(o, v, q, seed, sigma, -10, mode)
        runs["synthetic"][f"o{o}_v{v}_s{seed}"] = dict(nocc=o, nvir=v, naux=q, seed=seed, sigma=sigma, log10_tol=-10,
                                                        iter=r["iter"], e_corr=r["ecorr"])
    for basis, geom, tol in H2O:
        res = run_h2o(basis, geom, tol, mode)[0]
        tag = "incarsym" if geom.startswith("yz:1.079252") else geom
        name = f"h2o_{basis.lower().replace('-', '')}_{tag}_tol{-tol}.npz"
        runs["h2o"][name] = dict(iter=res["ccsd1_iter"], e_corr=res["ccsd1_ecorr"])
    (GOLD / out).write_text(json.dumps(runs, indent=1))
    print(json.dumps(runs, indent=1))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] in CCSDT_METHODS:
        main_ccsdt(sys.argv[1])
    else:
        main()
