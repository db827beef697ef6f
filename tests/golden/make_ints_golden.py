"""Golden Gaussian-integral fixtures from the reference's own RHF and integral
engine (hartree_fock_solver.cpp, hartree_integrals.cpp, compiled unchanged by
oracle/ref_build/build_ref.py into oracle/_ref/ref_ints).

Each tests/golden/ints_<name>.npz holds:
  - the basis description the reference's Hartree_Integrals::Set_Input receives
    (Z, R, atom, powers, nprim, alpha, normalised coef);
  - S, lap (<mu|nabla^2|nu>) and nuc (sum_C Z_C <mu|1/r_C|nu>) as the reference returns them;
  - the AO integrals (mu nu|la si): the whole tensor ("eri") up to 13 functions, else
    the values at a seeded sample of unique quartets ("eri_idx" [k, 4], "eri_val" [k]);
  - E_nuc, E_HF, the orbital energies eps and C[mu][p] of its SCF (run to
    tolerance 10^log10_tol; OH, with 9 electrons, is there for its basis only).
tests/golden/reference_uhf.json holds the reference's UHF energies (get_Energy(toler, 1)
after Set_UP_DOWN) on open shells of those molecules.

    python tests/golden/make_ints_golden.py      # needs the reference sources
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

WATER = "8,0,0,0;1,1.4305,1.1071,0;1,-1.4305,1.1071,0"
AMMONIA = "7,0,0,0.2;1,1.77,0,-0.48;1,-0.885,1.533,-0.48;1,-0.885,-1.533,-0.48"
# name, basis, atoms (Z,x,y,z bohr), electrons, log10 SCF tolerance
CASES = [("h2o_sto3g", "STO-3G", WATER, 10, -10), ("nh3_sto3g", "STO-3G", AMMONIA, 10, -10),
         ("h2o_631g", "6-31G", WATER, 10, -10), ("h2o_ccpvdz", "cc-pVDZ", WATER, 10, -10),
         ("o_ccpvtz", "cc-pVTZ", "8,0,0,0", 8, -6)]
HYDROXYL = "8,0,0,0;1,1.8,0,0"
# the reference's UHF (get_Energy(toler, 1)) on open shells: basis fixture, n_up, n_down
UHF_CASES = [("oh_sto3g", 5, 4), ("h2o_sto3g", 5, 4), ("oh_631g", 5, 4), ("h2o_sto3g", 6, 4)]
CASES += [("oh_sto3g", "STO-3G", HYDROXYL, 9, -10), ("oh_631g", "6-31G", HYDROXYL, 9, -10)]
FULL_MAX = 13
SAMPLE = 3000


def load_dump(path: Path) -> dict:
    b = path.read_bytes()
    off = 0

    def take(dtype, k):
        nonlocal off
        a = np.frombuffer(b, dtype, k, off).copy()
        off += a.nbytes
        return a

    na, n, mp, ne = (int(x) for x in take(np.int32, 4))
    d = dict(nelec=ne, Z=take(np.float64, na), R=take(np.float64, 3 * na).reshape(na, 3))
    d["atom"] = take(np.int32, n)
    d["nprim"] = take(np.int32, n)
    d["powers"] = take(np.int32, 3 * n).reshape(n, 3)
    d["alpha"] = take(np.float64, n * mp).reshape(n, mp)
    d["coef"] = take(np.float64, n * mp).reshape(n, mp)
    for k in ("S", "lap", "nuc"):
        d[k] = take(np.float64, n * n).reshape(n, n)
    d["eri_full"] = take(np.float64, n ** 4).reshape(n, n, n, n)
    tail = take(np.float64, 2 + n)
    d["e_nuc"], d["e_hf"], d["eps"] = tail[0], tail[1], tail[2:]
    d["C"] = take(np.float64, n * n).reshape(n, n)
    assert off == len(b)
    return d


def unique_quartets(n: int) -> np.ndarray:
    out = []
    for i in range(n):
        for j in range(i + 1):
            for k in range(i + 1):
                for l in range(k + 1 if k < i else j + 1):
                    out.append((i, j, k, l))
    return np.array(out, dtype=np.int32)


def main():
    from oracle.ref_build.build_ref import build
    if not build(quiet=True):
        sys.exit("reference sources not present")
    exe = ROOT / "oracle" / "_ref" / "ref_ints"
    with tempfile.TemporaryDirectory() as tmp:
        for name, basis, atoms, ne, tol in CASES:
            dump = Path(tmp) / f"{name}.bin"
            subprocess.run([str(exe), basis, atoms, str(ne), str(tol), str(dump)], check=True, cwd=tmp,
                           capture_output=True)
            d = load_dump(dump)
            n = d["atom"].shape[0]
            G = d.pop("eri_full")
            if n <= FULL_MAX:
                d["eri"] = G
            else:
                q = unique_quartets(n)
                rng = np.random.default_rng(2024)
                sel = np.sort(rng.choice(len(q), size=min(SAMPLE, len(q)), replace=False))
                d["eri_idx"] = q[sel]
                d["eri_val"] = G[tuple(q[sel].T)]
            d["basis_name"] = np.array(basis)
            d["log10_tol"] = np.array(tol)
            np.savez_compressed(HERE / f"ints_{name}.npz", **d)
            print(f"ints_{name}.npz: nbf {n}, E_HF {d['e_hf']:.12f}")
        spec = {name: (basis, atoms, ne) for name, basis, atoms, ne, _ in CASES}
        uhf = []
        for name, nu, nd in UHF_CASES:
            basis, atoms, ne = spec[name]
            out = subprocess.run([str(exe), basis, atoms, str(ne), "-10", str(Path(tmp) / "u.bin"), "uhf", str(nu),
                                  str(nd)], check=True, cwd=tmp, capture_output=True, text=True).stdout.split()
            uhf.append(dict(basis_fixture=f"ints_{name}.npz", n_up=nu, n_down=nd, log10_tol=-10,
                            e_uhf=float(out[-2]), steps=int(out[-1])))
            print(f"UHF {name} ({nu}, {nd}): {uhf[-1]['e_uhf']:.12f}")
        import json
        (HERE / "reference_uhf.json").write_text(json.dumps(uhf, indent=1) + "\n")


if __name__ == "__main__":
    main()
