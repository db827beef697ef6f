"""Compile the reference's own C++ sources, unchanged, into oracle/_ref/
(TEST INFRASTRUCTURE ONLY).

The sources stay where they lie in the read-only reference tree; only object
files and two drivers are written, into oracle/_ref/ (git-ignored).  The
reference needs Armadillo and MPI, neither of which is installed; the
project-written headers under oracle/ref_build/shim/ provide the Armadillo
subset and a single-rank MPI it uses.  Its unguarded `#include
"../../home/ole/Desktop/include/armadillo"` resolves through the include
directory shim/x/y.  Flags: -O2 and -ftrivial-auto-var-init=zero, which gives
the uninitialised `double temp` read in the reference's W_4 build
(ccsd_memory_optimized.cpp:4789,4837) the value 0 it has on the even path.

    python -m oracle.ref_build.build_ref        # builds ref_synthetic, ref_probe, ref_h2o and ref_ints

The reference tree is read from $CCSD_REFERENCE_DIR, default /root/reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
REFERENCE = Path(os.environ.get("CCSD_REFERENCE_DIR", "/root/reference"))
SHIM = HERE / "shim"
FLAGS = ["-std=c++17", "-O2", "-ftrivial-auto-var-init=zero", "-w",
         "-I", str(SHIM / "x" / "y"), "-I", str(SHIM), "-I", str(REFERENCE)]

COMMON = ["ccsd_memory_optimized", "ccsd_non_iterative_part", "hartree_integrals", "ccsdt"]
SCF = ["hartree_fock_solver", "fill_alpha", "fill_alpha2", "matrix_size_setter"]


def _compile(src: Path, obj: Path):
    if obj.exists() and obj.stat().st_mtime > max(src.stat().st_mtime, *(p.stat().st_mtime for p in SHIM.rglob("*") if p.is_file())):
        return
    r = subprocess.run(["g++", *FLAGS, "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{r.stderr[-4000:]}")


def build(quiet: bool = False) -> bool:
    """Build the drivers; returns False when the reference sources are absent."""
    if not (REFERENCE / "ccsd_memory_optimized.cpp").exists():
        if not quiet:
            print("reference sources not present: oracle/_ref not built")
        return False
    OUT.mkdir(exist_ok=True)
    jobs = [(REFERENCE / f"{s}.cpp", OUT / f"{s}.o") for s in COMMON + SCF]
    jobs += [(HERE / f"{d}.cpp", OUT / f"{d}.o") for d in ("ref_synthetic", "ref_probe", "ref_h2o", "ref_ints")]
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        list(ex.map(lambda a: _compile(*a), jobs))
    common = [str(OUT / f"{s}.o") for s in COMMON]
    for exe, extra in (("ref_synthetic", ["ref_synthetic.o"]), ("ref_probe", ["ref_probe.o"]),
                       ("ref_h2o", ["ref_h2o.o"] + [f"{s}.o" for s in SCF]),
                       ("ref_ints", ["ref_ints.o"] + [f"{s}.o" for s in SCF])):
        r = subprocess.run(["g++", "-o", str(OUT / exe), *[str(OUT / e) for e in extra], *common],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking {exe} failed:\n{r.stderr[-4000:]}")
    if not quiet:
        print(f"built ref_synthetic, ref_probe, ref_h2o and ref_ints in {OUT}")
    return True


if __name__ == "__main__":
    sys.exit(0 if build() else 1)
