"""The C++ drop-in header (include/ccsd_gb300.hpp): it compiles against the C
ABI header on the CPU, and on the GPU a C++ host program built on it gives
the oracle's converged energy through the reference's stopping rule."""
import json
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
EXAMPLE = ROOT / "ccsd_parallel_gb300" / "examples" / "dropin_synthetic.cpp"
LIBDIR = ROOT / "ccsd_parallel_gb300" / "_lib"


def test_header_and_example_compile():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(ROOT / "include"), str(EXAMPLE)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_host_program_matches_golden(tmp_path):
    exe = tmp_path / "dropin"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(EXAMPLE), "-L", str(LIBDIR),
                    "-lccsd_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], check=True)
    c = json.loads((ROOT / "tests" / "golden" / "synthetic_oracle.json").read_text())["syn_o10_v90_q300_s2024_sig0.05"]
    out = subprocess.run([str(exe), "10", "90", "300", "2024", "-10"], capture_output=True, text=True, check=True).stdout
    line = out.split()
    assert int(line[1]) == c["iter"]
    assert abs(float(line[3]) - c["e_corr"]) < 1e-10


INCAR_MAIN = ROOT / "ccsd_parallel_gb300" / "examples" / "ccsd_incar.cpp"


def test_incar_program_compiles():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(ROOT / "include"), str(INCAR_MAIN)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_incar_program_runs_h2o(tmp_path):
    """The reference's program flow (read INCAR, Initializer::Go) as a C++ program
    on the engine: H2O 6-31G CCSD gives the reference's total energy."""
    import numpy as np
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from incar_util import g94_from_fixture, incar_text
    d = np.load(ROOT / "tests" / "golden" / "ints_h2o_631g.npz")
    h = np.load(ROOT / "tests" / "golden" / "h2o_631g_config_tol10.npz")
    (tmp_path / "INCAR").write_text(incar_text(d, "CCSD", -10))
    (tmp_path / "basis.g94").write_text(g94_from_fixture(d))
    exe = tmp_path / "ccsd_incar"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(INCAR_MAIN), "-L", str(LIBDIR),
                    "-lccsd_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path / "INCAR"), str(tmp_path / "basis.g94")], capture_output=True,
                         text=True, check=True).stdout
    energy = float(out.strip().splitlines()[-1].split("=")[1])
    assert abs(energy - float(h["ref_e_total"])) < 1e-9  # Method CCSD = the memory-optimised class
