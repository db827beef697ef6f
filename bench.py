"""Benchmark: CCSD seconds per amplitude update on one GB300, split-precision
tensor-core path vs. the plain FP64 path, at |dE_corr| <= 1e-8 Eh.

Workload (default): synthetic closed-shell CCSD, nocc = 24, nvir = 300,
naux = 900 (seeded DF factors, 65 GB (vv|vv) block in HBM), DIIS(6).  One
step = one amplitude update (residual + denominator update + DIIS + energy).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision split3]
    python bench.py --impl reference ...   # CPU implementation of the update

The headline `value` is the mean device time of the K timed updates (CUDA
events on the engine's stream, integrals resident in HBM).  `e2e` is the
same metric through the C ABI from host buffers: ccsd_create (upload + block
build) + ccsd_solve (W + K updates) + amplitude read-back, wall clock, divided
by the updates.  Under torchrun (N > 1) every rank solves its own replica
(the path has no exchange step on one system); value is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "CCSD s/iteration + TFLOP/s: split-prec vs FP64 GPU at |ΔE_corr|≤1e-8 Eh"
UNIT = "s/iteration"
WORKLOAD = dict(nocc=24, nvir=300, naux=900, seed=2024, diis=6)
SLICES = {"split2": 3, "split3": 6, "split4": 10}   # BF16 products per split contraction
SLICES_PLANES = {"split2": 2, "split3": 3, "split4": 4}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--only", default="", choices=["", "scf"],
                    help="scf: only the integrals + RHF measurement (a water cluster), one JSON line")
    ap.add_argument("--waters", type=int, default=6, help="cluster size for --only scf")
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split3", choices=["split2", "split3", "split4"])
    ap.add_argument("--nocc", type=int, default=WORKLOAD["nocc"])
    ap.add_argument("--nvir", type=int, default=WORKLOAD["nvir"])
    ap.add_argument("--naux", type=int, default=WORKLOAD["naux"])
    ap.add_argument("--fp64-updates", type=int, default=6,
                    help="updates of the FP64 comparison run (0 skips it)")
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--compare-split2", type=int, default=1,
                    help="also time the two-plane split and state its accuracy (split3 runs only)")
    ap.add_argument("--extras", type=int, default=1,
                    help="also measure the Lambda gradient at this workload and the 64-system batched solve")
    ap.add_argument("--method", default="ccsd", choices=["ccsd", "ccsdt-1a"],
                    help="amplitude equations of the timed run (ccsdt-1a: no DIIS, as the reference runs it)")
    ap.add_argument("--sites-out", default="",
                    help="write the per-contraction-site device profile of the profiled run (JSON) here")
    return ap.parse_args()


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"  # gloo reduces host tensors
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"ccsd_bench_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), power=float(parts[3]),
                                 hw=parts[5], hwt=parts[6], swt=parts[7], swp=parts[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        smax = max(r["smax"] for r in rows)
        load = [r for r in rows if r["power"] > 300.0] or rows
        reasons = set()
        for r in rows:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("swp", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in load), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(rows), "samples_under_load": len(load),
                "power_w_max": max(r["power"] for r in rows)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def ladder_traffic(nocc, nvir):
    """DRAM bytes of one pp ladder (its two pair-form launches) from the
    committed ncu capture (profiles/pp_ladder_pairs_traffic.json, a smaller
    nvir at the same nocc), scaled to this nvir by the split W+/W- plane
    bytes, which grow as nvir^4."""
    p = ROOT / "profiles" / "pp_ladder_pairs_traffic.json"
    if not p.exists():
        return None, None
    d = json.loads(p.read_text())
    if d["nocc"] != nocc:
        return None, d
    return d["dram_bytes_per_ladder"] * (nvir / d["nvir"]) ** 4, d


def workload_config(args, world=1):
    """The `config` object of both arms (the same workload, so the same dict)."""
    o, v, q = args.nocc, args.nvir, args.naux
    return dict(workload=f"synthetic closed-shell {args.method.upper()} nocc={o} nvir={v} naux={q} (seed "
                         f"{WORKLOAD['seed']}), DIIS({WORKLOAD['diis']}), 1 step = 1 amplitude update",
                precision=args.precision, l2="inputs larger than L2: split W+/W- planes "
                f"{SLICES_PLANES.get(args.precision, 0) * 2 * (v * (v + 1) // 2) ** 2 * 2 / 1e9:.0f} GB "
                "resident in HBM",
                parallelism="replicas" if world > 1 else "single GPU")


CPU_SAMPLE = ("complete FP64 amplitude updates (residual, denominators, DIIS(6), energy; no term sampled) of "
              "the closed-shell restatement of the reference's CCSD map (oracle.cpu_update, numpy + OpenBLAS on "
              "all host threads, pp ladder in the engine's pair form); integral blocks and W+/W- built once "
              "outside the timed steps")


def cpu_full_update(o, v, q, steps=1):
    """Seconds of `steps` complete CPU updates at this workload (after one untimed set-up)."""
    from oracle import synthetic as syn
    from oracle.cpu_update import FullUpdate, cores
    fock, df = syn.make_system(o, v, q, WORKLOAD["seed"])
    t0 = time.perf_counter()
    s = FullUpdate(fock, o, df, diis_size=WORKLOAD["diis"], diis_start=2)
    setup = time.perf_counter() - t0
    res = [s.step() for _ in range(steps)]
    return res, setup, cores()


def run_reference(args, rank, world):
    """The CPU implementation of the path on the host cores: the oracle port (the
    reference's sources are not on this host), on this arm's workload, every step
    one complete update.  It maps none of this repository's libraries."""
    if rank != 0:
        return
    from oracle import synthetic as syn
    from oracle.cpu_update import FullUpdate, cores
    fock, df = syn.make_system(args.nocc, args.nvir, args.naux, WORKLOAD["seed"])
    t0 = time.perf_counter()
    s = FullUpdate(fock, args.nocc, df, diis_size=WORKLOAD["diis"], diis_start=2)
    setup = time.perf_counter() - t0
    for _ in range(args.warmup):
        s.step()
    times = [s.step()["seconds"] for _ in range(args.steps)]
    v = float(np.mean(times))
    sample = f"{CPU_SAMPLE}; set-up {setup:.1f} s; {args.warmup} untimed + {args.steps} timed updates"
    line = dict(impl="reference", metric=METRIC, value=v, unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=v * 1e3, higher_is_better=False, scaling="weak",
                vs_baseline=None, dtype="f64", data="synthetic", config=workload_config(args, world),
                cpu_baseline=dict(value=v, unit=UNIT, cores=cores(), kind="port", sample=sample),
                e2e=dict(value=v, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                tflops_alg=flops_per_update(args.nocc, args.nvir) / v / 1e12, e_corr=s.energy(s.t1, s.t2))
    print(json.dumps(line), flush=True)


def flops_per_update(o, v):
    """The fixed algorithmic count 2 o^2 v^4 + 4 o^4 v^2 + 8 o^3 v^3 (ccsd_flops_per_update)."""
    o, v = float(o), float(v)
    return 2 * o ** 2 * v ** 4 + 4 * o ** 4 * v ** 2 + 8 * o ** 3 * v ** 3


def measure_extras(cg, fock, df, o, precision):
    """Untimed-by-the-headline extras: the Lambda gradient (dE/dB) at the bench
    workload and the batched solve of 64 small systems (nocc 4..12, nvir 20..80)."""
    out = {}
    t0 = time.perf_counter()
    with cg.Solver(fock, o, df=df, precision=precision, energy_tol=1e-9, diis_size=WORKLOAD["diis"],
                   diis_start=2) as s:
        r = s.solve(amplitudes=False)
        t1 = time.perf_counter()
        g = s.lambda_grad(tol=1e-8, max_iter=200)
        t2 = time.perf_counter()
    out["gradient"] = dict(workload="dE_corr/dB and dE_corr/dfock at this workload after a 1e-9 solve",
                           precision=precision, solve_s=t1 - t0, solve_updates=r["iterations"],
                           lambda_grad_s=t2 - t1, lambda_iterations=g["iterations"],
                           lambda_residual=g["residual_norm"])
    # C2 (o=10, v=90, naux=300): the reference's own CCSD_Memory_optimized::CCSD, compiled unchanged,
    # takes a median 248.9 s per iteration on one x86-64 core (its own clock, 8 iterations to 1e-10)
    f2, b2 = cg.make_synthetic(10, 90, 300, 2024)
    c2 = dict(workload="synthetic o=10 v=90 naux=300 (seed 2024), 7 updates from the MP2 start",
              reference_memory_optimized_s_per_iteration=248.9,
              reference_note="CCSD_Memory_optimized::CCSD compiled unchanged, single rank, 1 x86-64 core, median of its "
                             "own per-iteration clock")
    for prec in ("fp64", precision):
        r2 = cg.solve(f2, 10, df=b2, fixed_iterations=7, precision=prec, amplitudes=False)
        c2[prec + "_update_ms"] = float(np.median(r2["update_ms"][1:]))
        c2[prec + "_e_corr"] = r2["e_corr"]
    out["c2"] = c2
    rng = np.random.default_rng(4)
    systems = []
    for k in range(64):
        so, sv = int(rng.integers(4, 13)), int(rng.integers(20, 81))
        f_k, b_k = cg.make_synthetic(so, sv, 3 * (so + sv) // 2, 1000 + k)
        systems.append(dict(fock=f_k, nocc=so, df=b_k))
    def timed_batch(prec):
        with cg.Batch(systems, energy_tol=1e-10, precision=prec) as b:
            b.solve(amplitudes=False)                 # autotunes, splits constants, captures the graphs
            t0 = time.perf_counter()
            res = b.solve(amplitudes=False)
            return res, time.perf_counter() - t0, b.report()

    rb, tb, rep = timed_batch("fp64")
    rs, ts3, rep3 = timed_batch(precision)
    solvers = [cg.Solver(**sy, energy_tol=1e-10) for sy in systems]
    for sv_ in solvers:
        sv_.solve(amplitudes=False)
    t0 = time.perf_counter()
    for sv_ in solvers:
        sv_.solve(amplitudes=False)
    ts = time.perf_counter() - t0
    for sv_ in solvers:
        sv_.close()
    flops = sum(x["flops_per_update"] * x["iterations"] for x in rb)
    nsplit = sum(1 for op in rep3["ops"] if op["kind"] == "contraction" and op.get("path") == "split")
    out["batch_c4"] = dict(workload="64 synthetic systems, nocc in [4,12], nvir in [20,80], tol 1e-10",
                           batched_fp64_s=tb, sequential_fp64_s=ts, speedup_fp64=ts / tb,
                           batched_split_s=ts3, split_precision=precision, speedup_split_vs_sequential=ts / ts3,
                           split_contraction_sites=nsplit,
                           max_abs_dE_split_vs_fp64=max(abs(x["e_corr"] - y["e_corr"]) for x, y in zip(rs, rb)),
                           system_updates=sum(x["iterations"] for x in rb),
                           algorithmic_tflops_fp64=flops / tb / 1e12, algorithmic_tflops_split=flops / ts3 / 1e12,
                           launches_per_update=rep["launches_per_update"])
    return out


def measure_ccsdt1a(cg, precision, pk):
    """CCSDT-1a (the reference's CCSDT::Calc_Energy(toler, 1), T3 in spin
    orbitals) at a synthetic nocc=6, nvir=40 system: per-update device time in
    FP64 and split precision, the T3 assembly's HBM roofline, and at a small
    size (nocc=4, nvir=16) the update time of the spin-orbital oracle on the
    host beside the GPU's."""
    from oracle.ccsd_spinorb import SpinOrbitalCCSD
    from oracle.cpu_update import cores
    o, v = 6, 40
    O, V = 2 * o, 2 * v
    n3 = V ** 3 * O ** 3
    fock, b = cg.make_synthetic(o, v, 3 * (o + v) // 2, 77)
    out = dict(workload=f"synthetic nocc={o} nvir={v} naux={3 * (o + v) // 2} (seed 77), CCSDT-1a, "
                        f"T3 = {n3 * 8 / 1e9:.1f} GB in spin orbitals, 5 updates from the MP2 start")
    e = {}
    for prec in ("fp64", precision):
        with cg.Solver(fock, o, df=b, precision=prec, method="ccsdt-1a", fixed_iterations=5, profile=True) as s:
            r = s.solve(amplitudes=False)
            prof = s.profile()
        e[prec] = r["e_corr"]
        upd = float(np.median(r["update_ms"][1:]))
        sites = {x["site"]: x for x in prof["sites"]}
        t3 = {k: sites[k]["ms"] / sites[k]["calls"] for k in sites if k.startswith(("T3_", "R1_T3", "R2_T3"))}
        out[prec] = dict(update_ms=upd, triples_sites_ms=t3)
        if prec == "fp64":
            asm = t3["T3_assemble"]
            # per virtual triple a<b<c: three Y and three Z slabs of O^3 read, six t3 slabs written
            triples = V * (V - 1) * (V - 2) // 6
            bytes_alg = 8.0 * 12 * triples * O ** 3
            out["assemble_roofline"] = dict(bound="hbm", achieved=bytes_alg / asm / 1e6, peak=pk["hbm_gbs"],
                                            unit="GB/s", frac=bytes_alg / asm / 1e6 / pk["hbm_gbs"],
                                            basis="12 O^3 doubles per virtual triple a<b<c (3 Y + 3 Z slabs "
                                                  "read, 6 t3 slabs written) / CUDA-event time",
                                            bytes_per_launch=bytes_alg, ms=asm)
    out["abs_dE_split_vs_fp64"] = abs(e[precision] - e["fp64"])
    # CCSDT-1b (Method_Nr 2: + the T3 T1 term of T2), CCSDT-2 (Method_Nr 3: + dressed
    # X1/X2 and the X12/X13 terms of T3) and CCSDT-3 (Method_Nr 4: + T1 terms and X14/X15)
    # on the same system; CCSDT-4 (Method_Nr 5: + X3/X4/X6 terms of T3) and CCSDT (Method_Nr 6:
    # + T3 in X1/X2, dressed X3/X4/X6, X7/X8), whose X4 term is O(V^5 O^3), on a smaller one
    mo, mv_ = 4, 24
    f_m, b_m = cg.make_synthetic(mo, mv_, 3 * (mo + mv_) // 2, 79)
    for meth in ("ccsdt-1b", "ccsdt-2", "ccsdt-3", "ccsdt-4", "ccsdt"):
        small = meth in ("ccsdt-4", "ccsdt")
        ms = {"workload": f"synthetic nocc={mo} nvir={mv_} (seed 79)"} if small else {}
        for prec in ("fp64", precision):
            with cg.Solver(*((f_m, mo) if small else (fock, o)), df=b_m if small else b, precision=prec,
                           method=meth, fixed_iterations=5, profile=small) as s:
                r = s.solve(amplitudes=False)
                if small:
                    top = sorted(s.profile()["sites"], key=lambda x: -x["ms"])[:6]
                    ms[prec + "_top_sites_ms"] = {x["site"]: x["ms"] / x["calls"] for x in top}
            ms[prec + "_update_ms"] = float(np.median(r["update_ms"][1:]))
            ms[prec + "_e_corr"] = r["e_corr"]
        out[meth.replace("-", "")] = ms
    so, sv = 4, 16
    f_s, b_s = cg.make_synthetic(so, sv, 3 * (so + sv) // 2, 78)
    eri = np.einsum("Qpq,Qrs->pqrs", b_s, b_s)
    ref = SpinOrbitalCCSD(f_s, eri, so, method=1)
    t1, t2 = ref.mp2_guess()
    t3 = np.zeros((2 * sv,) * 3 + (2 * so,) * 3)
    t0 = time.perf_counter()
    for _ in range(3):
        t1, t2, t3 = ref.update(t1, t2, t3)
    cpu_ms = (time.perf_counter() - t0) / 3 * 1e3
    with cg.Solver(f_s, so, df=b_s, method="ccsdt-1a", fixed_iterations=5) as s:
        r = s.solve(amplitudes=False)
    out["small"] = dict(workload=f"synthetic nocc={so} nvir={sv} (seed 78)", gpu_fp64_update_ms=float(
        np.median(r["update_ms"][1:])), cpu_port_update_ms=cpu_ms, cpu_kind="port (numpy, spin orbitals)",
        cpu_cores=cores())
    return out


def water_cluster(d, k: int, spacing: float = 5.6) -> dict:
    """k copies of a one-water basis description (the reference's own exponents and
    normalised coefficients, tests/golden/ints_*.npz) on a cubic grid of the given
    spacing (bohr)."""
    side = int(np.ceil(k ** (1.0 / 3.0) - 1e-9))
    shifts = [np.array([x, y, z]) * spacing for x in range(side) for y in range(side) for z in range(side)][:k]
    na = len(d["Z"])
    return dict(Z=np.tile(d["Z"], k), R=np.concatenate([d["R"] + s for s in shifts]),
                atom=np.concatenate([d["atom"] + na * w for w in range(k)]), powers=np.tile(d["powers"], (k, 1)),
                nprim=np.tile(d["nprim"], k), alpha=np.tile(d["alpha"], (k, 1)), coef=np.tile(d["coef"], (k, 1)))


def measure_scf(cg, k: int = 6) -> dict:
    """The CCSD inputs' producer on a water cluster in cc-pVDZ (the reference's H2O
    basis description tiled k times): the GPU integrals alone (device outputs; unique
    quartets (ij|kl), ij >= kl, and their primitive quartets per second), the whole
    RHF, and the integral oracle's quartet rate on the host for comparison."""
    import ctypes as C
    import torch
    from ccsd_parallel_gb300 import _abi
    from oracle.gto_ints import Basis, Integrals
    d = np.load(Path(__file__).parent / "tests" / "golden" / "ints_h2o_ccpvdz.npz")
    bas = water_cluster(d, k)
    n = len(bas["atom"])
    pp = np.array([bas["nprim"][i] * bas["nprim"][j] for i in range(n) for j in range(i + 1)], dtype=np.float64)
    npair = len(pp)
    quartets = npair * (npair + 1) // 2
    prim_quartets = (pp.sum() ** 2 + (pp ** 2).sum()) / 2
    b, keep = cg._basis(bas)
    G = torch.empty(n ** 4, dtype=torch.float64, device="cuda")
    S = torch.empty(n * n, dtype=torch.float64, device="cuda")
    e_nuc = C.c_double()
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _abi.check(_abi.lib().ccsd_ao_integrals(C.byref(b), S.data_ptr(), None, None, G.data_ptr(), C.byref(e_nuc),
                                                1, None))
        times.append(time.perf_counter() - t0)
    t_int = float(np.median(times))
    del G, S
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    scf = cg.rhf(bas, 10 * k, tol=1e-10, eri=False)
    t_scf = time.perf_counter() - t0
    # the oracle on a few quartets of the same basis
    I = Integrals(Basis.from_dict(bas))
    rng = np.random.default_rng(0)
    sample = rng.integers(0, n, size=(12, 4))
    t0 = time.perf_counter()
    for q in sample:
        I.eri(*map(int, q))
    cpu_q_per_s = len(sample) / (time.perf_counter() - t0)
    return dict(workload=f"(H2O)_{k} cc-pVDZ, {n} Cartesian basis functions, grid spacing 5.6 bohr",
                nbf=n, unique_quartets=quartets, primitive_quartets=prim_quartets,
                integrals_s=t_int, quartets_per_s=quartets / t_int, primitive_quartets_per_s=prim_quartets / t_int,
                eri_gb=n ** 4 * 8 / 1e9,
                rhf_s=t_scf, rhf_iterations=scf["iterations"], e_hf=scf["e_hf"],
                cpu_port_quartets_per_s=cpu_q_per_s,
                cpu_port_note="the numpy integral oracle (oracle/gto_ints.py), one thread, on 12 sampled quartets")


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import ccsd_parallel_gb300 as cg
    if args.only == "scf":
        if rank == 0:
            print(json.dumps(measure_scf(cg, args.waters)), flush=True)
        return
    o, v, q = args.nocc, args.nvir, args.naux
    W, K = max(args.warmup, 3), args.steps
    U = W + K
    fock, df = cg.make_synthetic(o, v, q, WORKLOAD["seed"] + 0)
    pk, pk_kind = peaks()

    # process start-up (CUDA context, module load) outside the timed region: two updates
    # of a small system through the same API
    fw, bw = cg.make_synthetic(6, 40, 120, 7)
    with cg.Solver(fw, 6, df=bw, precision=args.precision, fixed_iterations=2, diis_size=0,
                   method=args.method) as w:
        w.solve(amplitudes=False)

    # ---- split-precision run: e2e wall clock + per-update device events ----
    barrier(world)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t0 = time.perf_counter()
        diis = WORKLOAD["diis"] if args.method == "ccsd" else 0
        s = cg.Solver(fock, o, df=df, precision=args.precision, fixed_iterations=U,
                      diis_size=diis, diis_start=2, method=args.method)
        r = s.solve(amplitudes=True)
        t1 = time.perf_counter()
    # The same solve again with per-site CUDA events (profile mode), for the ladder's
    # launch times and the launch count.  It issues the kernels directly: an update
    # replayed from a CUDA graph (the timed solve above, from its second update on)
    # cannot carry the per-site events.
    s.set_options(precision=args.precision, fixed_iterations=U, diis_size=diis, diis_start=2,
                  method=args.method, profile=True)
    rp = s.solve(amplitudes=False)
    prof = s.profile()
    # the two-plane form (hi/lo BF16, 3 products) on the same system, for its time and its
    # accuracy against the FP64 run below; the split3 line above is the headline
    r2 = None
    if args.precision == "split3" and args.compare_split2 and args.method == "ccsd":
        s.set_options(precision="split2", fixed_iterations=U, diis_size=diis, diis_start=2, method=args.method)
        r2 = s.solve(amplitudes=True)
    s.close()
    profiled_ms = float(np.asarray(rp["update_ms"])[W:W + K].mean())
    if args.sites_out and rank == 0:
        Path(args.sites_out).write_text(json.dumps(prof, indent=1))
    ms = np.asarray(r["update_ms"])
    timed_ms = ms[W:W + K]
    value = max_over_ranks(float(timed_ms.mean()) / 1e3, world)
    e2e_s = max_over_ranks((t1 - t0) / U, world)
    sites = {x["site"]: x for x in prof["sites"]}
    # the pp ladder runs as two pair-form contractions (S+ = W+ tau+^T, S- = W- tau-^T); its
    # algorithmic count stays the fixed 2 o^2 v^4 of the plain formulation
    lad_sites = [sites[k] for k in ("pp_ladder_sym", "pp_ladder_anti") if k in sites]
    lad_ms = sum(x["ms"] / x["calls"] for x in lad_sites)
    lad_exec = sum(x["flops"] / x["calls"] for x in lad_sites)   # 2 M N K of the two contractions
    lad_flops = 2.0 * o * o * float(v) ** 4
    nprod = SLICES[args.precision]
    peak_t = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    achieved = lad_flops / (lad_ms * 1e-3) / 1e12
    hw_tflops = lad_exec * nprod / (lad_ms * 1e-3) / 1e12
    traffic, traffic_src = ladder_traffic(o, v)
    flops_upd = r["flops_per_update"]
    # kernels per update: the profiled solve's count (a graph replays the same kernels)
    launches = prof.get("launches", 0) / max(prof["updates"], 1) * K

    # ---- FP64 comparison run (same inputs, same number of updates) --------
    fp64 = {}
    split2 = None
    nf = min(args.fp64_updates, U)
    if nf > 0:
        with cg.Solver(fock, o, df=df, precision="fp64", fixed_iterations=nf, diis_size=diis,
                       diis_start=2, method=args.method) as s64:
            r64 = s64.solve(amplitudes=True)
        ms64 = np.asarray(r64["update_ms"])
        f64_s = float(ms64[min(2, nf - 1):].mean()) / 1e3
        de = abs(r["energies"][nf] - r64["energies"][nf])
        if r2 is not None:
            s2 = float(np.asarray(r2["update_ms"])[W:W + K].mean()) / 1e3
            split2 = dict(s_per_iteration=s2, speedup_vs_fp64=f64_s / s2,
                          abs_dE_corr_vs_fp64=abs(r2["energies"][nf] - r64["energies"][nf]), compared_at_update=nf,
                          max_abs_dT2_vs_fp64=float(np.abs(r2["t2"] - r64["t2"]).max()) if nf == U else None)
        fp64 = dict(fp64_s_per_iteration=f64_s, speedup_vs_fp64=f64_s / value,
                    abs_dE_corr_vs_fp64=de, compared_at_update=nf,
                    max_abs_dT2_vs_fp64=float(np.abs(r["t2"] - r64["t2"]).max()) if nf == U else None,
                    e_corr_fp64=r64["energies"][nf], fp64_tflops_alg=flops_upd / f64_s / 1e12)

    cpu = None
    if args.cpu_baseline and rank == 0:
        res, setup, ncores = cpu_full_update(o, v, q, steps=1)
        cpu = dict(value=res[0]["seconds"], unit=UNIT, cores=ncores, kind="port",
                   sample=f"one {CPU_SAMPLE.replace('updates', 'update', 1)}; set-up {setup:.1f} s")

    extras = {}
    if args.extras and rank == 0:
        extras = measure_extras(cg, fock, df, o, args.precision)
        extras["ccsdt1a"] = measure_ccsdt1a(cg, args.precision, pk)
        extras["scf"] = measure_scf(cg)

    if rank != 0:
        return
    h2d = fock.nbytes + df.nbytes
    d2h = (o * v + o * o * v * v) * 8 + 8 * (U + 1)
    line = dict(
        metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=K, warmup=W,
        ms_per_step=value * 1e3, higher_is_better=False, scaling="weak", vs_baseline=None,
        dtype=f"bf16x{nprod}-products/fp32-acc + f64 ({args.precision})", data="synthetic",
        config=workload_config(args, world),
        tflops_alg=flops_upd / value / 1e12,
        e_corr=r["energies"][U], abs_dE_corr_vs_fp64=fp64.get("abs_dE_corr_vs_fp64"),
        **{k: val for k, val in fp64.items() if k != "abs_dE_corr_vs_fp64"},
        roofline=dict(bound="tensor", achieved=achieved, peak=peak_t, unit="TFLOP/s", frac=achieved / peak_t,
                      traffic=traffic,
                      kernel="split_gemm_kernel x2 (pp ladder in pair form: S+ = W+ tau+^T over a>=b, i>=j, "
                             "c>=d; S- = W- tau-^T over strict pairs)",
                      achieved_basis="algorithmic 2 o^2 v^4 per ladder / CUDA-event time of its two launches",
                      hw_tflops=hw_tflops, hw_frac=hw_tflops / peak_t,
                      executed_tflop_per_ladder=lad_exec / 1e12,
                      peak_source=f"bf16_tflops_sustained of {pk_kind}", ladder_ms=lad_ms,
                      timed_in=f"profiled solve of the same workload right after the timed one "
                               f"(updates {W}..{U - 1}; {profiled_ms:.2f} ms per update without graphs)"),
        cpu_baseline=cpu,
        split2=split2,
        e2e=dict(value=e2e_s, unit=UNIT, h2d_bytes_per_step=h2d / U, d2h_bytes_per_step=d2h / U,
                 includes="ccsd_create (H2D of fock + DF factors, block build) + ccsd_solve + T1/T2 read-back; "
                          "the CUDA context and most kernel loads happen before it (a 2-update solve of o=6, v=40)"),
        gpu_launches=int(round(launches)),
        clocks=clk.summary(),
        **extras,
    )
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
