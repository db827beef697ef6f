"""GB300-native CCSD amplitude engine (sm_103a CUDA behind a C ABI).

Python host binding over ``include/ccsd_gb300.h``.  The class
``CCSD_Memory_optimized`` mirrors the reference class of the same name
(``ccsd_memory_optimized.h:15-47``): construct it with the inputs of the
iterative part (MO Fock matrix, MO integrals, occupied count) and call
``CCSD(toler, print_stuff)``, which returns E_HF + E_corr exactly like the
reference method; the converged amplitudes and the correlation energy stay on
the object (``t1``, ``t2``, ``E_new``).

Every compute call goes through the CUDA library; when it is missing or no GPU
is present the call raises (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import (CCSD_INTS_AO_DENSE, CCSD_INTS_DF, CCSD_INTS_MO_DENSE, CCSD_INTS_SO_ANTISYM, CCSD_PREC_FP64,
                   CCSD_PREC_SPLIT2, CCSD_PREC_SPLIT3, CCSD_PREC_SPLIT4, CCSDError)

PRECISIONS = {"fp64": CCSD_PREC_FP64, "split2": CCSD_PREC_SPLIT2, "split3": CCSD_PREC_SPLIT3,
              "split4": CCSD_PREC_SPLIT4}

__all__ = ["Solver", "solve", "Batch", "solve_batched", "make_synthetic", "flops_per_update", "frozen_core_count",
           "ao_integrals", "rhf", "uhf", "ccsd_inputs", "parse_incar", "run_incar", "CCSD_Memory_optimized", "CCSDError",
           "PRECISIONS"]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def make_synthetic(nocc: int, nvir: int, naux: int, seed: int):
    """Seeded synthetic system from the library's generator: (fock, B[naux,n,n])."""
    n = nocc + nvir
    fock = np.empty((n, n))
    df = np.empty((naux, n, n)) if naux > 0 else None
    _abi.check(_abi.lib().ccsd_make_synthetic(nocc, nvir, naux, seed, _ptr(fock), _ptr(df)))
    return fock, df


def flops_per_update(nocc: int, nvir: int) -> float:
    return float(_abi.lib().ccsd_flops_per_update(nocc, nvir))


METHODS = {"ccsd": _abi.CCSD_METHOD_CCSD, "ccsdt-1a": _abi.CCSD_METHOD_CCSDT1A,
           "ccsdt-1b": _abi.CCSD_METHOD_CCSDT1B, "ccsdt-2": _abi.CCSD_METHOD_CCSDT2,
           "ccsdt-3": _abi.CCSD_METHOD_CCSDT3, "ccsdt-4": _abi.CCSD_METHOD_CCSDT4,
           "ccsdt": _abi.CCSD_METHOD_CCSDT}
# the reference's two CCSD maps: "ccsd" = the CCSD equations of its dense CCSD1
# (ccsdt.cpp:625-727); "memory_optimized" = CCSD_Memory_optimized as written,
# F_mi contracted transposed in T2 (ccsd_memory_optimized.cpp:2085-2086 and its
# five other spin cases)
VARIANTS = {"ccsd": _abi.CCSD_VARIANT_CCSD, "memory_optimized": _abi.CCSD_VARIANT_MEMORY_OPTIMIZED}


def _options(precision="fp64", energy_tol=1e-10, residual_tol=0.0, max_iter=999,
             fixed_iterations=0, diis_size=0, diis_start=0, verbose=False, profile=False,
             stream=None, method="ccsd", t1_start=None, t2_start=None, variant="ccsd"):
    o = _abi.Options()
    _abi.check(_abi.lib().ccsd_default_options(C.byref(o)))
    o.energy_tol = energy_tol
    o.residual_tol = residual_tol
    o.max_iter = max_iter
    o.fixed_iterations = fixed_iterations
    o.diis_size = diis_size
    o.diis_start = diis_start
    o.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.verbose = int(bool(verbose))
    o.profile = int(bool(profile))
    o.method = METHODS[method] if isinstance(method, str) else int(method)
    o.stream = stream
    # restart amplitudes: the arrays must outlive the solve, so the caller keeps them (Solver does)
    o.t1_start, o.t2_start = _ptr(t1_start), _ptr(t2_start)
    o.variant = VARIANTS[variant] if isinstance(variant, str) else int(variant)
    return o


def frozen_core_count(Z) -> int:
    """Frozen core orbitals by the reference's rule (one per atom with 2 < Z < 11;
    ``ccsd_frozen_core_count``) for the nuclear charges Z."""
    z = np.ascontiguousarray(Z, dtype=np.float64).ravel()
    rc = _abi.lib().ccsd_frozen_core_count(_ptr(z), z.size)
    _abi.check(min(rc, 0))
    return int(rc)


def _basis(basis, accurate_boys=False):
    """ccsd_basis over host arrays from a dict with the keys Z, R, atom, powers,
    nprim, alpha, coef (the reference's Set_Input description); returns
    (struct, arrays to keep alive)."""
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    Z, R = _f64(np.ravel(basis["Z"])), _f64(np.reshape(basis["R"], (-1, 3)))
    atom, powers, nprim = i32(basis["atom"]), i32(np.reshape(basis["powers"], (-1, 3))), i32(basis["nprim"])
    alpha, coef = _f64(np.atleast_2d(basis["alpha"])), _f64(np.atleast_2d(basis["coef"]))
    b = _abi.Basis()
    b.natoms, b.nbf, b.maxprim = Z.size, atom.size, alpha.shape[1]
    b.flags = _abi.CCSD_BASIS_ACCURATE_BOYS if accurate_boys else 0
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
    b.Z, b.R, b.alpha, b.coef = _ptr(Z), _ptr(R), _ptr(alpha), _ptr(coef)
    b.atom, b.powers, b.nprim = ip(atom), ip(powers), ip(nprim)
    return b, [Z, R, atom, powers, nprim, alpha, coef]


def ao_integrals(basis, eri: bool = True, accurate_boys: bool = False) -> dict:
    """S, T, V (= -sum_C Z_C <mu|1/r_C|nu>), the ERIs (mu nu|la si) and E_nuc of a
    contracted Cartesian Gaussian basis, computed on the GPU (ccsd_ao_integrals).
    accurate_boys: CCSD_BASIS_ACCURATE_BOYS (the reference's Boys function is
    reproduced by default)."""
    b, keep = _basis(basis, accurate_boys)
    n = b.nbf
    S, T, V = np.empty((n, n)), np.empty((n, n)), np.empty((n, n))
    G = np.empty((n, n, n, n)) if eri else None
    e_nuc = C.c_double()
    _abi.check(_abi.lib().ccsd_ao_integrals(C.byref(b), S.ctypes.data, T.ctypes.data, V.ctypes.data,
                                            None if G is None else G.ctypes.data, C.byref(e_nuc), 0, None))
    del keep
    return dict(S=S, T=T, V=V, eri=G, e_nuc=e_nuc.value)


def rhf(basis, n_electrons: int, tol: float = 1e-10, max_iter: int = 0, eri: bool = True,
        accurate_boys: bool = False) -> dict:
    """Closed-shell Hartree-Fock on the GPU integrals (ccsd_rhf), step for step as
    the reference's Hartree_Fock_Solver::get_Energy: e_hf, e_nuc, eps, C[mu][p],
    the AO integrals and the SCF step count.  ``ccsd_inputs(r)`` turns the result
    into the keyword arguments of :func:`solve` (AO input)."""
    b, keep = _basis(basis, accurate_boys)
    n = b.nbf
    r = _abi.ScfResult()
    eps, Cm = np.empty(n), np.empty((n, n))
    G = np.empty((n, n, n, n)) if eri else None
    r.eps, r.C, r.eri = _ptr(eps), _ptr(Cm), _ptr(G)
    _abi.check(_abi.lib().ccsd_rhf(C.byref(b), n_electrons, tol, max_iter, C.byref(r)))
    del keep
    return dict(e_hf=r.e_hf, e_nuc=r.e_nuc, iterations=r.iterations, converged=bool(r.converged), eps=eps,
                C=Cm, eri=G, nocc=n_electrons // 2)


def parse_incar(incar_text: str, basis_text: str = "") -> dict:
    """The reference's INCAR keywords and atoms with a Gaussian94 basis (or the
    INCAR's Basis_File), expanded to the ccsd_basis arrays (ccsd_incar_parse; host only)."""
    inc = _abi.Incar()
    lib = _abi.lib()
    a, b = incar_text.encode(), basis_text.encode()
    _abi.check(lib.ccsd_incar_parse(a, b, C.byref(inc)))
    na, n, mp = inc.natoms, inc.nbf, inc.maxprim
    out = dict(Z=np.empty(na), R=np.empty((na, 3)), atom=np.empty(n, np.int32), powers=np.empty((n, 3), np.int32),
               nprim=np.empty(n, np.int32), alpha=np.empty((n, mp)), coef=np.empty((n, mp)))
    inc.capacity_atoms, inc.capacity_bf, inc.capacity_prim = na, n, mp
    inc.Z, inc.R, inc.alpha, inc.coef = _ptr(out["Z"]), _ptr(out["R"]), _ptr(out["alpha"]), _ptr(out["coef"])
    ip = lambda x: x.ctypes.data_as(C.POINTER(C.c_int32))
    inc.atom, inc.powers, inc.nprim = ip(out["atom"]), ip(out["powers"]), ip(out["nprim"])
    _abi.check(lib.ccsd_incar_parse(a, b, C.byref(inc)))
    out.update(basis_set=inc.basis_set.decode(), method=inc.method.decode(), tol=inc.convergance_criteria,
               freeze_core=bool(inc.freeze_core), relax_pos=bool(inc.relax_pos), use_angstrom=bool(inc.use_angstrom),
               print_stuffies=bool(inc.print_stuffies), n_electrons=inc.n_electrons, nfrozen=inc.nfrozen)
    return out


def run_incar(incar_text: str, basis_text: str = "", precision="fp64") -> dict:
    """The reference's Initializer::Go on the engine (ccsd_incar_run): returns the
    energy it would print (E_HF for HF, E_HF + E_corr otherwise) and its parts."""
    r = _abi.IncarResult()
    prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    _abi.check(_abi.lib().ccsd_incar_run(incar_text.encode(), basis_text.encode(), prec, C.byref(r)))
    return dict(energy=r.energy, e_hf=r.e_hf, e_corr=r.e_corr, scf_iterations=r.scf_iterations, cc_iter=r.cc_iter,
                method=r.method, nbf=r.nbf)


def uhf(basis, n_up: int, n_down: int, tol: float = 1e-10, max_iter: int = 0, seed: int = 0,
        accurate_boys: bool = False) -> dict:
    """Unrestricted Hartree-Fock on the GPU integrals (ccsd_uhf), step for step as the
    reference's get_Energy(toler, 1), from a seeded random start."""
    b, keep = _basis(basis, accurate_boys)
    n = b.nbf
    r = _abi.UhfResult()
    out = dict(eps_up=np.empty(n), eps_down=np.empty(n), C_up=np.empty((n, n)), C_down=np.empty((n, n)))
    r.eps_up, r.eps_down, r.C_up, r.C_down = (_ptr(out[k]) for k in ("eps_up", "eps_down", "C_up", "C_down"))
    r.seed = seed
    _abi.check(_abi.lib().ccsd_uhf(C.byref(b), n_up, n_down, tol, max_iter, C.byref(r)))
    del keep
    out.update(e_uhf=r.e_uhf, e_nuc=r.e_nuc, iterations=r.iterations, converged=bool(r.converged))
    return out


def ccsd_inputs(scf: dict) -> dict:
    """fock / nocc / ao_eri / mo_coeff for :func:`solve` from an :func:`rhf` result."""
    return dict(fock=np.diag(scf["eps"]), nocc=scf["nocc"], ao_eri=scf["eri"], mo_coeff=scf["C"])


def _problem(fock, nocc, eri=None, df=None, ao_eri=None, mo_coeff=None, so_eri=None, nfrozen=0):
    """ccsd_problem over host arrays; returns (problem, arrays to keep alive).

    Integrals: ``eri`` spatial (pq|rs) [n]^4, ``df`` factors B[Q][p][q],
    ``ao_eri`` + ``mo_coeff``, or ``so_eri`` = <PQ||RS> over 2n interleaved
    spin orbitals (the reference's antisymmetrised integrals).  ``nocc`` counts
    the occupied orbitals of these arrays; ``nfrozen`` of them (the lowest) are
    frozen core, so the amplitudes cover nocc - nfrozen occupied orbitals."""
    fock = _f64(fock)
    n = fock.shape[0]
    p = _abi.Problem()
    p.nocc, p.nvir, p.nfrozen = nocc - nfrozen, n - nocc, nfrozen
    keep = [fock]
    p.fock = _ptr(fock)
    if df is not None:
        df = _f64(df)
        p.integral_kind, p.naux, p.df = CCSD_INTS_DF, df.shape[0], _ptr(df)
        keep.append(df)
    elif ao_eri is not None:
        ao_eri, mo_coeff = _f64(ao_eri), _f64(mo_coeff)
        p.integral_kind, p.nao = CCSD_INTS_AO_DENSE, ao_eri.shape[0]
        p.eri, p.mo_coeff = _ptr(ao_eri), _ptr(mo_coeff)
        keep += [ao_eri, mo_coeff]
    elif so_eri is not None:
        so_eri = _f64(so_eri)
        if so_eri.shape != (2 * n,) * 4:
            raise ValueError("so_eri must be (2n)^4 spin-orbital integrals <PQ||RS>")
        p.integral_kind, p.eri = CCSD_INTS_SO_ANTISYM, _ptr(so_eri)
        keep.append(so_eri)
    elif eri is not None:
        eri = _f64(eri)
        p.integral_kind, p.eri = CCSD_INTS_MO_DENSE, _ptr(eri)
        keep.append(eri)
    else:
        raise ValueError("one of eri / df / ao_eri / so_eri is required")
    return p, keep


class Solver:
    """One device-resident system (integrals uploaded/transformed once)."""

    def __init__(self, fock, nocc, eri=None, df=None, ao_eri=None, mo_coeff=None, so_eri=None, nfrozen=0, **opts):
        p, self._keep = _problem(fock, nocc, eri=eri, df=df, ao_eri=ao_eri, mo_coeff=mo_coeff, so_eri=so_eri,
                                 nfrozen=nfrozen)
        n = p.nfrozen + p.nocc + p.nvir
        self.nocc, self.nvir = p.nocc, p.nvir  # active orbitals (the amplitudes' shape)
        self._opts = _options(**self._restart(opts))
        h = C.c_void_p()
        _abi.check(_abi.lib().ccsd_create(C.byref(p), C.byref(self._opts), C.byref(h)))
        self._h = h
        self._problem = p  # re-read by lambda_grad (the arrays in _keep stay referenced)
        self._n = n

    def _restart(self, opts):
        """t1_start / t2_start (a restart) as contiguous FP64 arrays kept alive here.
        Their shapes are checked against this system's (o, v) and (o, o, v, v):
        the library copies exactly that many doubles from the pointers."""
        self._restart_keep = []
        o, v = self.nocc, self.nvir
        for k, shape in (("t1_start", (o, v)), ("t2_start", (o, o, v, v))):
            if opts.get(k) is not None:
                a = _f64(opts[k])
                if a.shape != shape:
                    raise CCSDError(_abi.CCSD_ERR_INVALID_ARG,
                                    f"{k} has shape {a.shape}; this system's amplitudes are {shape}")
                opts[k] = a
                self._restart_keep.append(a)
        return opts

    def set_options(self, **opts):
        self._opts = _options(**self._restart(opts))
        _abi.check(_abi.lib().ccsd_set_options(self._h, C.byref(self._opts)))

    def solve(self, amplitudes: bool = True, history: int = 1001) -> dict:
        o, v = self.nocc, self.nvir
        r = _abi.Result()
        t1 = np.empty((o, v)) if amplitudes else None
        t2 = np.empty((o, o, v, v)) if amplitudes else None
        eh = np.zeros(history)
        ms = np.zeros(history)
        r.t1, r.t2 = _ptr(t1), _ptr(t2)
        r.energy_history, r.update_ms, r.history_capacity = _ptr(eh), _ptr(ms), history
        _abi.check(_abi.lib().ccsd_solve(self._h, C.byref(r)))
        return dict(e_corr=r.e_corr, iterations=r.iterations, converged=bool(r.converged),
                    residual_norm=r.residual_norm, energies=eh[:r.history_len].copy(),
                    update_ms=ms[:r.iterations].copy(), flops_per_update=r.flops_per_update,
                    t1=t1, t2=t2)

    def lambda_grad(self, tol: float = 1e-10, max_iter: int = 500, lambdas: bool = False) -> dict:
        """Lambda equations at the last solve and dE_corr/d(inputs) (see ccsd_lambda_grad)."""
        o, v, n = self.nocc, self.nvir, self._n
        p = self._problem
        g = _abi.Grad()
        out = {"d_fock": np.zeros((n, n))}
        if p.integral_kind == CCSD_INTS_DF:
            out["d_df"] = np.zeros((p.naux, n, n))
        elif p.integral_kind == CCSD_INTS_AO_DENSE:
            out["d_eri"] = np.zeros((p.nao,) * 4)
            out["d_mo_coeff"] = np.zeros((p.nao, n))
        elif p.integral_kind == CCSD_INTS_SO_ANTISYM:
            out["d_eri"] = np.zeros((2 * n,) * 4)
        else:
            out["d_eri"] = np.zeros((n,) * 4)
        if lambdas:
            out["lambda1"] = np.zeros((o, v))
            out["lambda2"] = np.zeros((o, o, v, v))
        for k, arr in out.items():
            setattr(g, k, _ptr(arr))
        g.tol, g.max_iter = tol, max_iter
        _abi.check(_abi.lib().ccsd_lambda_grad(self._h, C.byref(p), C.byref(g)))
        out.update(iterations=g.iterations, residual_norm=g.residual_norm, e_corr=g.e_corr)
        return out

    def profile(self) -> dict:
        """Per-contraction device times of the last solve (needs profile=True)."""
        import json
        n = _abi.lib().ccsd_profile_report(self._h, None, 0)
        if n < 0:
            _abi.check(n)
        buf = C.create_string_buffer(n + 1)
        _abi.lib().ccsd_profile_report(self._h, buf, n + 1)
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None):
            _abi.lib().ccsd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def solve(fock, nocc, eri=None, df=None, ao_eri=None, mo_coeff=None, so_eri=None, amplitudes=True, nfrozen=0,
          **opts):
    with Solver(fock, nocc, eri=eri, df=df, ao_eri=ao_eri, mo_coeff=mo_coeff, so_eri=so_eri, nfrozen=nfrozen,
                **opts) as s:
        return s.solve(amplitudes=amplitudes)


class Batch:
    """Many systems of uneven nocc/nvir iterated together (ccsd_batch_*).

    ``systems`` is a sequence of dicts with the keyword arguments of
    :class:`Solver` (``fock``, ``nocc`` and one of ``eri`` / ``df`` /
    ``ao_eri`` + ``mo_coeff``).  Every operation of the amplitude update runs
    as one grouped launch over the batch, replayed from a CUDA graph."""

    def __init__(self, systems, **opts):
        probs, self._keep = [], []
        for sysd in systems:
            p, keep = _problem(**sysd)
            probs.append(p)
            self._keep += keep
        self._probs = probs
        self._arr = (C.POINTER(_abi.Problem) * len(probs))(*[C.pointer(p) for p in probs])
        self._opts = _options(**opts)
        h = C.c_void_p()
        _abi.check(_abi.lib().ccsd_batch_create(self._arr, len(probs), C.byref(self._opts), C.byref(h)))
        self._h = h

    def __len__(self):
        return len(self._probs)

    def solve(self, amplitudes: bool = True, history: int = 1001) -> list:
        res = (_abi.Result * len(self._probs))()
        bufs = []
        for r, p in zip(res, self._probs):
            o, v = p.nocc, p.nvir
            t1 = np.empty((o, v)) if amplitudes else None
            t2 = np.empty((o, o, v, v)) if amplitudes else None
            eh, ms = np.zeros(history), np.zeros(history)
            r.t1, r.t2 = _ptr(t1), _ptr(t2)
            r.energy_history, r.update_ms, r.history_capacity = _ptr(eh), _ptr(ms), history
            bufs.append((t1, t2, eh, ms))
        rc = _abi.lib().ccsd_batch_solve(self._h, res)
        out = []
        for r, (t1, t2, eh, ms) in zip(res, bufs):
            out.append(dict(e_corr=r.e_corr, iterations=r.iterations, converged=bool(r.converged),
                            residual_norm=r.residual_norm, energies=eh[:r.history_len].copy(),
                            update_ms=ms[:r.iterations].copy(), flops_per_update=r.flops_per_update,
                            t1=t1, t2=t2))
        if rc != 0:
            err = CCSDError(rc, _abi.last_error())
            err.results = out
            raise err
        return out

    def report(self) -> dict:
        """Grouped operations, tile plans, autotuning and launches per update."""
        import json
        n = _abi.lib().ccsd_batch_report(self._h, None, 0)
        if n < 0:
            _abi.check(n)
        buf = C.create_string_buffer(n + 1)
        _abi.lib().ccsd_batch_report(self._h, buf, n + 1)
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None):
            _abi.lib().ccsd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def solve_batched(systems, amplitudes=True, **opts) -> list:
    """Solve many systems in one batch; one result dict per system."""
    with Batch(systems, **opts) as b:
        return b.solve(amplitudes=amplitudes)


class CCSD_Memory_optimized:
    """Drop-in for the iterative part of the reference class.

    reference (ccsd_memory_optimized.h)        here
    ------------------------------------------------------------------
    CCSD_Memory_optimized(n_N, Z, R, basis,     CCSD_Memory_optimized(fock, nocc, eri=|df=|ao_eri=,
      n_Elec, rank, size, HartFock*, frozen)      mo_coeff=, E_HF=, nfrozen=) -- the integrals that
                                                  Prepear_AOs would build are passed in; frozen=true
                                                  is nfrozen=frozen_core_count(Z)
    double CCSD(double toler, bool print)      CCSD(toler, print_stuff) -> E_HF + E_corr
    E_new, T_1, t2                             E_new, t1 (o x v), t2 (o,o,v,v) over active orbitals
    n_Electrons, unocc_orb (spin orbitals)     n_Electrons = 2 (nocc - nfrozen), unocc_orb = 2 nvir
                                                  (the reference subtracts the frozen electrons,
                                                  ccsd_memory_optimized.cpp:3520)

    Like the reference, CCSD() runs plain Jacobi updates from the MP2 guess
    until |E_new - E_old| < toler or 999 updates (iter reaching 1000).  It
    iterates the reference class's own map by default (variant
    "memory_optimized": F_mi contracted transposed in T2,
    ccsd_memory_optimized.cpp:2085-2086), so energies and counters are the
    class's; variant="ccsd" iterates the CCSD equations of the reference's
    dense CCSD1 instead.
    """

    def __init__(self, fock, nocc, eri=None, df=None, ao_eri=None, mo_coeff=None, E_HF=0.0,
                 precision="fp64", so_eri=None, nfrozen=0, variant="memory_optimized"):
        self._variant = variant
        self._solver = Solver(fock, nocc, eri=eri, df=df, ao_eri=ao_eri, mo_coeff=mo_coeff, so_eri=so_eri,
                              precision=precision, nfrozen=nfrozen, variant=variant)
        self.n_Electrons = 2 * (nocc - nfrozen)
        self.unocc_orb = 2 * (np.asarray(fock).shape[0] - nocc)
        self.E_HF = E_HF
        self.E_new = 0.0
        self.t1 = self.t2 = None
        self.iter = 1

    def CCSD(self, toler: float, print_stuff: bool = False) -> float:
        self._solver.set_options(precision=self._solver._opts.precision, energy_tol=toler,
                                 max_iter=999, verbose=print_stuff, variant=self._variant)
        r = self._solver.solve()
        self.E_new, self.t1, self.t2 = r["e_corr"], r["t1"], r["t2"]
        self.iter = r["iterations"] + 1  # the reference counter starts at 1
        self.energies = r["energies"]
        if print_stuff:
            print(f"CCSD correction [au] = {self.E_new:.15e}")
        return self.E_new + self.E_HF
