/*
 * ccsd_gb300.h -- C ABI of the GB300 (sm_103a) CCSD amplitude engine.
 *
 * The engine is a drop-in for the iterative part of the reference class
 * CCSD_Memory_optimized (otnorli/CCSD_PARALLEL):
 *
 *   reference                                         this ABI
 *   ---------------------------------------------------------------------------
 *   CCSD_Memory_optimized::CCSD(double toler, bool)   ccsd_create + ccsd_solve
 *     (ccsd_memory_optimized.h:47, .cpp:16-567)
 *   Prepear_AOs (AO->MO, .cpp:2698-3522)              integral_kind AO_DENSE /
 *                                                     MO_DENSE / DF in ccsd_problem
 *   Fill_FS (diagonal spin-orbital Fock, .cpp:3560)   ccsd_problem.fock (spatial)
 *   MP2 guess + loop (.cpp:473-557)                   ccsd_solve
 *   t2 / T_1 / E_new (class members)                  ccsd_result.t2 / t1 / e_corr
 *   (no counterpart)                                  ccsd_lambda_grad, ccsd_solve_batched
 *
 * Conventions
 *   - Spatial closed-shell quantities.  nocc / nvir are spatial counts
 *     (reference: n_Electrons = 2*nocc, unocc_orb = 2*nvir).  Amplitudes are
 *     returned as t1[i][a] (nocc x nvir) and t2[i][j][a][b]; the spin-orbital
 *     amplitude of the reference is t(a alpha, b beta, i alpha, j beta) =
 *     t2[i][j][a][b] and the same-spin block is t2[i][j][a][b] - t2[j][i][a][b].
 *   - Integrals are real, chemist notation (pq|rs), 8-fold symmetric.
 *   - Every function returns CCSD_OK (0) or a negative error code; the text of
 *     the last error of the calling thread is available from ccsd_last_error.
 *     No C++ exception crosses this boundary.
 *   - The caller owns every host buffer.  A handle owns its device memory.
 *     One handle must not be used by two threads at once.
 *   - There is no CPU path: ccsd_create fails with CCSD_ERR_NO_DEVICE when no
 *     CUDA device is present.
 */
#ifndef CCSD_GB300_H
#define CCSD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define CCSD_OK 0
#define CCSD_ERR_INVALID_ARG (-1)
#define CCSD_ERR_CUDA (-2)
#define CCSD_ERR_OUT_OF_MEMORY (-3)
#define CCSD_ERR_DIVERGED (-4)      /* NaN/Inf in residual or energy        */
#define CCSD_ERR_NO_DEVICE (-5)
#define CCSD_ERR_TIMEOUT (-6)       /* a bounded device-side wait gave up   */
#define CCSD_ERR_UNSUPPORTED (-7)
#define CCSD_ERR_NOT_CONVERGED (-8) /* only from the C++ wrapper            */

/* ---- integral input forms -------------------------------------------- */
#define CCSD_INTS_MO_DENSE 0 /* eri = n^4 MO (pq|rs), row-major p,q,r,s         */
#define CCSD_INTS_DF 1       /* df  = naux*n*n factors B[Q][p][q], (pq|rs) = sum_Q B B */
#define CCSD_INTS_AO_DENSE 2 /* eri = nao^4 AO (mu nu|la si), mo_coeff = C[mu][p] */
/* eri = <PQ||RS> over N = 2n spin orbitals, physicist order, alpha/beta
 * interleaved (spin orbital P -> spatial P/2, spin P%2), the reference's
 * antisymmetrised spin-orbital integrals (ccsdt.cpp:1466-1478).  They must be
 * those of a closed-shell determinant; the engine reads the alpha-beta block,
 * (pq|rs) = <p_alpha r_beta || q_alpha s_beta>, and (host inputs) checks a
 * sample of same-spin elements against (pr|qs) - (ps|qr). */
#define CCSD_INTS_SO_ANTISYM 3

/* ---- contraction precision ------------------------------------------- */
#define CCSD_PREC_FP64 0      /* every contraction in FP64 (DFMA)              */
#define CCSD_PREC_SPLIT2 2    /* BF16 hi/lo slices, 3 tcgen05 products         */
#define CCSD_PREC_SPLIT3 3    /* 3 BF16 slices, 6 tcgen05 products             */
#define CCSD_PREC_SPLIT4 4    /* 4 BF16 slices, 10 tcgen05 products            */

typedef struct ccsd_problem {
    int32_t nocc;          /* spatial occupied orbitals (> 0)                  */
    int32_t nvir;          /* spatial virtual orbitals (> 0)                   */
    int32_t integral_kind; /* CCSD_INTS_*                                      */
    int32_t naux;          /* DF: number of auxiliary functions                */
    int32_t nao;           /* AO_DENSE: number of basis functions (>= n)       */
    int32_t device_inputs; /* 0: pointers below are host memory; 1: device     */
    const double *fock;    /* n x n MO Fock matrix, n = nocc + nvir            */
    const double *eri;     /* MO_DENSE: n^4; AO_DENSE: nao^4; SO_ANTISYM: (2n)^4 */
    const double *df;      /* DF: naux * n * n                                 */
    const double *mo_coeff;/* AO_DENSE: nao x n, row-major C[mu][p]            */
    int32_t nfrozen;       /* frozen core: the first nfrozen spatial orbitals of
                              the inputs stay doubly occupied and out of the
                              correlation treatment (the reference's Freeze_Core,
                              Prepear_AOs(nr_freeze), ccsd_memory_optimized.cpp:
                              2698-2709, 3520-3521).  The arrays above then cover
                              n = nfrozen + nocc + nvir orbitals; nocc counts the
                              active occupied ones.  0 = all electrons.          */
} ccsd_problem;

typedef struct ccsd_options {
    double energy_tol;         /* stop when |E_new - E_old| < energy_tol
                                  (ccsd_memory_optimized.cpp:552)             */
    double residual_tol;       /* also require ||T_new - T_old||_2 < this; 0 = off */
    int32_t max_iter;          /* cap on amplitude updates (reference: 999)    */
    int32_t fixed_iterations;  /* > 0: run exactly this many updates           */
    int32_t diis_size;         /* 0 = plain Jacobi (reference); else vectors kept */
    int32_t diis_start;        /* first update index that extrapolates         */
    int32_t precision;         /* CCSD_PREC_*                                   */
    int32_t verbose;           /* print one line per update to stdout          */
    int32_t profile;           /* 1: time every contraction with CUDA events   */
    int32_t method;            /* CCSD_METHOD_*                                 */
    void *stream;              /* cudaStream_t, or NULL for a private stream   */
    const double *t1_start;    /* restart: ccsd_solve starts from these host   */
    const double *t2_start;    /*   amplitudes ([i][a], [i][j][a][b]) instead of
                                    T1 = 0, T2 = MP2 when t2_start is set (t1_start
                                    NULL: T1 = 0); t1_start without t2_start is
                                    rejected (CCSD_ERR_INVALID_ARG); single solves
                                    only; the DIIS history and T3 start afresh.  A
                                    checkpoint is ccsd_result.t1 / t2 of an earlier
                                    solve.                                       */
    int32_t variant;           /* CCSD_VARIANT_*: which of the reference's two
                                  CCSD maps is iterated (method CCSD only)      */
} ccsd_options;

/* ---- CCSD map (ccsd_options.variant) --------------------------------------
 * The reference holds two CCSD codes that iterate different maps.
 * CCSD_VARIANT_CCSD is the CCSD equations as its dense spin-orbital CCSD
 * ("CCSD1", CCSDT::Calc_Energy(toler, -1), ccsdt.cpp:625-727) states them:
 *   R_ij^ab += sum_k t_jk^ab F_ki - sum_k t_ik^ab F_kj.
 * CCSD_VARIANT_MEMORY_OPTIMIZED is CCSD_Memory_optimized::CCSD as written (the
 * INCAR method "CCSD", initializer.cpp:191-195): its Fill_t2_new contracts the
 * occupied Fock intermediate transposed, in every spin case,
 *   R_ij^ab += sum_k t_jk^ab F_ik - sum_k t_ik^ab F_jk
 * (D2.row(i/2), ccsd_memory_optimized.cpp:2085-2086, 2143-2144, 2193-2194,
 * 2269-2270, 2324-2325, 2375-2376, where D2(k,i) = F_ki), while its T1 equation
 * uses F_ki (:2444).  F_ki is not symmetric once T1/T2 are non-zero, so the
 * two maps reach fixed points ~1e-8 Eh apart on molecules (H2O/6-31G:
 * 1.9e-8).  The default is CCSD_VARIANT_CCSD. */
#define CCSD_VARIANT_CCSD 0
#define CCSD_VARIANT_MEMORY_OPTIMIZED 1

/* ---- coupled-cluster method (ccsd_options.method) ------------------------ */
#define CCSD_METHOD_CCSD 0     /* CCSD (the reference's CCSD / CCSD1)            */
/* CCSDT-1a, the reference's CCSDT::Calc_Energy(toler, 1) (initializer.cpp:104-108):
 * T3 from T2 and the bare integrals, T3 terms in T1/T2 (ccsdt.cpp:419-434,
 * 640-670, 995-1290), iterated with T1/T2 (Jacobi; DIIS, when set, acts on T1/T2).
 * T3 is kept in the reference's spin-orbital form, 3 (2 nocc)^3 (2 nvir)^3
 * doubles of device memory with its two contraction intermediates.  Single
 * systems only (no batched solve, no ccsd_lambda_grad). */
#define CCSD_METHOD_CCSDT1A 1
/* CCSDT-1b, CCSDT::Calc_Energy(toler, 2) (initializer.cpp:110-114): CCSDT-1a plus
 * the T3 T1 term of T2 (ccsdt.cpp:676-700).  Same memory and restrictions. */
#define CCSD_METHOD_CCSDT1B 2
/* CCSDT-2, CCSDT::Calc_Energy(toler, 3) (initializer.cpp:116-120): CCSDT-1b with
 * T2-dressed X1/X2 and the X12/X13 terms of T3 (ccsdt.cpp:1078-1130, 1960-2040,
 * 2301-2390).  Two more V^3 O^3 arrays (5 in all); same restrictions. */
#define CCSD_METHOD_CCSDT2 3
/* CCSDT-3, CCSDT::Calc_Energy(toler, 4) (initializer.cpp:122-126): CCSDT-2 with T1
 * terms in X12/X13 and the X14/X15 terms of T3 (ccsdt.cpp:1028-1070, 2043-2125,
 * 2321-2383).  Also keeps the spin-orbital <ab||cd> block ((2 nvir)^4 doubles);
 * the method must be set at ccsd_create. */
#define CCSD_METHOD_CCSDT3 4
/* CCSDT-4, CCSDT::Calc_Energy(toler, 5) (initializer.cpp:128-132): CCSDT-3 with the
 * X3/X4/X6 terms of the previous T3 in T3 (ccsdt.cpp:1134-1180); same memory as CCSDT-3. */
#define CCSD_METHOD_CCSDT4 5
/* CCSDT, CCSDT::Calc_Energy(toler, 6) (initializer.cpp:93-96): CCSDT-4 with T3 terms in
 * X1/X2, dressed X3/X4/X6 and the X7/X8 terms (ccsdt.cpp:1183-1200, 1960-2040,
 * 2128-2300), following the reference's X3 as written (its tau loop over (d,e),
 * ccsdt.cpp:2199-2206, visits e = the first virtual only). That loop breaks the
 * alpha/beta symmetry of the reference's iterates; the closed-shell t2 keeps one
 * amplitude per pair t2[ij][ab] = t2[ji][ba], the mean of the two, and the energies
 * stay within 1e-8 of the reference's with the same iteration counts. Same memory
 * as CCSDT-3. */
#define CCSD_METHOD_CCSDT 6

typedef struct ccsd_result {
    double e_corr;             /* correlation energy (E_new of the reference)  */
    double residual_norm;      /* ||T_new - T_old||_2 of the last update       */
    int32_t iterations;        /* amplitude updates performed                  */
    int32_t converged;         /* 1 when the stopping rule was met             */
    double *t1;                /* optional out: nocc*nvir host doubles         */
    double *t2;                /* optional out: nocc^2*nvir^2 host doubles     */
    double *energy_history;    /* optional out: E after 0..iterations updates  */
    double *update_ms;         /* optional out: device ms of each update       */
    int32_t history_capacity;  /* length of energy_history / update_ms         */
    int32_t history_len;       /* entries written                              */
    double flops_per_update;   /* algorithmic FLOP of one update (fixed count) */
} ccsd_result;

/* Output of ccsd_lambda_grad.  Every array is optional (NULL = not wanted)
 * and caller-owned host memory.  Derivatives are taken with respect to each
 * element of the input arrays as given to ccsd_create, each element treated
 * as independent (an element the engine never reads has derivative 0). */
typedef struct ccsd_grad {
    double *d_fock;      /* n x n: dE_corr / d fock[p][q]                         */
    double *d_eri;       /* MO_DENSE: n^4, AO_DENSE: nao^4, SO_ANTISYM: (2n)^4   */
    double *d_df;        /* DF: naux*n*n: dE_corr / d B[Q][p][q]                  */
    double *d_mo_coeff;  /* AO_DENSE: nao*n: dE_corr / d C[mu][p]                 */
    double *lambda1;     /* o*v: Lambda amplitudes l1[i][a]                       */
    double *lambda2;     /* o^2 v^2: l2[i][j][a][b]                               */
    double tol;          /* in: stop when ||l_new - l||_2 < tol (0: 1e-10)        */
    int32_t max_iter;    /* in: cap on Lambda updates (0: 500)                    */
    int32_t iterations;  /* out: Lambda updates performed                         */
    double residual_norm;/* out: ||l_new - l||_2 of the last update               */
    double e_corr;       /* out: E_corr of the solution the gradient belongs to   */
} ccsd_grad;

typedef struct ccsd_handle ccsd_handle;

/* Defaults: energy_tol 1e-10, max_iter 999, FP64, no DIIS (reference rules). */
int ccsd_default_options(ccsd_options *opts);

/* Upload/transform the integrals and allocate the amplitude engine.
 * Replaces the set-up half of CCSD_Memory_optimized::CCSD
 * (ccsd_memory_optimized.cpp:49-466: AO->MO, Fill_FS, denominators). */
int ccsd_create(const ccsd_problem *problem, const ccsd_options *opts, ccsd_handle **out);

/* Run the amplitude iteration from the MP2 guess (T1 = 0) and fill `res`.
 * Replaces ccsd_memory_optimized.cpp:473-566 (MP2 guess, loop, E_new). */
int ccsd_solve(ccsd_handle *h, ccsd_result *res);

/* Backward pass of a converged ccsd_solve: solves the CCSD Lambda (adjoint)
 * equations  Lambda = (dE/dT + J^T Lambda) / D  with the same contraction
 * kernels, transposed, and returns dE_corr/d(fock) and dE_corr/d(integrals):
 * the one- and two-particle response densities of the correlation energy in
 * the input representation.  `problem` must be the problem the handle was
 * created with (its arrays are read again).  No counterpart in the reference,
 * which has no Lambda equations or gradients. */
int ccsd_lambda_grad(ccsd_handle *h, const ccsd_problem *problem, ccsd_grad *grad);

/* Change options (precision, tolerances, DIIS, stream) between solves. */
int ccsd_set_options(ccsd_handle *h, const ccsd_options *opts);

int ccsd_destroy(ccsd_handle *h);

/* ---- batched solve: many systems of uneven nocc/nvir iterated together ----
 * No counterpart in the reference, which solves one molecule per process.
 * Every operation of the amplitude update runs as one grouped launch over all
 * systems of the batch (contractions on a persistent grouped FP64 kernel
 * whose tile shape and split-K are chosen per operation by timing candidates
 * on the batch's own shapes), and the update is replayed from a captured CUDA
 * graph.  Each system follows exactly the single-system rules of ccsd_solve
 * (MP2 start, its own |dE| stop, cap, DIIS); a stopped system is masked off
 * on the device and keeps its last iterate.  In split precision the larger
 * contractions run as grouped tcgen05 launches over packed split operands;
 * in FP64 on a persistent grouped DFMA kernel.
 * results[i] is filled like ccsd_solve's result (caller-provided t1/t2/
 * history arrays per system).  When a system diverges, every result is still
 * filled and the call returns CCSD_ERR_DIVERGED naming the first such system. */
typedef struct ccsd_batch ccsd_batch;
int ccsd_batch_create(const ccsd_problem *const *problems, int32_t n, const ccsd_options *opts,
                      ccsd_batch **out);
int ccsd_batch_solve(ccsd_batch *b, ccsd_result *results);
/* JSON: grouped operations with their tile plans, autotuning times and the
 * kernel launches of one update.  Returns the report length. */
int ccsd_batch_report(ccsd_batch *b, char *buf, size_t len);
int ccsd_batch_destroy(ccsd_batch *b);
/* create + solve + destroy. */
int ccsd_solve_batched(const ccsd_problem *const *problems, int32_t n, const ccsd_options *opts,
                       ccsd_result *results);

/* JSON report of the last solve when options.profile was set: per
 * contraction site the calls, device ms of the contraction kernel, device ms
 * of the operand splitting (split modes), algorithmic FLOP and the path that
 * ran.  Times come from CUDA events recorded on the engine's stream.  The
 * reference only prints clock() CPU time per iteration
 * (ccsd_memory_optimized.cpp:515,542-548).  Returns the report length. */
int ccsd_profile_report(ccsd_handle *h, char *buf, size_t len);

/* Copy the calling thread's last error message; returns its length. */
int ccsd_last_error(char *buf, size_t len);

/* Algorithmic FLOP of one update: 2 o^2 v^4 + 4 o^4 v^2 + 8 o^3 v^3. */
double ccsd_flops_per_update(int32_t nocc, int32_t nvir);

/* Frozen core orbitals for ccsd_problem.nfrozen by the reference's rule
 * (CCSD_Memory_optimized::Freeze_How_Meny_Orbitals, ccsd_memory_optimized.cpp:
 * 5203-5231): one spatial orbital per atom with 2 < Z < 11 (Li-Ne), none for H
 * and He or beyond Ne.  The reference's loop runs over the electrons and reads
 * the nuclear charge Z(i) at the electron index; this counts per atom, as its
 * comments state.  Z holds the n_atoms nuclear charges (the reference's vec Z).
 * Returns the count, or CCSD_ERR_INVALID_ARG for n_atoms < 0 or a NULL Z. */
int ccsd_frozen_core_count(const double *Z, int32_t n_atoms);

/* ---- Gaussian integrals (the producer of the CCSD inputs) -------------- */
/* A contracted Cartesian Gaussian basis as the reference's integral engine
 * receives it (Hartree_Integrals::Set_Input, hartree_integrals.cpp:8-21): per
 * basis function its atom, Cartesian powers (l, m, n), primitive count,
 * exponents and contraction coefficients normalised as Normalize_small_c
 * leaves them (hartree_fock_solver.cpp:236-462).  Host arrays. */
typedef struct ccsd_basis {
    int32_t natoms;
    int32_t nbf;
    int32_t maxprim;        /* row length of alpha / coef                       */
    int32_t flags;          /* CCSD_BASIS_* bits; 0 = the reference's arithmetic */
    const double *Z;        /* [natoms] nuclear charges                        */
    const double *R;        /* [natoms][3] positions (bohr)                    */
    const int32_t *atom;    /* [nbf] atom of each basis function               */
    const int32_t *powers;  /* [nbf][3] Cartesian powers, l + m + n <= 3        */
    const int32_t *nprim;   /* [nbf] primitives (<= maxprim)                   */
    const double *alpha;    /* [nbf][maxprim] exponents                        */
    const double *coef;     /* [nbf][maxprim] normalised coefficients          */
} ccsd_basis;

/* The reference's Boys function takes x > 50 from an asymptotic form of F_30
 * (hartree_integrals.cpp:656-666) that is off by up to 1.2e-3 (relative) for
 * 50 < x < 80 and gives 0 above x = 1.1e5 (x^61 overflows); by default the
 * engine reproduces it, so its integrals equal the reference's.  This flag takes
 * x > 50 from F_0 = sqrt(pi/x)/2 instead, accurate to e^{-x}. */
#define CCSD_BASIS_ACCURATE_BOYS 1

/* Overlap, kinetic, nuclear-attraction and electron-repulsion integrals on the
 * GPU (McMurchie-Davidson, FP64), replacing Hartree_Integrals::Overlap_Matrix,
 * Kinetic_Energy, Nuclei_Electron_Interaction, Nuclei_Nuclei_Interaction
 * (hartree_integrals.cpp:293-718) and the (mu nu|la si) loop of
 * Hartree_Fock_Solver::get_Energy (hartree_fock_solver.cpp:714-817):
 *   S[mu][nu], T = -1/2 <mu|nabla^2|nu> (the reference's Kinetic_Energy is the
 *   nabla^2 matrix), V = -sum_C Z_C <mu|1/r_C|nu> (its Nuclei_Electron_Interaction
 *   is + the sum), so T + V is its EK; eri = (mu nu|la si), nbf^4 row-major;
 *   e_nuc = sum_{A<B} Z_A Z_B / R_AB.
 * Each output is optional (NULL).  device_outputs = 1: S/T/V/eri are device
 * pointers (e_nuc stays host).  stream may be NULL.  Returns after the work is
 * done.  CCSD_ERR_UNSUPPORTED above f functions. */
int ccsd_ao_integrals(const ccsd_basis *basis, double *S, double *T, double *V, double *eri, double *e_nuc,
                      int32_t device_outputs, void *stream);

typedef struct ccsd_scf_result {
    double e_hf;            /* out: E_HF with E_nuc (what get_Energy returns)   */
    double e_nuc;           /* out: nuclear repulsion                           */
    int32_t iterations;     /* out: SCF steps (the reference's steppp)          */
    int32_t converged;      /* out: 1 when the stopping rule was met            */
    double *eps;            /* optional out: nbf orbital energies, ascending    */
    double *C;              /* optional out: nbf x nbf MO coefficients C[mu][p] */
    double *eri;            /* optional out: nbf^4 AO integrals (mu nu|la si)   */
    void *stream;           /* in: cudaStream_t, or NULL                        */
} ccsd_scf_result;

/* Closed-shell Hartree-Fock on the GPU integrals, step for step as
 * Hartree_Fock_Solver::get_Energy(toler, 0) (hartree_fock_solver.cpp:578-1229):
 * canonical orthogonalisation, zero-density start, DIIS over 3 Fock matrices,
 * stop when the sum of occupied orbital energies moves by less than tol
 * (0: 1e-10) or after max_iter (0: the reference's 300) steps.  J and K are
 * contractions over the device-resident ERI tensor; the n x n algebra runs on
 * the host in FP64.  Its eps, C and eri are the CCSD inputs (ccsd_problem with
 * CCSD_INTS_AO_DENSE and fock = diag(eps)). */
int ccsd_rhf(const ccsd_basis *basis, int32_t n_electrons, double tol, int32_t max_iter, ccsd_scf_result *res);

typedef struct ccsd_uhf_result {
    double e_uhf;           /* out: E_UHF with E_nuc                           */
    double e_nuc;           /* out                                             */
    int32_t iterations;     /* out: SCF steps                                  */
    int32_t converged;      /* out                                             */
    double *eps_up, *eps_down;  /* optional out: nbf orbital energies each     */
    double *C_up, *C_down;      /* optional out: nbf x nbf, C[mu][p]           */
    uint64_t seed;          /* in: seed of the random start (0: 2024)          */
    void *stream;           /* in: cudaStream_t, or NULL                       */
} ccsd_uhf_result;

/* Unrestricted Hartree-Fock with n_up / n_down electrons, step for step as
 * get_Energy(toler, 1) (hartree_fock_solver.cpp:959-1025): F_up = h + J(P_up +
 * P_down) - K(P_up), F_down likewise, no DIIS, stop when the lowest orbital energy
 * of each spin moves by less than tol in sum (0: 1e-10) or after max_iter (0: 300)
 * steps, the reference's energy expression.  The reference starts from random
 * densities (Armadillo randn, Initialize_UHF); this starts from a seeded generator,
 * so a run is repeatable and, like the reference, can reach a lower state than a
 * core-Hamiltonian start. */
int ccsd_uhf(const ccsd_basis *basis, int32_t n_up, int32_t n_down, double tol, int32_t max_iter,
             ccsd_uhf_result *res);

/* ---- INCAR front end (main.cpp:83-298, initializer.cpp:17-210) ----------- */
/* The reference's INCAR keywords (Basis_Set, Method, convergance_criteria as
 * log10, Freeze_Core, Relax_Pos, use_angstrom, print_stuffies) and its atom
 * lines "<element> x y z" (optionally between "#ATOMS START" and a '#' line),
 * read line by line: a keyword counts only at the start of a line, a missing
 * Method or an empty atom list is CCSD_ERR_INVALID_ARG, blanks of any length
 * separate values.  The basis is Gaussian94 text (S, P, D, F, SP shells per
 * element), expanded to Cartesian functions in the reference's order with its
 * primitive normalisation; the reference's own basis tables are not included. */
typedef struct ccsd_incar {
    char basis_set[64];            /* out: the Basis_Set value (a name only)      */
    char method[32];               /* out: the Method value                       */
    double convergance_criteria;   /* out: 10^value (default 1e-8)                */
    int32_t freeze_core, relax_pos, use_angstrom, print_stuffies;  /* out: flags */
    int32_t natoms, nbf, maxprim;  /* out: sizes                                  */
    int32_t n_electrons;           /* out: sum of the nuclear charges             */
    int32_t nfrozen;               /* out: ccsd_frozen_core_count when Freeze_Core */
    int32_t capacity_atoms;        /* in: rows of Z / R (0: sizes only)           */
    int32_t capacity_bf;           /* in: rows of atom / powers / nprim / alpha / coef */
    int32_t capacity_prim;         /* in: row length of alpha / coef              */
    double *Z, *R;                 /* out: [natoms], [natoms][3] in bohr          */
    int32_t *atom, *powers, *nprim;/* out: the ccsd_basis arrays                  */
    double *alpha, *coef;          /* out: [nbf][capacity_prim]                   */
} ccsd_incar;

/* Parse only (no GPU): call once with capacities 0 for the sizes, then with arrays.
 * basis_text NULL or empty: the basis file named by an INCAR line "Basis_File <path>"
 * (this engine's keyword; the reference selects built-in tables by Basis_Set). */
int ccsd_incar_parse(const char *incar_text, const char *basis_text, ccsd_incar *inc);

typedef struct ccsd_incar_result {
    double energy;          /* what Initializer::Go returns: E_HF (HF) or E_HF + E_corr */
    double e_hf, e_corr;
    int32_t scf_iterations; /* SCF steps                                           */
    int32_t cc_iter;        /* the reference's counter (updates + 1); 0 for HF     */
    int32_t method;         /* CCSD_METHOD_* that ran; -1 for HF, -2 for UHF       */
    int32_t nbf;
} ccsd_incar_result;

/* Initializer::Go on the engine: the molecule and method of incar_text with the
 * basis of basis_text, n_electrons = sum Z, the SCF and the amplitudes both to
 * convergance_criteria; HF, UHF (odd: n/2 + 1 up, n/2 down; even: the singlet, then
 * the triplet n/2 + 1, n/2 - 1, whose energy is returned, as Go does), CCSD / CCSD1
 * (one engine), CCSDT-1a ... CCSDT; Freeze_Core freezes ccsd_frozen_core_count(Z)
 * orbitals; UCCSDT and CCSDT--Q (not working in the reference) are
 * CCSD_ERR_UNSUPPORTED.  precision: CCSD_PREC_* of the amplitudes. */
int ccsd_incar_run(const char *incar_text, const char *basis_text, int32_t precision, ccsd_incar_result *res);

/* One contraction on the engine's kernels, for row-major FP64 device matrices:
 *   C[M][N] = alpha * A[M][K] * B[N][K]^T + beta * C     (leading dims lda/ldb/ldc)
 * precision CCSD_PREC_FP64 runs the DFMA kernel, CCSD_PREC_SPLIT* the
 * tcgen05 split-precision kernel.  It replaces the element-wise dot products
 * accu(A % B) through which the reference forms every contraction (e.g. the
 * particle-particle ladder, ccsd_memory_optimized.cpp:2093).  stream may be
 * NULL (legacy default stream); the call returns after the work completes.
 * Allocates its temporaries with cudaMalloc. */
int ccsd_gemm(int32_t precision, int32_t M, int32_t N, int32_t K, double alpha, const double *A,
              int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
              void *stream);

/* ccsd_gemm without any device allocation, for callers that may not call
 * cudaMalloc/cudaFree: a process whose device memory belongs to another
 * allocator with a fixed budget (a framework's caching allocator, a serving
 * runtime that reserves all of HBM up front), or code in the middle of a
 * pipelined stream that cannot take the device-wide synchronisation of
 * cudaFree.  No counterpart in the reference.
 *   - precision must be CCSD_PREC_SPLIT2/3/4 (the tensor-core kernel); the
 *     result equals ccsd_gemm's within the split kernel's error bound.
 *   - Scratch (BF16 planes, row scales, split-K partials, error word) lives in
 *     one static device array of 64 MiB that every GPU loading the library
 *     holds until exit.  Shapes whose scratch exceeds it are rejected with
 *     CCSD_ERR_INVALID_ARG and a message giving the bytes needed; roughly
 *     S * (M + N) * K * 2 bytes must stay below 64 MiB.
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.
 *   - All calls share the array: calls whose work overlaps on the GPU (other
 *     streams or threads on the same device) race; serialise them.
 *   - Returns after the work completes (it synchronises `stream`). */
int ccsd_gemm_noalloc(int32_t precision, int32_t M, int32_t N, int32_t K, double alpha,
                      const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                      double *C, int64_t ldc, void *stream);

/* Failure injection for tests; no counterpart in the reference, whose only
 * failure handling is its 1000-iteration cap (ccsd_memory_optimized.cpp:42,553).
 * While stall_ns > 0, the MMA thread of every split-precision contraction
 * launched afterwards on the current device first waits on an mbarrier that
 * nothing arrives at, for at most stall_ns nanoseconds.  The wait gives up and
 * the kernel leaves through the path of a real device-side stall: the error
 * word is set, the other roles stop, in-flight TMA loads are awaited and TMEM
 * is freed, so the context stays usable.  ccsd_gemm and ccsd_solve then return
 * CCSD_ERR_TIMEOUT.  ccsd_debug_stall_split_mma(0) restores normal operation;
 * a later ccsd_solve on the same handle starts with a clean error word. */
int ccsd_debug_stall_split_mma(uint64_t stall_ns);

/* Inner product of the plain-FP64 tiled contraction kernel, process-wide (a
 * tuning switch with no reference counterpart; the reference's FP64 products are
 * Armadillo element loops, e.g. accu(integ3_2D % tau3), ccsd_memory_optimized.cpp:2093).
 *   CCSD_FP64_DFMA  fused multiply-adds on the CUDA cores (default)
 *   CCSD_FP64_DMMA  mma.sync m8n8k4 on the FP64 tensor pipe
 * Both sum each output's K products in a different order, so results agree to
 * rounding, not bit for bit.  Returns the previous kind, or CCSD_ERR_INVALID_ARG. */
#define CCSD_FP64_DFMA 0
#define CCSD_FP64_DMMA 1
int ccsd_set_fp64_kernel(int32_t kind);

/* Seeded synthetic closed-shell system (host only, no GPU needed): diagonal
 * fock (n x n) with occupied U[-2,-0.3] / virtual U[0.1,3] energies, and
 * DF factors B[Q][p][q] = 0.05 z / sqrt(naux), z ~ N(0,1), symmetric in p,q.
 * Either output pointer may be NULL. */
int ccsd_make_synthetic(int32_t nocc, int32_t nvir, int32_t naux, uint64_t seed,
                        double *fock, double *df);

#ifdef __cplusplus
}
#endif
#endif /* CCSD_GB300_H */
