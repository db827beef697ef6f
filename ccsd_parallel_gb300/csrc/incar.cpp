// INCAR front end: the reference's input reader (main.cpp:83-298: find_and_write,
// find_start_of_atoms, Fill_One_Atom, return_charge) and Initializer::Go's dispatch
// (initializer.cpp:17-210) onto the engine: HF -> ccsd_rhf; UHF -> ccsd_uhf; CCSD ->
// RHF + ccsd_solve of the memory-optimised map (the reference's "CCSD" runs the class
// CCSD_Memory_optimized, initializer.cpp:191-195); CCSD1 -> RHF + ccsd_solve of the
// CCSD equations (the reference's dense CCSDT::Calc_Energy(toler, -1)); CCSDT-1a ...
// CCSDT -> RHF + the triples methods.
//
// Differences from the reference's reader (its parsing hazards):
//   - a keyword counts only at the start of a line (the reference takes the first
//     strstr match anywhere, e.g. inside a comment or another keyword's value);
//   - a missing keyword is an error or takes a stated default (the reference
//     dereferences NULL); values end at the end of their line, with no overrun;
//   - atom lines are split on any run of blanks (the reference needs single spaces);
//     the "#ATOMS START" marker is optional (the reference's INCAR~ sample lacks it),
//     the block ends at a line starting with '#' or at the end of the file;
//   - the basis comes from text in the Gaussian94 format (the reference's tables in
//     fill_alpha*.cpp are its own data); each shell becomes Cartesian functions in the
//     reference's component order with its primitive normalisation
//     N = (2a/pi)^{3/4} (4a)^{L/2} / sqrt((2l-1)!! (2m-1)!! (2n-1)!!)
//     (Normalize_small_c, hartree_fock_solver.cpp:236-462); SP shells give S then P.
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ccsd_gb300.h"
#include "common.h"

namespace ccsd {
void set_last_error(const std::string &msg);

namespace {

const char *const kElements[] = {"H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg",
                                 "Al", "Si", "P",  "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr",
                                 "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"};
constexpr int kNElements = sizeof(kElements) / sizeof(kElements[0]);
constexpr double kBohrPerAngstrom = 1.889725989;  // Initializer::Go (initializer.cpp:55-58)

int element_charge(const std::string &s) {
    for (int i = 0; i < kNElements; ++i)
        if (s == kElements[i]) return i + 1;
    return 0;
}

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

std::vector<std::string> split(const std::string &s) {
    std::istringstream is(s);
    std::vector<std::string> out;
    std::string t;
    while (is >> t) out.push_back(t);
    return out;
}

bool parse_double(std::string t, double &x) {
    for (char &c : t)
        if (c == 'D' || c == 'd') c = 'E';  // Fortran exponents in basis files
    char *end = nullptr;
    x = std::strtod(t.c_str(), &end);
    return end && *end == '\0' && !t.empty();
}

struct Shell {
    int L;
    std::vector<double> exps, coefs;
};
using Library = std::map<int, std::vector<Shell>>;  // nuclear charge -> shells

Library parse_g94(const std::string &text) {
    Library lib;
    std::istringstream is(text);
    std::string line;
    int Z = 0;
    int lineno = 0;
    auto fail = [&](const std::string &m) {
        throw Error(CCSD_ERR_INVALID_ARG, "basis text, line " + std::to_string(lineno) + ": " + m);
    };
    while (std::getline(is, line)) {
        ++lineno;
        const std::string t = trim(line);
        if (t.empty() || t[0] == '!' || t[0] == '#') continue;
        if (t.rfind("****", 0) == 0) {
            Z = 0;
            continue;
        }
        const std::vector<std::string> tok = split(t);
        if (Z == 0) {  // element header "<symbol> 0"
            Z = element_charge(tok[0]);
            if (!Z) fail("unknown element '" + tok[0] + "'");
            lib[Z].clear();
            continue;
        }
        if (tok.size() < 2) fail("expected '<shell type> <primitives> [scale]'");
        std::string type = tok[0];
        for (char &c : type) c = (char)std::toupper((unsigned char)c);
        const int np = std::atoi(tok[1].c_str());
        if (np <= 0) fail("bad primitive count");
        std::vector<int> Ls;
        if (type == "S") Ls = {0};
        else if (type == "P") Ls = {1};
        else if (type == "D") Ls = {2};
        else if (type == "F") Ls = {3};
        else if (type == "SP" || type == "L") Ls = {0, 1};
        else fail("shell type '" + type + "' (S, P, D, F, SP)");
        std::vector<Shell> sh(Ls.size());
        for (size_t k = 0; k < Ls.size(); ++k) sh[k].L = Ls[k];
        for (int p = 0; p < np; ++p) {
            if (!std::getline(is, line)) fail("missing primitive lines");
            ++lineno;
            const std::vector<std::string> v = split(line);
            if (v.size() < 1 + Ls.size()) fail("expected an exponent and " + std::to_string(Ls.size()) + " coefficient(s)");
            double e;
            if (!parse_double(v[0], e) || e <= 0.0) fail("bad exponent");
            for (size_t k = 0; k < Ls.size(); ++k) {
                double c;
                if (!parse_double(v[1 + k], c)) fail("bad coefficient");
                sh[k].exps.push_back(e);
                sh[k].coefs.push_back(c);
            }
        }
        for (Shell &s : sh) lib[Z].push_back(s);
    }
    return lib;
}

struct Input {
    std::map<std::string, std::string> kw;
    std::vector<double> Z, R;
};

Input parse_incar(const std::string &text) {
    static const char *const keys[] = {"Basis_Set", "Method", "convergance_criteria", "Freeze_Core",
                                       "Relax_Pos", "use_angstrom", "print_stuffies", "Basis_File"};
    Input in;
    std::istringstream is(text);
    std::string line;
    bool in_atoms = false, atoms_done = false;
    int lineno = 0;
    while (std::getline(is, line)) {
        ++lineno;
        const std::string t = trim(line);
        if (t.empty()) continue;
        if (t[0] == '#') {
            if (t.rfind("#ATOMS START", 0) == 0 && !atoms_done) in_atoms = true;
            else if (in_atoms) {
                in_atoms = false;
                atoms_done = true;
            }
            continue;
        }
        const std::vector<std::string> tok = split(t);
        bool is_key = false;
        for (const char *k : keys)
            if (tok[0] == k) {
                in.kw[k] = trim(t.substr(tok[0].size()));
                is_key = true;
            }
        if (is_key) continue;
        // an atom line: symbol x y z (inside the block, or anywhere when there is no marker)
        double x, y, z;
        if (!atoms_done && tok.size() >= 4 && element_charge(tok[0]) && parse_double(tok[1], x) &&
            parse_double(tok[2], y) && parse_double(tok[3], z)) {
            in.Z.push_back(element_charge(tok[0]));
            in.R.insert(in.R.end(), {x, y, z});
            continue;
        }
        if (in_atoms)
            throw Error(CCSD_ERR_INVALID_ARG, "INCAR line " + std::to_string(lineno) + ": expected '<element> x y z'");
        // anything else (comments, unknown keywords) is left alone, as the reference does
    }
    return in;
}

std::vector<std::array<int, 3>> components(int L) {
    switch (L) {
    case 0: return {{0, 0, 0}};
    case 1: return {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    case 2: return {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}};
    default:
        return {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1},
                {1, 2, 0}, {0, 2, 1}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1}};
    }
}

double odd_factorial(int k) {  // (2k - 1)!!
    double r = 1.0;
    for (int x = 2 * k - 1; x > 1; x -= 2) r *= x;
    return r;
}

struct Parsed {
    std::string basis_set, method;
    double tol = 1e-8;
    bool freeze = false, relax = false, angstrom = false, print = false;
    std::vector<double> Z, R;
    std::vector<int32_t> atom, powers, nprim;
    std::vector<double> alpha, coef;  // [nbf][maxprim]
    int maxprim = 0;
};

bool flag(const std::map<std::string, std::string> &kw, const char *k) {
    auto it = kw.find(k);
    return it != kw.end() && it->second.rfind("true", 0) == 0;  // as the reference: strncmp(.., "true", 4)
}

Parsed parse_all(const char *incar_text, const char *basis_text) {
    if (!incar_text) throw Error(CCSD_ERR_INVALID_ARG, "INCAR text is NULL");
    const Input in = parse_incar(incar_text);
    Parsed p;
    auto get = [&](const char *k) -> const std::string * {
        auto it = in.kw.find(k);
        return it == in.kw.end() ? nullptr : &it->second;
    };
    if (!get("Method")) throw Error(CCSD_ERR_INVALID_ARG, "INCAR: no Method line");
    p.method = *get("Method");
    p.basis_set = get("Basis_Set") ? *get("Basis_Set") : "";
    if (get("convergance_criteria")) {
        double e;
        if (!parse_double(*get("convergance_criteria"), e))
            throw Error(CCSD_ERR_INVALID_ARG, "INCAR: convergance_criteria is not a number");
        p.tol = std::pow(10.0, e);
    }
    p.freeze = flag(in.kw, "Freeze_Core");
    p.relax = flag(in.kw, "Relax_Pos");
    p.angstrom = flag(in.kw, "use_angstrom");
    p.print = flag(in.kw, "print_stuffies");
    if (in.Z.empty()) throw Error(CCSD_ERR_INVALID_ARG, "INCAR: no atoms");
    p.Z = in.Z;
    p.R = in.R;
    if (p.angstrom)
        for (double &x : p.R) x *= kBohrPerAngstrom;
    std::string file_text;
    if (!basis_text || !*basis_text) {  // the INCAR's own Basis_File line (this engine's keyword)
        if (!get("Basis_File"))
            throw Error(CCSD_ERR_INVALID_ARG, "no basis: pass Gaussian94 text or give a Basis_File line");
        std::ifstream f(*get("Basis_File"));
        if (!f) throw Error(CCSD_ERR_INVALID_ARG, "cannot read Basis_File '" + *get("Basis_File") + "'");
        std::stringstream ss;
        ss << f.rdbuf();
        file_text = ss.str();
        basis_text = file_text.c_str();
    }
    const Library lib = parse_g94(basis_text);
    for (size_t a = 0; a < p.Z.size(); ++a) {
        auto it = lib.find((int)p.Z[a]);
        if (it == lib.end())
            throw Error(CCSD_ERR_INVALID_ARG, std::string("basis text has no shells for ") + kElements[(int)p.Z[a] - 1]);
        for (const Shell &s : it->second) p.maxprim = std::max(p.maxprim, (int)s.exps.size());
    }
    for (size_t a = 0; a < p.Z.size(); ++a)
        for (const Shell &s : lib.at((int)p.Z[a]))
            for (const auto &c : components(s.L)) {
                p.atom.push_back((int32_t)a);
                p.powers.insert(p.powers.end(), {c[0], c[1], c[2]});
                p.nprim.push_back((int32_t)s.exps.size());
                std::vector<double> al(p.maxprim, 0.0), co(p.maxprim, 0.0);
                for (size_t k = 0; k < s.exps.size(); ++k) {
                    const double e = s.exps[k];
                    const double N = std::pow(2.0 * e / M_PI, 0.75) * std::pow(4.0 * e, 0.5 * s.L) /
                                     std::sqrt(odd_factorial(c[0]) * odd_factorial(c[1]) * odd_factorial(c[2]));
                    al[k] = e;
                    co[k] = s.coefs[k] * N;
                }
                p.alpha.insert(p.alpha.end(), al.begin(), al.end());
                p.coef.insert(p.coef.end(), co.begin(), co.end());
            }
    return p;
}

void copy_name(char *dst, size_t cap, const std::string &s) {
    std::snprintf(dst, cap, "%s", s.c_str());
}

int method_of(const std::string &m) {
    if (m == "HF") return -1;
    if (m == "UHF") return -2;
    if (m == "CCSD" || m == "CCSD1") return CCSD_METHOD_CCSD;
    if (m == "CCSDT-1a") return CCSD_METHOD_CCSDT1A;
    if (m == "CCSDT-1b") return CCSD_METHOD_CCSDT1B;
    if (m == "CCSDT-2") return CCSD_METHOD_CCSDT2;
    if (m == "CCSDT-3") return CCSD_METHOD_CCSDT3;
    if (m == "CCSDT-4") return CCSD_METHOD_CCSDT4;
    if (m == "CCSDT") return CCSD_METHOD_CCSDT;
    throw Error(CCSD_ERR_UNSUPPORTED, "Method '" + m + "' is not built (HF, UHF, CCSD, CCSD1, CCSDT-1a ... CCSDT are)");
}

}  // namespace
}  // namespace ccsd

extern "C" int ccsd_incar_parse(const char *incar_text, const char *basis_text, ccsd_incar *inc) {
    try {
        ccsd::set_last_error("");
        if (!inc) throw ccsd::Error(CCSD_ERR_INVALID_ARG, "ccsd_incar_parse: result is NULL");
        const ccsd::Parsed p = ccsd::parse_all(incar_text, basis_text);
        ccsd::copy_name(inc->basis_set, sizeof inc->basis_set, p.basis_set);
        ccsd::copy_name(inc->method, sizeof inc->method, p.method);
        inc->convergance_criteria = p.tol;
        inc->freeze_core = p.freeze;
        inc->relax_pos = p.relax;
        inc->use_angstrom = p.angstrom;
        inc->print_stuffies = p.print;
        inc->natoms = (int32_t)p.Z.size();
        inc->nbf = (int32_t)p.atom.size();
        inc->maxprim = p.maxprim;
        int ne = 0;
        for (double z : p.Z) ne += (int)z;
        inc->n_electrons = ne;
        inc->nfrozen = p.freeze ? ccsd_frozen_core_count(p.Z.data(), inc->natoms) : 0;
        if (inc->capacity_atoms >= inc->natoms && inc->Z && inc->R) {
            std::memcpy(inc->Z, p.Z.data(), sizeof(double) * p.Z.size());
            std::memcpy(inc->R, p.R.data(), sizeof(double) * p.R.size());
        }
        if (inc->capacity_bf >= inc->nbf && inc->capacity_prim >= inc->maxprim && inc->atom && inc->powers &&
            inc->nprim && inc->alpha && inc->coef) {
            std::memcpy(inc->atom, p.atom.data(), sizeof(int32_t) * p.atom.size());
            std::memcpy(inc->powers, p.powers.data(), sizeof(int32_t) * p.powers.size());
            std::memcpy(inc->nprim, p.nprim.data(), sizeof(int32_t) * p.nprim.size());
            for (int i = 0; i < inc->nbf; ++i)
                for (int k = 0; k < inc->capacity_prim; ++k) {
                    const bool in = k < p.maxprim;
                    inc->alpha[(size_t)i * inc->capacity_prim + k] = in ? p.alpha[(size_t)i * p.maxprim + k] : 0.0;
                    inc->coef[(size_t)i * inc->capacity_prim + k] = in ? p.coef[(size_t)i * p.maxprim + k] : 0.0;
                }
        }
        return CCSD_OK;
    } catch (const ccsd::Error &e) {
        ccsd::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        ccsd::set_last_error(e.what());
        return CCSD_ERR_INVALID_ARG;
    }
}

extern "C" int ccsd_incar_run(const char *incar_text, const char *basis_text, int32_t precision,
                              ccsd_incar_result *res) {
    try {
        ccsd::set_last_error("");
        if (!res) throw ccsd::Error(CCSD_ERR_INVALID_ARG, "ccsd_incar_run: result is NULL");
        const ccsd::Parsed p = ccsd::parse_all(incar_text, basis_text);
        const int method = ccsd::method_of(p.method);
        *res = ccsd_incar_result{};
        res->method = method;
        ccsd_basis b{};
        b.natoms = (int32_t)p.Z.size();
        b.nbf = (int32_t)p.atom.size();
        b.maxprim = p.maxprim;
        b.Z = p.Z.data();
        b.R = p.R.data();
        b.atom = p.atom.data();
        b.powers = p.powers.data();
        b.nprim = p.nprim.data();
        b.alpha = p.alpha.data();
        b.coef = p.coef.data();
        int ne = 0;
        for (double z : p.Z) ne += (int)z;
        const int n = b.nbf;
        res->nbf = n;
        if (method == -2) {  // UHF as Initializer::Go (initializer.cpp:163-185)
            const int half = ne / 2;
            ccsd_uhf_result u{};
            int rc = CCSD_OK;
            if (ne % 2) {
                rc = ccsd_uhf(&b, half + 1, half, p.tol, 0, &u);
            } else {
                rc = ccsd_uhf(&b, half, half, p.tol, 0, &u);  // the singlet, which Go prints
                if (rc == CCSD_OK && p.print) std::printf("Energy = %.12f (UHF singlet)\n", u.e_uhf);
                if (rc == CCSD_OK) rc = ccsd_uhf(&b, half + 1, half - 1, p.tol, 0, &u);
            }
            if (rc != CCSD_OK) return rc;
            res->e_hf = res->energy = u.e_uhf;
            res->scf_iterations = u.iterations;
            if (p.print) std::printf("Energy = %.12f (UHF)\n", u.e_uhf);
            return CCSD_OK;
        }
        std::vector<double> eps(n), C((size_t)n * n), eri(method >= 0 ? (size_t)n * n * n * n : 0);
        ccsd_scf_result scf{};
        scf.eps = eps.data();
        scf.C = C.data();
        scf.eri = method >= 0 ? eri.data() : nullptr;
        int rc = ccsd_rhf(&b, ne, p.tol, 0, &scf);
        if (rc != CCSD_OK) return rc;
        res->e_hf = scf.e_hf;
        res->scf_iterations = scf.iterations;
        res->energy = scf.e_hf;
        if (p.print) std::printf("Energy = %.12f (Hartree-Fock, tolerance %g)\n", scf.e_hf, p.tol);
        if (method < 0) return CCSD_OK;
        const int nocc = ne / 2;
        const int nfrozen = p.freeze ? ccsd_frozen_core_count(p.Z.data(), b.natoms) : 0;
        std::vector<double> fock((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i) fock[(size_t)i * n + i] = eps[i];
        ccsd_problem prob{};
        prob.nocc = nocc - nfrozen;
        prob.nvir = n - nocc;
        prob.nfrozen = nfrozen;
        prob.integral_kind = CCSD_INTS_AO_DENSE;
        prob.nao = n;
        prob.fock = fock.data();
        prob.eri = eri.data();
        prob.mo_coeff = C.data();
        ccsd_options opt;
        ccsd_default_options(&opt);
        opt.energy_tol = p.tol;
        opt.precision = precision;
        opt.method = method;
        opt.variant = p.method == "CCSD" ? CCSD_VARIANT_MEMORY_OPTIMIZED : CCSD_VARIANT_CCSD;
        opt.verbose = p.print ? 1 : 0;
        ccsd_handle *h = nullptr;
        rc = ccsd_create(&prob, &opt, &h);
        if (rc != CCSD_OK) return rc;
        ccsd_result r{};
        rc = ccsd_solve(h, &r);
        ccsd_destroy(h);
        if (rc != CCSD_OK) return rc;
        res->e_corr = r.e_corr;
        res->cc_iter = r.iterations + 1;
        res->energy = scf.e_hf + r.e_corr;
        if (p.print) std::printf("Energy = %.12f (%s)\n", res->energy, p.method.c_str());
        return CCSD_OK;
    } catch (const ccsd::Error &e) {
        ccsd::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        ccsd::set_last_error(e.what());
        return CCSD_ERR_INVALID_ARG;
    }
}
