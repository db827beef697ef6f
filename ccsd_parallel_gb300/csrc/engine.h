// CCSD amplitude engine: device-resident integrals, amplitudes and
// intermediates for one closed-shell system, and the iteration driver.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ccsd_gb300.h"
#include "common.h"
#include "split_gemm.h"

namespace ccsd {

// Owning device buffer of doubles.
struct DBuf {
    double *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    explicit DBuf(size_t count);
    ~DBuf();
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf &operator=(DBuf &&o) noexcept;
    void alloc(size_t count);
    void ensure(size_t count) {
        if (!p || n != count) alloc(count);
    }
    void zero(cudaStream_t st);
};

// One recorded operation of the forward computation (build or residual),
// replayed backwards for the adjoint (Lambda) equations and the gradient.
struct TapeOp {
    // TauSym: (t1 = tau) -> out1 = tau+, out2 = tau-;  Unpack: (t1 = S+, t2 = S-) -> out1 = R (+=);
    // WSym: (t1 = W) -> out1 = W+, out2 = W-   (ladder_sym.cu)
    enum Kind { Gemm, Axpby, Copy, Tau, Theta, TauSym, Unpack, WSym } kind;
    int M = 0, N = 0, K = 0;  // Gemm: sizes; Axpby: R = M, C = N; Copy: count = M
    double alpha = 0.0, beta = 0.0;
    MatView A, B;  // Gemm operands; Axpby/Copy: A = source
    OutView C;     // destination
    const double *t1 = nullptr, *t2 = nullptr;  // Tau/Theta inputs
    double *out1 = nullptr, *out2 = nullptr;    // Tau: out1 = tau; Theta: out1 = th1, out2 = th2
    const char *site = nullptr;                 // Gemm: contraction site name
    int key_a = 0, key_b = 0;                   // Gemm: split-cache keys of the operands
};

class Batch;

class Engine {
    friend class Batch;  // the batched solve groups the recorded residuals of many engines

  public:
    Engine(const ccsd_problem &prob, const ccsd_options &opts);
    ~Engine();
    void set_options(const ccsd_options &opts);
    void solve(ccsd_result *res);
    // Lambda equations at the last solution and dE_corr/d(inputs); see abi.cpp.
    void lambda_grad(const ccsd_problem &prob, ccsd_grad *out);

    int nocc() const { return o_; }
    int nvir() const { return v_; }

  private:
    // set-up
    void build_integrals(const ccsd_problem &prob);
    // (pq|rs) with leading dimension ld, active orbitals from orbital `off` on
    void build_from_mo_dense(const double *eri_dev, int64_t ld, int64_t off);
    void build_from_df(const double *b_dev, int naux);
    void ao_to_mo(const double *ao_dev, const double *c_dev, int nao, DBuf &mo_out);
    void build_derived();
    static void check_closed_shell_so(const double *so_host, int n);

    // contractions: C(m,n) = alpha sum_k A(m,k) B(n,k) + beta C(m,n).
    // `cache_a/b` != 0 marks an operand view over constant integrals whose
    // split form is kept between updates.
    void gemm(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
              const OutView &C, int cache_a = 0, int cache_b = 0, const char *site = nullptr);
    bool use_split(int M, int N, int K) const;

    // contraction profiling (options.profile)
    struct ProfSite {
        long calls = 0;
        double ms = 0.0, split_ms = 0.0, flops = 0.0;
        bool split = false;
    };
    struct ProfPending {
        const char *site;
        cudaEvent_t a, b, c;
        double flops;
        bool split;
    };
    // One update's residual and amplitude-update kernels as a CUDA graph, one per
    // parity of the swapped amplitude buffers; replayed instead of re-issuing ~130
    // launches and their host work.  Kept for one solve; not used while profiling
    // (the per-site CUDA events cannot be timed from a graph).
    struct UpdateGraph {
        cudaGraphExec_t exec = nullptr;
        const double *t1 = nullptr, *t2 = nullptr;
        long launches = 0;
    };
    UpdateGraph graphs_[2];
    bool graphs_ok_ = true;
    void update_step();
    void update_step_graph();
    void release_graphs();
    cudaEvent_t prof_event();
    void prof_flush();
    std::map<std::string, ProfSite> prof_;
    std::vector<ProfPending> prof_pending_;
    std::vector<cudaEvent_t> prof_pool_;
    double prof_update_ms_ = 0.0;
    int prof_updates_ = 0;

  public:
    std::string profile_json() const;

  private:

    // one amplitude update: residual numerators from (t1_, t2_)
    void residual();
    // CCSDT-1a (triples.cpp): spin-orbital T3, its contraction intermediates and
    // the spin-orbital integral blocks it reads
    void triples_setup();
    void triples_step();
    DBuf t3_, y3_, z3_, t2so_, so_vvvo_, so_ovoo_, so_oovv_, so_vovv_, so_ooov_;
    DBuf t1so_, g1b_, g2b_, h3b_, h4b_, f1b_, w5b_;  // CCSDT-1b T3 T1 intermediates
    DBuf x1d_, x2d_, x12_, x13_, q12_, q13_;         // CCSDT-2: dressed X1/X2, X12/X13 and their products
    DBuf so_voov_, so_oooo_, so_vvvv_, tauso_;       // CCSDT-3
    DBuf p1_, p2_, p3_, p4_, a1_, d14_, e15_, g15_, x14_, x15_;
    DBuf x3_, x4_, x6_, x7_, x8_, fsoT_;             // CCSDT: dressed X3/X4/X6, X7, X8
    void triples_m4_terms();
    void triples_m5_terms();
    void triples_1b_terms();
    void triples_m3_products();

    // recordable element-wise operations (every op of build and residual goes
    // through these or through gemm())
    void axpby(int R, int C, double alpha, const MatView &X, double beta, const OutView &Y);
    void copy(double *dst, const double *src, size_t n);
    void tau_op(const double *t1, const double *t2, double *tau);
    void theta_op(const double *t1, const double *t2, double *th1, double *th2);
    void tau_sym_op(const double *tau, double *tp, double *tm);
    void unpack_op(const double *sp, const double *sm, double *R);
    void w_sym_op(const double *W, double *wp, double *wm);

    // reverse mode
    std::vector<TapeOp> *tape_ = nullptr;  // recording target, or null
    bool record_only_ = false;             // record into tape_ without running
    bool grad_lean_vvvv_ = false;          // DF gradient: no (ac|bd) / W+- in the recorded build
    // dE/dB of the pp ladder for DF inputs without the v^4 adjoints (adjoint.cpp)
    void ladder_df_grad(const double *lam2, int naux);
    struct Reg {
        DBuf *buf;
        bool active;  // depends on the amplitudes (Lambda mode propagates into these only)
    };
    std::vector<Reg> regs_;
    std::map<DBuf *, DBuf> adj_;
    bool full_adjoint_ = false;
    void reg(DBuf &b, bool active) { regs_.push_back(Reg{&b, active}); }
    // adjoint pointer for a forward pointer, or null when no adjoint is kept
    double *adj_of(const double *p, bool *active = nullptr);
    void reverse(const std::vector<TapeOp> &tape);
    void zero_adjoints();
    std::vector<std::unique_ptr<DBuf>> keep_;  // inputs kept alive for a recorded build
    DBuf *input_eri_ = nullptr, *input_df_ = nullptr, *input_c_ = nullptr;
    DBuf qtmp_;                                // scratch of the Theta adjoint
    bool solved_ = false;
    double last_e_ = 0.0;
    double energy_of(const double *t1, const double *t2);  // leaves tau(t1, t2) in tau_
    bool tau_fresh_ = false;  // tau_ holds tau(t1_, t2_) from energy_of
    double reduce_sum(int nparts);
    void diis_step(int update_index);
    int diis_store_async(double *dots_dev);                    // DIIS store + overlaps, no sync
    void diis_finish(int update_index, const double *dots);    // B matrix, solve, extrapolation
    int diis_slot_ = 0;                                         // the slot the last store used
    double diis_self_ = 0.0;     // <E, E> of the vector the last diis_step stored
    bool norm_in_diis_ = false;  // this solve takes |T_new - T_old| from diis_self_

    int o_ = 0, v_ = 0, n_ = 0;
    int nf_ = 0, nt_ = 0;  // frozen core orbitals; orbitals of the input arrays (nf_ + n_)
    ccsd_options opt_{};
    cudaStream_t st_ = nullptr;
    bool own_stream_ = false;

    // fock-derived
    DBuf eo_, ev_, f_oo_off_, f_vv_off_, f_ov_;
    // integral blocks (chemist): ovov[i][a][j][b], oovv[i][j][a][b], ovoo[i][a][j][k],
    // oooo[i][j][k][l], ovvv[i][a][b][c], Wv[a][b][c][d] = (ac|bd)
    DBuf ovov_, oovv_, ovoo_, oooo_, ovvv_, wv_;
    // derived: L-combinations; W+ [tri(a,b)][tri(c,d)] and W- [stri][stri] of the ladder;
    // V+ [(k,a)][tri(c,d)] and V- [(k,a)][stri(c,d)] of the pair-form Z, U+ [(k,l)][tri(c,d)]
    // and U- [(k,l)][stri(c,d)] of the pair-form X (unrecorded DF builds)
    DBuf Lovov_, Lovoo_, Lovvv_, LT1_, Lijab_, Wp_, Wm_, Vzp_, Vzm_, Uxp_, Uxm_;
    // ladder pair forms per update: tau+-, S+- (S stored [ij pair][ab pair]); Zs, Za of the
    // pair-form Z, stored [ij pair][(k,a)]; Xs, Xa of the pair-form X, stored [(k,l)][ij pair];
    // W+- [ij pair][kl pair] of the pair-form hh ladder
    DBuf taup_, taum_, Sp_, Sm_, Zs_, Za_, Xs_, Xa_, Whp_, Whm_;
    // amplitudes and intermediates
    DBuf t1_, t2_, t1n_, t2n_, tau_, th1_, th2_;
    DBuf R1_, R_, Rp_;
    DBuf Foo_, Fvv_, Fov_, Loo_, Lvv_, tmpo_, tmpo2_;
    DBuf Woooo_, Wvoov_, Wvovo_, Wa_, Z_, tmpB_, Vk_;
    DBuf ws_, partials_, scalars_;
    DBuf dinv2_;          // 1 / D_ij^ab, [i][j][a][b] (the update multiplies by it)
    bool df_input_ = false;  // integrals from DF factors: (pq|rs) = (rs|pq) for any input
    DBuf Xoooo_;             // sum_cd (kc|ld) tau[i,j,c,d], shared by Foo and Woooo
    DBuf S3_;                // [i][j][a][k]: the o^3 v operands of Rp's t1 terms, summed
    DBuf diis_partials_;  // DIIS overlaps: block partials per stored vector
    // DIIS storage: vectors (T) and errors (T_new - T_old), each o*v + o^2 v^2
    std::vector<DBuf> diis_t_, diis_e_;
    int diis_count_ = 0, diis_next_ = 0;
    std::vector<double> diis_b_;  // (n x n) overlap matrix of stored errors

    std::unique_ptr<SplitEngine> split_;
    // Split modes build the integral blocks from DF factors / AO integrals on
    // a 4-plane engine (relative error ~1e-10), FP64 mode in FP64.
    std::unique_ptr<SplitEngine> build_split_;
    long prof_launches_ = 0;
    double last_resid_ = 0.0;
};

}  // namespace ccsd
