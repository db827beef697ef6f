// CCSD amplitude engine (host side, C++).
//
// Replaces the iterative part of CCSD_Memory_optimized::CCSD
// (ccsd_memory_optimized.cpp:473-557).  The reference iterates a spin-orbital
// Jacobi map with T1 = 0 / MP2 T2 start and stops on |E_new - E_old| < toler
// (:552); this engine iterates the same map written over spatial orbitals for
// a closed-shell determinant (every iterate agrees with the spin-orbital one:
// t(a alpha b beta, i alpha j beta) = t2[i][j][a][b]).  The residual uses
// spin-adapted Stanton-Gauss intermediates; the particle-particle ladder
// contracts the bare (ac|bd) with tau as the reference does (:2093) and adds
// the T1 dressing through one o^3 v^3 contraction.
//
// Every contraction is expressed as C(m,n) = alpha sum_k A(m,k) B(n,k) +
// beta C(m,n) over strided views of the stored tensors (no transposed copies)
// and runs either on the FP64 kernel or on the split-precision tensor-core
// engine, selected per call by the precision option.
#include "engine.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

namespace ccsd {

// ---------------------------------------------------------------------------
DBuf::DBuf(size_t count) { alloc(count); }
DBuf::~DBuf() {
    if (p) cudaFree(p);
}
DBuf &DBuf::operator=(DBuf &&o) noexcept {
    if (this != &o) {
        if (p) cudaFree(p);
        p = o.p;
        n = o.n;
        o.p = nullptr;
        o.n = 0;
    }
    return *this;
}
void DBuf::alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (count == 0) return;
    cudaError_t e = cudaMalloc(&p, count * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        throw Error(CCSD_ERR_OUT_OF_MEMORY,
                    "cudaMalloc of " + std::to_string(count * sizeof(double)) +
                        " bytes failed: " + cudaGetErrorString(e));
    }
}
void DBuf::zero(cudaStream_t st) {
    if (n) CCSD_CUDA(cudaMemsetAsync(p, 0, n * sizeof(double), st));
}

namespace {
struct NvtxScope {
    bool on;
    explicit NvtxScope(const char *name) : on(name != nullptr) {
        if (on) nvtxRangePushA(name);
    }
    ~NvtxScope() {
        if (on) nvtxRangePop();
    }
};

inline MatView mv(const double *p, Dim r, Dim c) {
    MatView m;
    m.p = p;
    m.row = r;
    m.col = c;
    return m;
}
inline OutView ovw(double *p, Dim r, Dim c) {
    OutView m;
    m.p = p;
    m.row = r;
    m.col = c;
    return m;
}
}  // namespace

// ---------------------------------------------------------------------------
Engine::Engine(const ccsd_problem &prob, const ccsd_options &opts) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
    }
    if (prob.nocc <= 0 || prob.nvir <= 0)
        throw Error(CCSD_ERR_INVALID_ARG, "nocc and nvir must be positive");
    if (!prob.fock) throw Error(CCSD_ERR_INVALID_ARG, "fock is NULL");
    if (prob.nfrozen < 0) throw Error(CCSD_ERR_INVALID_ARG, "nfrozen must be >= 0");
    o_ = prob.nocc;
    v_ = prob.nvir;
    n_ = o_ + v_;
    nf_ = prob.nfrozen;
    nt_ = nf_ + n_;
    const double ov2 = (double)o_ * o_ * v_ * v_;
    if (ov2 > 2.0e9 || (double)v_ * v_ >= 2.0e9)
        throw Error(CCSD_ERR_UNSUPPORTED, "shape too large for 32-bit tile indices");
    set_options(opts);
    if (opt_.precision != CCSD_PREC_FP64) build_split_.reset(new SplitEngine(CCSD_PREC_SPLIT4, st_));
    build_integrals(prob);
    build_derived();
    CCSD_CUDA(cudaStreamSynchronize(st_));
    if (build_split_ && build_split_->error_status())
        throw Error(CCSD_ERR_TIMEOUT, "split-precision kernel of the integral build reported a bounded-wait timeout");
    build_split_.reset();
    // the ladder reads W+ and W- (a gradient rebuilds (ac|bd) from the inputs); CCSDT-3
    // builds its spin-orbital <ab||cd> block from (ac|bd) and keeps it
    if (opt_.method < CCSD_METHOD_CCSDT3) wv_.alloc(0);

    const size_t o = o_, v = v_;
    const size_t nT2 = o * o * v * v, nT1 = o * v;
    const size_t To = o * (o + 1) / 2, Tmo = o * (o - 1) / 2, Tv = v * (v + 1) / 2, Tmv = v * (v - 1) / 2;
    taup_.alloc(To * Tv);
    taum_.alloc(Tmo * Tmv);
    Sp_.alloc(To * Tv);
    Sm_.alloc(Tmo * Tmv);
    Zs_.alloc(To * o * v);
    Za_.alloc(Tmo * o * v);
    Xs_.alloc(o * o * To);
    Xa_.alloc(o * o * Tmo);
    Whp_.alloc(To * To);
    Whm_.alloc(Tmo * Tmo);
    t1_.alloc(nT1);
    t2_.alloc(nT2);
    t1n_.alloc(nT1);
    t2n_.alloc(nT2);
    tau_.alloc(nT2);
    th1_.alloc(nT2);
    th2_.alloc(nT2);
    R1_.alloc(nT1);
    R_.alloc(nT2);
    Rp_.alloc(nT2);
    Foo_.alloc(o * o);
    Fvv_.alloc(v * v);
    Fov_.alloc(o * v);
    Loo_.alloc(o * o);
    Lvv_.alloc(v * v);
    tmpo_.alloc(o * o);
    tmpo2_.alloc(o * o);
    Woooo_.alloc(o * o * o * o);
    Wvoov_.alloc(nT2);
    Wvovo_.alloc(nT2);
    Wa_.alloc(nT2);
    Z_.alloc(o * o * o * v);
    tmpB_.alloc(o * o * o * v);
    Vk_.alloc(o * o * o * v);
    ws_.alloc(4u << 20);
    partials_.alloc(reduce_blocks() + 8);
    scalars_.alloc(8);
    CCSD_CUDA(cudaStreamSynchronize(st_));
}

Engine::~Engine() {
    if (st_) cudaStreamSynchronize(st_);
    release_graphs();
    for (const ProfPending &p : prof_pending_) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
        cudaEventDestroy(p.c);
    }
    for (cudaEvent_t e : prof_pool_) cudaEventDestroy(e);
    split_.reset();
    if (own_stream_ && st_) cudaStreamDestroy(st_);
}

void Engine::set_options(const ccsd_options &opts) {
    if (opts.precision != CCSD_PREC_FP64 && opts.precision != CCSD_PREC_SPLIT2 &&
        opts.precision != CCSD_PREC_SPLIT3 && opts.precision != CCSD_PREC_SPLIT4)
        throw Error(CCSD_ERR_INVALID_ARG, "unknown precision mode");
    if (opts.diis_size < 0 || opts.diis_size > 16)
        throw Error(CCSD_ERR_INVALID_ARG, "diis_size must be in [0, 16]");
    if (opts.max_iter < 0 || opts.fixed_iterations < 0)
        throw Error(CCSD_ERR_INVALID_ARG, "iteration counts must be >= 0");
    if (opts.method < CCSD_METHOD_CCSD || opts.method > CCSD_METHOD_CCSDT)
        throw Error(CCSD_ERR_INVALID_ARG, "unknown method");
    if (opts.variant != CCSD_VARIANT_CCSD && opts.variant != CCSD_VARIANT_MEMORY_OPTIMIZED)
        throw Error(CCSD_ERR_INVALID_ARG, "unknown CCSD variant");
    if (opts.variant == CCSD_VARIANT_MEMORY_OPTIMIZED && opts.method != CCSD_METHOD_CCSD)
        throw Error(CCSD_ERR_INVALID_ARG,
                    "the memory-optimised CCSD map is a CCSD method; the triples methods iterate the CCSD1 equations");
    if (opts.t1_start && !opts.t2_start)
        throw Error(CCSD_ERR_INVALID_ARG, "t1_start needs t2_start (a restart sets both, or T2 alone)");
    if (opts.stream) {
        if (own_stream_ && st_) cudaStreamDestroy(st_);
        st_ = (cudaStream_t)opts.stream;
        own_stream_ = false;
    } else if (!st_) {
        CCSD_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    opt_ = opts;
    if (opt_.precision != CCSD_PREC_FP64) {
        if (!split_ || split_->nslices() != opt_.precision) split_.reset(new SplitEngine(opt_.precision, st_));
        split_->set_stream(st_);
    }
}

// ---------------------------------------------------------------------------
// Integral set-up (the reference's Prepear_AOs + Fill_FS, ccsd_memory_optimized.cpp:71-74)
void Engine::build_integrals(const ccsd_problem &prob) {
    const int n = n_, o = o_, v = v_, nt = nt_, nf = nf_;
    // Fock, on the host: the diagonal goes to the denominators; the
    // off-diagonal blocks enter the intermediates (the reference only supports
    // a diagonal matrix, Fill_FS :3560).  Frozen core orbitals (the first nf of
    // the nt input orbitals) are left out: the active block starts at nf.
    {
        std::vector<double> hf((size_t)nt * nt);
        if (prob.device_inputs)
            CCSD_CUDA(cudaMemcpy(hf.data(), prob.fock, sizeof(double) * nt * nt, cudaMemcpyDeviceToHost));
        else
            std::memcpy(hf.data(), prob.fock, sizeof(double) * nt * nt);
        auto F = [&](int p, int q) { return hf[(size_t)(nf + p) * nt + nf + q]; };
        std::vector<double> eo(o), ev(v), oo((size_t)o * o), vv((size_t)v * v), ov((size_t)o * v);
        for (int i = 0; i < o; ++i) eo[i] = F(i, i);
        for (int a = 0; a < v; ++a) ev[a] = F(o + a, o + a);
        for (int i = 0; i < o; ++i)
            for (int j = 0; j < o; ++j) oo[i * o + j] = i == j ? 0.0 : F(i, j);
        for (int a = 0; a < v; ++a)
            for (int b = 0; b < v; ++b) vv[a * v + b] = a == b ? 0.0 : F(o + a, o + b);
        for (int i = 0; i < o; ++i)
            for (int a = 0; a < v; ++a) ov[i * v + a] = F(i, o + a);
        eo_.ensure(o);
        ev_.ensure(v);
        f_oo_off_.ensure((size_t)o * o);
        f_vv_off_.ensure((size_t)v * v);
        f_ov_.ensure((size_t)o * v);
        CCSD_CUDA(cudaMemcpyAsync(eo_.p, eo.data(), sizeof(double) * o, cudaMemcpyHostToDevice, st_));
        CCSD_CUDA(cudaMemcpyAsync(ev_.p, ev.data(), sizeof(double) * v, cudaMemcpyHostToDevice, st_));
        CCSD_CUDA(cudaMemcpyAsync(f_oo_off_.p, oo.data(), sizeof(double) * o * o, cudaMemcpyHostToDevice, st_));
        CCSD_CUDA(cudaMemcpyAsync(f_vv_off_.p, vv.data(), sizeof(double) * v * v, cudaMemcpyHostToDevice, st_));
        CCSD_CUDA(cudaMemcpyAsync(f_ov_.p, ov.data(), sizeof(double) * o * v, cudaMemcpyHostToDevice, st_));
        if (!tape_) {  // the update's reciprocal denominators (not part of a recorded build)
            dinv2_.ensure((size_t)o * o * v * v);
            k_dinv2(o, v, eo_.p, ev_.p, dinv2_.p, st_);
        }
        CCSD_CUDA(cudaStreamSynchronize(st_));
    }

    // Input copies (and transform intermediates) stay alive while a build is
    // recorded for the gradient; otherwise they are freed on return.
    keep_.clear();
    auto keep = [&](std::unique_ptr<DBuf> b) {
        if (tape_) keep_.push_back(std::move(b));
    };
    const cudaMemcpyKind kind = prob.device_inputs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (prob.integral_kind == CCSD_INTS_MO_DENSE) {
        if (!prob.eri) throw Error(CCSD_ERR_INVALID_ARG, "eri is NULL");
        std::unique_ptr<DBuf> eri(new DBuf((size_t)nt * nt * nt * nt));
        CCSD_CUDA(cudaMemcpyAsync(eri->p, prob.eri, sizeof(double) * eri->n, kind, st_));
        build_from_mo_dense(eri->p, nt, nf);
        CCSD_CUDA(cudaStreamSynchronize(st_));
        input_eri_ = eri.get();
        keep(std::move(eri));
    } else if (prob.integral_kind == CCSD_INTS_DF) {
        df_input_ = true;
        if (!prob.df || prob.naux <= 0) throw Error(CCSD_ERR_INVALID_ARG, "df factors missing");
        std::unique_ptr<DBuf> b(new DBuf((size_t)prob.naux * nt * nt));
        CCSD_CUDA(cudaMemcpyAsync(b->p, prob.df, sizeof(double) * b->n, kind, st_));
        build_from_df(b->p, prob.naux);
        CCSD_CUDA(cudaStreamSynchronize(st_));
        input_df_ = b.get();
        keep(std::move(b));
    } else if (prob.integral_kind == CCSD_INTS_AO_DENSE) {
        if (!prob.eri || !prob.mo_coeff || prob.nao < nt)
            throw Error(CCSD_ERR_INVALID_ARG, "AO integrals / mo_coeff missing or nao < n");
        const size_t nao = prob.nao;
        std::unique_ptr<DBuf> ao(new DBuf(nao * nao * nao * nao)), c(new DBuf(nao * nt));
        CCSD_CUDA(cudaMemcpyAsync(ao->p, prob.eri, sizeof(double) * ao->n, kind, st_));
        CCSD_CUDA(cudaMemcpyAsync(c->p, prob.mo_coeff, sizeof(double) * c->n, kind, st_));
        std::unique_ptr<DBuf> mo(new DBuf());
        ao_to_mo(ao->p, c->p, (int)nao, *mo);
        build_from_mo_dense(mo->p, n, 0);
        CCSD_CUDA(cudaStreamSynchronize(st_));
        input_eri_ = ao.get();
        input_c_ = c.get();
        keep(std::move(ao));
        keep(std::move(c));
        keep(std::move(mo));
    } else if (prob.integral_kind == CCSD_INTS_SO_ANTISYM) {
        // <PQ||RS> over N = 2n interleaved spin orbitals (ccsdt.cpp:1466-1478).  For a
        // closed-shell determinant (pq|rs) = <p_alpha r_beta || q_alpha s_beta>
        // = so[2p][2r+1][2q][2s+1]: one strided copy (recorded, so the gradient
        // lands on these elements of the input).
        if (!prob.eri) throw Error(CCSD_ERR_INVALID_ARG, "eri is NULL");
        const int64_t N = 2 * (int64_t)nt, nn = n, f2 = 2 * (int64_t)nf;
        if (!prob.device_inputs) check_closed_shell_so(prob.eri, nt);
        std::unique_ptr<DBuf> so(new DBuf((size_t)(N * N * N * N))), mo(new DBuf((size_t)(nn * nn * nn * nn)));
        CCSD_CUDA(cudaMemcpyAsync(so->p, prob.eri, sizeof(double) * so->n, kind, st_));
        // active block: spin orbitals from 2 nf on
        axpby((int)(nn * nn), (int)(nn * nn), 1.0,
              mv(so->p + f2 * (N * N * N + N * N + N + 1) + N * N + 1, ix2((uint32_t)n, 2 * N * N * N, 2 * N),
                 ix2((uint32_t)n, 2 * N * N, 2)),
              0.0, ovw(mo->p, ix1(nn * nn), ix1(1)));
        build_from_mo_dense(mo->p, n, 0);
        CCSD_CUDA(cudaStreamSynchronize(st_));
        input_eri_ = so.get();
        keep(std::move(so));
        keep(std::move(mo));
    } else {
        throw Error(CCSD_ERR_INVALID_ARG, "unknown integral_kind");
    }
}

// Host check that spin-orbital integrals belong to a closed-shell determinant:
// a fixed sample of same-spin elements must equal (pr|qs) - (ps|qr) built from
// the alpha-beta block, and the spin-forbidden <p_a q_b || r_a s_a> must vanish,
// to 1e-4 of the largest sampled value (it catches open-shell or mis-ordered
// integrals, not rounding).
void Engine::check_closed_shell_so(const double *so, int n) {
    const int64_t N = 2 * (int64_t)n;
    auto at = [&](int64_t P, int64_t Q, int64_t R, int64_t S) { return so[((P * N + Q) * N + R) * N + S]; };
    auto chem = [&](int p, int q, int r, int s) { return at(2 * p, 2 * r + 1, 2 * q, 2 * s + 1); };
    double scale = 0.0, worst = 0.0;
    uint64_t x = 0x9E3779B97F4A7C15ull;
    for (int t = 0; t < 4096; ++t) {
        int idx[4];
        for (int &k : idx) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            k = (int)(x % (uint64_t)n);
        }
        const int p = idx[0], q = idx[1], r = idx[2], s = idx[3];
        const double ref = chem(p, r, q, s) - chem(p, s, q, r);
        scale = std::max(scale, std::fabs(ref));
        worst = std::max(worst, std::fabs(at(2 * p, 2 * q, 2 * r, 2 * s) - ref));
        worst = std::max(worst, std::fabs(at(2 * p + 1, 2 * q + 1, 2 * r + 1, 2 * s + 1) - ref));
        worst = std::max(worst, std::fabs(at(2 * p, 2 * q + 1, 2 * r, 2 * s)));
    }
    if (worst > 1e-4 * std::max(scale, 1e-12))
        throw Error(CCSD_ERR_INVALID_ARG,
                    "spin-orbital integrals are not those of a closed-shell determinant (same-spin elements differ "
                    "from (pr|qs) - (ps|qr) of the alpha-beta block by " + std::to_string(worst) + ")");
}

// Y[p'][q'][r'][s'] = eri[p0+p'][q0+q'][r0+r'][s0+s'] for every block.
void Engine::build_from_mo_dense(const double *eri, int64_t ld, int64_t off) {
    const int64_t n = ld, o = o_, v = v_;
    eri += ((off * n + off) * n + off) * n + off;
    auto blk = [&](DBuf &dst, int64_t p0, int64_t ep, int64_t q0, int64_t eq, int64_t r0,
                   int64_t er, int64_t s0, int64_t es) {
        dst.ensure((size_t)(ep * eq * er * es));
        const double *base = eri + ((p0 * n + q0) * n + r0) * n + s0;
        axpby((int)(ep * eq), (int)(er * es), 1.0,
              mv(base, ix2((uint32_t)eq, n * n * n, n * n), ix2((uint32_t)es, n, 1)), 0.0,
              ovw(dst.p, ix1(er * es), ix1(1)));
    };
    blk(ovov_, 0, o, o, v, 0, o, o, v);
    blk(oovv_, 0, o, 0, o, o, v, o, v);
    blk(ovoo_, 0, o, o, v, 0, o, 0, o);
    blk(oooo_, 0, o, 0, o, 0, o, 0, o);
    blk(ovvv_, 0, o, o, v, o, v, o, v);
    // Wv[a][b][c][d] = (ac|bd) = eri[o+a][o+c][o+b][o+d]
    wv_.ensure((size_t)(v * v * v * v));
    const double *base = eri + ((o * n + o) * n + o) * n + o;
    axpby((int)(v * v), (int)(v * v), 1.0,
          mv(base, ix2((uint32_t)v, n * n * n, n), ix2((uint32_t)v, n * n, 1)), 0.0,
          ovw(wv_.p, ix1(v * v), ix1(1)));
}

// (pq|rs) = sum_Q B[Q][p][q] B[Q][r][s] as contractions over Q.
void Engine::build_from_df(const double *B, int naux) {
    // B[Q][p][q] over the nt_ input orbitals; the active ones start at nf_
    const int64_t n = nt_, o = o_, v = v_, nn = n * n;
    B += (int64_t)nf_ * n + nf_;
    auto blk = [&](DBuf &dst, int64_t p0, int64_t ep, int64_t q0, int64_t eq, int64_t r0,
                   int64_t er, int64_t s0, int64_t es) {
        dst.ensure((size_t)(ep * eq * er * es));
        gemm((int)(ep * eq), (int)(er * es), naux, 1.0,
             mv(B + p0 * n + q0, ix2((uint32_t)eq, n, 1), ix1(nn)),
             mv(B + r0 * n + s0, ix2((uint32_t)es, n, 1), ix1(nn)), 0.0,
             ovw(dst.p, ix1(er * es), ix1(1)));
    };
    blk(ovov_, 0, o, o, v, 0, o, o, v);
    blk(oovv_, 0, o, 0, o, o, v, o, v);
    blk(ovoo_, 0, o, o, v, 0, o, 0, o);
    blk(oooo_, 0, o, 0, o, 0, o, 0, o);
    blk(ovvv_, 0, o, o, v, o, v, o, v);
    // Wv[a][b][c][d] = (ac|bd): M = (a,c), N = (b,d), K = Q.  A gradient with DF
    // inputs takes the ladder's dE/dB directly (Engine::ladder_df_grad) and
    // records the build without this block and its pair forms.
    if (grad_lean_vvvv_) return;
    wv_.ensure((size_t)(v * v * v * v));
    const double *bvv = B + o * n + o;
    gemm((int)(v * v), (int)(v * v), naux, 1.0, mv(bvv, ix2((uint32_t)v, n, 1), ix1(nn)),
         mv(bvv, ix2((uint32_t)v, n, 1), ix1(nn)), 0.0,
         ovw(wv_.p, ix2((uint32_t)v, v * v * v, v), ix2((uint32_t)v, v * v, 1)));
}

// Four quarter transforms (mu nu|la si) -> (pq|rs) with C[mu][p]
// (the reference's Prepear_AOs quarter matvecs, ccsd_memory_optimized.cpp:2990-3037).
void Engine::ao_to_mo(const double *ao, const double *c_in, int nao_i, DBuf &mo) {
    // C[mu][p] over the nt_ input orbitals (row stride nt_); the active columns start at nf_
    const int64_t N = nao_i, n = n_, ldc = nt_;
    const double *c = c_in + nf_;
    std::unique_ptr<DBuf> x1(new DBuf((size_t)(n * N * N * N))), x2(new DBuf((size_t)(n * n * N * N))),
        x3(new DBuf((size_t)(n * n * n * N)));
    mo.ensure((size_t)(n * n * n * n));
    // x1[p][nu][la][si] = sum_mu C[mu][p] ao[mu][nu la si]
    gemm((int)n, (int)(N * N * N), (int)N, 1.0, mv(c, ix1(1), ix1(ldc)),
         mv(ao, ix1(1), ix1(N * N * N)), 0.0, ovw(x1->p, ix1(N * N * N), ix1(1)));
    // x2[p][q][la si] = sum_nu C[nu][q] x1[p][nu][la si]; M = q, N = (p, lasi)
    gemm((int)n, (int)(n * N * N), (int)N, 1.0, mv(c, ix1(1), ix1(ldc)),
         mv(x1->p, ix2((uint32_t)(N * N), N * N * N, 1), ix1(N * N)), 0.0,
         ovw(x2->p, ix1(N * N), ix2((uint32_t)(N * N), n * N * N, 1)));
    // x3[pq][r][si] = sum_la C[la][r] x2[pq][la][si]; M = r, N = (pq, si)
    gemm((int)n, (int)(n * n * N), (int)N, 1.0, mv(c, ix1(1), ix1(ldc)),
         mv(x2->p, ix2((uint32_t)N, N * N, 1), ix1(N)), 0.0,
         ovw(x3->p, ix1(N), ix2((uint32_t)N, n * N, 1)));
    // mo[pqr][s] = sum_si C[si][s] x3[pqr][si]; M = s, N = pqr
    gemm((int)n, (int)(n * n * n), (int)N, 1.0, mv(c, ix1(1), ix1(ldc)),
         mv(x3->p, ix1(N), ix1(1)), 0.0, ovw(mo.p, ix1(1), ix1(n)));
    CCSD_CUDA(cudaStreamSynchronize(st_));
    if (tape_) {
        keep_.push_back(std::move(x1));
        keep_.push_back(std::move(x2));
        keep_.push_back(std::move(x3));
    }
}

// L-combinations of the integrals, built once.
void Engine::build_derived() {
    const int64_t o = o_, v = v_;
    const size_t nT2 = (size_t)(o * o * v * v);
    // Lovov[k][c][l][d] = 2 (kc|ld) - (kd|lc)
    Lovov_.ensure(nT2);
    axpby((int)(o * v), (int)(o * v), 2.0, mv(ovov_.p, ix1(o * v), ix1(1)), 0.0,
          ovw(Lovov_.p, ix1(o * v), ix1(1)));
    axpby((int)(o * v), (int)(o * v), -1.0,
          mv(ovov_.p, ix2((uint32_t)v, v * o * v, 1), ix2((uint32_t)v, v, o * v)), 1.0,
          ovw(Lovov_.p, ix1(o * v), ix1(1)));
    // Lovoo[l][c][k][i] = 2 (lc|ki) - (kc|li)
    Lovoo_.ensure((size_t)(o * v * o * o));
    axpby((int)(o * v), (int)(o * o), 2.0, mv(ovoo_.p, ix1(o * o), ix1(1)), 0.0,
          ovw(Lovoo_.p, ix1(o * o), ix1(1)));
    // (kc|li) at [l][c][k][i]: row (l,c) -> l: o (in ovoo[k][c][l][i], l stride o), c: o*o
    axpby((int)(o * v), (int)(o * o), -1.0,
          mv(ovoo_.p, ix2((uint32_t)v, o, o * o), ix2((uint32_t)o, v * o * o, 1)), 1.0,
          ovw(Lovoo_.p, ix1(o * o), ix1(1)));
    // Lovvv[k][d][a][c] = 2 (kd|ac) - (kc|ad)
    const size_t nov3 = (size_t)(o * v * v * v);
    Lovvv_.ensure(nov3);
    axpby((int)(o * v), (int)(v * v), 2.0, mv(ovvv_.p, ix1(v * v), ix1(1)), 0.0,
          ovw(Lovvv_.p, ix1(v * v), ix1(1)));
    // (kc|ad) = ovvv[k][c][a][d] placed at [k][d][a][c]: row (k,d): k v^3, d: 1; col (a,c): a v, c v^2
    axpby((int)(o * v), (int)(v * v), -1.0,
          mv(ovvv_.p, ix2((uint32_t)v, v * v * v, 1), ix2((uint32_t)v, v, v * v)), 1.0,
          ovw(Lovvv_.p, ix1(v * v), ix1(1)));
    // LT1[i][a][k][c] = 2 (kc|ia) - (ki|ac)
    LT1_.ensure(nT2);
    axpby((int)(o * v), (int)(o * v), 2.0, mv(ovov_.p, ix1(1), ix1(o * v)), 0.0,
          ovw(LT1_.p, ix1(o * v), ix1(1)));
    // (ki|ac) = oovv[k][i][a][c]: row (i,a): i v^2, a v; col (k,c): k o v^2, c 1
    axpby((int)(o * v), (int)(o * v), -1.0,
          mv(oovv_.p, ix2((uint32_t)v, v * v, v), ix2((uint32_t)v, o * v * v, 1)), 1.0,
          ovw(LT1_.p, ix1(o * v), ix1(1)));
    // Lijab[i][j][a][b] = 2 (ia|jb) - (ib|ja)
    Lijab_.ensure(nT2);
    axpby((int)(o * o), (int)(v * v), 2.0,
          mv(ovov_.p, ix2((uint32_t)o, v * o * v, v), ix2((uint32_t)v, o * v, 1)), 0.0,
          ovw(Lijab_.p, ix1(v * v), ix1(1)));
    axpby((int)(o * o), (int)(v * v), -1.0,
          mv(ovov_.p, ix2((uint32_t)o, v * o * v, v), ix2((uint32_t)v, 1, o * v)), 1.0,
          ovw(Lijab_.p, ix1(v * v), ix1(1)));
    const size_t Tv = (size_t)(v * (v + 1) / 2), Tmv = (size_t)(v * (v - 1) / 2);
    // V+- and U+- of the pair-form Z and X, for the unrecorded residuals of DF inputs (the
    // others contract ovvv and ovov directly); a recorded build leaves them as they are.
    // V+- hold about as much as ovvv, and their split planes up to as much again, so they are
    // built only when the device keeps room for them next to what is still to come (W+- and
    // their planes, the per-update tensors and DIIS vectors, 2 GiB spare); a system near the
    // device's capacity contracts ovvv directly for Z, as before.
    if (!tape_ && df_input_) {
        const double vbytes = 8.0 * (double)(o * v) * (double)(Tv + Tmv);
        const double need = 2.0 * vbytes + 16.0 * ((double)Tv * Tv + (double)Tmv * Tmv) +
                            192.0 * (double)(o * o) * (double)(v * v) + 2.0 * (1 << 30);
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && (double)free_b > need) {
            Vzp_.ensure((size_t)(o * v) * Tv);
            Vzm_.ensure((size_t)(o * v) * Tmv);
            k_ovvv_pair_pack((int)o, (int)v, ovvv_.p, Vzp_.p, Vzm_.p, st_);
        } else {
            cudaGetLastError();
            Vzp_.alloc(0);
            Vzm_.alloc(0);
        }
        Uxp_.ensure((size_t)(o * o) * Tv);
        Uxm_.ensure((size_t)(o * o) * Tmv);
        k_ovov_pair_pack((int)o, (int)v, ovov_.p, Uxp_.p, Uxm_.p, st_);
    }
    // W+ [tri(a,b)][tri(c,d)] and W- [stri(a,b)][stri(c,d)] of the pair-form ladder
    if (grad_lean_vvvv_) return;
    Wp_.ensure(Tv * Tv);
    Wm_.ensure(Tmv * Tmv);
    w_sym_op(wv_.p, Wp_.p, Wm_.p);
}

// ---------------------------------------------------------------------------
bool Engine::use_split(int M, int N, int K) const {
    if (opt_.precision == CCSD_PREC_FP64 || (!split_ && !build_split_)) return false;
    return M >= 16 && N >= 16 && K >= 4 && (double)M * N * K >= 1.0e7;
}

void Engine::gemm(int M, int N, int K, double alpha, const MatView &A, const MatView &B,
                  double beta, const OutView &C, int cache_a, int cache_b, const char *site) {
    if (tape_) {  // record, then run the same call unrecorded
        TapeOp op;
        op.kind = TapeOp::Gemm;
        op.M = M;
        op.N = N;
        op.K = K;
        op.alpha = alpha;
        op.beta = beta;
        op.A = A;
        op.B = B;
        op.C = C;
        op.site = site;
        op.key_a = cache_a;
        op.key_b = cache_b;
        tape_->push_back(op);
        if (record_only_) return;
        std::vector<TapeOp> *t = tape_;
        tape_ = nullptr;
        gemm(M, N, K, alpha, A, B, beta, C, cache_a, cache_b, site);
        tape_ = t;
        return;
    }
    const bool prof = opt_.profile && site;
    const bool split = use_split(M, N, K);
    if (split && SplitEngine::prefer_swap(M, N, C)) {
        gemm(N, M, K, alpha, B, A, beta, OutView{C.p, C.col, C.row}, cache_b, cache_a, site);
        return;
    }
    cudaEvent_t ea = nullptr, eb = nullptr, ec = nullptr;
    NvtxScope nvtx(prof ? site : nullptr);  // lets ncu --nvtx-include pick one contraction site
    if (prof) {
        ea = prof_event();
        eb = prof_event();
        ec = prof_event();
        CCSD_CUDA(cudaEventRecord(ea, st_));
    }
    if (split) {
        SplitEngine *se = build_split_ ? build_split_.get() : split_.get();
        SplitOperand *a = se->prepare(cache_a, M, K, A, 0);
        SplitOperand *b = se->prepare(cache_b, N, K, B, 1);
        if (prof) CCSD_CUDA(cudaEventRecord(eb, st_));
        se->run(*a, *b, M, N, alpha, beta, C);
    } else {
        if (prof) CCSD_CUDA(cudaEventRecord(eb, st_));
        gemm_f64(M, N, K, alpha, A, B, beta, C, ws_.p, ws_.n, st_);
    }
    if (prof) {
        CCSD_CUDA(cudaEventRecord(ec, st_));
        prof_pending_.push_back(ProfPending{site, ea, eb, ec, 2.0 * M * (double)N * K, split});
    }
}

cudaEvent_t Engine::prof_event() {
    if (!prof_pool_.empty()) {
        cudaEvent_t e = prof_pool_.back();
        prof_pool_.pop_back();
        return e;
    }
    cudaEvent_t e;
    CCSD_CUDA(cudaEventCreate(&e));
    return e;
}

// Resolve the recorded events (the stream has been synchronised).
void Engine::prof_flush() {
    for (const ProfPending &p : prof_pending_) {
        float split_ms = 0.f, ms = 0.f;
        CCSD_CUDA(cudaEventElapsedTime(&split_ms, p.a, p.b));
        CCSD_CUDA(cudaEventElapsedTime(&ms, p.b, p.c));
        ProfSite &s = prof_[p.site];
        s.calls += 1;
        s.ms += ms;
        s.split_ms += split_ms;
        s.flops += p.flops;
        s.split = p.split;
        prof_pool_.push_back(p.a);
        prof_pool_.push_back(p.b);
        prof_pool_.push_back(p.c);
    }
    prof_pending_.clear();
}

std::string Engine::profile_json() const {
    std::string s = "{\"updates\": " + std::to_string(prof_updates_) +
                    ", \"update_ms_total\": " + std::to_string(prof_update_ms_) +
                    ", \"launches\": " + std::to_string(prof_launches_) + ", \"sites\": [";
    bool first = true;
    char buf[512];
    for (const auto &kv : prof_) {
        std::snprintf(buf, sizeof buf,
                      "%s{\"site\": \"%s\", \"calls\": %ld, \"ms\": %.6f, \"split_ms\": %.6f, \"flops\": %.6e, "
                      "\"path\": \"%s\"}",
                      first ? "" : ", ", kv.first.c_str(), kv.second.calls, kv.second.ms, kv.second.split_ms,
                      kv.second.flops, kv.second.split ? "split" : "fp64");
        s += buf;
        first = false;
    }
    s += "]}";
    return s;
}

// ---------------------------------------------------------------------------
// Residual numerators (diagonal Fock moved to the denominators).
//   R1[i][a]      T1 numerator
//   R[i][j][a][b] terms already symmetric under (ij,ab) -> (ji,ba)
//   Rp            terms to be symmetrised: R2 = R + Rp + Rp^T
void Engine::residual() {
    const int64_t o = o_, v = v_, ov = o * v, v2 = v * v, ov2 = o * v2, o2 = o * o;
    const int io = (int)o, iv = (int)v;
    cudaStream_t st = st_;
    const double *t1 = t1_.p, *t2 = t2_.p, *tau = tau_.p;

    // tau of these amplitudes is already in tau_ when the energy was last taken on them
    // (every update of a CCSD solve); a recorded residual keeps its own tau step
    if (!(tau_fresh_ && tape_ == nullptr && opt_.method == CCSD_METHOD_CCSD)) tau_op(t1, t2, tau_.p);
    tau_fresh_ = false;
    theta_op(t1, t2, th1_.p, th2_.p);
    // the split forms of tau as (ij|cd) (key -1) and of the ring view of t2
    // (key -2) are shared by several contractions of this update, and so are
    // tau read as [i][(l,c,d)] (key -5: Foo, R1_ovvv_tau) and as [a][(k,l,d)]
    // (key -6: Fvv, R1_ovoo_tau), and t2 read as [(j,b)][(k,c)] = t2[j][k][b][c]
    // (key -7: Wvoov_t2, ring1 with symmetric amplitudes)
    if (split_ && opt_.precision != CCSD_PREC_FP64) split_->begin_update();

    // Foo[k][i] = f_oo' + sum_{lcd} Lovov[k,c,l,d] tau[i,l,c,d].  With symmetric amplitudes
    // (DF input, no tape: see r1_from_z below) it is sum_l (2 X[k,l,i,l] - X[k,l,l,i]) of the
    // o^4 product X[k][l][i][j] = sum_cd (kc|ld) tau[i,j,c,d] that Woooo needs anyway, so X is
    // formed here (site Woooo_tau, in pair form Woooo_tau_sym/_anti) and the o x o x o v^2
    // contraction is not run.
    const bool sym_amps = tape_ == nullptr && df_input_;
    // With symmetric amplitudes the contractions over a (c,d) or (k,l) pair of tau (X here,
    // the two ladders and Z below) run in pair form on the ladder's tau+- (ladder_sym.cu),
    // formed once here, and their splits (keys -3, -4) are shared.  The pair forms are the
    // plain ones on tau symmetrised over its partners, so they are kept to DF inputs, whose
    // (pq|rs) = (rs|pq) keeps the amplitudes symmetric also under a perturbed input (a dense
    // input perturbed in one element does not, and its gradient is that of the plain forms).
    const bool pairs = sym_amps && Uxp_.p, zpairs = pairs && Vzp_.p;
    const int64_t To = o * (o + 1) / 2, Tmo = o * (o - 1) / 2, Tv = v * (v + 1) / 2, Tmv = v * (v - 1) / 2;
    const bool anti = Tmo > 0 && Tmv > 0;
    if (pairs) tau_sym_op(tau, taup_.p, taum_.p);
    copy(Foo_.p, f_oo_off_.p, (size_t)(o2));
    if (sym_amps) {
        Xoooo_.ensure((size_t)o2 * o2);
        if (pairs) {
            // Xs = U+ tau+^T, Xa = U- tau-^T, X = unpack(Xs, Xa): half of the plain 2 o^4 v^2
            gemm((int)o2, (int)To, (int)Tv, 1.0, mv(Uxp_.p, ix1(Tv), ix1(1)), mv(taup_.p, ix1(Tv), ix1(1)), 0.0,
                 ovw(Xs_.p, ix1(To), ix1(1)), 19, -3, "Woooo_tau_sym");
            if (anti)
                gemm((int)o2, (int)Tmo, (int)Tmv, 1.0, mv(Uxm_.p, ix1(Tmv), ix1(1)), mv(taum_.p, ix1(Tmv), ix1(1)),
                     0.0, ovw(Xa_.p, ix1(Tmo), ix1(1)), 20, -4, "Woooo_tau_anti");
            k_x_pair_unpack(io, Xs_.p, anti ? Xa_.p : nullptr, Xoooo_.p, st_);
        } else {
            gemm((int)o2, (int)o2, (int)v2, 1.0,
                 mv(ovov_.p, ix2((uint32_t)o, v * o * v, v), ix2((uint32_t)v, o * v, 1)),
                 mv(tau, ix1(v2), ix1(1)), 0.0, ovw(Xoooo_.p, ix1(o2), ix1(1)), 5, -1, "Woooo_tau");
        }
        k_foo_from_x(io, Xoooo_.p, Foo_.p, st_);
    } else {
        gemm(io, io, (int)(o * v2), 1.0, mv(Lovov_.p, ix1(v * o * v), ix3((uint32_t)v, (uint32_t)v, v, o * v, 1)),
             mv(tau, ix1(ov2), ix1(1)), 1.0, ovw(Foo_.p, ix1(o), ix1(1)), 1, -5, "Foo");
    }
    // Fvv[a][c] = f_vv' - sum_{kld} Lovov[k,c,l,d] tau[k,l,a,d]
    copy(Fvv_.p, f_vv_off_.p, (size_t)(v2));
    gemm(iv, iv, (int)(o * o * v), -1.0, mv(tau, ix1(v), ix3((uint32_t)o, (uint32_t)v, ov2, v2, 1)),
         mv(Lovov_.p, ix1(o * v), ix3((uint32_t)o, (uint32_t)v, v * o * v, v, 1)), 1.0,
         ovw(Fvv_.p, ix1(v), ix1(1)), -6, 2, "Fvv");
    // Fov[k][c] = f_ov + sum_ld Lovov[k,c,l,d] t1[l,d]
    copy(Fov_.p, f_ov_.p, (size_t)(ov));
    gemm((int)ov, 1, (int)ov, 1.0, mv(Lovov_.p, ix1(ov), ix1(1)), mv(t1, ix1(0), ix1(1)), 1.0,
         ovw(Fov_.p, ix1(1), ix1(0)), 0, 0, "Fov");
    // Loo[k][i] = Foo + sum_c f_kc t1[i,c] + sum_lc Lovoo[l,c,k,i] t1[l,c]
    copy(Loo_.p, Foo_.p, (size_t)(o2));
    gemm(io, io, iv, 1.0, mv(f_ov_.p, ix1(v), ix1(1)), mv(t1, ix1(v), ix1(1)), 1.0,
         ovw(Loo_.p, ix1(o), ix1(1)), 0, 0, "Loo_f");
    gemm((int)o2, 1, (int)ov, 1.0, mv(Lovoo_.p, ix1(1), ix1(o2)), mv(t1, ix1(0), ix1(1)), 1.0,
         ovw(Loo_.p, ix1(1), ix1(0)), 0, 0, "Loo_t1");
    // Lvv[a][c] = Fvv - sum_k t1[k,a] f_kc + sum_kd Lovvv[k,d,a,c] t1[k,d]
    copy(Lvv_.p, Fvv_.p, (size_t)(v2));
    gemm(iv, iv, io, -1.0, mv(t1, ix1(1), ix1(v)), mv(f_ov_.p, ix1(1), ix1(v)), 1.0,
         ovw(Lvv_.p, ix1(v), ix1(1)), 0, 0, "Lvv_f");
    // With symmetric amplitudes (sym_amps) the Lovvv t1 term is not read from the o v^3 block
    // here: sum_kd Lovvv[k,d,a,c] t1[k,d] = 2 sum_k X[(k,a,c)][k] - sum_k Y[(k,c,a)][k] with
    // the products X of site Wvovo_t1v and Y of site Rp_ovvv_t1 below, whose diagonals are
    // added to Lvv there (Lvv is first read by Rp_Lvv, after both).
    if (!sym_amps)
        gemm((int)v2, 1, (int)ov, 1.0, mv(Lovvv_.p, ix1(1), ix1(v2)), mv(t1, ix1(0), ix1(1)), 1.0,
             ovw(Lvv_.p, ix1(1), ix1(0)), 0, 0, "Lvv_t1");

    // ---- T1 numerator ----------------------------------------------------
    copy(R1_.p, f_ov_.p, (size_t)(ov));
    // -2 sum_kc f_kc t1[k,a] t1[i,c]: tmpo[i][k] = sum_c t1[i,c] f_kc
    gemm(io, io, iv, 1.0, mv(t1, ix1(v), ix1(1)), mv(f_ov_.p, ix1(v), ix1(1)), 0.0,
         ovw(tmpo_.p, ix1(o), ix1(1)), 0, 0, "R1_ft1");
    gemm(io, iv, io, -2.0, mv(tmpo_.p, ix1(o), ix1(1)), mv(t1, ix1(1), ix1(v)), 1.0,
         ovw(R1_.p, ix1(v), ix1(1)), 0, 0, "R1_ft1t1");
    // + sum_c Fvv'[a,c] t1[i,c]
    gemm(io, iv, iv, 1.0, mv(t1, ix1(v), ix1(1)), mv(Fvv_.p, ix1(v), ix1(1)), 1.0,
         ovw(R1_.p, ix1(v), ix1(1)), 0, 0, "R1_Fvv");
    // - sum_k Foo'[k,i] t1[k,a]
    gemm(io, iv, io, -1.0, mv(Foo_.p, ix1(1), ix1(o)), mv(t1, ix1(1), ix1(v)), 1.0,
         ovw(R1_.p, ix1(v), ix1(1)), 0, 0, "R1_Foo");
    // + sum_kc Fov[k,c] (2 t2[k,i,c,a] - t2[i,k,c,a]).  With symmetric amplitudes
    // (t2[i,k,c,a] = t2[k,i,a,c]) this is 2 sum_kc Fov[k,c] th1[k,c,i,a] + 2 sum_kc Fov[k,c] t1[k,a] t1[i,c]:
    // one pass over th1 instead of two over t2, the second part joining the next term
    const bool fov_th1 = sym_amps;
    if (fov_th1) {
        gemm((int)ov, 1, (int)ov, 2.0, mv(th1_.p, ix1(1), ix1(ov)), mv(Fov_.p, ix1(0), ix1(1)), 1.0,
             ovw(R1_.p, ix1(1), ix1(0)), 0, 0, "R1_Fov_th1");
    } else {
        gemm((int)ov, 1, (int)ov, 2.0, mv(t2, ix2((uint32_t)v, v2, 1), ix2((uint32_t)v, ov2, v)),
             mv(Fov_.p, ix1(0), ix1(1)), 1.0, ovw(R1_.p, ix1(1), ix1(0)), 0, 0, "R1_Fov_t2a");
        gemm((int)ov, 1, (int)ov, -1.0, mv(t2, ix2((uint32_t)v, ov2, 1), ix2((uint32_t)v, v2, v)),
             mv(Fov_.p, ix1(0), ix1(1)), 1.0, ovw(R1_.p, ix1(1), ix1(0)), 0, 0, "R1_Fov_t2b");
    }
    // + sum_kc Fov[k,c] t1[i,c] t1[k,a] (three times that with fov_th1)
    gemm(io, io, iv, 1.0, mv(t1, ix1(v), ix1(1)), mv(Fov_.p, ix1(v), ix1(1)), 0.0,
         ovw(tmpo2_.p, ix1(o), ix1(1)), 0, 0, "R1_Fovt1");
    gemm(io, iv, io, fov_th1 ? 3.0 : 1.0, mv(tmpo2_.p, ix1(o), ix1(1)), mv(t1, ix1(1), ix1(v)), 1.0,
         ovw(R1_.p, ix1(v), ix1(1)), 0, 0, "R1_Fovt1t1");
    // + sum_kc LT1[i,a,k,c] t1[k,c]
    gemm((int)ov, 1, (int)ov, 1.0, mv(LT1_.p, ix1(ov), ix1(1)), mv(t1, ix1(0), ix1(1)), 1.0,
         ovw(R1_.p, ix1(1), ix1(0)), 0, 0, "R1_LT1");
    // + sum_kcd Lovvv[k,d,a,c] tau[i,k,c,d].  With tau[i,k,d,c] = tau[k,i,c,d] this equals
    // sum_k (2 Z[i,k,k,a] - Z[k,i,k,a]) with Z of Rp_Z below, so the o v^3 block need not
    // be read a second time (r1_from_z).  The amplitudes keep that symmetry whenever
    // (pq|rs) = (rs|pq), which DF factors guarantee for any B; dense inputs may break it
    // (one perturbed element, as a finite-difference check does), and a recorded
    // residual (gradient, batched solve) follows the contraction's per-element
    // derivative convention, so both keep the contraction.
    const bool r1_from_z = sym_amps;
    if (!r1_from_z)
    gemm(io, iv, (int)(o * v2), 1.0, mv(tau, ix1(ov2), ix1(1)),
         mv(Lovvv_.p, ix1(v), ix3((uint32_t)v, (uint32_t)v, v * v2, 1, v2)), 1.0,
         ovw(R1_.p, ix1(v), ix1(1)), -5, 3, "R1_ovvv_tau");
    // - sum_klc Lovoo[l,c,k,i] tau[k,l,a,c]
    gemm(io, iv, (int)(o2 * v), -1.0,
         mv(Lovoo_.p, ix1(1), ix3((uint32_t)o, (uint32_t)v, o, v * o2, o2)),
         mv(tau, ix1(v), ix3((uint32_t)o, (uint32_t)v, ov2, v2, 1)), 1.0,
         ovw(R1_.p, ix1(v), ix1(1)), 4, -6, "R1_ovoo_tau");

    // ---- Woooo[k][l][i][j] ------------------------------------------------
    axpby((int)o2, (int)o2, 1.0, mv(oooo_.p, ix2((uint32_t)o, o * o2, o), ix2((uint32_t)o, o2, 1)),
               0.0, ovw(Woooo_.p, ix1(o2), ix1(1)));
    // + sum_c (lc|ki) t1[j,c]: M = (k,l,i), N = j, K = c
    gemm((int)(o * o2), io, iv, 1.0,
         mv(ovoo_.p, ix3((uint32_t)o, (uint32_t)o, o, v * o2, 1), ix1(o2)), mv(t1, ix1(v), ix1(1)),
         1.0, ovw(Woooo_.p, ix1(o), ix1(1)), 0, 0, "Woooo_t1a");
    // + sum_c (kc|lj) t1[i,c]: M = (k,l,j), N = i
    gemm((int)(o * o2), io, iv, 1.0,
         mv(ovoo_.p, ix3((uint32_t)o, (uint32_t)o, v * o2, o, 1), ix1(o2)), mv(t1, ix1(v), ix1(1)),
         1.0, ovw(Woooo_.p, ix3((uint32_t)o, (uint32_t)o, o * o2, o2, 1), ix1(o)), 0, 0, "Woooo_t1b");
    // + sum_cd (kc|ld) tau[i,j,c,d]: M = (k,l), N = (i,j), K = (c,d) (already formed as X above
    // when the amplitudes are symmetric)
    if (sym_amps)
        k_lincomb2((size_t)o2 * o2, 1.0, Woooo_.p, 1.0, Xoooo_.p, Woooo_.p, st_);
    else
        gemm((int)o2, (int)o2, (int)v2, 1.0,
             mv(ovov_.p, ix2((uint32_t)o, v * o * v, v), ix2((uint32_t)v, o * v, 1)),
             mv(tau, ix1(v2), ix1(1)), 1.0, ovw(Woooo_.p, ix1(o2), ix1(1)), 5, -1, "Woooo_tau");

    // ---- Wvoov_s[i][a][k][c] = W_akic ------------------------------------
    // + sum_d (kc|ad) t1[i,d] is the product Y[(p,q,r)][j] = sum_s (pq|rs) t1[j,s] that
    // also opens Rp (Rp[i][j][a][b] = Y[(i,a,b)][j], its first write of the update):
    // Y is formed once, into Rp, and Wvoov[i][a][k][c] = ovov[i][a][k][c] + Y[(k,c,a)][i]
    // (Rp[k][i][c][a]), one pass over both when unrecorded (no copy of ovov first)
    if (tape_) copy(Wvoov_.p, ovov_.p, (size_t)(ov * ov));
    gemm((int)(o * v2), io, iv, 1.0, mv(ovvv_.p, ix1(v), ix1(1)), mv(t1, ix1(v), ix1(1)), 0.0,
         ovw(Rp_.p, ix3((uint32_t)v, (uint32_t)v, ov2, v, 1), ix1(v2)), 6, 0, "Rp_ovvv_t1");
    // Lvv[a][c] -= sum_k Y[(k,c,a)][k] = sum_k Rp[k][k][c][a]
    if (sym_amps) k_diag_acc(o_, v_, -1.0, Rp_.p, (int64_t)(o + 1) * v2, 1, v, Lvv_.p, st_);
    {
        const MatView yv = mv(Rp_.p, ix3((uint32_t)v, (uint32_t)v, ov2, v, 1), ix1(v2));
        const OutView wv = ovw(Wvoov_.p, ix3((uint32_t)v, (uint32_t)v, v, 1, ov), ix1(v * ov));
        if (tape_ || !axpby_view_from((int)(ov * v), io, 1.0, yv, 1.0, ovov_.p, wv, st_)) {
            if (!tape_) copy(Wvoov_.p, ovov_.p, (size_t)(ov * ov));
            axpby((int)(ov * v), io, 1.0, yv, 1.0, wv);
        }
    }
    // - sum_l (kc|li) t1[l,a]: M = (i,k,c) (c, contiguous in Wvoov, innermost), N = a, K = l
    gemm((int)(ov * o), iv, io, -1.0,
         mv(ovoo_.p, ix3((uint32_t)o, (uint32_t)v, 1, v * o2, o2), ix1(o)), mv(t1, ix1(1), ix1(v)),
         1.0, ovw(Wvoov_.p, ix3((uint32_t)o, (uint32_t)v, v * ov, v, 1), ix1(ov)), 13, 0, "Wvoov_t1o");
    // + sum_ld th1[i,a,l,d] (ld|kc), read at ovov[l][d][k][c] (the position the closed-shell
    // equations name, so that dE/d(pq|rs) is assigned per element like the oracle's)
    gemm((int)ov, (int)ov, (int)ov, 1.0, mv(th1_.p, ix1(ov), ix1(1)), mv(ovov_.p, ix1(1), ix1(ov)),
         1.0, ovw(Wvoov_.p, ix1(ov), ix1(1)), 0, 7, "Wvoov_th1");
    // - 1/2 sum_ld (lc|kd) t2[i,l,a,d]
    gemm((int)ov, (int)ov, (int)ov, -0.5, mv(t2, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1)),
         mv(ovov_.p, ix2((uint32_t)v, v, ov), ix2((uint32_t)v, v * ov, 1)), 1.0,
         ovw(Wvoov_.p, ix1(ov), ix1(1)), -7, 8, "Wvoov_t2");

    // ---- Wvovo_s[i][a][k][c] = W_akci ------------------------------------
    axpby((int)ov, (int)ov, 1.0, mv(oovv_.p, ix2((uint32_t)v, v2, v), ix2((uint32_t)v, ov2, 1)),
               0.0, ovw(Wvovo_.p, ix1(ov), ix1(1)));
    // + sum_d (kd|ac) t1[i,d]: M = (k,a,c), N = i, K = d.  Lvv[a][c] += 2 sum_k X[(k,a,c)][k],
    // the change of sum_k Wvovo[k][a][k][c] across this product
    const int64_t wv_k = (int64_t)v * (ov + 1);  // Wvovo[k][a][k][c]: k stride, a stride ov
    if (sym_amps) k_diag_acc(o_, v_, -2.0, Wvovo_.p, wv_k, ov, 1, Lvv_.p, st_);
    gemm((int)(ov * v), io, iv, 1.0,
         mv(ovvv_.p, ix3((uint32_t)v, (uint32_t)v, v * v2, v, 1), ix1(v2)), mv(t1, ix1(v), ix1(1)),
         1.0, ovw(Wvovo_.p, ix3((uint32_t)v, (uint32_t)v, v, ov, 1), ix1(v * ov)), 9, 0, "Wvovo_t1v");
    if (sym_amps) k_diag_acc(o_, v_, 2.0, Wvovo_.p, wv_k, ov, 1, Lvv_.p, st_);
    // - sum_l (lc|ki) t1[l,a]: M = (i,k,c) (c innermost), N = a, K = l
    gemm((int)(ov * o), iv, io, -1.0,
         mv(ovoo_.p, ix3((uint32_t)o, (uint32_t)v, 1, o, o2), ix1(v * o2)), mv(t1, ix1(1), ix1(v)),
         1.0, ovw(Wvovo_.p, ix3((uint32_t)o, (uint32_t)v, v * ov, v, 1), ix1(ov)), 14, 0, "Wvovo_t1o");
    // - sum_ld th2[i,a,l,d] (lc|kd)
    gemm((int)ov, (int)ov, (int)ov, -1.0, mv(th2_.p, ix1(ov), ix1(1)),
         mv(ovov_.p, ix2((uint32_t)v, v, ov), ix2((uint32_t)v, v * ov, 1)), 1.0,
         ovw(Wvovo_.p, ix1(ov), ix1(1)), 0, 8, "Wvovo_th2");
    // Wa = 2 Wvoov - Wvovo (one pass unless a tape records the two steps)
    if (tape_) {
        axpby((int)ov, (int)ov, -1.0, mv(Wvovo_.p, ix1(ov), ix1(1)), 0.0, ovw(Wa_.p, ix1(ov), ix1(1)));
        axpby((int)ov, (int)ov, 2.0, mv(Wvoov_.p, ix1(ov), ix1(1)), 1.0, ovw(Wa_.p, ix1(ov), ix1(1)));
    } else {
        k_lincomb2((size_t)(ov * ov), 2.0, Wvoov_.p, -1.0, Wvovo_.p, Wa_.p, st_);
    }

    // ---- R (symmetric terms) ---------------------------------------------
    // (ia|jb)
    axpby((int)o2, (int)v2, 1.0,
               mv(ovov_.p, ix2((uint32_t)o, v * o * v, v), ix2((uint32_t)v, o * v, 1)), 0.0,
               ovw(R_.p, ix1(v2), ix1(1)));
    // + sum_kl Woooo[k,l,i,j] tau[k,l,a,b] (in the ladder's halves below with the pair forms)
    if (!pairs)
        gemm((int)o2, (int)v2, (int)o2, 1.0, mv(Woooo_.p, ix1(1), ix1(o2)), mv(tau, ix1(1), ix1(v2)),
             1.0, ovw(R_.p, ix1(v2), ix1(1)), 0, 0, "hh_ladder");
    // + sum_cd (ac|bd) tau[i,j,c,d]: the v^4 particle-particle ladder in pair form
    // (ladder_sym.cu): S+ = W+ tau+^T over (a>=b, i>=j, c>=d), S- = W- tau-^T over strict
    // pairs, a quarter of the plain 2 o^2 v^4; R += unpack(S+, S-).  S is stored [ij][ab].
    {
        if (!pairs) tau_sym_op(tau, taup_.p, taum_.p);
        gemm((int)Tv, (int)To, (int)Tv, 1.0, mv(Wp_.p, ix1(Tv), ix1(1)), mv(taup_.p, ix1(Tv), ix1(1)), 0.0,
             ovw(Sp_.p, ix1(1), ix1(Tv)), 10, -3, "pp_ladder_sym");
        gemm((int)Tmv, (int)Tmo, (int)Tmv, 1.0, mv(Wm_.p, ix1(Tmv), ix1(1)), mv(taum_.p, ix1(Tmv), ix1(1)), 0.0,
             ovw(Sm_.p, ix1(1), ix1(Tmv)), 11, -4, "pp_ladder_anti");
        if (pairs) {
            // the hh ladder in the same halves: S+ += W+ tau+ and S- += W- tau- over (k,l)
            // pairs, with W+- the (k,l) packs of Woooo[.,ij] and tau+- read as [ab pair][kl
            // pair] (keys -8, -9): a quarter of the plain 2 o^4 v^2, and no pass of its own over R
            k_oooo_pair_pack(io, Woooo_.p, Whp_.p, Whm_.p, st_);
            gemm((int)To, (int)Tv, (int)To, 1.0, mv(Whp_.p, ix1(To), ix1(1)), mv(taup_.p, ix1(1), ix1(Tv)), 1.0,
                 ovw(Sp_.p, ix1(Tv), ix1(1)), 0, -8, "hh_ladder_sym");
            if (anti)
                gemm((int)Tmo, (int)Tmv, (int)Tmo, 1.0, mv(Whm_.p, ix1(Tmo), ix1(1)), mv(taum_.p, ix1(1), ix1(Tmv)),
                     1.0, ovw(Sm_.p, ix1(Tmv), ix1(1)), 0, -9, "hh_ladder_anti");
        }
        unpack_op(Sp_.p, Sm_.p, R_.p);
    }

    // ---- Rp (terms under P(ij,ab)) -----------------------------------------
    // + sum_c (ia|bc) t1[j,c] is already in Rp (formed with Wvoov above)
    // - sum_k t1[k,a] sum_c (ki|bc) t1[j,c]: Vk[k][i][b][j] = sum_c oovv[k,i,b,c] t1[j,c]
    gemm((int)(o2 * v), io, iv, 1.0, mv(oovv_.p, ix1(v), ix1(1)), mv(t1, ix1(v), ix1(1)), 0.0,
         ovw(Vk_.p, ix1(o), ix1(1)), 15, 0, "Rp_oovv_t1");
    // Unrecorded, the three o^3 v x t1 terms of Rp (this one, tmpB's and Z's below) are summed
    // into one operand and contracted once (site Rp_t1_o3v), one pass over Rp instead of
    // three.  This term enters as its transpose Rp^T[i][j][a][b] = Rp[j][i][b][a], which the
    // update adds anyway (R2 = R + Rp + Rp^T): -sum_k Vk[k][j][a][i] t1[k,b].
    const bool merge_t1 = tape_ == nullptr;
    if (!merge_t1)
        gemm((int)(o * v * o), iv, io, -1.0,
             mv(Vk_.p, ix3((uint32_t)o, (uint32_t)v, v * o, 1, o), ix1(o * v * o)), mv(t1, ix1(1), ix1(v)),
             1.0, ovw(Rp_.p, ix3((uint32_t)o, (uint32_t)v, ov2, v2, 1), ix1(v)), 0, 0, "Rp_oovv_t1t1");
    // - sum_k tmpB[k,i,a,j] t1[k,b], tmpB = (ia|jk) + sum_c (kc|ia) t1[j,c]
    axpby((int)(o * ov), io, 1.0,
               mv(ovoo_.p, ix3((uint32_t)o, (uint32_t)v, 1, v * o2, o2), ix1(o)), 0.0,
               ovw(tmpB_.p, ix1(o), ix1(1)));
    gemm((int)(o * ov), io, iv, 1.0,
         mv(ovov_.p, ix3((uint32_t)o, (uint32_t)v, v * o * v, v, 1), ix1(o * v)), mv(t1, ix1(v), ix1(1)),
         1.0, ovw(tmpB_.p, ix1(o), ix1(1)), 16, 0, "Rp_ovov_t1");
    if (!merge_t1)
        gemm((int)(o2 * v), iv, io, -1.0,
             mv(tmpB_.p, ix3((uint32_t)o, (uint32_t)v, v * o, 1, o), ix1(o2 * v)), mv(t1, ix1(1), ix1(v)),
             1.0, ovw(Rp_.p, ix1(v), ix1(1)), 0, 0, "Rp_tmpB_t1");
    // - sum_k Z[i,j,k,a] t1[k,b], Z[i][j][k][a] = sum_cd (kd|ac) tau[i,j,c,d].  In pair form
    // (see the top of this function): Zs = V+ tau+^T over i >= j, c >= d and Za = V- tau-^T
    // over strict pairs, half of the plain 2 o^3 v^3; Z = unpack(Zs, Za).
    if (zpairs) {
        gemm((int)ov, (int)To, (int)Tv, 1.0, mv(Vzp_.p, ix1(Tv), ix1(1)), mv(taup_.p, ix1(Tv), ix1(1)), 0.0,
             ovw(Zs_.p, ix1(1), ix1(ov)), 17, -3, "Rp_Z_sym");
        if (anti)
            gemm((int)ov, (int)Tmo, (int)Tmv, 1.0, mv(Vzm_.p, ix1(Tmv), ix1(1)), mv(taum_.p, ix1(Tmv), ix1(1)),
                 0.0, ovw(Za_.p, ix1(1), ix1(ov)), 18, -4, "Rp_Z_anti");
        k_z_pair_unpack(io, iv, Zs_.p, anti ? Za_.p : nullptr, Z_.p, st_);
    } else {
        gemm((int)o2, (int)ov, (int)v2, 1.0, mv(tau, ix1(v2), ix1(1)),
             mv(ovvv_.p, ix2((uint32_t)v, v * v2, v), ix2((uint32_t)v, 1, v2)), 0.0,
             ovw(Z_.p, ix1(ov), ix1(1)), -1, 12, "Rp_Z");
    }
    if (r1_from_z) k_r1_from_z(io, iv, Z_.p, R1_.p, st_);
    if (merge_t1) {
        // S[i][j][a][k] = tmpB[k][i][a][j] + Z[i][j][k][a] + Vk[k][j][a][i]; Rp -= S t1
        S3_.ensure((size_t)o2 * ov);
        k_t1_terms(io, iv, tmpB_.p, Z_.p, Vk_.p, S3_.p, st_);
        gemm((int)(o2 * v), iv, io, -1.0, mv(S3_.p, ix1(o), ix1(1)), mv(t1, ix1(1), ix1(v)), 1.0,
             ovw(Rp_.p, ix1(v), ix1(1)), 0, 0, "Rp_t1_o3v");
    } else {
        gemm((int)(o2 * v), iv, io, -1.0, mv(Z_.p, ix2((uint32_t)v, ov, 1), ix1(v)), mv(t1, ix1(1), ix1(v)),
             1.0, ovw(Rp_.p, ix1(v), ix1(1)), 0, 0, "Rp_Z_t1");
    }
    // + sum_c Lvv'[a,c] t2[i,j,c,b]: M = a, N = (i,j,b), K = c
    gemm(iv, (int)(o2 * v), iv, 1.0, mv(Lvv_.p, ix1(v), ix1(1)),
         mv(t2, ix2((uint32_t)v, v2, 1), ix1(v)), 1.0, ovw(Rp_.p, ix1(v), ix2((uint32_t)v, v2, 1)), 0, 0, "Rp_Lvv");
    // - sum_k Loo'[k,i] t2[k,j,a,b]: M = i, N = (j,a,b), K = k.  The memory-optimised
    // map reads Loo' transposed here, Loo'[i,k] (ccsd_memory_optimized.cpp:2085-2086)
    const bool fik = opt_.variant == CCSD_VARIANT_MEMORY_OPTIMIZED;
    gemm(io, (int)ov2, io, -1.0, fik ? mv(Loo_.p, ix1(o), ix1(1)) : mv(Loo_.p, ix1(1), ix1(o)),
         mv(t2, ix1(1), ix1(ov2)), 1.0, ovw(Rp_.p, ix1(ov2), ix1(1)), 0, 0, "Rp_Loo");
    // rings, M = (i,a), N = (j,b), K = (k,c)
    // + sum_kc Wa[i,a,k,c] t2[k,j,c,b].  With symmetric amplitudes t2[k,j,c,b] = t2[j,k,b,c]:
    // the view of site Wvoov_t2 (key -7), read along c, whose split is reused here
    gemm((int)ov, (int)ov, (int)ov, 1.0, mv(Wa_.p, ix1(ov), ix1(1)),
         sym_amps ? mv(t2, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1))
                  : mv(t2, ix2((uint32_t)v, v2, 1), ix2((uint32_t)v, ov2, v)),
         1.0, ovw(Rp_.p, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1)), 0, sym_amps ? -7 : 0, "ring1");
    // - sum_kc Wvoov[i,a,k,c] t2[k,j,b,c]
    gemm((int)ov, (int)ov, (int)ov, -1.0, mv(Wvoov_.p, ix1(ov), ix1(1)),
         mv(t2, ix2((uint32_t)v, v2, v), ix2((uint32_t)v, ov2, 1)), 1.0,
         ovw(Rp_.p, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1)), 0, -2, "ring2");
    // - sum_kc Wvovo[i,b,k,c] t2[k,j,a,c]: M = (i,b), N = (j,a)
    gemm((int)ov, (int)ov, (int)ov, -1.0, mv(Wvovo_.p, ix1(ov), ix1(1)),
         mv(t2, ix2((uint32_t)v, v2, v), ix2((uint32_t)v, ov2, 1)), 1.0,
         ovw(Rp_.p, ix2((uint32_t)v, ov2, 1), ix2((uint32_t)v, v2, v)), 0, -2, "ring3");
}

double Engine::reduce_sum(int nparts) {
    k_sum(nparts, partials_.p, scalars_.p, st_);
    double h = 0.0;
    CCSD_CUDA(cudaMemcpyAsync(&h, scalars_.p, sizeof(double), cudaMemcpyDeviceToHost, st_));
    CCSD_CUDA(cudaStreamSynchronize(st_));
    return h;
}

// E = sum_ijab [2(ia|jb) - (ib|ja)] tau_ij^ab  (ccsd_memory_optimized.cpp:592-648,
// without the f_ia t_i^a term, :646)
double Engine::energy_of(const double *t1, const double *t2) {
    k_tau_dot(o_, v_, t1, t2, Lijab_.p, tau_.p, partials_.p, reduce_blocks(), st_);
    tau_fresh_ = t1 == t1_.p && t2 == t2_.p;
    return reduce_sum(reduce_blocks());
}

// Pulay DIIS on the amplitude vector (t1, t2) with errors T_new - T_old.
// No counterpart in the reference CCSD; the reference's SCF DIIS
// (hartree_fock_solver.cpp:1252-1311) builds B_ij = <e_i, e_j> and solves the
// bordered system the same way.  A singular system keeps the plain step.
// DIIS, first half (no host synchronisation): T_new and E = T_new - T_old go to the
// next slot, and the overlaps <E, E_j> with every stored slot j (slot order, E itself
// included) are launched into dots_dev.  Returns their count.
int Engine::diis_store_async(double *dots_dev) {
    const int m = opt_.diis_size;
    const size_t nT1 = (size_t)o_ * v_, nT2 = nT1 * o_ * v_, len = nT1 + nT2;
    if ((int)diis_t_.size() != m) {
        diis_t_.clear();
        diis_e_.clear();
        for (int i = 0; i < m; ++i) {
            diis_t_.emplace_back(len);
            diis_e_.emplace_back(len);
        }
        diis_b_.assign((size_t)m * m, 0.0);
        diis_count_ = 0;
        diis_next_ = 0;
    }
    const int slot = diis_next_;
    DBuf &T = diis_t_[slot], &E = diis_e_[slot];
    diis_slot_ = slot;
    diis_next_ = (diis_next_ + 1) % m;
    diis_count_ = std::min(diis_count_ + 1, m);
    // one pass: T = x_new, E = x_new - x_old and <E, E_j> for every stored slot j (E itself as NULL)
    std::vector<const double *> others;
    for (int j = 0; j < diis_count_; ++j) others.push_back(j == slot ? nullptr : diis_e_[j].p);
    const int nb = reduce_blocks();
    diis_partials_.ensure((size_t)m * nb);
    k_diis_store(nT1, nT2, t1n_.p, t2n_.p, t1_.p, t2_.p, T.p, E.p, others.data(), (int)others.size(),
                 diis_partials_.p, nb, st_);
    k_multi_sum((int)others.size(), nb, diis_partials_.p, dots_dev, st_);
    return (int)others.size();
}

void Engine::diis_step(int update_index) {
    const int m = opt_.diis_size;
    if (m <= 0) return;
    if (scalars_.n < (size_t)m) scalars_.alloc(std::max<size_t>(m, 8));
    const int nd = diis_store_async(scalars_.p);
    std::vector<double> dots(nd);
    CCSD_CUDA(cudaMemcpyAsync(dots.data(), scalars_.p, sizeof(double) * nd, cudaMemcpyDeviceToHost, st_));
    CCSD_CUDA(cudaStreamSynchronize(st_));
    diis_finish(update_index, dots.data());
}

// DIIS, second half, with the overlaps of diis_store_async on the host: the B matrix,
// the bordered solve and the extrapolation into (t1n, t2n).
void Engine::diis_finish(int update_index, const double *dots) {
    const int m = opt_.diis_size;
    const size_t nT1 = (size_t)o_ * v_, nT2 = nT1 * o_ * v_;
    const int slot = diis_slot_;
    for (int j = 0; j < diis_count_; ++j) {
        diis_b_[(size_t)slot * m + j] = dots[j];
        diis_b_[(size_t)j * m + slot] = dots[j];
    }
    diis_self_ = diis_b_[(size_t)slot * m + slot];
    if (diis_count_ < 2 || update_index < opt_.diis_start) return;
    // bordered system [B -1; -1 0] [c; lam] = [0; -1], scaled for conditioning
    const int k = diis_count_;
    std::vector<int> idx;
    for (int j = 0; j < m && (int)idx.size() < k; ++j) idx.push_back(j);
    const int nn = k + 1;
    std::vector<double> A((size_t)nn * nn, 0.0), rhs(nn, 0.0);
    double scale = 0.0;
    for (int a = 0; a < k; ++a) scale = std::max(scale, std::fabs(diis_b_[(size_t)idx[a] * m + idx[a]]));
    if (!(scale > 0.0) || !std::isfinite(scale)) return;
    for (int a = 0; a < k; ++a) {
        for (int b = 0; b < k; ++b) A[(size_t)a * nn + b] = diis_b_[(size_t)idx[a] * m + idx[b]] / scale;
        A[(size_t)a * nn + k] = -1.0;
        A[(size_t)k * nn + a] = -1.0;
    }
    rhs[k] = -1.0;
    // Gaussian elimination with partial pivoting
    for (int c = 0; c < nn; ++c) {
        int piv = c;
        for (int r = c + 1; r < nn; ++r)
            if (std::fabs(A[(size_t)r * nn + c]) > std::fabs(A[(size_t)piv * nn + c])) piv = r;
        if (std::fabs(A[(size_t)piv * nn + c]) < 1e-14) return;  // singular: keep the Jacobi step
        if (piv != c) {
            for (int q = 0; q < nn; ++q) std::swap(A[(size_t)c * nn + q], A[(size_t)piv * nn + q]);
            std::swap(rhs[c], rhs[piv]);
        }
        for (int r = c + 1; r < nn; ++r) {
            double f = A[(size_t)r * nn + c] / A[(size_t)c * nn + c];
            for (int q = c; q < nn; ++q) A[(size_t)r * nn + q] -= f * A[(size_t)c * nn + q];
            rhs[r] -= f * rhs[c];
        }
    }
    std::vector<double> x(nn);
    for (int r = nn - 1; r >= 0; --r) {
        double s = rhs[r];
        for (int q = r + 1; q < nn; ++q) s -= A[(size_t)r * nn + q] * x[q];
        x[r] = s / A[(size_t)r * nn + r];
    }
    for (int a = 0; a < k; ++a)
        if (!std::isfinite(x[a])) return;
    // T_new = sum_a c_a T_a, one pass over the stored vectors
    std::vector<const double *> vecs(k);
    for (int a = 0; a < k; ++a) vecs[a] = diis_t_[idx[a]].p;
    k_diis_combine(nT1, nT2, vecs.data(), x.data(), k, t1n_.p, t2n_.p, st_);
}

// ---------------------------------------------------------------------------
// One amplitude update up to the residual norm's partial sums: residual, (T3 terms,)
// T2 and T1 from the denominators.
void Engine::update_step() {
    residual();
    if (opt_.method != CCSD_METHOD_CCSD) triples_step();  // T3 terms, then T3 from this T2
    k_update_t2(o_, v_, R_.p, Rp_.p, eo_.p, ev_.p, dinv2_.p, t2_.p, t2n_.p, norm_in_diis_ ? nullptr : partials_.p,
                reduce_blocks(), st_);
    k_update_t1(o_, v_, R1_.p, eo_.p, ev_.p, t1_.p, t1n_.p, partials_.p + reduce_blocks(), st_);
}

// The same through a CUDA graph: captured the first time a parity of the amplitude
// buffers comes up, replayed afterwards.  Every pointer the update touches is fixed
// for a solve except the swapped t1/t2 buffers, hence one graph per parity.  A capture
// that fails leaves graphs off and runs the update directly.
void Engine::update_step_graph() {
    for (UpdateGraph &g : graphs_) {
        if (g.exec && g.t1 == t1_.p && g.t2 == t2_.p) {
            CCSD_CUDA(cudaGraphLaunch(g.exec, st_));
            note_launch((int)g.launches);
            return;
        }
    }
    UpdateGraph &g = graphs_[graphs_[0].exec ? 1 : 0];
    if (g.exec) {  // both parities taken by other buffers: start over
        release_graphs();
    }
    const long l0 = launch_count();
    if (cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        graphs_ok_ = false;
        update_step();
        return;
    }
    auto drop_capture = [&]() {
        cudaGraph_t gg = nullptr;
        cudaStreamEndCapture(st_, &gg);
        if (gg) cudaGraphDestroy(gg);
        cudaGetLastError();
        note_launch(-(int)(launch_count() - l0));  // captured launches that never ran
    };
    try {
        update_step();
    } catch (const CaptureMiss &) {
        // an operand buffer had to grow: nothing captured has run, so run the update
        // directly (it makes the allocation); the next update captures again
        drop_capture();
        update_step();
        return;
    } catch (...) {
        drop_capture();
        graphs_ok_ = false;
        throw;
    }
    cudaGraph_t gg = nullptr;
    cudaError_t e = cudaStreamEndCapture(st_, &gg);
    if (e == cudaSuccess && gg) e = cudaGraphInstantiate(&g.exec, gg, 0);
    if (gg) cudaGraphDestroy(gg);
    if (e != cudaSuccess || !g.exec) {  // not capturable here: run this and later updates directly
        cudaGetLastError();
        g.exec = nullptr;
        graphs_ok_ = false;
        update_step();
        return;
    }
    g.t1 = t1_.p;
    g.t2 = t2_.p;
    g.launches = launch_count() - l0;
    CCSD_CUDA(cudaGraphLaunch(g.exec, st_));
}

void Engine::release_graphs() {
    for (UpdateGraph &g : graphs_) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = UpdateGraph();
    }
}

void Engine::solve(ccsd_result *res) {
    const int o = o_, v = v_;
    const size_t nT1 = (size_t)o * v, nT2 = nT1 * o * v;
    // the DIIS vectors stay allocated between solves (2 m amplitude-sized
    // cudaMallocs cost tens of ms at the bench size); only the history restarts
    diis_count_ = diis_next_ = 0;
    std::fill(diis_b_.begin(), diis_b_.end(), 0.0);
    if (split_) split_->clear_error();  // a time-out of an earlier solve does not carry over
    prof_.clear();
    prof_pending_.clear();
    prof_update_ms_ = 0.0;
    prof_updates_ = 0;
    prof_launches_ = 0;
    // T1 = 0, T2 = MP2 (ccsd_memory_optimized.cpp:473-490), or the caller's amplitudes (a restart)
    if (opt_.t2_start) {
        CCSD_CUDA(cudaMemcpyAsync(t2_.p, opt_.t2_start, sizeof(double) * nT2, cudaMemcpyHostToDevice, st_));
        if (opt_.t1_start)
            CCSD_CUDA(cudaMemcpyAsync(t1_.p, opt_.t1_start, sizeof(double) * nT1, cudaMemcpyHostToDevice, st_));
        else
            t1_.zero(st_);
        CCSD_CUDA(cudaStreamSynchronize(st_));  // the host arrays may go away after the call
    } else {
        t1_.zero(st_);
        k_mp2_guess(o, v, ovov_.p, eo_.p, ev_.p, t2_.p, st_);
    }
    if (opt_.method != CCSD_METHOD_CCSD) triples_setup();  // T3 = 0
    tau_fresh_ = false;
    double e_new = energy_of(t1_.p, t2_.p);
    int hist = 0;
    if (res->energy_history && res->history_capacity > 0) res->energy_history[hist] = e_new;
    hist = 1;

    cudaEvent_t ev0, ev1;
    CCSD_CUDA(cudaEventCreate(&ev0));
    CCSD_CUDA(cudaEventCreate(&ev1));
    // from the second update on, the residual and amplitude update run as captured graphs
    // (CCSD on a private or user stream, the legacy default stream cannot be captured;
    // not while profiling, whose per-site events a graph cannot time)
    release_graphs();
    // with DIIS the residual norm is the store's <E, E> (E = T_new - T_old), so the T2 update
    // neither reads T_old nor sums it
    norm_in_diis_ = opt_.diis_size > 0 && dinv2_.p != nullptr && opt_.method == CCSD_METHOD_CCSD;
    const bool use_graphs = graphs_ok_ && opt_.method == CCSD_METHOD_CCSD && st_ != nullptr && tape_ == nullptr &&
                            !opt_.profile;
    int updates = 0;
    bool converged = false;
    const int cap = opt_.fixed_iterations > 0 ? opt_.fixed_iterations : std::max(opt_.max_iter, 1);
    try {
        while (true) {
            const double e_old = e_new;
            const long launches0 = launch_count();
            CCSD_CUDA(cudaEventRecord(ev0, st_));
            if (use_graphs && updates >= 1)
                update_step_graph();
            else
                update_step();
            // |T_new - T_old|^2: the DIIS store's <E, E> when DIIS runs, else the update's partials
            const double rn2 = norm_in_diis_ ? 0.0 : reduce_sum(reduce_blocks() + 1);
            diis_step(updates);
            last_resid_ = std::sqrt(std::max(norm_in_diis_ ? diis_self_ : rn2, 0.0));
            std::swap(t1_, t1n_);
            std::swap(t2_, t2n_);
            e_new = energy_of(t1_.p, t2_.p);
            CCSD_CUDA(cudaEventRecord(ev1, st_));
            CCSD_CUDA(cudaEventSynchronize(ev1));
            float ms = 0.f;
            CCSD_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
            if (opt_.profile) {
                prof_flush();
                prof_update_ms_ += ms;
                prof_updates_ += 1;
                prof_launches_ += launch_count() - launches0;
            }
            ++updates;
            if (res->update_ms && updates - 1 < res->history_capacity) res->update_ms[updates - 1] = ms;
            if (res->energy_history && hist < res->history_capacity) res->energy_history[hist] = e_new;
            ++hist;
            if (split_) {
                int st = split_->error_status();
                if (st) throw Error(CCSD_ERR_TIMEOUT, "split-precision kernel reported a bounded-wait timeout");
            }
            if (opt_.verbose)
                std::printf("ccsd update %3d  E_corr = %.15e  dE = %.3e  |dT| = %.3e  %.3f ms\n", updates,
                            e_new, e_new - e_old, last_resid_, ms);
            if (!std::isfinite(e_new) || !std::isfinite(last_resid_))
                throw Error(CCSD_ERR_DIVERGED, "amplitude iteration diverged (NaN/Inf)");
            if (opt_.fixed_iterations > 0) {
                if (updates >= opt_.fixed_iterations) break;
                continue;
            }
            bool ok = std::fabs(e_new - e_old) < opt_.energy_tol;
            if (opt_.residual_tol > 0.0) ok = ok && last_resid_ < opt_.residual_tol;
            if (ok) {
                converged = true;
                break;
            }
            if (updates >= cap) break;
        }
    } catch (...) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        release_graphs();
        throw;
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    release_graphs();
    solved_ = true;
    last_e_ = e_new;
    res->e_corr = e_new;
    res->residual_norm = last_resid_;
    res->iterations = updates;
    res->converged = converged ? 1 : 0;
    res->history_len = std::min(hist, std::max(res->history_capacity, 0));
    res->flops_per_update = ccsd_flops_per_update(o, v);
    if (res->t1) CCSD_CUDA(cudaMemcpyAsync(res->t1, t1_.p, nT1 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    if (res->t2) CCSD_CUDA(cudaMemcpyAsync(res->t2, t2_.p, nT2 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CCSD_CUDA(cudaStreamSynchronize(st_));
}

}  // namespace ccsd
