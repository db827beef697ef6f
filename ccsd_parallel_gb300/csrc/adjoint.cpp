// Reverse mode over the engine's own operations: the CCSD Lambda (adjoint)
// equations and dE_corr/d(inputs).
//
// No counterpart in the reference (it has no Lambda equations or gradients).
// With the residual G(T; theta) = R(T; theta) - D(theta) o T, where R is the
// Jacobi numerator of Engine::residual() and D the orbital-energy
// denominators, the Lagrangian E + Lambda^T G gives
//     Lambda = (dE/dT + J^T Lambda) / D,          J = dR/dT,
//     dE/dtheta = dE/dtheta|_T + Lambda^T dR/dtheta - Lambda^T (dD/dtheta o T).
// J^T Lambda and Lambda^T dR/dtheta are vector-Jacobian products obtained by
// replaying a recorded tape of the forward operations backwards: a
// contraction C += alpha A B^T gives  Abar += alpha Cbar B  and
// Bbar += alpha Cbar^T A, i.e. the same view-based contraction kernels with
// the row and column index groups exchanged (FP64 or split precision, as the
// forward pass).  Lambda is iterated like the amplitudes (Jacobi on D).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "engine.h"

namespace ccsd {

namespace {
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

// ---- recordable element-wise operations -----------------------------------------
void Engine::axpby(int R, int C, double alpha, const MatView &X, double beta, const OutView &Y) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::Axpby;
        op.M = R;
        op.N = C;
        op.alpha = alpha;
        op.beta = beta;
        op.A = X;
        op.C = Y;
        tape_->push_back(op);
        if (record_only_) return;
    }
    axpby_view(R, C, alpha, X, beta, Y, st_);
}

void Engine::copy(double *dst, const double *src, size_t n) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::Copy;
        op.M = (int)n;
        op.A = mv(src, ix1(0), ix1(1));
        op.C = ovw(dst, ix1(0), ix1(1));
        tape_->push_back(op);
        if (record_only_) return;
    }
    CCSD_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, st_));
}

void Engine::tau_op(const double *t1, const double *t2, double *tau) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::Tau;
        op.t1 = t1;
        op.t2 = t2;
        op.out1 = tau;
        tape_->push_back(op);
        if (record_only_) return;
    }
    k_tau(o_, v_, t1, t2, tau, st_);
}

void Engine::theta_op(const double *t1, const double *t2, double *th1, double *th2) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::Theta;
        op.t1 = t1;
        op.t2 = t2;
        op.out1 = th1;
        op.out2 = th2;
        tape_->push_back(op);
        if (record_only_) return;
    }
    k_theta(o_, v_, t1, t2, th1, th2, st_);
}

void Engine::tau_sym_op(const double *tau, double *tp, double *tm) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::TauSym;
        op.t1 = tau;
        op.out1 = tp;
        op.out2 = tm;
        tape_->push_back(op);
        if (record_only_) return;
    }
    k_tau_sym(o_, v_, tau, tp, tm, st_);
}

void Engine::unpack_op(const double *sp, const double *sm, double *R) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::Unpack;
        op.t1 = sp;
        op.t2 = sm;
        op.out1 = R;
        tape_->push_back(op);
        if (record_only_) return;
    }
    k_ladder_unpack(o_, v_, sp, sm, R, st_);
}

void Engine::w_sym_op(const double *W, double *wp, double *wm) {
    if (tape_) {
        TapeOp op;
        op.kind = TapeOp::WSym;
        op.t1 = W;
        op.out1 = wp;
        op.out2 = wm;
        tape_->push_back(op);
        if (record_only_) return;
    }
    k_w_sym(v_, W, wp, wm, st_);
}

// ---- adjoint storage ------------------------------------------------------------
double *Engine::adj_of(const double *p, bool *active) {
    if (!p) return nullptr;
    for (const Reg &r : regs_) {
        const DBuf *b = r.buf;
        if (b->p && p >= b->p && p < b->p + b->n) {
            if (active) *active = r.active;
            if (!full_adjoint_ && !r.active) return nullptr;
            DBuf &a = adj_[r.buf];
            if (!a.p || a.n != b->n) {
                a.alloc(b->n);
                a.zero(st_);
            }
            return a.p + (p - b->p);
        }
    }
    return nullptr;  // not registered: a constant
}

void Engine::zero_adjoints() {
    for (auto &kv : adj_) kv.second.zero(st_);
}

// ---- the backward sweep -----------------------------------------------------------
void Engine::reverse(const std::vector<TapeOp> &tape) {
    const int64_t o = o_, v = v_, ov = o * v, v2 = v * v, ov2 = o * v2;
    const size_t nT2 = (size_t)(o * o * v * v);
    const size_t pair_o = (size_t)(o * (o + 1) / 2), spair_o = (size_t)(o * (o - 1) / 2);
    const size_t pair_v = (size_t)(v * (v + 1) / 2), spair_v = (size_t)(v * (v - 1) / 2);
    auto scale = [&](int R, int C, double beta, const OutView &Y) {  // Ybar_old = beta Ybar
        if (beta == 1.0) return;
        axpby_view(R, C, 0.0, mv(Y.p, Y.row, Y.col), beta, Y, st_);
    };
    for (auto it = tape.rbegin(); it != tape.rend(); ++it) {
        const TapeOp &op = *it;
        switch (op.kind) {
            case TapeOp::Gemm: {
                double *Cb = adj_of(op.C.p);
                if (!Cb) break;
                // The operand held fixed in each product (integrals, or amplitudes at the
                // solution) does not change during the Lambda iteration: its transposed view
                // is split once and cached under a key of its own (key +- 1000).
                auto tkey = [](int k) { return k > 0 ? k + 1000 : (k < 0 ? k - 1000 : 0); };
                if (double *Ab = adj_of(op.A.p))  // Abar(m,k) += alpha sum_n Cbar(m,n) B(n,k)
                    gemm(op.M, op.K, op.N, op.alpha, mv(Cb, op.C.row, op.C.col), mv(op.B.p, op.B.col, op.B.row),
                         1.0, ovw(Ab, op.A.row, op.A.col), 0, tkey(op.key_b));
                if (double *Bb = adj_of(op.B.p))  // Bbar(n,k) += alpha sum_m Cbar(m,n) A(m,k)
                    gemm(op.N, op.K, op.M, op.alpha, mv(Cb, op.C.col, op.C.row), mv(op.A.p, op.A.col, op.A.row),
                         1.0, ovw(Bb, op.B.row, op.B.col), 0, tkey(op.key_a));
                scale(op.M, op.N, op.beta, ovw(Cb, op.C.row, op.C.col));
                break;
            }
            case TapeOp::Axpby:
            case TapeOp::Copy: {
                const int R = op.kind == TapeOp::Copy ? 1 : op.M;
                const int Cn = op.kind == TapeOp::Copy ? op.M : op.N;
                const double alpha = op.kind == TapeOp::Copy ? 1.0 : op.alpha;
                const double beta = op.kind == TapeOp::Copy ? 0.0 : op.beta;
                double *Yb = adj_of(op.C.p);
                if (!Yb) break;
                if (double *Xb = adj_of(op.A.p))
                    axpby_view(R, Cn, alpha, mv(Yb, op.C.row, op.C.col), 1.0, ovw(Xb, op.A.row, op.A.col), st_);
                scale(R, Cn, beta, ovw(Yb, op.C.row, op.C.col));
                break;
            }
            case TapeOp::Tau: {  // tau[i,j,a,b] = t2[i,j,a,b] + t1[i,a] t1[j,b]
                double *Tb = adj_of(op.out1);
                if (!Tb) break;
                if (double *t2b = adj_of(op.t2))
                    axpby_view(1, (int)nT2, 1.0, mv(Tb, ix1(0), ix1(1)), 1.0, ovw(t2b, ix1(0), ix1(1)), st_);
                if (double *t1b = adj_of(op.t1)) {
                    // t1bar[i,a] += sum_jb taubar[i,j,a,b] t1[j,b] + sum_jb taubar[j,i,b,a] t1[j,b]
                    gemm((int)ov, 1, (int)ov, 1.0, mv(Tb, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1)),
                         mv(op.t1, ix1(0), ix1(1)), 1.0, ovw(t1b, ix1(1), ix1(0)));
                    gemm((int)ov, 1, (int)ov, 1.0, mv(Tb, ix2((uint32_t)v, v2, 1), ix2((uint32_t)v, ov2, v)),
                         mv(op.t1, ix1(0), ix1(1)), 1.0, ovw(t1b, ix1(1), ix1(0)));
                }
                axpby_view(1, (int)nT2, 0.0, mv(Tb, ix1(0), ix1(1)), 0.0, ovw(Tb, ix1(0), ix1(1)), st_);
                break;
            }
            case TapeOp::Theta: {
                // th1[i,a,l,d] = t2[i,l,a,d] - t2[i,l,d,a]/2 - t1[i,d] t1[l,a]
                // th2[i,a,l,d] = t2[i,l,d,a]/2 + t1[i,d] t1[l,a]
                double *h1 = adj_of(op.out1), *h2 = adj_of(op.out2);
                if (!h1 && !h2) break;
                qtmp_.ensure(nT2);
                double *Q = qtmp_.p;  // Q = th2bar - th1bar
                CCSD_CUDA(cudaMemsetAsync(Q, 0, nT2 * sizeof(double), st_));
                if (h2) axpby_view(1, (int)nT2, 1.0, mv(h2, ix1(0), ix1(1)), 1.0, ovw(Q, ix1(0), ix1(1)), st_);
                if (h1) axpby_view(1, (int)nT2, -1.0, mv(h1, ix1(0), ix1(1)), 1.0, ovw(Q, ix1(0), ix1(1)), st_);
                if (double *t2b = adj_of(op.t2)) {
                    if (h1)  // t2bar[i,l,a,d] += th1bar[i,a,l,d]
                        axpby_view((int)ov, (int)ov, 1.0, mv(h1, ix1(ov), ix1(1)), 1.0,
                                   ovw(t2b, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1)), st_);
                    // t2bar[i,l,d,a] += Q[i,a,l,d] / 2
                    axpby_view((int)ov, (int)ov, 0.5, mv(Q, ix1(ov), ix1(1)), 1.0,
                               ovw(t2b, ix2((uint32_t)v, ov2, 1), ix2((uint32_t)v, v2, v)), st_);
                }
                if (double *t1b = adj_of(op.t1)) {
                    // t1bar[i,d] += sum_la Q[i,a,l,d] t1[l,a]; t1bar[l,a] += sum_id Q[i,a,l,d] t1[i,d]
                    gemm((int)ov, 1, (int)ov, 1.0,
                         mv(Q, ix2((uint32_t)v, v * o * v, 1), ix2((uint32_t)v, v, ov)), mv(op.t1, ix1(0), ix1(1)),
                         1.0, ovw(t1b, ix1(1), ix1(0)));
                    gemm((int)ov, 1, (int)ov, 1.0,
                         mv(Q, ix2((uint32_t)v, v, ov), ix2((uint32_t)v, v * o * v, 1)), mv(op.t1, ix1(0), ix1(1)),
                         1.0, ovw(t1b, ix1(1), ix1(0)));
                }
                if (h1) CCSD_CUDA(cudaMemsetAsync(h1, 0, nT2 * sizeof(double), st_));
                if (h2) CCSD_CUDA(cudaMemsetAsync(h2, 0, nT2 * sizeof(double), st_));
                break;
            }
            case TapeOp::TauSym: {  // (tau+, tau-) = P(tau): taubar += P^T (tau+bar, tau-bar)
                double *pb = adj_of(op.out1), *mb = adj_of(op.out2);
                if (!pb) break;
                if (double *tb = adj_of(op.t1)) k_tau_sym_adj((int)o, (int)v, pb, mb, tb, st_);
                CCSD_CUDA(cudaMemsetAsync(pb, 0, sizeof(double) * pair_o * pair_v, st_));
                if (mb) CCSD_CUDA(cudaMemsetAsync(mb, 0, sizeof(double) * spair_o * spair_v, st_));
                break;
            }
            case TapeOp::Unpack: {  // R += U(S+, S-): (S+bar, S-bar) += U^T Rbar; Rbar unchanged
                double *Rb = adj_of(op.out1);
                if (!Rb) break;
                double *pb = adj_of(op.t1), *mb = adj_of(op.t2);
                if (pb) k_ladder_unpack_adj((int)o, (int)v, Rb, pb, mb, st_);
                break;
            }
            case TapeOp::WSym: {  // (W+, W-) = Q(W): Wbar += Q^T (W+bar, W-bar)
                double *pb = adj_of(op.out1), *mb = adj_of(op.out2);
                if (!pb) break;
                if (double *Wb = adj_of(op.t1)) k_w_sym_adj((int)v, pb, mb, Wb, st_);
                CCSD_CUDA(cudaMemsetAsync(pb, 0, sizeof(double) * pair_v * pair_v, st_));
                if (mb) CCSD_CUDA(cudaMemsetAsync(mb, 0, sizeof(double) * spair_v * spair_v, st_));
                break;
            }
        }
    }
}

// ---- the ladder's dE/dB for density-fitted inputs --------------------------------------
// The ladder reads W[a][b][c][d] = (ac|bd) = sum_Q B[Q][a][c] B[Q][b][d] (virtual
// indices, offset o) through its pair forms, i.e. the plain ladder on the
// symmetrised inputs W_s and P tau.  With Rbar = Lambda2 (the adjoint of R at the
// ladder), its contribution to dE/dB is
//   Bbar[Q][x][y] += sum_{ij,b,d} Lh[ij][x][b] B[Q][b][d] (P tau)[ij][y][d],
//   Lh[ij][x][b] = l2[ij][x][b] + l2[ji][b][x],  (P tau)[ij][y][d] = (tau[ijyd] + tau[jidy]) / 2,
// evaluated as two contractions per block of Q, so neither (ac|bd), W+- nor
// their adjoints (v^4 each) are formed.  Lh and P tau are split once per call
// (per-update cache keys, dropped at the next residual).
void Engine::ladder_df_grad(const double *lam2, int naux) {
    // B[Q][p][q] over the nt_ input orbitals, the active ones from nf_ on
    const int64_t o = o_, v = v_, n = nt_, o2 = o * o, v2 = v * v, nn = n * n, f0 = (int64_t)nf_ * n + nf_;
    double *Bb = adj_of(input_df_ ? input_df_->p : nullptr);
    if (!Bb) return;
    Bb += f0;
    const double *B = input_df_->p + f0;
    DBuf lh((size_t)(o2 * v2)), pt((size_t)(o2 * v2));
    // element (i,j | x,b) of a [j][i][b][x] read: row (i,j) strides (v2, o v2), column (x,b) strides (1, v)
    const MatView lt = mv(lam2, ix2((uint32_t)o, v2, o * v2), ix2((uint32_t)v, 1, v));
    axpby_view((int)o2, (int)v2, 1.0, mv(lam2, ix1(v2), ix1(1)), 0.0, ovw(lh.p, ix1(v2), ix1(1)), st_);
    axpby_view((int)o2, (int)v2, 1.0, lt, 1.0, ovw(lh.p, ix1(v2), ix1(1)), st_);
    const MatView tt = mv(tau_.p, ix2((uint32_t)o, v2, o * v2), ix2((uint32_t)v, 1, v));
    axpby_view((int)o2, (int)v2, 0.5, mv(tau_.p, ix1(v2), ix1(1)), 0.0, ovw(pt.p, ix1(v2), ix1(1)), st_);
    axpby_view((int)o2, (int)v2, 0.5, tt, 1.0, ovw(pt.p, ix1(v2), ix1(1)), st_);
    // Q blocks so that U = Lh B stays near 2 GB
    const int64_t per_q = o2 * v2;
    const int qc_max = (int)std::max<int64_t>(1, std::min<int64_t>(naux, (int64_t)(2.0e9 / 8.0) / per_q));
    DBuf U((size_t)(per_q * qc_max));
    const double *Bvv = B + o * n + o;
    double *Bbvv = Bb + o * n + o;
    for (int q0 = 0; q0 < naux; q0 += qc_max) {
        const int64_t qc = std::min<int64_t>(qc_max, naux - q0);
        // U[(ij,x)][(Q,d)] = sum_b Lh[ij][x][b] B[q0+Q][b][d]
        gemm((int)(o2 * v), (int)(qc * v), (int)v, 1.0, mv(lh.p, ix1(v), ix1(1)),
             mv(Bvv + q0 * nn, ix2((uint32_t)v, nn, 1), ix1(n)), 0.0, ovw(U.p, ix1(qc * v), ix1(1)), -1101, 0);
        // Bbar[q0+Q][x][y] += sum_{ij,d} U[(ij,x)][(Q,d)] (P tau)[ij][y][d]
        gemm((int)(qc * v), (int)v, (int)(o2 * v), 1.0,
             mv(U.p, ix2((uint32_t)v, v, qc * v), ix2((uint32_t)v, v * qc * v, 1)),
             mv(pt.p, ix1(v), ix2((uint32_t)v, v2, 1)), 1.0, ovw(Bbvv + q0 * nn, ix2((uint32_t)v, nn, n), ix1(1)),
             0, -1102);
    }
}

// ---- Lambda equations and the gradient ----------------------------------------------
void Engine::lambda_grad(const ccsd_problem &prob, ccsd_grad *out) {
    if (!solved_) throw Error(CCSD_ERR_INVALID_ARG, "ccsd_lambda_grad needs a completed ccsd_solve first");
    if (opt_.method != CCSD_METHOD_CCSD)
        throw Error(CCSD_ERR_UNSUPPORTED, "ccsd_lambda_grad is built for CCSD (method CCSD_METHOD_CCSD)");
    if (prob.nocc != o_ || prob.nvir != v_ || prob.nfrozen != nf_)
        throw Error(CCSD_ERR_INVALID_ARG, "problem shape differs from the handle's");
    const int o = o_, v = v_;
    const int64_t ov = (int64_t)o * v, v2 = (int64_t)v * v, ov2 = (int64_t)o * v2, o2 = (int64_t)o * o;
    const size_t nT1 = (size_t)ov, nT2 = (size_t)(o2 * v2);

    struct Cleanup {
        Engine *e;
        ~Cleanup() {
            e->tape_ = nullptr;
            e->full_adjoint_ = false;
            e->adj_.clear();
            e->regs_.clear();
            e->keep_.clear();
            e->build_split_.reset();
            e->wv_.alloc(0);  // (ac|bd) was rebuilt for the recorded build only
            e->grad_lean_vvvv_ = false;
        }
    } cleanup{this};

    regs_.clear();
    adj_.clear();
    for (DBuf *b : {&t1_, &t2_, &tau_, &th1_, &th2_, &R1_, &R_, &Rp_, &Foo_, &Fvv_, &Fov_, &Loo_, &Lvv_, &tmpo_,
                    &tmpo2_, &Woooo_, &Wvoov_, &Wvovo_, &Wa_, &Z_, &tmpB_, &Vk_, &taup_, &taum_, &Sp_, &Sm_})
        reg(*b, true);
    // DF inputs: the ladder's dE/dB comes from ladder_df_grad, so (ac|bd) and W+- get
    // no adjoints (at large nvir they would not fit next to the forward tensors)
    const bool lean = prob.integral_kind == CCSD_INTS_DF;
    for (DBuf *b : {&ovov_, &oovv_, &ovoo_, &oooo_, &ovvv_, &Lovov_, &Lovoo_, &Lovvv_, &LT1_, &Lijab_, &f_oo_off_,
                    &f_vv_off_, &f_ov_})
        reg(*b, false);
    if (!lean)
        for (DBuf *b : {&wv_, &Wp_, &Wm_}) reg(*b, false);

    // 1. record the integral build again (the inputs are re-read), then one residual at the solution
    std::vector<TapeOp> build_tape, res_tape;
    input_eri_ = input_df_ = input_c_ = nullptr;
    tape_ = &build_tape;
    if (opt_.precision != CCSD_PREC_FP64) build_split_.reset(new SplitEngine(CCSD_PREC_SPLIT4, st_));
    grad_lean_vvvv_ = lean;
    build_integrals(prob);
    build_derived();
    grad_lean_vvvv_ = false;
    tape_ = nullptr;
    CCSD_CUDA(cudaStreamSynchronize(st_));
    if (build_split_ && build_split_->error_status())
        throw Error(CCSD_ERR_TIMEOUT, "split-precision kernel of the integral build reported a bounded-wait timeout");
    build_split_.reset();
    for (auto &b : keep_) reg(*b, false);
    tape_ = &res_tape;
    residual();
    tape_ = nullptr;

    // 2. dE/dT for E = sum_ijab Lijab tau_ijab: e2 = Lijab, e1[i,a] = 2 sum_jb Lijab[i,j,a,b] t1[j,b]
    DBuf e1(nT1), e2(nT2), l1(nT1), l2(nT2), l1n(nT1), l2n(nT2), r1(nT1), r2(nT2), zero2(nT2);
    CCSD_CUDA(cudaMemcpyAsync(e2.p, Lijab_.p, nT2 * sizeof(double), cudaMemcpyDeviceToDevice, st_));
    gemm_f64((int)ov, 1, (int)ov, 2.0, mv(Lijab_.p, ix2((uint32_t)v, ov2, v), ix2((uint32_t)v, v2, 1)),
             mv(t1_.p, ix1(0), ix1(1)), 0.0, ovw(e1.p, ix1(1), ix1(0)), ws_.p, ws_.n, st_);
    l1.zero(st_);
    l2.zero(st_);
    zero2.zero(st_);

    auto seed = [&](const DBuf &lam1, const DBuf &lam2) {
        zero_adjoints();
        double *R1b = adj_of(R1_.p), *Rb = adj_of(R_.p), *Rpb = adj_of(Rp_.p);
        CCSD_CUDA(cudaMemcpyAsync(R1b, lam1.p, nT1 * sizeof(double), cudaMemcpyDeviceToDevice, st_));
        CCSD_CUDA(cudaMemcpyAsync(Rb, lam2.p, nT2 * sizeof(double), cudaMemcpyDeviceToDevice, st_));
        // R2 = R + Rp + Rp[j,i,b,a]  =>  Rpbar = l2 + l2[j,i,b,a]
        axpby_view((int)o2, (int)v2, 1.0, mv(lam2.p, ix1(v2), ix1(1)), 0.0, ovw(Rpb, ix1(v2), ix1(1)), st_);
        axpby_view((int)o2, (int)v2, 1.0, mv(lam2.p, ix2((uint32_t)o, v2, ov2), ix2((uint32_t)v, 1, v)), 1.0,
                   ovw(Rpb, ix1(v2), ix1(1)), st_);
    };

    // 3. Lambda = (dE/dT + J^T Lambda) / D (amplitude adjoints only)
    full_adjoint_ = false;
    const double tol = out->tol > 0.0 ? out->tol : 1e-10;
    const int max_iter = out->max_iter > 0 ? out->max_iter : 500;
    int it = 0;
    double resid = 0.0;
    for (; it < max_iter;) {
        seed(l1, l2);
        reverse(res_tape);
        const double *t1b = adj_of(t1_.p), *t2b = adj_of(t2_.p);
        CCSD_CUDA(cudaMemcpyAsync(r1.p, e1.p, nT1 * sizeof(double), cudaMemcpyDeviceToDevice, st_));
        CCSD_CUDA(cudaMemcpyAsync(r2.p, e2.p, nT2 * sizeof(double), cudaMemcpyDeviceToDevice, st_));
        axpby_view(1, (int)nT1, 1.0, mv(t1b, ix1(0), ix1(1)), 1.0, ovw(r1.p, ix1(0), ix1(1)), st_);
        axpby_view(1, (int)nT2, 1.0, mv(t2b, ix1(0), ix1(1)), 1.0, ovw(r2.p, ix1(0), ix1(1)), st_);
        k_update_t2(o, v, r2.p, zero2.p, eo_.p, ev_.p, dinv2_.p, l2.p, l2n.p, partials_.p, reduce_blocks(), st_);
        // r2 alone (Rp = 0, so Rp^T adds 0): l2n = r2 / D2
        k_update_t1(o, v, r1.p, eo_.p, ev_.p, l1.p, l1n.p, partials_.p + reduce_blocks(), st_);
        resid = std::sqrt(std::max(reduce_sum(reduce_blocks() + 1), 0.0));
        std::swap(l1, l1n);
        std::swap(l2, l2n);
        ++it;
        if (!std::isfinite(resid)) throw Error(CCSD_ERR_DIVERGED, "Lambda iteration diverged (NaN/Inf)");
        if (resid < tol) break;
    }

    // 4. full adjoint: Lambda^T dR/dtheta, plus dE/dtheta through Lijab, back through the build
    full_adjoint_ = true;
    seed(l1, l2);
    reverse(res_tape);
    {
        double *Lb = adj_of(Lijab_.p);
        axpby_view(1, (int)nT2, 1.0, mv(tau_.p, ix1(0), ix1(1)), 1.0, ovw(Lb, ix1(0), ix1(1)), st_);
    }
    reverse(build_tape);
    if (lean) ladder_df_grad(l2.p, prob.naux);
    CCSD_CUDA(cudaStreamSynchronize(st_));

    // 5. host assembly: the denominator term and the Fock matrix
    std::vector<double> hl1(nT1), hl2(nT2), ht1(nT1), ht2(nT2);
    CCSD_CUDA(cudaMemcpy(hl1.data(), l1.p, nT1 * sizeof(double), cudaMemcpyDeviceToHost));
    CCSD_CUDA(cudaMemcpy(hl2.data(), l2.p, nT2 * sizeof(double), cudaMemcpyDeviceToHost));
    CCSD_CUDA(cudaMemcpy(ht1.data(), t1_.p, nT1 * sizeof(double), cudaMemcpyDeviceToHost));
    CCSD_CUDA(cudaMemcpy(ht2.data(), t2_.p, nT2 * sizeof(double), cudaMemcpyDeviceToHost));
    const int n = nt_, nf = nf_;  // d_fock covers the input's nt_ orbitals; frozen rows stay 0
    if (out->d_fock) {
        std::vector<double> deo(o, 0.0), dev(v, 0.0);
        for (int i = 0; i < o; ++i)
            for (int a = 0; a < v; ++a) {
                const double x = hl1[i * v + a] * ht1[i * v + a];
                deo[i] -= x;
                dev[a] += x;
            }
        for (int i = 0; i < o; ++i)
            for (int j = 0; j < o; ++j)
                for (int a = 0; a < v; ++a)
                    for (int b = 0; b < v; ++b) {
                        const size_t k = (((size_t)i * o + j) * v + a) * v + b;
                        const double x = hl2[k] * ht2[k];
                        deo[i] -= x;
                        deo[j] -= x;
                        dev[a] += x;
                        dev[b] += x;
                    }
        std::vector<double> foo((size_t)o * o), fvv((size_t)v * v), fov((size_t)o * v);
        CCSD_CUDA(cudaMemcpy(foo.data(), adj_of(f_oo_off_.p), foo.size() * sizeof(double), cudaMemcpyDeviceToHost));
        CCSD_CUDA(cudaMemcpy(fvv.data(), adj_of(f_vv_off_.p), fvv.size() * sizeof(double), cudaMemcpyDeviceToHost));
        CCSD_CUDA(cudaMemcpy(fov.data(), adj_of(f_ov_.p), fov.size() * sizeof(double), cudaMemcpyDeviceToHost));
        double *F = out->d_fock;
        std::memset(F, 0, sizeof(double) * n * n);
        auto at = [&](int p, int q) -> double & { return F[(size_t)(nf + p) * n + nf + q]; };
        for (int i = 0; i < o; ++i)
            for (int j = 0; j < o; ++j) at(i, j) = i == j ? deo[i] : foo[i * o + j];
        for (int a = 0; a < v; ++a)
            for (int b = 0; b < v; ++b) at(o + a, o + b) = a == b ? dev[a] : fvv[a * v + b];
        for (int i = 0; i < o; ++i)
            for (int a = 0; a < v; ++a) at(i, o + a) = fov[i * v + a];
    }
    auto fetch = [&](double *dst, DBuf *src) {
        if (!dst) return;
        if (!src) throw Error(CCSD_ERR_INVALID_ARG, "requested gradient does not match the integral input form");
        double *a = adj_of(src->p);
        CCSD_CUDA(cudaMemcpy(dst, a, src->n * sizeof(double), cudaMemcpyDeviceToHost));
    };
    if (split_ && split_->error_status())
        throw Error(CCSD_ERR_TIMEOUT, "split-precision kernel of the Lambda sweep reported a bounded-wait timeout");
    fetch(out->d_eri, input_eri_);
    fetch(out->d_df, input_df_);
    fetch(out->d_mo_coeff, input_c_);
    if (out->lambda1) std::memcpy(out->lambda1, hl1.data(), nT1 * sizeof(double));
    if (out->lambda2) std::memcpy(out->lambda2, hl2.data(), nT2 * sizeof(double));
    out->iterations = it;
    out->residual_norm = resid;
    out->e_corr = last_e_;
}

}  // namespace ccsd
