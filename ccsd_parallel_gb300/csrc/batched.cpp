// Batched solve (batched.h).
//
// No counterpart in the reference, which solves one molecule per process.
// Every system keeps its own Engine (integral blocks, amplitudes,
// intermediates).  The residual of each engine is recorded once as a tape of
// operations (the same recording the gradient uses, without running it); the
// tapes of all systems have the same sequence of operations, so operation k
// of every tape becomes ONE grouped launch over the batch:
//   - contractions: the persistent grouped FP64 kernel (grouped.cu) whose
//     tile shape and split-K target are picked per operation by timing the
//     candidates on the batch's own shapes (autotuner, cached per process);
//   - element-wise operations: grouped kernels with the system in blockIdx.y.
// One update = graph 1 (residual + Jacobi update + |dT|) and graph 2 (copy of
// the new amplitudes + energy); DIIS, when enabled, runs per system between
// the two.  Systems that stop (converged, capped, diverged) are masked off
// on the device, so each keeps exactly the iterate its own solve would stop at.
#include "batched.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <set>

namespace ccsd {

namespace {

std::mutex g_tune_mu;
std::map<std::string, std::pair<int, int>> g_tune;  // op signature -> (tile, target)

std::string signature(const std::vector<GGemm> &parts, int sms) {
    std::string s = std::to_string(sms) + ":";
    for (const GGemm &g : parts)
        s += std::to_string(g.M) + "," + std::to_string(g.N) + "," + std::to_string(g.K) +
             (g.A.col.s2 == 1 ? "a" : "") + (g.B.col.s2 == 1 ? "b" : "") + ";";
    return s;
}

template <class T>
size_t append(std::vector<char> &blob, const std::vector<T> &v) {
    const size_t off = (blob.size() + 255) / 256 * 256;
    blob.resize(off + v.size() * sizeof(T));
    std::memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
    return off;
}

const char *tile_name(int cfg) {
    static const char *names[kNumGTiles] = {"64x64", "32x64", "64x32", "32x32", "128x64"};
    return names[cfg];
}

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

Batch::Batch(const ccsd_problem *const *problems, int n, const ccsd_options &opts) {
    if (n <= 0 || !problems) throw Error(CCSD_ERR_INVALID_ARG, "batched solve needs n >= 1 problems");
    for (int i = 0; i < n; ++i)
        if (!problems[i]) throw Error(CCSD_ERR_INVALID_ARG, "problem " + std::to_string(i) + " is NULL");
    if (opts.t1_start || opts.t2_start)
        throw Error(CCSD_ERR_INVALID_ARG, "restart amplitudes (t1_start / t2_start) are for single solves");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
    }
    if (opts.method != CCSD_METHOD_CCSD)
        throw Error(CCSD_ERR_UNSUPPORTED, "the batched solve runs CCSD (method CCSD_METHOD_CCSD)");
    opt_ = opts;
    if (opts.stream) {
        st_ = (cudaStream_t)opts.stream;
    } else {
        CCSD_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    try {
        int dev = 0;
        CCSD_CUDA(cudaGetDevice(&dev));
        CCSD_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
        ccsd_options eo = opts;
        eo.stream = st_;
        eo.profile = 0;
        eo.verbose = 0;
        for (int i = 0; i < n; ++i) {
            eng_.emplace_back(new Engine(*problems[i], eo));
            // the batch replays recorded residuals, which contract ovvv directly:
            // the V+- and U+- packs of the unrecorded pair forms are not kept
            eng_.back()->Vzp_.alloc(0);
            eng_.back()->Vzm_.alloc(0);
            eng_.back()->Uxp_.alloc(0);
            eng_.back()->Uxm_.alloc(0);
        }
        const int per = grouped_partials_per_part();
        CCSD_CUDA(cudaMalloc(&active_, sizeof(int) * n));
        CCSD_CUDA(cudaMalloc(&partials_, sizeof(double) * per * n));
        CCSD_CUDA(cudaMalloc(&e_dev_, sizeof(double) * n));
        CCSD_CUDA(cudaMalloc(&n2_dev_, sizeof(double) * n));
        CCSD_CUDA(cudaMallocHost(&h_e_, sizeof(double) * n));
        CCSD_CUDA(cudaMallocHost(&h_n2_, sizeof(double) * n));
        CCSD_CUDA(cudaMallocHost(&h_active_, sizeof(int) * n));
        CCSD_CUDA(cudaMalloc(&diis_dots_dev_, sizeof(double) * kDiisSlots * n));
        CCSD_CUDA(cudaMallocHost(&h_diis_dots_, sizeof(double) * kDiisSlots * n));
        CCSD_CUDA(cudaMalloc(&d_err_, sizeof(int)));
        CCSD_CUDA(cudaMemset(d_err_, 0, sizeof(int)));
        record();
    } catch (...) {
        release();
        throw;
    }
}

void Batch::destroy_graphs() {
    if (g_update_) cudaGraphExecDestroy(g_update_);
    if (g_energy_) cudaGraphExecDestroy(g_energy_);
    g_update_ = g_energy_ = nullptr;
}

Batch::~Batch() { release(); }

// Frees every resource the batch owns (the engines first: they use the stream).
void Batch::release() {
    if (st_) cudaStreamSynchronize(st_);
    destroy_graphs();
    eng_.clear();
    if (desc_) cudaFree(desc_);
    if (active_) cudaFree(active_);
    if (partials_) cudaFree(partials_);
    if (e_dev_) cudaFree(e_dev_);
    if (n2_dev_) cudaFree(n2_dev_);
    if (ws_) cudaFree(ws_);
    for (Pack &P : packs_) packed_split_free(P.buf);
    packs_.clear();
    if (d_err_) cudaFree(d_err_);
    d_err_ = nullptr;
    if (h_e_) cudaFreeHost(h_e_);
    if (h_n2_) cudaFreeHost(h_n2_);
    if (h_active_) cudaFreeHost(h_active_);
    if (diis_dots_dev_) cudaFree(diis_dots_dev_);
    if (h_diis_dots_) cudaFreeHost(h_diis_dots_);
    diis_dots_dev_ = h_diis_dots_ = nullptr;
    desc_ = nullptr;
    active_ = nullptr;
    partials_ = e_dev_ = n2_dev_ = ws_ = h_e_ = h_n2_ = nullptr;
    h_active_ = nullptr;
    if (own_stream_ && st_) cudaStreamDestroy(st_);
    st_ = nullptr;
    own_stream_ = false;
}

// Record one residual of every engine (no kernel runs) and check that the
// tapes line up operation by operation.
void Batch::record() {
    const int n = size();
    tapes_.assign(n, {});
    for (int s = 0; s < n; ++s) {
        Engine &E = *eng_[s];
        E.tape_ = &tapes_[s];
        E.record_only_ = true;
        try {
            E.residual();
        } catch (...) {
            E.tape_ = nullptr;
            E.record_only_ = false;
            throw;
        }
        E.tape_ = nullptr;
        E.record_only_ = false;
    }
    for (int s = 1; s < n; ++s) {
        if (tapes_[s].size() != tapes_[0].size())
            throw Error(CCSD_ERR_INVALID_ARG, "batched residual tapes differ in length");
        for (size_t k = 0; k < tapes_[0].size(); ++k)
            if (tapes_[s][k].kind != tapes_[0][k].kind)
                throw Error(CCSD_ERR_INVALID_ARG, "batched residual tapes differ in operation kinds");
    }
    ops_.clear();
    for (size_t k = 0; k < tapes_[0].size(); ++k) {
        GOp op;
        op.kind = tapes_[0][k].kind;
        op.site = tapes_[0][k].site;
        ops_.push_back(op);
    }
}

// Time every candidate (tile shape x split-K target) of one grouped
// contraction on the batch's own operands and keep the fastest.  The residual
// recomputes every intermediate from (t1, t2) and the integrals, so running
// the contraction repeatedly here does not affect the next update.
void Batch::tune(GOp &op, std::vector<GGemm> &parts) {
    const int n = size();
    const std::string sig = signature(parts, sms_);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(sig);
        if (it != g_tune.end()) {
            op.plan = plan_grouped_gemm(parts, it->second.first, it->second.second, sms_);
            return;
        }
    }
    GGemm *d_parts = nullptr;
    CCSD_CUDA(cudaMalloc(&d_parts, sizeof(GGemm) * n));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double best = 1e300;
    int best_cfg = kTile64x64, best_target = 2 * sms_;
    try {
        CCSD_CUDA(cudaEventCreate(&e0));
        CCSD_CUDA(cudaEventCreate(&e1));
        const int targets[] = {0, sms_, 2 * sms_, 4 * sms_, 8 * sms_};
        std::vector<std::pair<int, int>> seen;
        for (int cfg = 0; cfg < kNumGTiles; ++cfg) {
            for (int target : targets) {
                std::vector<GGemm> trial = parts;
                GGemmPlan p = plan_grouped_gemm(trial, cfg, target, sms_);
                if (std::find(seen.begin(), seen.end(), std::make_pair(cfg, p.total_items)) != seen.end()) continue;
                seen.emplace_back(cfg, p.total_items);
                if (p.ws_elems > ws_elems_) {
                    CCSD_CUDA(cudaStreamSynchronize(st_));
                    if (ws_) cudaFree(ws_);
                    ws_ = nullptr;
                    ws_elems_ = 0;
                    CCSD_CUDA(cudaMalloc(&ws_, sizeof(double) * p.ws_elems));
                    ws_elems_ = p.ws_elems;
                }
                CCSD_CUDA(cudaMemcpyAsync(d_parts, trial.data(), sizeof(GGemm) * n, cudaMemcpyHostToDevice, st_));
                // one timed launch; short launches are re-timed as the mean of three
                auto timed = [&](int reps) {
                    CCSD_CUDA(cudaEventRecord(e0, st_));
                    for (int r = 0; r < reps; ++r) launch_grouped_gemm(p, d_parts, n, active_, ws_, st_);
                    CCSD_CUDA(cudaEventRecord(e1, st_));
                    CCSD_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    CCSD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    return (double)ms / reps;
                };
                double ms = timed(1);
                if (ms < 2.0) ms = timed(3);
                op.candidates += 1;
                if (ms < best) {
                    best = ms;
                    best_cfg = cfg;
                    best_target = target;
                }
            }
        }
    } catch (...) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(d_parts);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_parts);
    op.tuned_ms = best;
    op.plan = plan_grouped_gemm(parts, best_cfg, best_target, sms_);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[sig] = std::make_pair(best_cfg, best_target);
}

// Grouped descriptors of every operation (contractions tuned), uploaded once.
void Batch::build_ops() {
    const int n = size();
    CCSD_CUDA(cudaStreamSynchronize(st_));
    for (int s = 0; s < n; ++s) h_active_[s] = 1;
    CCSD_CUDA(cudaMemcpyAsync(active_, h_active_, sizeof(int) * n, cudaMemcpyHostToDevice, st_));
    blob_.clear();
    cudaEvent_t a = nullptr, b = nullptr;
    CCSD_CUDA(cudaEventCreate(&a));
    CCSD_CUDA(cudaEventCreate(&b));
    CCSD_CUDA(cudaEventRecord(a, st_));
    size_t need_ws = 0;
    for (size_t k = 0; k < ops_.size(); ++k) {
        GOp &op = ops_[k];
        switch (op.kind) {
            case TapeOp::Gemm: {
                std::vector<GroupedSplitPart> sparts;
                if (opt_.precision != CCSD_PREC_FP64 && plan_split(op, k, sparts)) {
                    op.off = append(blob_, sparts);
                    break;
                }
                std::vector<GGemm> parts(n);
                for (int s = 0; s < n; ++s) {
                    const TapeOp &t = tapes_[s][k];
                    GGemm &g = parts[s];
                    g.A = t.A;
                    g.B = t.B;
                    g.C = t.C;
                    g.alpha = t.alpha;
                    g.beta = t.beta;
                    g.M = t.M;
                    g.N = t.N;
                    g.K = t.K;
                    g.sys = s;
                }
                op.plan = plan_grouped_gemm(parts, kTile64x64, 2 * sms_, sms_);
                if (!op.plan.gemv) tune(op, parts);
                need_ws = std::max(need_ws, op.plan.ws_elems);
                op.off = append(blob_, parts);
                break;
            }
            case TapeOp::Axpby:
            case TapeOp::Copy: {
                std::vector<GAxpby> parts(n);
                for (int s = 0; s < n; ++s) {
                    const TapeOp &t = tapes_[s][k];
                    GAxpby &g = parts[s];
                    g.X = t.A;
                    g.Y = t.C;
                    g.sys = s;
                    if (op.kind == TapeOp::Copy) {
                        g.R = 1;
                        g.C = t.M;
                        g.alpha = 1.0;
                        g.beta = 0.0;
                    } else {
                        g.R = t.M;
                        g.C = t.N;
                        g.alpha = t.alpha;
                        g.beta = t.beta;
                    }
                    op.max_elems = std::max(op.max_elems, (size_t)g.R * g.C);
                }
                op.off = append(blob_, parts);
                break;
            }
            case TapeOp::Tau:
            case TapeOp::Theta:
            case TapeOp::TauSym:
            case TapeOp::Unpack: {
                std::vector<GAmp> parts(n);
                for (int s = 0; s < n; ++s) {
                    const TapeOp &t = tapes_[s][k];
                    GAmp &g = parts[s];
                    g.t1 = t.t1;
                    g.t2 = t.t2;
                    g.out1 = t.out1;
                    g.out2 = t.out2;
                    g.o = eng_[s]->o_;
                    g.v = eng_[s]->v_;
                    g.sys = s;
                    const size_t elems = op.kind == TapeOp::TauSym
                                             ? (size_t)g.o * (g.o + 1) / 2 * ((size_t)g.v * (g.v + 1) / 2)
                                             : (size_t)g.o * g.o * g.v * g.v;
                    op.max_elems = std::max(op.max_elems, elems);
                }
                op.off = append(blob_, parts);
                break;
            }
            case TapeOp::WSym:
                throw Error(CCSD_ERR_INVALID_ARG, "batched residual tape holds an integral-build operation");
        }
    }
    CCSD_CUDA(cudaEventRecord(b, st_));
    CCSD_CUDA(cudaEventSynchronize(b));
    float ms = 0.f;
    CCSD_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    tune_ms_ = ms;

    // update, amplitude copy, tau and energy descriptors
    std::vector<GUpdate> upd(n);
    std::vector<GAxpby> cp1(n), cp2(n);
    std::vector<GAmp> tau(n);
    std::vector<GDot> dot(n);
    max_t1_ = max_t2_ = 0;
    for (int s = 0; s < n; ++s) {
        Engine &E = *eng_[s];
        const size_t nT1 = (size_t)E.o_ * E.v_, nT2 = nT1 * E.o_ * E.v_;
        max_t1_ = std::max(max_t1_, nT1);
        max_t2_ = std::max(max_t2_, nT2);
        GUpdate &u = upd[s];
        u.R = E.R_.p;
        u.Rp = E.Rp_.p;
        u.R1 = E.R1_.p;
        u.eo = E.eo_.p;
        u.ev = E.ev_.p;
        u.t1_old = E.t1_.p;
        u.t2_old = E.t2_.p;
        u.t1_new = E.t1n_.p;
        u.t2_new = E.t2n_.p;
        u.o = E.o_;
        u.v = E.v_;
        u.sys = s;
        cp1[s].X = mv(E.t1n_.p, ix1(0), ix1(1));
        cp1[s].Y = ovw(E.t1_.p, ix1(0), ix1(1));
        cp1[s].R = 1;
        cp1[s].C = (int)nT1;
        cp1[s].alpha = 1.0;
        cp1[s].sys = s;
        cp2[s].X = mv(E.t2n_.p, ix1(0), ix1(1));
        cp2[s].Y = ovw(E.t2_.p, ix1(0), ix1(1));
        cp2[s].R = 1;
        cp2[s].C = (int)nT2;
        cp2[s].alpha = 1.0;
        cp2[s].sys = s;
        tau[s].t1 = E.t1_.p;
        tau[s].t2 = E.t2_.p;
        tau[s].out1 = E.tau_.p;
        tau[s].o = E.o_;
        tau[s].v = E.v_;
        tau[s].sys = s;
        dot[s].x = E.Lijab_.p;
        dot[s].y = E.tau_.p;
        dot[s].n = (long long)nT2;
        dot[s].sys = s;
    }
    for (size_t i = 0; i < packs_.size(); ++i) packs_[i].off = append(blob_, pack_parts_[i]);
    upd_off_ = append(blob_, upd);
    cp1_off_ = append(blob_, cp1);
    cp2_off_ = append(blob_, cp2);
    tau_off_ = append(blob_, tau);
    dot_off_ = append(blob_, dot);

    if (desc_) cudaFree(desc_);
    desc_ = nullptr;
    CCSD_CUDA(cudaMalloc(&desc_, blob_.size()));
    CCSD_CUDA(cudaMemcpy(desc_, blob_.data(), blob_.size(), cudaMemcpyHostToDevice));
    if (need_ws > ws_elems_) {
        if (ws_) cudaFree(ws_);
        ws_ = nullptr;
        ws_elems_ = 0;
        CCSD_CUDA(cudaMalloc(&ws_, sizeof(double) * need_ws));
        ws_elems_ = need_ws;
    }
    // operands over constant integrals are split once, here
    for (Pack &P : packs_)
        if (P.key > 0)
            grouped_split_operand_launch(P.buf, reinterpret_cast<const GroupedSplitOperandPart *>(desc_ + P.off), n,
                                         P.max_rows, P.max_kpad, P.rowc, active_, st_);
    CCSD_CUDA(cudaStreamSynchronize(st_));
}

// A contraction whose largest system has M N K >= 1e7 runs on the tensor
// cores: operands split into packed buffers (rows and K padded with zeros, so
// small systems need no minimum size), one grouped tcgen05 launch.  The
// orientation (A/B swap) follows the single-system rule for the first system.
bool Batch::plan_split(GOp &op, size_t k, std::vector<GroupedSplitPart> &sp) {
    const int n = size();
    long long maxmnk = 0;
    for (int s = 0; s < n; ++s) {
        const TapeOp &t = tapes_[s][k];
        if (t.M < 1 || t.N < 1 || t.K < 1) return false;
        maxmnk = std::max(maxmnk, (long long)t.M * t.N * t.K);
    }
    if (maxmnk < 10000000ll) return false;
    const TapeOp &t0 = tapes_[0][k];
    const bool swap = SplitEngine::prefer_swap(t0.M, t0.N, t0.C);
    std::vector<GroupedSplitOperandPart> pa(n), pb(n);
    int kmax = 0, nmax = 0;
    for (int s = 0; s < n; ++s) {
        const TapeOp &t = tapes_[s][k];
        pa[s].v = swap ? t.B : t.A;
        pa[s].rows = swap ? t.N : t.M;
        pb[s].v = swap ? t.A : t.B;
        pb[s].rows = swap ? t.M : t.N;
        pa[s].K = pb[s].K = t.K;
        pa[s].sys = pb[s].sys = s;
        kmax = std::max(kmax, t.K);
        nmax = std::max(nmax, pb[s].rows);
    }
    const int pitch = (kmax + 31) / 32 * 32;
    op.packA = pack_for(swap ? t0.key_b : t0.key_a, pa, pitch);
    op.packB = pack_for(swap ? t0.key_a : t0.key_b, pb, pitch);
    op.bn = grouped_split_bn(nmax);
    sp.assign(n, GroupedSplitPart());
    int tiles = 0;
    for (int s = 0; s < n; ++s) {
        const TapeOp &t = tapes_[s][k];
        GroupedSplitPart &g = sp[s];
        g.C = swap ? OutView{t.C.p, t.C.col, t.C.row} : t.C;
        g.alpha = t.alpha;
        g.beta = t.beta;
        g.M = pa[s].rows;
        g.N = pb[s].rows;
        g.nkb = (t.K + 31) / 32;
        g.rowA0 = pack_parts_[op.packA][s].row0;
        g.rowB0 = pack_parts_[op.packB][s].row0;
        g.scaleA = packs_[op.packA].buf.scale + g.rowA0;
        g.scaleB = packs_[op.packB].buf.scale + g.rowB0;
        g.tiles_m = (g.M + 127) / 128;
        g.tiles_n = (g.N + op.bn - 1) / op.bn;
        g.tile_begin = tiles;
        g.sys = s;
        tiles += g.tiles_m * g.tiles_n;
    }
    op.total_tiles = tiles;
    op.split = true;
    return true;
}

// The packed buffer of one operand view; views with the same nonzero split-cache
// key (the same tensor view in every system) share one buffer.
int Batch::pack_for(int key, const std::vector<GroupedSplitOperandPart> &parts, int pitch) {
    if (key != 0)
        for (size_t i = 0; i < packs_.size(); ++i)
            if (packs_[i].key == key && packs_[i].buf.kpad == pitch) return (int)i;
    std::vector<GroupedSplitOperandPart> pp = parts;
    int rows = 0, max_rows = 0;
    for (GroupedSplitOperandPart &g : pp) {
        g.row0 = rows;
        rows += (g.rows + 127) / 128 * 128;
        max_rows = std::max(max_rows, g.rows);
    }
    Pack P;
    P.key = key;
    P.max_rows = max_rows;
    P.max_kpad = pitch;
    P.rowc = pp[0].v.row.s2 == 1 && pp[0].v.col.s2 != 1;
    packed_split_alloc(P.buf, rows, pitch, opt_.precision);
    packs_.push_back(P);
    pack_parts_.push_back(pp);
    return (int)packs_.size() - 1;
}

void Batch::launch_op(const GOp &op) {
    const int n = size();
    switch (op.kind) {
        case TapeOp::Gemm:
            if (op.split) {
                for (int pk : {op.packA, op.packB}) {
                    Pack &P = packs_[pk];
                    if (P.key > 0) continue;  // constant: split once at set-up
                    if (P.key < 0 && split_done_.count(P.key)) continue;  // shared, already split this update
                    grouped_split_operand_launch(P.buf, reinterpret_cast<const GroupedSplitOperandPart *>(desc_ + P.off),
                                                 n, P.max_rows, P.max_kpad, P.rowc, active_, st_);
                    if (P.key < 0) split_done_.insert(P.key);
                }
                grouped_split_gemm_launch(packs_[op.packA].buf, packs_[op.packB].buf, op.bn,
                                          reinterpret_cast<const GroupedSplitPart *>(desc_ + op.off), n, op.total_tiles,
                                          active_, d_err_, st_);
            } else {
                launch_grouped_gemm(op.plan, reinterpret_cast<const GGemm *>(desc_ + op.off), n, active_, ws_, st_);
            }
            break;
        case TapeOp::Axpby:
        case TapeOp::Copy:
            launch_grouped_axpby(reinterpret_cast<const GAxpby *>(desc_ + op.off), n, op.max_elems, active_, st_);
            break;
        case TapeOp::Tau:
            launch_grouped_tau(reinterpret_cast<const GAmp *>(desc_ + op.off), n, op.max_elems, active_, st_);
            break;
        case TapeOp::Theta:
            launch_grouped_theta(reinterpret_cast<const GAmp *>(desc_ + op.off), n, op.max_elems, active_, st_);
            break;
        case TapeOp::TauSym:
            launch_grouped_tau_sym(reinterpret_cast<const GAmp *>(desc_ + op.off), n, op.max_elems, active_, st_);
            break;
        case TapeOp::Unpack:
            launch_grouped_unpack(reinterpret_cast<const GAmp *>(desc_ + op.off), n, op.max_elems, active_, st_);
            break;
        case TapeOp::WSym:
            break;
    }
}

void Batch::capture() {
    destroy_graphs();
    const int n = size();
    const long l0 = launch_count();
    for (int g = 0; g < 2; ++g) {
        cudaGraph_t graph = nullptr;
        CCSD_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        try {
            if (g == 0) {
                split_done_.clear();
                for (const GOp &op : ops_) launch_op(op);
                launch_grouped_update(reinterpret_cast<const GUpdate *>(desc_ + upd_off_), n, active_, partials_, st_);
                launch_grouped_sum(n, active_, partials_, n2_dev_, st_);
            } else {
                launch_grouped_axpby(reinterpret_cast<const GAxpby *>(desc_ + cp1_off_), n, max_t1_, active_, st_);
                launch_grouped_axpby(reinterpret_cast<const GAxpby *>(desc_ + cp2_off_), n, max_t2_, active_, st_);
                launch_grouped_tau(reinterpret_cast<const GAmp *>(desc_ + tau_off_), n, max_t2_, active_, st_);
                launch_grouped_dot(reinterpret_cast<const GDot *>(desc_ + dot_off_), n, active_, partials_, st_);
                launch_grouped_sum(n, active_, partials_, e_dev_, st_);
            }
        } catch (...) {
            cudaStreamEndCapture(st_, &graph);
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            throw;
        }
        CCSD_CUDA(cudaStreamEndCapture(st_, &graph));
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CCSD_CUDA(e);
        (g == 0 ? g_update_ : g_energy_) = exec;
    }
    launches_per_update_ = (int)(launch_count() - l0);
}

void Batch::solve(ccsd_result *res) {
    const int n = size();
    if (!res) throw Error(CCSD_ERR_INVALID_ARG, "results is NULL");
    std::vector<double> e(n), resid(n, 0.0);
    std::vector<int> updates(n, 0), hist(n, 0), conv(n, 0), status(n, CCSD_OK);
    // T1 = 0, T2 = MP2 for every system (ccsd_memory_optimized.cpp:473-490)
    for (int s = 0; s < n; ++s) {
        Engine &E = *eng_[s];
        E.diis_t_.clear();
        E.diis_e_.clear();
        E.diis_count_ = E.diis_next_ = 0;
        E.t1_.zero(st_);
        k_mp2_guess(E.o_, E.v_, E.ovov_.p, E.eo_.p, E.ev_.p, E.t2_.p, st_);
        e[s] = E.energy_of(E.t1_.p, E.t2_.p);
        if (res[s].energy_history && res[s].history_capacity > 0) res[s].energy_history[0] = e[s];
        hist[s] = 1;
    }
    if (!tuned_) {
        build_ops();
        capture();
        tuned_ = true;
    }
    const int cap = opt_.fixed_iterations > 0 ? opt_.fixed_iterations : std::max(opt_.max_iter, 1);
    for (int s = 0; s < n; ++s) h_active_[s] = 1;
    int nactive = n;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    CCSD_CUDA(cudaEventCreate(&ev0));
    CCSD_CUDA(cudaEventCreate(&ev1));
    try {
        while (nactive > 0) {
            CCSD_CUDA(cudaMemcpyAsync(active_, h_active_, sizeof(int) * n, cudaMemcpyHostToDevice, st_));
            CCSD_CUDA(cudaEventRecord(ev0, st_));
            CCSD_CUDA(cudaGraphLaunch(g_update_, st_));
            if (opt_.diis_size > 0) {
                // every active system's DIIS store and overlaps, then one read-back and one
                // synchronisation for all of them, then the host solves and extrapolations
                for (int s = 0; s < n; ++s)
                    if (h_active_[s]) eng_[s]->diis_store_async(diis_dots_dev_ + (size_t)s * kDiisSlots);
                CCSD_CUDA(cudaMemcpyAsync(h_diis_dots_, diis_dots_dev_, sizeof(double) * kDiisSlots * n,
                                          cudaMemcpyDeviceToHost, st_));
                CCSD_CUDA(cudaStreamSynchronize(st_));
                for (int s = 0; s < n; ++s)
                    if (h_active_[s]) eng_[s]->diis_finish(updates[s], h_diis_dots_ + (size_t)s * kDiisSlots);
            }
            CCSD_CUDA(cudaGraphLaunch(g_energy_, st_));
            CCSD_CUDA(cudaEventRecord(ev1, st_));
            CCSD_CUDA(cudaMemcpyAsync(h_e_, e_dev_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
            CCSD_CUDA(cudaMemcpyAsync(h_n2_, n2_dev_, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
            CCSD_CUDA(cudaStreamSynchronize(st_));
            float ms = 0.f;
            CCSD_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
            note_launch(launches_per_update_);  // kernels replayed from the graphs
            for (int s = 0; s < n; ++s) {
                if (!h_active_[s]) continue;
                const double e_old = e[s];
                e[s] = h_e_[s];
                resid[s] = std::sqrt(std::max(h_n2_[s], 0.0));
                ccsd_result &r = res[s];
                if (r.update_ms && updates[s] < r.history_capacity) r.update_ms[updates[s]] = ms;
                ++updates[s];
                if (r.energy_history && hist[s] < r.history_capacity) r.energy_history[hist[s]] = e[s];
                ++hist[s];
                bool stop = false;
                if (!std::isfinite(e[s]) || !std::isfinite(resid[s])) {
                    status[s] = CCSD_ERR_DIVERGED;
                    stop = true;
                } else if (opt_.fixed_iterations > 0) {
                    stop = updates[s] >= opt_.fixed_iterations;
                } else {
                    bool ok = std::fabs(e[s] - e_old) < opt_.energy_tol;
                    if (opt_.residual_tol > 0.0) ok = ok && resid[s] < opt_.residual_tol;
                    if (ok) {
                        conv[s] = 1;
                        stop = true;
                    } else if (updates[s] >= cap) {
                        stop = true;
                    }
                }
                if (stop) {
                    h_active_[s] = 0;
                    --nactive;
                }
            }
            if (opt_.verbose)
                std::printf("ccsd batch update: %d of %d systems still iterating, %.3f ms\n", nactive, n, ms);
        }
    } catch (...) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        throw;
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    {
        int err = 0;
        CCSD_CUDA(cudaMemcpy(&err, d_err_, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) throw Error(CCSD_ERR_TIMEOUT, "split-precision kernel reported a bounded-wait timeout");
    }

    int first_bad = -1;
    for (int s = 0; s < n; ++s) {
        Engine &E = *eng_[s];
        ccsd_result &r = res[s];
        const size_t nT1 = (size_t)E.o_ * E.v_, nT2 = nT1 * E.o_ * E.v_;
        r.e_corr = e[s];
        r.residual_norm = resid[s];
        r.iterations = updates[s];
        r.converged = conv[s];
        r.history_len = std::min(hist[s], std::max(r.history_capacity, 0));
        r.flops_per_update = ccsd_flops_per_update(E.o_, E.v_);
        if (r.t1) CCSD_CUDA(cudaMemcpy(r.t1, E.t1_.p, nT1 * sizeof(double), cudaMemcpyDeviceToHost));
        if (r.t2) CCSD_CUDA(cudaMemcpy(r.t2, E.t2_.p, nT2 * sizeof(double), cudaMemcpyDeviceToHost));
        E.solved_ = status[s] == CCSD_OK;
        E.last_e_ = e[s];
        if (status[s] != CCSD_OK && first_bad < 0) first_bad = s;
    }
    if (first_bad >= 0)
        throw Error(status[first_bad], "batched system " + std::to_string(first_bad) + " diverged (NaN/Inf)");
}

std::string Batch::report() const {
    std::string s = "{\"systems\": " + std::to_string(size()) + ", \"launches_per_update\": " +
                    std::to_string(launches_per_update_) + ", \"tune_ms\": " + std::to_string(tune_ms_) +
                    ", \"ops\": [";
    char buf[512];
    bool first = true;
    for (size_t k = 0; k < ops_.size(); ++k) {
        const GOp &op = ops_[k];
        const char *kind = op.kind == TapeOp::Gemm     ? "contraction"
                           : op.kind == TapeOp::Axpby  ? "axpby"
                           : op.kind == TapeOp::Copy   ? "copy"
                           : op.kind == TapeOp::Tau    ? "tau"
                           : op.kind == TapeOp::Theta  ? "theta"
                           : op.kind == TapeOp::TauSym ? "tau_pairs"
                           : op.kind == TapeOp::Unpack ? "ladder_unpack"
                                                       : "w_pairs";
        if (op.kind == TapeOp::Gemm && op.split)
            std::snprintf(buf, sizeof buf,
                          "%s{\"op\": %zu, \"kind\": \"%s\", \"site\": \"%s\", \"path\": \"split\", "
                          "\"bn\": %d, \"tiles\": %d}",
                          first ? "" : ", ", k, kind, op.site ? op.site : "", op.bn, op.total_tiles);
        else if (op.kind == TapeOp::Gemm)
            std::snprintf(buf, sizeof buf,
                          "%s{\"op\": %zu, \"kind\": \"%s\", \"site\": \"%s\", \"path\": \"%s\", \"tile\": \"%s\", "
                          "\"target\": %d, \"items\": %d, \"grid\": %d, \"candidates\": %d, \"cached\": %s, "
                          "\"tuned_ms\": %.6f}",
                          first ? "" : ", ", k, kind, op.site ? op.site : "", op.plan.gemv ? "gemv" : "tiled",
                          tile_name(op.plan.cfg), op.plan.target, op.plan.total_items, op.plan.grid, op.candidates,
                          (!op.plan.gemv && op.candidates == 0) ? "true" : "false", op.tuned_ms);
        else
            std::snprintf(buf, sizeof buf, "%s{\"op\": %zu, \"kind\": \"%s\", \"max_elems\": %zu}", first ? "" : ", ",
                          k, kind, op.max_elems);
        s += buf;
        first = false;
    }
    s += "]}";
    return s;
}

}  // namespace ccsd
