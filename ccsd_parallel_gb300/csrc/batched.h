// Batched solve: many closed-shell systems of uneven nocc/nvir iterated
// together, one grouped launch per operation of the amplitude update, the
// whole update replayed from a captured CUDA graph.
#pragma once

#include <memory>
#include <set>
#include <string>
#include <vector>

#include "engine.h"
#include "grouped.h"
#include "split_gemm.h"

namespace ccsd {

class Batch {
  public:
    Batch(const ccsd_problem *const *problems, int n, const ccsd_options &opts);
    ~Batch();
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;

    // Iterate every system from its MP2 guess with the single-system rules
    // (per-system stop, cap and DIIS); fills results[0..n).  Throws the first
    // per-system failure (e.g. divergence) after every result is filled.
    void solve(ccsd_result *results);
    int size() const { return (int)eng_.size(); }
    // JSON: the grouped operations, their tile plans and the autotuning times.
    std::string report() const;
    // Kernel launches in one replay of the update graphs.
    int launches_per_update() const { return launches_per_update_; }

  private:
    struct GOp {
        TapeOp::Kind kind;
        const char *site = nullptr;
        size_t off = 0;          // byte offset of the descriptors in desc_
        size_t max_elems = 0;    // element-wise ops: largest per-system size
        GGemmPlan plan;          // contractions
        double tuned_ms = 0.0;   // best autotuned time
        int candidates = 0;
        // split-precision contraction on the tensor cores (packed operands)
        bool split = false;
        int packA = -1, packB = -1, bn = 0, total_tiles = 0;
    };
    // one packed split operand (all systems' rows of one operand view)
    struct Pack {
        PackedSplit buf;
        size_t off = 0;      // GroupedSplitOperandPart[] in desc_
        int key = 0;         // split-cache key of the view (> 0 constant, < 0 per update, 0 private)
        int max_rows = 0, max_kpad = 0;
        bool rowc = false;
    };

    void record();
    void build_ops();
    bool plan_split(GOp &op, size_t k, std::vector<GroupedSplitPart> &parts);
    int pack_for(int key, const std::vector<GroupedSplitOperandPart> &parts, int pitch);
    void tune(GOp &op, std::vector<GGemm> &parts);
    void capture();
    void launch_op(const GOp &op);
    void destroy_graphs();
    void release();

    std::vector<std::unique_ptr<Engine>> eng_;
    ccsd_options opt_{};
    cudaStream_t st_ = nullptr;
    bool own_stream_ = false;
    int sms_ = 152;

    std::vector<std::vector<TapeOp>> tapes_;
    std::vector<GOp> ops_;
    std::vector<Pack> packs_;
    std::vector<std::vector<GroupedSplitOperandPart>> pack_parts_;  // host copies until the upload
    int *d_err_ = nullptr;  // split kernels' bounded-wait error word
    std::set<int> split_done_;  // per-update shared packs already split in the graph being captured
    std::vector<char> blob_;   // host copy of every descriptor array
    char *desc_ = nullptr;     // device copy
    size_t upd_off_ = 0, cp1_off_ = 0, cp2_off_ = 0, tau_off_ = 0, dot_off_ = 0;
    size_t max_t2_ = 0, max_t1_ = 0;
    int *active_ = nullptr;    // device, one flag per system
    double *partials_ = nullptr, *e_dev_ = nullptr, *n2_dev_ = nullptr;
    double *ws_ = nullptr;
    size_t ws_elems_ = 0;
    double *h_e_ = nullptr, *h_n2_ = nullptr;  // pinned host
    static constexpr int kDiisSlots = 16;       // DIIS overlaps per system (the largest diis_size)
    double *diis_dots_dev_ = nullptr, *h_diis_dots_ = nullptr;
    int *h_active_ = nullptr;
    cudaGraphExec_t g_update_ = nullptr, g_energy_ = nullptr;
    int launches_per_update_ = 0;
    bool tuned_ = false;
    double tune_ms_ = 0.0;
};

}  // namespace ccsd
