// Multifrontal plan for the normal matrix M = A Theta A^T of a batch of LPs.
//
// The batch is one block-diagonal LP (A = diag(A_1..A_k)); its elimination tree
// is a forest. Columns of M are grouped into supernodes; supernode s owns the
// permuted columns [first, first+ncols) and the sorted row structure R_s
// (|R_s| = nrows, own columns first). Its frontal matrix F_s is a dense
// nrows x nrows column-major block (leading dimension lda = nrows rounded up to
// a multiple of 4, so every column starts 16-byte aligned) in one device buffer:
//   F_s[:, :ncols]           -> the factor panel L(R_s, cols(s)) after factorisation
//   F_s[ncols:, ncols:]      -> the update matrix passed to the parent (extend-add)
// Levels: leaves are level 0, a parent is one above its highest child. Every
// level is factored with tile steps of width kTile; child updates are added to
// parents in "rounds" (one child per parent per round) so that the sum order is
// fixed and no atomics are needed.
//
// Assembly of M (sparse mode) is an SpMV over the Khatri-Rao map W:
//   M[slot] = sum_t w_val[t] * theta[w_col[t]],  w_val = a_ik * a_jk,
// slots 0..M-1 are the diagonal (permuted order), then the strict lower
// nonzeros of A A^T; slot_pos gives each slot's F position. In dense mode (A A^T
// dense enough that one front per LP is cheaper) there is no W: columns of M
// are formed directly from A on the device.
#pragma once

#include <cstdint>
#include <vector>

#include "core/sparse_matrix.hpp"

namespace sankhya {
namespace ipm {

constexpr int kTile = 64;

struct LpView {
    Index m = 0, n = 0;
    const Index* col_ptrs = nullptr;
    const Index* row_idx = nullptr;
    const Float* vals = nullptr;
};

struct PlanStep {            // one tile step of one level
    int level = 0;
    int k = 0;               // column block index within each front
    int item_off = 0;        // into step_items (supernodes active at this step)
    int nitems = 0;
    int trsm_prefix_off = 0; // into step_prefix: nitems+1 entries (row tiles below the block)
    int upd_prefix_off = 0;  // into step_prefix: nitems+1 entries (lower tiles of the trailing part)
    int64_t trsm_tiles = 0;
    int64_t upd_tiles = 0;
    int upd2_prefix_off = 0; // into step_prefix: nitems+1 entries (lower 128x128 blocks of the trailing part)
    int64_t upd2_blocks = 0;
    // emulated FP64 update: 128-row x 64-column blocks of the trailing lower part
    // (row block i holds column blocks 0..2i+1), and each item's first row in the
    // digit buffer (its trailing rows padded to a multiple of 128)
    int upd3_prefix_off = 0; // into step_prefix: nitems+1 entries
    int64_t upd3_blocks = 0;
    int digit_row_off = 0;   // into step_prefix: nitems+1 entries
    int64_t digit_rows = 0;
};

struct PlanRound {           // one extend-add round after a level
    int level = 0;
    int item_off = 0;        // into round_items (children)
    int nitems = 0;
    int prefix_off = 0;      // into round_prefix: nitems+1 entries (32x32 tiles of each update matrix)
    int64_t tiles = 0;
};

struct FrontPlan {
    int nlp = 0;
    Index M = 0, N = 0;
    int64_t nnzA = 0;
    std::vector<Index> row_off, col_off;   // nlp+1 each
    bool dense_mode = false;
    int ordering_used = 0;
    int64_t max_digit_rows = 0;            // largest PlanStep::digit_rows of any step

    std::vector<Index> perm, iperm;        // perm[k] = batch row at elimination position k

    int ns = 0;
    std::vector<Index> sn_first, sn_ncols, sn_nrows, sn_lda, sn_parent, sn_level, sn_lp, sn_of_col;
    std::vector<int64_t> sn_rows_off, sn_F_off, sn_f_off;  // f_off: frontal vectors of the solves
    std::vector<Index> rows;               // concatenated R_s (permuted ids)
    std::vector<int64_t> ea_off;           // per supernode, into ea_map (nrows-ncols entries)
    std::vector<Index> ea_map;             // position of R_c[ncols_c + t] in R_parent
    std::vector<Index> ch_ptr, ch_list;    // children of each supernode (fixed order)
    int64_t F_size = 0, f_size = 0;
    int64_t nnz_factor = 0;
    double flops_factor = 0.0;

    int nlevels = 0;
    std::vector<int> level_ptr, level_sn;
    std::vector<PlanStep> steps;           // ordered by level then k
    std::vector<int> step_level_ptr;       // steps of level l: [step_level_ptr[l], step_level_ptr[l+1])
    std::vector<int> step_items;
    std::vector<int> step_prefix;          // int32 prefix counts
    std::vector<PlanRound> rounds;
    std::vector<int> round_level_ptr;
    std::vector<int> round_items;
    std::vector<int> round_prefix;

    // sparse-mode assembly
    int64_t nslots = 0;
    std::vector<int64_t> slot_pos;
    std::vector<Index> slot_i, slot_j;     // permuted row / column of each slot
    std::vector<int64_t> w_ptr;            // nslots+1
    std::vector<Index> w_col;
    std::vector<Float> w_val;
};

// Builds the plan. ordering: 0 auto (dense or approximate minimum degree; from
// 50000 rows on the given row order or nested dissection, whichever needs fewer
// flops), 1 reference exact minimum degree, 2 natural, 3 approximate minimum
// degree, 4 nested dissection.
// ordering_used: 0 minimum degree, 1 reference, 2 natural / dense, 3 explicit,
// 4 nested dissection. A_csr is the batch matrix (block diagonal) in CSR.
// explicit_perm (optional, sparse mode): use this elimination order as given
// (no postorder relabelling), e.g. the reference's ordering in parity tests.
void build_front_plan(const std::vector<LpView>& lps, const core::CSRMatrix& A_csr, int ordering,
                      FrontPlan& plan, const std::vector<Index>* explicit_perm = nullptr);

// True when A A^T of this LP should be handled as one dense front.
bool prefer_dense_front(const LpView& lp);

// LP of each supernode (fronts never span LPs): the LP that owns its first row.
std::vector<int> supernode_lps(const FrontPlan& plan);

// The plan's tile steps restricted to the fronts of the LPs with on[lp] != 0 (a
// factorisation of some LPs of a batch launches their blocks only). Per step: the
// items whose LP is on, in the plan's order, and for each of the five per-item
// counts (trsm tiles, update tiles, 128x128 blocks, 128x64 blocks, digit rows) the
// kept items' counts summed again from 0 into `prefix`, the step's offsets pointing
// there and its totals recomputed; steps left without items are dropped. level_ptr
// (nlevels + 1) indexes `steps` per level.
struct RestrictedSteps {
    std::vector<PlanStep> steps;
    std::vector<int> level_ptr, items, prefix;
};
void restrict_steps(const FrontPlan& plan, const std::vector<int>& sn_lp, const std::vector<int>& on,
                    RestrictedSteps& out);

}  // namespace ipm
}  // namespace sankhya
