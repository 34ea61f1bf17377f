// Standard form of an LP with variable bounds, for the IPM (which solves
// min c^T x, A x = b, x >= 0). The reference's device IPM ignores lb / ub
// (src/ipm/mehrotra_device.cu never reads them although parsers::read_mps sets
// them, src/parsers/mps_reader.cpp:259-298); honouring them is this module's job.
//
// Per column j (bounds +-infinity = unbounded):
//   lb finite:            x_j = lb_j + x'_j, and if ub_j is finite as well one more
//                         row x'_j + w_j = ub_j - lb_j with a new column w_j >= 0;
//   lb = -inf, ub finite: x_j = ub_j - x'_j (column and cost negated);
//   both infinite:        x_j = x'_j - x''_j (two columns).
// b is shifted by the fixed parts, and c^T x = c'^T x' + offset.
#pragma once

#include <vector>

#include "sankhya/types.hpp"

namespace sankhya {
namespace core {

struct BoundedLp {
    Index m = 0, n = 0;
    const Index* col_ptrs = nullptr;   // CSC of A (m x n)
    const Index* row_idx = nullptr;
    const Float* vals = nullptr;
    const Float* b = nullptr;
    const Float* c = nullptr;
    const Float* lb = nullptr;         // nullptr: all 0
    const Float* ub = nullptr;         // nullptr: all +inf
};

struct StandardForm {
    Index m = 0, n = 0;                // sizes of the standard-form LP
    std::vector<Index> col_ptrs, row_idx;
    std::vector<Float> vals, b, c;
    Float obj_offset = 0.0;            // c^T x = c'^T x' + obj_offset
    enum Kind : int { kShift = 0, kReflect = 1, kFree = 2 };
    std::vector<int> kind;             // per original column
    std::vector<Index> pos, neg;       // standard-form column of x'_j (and x''_j for free columns)
    Index bound_rows = 0;              // rows added for finite upper bounds (after the first m)
};

// Throws std::invalid_argument on lb > ub or non-finite data.
StandardForm to_standard_form(const BoundedLp& lp);

// Maps a standard-form solution (x', y') back: x (n), y (m: the duals of the
// original rows), s = c - A^T y (n); returns c^T x.
Float recover_solution(const BoundedLp& lp, const StandardForm& sf, const Float* xs, const Float* ys, Float* x,
                       Float* y, Float* s);

}  // namespace core
}  // namespace sankhya
