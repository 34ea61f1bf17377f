// Presolve: Ruiz equilibration of an LP model on the host.
// Same entry point as the reference (src/presolve/scaling.hpp:25):
// presolve::apply_ruiz_scaling(core::Model&, int max_iterations = 10).
#pragma once

#include "core/problem.hpp"

namespace sankhya {
namespace presolve {

// Scales A's rows and then its columns by 1/sqrt(largest |entry|) per pass, up to
// max_iterations passes, stopping once every scaled row's and every scaled
// column's largest |entry| was within 1e-4 of 1 at the start of a pass. Integer
// and binary columns are never scaled; rows / columns with no entry above 1e-15
// keep factor 1. The factors accumulate in model.row_scale / model.col_scale
// (created as ones when empty); afterwards rhs <- row_scale .* rhs,
// obj <- col_scale .* obj and finite bounds lb, ub <- bound ./ col_scale, so a
// solution x_s of the scaled model maps back as x = col_scale .* x_s.
void apply_ruiz_scaling(core::Model& model, int max_iterations = 10);

// The same on raw CSC arrays (m x n, int32 indices): vals, rhs, obj and the
// optional lb / ub are scaled in place; integer_cols (optional, one flag per
// column) marks columns never scaled; row_scale (m) and col_scale (n) hold the
// current scale vectors on entry (ones for an unscaled model) and the
// accumulated ones on return. Returns the number of passes made.
int ruiz_scale_csc(Index m, Index n, const Index* col_ptrs, const Index* row_idx, Float* vals, Float* rhs,
                   Float* obj, Float* lb, Float* ub, const unsigned char* integer_cols, int max_iterations,
                   Float* row_scale, Float* col_scale);

}  // namespace presolve
}  // namespace sankhya
