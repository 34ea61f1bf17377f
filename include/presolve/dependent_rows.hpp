// Presolve: linearly dependent rows of an LP's constraint matrix, found on the
// device. No counterpart in the reference, whose presolve is the Ruiz scaling of
// presolve/scaling.hpp and whose IPM absorbs a rank-deficient A through the delta
// regularisation. The IPM drops such rows itself with
// ipm::MehrotraOptions::dependent_rows = 1 (sk_options.dependent_rows).
#pragma once

#include <vector>

#include "core/problem.hpp"

namespace sankhya {
namespace presolve {

struct DependentRows {
    std::vector<Index> rows;   // rows of A linearly dependent on the others (ascending), when
                               // b is consistent; empty otherwise
    Float inconsistency = 0.0; // ||b - A A^T w||_inf / (1 + ||b||_inf) after refinement
    bool consistent = true;    // inconsistency <= 1e-9: the rows' equations follow from the others
};

// A A^T is factored in FP64 on the device in a fill-reducing order; a row whose
// pivot L_kk^2 (unit-diagonal equilibration: its squared distance from the span of the
// rows eliminated before it) is at most 1e-6 counts as dependent on them
// (sk_presolve_dependent_rows). Throws std::runtime_error on device errors
// and std::invalid_argument on a malformed model.
DependentRows find_dependent_rows(const core::Model& model);

}  // namespace presolve
}  // namespace sankhya
