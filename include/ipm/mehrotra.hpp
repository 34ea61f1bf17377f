// C++ solve API of the device Mehrotra IPM. Source-compatible with the
// reference's src/ipm/mehrotra.hpp:10-31 (MehrotraResult fields, the
// MehrotraSolver(const core::Model&) constructor, solve()); adds an options
// struct, the reduced costs s, run statistics and a batch entry point.
//
// Error behaviour follows the reference: CUDA failures throw std::runtime_error,
// exhausted device memory throws std::bad_alloc, malformed input throws
// std::invalid_argument, and numerical trouble is reported as
// status = IterationLimit. The model must outlive the solver.
#pragma once

#include <vector>

#include "core/problem.hpp"
#include "sankhya/sk_ipm.h"
#include "sankhya/types.hpp"
#include "simplex/primal.hpp"

namespace sankhya {
namespace ipm {

struct MehrotraOptions {
    int precision = SK_PREC_MIXED;
    int start = SK_START_UNIT;
    int criteria = SK_CRIT_RELATIVE;
    double tol = 1e-8;
    int max_iter = 200;
    int ordering = SK_ORDER_AUTO;
    int verbose = 0;
    double mu_switch = 1e-4;
    int ruiz_passes = 10;
    int strict = 0;
    double delta32 = 1e-8;
    double delta64 = 1e-14;
    int fp64_update = SK_FP64_UPDATE_AUTO;
    // 1: linearly dependent rows of A are dropped before the solve (sk_options.dependent_rows)
    int dependent_rows = 0;
    // false (default, as the reference): lb / ub of the model are ignored and x >= 0
    // is solved; true: the model's bounds are honoured through the host standard form
    // (core/standard_form.hpp).
    bool honor_bounds = false;
};

struct MehrotraResult {
    simplex::SimplexStatus status = simplex::SimplexStatus::IterationLimit;
    Float objective_value = 0.0;
    Index iterations = 0;
    Float primal_residual = 0.0;
    Float dual_residual = 0.0;
    Float duality_gap = 0.0;
    std::vector<Float> x;
    std::vector<Float> pi;
    // additions
    std::vector<Float> s;
    sk_info info{};
};

class MehrotraSolver {
public:
    explicit MehrotraSolver(const core::Model& model);
    MehrotraSolver(const core::Model& model, const MehrotraOptions& opts);
    ~MehrotraSolver();
    MehrotraSolver(const MehrotraSolver&) = delete;
    MehrotraSolver& operator=(const MehrotraSolver&) = delete;

    MehrotraResult solve();

private:
    class Impl;
    Impl* impl_;
};

// Solves independent LPs together in one batch (block-diagonal) run.
std::vector<MehrotraResult> solve_batch(const std::vector<const core::Model*>& models,
                                        const MehrotraOptions& opts = MehrotraOptions());

}  // namespace ipm
}  // namespace sankhya
