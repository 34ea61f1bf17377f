// Convex QP data model: minimise 1/2 x^T H x + c^T x subject to A x = b and
// lb <= x <= ub, with H symmetric and given by its lower triangle (diagonal
// included) in CSC. Same type, members and validation rules as the reference's
// src/qp/qp_model.hpp:18-72 (QPConvexityStatus, QPModel{lp_part, H, convexity},
// validate()), so the reference's QP callers compile unchanged.
#pragma once

#include <stdexcept>
#include <vector>

#include "core/problem.hpp"
#include "core/sparse_matrix.hpp"
#include "sankhya/types.hpp"

namespace sankhya {
namespace qp {

enum class QPConvexityStatus {
    Unknown,      // not checked: the solver treats it as unsupported
    ConvexPSD,    // H positive semidefinite (supported)
    Nonconvex     // indefinite or negative definite (unsupported)
};

class QPModel {
public:
    core::Model lp_part;     // A, rhs (b), obj (c), lb, ub, sense
    core::CSCMatrix H;       // n x n, lower triangle incl. diagonal
    QPConvexityStatus convexity = QPConvexityStatus::Unknown;

    QPModel() : H(0, 0, {}, {}, {0}) {}

    // Throws std::invalid_argument when the sense is not Minimize, H is not n x n,
    // lb / ub do not have n entries, some lb > ub, or the model is marked Nonconvex.
    void validate() const {
        if (lp_part.sense != OptimizationSense::Minimize)
            throw std::invalid_argument("QPModel: only minimisation is supported");
        if (H.rows != lp_part.A.cols || H.cols != lp_part.A.cols)
            throw std::invalid_argument("QPModel: H must be n x n for n variables");
        const size_t n = static_cast<size_t>(lp_part.A.cols);
        if (lp_part.lb.size() != n || lp_part.ub.size() != n)
            throw std::invalid_argument("QPModel: lb and ub need one entry per variable");
        for (size_t j = 0; j < n; ++j)
            if (lp_part.lb[j] > lp_part.ub[j]) throw std::invalid_argument("QPModel: lb > ub");
        if (convexity == QPConvexityStatus::Nonconvex)
            throw std::invalid_argument("QPModel: a nonconvex QP is not supported");
    }
};

}  // namespace qp
}  // namespace sankhya
