// Convex QP interior-point solver on the device. Interface of the reference's
// src/qp/qp_solver.hpp:17-66 (QPSolverStatus, QPResult, QPSolver with Options
// {feasibility_tol, dual_tol, grad_tol, max_iterations}, solve, solve_with_diagnostics);
// the reference solves on the host with dense matrices (src/qp/qp_solver.cpp).
//
// Here every iteration runs on the GPU: the reference's primal-dual path-following
// steps (sigma = 0.2, fraction to the boundary 0.995, separate primal and dual
// steps, the same stopping and status rules) with W = H + D diagonal, so the Schur
// complement S = A W^-1 A^T is A diag(theta) A^T and is factored by the LP engine's
// multifrontal Cholesky (FP64 fronts, equilibration, delta ladder, PCG to a
// 1e-13 relative residual). A non-diagonal H is first lifted on the host: a
// pivoted Cholesky gives H = F^T F (F r x n), and the solver works on
// min 1/2 w^T w + c^T x, A x = b, F x - w = 0 with w free, whose Hessian is
// diagonal (dense H, n <= QP_MAX_LIFTED_COLS). x, y (of A's rows) and z = zl - zu
// are returned for the original variables; objective_value is 1/2 x^T H x + c^T x.
#pragma once

#include <vector>

#include "qp/qp_model.hpp"
#include "sankhya/types.hpp"

namespace sankhya {
namespace qp {

enum class QPSolverStatus {
    Optimal,
    Infeasible,
    Unbounded,
    IterationLimit,
    NumericalFailure,
    UnsupportedNonconvex,
    InvalidModel
};

struct QPResult {
    QPSolverStatus status = QPSolverStatus::InvalidModel;
    Float objective_value = 0.0;
    Index iterations = 0;
    Float primal_residual = 0.0;     // ||A x - b||_inf (lifted rows included)
    Float dual_residual = 0.0;       // ||H x + c - A^T y - zl + zu||_inf
    Float complementarity = 0.0;     // mu over the finite bounds
};

// Largest n for which a non-diagonal H is lifted (dense pivoted Cholesky on the host).
constexpr Index QP_MAX_LIFTED_COLS = 4096;

class QPSolver {
public:
    struct Options {
        Float feasibility_tol = math::kDefaultFeasibilityTol;
        Float dual_tol = math::kDefaultFeasibilityTol;
        Float grad_tol = 1e-6;
        Index max_iterations = 200;
    };

    QPSolver() = default;
    explicit QPSolver(const Options& options) : options_(options) {}

    QPSolverStatus solve(const QPModel& qp, std::vector<Float>& x, std::vector<Float>& y, std::vector<Float>& z);
    QPResult solve_with_diagnostics(const QPModel& qp, std::vector<Float>& x, std::vector<Float>& y,
                                    std::vector<Float>& z);

private:
    Options options_;
};

}  // namespace qp
}  // namespace sankhya
