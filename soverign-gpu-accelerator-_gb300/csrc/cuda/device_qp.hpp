// Device convex QP interior-point iteration with a diagonal Hessian (see
// include/qp/qp_solver.hpp for the method and the lifting of a general H).
#pragma once

#include <vector>

namespace sankhya {
namespace dev {

// min 1/2 sum_j h_j x_j^2 + c^T x, A x = b (A m x n in CSC, rows sorted within each
// column), lb <= x <= ub; a bound is finite when lb > -1e15 / ub < 1e15.
struct QpProblem {
    int m = 0, n = 0;
    std::vector<int> col_ptrs, row_idx;
    std::vector<double> vals, b, c, lb, ub, h;
};

struct QpSettings {
    double feas_tol = 1e-6, dual_tol = 1e-6, grad_tol = 1e-6;
    int max_iter = 200;
};

// status uses the numbering of qp::QPSolverStatus (0 Optimal, 1 Infeasible,
// 2 Unbounded, 3 IterationLimit, 4 NumericalFailure).
struct QpOutcome {
    int status = 4;
    int iterations = 0;
    double objective = 0.0, primal_residual = 0.0, dual_residual = 0.0, complementarity = 0.0;
    std::vector<double> x, y, z;   // z = zl - zu; filled for Optimal and IterationLimit
};

// Runs the iteration on the current CUDA device (throws api::sk_exception on a
// CUDA error or when no device is visible).
QpOutcome solve_qp_device(const QpProblem& qp, const QpSettings& s);

}  // namespace dev
}  // namespace sankhya
