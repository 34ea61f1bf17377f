// qp::QPSolver (include/qp/qp_solver.hpp): validation with the reference's status
// rules (src/qp/qp_solver.cpp:158-185), the lifting of a non-diagonal H, and the
// device iteration (csrc/cuda/device_qp.cu).
#include "qp/qp_solver.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "api/sk_error.hpp"
#include "cuda/device_qp.hpp"

namespace sankhya {
namespace qp {

namespace {

// Pivoted Cholesky of the dense PSD matrix H (n x n, row-major): rows of F with
// H = F^T F, stopping once the largest remaining diagonal entry is at most
// 1e-14 max(1, max_j H_jj). Greedy largest-diagonal pivoting (Higham, "Accuracy
// and Stability of Numerical Algorithms", 10.3) keeps the rank-revealing order.
std::vector<std::vector<double>> pivoted_factor(int n, const std::vector<double>& H) {
    std::vector<double> d(static_cast<size_t>(n));
    double dmax = 1.0;
    for (int j = 0; j < n; ++j) {
        d[j] = H[static_cast<size_t>(j) * n + j];
        dmax = std::max(dmax, d[j]);
    }
    const double stop = 1e-14 * dmax;
    std::vector<std::vector<double>> F;
    for (int k = 0; k < n; ++k) {
        int p = 0;
        for (int j = 1; j < n; ++j) if (d[j] > d[p]) p = j;
        if (!(d[p] > stop)) break;
        std::vector<double> row(static_cast<size_t>(n));
        const double piv = std::sqrt(d[p]);
        for (int j = 0; j < n; ++j) {
            double v = H[static_cast<size_t>(p) * n + j];
            for (const auto& f : F) v -= f[p] * f[j];
            row[j] = v / piv;
        }
        for (int j = 0; j < n; ++j) d[j] -= row[j] * row[j];
        d[p] = 0.0;
        F.push_back(std::move(row));
    }
    return F;
}

}  // namespace

QPResult QPSolver::solve_with_diagnostics(const QPModel& qp, std::vector<Float>& x_out, std::vector<Float>& y_out,
                                          std::vector<Float>& z_out) {
    QPResult result;
    if (qp.convexity == QPConvexityStatus::Nonconvex) {
        result.status = QPSolverStatus::UnsupportedNonconvex;
        return result;
    }
    try {
        qp.validate();
    } catch (const std::invalid_argument&) {
        result.status = QPSolverStatus::InvalidModel;
        return result;
    }
    if (qp.convexity == QPConvexityStatus::Unknown) {
        result.status = QPSolverStatus::UnsupportedNonconvex;
        return result;
    }
    const core::CSCMatrix& A = qp.lp_part.A;
    const int n = A.cols, m = A.rows;
    if (n == 0) {
        result.status = QPSolverStatus::InvalidModel;
        return result;
    }
    if (qp.lp_part.rhs.size() != static_cast<size_t>(m) || qp.lp_part.obj.size() != static_cast<size_t>(n) ||
        qp.H.col_ptrs.size() != static_cast<size_t>(n) + 1) {
        result.status = QPSolverStatus::InvalidModel;
        return result;
    }
    // H: diagonal or not (entries of the stored lower triangle)
    std::vector<double> hdiag(static_cast<size_t>(n), 0.0);
    bool diagonal = true;
    for (int j = 0; j < n; ++j)
        for (int p = qp.H.col_ptrs[j]; p < qp.H.col_ptrs[j + 1]; ++p) {
            const int i = qp.H.row_indices[p];
            if (i < 0 || i >= n) { result.status = QPSolverStatus::InvalidModel; return result; }
            if (i == j) hdiag[j] += qp.H.values[p];
            else if (qp.H.values[p] != 0.0) diagonal = false;
        }
    dev::QpProblem P;
    std::vector<std::vector<double>> F;
    if (diagonal) {
        P.m = m;
        P.n = n;
        P.col_ptrs.assign(A.col_ptrs.begin(), A.col_ptrs.end());
        P.row_idx.assign(A.row_indices.begin(), A.row_indices.end());
        P.vals.assign(A.values.begin(), A.values.end());
        P.b = qp.lp_part.rhs;
        P.c = qp.lp_part.obj;
        P.lb = qp.lp_part.lb;
        P.ub = qp.lp_part.ub;
        P.h = hdiag;
    } else {
        if (n > QP_MAX_LIFTED_COLS) {
            result.status = QPSolverStatus::InvalidModel;
            return result;
        }
        std::vector<double> Hd(static_cast<size_t>(n) * n, 0.0);
        for (int j = 0; j < n; ++j)
            for (int p = qp.H.col_ptrs[j]; p < qp.H.col_ptrs[j + 1]; ++p) {
                const int i = qp.H.row_indices[p];
                Hd[static_cast<size_t>(i) * n + j] += qp.H.values[p];
                if (i != j) Hd[static_cast<size_t>(j) * n + i] += qp.H.values[p];
            }
        F = pivoted_factor(n, Hd);
        const int r = static_cast<int>(F.size());
        // variables [x (n), w (r)], rows [A x = b (m), F x - w = 0 (r)]
        P.m = m + r;
        P.n = n + r;
        P.col_ptrs.assign(1, 0);
        for (int j = 0; j < n; ++j) {
            for (int p = A.col_ptrs[j]; p < A.col_ptrs[j + 1]; ++p) {
                P.row_idx.push_back(A.row_indices[p]);
                P.vals.push_back(A.values[p]);
            }
            for (int q = 0; q < r; ++q)
                if (F[q][j] != 0.0) {
                    P.row_idx.push_back(m + q);
                    P.vals.push_back(F[q][j]);
                }
            P.col_ptrs.push_back(static_cast<int>(P.row_idx.size()));
        }
        for (int q = 0; q < r; ++q) {
            P.row_idx.push_back(m + q);
            P.vals.push_back(-1.0);
            P.col_ptrs.push_back(static_cast<int>(P.row_idx.size()));
        }
        P.b = qp.lp_part.rhs;
        P.b.resize(static_cast<size_t>(m + r), 0.0);
        P.c = qp.lp_part.obj;
        P.c.resize(static_cast<size_t>(n + r), 0.0);
        P.lb = qp.lp_part.lb;
        P.lb.resize(static_cast<size_t>(n + r), -math::kInfinity);
        P.ub = qp.lp_part.ub;
        P.ub.resize(static_cast<size_t>(n + r), math::kInfinity);
        P.h.assign(static_cast<size_t>(n), 0.0);
        P.h.resize(static_cast<size_t>(n + r), 1.0);
    }
    dev::QpSettings s;
    s.feas_tol = options_.feasibility_tol;
    s.dual_tol = options_.dual_tol;
    s.grad_tol = options_.grad_tol;
    s.max_iter = options_.max_iterations;
    const dev::QpOutcome o = dev::solve_qp_device(P, s);
    result.status = static_cast<QPSolverStatus>(o.status);
    result.iterations = o.iterations;
    result.primal_residual = o.primal_residual;
    result.dual_residual = o.dual_residual;
    result.complementarity = o.complementarity;
    result.objective_value = o.objective;
    if (!o.x.empty()) {
        x_out.assign(o.x.begin(), o.x.begin() + n);
        y_out.assign(o.y.begin(), o.y.begin() + m);
        z_out.assign(o.z.begin(), o.z.begin() + n);
        if (!diagonal) {      // objective of the original QP: 1/2 x^T H x + c^T x
            double obj = 0.0;
            for (int j = 0; j < n; ++j) obj += qp.lp_part.obj[j] * x_out[j];
            for (int j = 0; j < n; ++j)
                for (int p = qp.H.col_ptrs[j]; p < qp.H.col_ptrs[j + 1]; ++p) {
                    const int i = qp.H.row_indices[p];
                    const double t = qp.H.values[p] * x_out[i] * x_out[j];
                    obj += i == j ? 0.5 * t : t;
                }
            result.objective_value = obj;
        }
    }
    return result;
}

QPSolverStatus QPSolver::solve(const QPModel& qp, std::vector<Float>& x, std::vector<Float>& y,
                               std::vector<Float>& z) {
    return solve_with_diagnostics(qp, x, y, z).status;
}

}  // namespace qp
}  // namespace sankhya
