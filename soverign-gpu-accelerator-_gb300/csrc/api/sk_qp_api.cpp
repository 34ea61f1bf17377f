// C ABI of the device convex QP solver (sk_qp_solve, include/sankhya/sk_ipm.h).
#include <cmath>
#include <vector>

#include "api/sk_error.hpp"
#include "qp/qp_solver.hpp"
#include "sankhya/sk_ipm.h"

using namespace sankhya;

extern "C" void sk_qp_options_default(sk_qp_options* o) {
    if (!o) return;
    o->feasibility_tol = math::kDefaultFeasibilityTol;
    o->dual_tol = math::kDefaultFeasibilityTol;
    o->grad_tol = 1e-6;
    o->max_iterations = 200;
}

extern "C" int sk_qp_solve(int m, int n, const int* a_col_ptrs, const int* a_row_idx, const double* a_vals,
                           const double* b, const double* c, const double* lb, const double* ub,
                           const int* h_col_ptrs, const int* h_row_idx, const double* h_vals, int convexity,
                           const sk_qp_options* opts, double* x, double* y, double* z, int* status, double* info) {
    api::clear_error();
    if (m < 0 || n <= 0 || !a_col_ptrs || (a_col_ptrs[n] > 0 && (!a_row_idx || !a_vals)) || (m > 0 && !b) || !c ||
        !h_col_ptrs || (h_col_ptrs[n] > 0 && (!h_row_idx || !h_vals)) || !x || !z || (m > 0 && !y) || !status ||
        convexity < SK_QP_CONVEXITY_UNKNOWN || convexity > SK_QP_NONCONVEX) {
        api::set_error("sk_qp_solve: invalid argument");
        return SK_ERR_INVALID;
    }
    try {
        qp::QPModel model;
        model.lp_part.sense = OptimizationSense::Minimize;
        model.lp_part.obj.assign(c, c + n);
        model.lp_part.rhs.assign(b ? b : c, b ? b + m : c);
        model.lp_part.lb.assign(static_cast<size_t>(n), 0.0);
        model.lp_part.ub.assign(static_cast<size_t>(n), math::kInfinity);
        if (lb) model.lp_part.lb.assign(lb, lb + n);
        if (ub) model.lp_part.ub.assign(ub, ub + n);
        model.lp_part.vtype.assign(static_cast<size_t>(n), VariableType::Continuous);
        const int anz = a_col_ptrs[n], hnz = h_col_ptrs[n];
        for (int j = 0; j < n; ++j)
            if (a_col_ptrs[j + 1] < a_col_ptrs[j] || h_col_ptrs[j + 1] < h_col_ptrs[j])
                throw api::sk_exception(SK_ERR_INVALID, "sk_qp_solve: column pointers must not decrease");
        for (int q = 0; q < anz; ++q)
            if (a_row_idx[q] < 0 || a_row_idx[q] >= m || !std::isfinite(a_vals[q]))
                throw api::sk_exception(SK_ERR_INVALID, "sk_qp_solve: bad entry of A");
        for (int q = 0; q < hnz; ++q)
            if (h_row_idx[q] < 0 || h_row_idx[q] >= n || !std::isfinite(h_vals[q]))
                throw api::sk_exception(SK_ERR_INVALID, "sk_qp_solve: bad entry of H");
        for (int j = 0; j < n; ++j)
            for (int q = h_col_ptrs[j]; q < h_col_ptrs[j + 1]; ++q)
                if (h_row_idx[q] < j)
                    throw api::sk_exception(SK_ERR_INVALID, "sk_qp_solve: H must hold its lower triangle only");
        model.lp_part.A = core::CSCMatrix(m, n, std::vector<Float>(a_vals, a_vals + anz),
                                          std::vector<Index>(a_row_idx, a_row_idx + anz),
                                          std::vector<Index>(a_col_ptrs, a_col_ptrs + n + 1));
        model.H = core::CSCMatrix(n, n, std::vector<Float>(h_vals, h_vals + hnz),
                                  std::vector<Index>(h_row_idx, h_row_idx + hnz),
                                  std::vector<Index>(h_col_ptrs, h_col_ptrs + n + 1));
        model.convexity = static_cast<qp::QPConvexityStatus>(convexity);
        qp::QPSolver::Options o;
        if (opts) {
            o.feasibility_tol = opts->feasibility_tol;
            o.dual_tol = opts->dual_tol;
            o.grad_tol = opts->grad_tol;
            o.max_iterations = opts->max_iterations;
        }
        std::vector<Float> xv, yv, zv;
        const qp::QPResult r = qp::QPSolver(o).solve_with_diagnostics(model, xv, yv, zv);
        *status = static_cast<int>(r.status);
        if (xv.size() == static_cast<size_t>(n)) {
            for (int j = 0; j < n; ++j) { x[j] = xv[j]; z[j] = zv[j]; }
            for (int i = 0; i < m; ++i) y[i] = yv[i];
        }
        if (info) {
            info[0] = r.objective_value;
            info[1] = r.iterations;
            info[2] = r.primal_residual;
            info[3] = r.dual_residual;
            info[4] = r.complementarity;
        }
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}
