// C entry points over the reference's own CPU code, compiled from the reference
// sources where they lie (see Makefile target `ref`). TEST INFRASTRUCTURE ONLY:
// the reference is used here as a checker (symbolic analysis, simplex objective,
// certificate) and as the timed CPU baseline; nothing in the product links it.
#include <cmath>
#include <cstring>
#include <vector>

#include "core/problem.hpp"
#include "core/sparse_matrix.hpp"
#include "ipm/symbolic.hpp"
#include "numerics/sparse_lu.hpp"
#include "presolve/scaling.hpp"
#include "qp/qp_model.hpp"
#include "qp/qp_solver.hpp"
#include "simplex/phase1.hpp"
#include "verifier/certificate.hpp"

using namespace sankhya;

static core::CSRMatrix csr_of(int m, int n, const int* rp, const int* ci) {
    core::CSRMatrix A;
    A.rows = m;
    A.cols = n;
    A.row_ptrs.assign(rp, rp + m + 1);
    A.col_indices.assign(ci, ci + rp[m]);
    A.values.assign(static_cast<size_t>(rp[m]), 1.0);
    return A;
}

static core::Model model_of(int m, int n, const int* cp, const int* ri, const double* va,
                            const double* b, const double* c) {
    core::Model model;
    for (int j = 0; j < n; ++j) model.add_variable(c[j]);
    std::vector<std::vector<Index>> rc(static_cast<size_t>(m));
    std::vector<std::vector<Float>> rv(static_cast<size_t>(m));
    for (int j = 0; j < n; ++j)
        for (int k = cp[j]; k < cp[j + 1]; ++k) {
            rc[static_cast<size_t>(ri[k])].push_back(j);
            rv[static_cast<size_t>(ri[k])].push_back(va[k]);
        }
    for (int i = 0; i < m; ++i) model.add_constraint(rc[static_cast<size_t>(i)], rv[static_cast<size_t>(i)], b[i]);
    model.finalize();
    return model;
}

extern "C" {

int ref_min_degree(int m, int n, const int* rp, const int* ci, int* P) {
    try {
        auto p = ipm::compute_amd_ordering(csr_of(m, n, rp, ci));
        std::memcpy(P, p.data(), sizeof(int) * static_cast<size_t>(m));
        return 0;
    } catch (...) {
        return -1;
    }
}

int ref_symbolic(int m, int n, const int* rp, const int* ci, const int* P, int* P_inv, int* parent,
                 int* L_rp, int* L_ci, int cap) {
    try {
        ipm::SymbolicFactorization sym;
        std::vector<Index> pv(P, P + m);
        ipm::compute_symbolic_factorization(csr_of(m, n, rp, ci), pv, sym);
        const int nnz = sym.L_pattern.row_ptrs[static_cast<size_t>(m)];
        if (nnz > cap) return -1;
        std::memcpy(P_inv, sym.P_inv.data(), sizeof(int) * static_cast<size_t>(m));
        std::memcpy(parent, sym.parent.data(), sizeof(int) * static_cast<size_t>(m));
        std::memcpy(L_rp, sym.L_pattern.row_ptrs.data(), sizeof(int) * static_cast<size_t>(m + 1));
        std::memcpy(L_ci, sym.L_pattern.col_indices.data(), sizeof(int) * static_cast<size_t>(nnz));
        return nnz;
    } catch (...) {
        return -2;
    }
}

// Phase-I + primal simplex with the reference's sparse LU; returns the
// SimplexStatus as int (0 Optimal), objective and x.
int ref_simplex_solve(int m, int n, const int* cp, const int* ri, const double* va, const double* b,
                      const double* c, double* x_out, double* obj) {
    try {
        core::Model model = model_of(m, n, cp, ri, va, b, c);
        simplex::Basis basis;
        std::vector<Float> x;
        numerics::SparseLUFactorization lu;
        auto st = simplex::solve_with_phase1(model, basis, x, lu);
        double o = 0.0;
        for (size_t j = 0; j < x.size(); ++j) o += x[j] * model.obj[j];
        if (obj) *obj = o;
        if (x_out && x.size() == static_cast<size_t>(n)) std::memcpy(x_out, x.data(), sizeof(double) * static_cast<size_t>(n));
        return static_cast<int>(st);
    } catch (...) {
        return -1;
    }
}

int ref_verify_optimal(int m, int n, const int* cp, const int* ri, const double* va, const double* b,
                       const double* c, const double* x, const double* pi) {
    try {
        core::Model model = model_of(m, n, cp, ri, va, b, c);
        std::vector<Float> xv(x, x + n), pv(pi, pi + m);
        return verifier::verify_optimal(model, xv, pv) ? 1 : 0;
    } catch (...) {
        return -1;
    }
}

// The reference's presolve::apply_ruiz_scaling on the model built from the CSC
// arrays (bounds and integer flags included); writes back the scaled CSC values,
// b, c, lb, ub and the scale vectors. Returns -2 if the reference's CSC order
// differs from the input's (rows must be sorted within each column).
int ref_ruiz_scaling(int m, int n, const int* cp, const int* ri, const double* va, const double* b, const double* c,
                     const double* lb, const double* ub, const unsigned char* is_int, int max_iter,
                     double* vals_out, double* b_out, double* c_out, double* lb_out, double* ub_out,
                     double* row_scale, double* col_scale) {
    try {
        core::Model model;
        for (int j = 0; j < n; ++j)
            model.add_variable(c[j], lb[j], ub[j], is_int[j] ? VariableType::Integer : VariableType::Continuous);
        std::vector<std::vector<Index>> rc(static_cast<size_t>(m));
        std::vector<std::vector<Float>> rv(static_cast<size_t>(m));
        for (int j = 0; j < n; ++j)
            for (int k = cp[j]; k < cp[j + 1]; ++k) {
                rc[static_cast<size_t>(ri[k])].push_back(j);
                rv[static_cast<size_t>(ri[k])].push_back(va[k]);
            }
        for (int i = 0; i < m; ++i) model.add_constraint(rc[static_cast<size_t>(i)], rv[static_cast<size_t>(i)], b[i]);
        model.finalize();
        for (int j = 0; j <= n; ++j)
            if (model.A.col_ptrs[static_cast<size_t>(j)] != cp[j]) return -2;
        for (int k = 0; k < cp[n]; ++k)
            if (model.A.row_indices[static_cast<size_t>(k)] != ri[k]) return -2;
        presolve::apply_ruiz_scaling(model, max_iter);
        std::memcpy(vals_out, model.A.values.data(), sizeof(double) * static_cast<size_t>(cp[n]));
        std::memcpy(b_out, model.rhs.data(), sizeof(double) * static_cast<size_t>(m));
        std::memcpy(c_out, model.obj.data(), sizeof(double) * static_cast<size_t>(n));
        std::memcpy(lb_out, model.lb.data(), sizeof(double) * static_cast<size_t>(n));
        std::memcpy(ub_out, model.ub.data(), sizeof(double) * static_cast<size_t>(n));
        std::memcpy(row_scale, model.row_scale.data(), sizeof(double) * static_cast<size_t>(m));
        std::memcpy(col_scale, model.col_scale.data(), sizeof(double) * static_cast<size_t>(n));
        return 0;
    } catch (...) {
        return -1;
    }
}

// The reference's qp::QPSolver::solve_with_diagnostics on a QP given densely
// (H n x n row-major, symmetric; A m x n row-major), modelled as the reference's
// own QP tests model it (H's lower triangle in CSC, entries above 1e-15 in
// magnitude; convexity ConvexPSD). Writes x, y, z (when the solver returns them)
// and info = {objective, iterations, primal_residual, dual_residual,
// complementarity}; returns the QPSolverStatus as int (-1 on an exception).
int ref_qp_solve(int n, int m, const double* H, const double* c, const double* A, const double* b,
                 const double* lb, const double* ub, int max_iter, double* x_out, double* y_out, double* z_out,
                 double* info) {
    try {
        qp::QPModel qp;
        qp.lp_part.sense = OptimizationSense::Minimize;
        qp.lp_part.obj.assign(c, c + n);
        qp.lp_part.lb.assign(lb, lb + n);
        qp.lp_part.ub.assign(ub, ub + n);
        qp.lp_part.rhs.assign(b, b + m);
        qp.lp_part.vtype.assign(static_cast<size_t>(n), VariableType::Continuous);
        std::vector<Index> cp(static_cast<size_t>(n) + 1, 0), ri;
        std::vector<Float> va;
        for (int j = 0; j < n; ++j) {
            cp[static_cast<size_t>(j)] = static_cast<Index>(ri.size());
            for (int i = 0; i < m; ++i) {
                const double v = A[static_cast<size_t>(i) * n + j];
                if (std::abs(v) > 1e-15) { ri.push_back(i); va.push_back(v); }
            }
        }
        cp[static_cast<size_t>(n)] = static_cast<Index>(ri.size());
        qp.lp_part.A = core::CSCMatrix(m, n, va, ri, cp);
        std::vector<Index> hp(static_cast<size_t>(n) + 1, 0), hr;
        std::vector<Float> hv;
        for (int j = 0; j < n; ++j) {
            hp[static_cast<size_t>(j)] = static_cast<Index>(hr.size());
            for (int i = j; i < n; ++i) {
                const double v = H[static_cast<size_t>(i) * n + j];
                if (std::abs(v) > 1e-15) { hr.push_back(i); hv.push_back(v); }
            }
        }
        hp[static_cast<size_t>(n)] = static_cast<Index>(hr.size());
        qp.H = core::CSCMatrix(n, n, hv, hr, hp);
        qp.convexity = qp::QPConvexityStatus::ConvexPSD;
        qp::QPSolver::Options opts;
        opts.max_iterations = max_iter;
        qp::QPSolver solver(opts);
        std::vector<Float> x, y, z;
        auto r = solver.solve_with_diagnostics(qp, x, y, z);
        if (x.size() == static_cast<size_t>(n)) std::memcpy(x_out, x.data(), sizeof(double) * static_cast<size_t>(n));
        if (y.size() == static_cast<size_t>(m) && m > 0) std::memcpy(y_out, y.data(), sizeof(double) * static_cast<size_t>(m));
        if (z.size() == static_cast<size_t>(n)) std::memcpy(z_out, z.data(), sizeof(double) * static_cast<size_t>(n));
        info[0] = r.objective_value;
        info[1] = r.iterations;
        info[2] = r.primal_residual;
        info[3] = r.dual_residual;
        info[4] = r.complementarity;
        return static_cast<int>(r.status);
    } catch (...) {
        return -1;
    }
}

}  // extern "C"
