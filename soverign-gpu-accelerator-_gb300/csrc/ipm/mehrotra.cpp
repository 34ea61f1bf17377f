// MehrotraSolver: the reference-compatible C++ front end over the C ABI.
#include "ipm/mehrotra.hpp"

#include "core/standard_form.hpp"

#include <new>
#include <stdexcept>
#include <string>

namespace sankhya {
namespace ipm {

namespace {

sk_options to_c(const MehrotraOptions& o) {
    sk_options c;
    sk_options_default(&c);
    c.precision = o.precision;
    c.start = o.start;
    c.criteria = o.criteria;
    c.tol = o.tol;
    c.max_iter = o.max_iter;
    c.ordering = o.ordering;
    c.verbose = o.verbose;
    c.mu_switch = o.mu_switch;
    c.ruiz_passes = o.ruiz_passes;
    c.strict = o.strict;
    c.delta32 = o.delta32;
    c.delta64 = o.delta64;
    c.fp64_update = o.fp64_update;
    c.dependent_rows = o.dependent_rows;
    return c;
}

[[noreturn]] void raise(int rc, const char* where) {
    const std::string msg = std::string(where) + ": " + sk_last_error();
    if (rc == SK_ERR_ALLOC) throw std::bad_alloc();
    if (rc == SK_ERR_INVALID || rc == SK_ERR_TOO_LARGE) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

MehrotraResult to_result(const sk_info& info, std::vector<Float>&& x, std::vector<Float>&& y, std::vector<Float>&& s) {
    MehrotraResult r;
    r.status = static_cast<simplex::SimplexStatus>(info.status);
    r.objective_value = info.objective;
    r.iterations = info.iterations;
    r.primal_residual = info.primal_residual;
    r.dual_residual = info.dual_residual;
    r.duality_gap = info.duality_gap;
    r.x = std::move(x);
    r.pi = std::move(y);
    r.s = std::move(s);
    r.info = info;
    return r;
}

}  // namespace

class MehrotraSolver::Impl {
public:
    Impl(const core::Model& md, const MehrotraOptions& o) : model(md), opts(o) {
        if (model.A.rows <= 0 || model.A.cols <= 0) throw std::invalid_argument("MehrotraSolver: empty model");
        if (model.rhs.size() != static_cast<size_t>(model.A.rows) || model.obj.size() != static_cast<size_t>(model.A.cols))
            throw std::invalid_argument("MehrotraSolver: model dimensions inconsistent");
        const Float sign = model.sense == OptimizationSense::Maximize ? -1.0 : 1.0;
        cost.resize(model.obj.size());
        for (size_t j = 0; j < cost.size(); ++j) cost[j] = sign * model.obj[j];
        const sk_options c = to_c(opts);
        int m = model.A.rows, n = model.A.cols;
        const int* cp = model.A.col_ptrs.data();
        const int* ri = model.A.row_indices.data();
        const double* va = model.A.values.data();
        const double* b = model.rhs.data();
        const double* cc = cost.data();
        if (opts.honor_bounds) {
            if (model.lb.size() != static_cast<size_t>(n) || model.ub.size() != static_cast<size_t>(n))
                throw std::invalid_argument("MehrotraSolver: bounds need one entry per column");
            bl.m = m; bl.n = n; bl.col_ptrs = cp; bl.row_idx = ri; bl.vals = va; bl.b = b; bl.c = cc;
            bl.lb = model.lb.data(); bl.ub = model.ub.data();
            sf = core::to_standard_form(bl);
            m = sf.m; n = sf.n;
            cp = sf.col_ptrs.data(); ri = sf.row_idx.data(); va = sf.vals.data(); b = sf.b.data(); cc = sf.c.data();
        }
        const int rc = sk_solver_create(1, &m, &n, &cp, &ri, &va, &b, &cc, &c, &handle);
        if (rc != SK_OK) raise(rc, "MehrotraSolver");
    }
    ~Impl() { sk_solver_destroy(handle); }

    MehrotraResult solve() {
        int rc = sk_solver_run(handle);
        if (rc != SK_OK) raise(rc, "MehrotraSolver::solve");
        std::vector<Float> x(static_cast<size_t>(model.A.cols)), y(static_cast<size_t>(model.A.rows)),
            s(static_cast<size_t>(model.A.cols));
        sk_info info{};
        if (opts.honor_bounds) {
            std::vector<Float> xs(static_cast<size_t>(sf.n)), ys(static_cast<size_t>(sf.m)), ss(static_cast<size_t>(sf.n));
            rc = sk_solver_result(handle, 0, xs.data(), ys.data(), ss.data(), &info);
            if (rc != SK_OK) raise(rc, "MehrotraSolver::solve");
            info.objective = core::recover_solution(bl, sf, xs.data(), ys.data(), x.data(), y.data(), s.data());
        } else {
            rc = sk_solver_result(handle, 0, x.data(), y.data(), s.data(), &info);
            if (rc != SK_OK) raise(rc, "MehrotraSolver::solve");
        }
        if (model.sense == OptimizationSense::Maximize) {
            info.objective = -info.objective;
            for (auto& v : y) v = -v;
            for (auto& v : s) v = -v;
        }
        return to_result(info, std::move(x), std::move(y), std::move(s));
    }

    const core::Model& model;
    MehrotraOptions opts;
    std::vector<Float> cost;
    core::BoundedLp bl;
    core::StandardForm sf;
    sk_solver* handle = nullptr;
};

MehrotraSolver::MehrotraSolver(const core::Model& model) : impl_(new Impl(model, MehrotraOptions())) {}
MehrotraSolver::MehrotraSolver(const core::Model& model, const MehrotraOptions& opts) : impl_(new Impl(model, opts)) {}
MehrotraSolver::~MehrotraSolver() { delete impl_; }
MehrotraResult MehrotraSolver::solve() { return impl_->solve(); }

std::vector<MehrotraResult> solve_batch(const std::vector<const core::Model*>& models, const MehrotraOptions& opts) {
    const int k = static_cast<int>(models.size());
    if (k == 0) return {};
    std::vector<int> m(k), n(k);
    std::vector<const int*> cp(k), ri(k);
    std::vector<const double*> va(k), b(k), c(k);
    std::vector<std::vector<Float>> cost(k);
    for (int t = 0; t < k; ++t) {
        const core::Model& md = *models[t];
        m[t] = md.A.rows;
        n[t] = md.A.cols;
        cp[t] = md.A.col_ptrs.data();
        ri[t] = md.A.row_indices.data();
        va[t] = md.A.values.data();
        b[t] = md.rhs.data();
        const Float sign = md.sense == OptimizationSense::Maximize ? -1.0 : 1.0;
        cost[t].resize(md.obj.size());
        for (size_t j = 0; j < md.obj.size(); ++j) cost[t][j] = sign * md.obj[j];
        c[t] = cost[t].data();
    }
    const sk_options co = to_c(opts);
    sk_solver* h = nullptr;
    int rc = sk_solver_create(k, m.data(), n.data(), cp.data(), ri.data(), va.data(), b.data(), c.data(), &co, &h);
    if (rc != SK_OK) raise(rc, "solve_batch");
    rc = sk_solver_run(h);
    if (rc != SK_OK) { sk_solver_destroy(h); raise(rc, "solve_batch"); }
    std::vector<MehrotraResult> out;
    for (int t = 0; t < k; ++t) {
        std::vector<Float> x(static_cast<size_t>(n[t])), y(static_cast<size_t>(m[t])), s(static_cast<size_t>(n[t]));
        sk_info info{};
        rc = sk_solver_result(h, t, x.data(), y.data(), s.data(), &info);
        if (rc != SK_OK) { sk_solver_destroy(h); raise(rc, "solve_batch"); }
        if (models[t]->sense == OptimizationSense::Maximize) {
            info.objective = -info.objective;
            for (auto& v : y) v = -v;
            for (auto& v : s) v = -v;
        }
        out.push_back(to_result(info, std::move(x), std::move(y), std::move(s)));
    }
    sk_solver_destroy(h);
    return out;
}

}  // namespace ipm
}  // namespace sankhya
