// Device-side C ABI entry points (include/sankhya/sk_ipm.h): one-shot and
// persistent IPM solves, the KKT engine and the SpMV kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <memory>
#include <vector>

#include "api/sk_error.hpp"
#include "core/standard_form.hpp"
#include "cuda/autotune.hpp"
#include "cuda/crossover.hpp"
#include "cuda/device_ipm.hpp"
#include "cuda/gnn.hpp"
#include "cuda/kkt_engine.hpp"
#include "ipm/front_plan.hpp"
#include "sankhya/sk_ipm.h"

using namespace sankhya;

namespace {
// An LP with its linearly dependent rows dropped (sk_options.dependent_rows): the kept
// rows' CSC arrays and right-hand side, and the original index of each kept row.
struct ReducedLp {
    std::vector<int> rows;         // original row of each kept row; empty: LP not reduced
    std::vector<int> cp, ri;
    std::vector<double> v, b;
    int m_orig = 0;
    // the dropped rows' entries (row, column, value) and right-hand sides, to measure
    // their residual at the solution; binf = 1 + ||b||_inf of the original LP
    std::vector<int> drop_row, drop_col;
    std::vector<double> drop_val, drop_b;
    double binf = 1.0;
    bool reduced() const { return !rows.empty(); }
};
}  // namespace

struct sk_solver {
    std::unique_ptr<dev::DeviceIPM> ipm;
    std::vector<ReducedLp> red;    // per LP
};

struct sk_gnn {
    std::unique_ptr<dev::Gnn> net;
    cudaStream_t st = nullptr;
    ~sk_gnn() {
        net.reset();
        if (st) cudaStreamDestroy(st);
    }
};

// One graph (or a solver's whole batch) resident on the device, with targets.
struct sk_gnn_batch {
    dev::Arena arena;
    dev::Slot<int> a_rp, a_ci, t_rp, t_ci;
    dev::Slot<double> a_v, t_v, b, c, tlx, tls, ty;
    dev::DeviceLP lp;
    bool has_targets = false;
};

struct sk_kkt {
    int m = 0, n = 0, precision = 0;
    cudaStream_t st = nullptr;
    dev::Arena arena;
    dev::Slot<int> a_rp, a_ci, t_rp, t_ci, row_lp, col_lp;
    dev::Slot<double> a_v, t_v, theta, out, r, corr, bak, tmp, scratch, hostio;
    dev::DeviceLP lp;
    std::unique_ptr<dev::KktEngine> eng;
    bool factored = false;
    ~sk_kkt() {
        eng.reset();
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

sk_options opts_or_default(const sk_options* o) {
    sk_options d;
    sk_options_default(&d);
    return o ? *o : d;
}

void check_options(const sk_options& o) {
    if (o.precision != SK_PREC_FP64 && o.precision != SK_PREC_MIXED) throw std::invalid_argument("bad precision");
    if (o.start < SK_START_UNIT || o.start > SK_START_LEARNED) throw std::invalid_argument("bad start");
    if (o.criteria != SK_CRIT_RELATIVE && o.criteria != SK_CRIT_REFERENCE) throw std::invalid_argument("bad criteria");
    if (!(o.tol > 0.0) || o.max_iter < 0 || o.ruiz_passes < 0) throw std::invalid_argument("bad tolerance / limits");
    if (!(o.learned_accept >= 0.0)) throw std::invalid_argument("bad learned_accept");
    if (o.fp64_update < SK_FP64_UPDATE_AUTO || o.fp64_update > SK_FP64_UPDATE_TENSOR)
        throw std::invalid_argument("bad fp64_update");
    if (o.ordering < SK_ORDER_AUTO || o.ordering > SK_ORDER_DISSECTION) throw std::invalid_argument("bad ordering");
    if (o.dependent_rows != 0 && o.dependent_rows != 1) throw std::invalid_argument("bad dependent_rows");
}

void check_csc(int m, int n, const int* cp, const int* ri, const double* v, const double* b, const double* c) {
    if (m <= 0 || n <= 0 || !cp || !b || !c) throw std::invalid_argument("invalid LP arrays");
    if (cp[0] != 0) throw std::invalid_argument("col_ptrs[0] != 0");
    for (int j = 0; j < n; ++j) if (cp[j + 1] < cp[j]) throw std::invalid_argument("col_ptrs not monotone");
    if (cp[n] > 0 && (!ri || !v)) throw std::invalid_argument("invalid LP arrays");
}

// ---- linearly dependent rows of A ------------------------------------------------
// A A^T is factored on the device in FP64 (the KKT engine: equilibrated to a unit
// diagonal, delta from 1e-12) in its fill-reducing elimination order. The pivot L_kk^2
// of a row is its squared distance (rows normalised) from the span of the rows
// eliminated before it: 0 in exact arithmetic for a dependent row. Through the normal
// equations that distance carries FP64 rounding of about 1e-9 (a 2000-row dependency
// of a staircase LP gives 1.3e-9 and 3.2e-9 against 0.29 for the smallest independent
// row, dense FP64 Cholesky), so a row with L_kk^2 <= kDepPivot (or 10 delta) counts as
// dependent. b is consistent with A when b - A A^T w is ~0 for w from the regularised
// factor with iterative refinement (which converges on the range of A A^T, and leaves
// the part of b outside it, the inconsistency, in the residual).
constexpr double kDepPivot = 1e-6;
constexpr double kConsistent = 1e-9;   // inconsistency at which dependent rows are dropped

struct DependentRows {
    std::vector<char> dependent;
    int count = 0;
    double inconsistency = 0.0;        // ||b - A A^T w||_inf / (1 + ||b||_inf)
};

DependentRows find_dependent_rows(int m, int n, const int* cp, const int* ri, const double* v, const double* b) {
    DependentRows out;
    out.dependent.assign(static_cast<size_t>(m), 0);
    const int nz = cp[n];
    std::vector<int> rp(static_cast<size_t>(m) + 1, 0), ci(static_cast<size_t>(nz));
    std::vector<double> cv(static_cast<size_t>(nz));
    for (int q = 0; q < nz; ++q) {
        if (ri[q] < 0 || ri[q] >= m) throw std::invalid_argument("row index out of range");
        if (!std::isfinite(v[q])) throw std::invalid_argument("non-finite entry of A");
        rp[ri[q] + 1]++;
    }
    for (int i = 0; i < m; ++i) {
        if (!std::isfinite(b[i])) throw std::invalid_argument("non-finite entry of b");
        rp[i + 1] += rp[i];
    }
    std::vector<int> nx(rp.begin(), rp.end() - 1);
    for (int j = 0; j < n; ++j)
        for (int q = cp[j]; q < cp[j + 1]; ++q) {
            const int d = nx[ri[q]]++;
            ci[d] = j;
            cv[d] = v[q];
        }
    sk_kkt* raw = nullptr;
    const int rc = sk_kkt_create(m, n, rp.data(), ci.data(), cv.data(), nullptr, SK_PREC_FP64, &raw);
    if (rc != SK_OK) throw api::sk_exception(rc, std::string("dependent rows: ") + sk_last_error());
    std::unique_ptr<sk_kkt> k(raw);
    dev::KktEngine& E = *k->eng;
    cudaStream_t st = k->st;
    const std::vector<double> ones(static_cast<size_t>(n), 1.0);
    SK_CUDA(cudaMemcpyAsync(k->theta.ptr, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    double delta = 1e-12;
    bool ok = false;
    for (int t = 0; t < 6; ++t) {
        if ((ok = E.factor(k->theta.ptr, delta, false))) break;
        delta *= 10.0;
    }
    if (!ok) throw api::sk_exception(SK_ERR_NUMERICAL, "dependent rows: A A^T could not be factored");
    const double tau = std::max(kDepPivot, 10.0 * delta);
    const std::vector<double> piv = E.pivots_host();
    const auto& perm = E.plan().perm;
    for (int q = 0; q < m; ++q)
        if (!(piv[q] * piv[q] > tau)) {
            out.dependent[perm[q]] = 1;
            ++out.count;
        }
    // consistency: iterative refinement of (A A^T) w = b on the regularised factor
    double binf = 0.0;
    for (int i = 0; i < m; ++i) binf = std::max(binf, std::fabs(b[i]));
    std::vector<double> w(static_cast<size_t>(m), 0.0), r(b, b + m), h(static_cast<size_t>(m));
    double best = binf;
    for (int it = 0; it < 12 && best > 1e-15 * (1.0 + binf); ++it) {
        SK_CUDA(cudaMemcpyAsync(k->hostio.ptr, r.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
        E.apply_inverse(k->hostio.ptr, k->out.ptr);
        SK_CUDA(cudaMemcpyAsync(h.data(), k->out.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < m; ++i) w[i] += h[i];
        SK_CUDA(cudaMemcpyAsync(k->hostio.ptr, w.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
        E.apply_normal(k->theta.ptr, k->hostio.ptr, k->out.ptr);
        SK_CUDA(cudaMemcpyAsync(h.data(), k->out.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
        double rn = 0.0;
        for (int i = 0; i < m; ++i) {
            r[i] = b[i] - h[i];
            rn = std::max(rn, std::fabs(r[i]));
        }
        if (!(rn < best)) break;
        best = rn;
    }
    if (E.solve_error()) throw api::sk_exception(SK_ERR_CUDA, "dependent rows: triangular solve timed out");
    out.inconsistency = best / (1.0 + binf);
    return out;
}

// With o.dependent_rows set: the LP's dependent rows are looked for and, when b is
// consistent, dropped; red then holds the kept rows and view / bptr point at them.
void reduce_lp(const sk_options& o, int m, int n, const int* cp, const int* ri, const double* v, const double* b,
               ReducedLp& red, ipm::LpView& view, const double*& bptr) {
    view.m = m; view.n = n; view.col_ptrs = cp; view.row_idx = ri; view.vals = v;
    bptr = b;
    red = ReducedLp();
    red.m_orig = m;
    if (!o.dependent_rows) return;
    const DependentRows d = find_dependent_rows(m, n, cp, ri, v, b);
    if (d.count == 0 || d.count >= m || d.inconsistency > kConsistent) return;
    std::vector<int> newrow(static_cast<size_t>(m), -1), droprow(static_cast<size_t>(m), -1);
    for (int i = 0; i < m; ++i) {
        red.binf = std::max(red.binf, 1.0 + std::fabs(b[i]));
        if (!d.dependent[i]) {
            newrow[i] = static_cast<int>(red.rows.size());
            red.rows.push_back(i);
            red.b.push_back(b[i]);
        } else {
            droprow[i] = static_cast<int>(red.drop_b.size());
            red.drop_b.push_back(b[i]);
        }
    }
    red.cp.assign(1, 0);
    for (int j = 0; j < n; ++j) {
        for (int q = cp[j]; q < cp[j + 1]; ++q)
            if (newrow[ri[q]] >= 0) {
                red.ri.push_back(newrow[ri[q]]);
                red.v.push_back(v[q]);
            } else {
                red.drop_row.push_back(droprow[ri[q]]);
                red.drop_col.push_back(j);
                red.drop_val.push_back(v[q]);
            }
        red.cp.push_back(static_cast<int>(red.ri.size()));
    }
    view.m = static_cast<int>(red.rows.size());
    view.col_ptrs = red.cp.data();
    view.row_idx = red.ri.data();
    view.vals = red.v.data();
    bptr = red.b.data();
    if (o.verbose)
        std::fprintf(stderr, "[sk] %d dependent rows dropped (inconsistency %.2e)\n", d.count, d.inconsistency);
}

// Result of LP lp of a solver whose LP may have been reduced: y of the dropped rows is 0,
// and info->rel_pinf also covers the dropped rows' residuals at x (the original LP).
void reduced_result(const dev::DeviceIPM& ipm, const ReducedLp& red, int lp, double* x, double* y, double* s,
                    sk_info* info) {
    if (!red.reduced()) {
        ipm.result(lp, x, y, s, info);
        if (info) info->dependent_rows = 0;
        return;
    }
    std::vector<double> yr(red.rows.size());
    std::vector<double> xl;
    if (!x && info) xl.resize(static_cast<size_t>(ipm.plan().col_off[lp + 1] - ipm.plan().col_off[lp]));
    double* xv = x ? x : (xl.empty() ? nullptr : xl.data());
    ipm.result(lp, xv, y ? yr.data() : nullptr, s, info);
    if (info && xv) {
        std::vector<double> r(red.drop_b.size());
        for (size_t q = 0; q < red.drop_row.size(); ++q) r[red.drop_row[q]] += red.drop_val[q] * xv[red.drop_col[q]];
        double rmax = 0.0;
        for (size_t q = 0; q < r.size(); ++q) rmax = std::max(rmax, std::fabs(r[q] - red.drop_b[q]));
        info->rel_pinf = std::max(info->rel_pinf, rmax / red.binf);
    }
    if (y) {
        std::fill(y, y + red.m_orig, 0.0);
        for (size_t q = 0; q < red.rows.size(); ++q) y[red.rows[q]] = yr[q];
    }
    if (info) info->dependent_rows = red.m_orig - static_cast<int>(red.rows.size());
}

}  // namespace

extern "C" {

int sk_ipm_solve_csc(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, const double* b,
                     const double* c, const sk_options* opt, double* x, double* y, double* s, sk_info* info) {
    api::clear_error();
    try {
        const sk_options o = opts_or_default(opt);
        check_options(o);
        check_csc(m, n, col_ptrs, row_idx, vals, b, c);
        ipm::LpView v;
        ReducedLp red;
        const double* bp = b;
        reduce_lp(o, m, n, col_ptrs, row_idx, vals, b, red, v, bp);
        dev::DeviceIPM solver({v}, {bp}, {c}, o);
        solver.run();
        reduced_result(solver, red, 0, x, y, s, info);
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_ipm_solve_bounded(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                         const double* b, const double* c, const double* lb, const double* ub, const sk_options* opt,
                         double* x, double* y, double* s, sk_info* info) {
    api::clear_error();
    try {
        const sk_options o = opts_or_default(opt);
        check_options(o);
        check_csc(m, n, col_ptrs, row_idx, vals, b, c);
        core::BoundedLp bl;
        bl.m = m; bl.n = n; bl.col_ptrs = col_ptrs; bl.row_idx = row_idx; bl.vals = vals; bl.b = b; bl.c = c;
        bl.lb = lb; bl.ub = ub;
        const core::StandardForm sf = core::to_standard_form(bl);
        ipm::LpView v;
        ReducedLp red;
        const double* bp = nullptr;
        reduce_lp(o, sf.m, sf.n, sf.col_ptrs.data(), sf.row_idx.data(), sf.vals.data(), sf.b.data(), red, v, bp);
        dev::DeviceIPM solver({v}, {bp}, {sf.c.data()}, o);
        solver.run();
        std::vector<double> xs(sf.n), ys(sf.m), ss(sf.n);
        sk_info in{};
        reduced_result(solver, red, 0, xs.data(), ys.data(), ss.data(), &in);
        const double obj = core::recover_solution(bl, sf, xs.data(), ys.data(), x, y, s);
        in.objective = obj;
        if (info) *info = in;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_solver_create(int num_lps, const int* m, const int* n, const int* const* col_ptrs, const int* const* row_idx,
                     const double* const* vals, const double* const* b, const double* const* c, const sk_options* opt,
                     sk_solver** out) {
    api::clear_error();
    if (!out || num_lps <= 0 || !m || !n || !col_ptrs || !row_idx || !vals || !b || !c) return SK_ERR_INVALID;
    try {
        const sk_options o = opts_or_default(opt);
        check_options(o);
        std::vector<ipm::LpView> views(num_lps);
        std::vector<const double*> bv(num_lps), cv(num_lps);
        std::vector<ReducedLp> red(num_lps);
        for (int k = 0; k < num_lps; ++k) check_csc(m[k], n[k], col_ptrs[k], row_idx[k], vals[k], b[k], c[k]);
        for (int k = 0; k < num_lps; ++k) {
            reduce_lp(o, m[k], n[k], col_ptrs[k], row_idx[k], vals[k], b[k], red[k], views[k], bv[k]);
            cv[k] = c[k];
        }
        auto* h = new sk_solver;
        h->red = std::move(red);
        try {
            h->ipm.reset(new dev::DeviceIPM(views, bv, cv, o));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_solver_set_start(sk_solver* h, int lp, const double* x, const double* y, const double* s) {
    api::clear_error();
    if (!h) return SK_ERR_INVALID;
    try {
        if (lp < 0 || lp >= h->ipm->num_lps()) return SK_ERR_INVALID;
        const ReducedLp& red = h->red[lp];
        if (red.reduced() && y) {    // the start's y restricted to the kept rows
            std::vector<double> yr(red.rows.size());
            for (size_t q = 0; q < red.rows.size(); ++q) yr[q] = y[red.rows[q]];
            h->ipm->set_start(lp, x, yr.data(), s);
        } else {
            h->ipm->set_start(lp, x, y, s);
        }
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_solver_run(sk_solver* h) {
    api::clear_error();
    if (!h) return SK_ERR_INVALID;
    try {
        h->ipm->run();
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_solver_result(sk_solver* h, int lp, double* x, double* y, double* s, sk_info* info) {
    api::clear_error();
    if (!h) return SK_ERR_INVALID;
    try {
        if (lp < 0 || lp >= h->ipm->num_lps()) return SK_ERR_INVALID;
        reduced_result(*h->ipm, h->red[lp], lp, x, y, s, info);
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

void sk_solver_destroy(sk_solver* h) { delete h; }

int sk_solver_profile(sk_solver* h, int fp32, double* out, int cap) {
    api::clear_error();
    if (!h || !out || cap < 16) return -SK_ERR_INVALID;
    try {
        double all[18];
        h->ipm->profile(fp32 != 0, fp32 == 1, all);
        const int nv = cap >= 18 ? 18 : (cap >= 17 ? 17 : 16);
        for (int q = 0; q < nv; ++q) out[q] = all[q];
        return nv;
    } catch (...) {
        return -api::status_of_current_exception();
    }
}

int sk_kkt_create(int m, int n, const int* row_ptrs, const int* col_idx, const double* vals, const int* P,
                  int precision, sk_kkt** out) {
    api::clear_error();
    if (!out || m <= 0 || n <= 0 || !row_ptrs || !col_idx || !vals) return SK_ERR_INVALID;
    if (precision != SK_PREC_FP64 && precision != SK_PREC_MIXED) return SK_ERR_INVALID;
    try {
        core::CSRMatrix A = api::pattern_csr(m, n, row_ptrs, col_idx);
        A.values.assign(vals, vals + row_ptrs[m]);
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
            throw api::sk_exception(SK_ERR_NO_DEVICE, "no CUDA device visible");
        std::unique_ptr<sk_kkt> k(new sk_kkt);
        k->m = m;
        k->n = n;
        k->precision = precision;
        SK_CUDA(cudaStreamCreateWithFlags(&k->st, cudaStreamNonBlocking));
        // CSC of A
        const int nz = row_ptrs[m];
        std::vector<int> cp(n + 1, 0), ri(nz);
        std::vector<double> cv(nz);
        for (int q = 0; q < nz; ++q) cp[col_idx[q] + 1]++;
        for (int j = 0; j < n; ++j) cp[j + 1] += cp[j];
        std::vector<int> nx(cp.begin(), cp.end() - 1);
        for (int i = 0; i < m; ++i)
            for (int q = row_ptrs[i]; q < row_ptrs[i + 1]; ++q) {
                const int d = nx[col_idx[q]]++;
                ri[d] = i;
                cv[d] = vals[q];
            }
        ipm::LpView v;
        v.m = m; v.n = n; v.col_ptrs = cp.data(); v.row_idx = ri.data(); v.vals = cv.data();
        ipm::FrontPlan plan;
        std::vector<Index> pv;
        if (P) pv.assign(P, P + m);
        ipm::build_front_plan({v}, A, SK_ORDER_AUTO, plan, P ? &pv : nullptr);
        dev::Arena& ar = k->arena;
        dev::reserve(ar, k->a_rp, m + 1); dev::reserve(ar, k->a_ci, nz); dev::reserve(ar, k->a_v, nz);
        dev::reserve(ar, k->t_rp, n + 1); dev::reserve(ar, k->t_ci, nz); dev::reserve(ar, k->t_v, nz);
        dev::reserve(ar, k->row_lp, m); dev::reserve(ar, k->col_lp, n);
        for (auto* s : {&k->out, &k->r, &k->corr, &k->bak, &k->tmp, &k->hostio}) dev::reserve(ar, *s, m);
        dev::reserve(ar, k->theta, n);
        dev::reserve(ar, k->scratch, 64);
        ar.commit();
        for (auto* s : {&k->a_rp, &k->a_ci, &k->t_rp, &k->t_ci, &k->row_lp, &k->col_lp}) dev::bind(ar, *s);
        for (auto* s : {&k->a_v, &k->t_v, &k->out, &k->r, &k->corr, &k->bak, &k->tmp, &k->hostio, &k->theta,
                        &k->scratch})
            dev::bind(ar, *s);
        dev::upload(k->a_rp, A.row_ptrs, k->st); dev::upload(k->a_ci, A.col_indices, k->st);
        dev::upload(k->a_v, A.values, k->st); dev::upload(k->t_rp, cp, k->st); dev::upload(k->t_ci, ri, k->st);
        dev::upload(k->t_v, cv, k->st);
        SK_CUDA(cudaMemsetAsync(k->row_lp.ptr, 0, sizeof(int) * m, k->st));
        SK_CUDA(cudaMemsetAsync(k->col_lp.ptr, 0, sizeof(int) * n, k->st));
        auto& lp = k->lp;
        lp.nlp = 1; lp.M = m; lp.N = n; lp.nnz = nz;
        lp.a_rp = k->a_rp.ptr; lp.a_ci = k->a_ci.ptr; lp.a_v = k->a_v.ptr;
        lp.t_rp = k->t_rp.ptr; lp.t_ci = k->t_ci.ptr; lp.t_v = k->t_v.ptr;
        lp.row_lp = k->row_lp.ptr; lp.col_lp = k->col_lp.ptr;
        k->eng.reset(new dev::KktEngine(plan, k->lp, k->st));
        SK_CUDA(cudaStreamSynchronize(k->st));
        *out = k.release();
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_kkt_factorize_device(sk_kkt* k, const double* d_theta) {
    api::clear_error();
    if (!k || !d_theta) return SK_ERR_INVALID;
    try {
        SK_CUDA(cudaMemcpyAsync(k->theta.ptr, d_theta, sizeof(double) * k->n, cudaMemcpyDeviceToDevice, k->st));
        const bool fp32 = k->precision == SK_PREC_MIXED;
        double delta = fp32 ? 1e-7 : 1e-9;
        for (int retry = 0; retry < 5; ++retry, delta *= 10.0) {
            if (k->eng->factor(k->theta.ptr, delta, fp32)) {
                k->factored = true;
                return SK_OK;
            }
        }
        k->factored = false;
        api::set_error("factorisation failed: matrix is not positive definite for any regularisation");
        return SK_ERR_NUMERICAL;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_kkt_solve_device(sk_kkt* k, double* d_rhs, double tol) {
    api::clear_error();
    if (!k || !d_rhs) return SK_ERR_INVALID;
    if (!k->factored) { api::set_error("solve before a successful factorisation"); return SK_ERR_INVALID; }
    try {
        const int m = k->m;
        cudaStream_t st = k->st;
        auto& E = *k->eng;
        const double rn_rhs = dev::absmax_device(m, d_rhs, k->scratch.ptr, st);
        const double t = tol * std::max(1.0, rn_rhs);
        E.apply_inverse(d_rhs, k->out.ptr);
        auto resid = [&]() {
            E.apply_normal(k->theta.ptr, k->out.ptr, k->tmp.ptr);
            dev::vec_diff(m, d_rhs, k->tmp.ptr, k->r.ptr, st);
            return dev::absmax_device(m, k->r.ptr, k->scratch.ptr, st);
        };
        double rn = resid();
        const int max_ir = k->precision == SK_PREC_MIXED ? 30 : 10;
        for (int it = 0; it < max_ir && rn > t; ++it) {
            SK_CUDA(cudaMemcpyAsync(k->bak.ptr, k->out.ptr, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
            E.apply_inverse(k->r.ptr, k->corr.ptr);
            dev::vec_add(m, k->corr.ptr, k->out.ptr, st);
            const double rn2 = resid();
            if (rn2 >= rn) {
                SK_CUDA(cudaMemcpyAsync(k->out.ptr, k->bak.ptr, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
                break;
            }
            rn = rn2;
        }
        SK_CUDA(cudaMemcpyAsync(d_rhs, k->out.ptr, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
        SK_CUDA(cudaStreamSynchronize(st));
        if (E.solve_error()) {
            api::set_error("triangular solve: a task timed out waiting for a dependency");
            return SK_ERR_CUDA;
        }
        return rn <= t ? SK_OK : SK_ERR_NUMERICAL;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_kkt_factorize(sk_kkt* k, const double* theta) {
    api::clear_error();
    if (!k || !theta) return SK_ERR_INVALID;
    try {
        dev::Arena tmp;
        dev::Slot<double> th;
        dev::reserve(tmp, th, k->n);
        tmp.commit();
        dev::bind(tmp, th);
        SK_CUDA(cudaMemcpyAsync(th.ptr, theta, sizeof(double) * k->n, cudaMemcpyHostToDevice, k->st));
        SK_CUDA(cudaStreamSynchronize(k->st));
        return sk_kkt_factorize_device(k, th.ptr);
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_kkt_solve(sk_kkt* k, double* rhs, double tol) {
    api::clear_error();
    if (!k || !rhs) return SK_ERR_INVALID;
    try {
        SK_CUDA(cudaMemcpyAsync(k->hostio.ptr, rhs, sizeof(double) * k->m, cudaMemcpyHostToDevice, k->st));
        SK_CUDA(cudaStreamSynchronize(k->st));
        const int rc = sk_kkt_solve_device(k, k->hostio.ptr, tol);
        if (rc != SK_OK && rc != SK_ERR_NUMERICAL) return rc;
        SK_CUDA(cudaMemcpyAsync(rhs, k->hostio.ptr, sizeof(double) * k->m, cudaMemcpyDeviceToHost, k->st));
        SK_CUDA(cudaStreamSynchronize(k->st));
        return rc;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_kkt_get_factor(sk_kkt* k, double* L_dense, double* D) {
    api::clear_error();
    if (!k || !L_dense) return SK_ERR_INVALID;
    if (!k->factored) return SK_ERR_INVALID;
    try {
        const auto& p = k->eng->plan();
        std::vector<double> F = k->eng->fronts_host();
        const int m = k->m;
        std::memset(L_dense, 0, sizeof(double) * static_cast<size_t>(m) * m);
        for (int s = 0; s < p.ns; ++s) {
            const int N = p.sn_nrows[s], K = p.sn_ncols[s], f = p.sn_first[s];
            const int* R = p.rows.data() + p.sn_rows_off[s];
            for (int c = 0; c < K; ++c)
                for (int r = c; r < N; ++r)
                    L_dense[static_cast<size_t>(R[r]) * m + (f + c)] = F[p.sn_F_off[s] + r + static_cast<int64_t>(c) * p.sn_lda[s]];
        }
        if (D) {
            SK_CUDA(cudaMemcpyAsync(D, k->eng->diag_D(), sizeof(double) * m, cudaMemcpyDeviceToHost, k->st));
            SK_CUDA(cudaStreamSynchronize(k->st));
        }
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_kkt_set_fp64_update(sk_kkt* k, int mode) {
    api::clear_error();
    if (!k || mode < SK_FP64_UPDATE_AUTO || mode > SK_FP64_UPDATE_TENSOR) return SK_ERR_INVALID;
    k->eng->set_fp64_emulation(mode == SK_FP64_UPDATE_TENSOR);
    return SK_OK;
}

void sk_kkt_destroy(sk_kkt* k) { delete k; }

int sk_presolve_dependent_rows(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                               const double* b, int* keep, int* num_dependent, double* inconsistency) {
    api::clear_error();
    if (!keep || !num_dependent) return SK_ERR_INVALID;
    try {
        check_csc(m, n, col_ptrs, row_idx, vals, b, b);
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
            throw api::sk_exception(SK_ERR_NO_DEVICE, "no CUDA device visible");
        const DependentRows d = find_dependent_rows(m, n, col_ptrs, row_idx, vals, b);
        const bool drop = d.count > 0 && d.count < m && d.inconsistency <= kConsistent;
        for (int i = 0; i < m; ++i) keep[i] = drop && d.dependent[i] ? 0 : 1;
        *num_dependent = d.count;
        if (inconsistency) *inconsistency = d.inconsistency;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_spmv_csr(int rows, const int* d_row_ptrs, const int* d_col_idx, const double* d_vals, const double* d_x,
                double alpha, double beta, double* d_y, void* stream) {
    api::clear_error();
    if (rows < 0 || (rows > 0 && (!d_row_ptrs || !d_col_idx || !d_vals || !d_x || !d_y))) return SK_ERR_INVALID;
    try {
        dev::spmv_csr(rows, d_row_ptrs, d_col_idx, d_vals, d_x, alpha, beta, d_y, static_cast<cudaStream_t>(stream));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

struct sk_spmv_plan {
    int rows = 0, cols = 0;
    long long nnz = 0;
    const int* rp = nullptr;
    const int* ci = nullptr;
    const double* v = nullptr;
    dev::SpmvTuning tune;
    dev::SpmvWindows win;
    dev::SpmvShape shape;
};

int sk_spmv_plan_create(int rows, int cols, long long nnz, const int* d_row_ptrs, const int* d_col_idx,
                        const double* d_vals, void* stream, sk_spmv_plan** out) {
    api::clear_error();
    if (!out || rows < 0 || cols < 0 || nnz < 0 || !d_row_ptrs || (nnz > 0 && (!d_col_idx || !d_vals)))
        return SK_ERR_INVALID;
    *out = nullptr;
    double* xs = nullptr;
    double* ys = nullptr;
    try {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
            throw api::sk_exception(SK_ERR_NO_DEVICE, "no CUDA device visible");
        std::unique_ptr<sk_spmv_plan> p(new sk_spmv_plan);
        p->rows = rows;
        p->cols = cols;
        p->nnz = nnz;
        p->rp = d_row_ptrs;
        p->ci = d_col_idx;
        p->v = d_vals;
        auto st = static_cast<cudaStream_t>(stream);
        const int cached = dev::spmv_tuned_group(rows, cols, nnz);
        p->tune.heuristic = dev::spmv_heuristic_group(nnz, rows);
        p->tune.group = cached;
        if (rows > 0 && nnz > 0) {
            SK_CUDA(cudaMalloc(&xs, sizeof(double) * std::max(1, cols)));
            SK_CUDA(cudaMalloc(&ys, sizeof(double) * rows));
            SK_CUDA(cudaMemsetAsync(xs, 0, sizeof(double) * std::max(1, cols), st));
            p->win.build(rows, d_row_ptrs, d_col_idx, st);
            p->tune = dev::spmv_tune(rows, cols, nnz, d_row_ptrs, d_col_idx, d_vals, xs, ys, st, &p->win);
            SK_CUDA(cudaFree(xs));
            xs = nullptr;
            SK_CUDA(cudaFree(ys));
            ys = nullptr;
        }
        p->shape = p->win.shape(p->tune.group, p->tune.windowed);
        *out = p.release();
        return SK_OK;
    } catch (...) {
        if (xs) cudaFree(xs);
        if (ys) cudaFree(ys);
        return api::status_of_current_exception();
    }
}

int sk_spmv_plan_execute(const sk_spmv_plan* p, const double* d_x, double alpha, double beta, double* d_y,
                         void* stream) {
    api::clear_error();
    if (!p || (p->rows > 0 && (!d_x || !d_y))) return SK_ERR_INVALID;
    try {
        dev::spmv_axpby(p->rows, p->shape, p->rp, p->ci, p->v, d_x, alpha, beta, d_y,
                        static_cast<cudaStream_t>(stream));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_spmv_plan_info(const sk_spmv_plan* p, int* group, int* windowed, int* heuristic_group,
                      double* ms_per_group, double* ms_windowed_per_group) {
    api::clear_error();
    if (!p) return SK_ERR_INVALID;
    if (group) *group = p->shape.group;
    if (windowed) *windowed = p->shape.windowed ? 1 : 0;
    if (heuristic_group) *heuristic_group = p->tune.heuristic;
    for (int k = 0; k < dev::kSpmvNumGroups; ++k) {
        if (ms_per_group) ms_per_group[k] = p->tune.from_cache ? 0.0 : p->tune.ms[k];
        if (ms_windowed_per_group) ms_windowed_per_group[k] = p->tune.from_cache ? 0.0 : p->tune.ms_win[k];
    }
    return SK_OK;
}

int sk_spmv_plan_set_group(sk_spmv_plan* p, int group, int windowed) {
    api::clear_error();
    if (!p || (windowed != 0 && windowed != 1)) return SK_ERR_INVALID;
    for (int k = 0; k < dev::kSpmvNumGroups; ++k)
        if (dev::kSpmvGroups[k] == group) {
            if (windowed && p->rows > 0 && p->win.chunks() == 0) return SK_ERR_INVALID;
            p->shape = p->win.shape(group, windowed != 0);
            return SK_OK;
        }
    return SK_ERR_INVALID;
}

void sk_spmv_plan_destroy(sk_spmv_plan* p) { delete p; }

int sk_gnn_create(unsigned long long seed, sk_gnn** out) {
    api::clear_error();
    if (!out) return SK_ERR_INVALID;
    try {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
            throw api::sk_exception(SK_ERR_NO_DEVICE, "no CUDA device visible");
        std::unique_ptr<sk_gnn> g(new sk_gnn);
        SK_CUDA(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
        g->net.reset(new dev::Gnn(seed));
        *out = g.release();
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

void sk_gnn_destroy(sk_gnn* g) { delete g; }

int sk_gnn_num_params(const sk_gnn* g) { return g && g->net ? g->net->num_params() : -SK_ERR_INVALID; }

int sk_gnn_get_params(const sk_gnn* g, float* out) {
    api::clear_error();
    if (!g || !out) return SK_ERR_INVALID;
    try {
        g->net->get_params(out);
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_gnn_set_params(sk_gnn* g, const float* in) {
    api::clear_error();
    if (!g || !in) return SK_ERR_INVALID;
    try {
        g->net->set_params(in);
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_gnn_batch_create(int m, int n, const int* row_ptrs, const int* col_idx, const double* vals, const double* b,
                        const double* c, const double* t_logx, const double* t_logs, const double* t_y,
                        sk_gnn_batch** out) {
    api::clear_error();
    if (!out || m <= 0 || n <= 0 || !row_ptrs || !b || !c) return SK_ERR_INVALID;
    const bool tg = t_logx || t_logs || t_y;
    if (tg && !(t_logx && t_logs && t_y)) {
        api::set_error("targets: give all of t_logx, t_logs, t_y or none");
        return SK_ERR_INVALID;
    }
    try {
        core::CSRMatrix A = api::pattern_csr(m, n, row_ptrs, col_idx);
        const int nz = row_ptrs[m];
        if (nz > 0 && !vals) throw api::sk_exception(SK_ERR_INVALID, "vals missing");
        A.values.assign(vals, vals + nz);
        std::vector<int> cp(n + 1, 0), ri(nz);
        std::vector<double> cv(nz);
        for (int q = 0; q < nz; ++q) cp[col_idx[q] + 1]++;
        for (int j = 0; j < n; ++j) cp[j + 1] += cp[j];
        std::vector<int> nx(cp.begin(), cp.end() - 1);
        for (int i = 0; i < m; ++i)
            for (int q = row_ptrs[i]; q < row_ptrs[i + 1]; ++q) {
                const int d = nx[col_idx[q]]++;
                ri[d] = i;
                cv[d] = vals[q];
            }
        std::unique_ptr<sk_gnn_batch> bt(new sk_gnn_batch);
        dev::Arena& ar = bt->arena;
        dev::reserve(ar, bt->a_rp, m + 1); dev::reserve(ar, bt->a_ci, nz); dev::reserve(ar, bt->t_rp, n + 1);
        dev::reserve(ar, bt->t_ci, nz);
        dev::reserve(ar, bt->a_v, nz); dev::reserve(ar, bt->t_v, nz); dev::reserve(ar, bt->b, m);
        dev::reserve(ar, bt->c, n); dev::reserve(ar, bt->tlx, n); dev::reserve(ar, bt->tls, n);
        dev::reserve(ar, bt->ty, m);
        ar.commit();
        for (auto* s : {&bt->a_rp, &bt->a_ci, &bt->t_rp, &bt->t_ci}) dev::bind(ar, *s);
        for (auto* s : {&bt->a_v, &bt->t_v, &bt->b, &bt->c, &bt->tlx, &bt->tls, &bt->ty}) dev::bind(ar, *s);
        cudaStream_t st = nullptr;
        dev::upload(bt->a_rp, A.row_ptrs, st); dev::upload(bt->a_ci, A.col_indices, st);
        dev::upload(bt->a_v, A.values, st); dev::upload(bt->t_rp, cp, st); dev::upload(bt->t_ci, ri, st);
        dev::upload(bt->t_v, cv, st);
        dev::upload(bt->b, std::vector<double>(b, b + m), st);
        dev::upload(bt->c, std::vector<double>(c, c + n), st);
        if (tg) {
            dev::upload(bt->tlx, std::vector<double>(t_logx, t_logx + n), st);
            dev::upload(bt->tls, std::vector<double>(t_logs, t_logs + n), st);
            dev::upload(bt->ty, std::vector<double>(t_y, t_y + m), st);
            bt->has_targets = true;
        }
        SK_CUDA(cudaStreamSynchronize(st));
        auto& lp = bt->lp;
        lp.nlp = 1; lp.M = m; lp.N = n; lp.nnz = nz;
        lp.a_rp = bt->a_rp.ptr; lp.a_ci = bt->a_ci.ptr; lp.a_v = bt->a_v.ptr;
        lp.t_rp = bt->t_rp.ptr; lp.t_ci = bt->t_ci.ptr; lp.t_v = bt->t_v.ptr;
        lp.b = bt->b.ptr; lp.c = bt->c.ptr;
        *out = bt.release();
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_gnn_batch_from_solver(sk_solver* h, sk_gnn_batch** out) {
    api::clear_error();
    if (!h || !out) return SK_ERR_INVALID;
    try {
        dev::DeviceIPM& ipm = *h->ipm;
        if (!ipm.capture_complete())
            throw api::sk_exception(SK_ERR_INVALID, "no complete iterate capture (sk_solver_set_capture, then run)");
        const dev::DeviceLP& s = ipm.device_lp();
        const int m = s.M, n = s.N;
        const int64_t nz = s.nnz;
        std::unique_ptr<sk_gnn_batch> bt(new sk_gnn_batch);
        dev::Arena& ar = bt->arena;
        dev::reserve(ar, bt->a_rp, m + 1); dev::reserve(ar, bt->a_ci, nz); dev::reserve(ar, bt->t_rp, n + 1);
        dev::reserve(ar, bt->t_ci, nz);
        dev::reserve(ar, bt->a_v, nz); dev::reserve(ar, bt->t_v, nz); dev::reserve(ar, bt->b, m);
        dev::reserve(ar, bt->c, n); dev::reserve(ar, bt->tlx, n); dev::reserve(ar, bt->tls, n);
        dev::reserve(ar, bt->ty, m);
        ar.commit();
        for (auto* x : {&bt->a_rp, &bt->a_ci, &bt->t_rp, &bt->t_ci}) dev::bind(ar, *x);
        for (auto* x : {&bt->a_v, &bt->t_v, &bt->b, &bt->c, &bt->tlx, &bt->tls, &bt->ty}) dev::bind(ar, *x);
        auto cp = [](void* d, const void* src, size_t bytes) {
            SK_CUDA(cudaMemcpy(d, src, bytes, cudaMemcpyDeviceToDevice));
        };
        cp(bt->a_rp.ptr, s.a_rp, sizeof(int) * (m + 1)); cp(bt->a_ci.ptr, s.a_ci, sizeof(int) * nz);
        cp(bt->a_v.ptr, s.a_v, sizeof(double) * nz); cp(bt->t_rp.ptr, s.t_rp, sizeof(int) * (n + 1));
        cp(bt->t_ci.ptr, s.t_ci, sizeof(int) * nz); cp(bt->t_v.ptr, s.t_v, sizeof(double) * nz);
        cp(bt->b.ptr, s.b, sizeof(double) * m); cp(bt->c.ptr, s.c, sizeof(double) * n);
        cp(bt->tlx.ptr, ipm.capture_logx(), sizeof(double) * n);
        cp(bt->tls.ptr, ipm.capture_logs(), sizeof(double) * n);
        cp(bt->ty.ptr, ipm.capture_y(), sizeof(double) * m);
        bt->has_targets = true;
        auto& lp = bt->lp;
        lp.nlp = s.nlp; lp.M = m; lp.N = n; lp.nnz = nz;
        lp.a_rp = bt->a_rp.ptr; lp.a_ci = bt->a_ci.ptr; lp.a_v = bt->a_v.ptr;
        lp.t_rp = bt->t_rp.ptr; lp.t_ci = bt->t_ci.ptr; lp.t_v = bt->t_v.ptr;
        lp.b = bt->b.ptr; lp.c = bt->c.ptr;
        *out = bt.release();
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_gnn_batch_dims(const sk_gnn_batch* bt, int* m, int* n) {
    if (!bt) return SK_ERR_INVALID;
    if (m) *m = bt->lp.M;
    if (n) *n = bt->lp.N;
    return SK_OK;
}

int sk_gnn_batch_targets(const sk_gnn_batch* bt, double* logx, double* logs, double* y) {
    api::clear_error();
    if (!bt) return SK_ERR_INVALID;
    if (!bt->has_targets) { api::set_error("batch has no targets"); return SK_ERR_INVALID; }
    try {
        const int m = bt->lp.M, n = bt->lp.N;
        if (logx) SK_CUDA(cudaMemcpy(logx, bt->tlx.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (logs) SK_CUDA(cudaMemcpy(logs, bt->tls.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost));
        if (y) SK_CUDA(cudaMemcpy(y, bt->ty.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

void sk_gnn_batch_destroy(sk_gnn_batch* bt) { delete bt; }

int sk_gnn_predict(sk_gnn* g, sk_gnn_batch* bt, double* logx, double* logs, double* y) {
    api::clear_error();
    if (!g || !bt) return SK_ERR_INVALID;
    try {
        const int m = bt->lp.M, n = bt->lp.N;
        dev::Arena tmp;
        dev::Slot<double> ox, os, oy;
        dev::reserve(tmp, ox, n); dev::reserve(tmp, os, n); dev::reserve(tmp, oy, m);
        tmp.commit();
        dev::bind(tmp, ox); dev::bind(tmp, os); dev::bind(tmp, oy);
        g->net->forward(bt->lp, g->st, ox.ptr, os.ptr, oy.ptr);
        if (logx) SK_CUDA(cudaMemcpyAsync(logx, ox.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, g->st));
        if (logs) SK_CUDA(cudaMemcpyAsync(logs, os.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, g->st));
        if (y) SK_CUDA(cudaMemcpyAsync(y, oy.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost, g->st));
        SK_CUDA(cudaStreamSynchronize(g->st));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_gnn_loss_grad(sk_gnn* g, sk_gnn_batch* bt, double* loss, float* grad) {
    api::clear_error();
    if (!g || !bt) return SK_ERR_INVALID;
    if (!bt->has_targets) { api::set_error("batch has no targets"); return SK_ERR_INVALID; }
    try {
        const double l = g->net->forward(bt->lp, g->st, nullptr, nullptr, nullptr, bt->tlx.ptr, bt->tls.ptr, bt->ty.ptr);
        if (loss) *loss = l;
        g->net->backward(bt->lp, g->st, grad);
        SK_CUDA(cudaStreamSynchronize(g->st));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_gnn_train_step(sk_gnn* g, sk_gnn_batch* bt, float lr, double* loss) {
    api::clear_error();
    if (!g || !bt || !(lr > 0.f)) return SK_ERR_INVALID;
    if (!bt->has_targets) { api::set_error("batch has no targets"); return SK_ERR_INVALID; }
    try {
        const double l = g->net->forward(bt->lp, g->st, nullptr, nullptr, nullptr, bt->tlx.ptr, bt->tls.ptr, bt->ty.ptr);
        if (loss) *loss = l;
        g->net->backward(bt->lp, g->st, nullptr);
        g->net->adam_step(g->st, lr);
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_solver_set_gnn(sk_solver* h, sk_gnn* g) {
    api::clear_error();
    if (!h) return SK_ERR_INVALID;
    h->ipm->set_gnn(g ? g->net.get() : nullptr);
    return SK_OK;
}

int sk_solver_set_capture(sk_solver* h, double mu_threshold) {
    api::clear_error();
    if (!h) return SK_ERR_INVALID;
    try {
        h->ipm->set_capture(mu_threshold);
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

}  // extern "C"

extern "C" int sk_crossover(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                            const double* lb, const double* ub, const double* x, int* basic, int* status,
                            double* x_out) {
    api::clear_error();
    if (m <= 0 || n <= 0 || !col_ptrs || !row_idx || !vals || !x || !basic || !status) return SK_ERR_INVALID;
    if (m > SK_CROSSOVER_MAX_ROWS) {
        api::set_error("sk_crossover: m exceeds SK_CROSSOVER_MAX_ROWS");
        return SK_ERR_TOO_LARGE;
    }
    try {
        std::string msg;
        const int rc = dev::crossover(m, n, col_ptrs, row_idx, vals, lb, ub, x, basic, status, x_out, &msg);
        if (rc == dev::kCrossoverInvalidPivot) { api::set_error(msg); return SK_ERR_NUMERICAL; }
        if (rc == dev::kCrossoverRankDeficient) { api::set_error(msg); return SK_ERR_RANK_DEFICIENT; }
        if (rc == dev::kCrossoverTooLarge) return SK_ERR_TOO_LARGE;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}
