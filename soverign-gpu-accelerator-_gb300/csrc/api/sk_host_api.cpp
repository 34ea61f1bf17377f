// Host-side C ABI entry points: model input (generators, MPS), symbolic
// analysis, options and error reporting. See include/sankhya/sk_ipm.h.
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "api/sk_error.hpp"
#include "core/problem.hpp"
#include "gen/lpgen.hpp"
#include "ipm/front_plan.hpp"
#include "ipm/symbolic.hpp"
#include "parsers/mps_reader.hpp"
#include "presolve/scaling.hpp"
#include "core/standard_form.hpp"
#include "sankhya/sk_ipm.h"

struct sk_lp {
    sankhya::core::Model model;
};

namespace sankhya {
namespace api {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

int status_of_current_exception() {
    try {
        throw;
    } catch (const sk_exception& e) {
        set_error(e.what());
        return e.code;
    } catch (const std::bad_alloc& e) {
        set_error(std::string("allocation failed: ") + e.what());
        return SK_ERR_ALLOC;
    } catch (const std::invalid_argument& e) {
        set_error(e.what());
        return SK_ERR_INVALID;
    } catch (const std::out_of_range& e) {
        set_error(e.what());
        return SK_ERR_INVALID;
    } catch (const std::exception& e) {
        set_error(e.what());
        return SK_ERR_INTERNAL;
    } catch (...) {
        set_error("unknown exception");
        return SK_ERR_INTERNAL;
    }
}

core::CSRMatrix pattern_csr(int m, int n, const int* row_ptrs, const int* col_idx) {
    if (m < 0 || n < 0 || !row_ptrs || (row_ptrs[m] > 0 && !col_idx))
        throw std::invalid_argument("invalid CSR pattern");
    core::CSRMatrix A;
    A.rows = m;
    A.cols = n;
    A.row_ptrs.assign(row_ptrs, row_ptrs + m + 1);
    A.col_indices.assign(col_idx, col_idx + row_ptrs[m]);
    for (Index i = 0; i < m; ++i)
        if (A.row_ptrs[i + 1] < A.row_ptrs[i]) throw std::invalid_argument("CSR row_ptrs not monotone");
    for (Index c : A.col_indices)
        if (c < 0 || c >= n) throw std::invalid_argument("CSR column index out of range");
    A.values.assign(A.col_indices.size(), 1.0);
    return A;
}

}  // namespace api
}  // namespace sankhya

using namespace sankhya;

extern "C" {

const char* sk_last_error(void) { return api::g_last_error.c_str(); }

void sk_options_default(sk_options* opt) {
    if (!opt) return;
    opt->precision = SK_PREC_MIXED;
    opt->start = SK_START_UNIT;
    opt->criteria = SK_CRIT_RELATIVE;
    opt->tol = 1e-8;
    opt->max_iter = 200;
    opt->ordering = SK_ORDER_AUTO;
    opt->verbose = 0;
    opt->mu_switch = 1e-4;
    opt->ruiz_passes = 10;
    opt->strict = 0;
    opt->delta32 = 1e-8;
    opt->delta64 = 1e-14;
    opt->learned_accept = 0.5;
    opt->fp64_update = SK_FP64_UPDATE_AUTO;
    opt->dependent_rows = 0;
}

int sk_lp_generate(int family, int instance, sk_lp** out) {
    api::clear_error();
    if (!out) return SK_ERR_INVALID;
    try {
        auto g = gen::family_lp(family, instance);
        auto* lp = new sk_lp;
        lp->model = core::Model::from_csc(g.m, g.n, g.col_ptrs.data(), g.row_idx.data(), g.vals.data(),
                                          g.b.data(), g.c.data());
        *out = lp;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_lp_random(int m, int n, double density, unsigned long long seed, sk_lp** out) {
    api::clear_error();
    if (!out) return SK_ERR_INVALID;
    try {
        auto g = gen::random_sparse_lp(m, n, density, seed);
        auto* lp = new sk_lp;
        lp->model = core::Model::from_csc(g.m, g.n, g.col_ptrs.data(), g.row_idx.data(), g.vals.data(),
                                          g.b.data(), g.c.data());
        *out = lp;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_lp_standard_form(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, const double* b,
                        const double* c, const double* lb, const double* ub, sk_lp** out, double* obj_offset) {
    api::clear_error();
    if (!out) return SK_ERR_INVALID;
    try {
        core::BoundedLp bl;
        bl.m = m; bl.n = n; bl.col_ptrs = col_ptrs; bl.row_idx = row_idx; bl.vals = vals; bl.b = b; bl.c = c;
        bl.lb = lb; bl.ub = ub;
        const core::StandardForm sf = core::to_standard_form(bl);
        auto* lp = new sk_lp;
        lp->model = core::Model::from_csc(sf.m, sf.n, sf.col_ptrs.data(), sf.row_idx.data(), sf.vals.data(),
                                          sf.b.data(), sf.c.data());
        if (obj_offset) *obj_offset = sf.obj_offset;
        *out = lp;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_lp_staircase(unsigned long long seed, int stages, int supply, int demand, int cap, int arcs, sk_lp** out) {
    api::clear_error();
    if (!out || stages <= 0 || supply <= 0 || demand <= 0 || cap <= 1 || arcs < supply || arcs < demand)
        return SK_ERR_INVALID;
    try {
        auto g = gen::staircase_transport_lp(seed, stages, supply, demand, cap, arcs);
        auto* lp = new sk_lp;
        lp->model = core::Model::from_csc(g.m, g.n, g.col_ptrs.data(), g.row_idx.data(), g.vals.data(),
                                          g.b.data(), g.c.data());
        *out = lp;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_lp_block_angular(unsigned long long seed, int blocks, int block_rows, int block_cols, int link_rows,
                        int nnz_per_col, sk_lp** out) {
    api::clear_error();
    if (!out || blocks <= 0 || block_rows <= 0 || block_cols <= 0 || link_rows < 0 || nnz_per_col <= 0 ||
        nnz_per_col > block_rows)
        return SK_ERR_INVALID;
    try {
        auto g = gen::block_angular_lp(seed, blocks, block_rows, block_cols, link_rows, nnz_per_col);
        auto* lp = new sk_lp;
        lp->model = core::Model::from_csc(g.m, g.n, g.col_ptrs.data(), g.row_idx.data(), g.vals.data(),
                                          g.b.data(), g.c.data());
        *out = lp;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_lp_read_mps(const char* path, sk_lp** out) {
    api::clear_error();
    if (!path || !out) return SK_ERR_INVALID;
    try {
        auto* lp = new sk_lp;
        try {
            lp->model = parsers::read_mps(path);
        } catch (const std::runtime_error& e) {
            delete lp;
            api::set_error(e.what());
            return SK_ERR_INVALID;
        }
        *out = lp;
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_lp_dims(const sk_lp* lp, int* m, int* n, int* nnz) {
    if (!lp) return SK_ERR_INVALID;
    if (m) *m = lp->model.A.rows;
    if (n) *n = lp->model.A.cols;
    if (nnz) *nnz = lp->model.A.nnz();
    return SK_OK;
}

int sk_lp_arrays(const sk_lp* lp, const int** col_ptrs, const int** row_idx, const double** vals,
                 const double** b, const double** c) {
    if (!lp) return SK_ERR_INVALID;
    if (col_ptrs) *col_ptrs = lp->model.A.col_ptrs.data();
    if (row_idx) *row_idx = lp->model.A.row_indices.data();
    if (vals) *vals = lp->model.A.values.data();
    if (b) *b = lp->model.rhs.data();
    if (c) *c = lp->model.obj.data();
    return SK_OK;
}

int sk_lp_bounds(const sk_lp* lp, const double** lb, const double** ub) {
    if (!lp) return SK_ERR_INVALID;
    if (lb) *lb = lp->model.lb.data();
    if (ub) *ub = lp->model.ub.data();
    return SK_OK;
}

void sk_lp_free(sk_lp* lp) { delete lp; }

int sk_presolve_ruiz(int m, int n, const int* col_ptrs, const int* row_idx, double* vals, double* b, double* c,
                     double* lb, double* ub, const unsigned char* integer_cols, int max_iterations,
                     double* row_scale, double* col_scale) {
    sankhya::api::clear_error();
    if (m < 0 || n < 0 || max_iterations < 0) return SK_ERR_INVALID;
    if (m > 0 && n > 0 && (!col_ptrs || !row_idx || !vals || !row_scale || !col_scale)) return SK_ERR_INVALID;
    try {
        if (m > 0 && n > 0) {
            if (col_ptrs[0] != 0) throw std::invalid_argument("col_ptrs[0] must be 0");
            for (int j = 0; j < n; ++j)
                if (col_ptrs[j + 1] < col_ptrs[j]) throw std::invalid_argument("col_ptrs must not decrease");
            for (int q = 0; q < col_ptrs[n]; ++q)
                if (row_idx[q] < 0 || row_idx[q] >= m) throw std::invalid_argument("row index out of range");
        }
        return sankhya::presolve::ruiz_scale_csc(m, n, col_ptrs, row_idx, vals, b, c, lb, ub, integer_cols,
                                                 max_iterations, row_scale, col_scale) >= 0
                   ? SK_OK
                   : SK_ERR_INTERNAL;
    } catch (...) {
        return sankhya::api::status_of_current_exception();
    }
}

int sk_compute_amd_ordering(int m, int n, const int* row_ptrs, const int* col_idx, int* P) {
    api::clear_error();
    if (!P) return SK_ERR_INVALID;
    try {
        auto p = ipm::compute_amd_ordering(api::pattern_csr(m, n, row_ptrs, col_idx));
        std::memcpy(P, p.data(), sizeof(int) * static_cast<size_t>(m));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_fill_ordering(int m, int n, const int* row_ptrs, const int* col_idx, int* P) {
    api::clear_error();
    if (!P) return SK_ERR_INVALID;
    try {
        auto p = ipm::fill_reducing_ordering(api::pattern_csr(m, n, row_ptrs, col_idx));
        std::memcpy(P, p.data(), sizeof(int) * static_cast<size_t>(m));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_dissection_ordering(int m, int n, const int* row_ptrs, const int* col_idx, int* P) {
    api::clear_error();
    if (!P) return SK_ERR_INVALID;
    try {
        auto p = ipm::nested_dissection_ordering(api::pattern_csr(m, n, row_ptrs, col_idx));
        std::memcpy(P, p.data(), sizeof(int) * static_cast<size_t>(m));
        return SK_OK;
    } catch (...) {
        return api::status_of_current_exception();
    }
}

int sk_compute_symbolic(int m, int n, const int* row_ptrs, const int* col_idx, const int* P, int* P_inv,
                        int* parent, int* L_row_ptrs, int* L_cols, int cap) {
    api::clear_error();
    if (!P || !P_inv || !parent || !L_row_ptrs || (cap > 0 && !L_cols)) return -SK_ERR_INVALID;
    try {
        std::vector<Index> pv(P, P + m);
        std::vector<char> seen(static_cast<size_t>(m), 0);
        for (Index v : pv) {
            if (v < 0 || v >= m || seen[v]) throw std::invalid_argument("P is not a permutation");
            seen[v] = 1;
        }
        ipm::SymbolicFactorization sym;
        ipm::compute_symbolic_factorization(api::pattern_csr(m, n, row_ptrs, col_idx), pv, sym);
        const int nnz = sym.L_pattern.row_ptrs[static_cast<size_t>(m)];
        if (nnz > cap) return -1;
        std::memcpy(P_inv, sym.P_inv.data(), sizeof(int) * static_cast<size_t>(m));
        std::memcpy(parent, sym.parent.data(), sizeof(int) * static_cast<size_t>(m));
        std::memcpy(L_row_ptrs, sym.L_pattern.row_ptrs.data(), sizeof(int) * static_cast<size_t>(m + 1));
        if (nnz > 0) std::memcpy(L_cols, sym.L_pattern.col_indices.data(), sizeof(int) * static_cast<size_t>(nnz));
        return nnz;
    } catch (...) {
        return -api::status_of_current_exception();
    }
}

int sk_plan_stats(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, int ordering,
                  double* out, int cap) {
    api::clear_error();
    if (!out || cap < 16 || m <= 0 || n <= 0 || !col_ptrs) return -SK_ERR_INVALID;
    try {
        core::Model md = core::Model::from_csc(m, n, col_ptrs, row_idx, vals, std::vector<double>(m, 0.0).data(),
                                               std::vector<double>(n, 0.0).data());
        core::CSRMatrix A = core::to_csr(md.A);
        ipm::LpView v;
        v.m = m; v.n = n;
        v.col_ptrs = md.A.col_ptrs.data(); v.row_idx = md.A.row_indices.data(); v.vals = md.A.values.data();
        ipm::FrontPlan p;
        ipm::build_front_plan({v}, A, ordering, p);
        int64_t maxrows = 0, small = 0;
        for (int s = 0; s < p.ns; ++s) {
            maxrows = std::max<int64_t>(maxrows, p.sn_nrows[s]);
            small += p.sn_ncols[s] <= ipm::kTile;
        }
        // consistency: own columns first in each front, rows sorted, slots inside fronts
        bool ok = true;
        int64_t cols = 0;
        for (int s = 0; s < p.ns && ok; ++s) {
            const Index* R = p.rows.data() + p.sn_rows_off[s];
            cols += p.sn_ncols[s];
            for (Index q = 0; q < p.sn_ncols[s]; ++q) ok = ok && R[q] == p.sn_first[s] + q;
            for (Index q = 1; q < p.sn_nrows[s]; ++q) ok = ok && R[q] > R[q - 1];
        }
        ok = ok && cols == p.M;
        for (int64_t q = 0; q < p.nslots && ok; ++q) {
            const int t = p.sn_of_col[p.slot_j[q]];
            ok = p.slot_pos[q] >= p.sn_F_off[t] &&
                 p.slot_pos[q] < p.sn_F_off[t] + static_cast<int64_t>(p.sn_lda[t]) * p.sn_nrows[t];
        }
        int64_t solve_launches = 0, factor_launches = 0;
        for (int l = 0; l < p.nlevels; ++l) {
            const int ns = p.step_level_ptr[l + 1] - p.step_level_ptr[l];
            solve_launches += 1 + ns;
            factor_launches += (p.round_level_ptr[l + 1] - p.round_level_ptr[l]);
        }
        for (const auto& st : p.steps) factor_launches += 1 + (st.trsm_tiles > 0) + (st.upd_tiles > 0);
        const double vals16[16] = {static_cast<double>(p.ns), static_cast<double>(p.nlevels),
                                   static_cast<double>(p.steps.size()), static_cast<double>(p.rounds.size()),
                                   static_cast<double>(p.nnz_factor), p.flops_factor, static_cast<double>(p.F_size),
                                   static_cast<double>(maxrows), static_cast<double>(small),
                                   static_cast<double>(p.nslots), static_cast<double>(p.w_col.size()),
                                   p.dense_mode ? 1.0 : 0.0, static_cast<double>(p.ordering_used), ok ? 1.0 : 0.0,
                                   static_cast<double>(solve_launches), static_cast<double>(factor_launches)};
        for (int q = 0; q < 16; ++q) out[q] = vals16[q];
        return 16;
    } catch (...) {
        return -api::status_of_current_exception();
    }
}

}  // extern "C"
