// Standard form of an LP with variable bounds (see include/core/standard_form.hpp).
#include "core/standard_form.hpp"

#include <cmath>
#include <stdexcept>
#include <string>

namespace sankhya {
namespace core {

StandardForm to_standard_form(const BoundedLp& lp) {
    if (lp.m <= 0 || lp.n <= 0 || !lp.col_ptrs || !lp.b || !lp.c)
        throw std::invalid_argument("to_standard_form: invalid LP arrays");
    const Index m = lp.m, n = lp.n;
    StandardForm sf;
    sf.kind.assign(n, StandardForm::kShift);
    sf.pos.assign(n, -1);
    sf.neg.assign(n, -1);
    std::vector<Float> b(lp.b, lp.b + m);
    for (Index j = 0; j < n; ++j) {
        const Float l = lp.lb ? lp.lb[j] : 0.0, u = lp.ub ? lp.ub[j] : math::kInfinity;
        if (std::isnan(l) || std::isnan(u) || l > u || l == math::kInfinity || u == -math::kInfinity)
            throw std::invalid_argument("to_standard_form: bad bounds of column " + std::to_string(j));
        if (!std::isfinite(lp.c[j])) throw std::invalid_argument("to_standard_form: non-finite cost");
    }
    // columns of the standard form: x' for every original column, then x'' of the
    // free columns, then the slacks of the finite upper bounds (one row each)
    Index next = n;
    std::vector<Index> bound_row(n, -1);
    Index nrows = m;
    for (Index j = 0; j < n; ++j) {
        const Float l = lp.lb ? lp.lb[j] : 0.0, u = lp.ub ? lp.ub[j] : math::kInfinity;
        sf.pos[j] = j;
        if (std::isfinite(l)) {
            sf.kind[j] = StandardForm::kShift;
            if (std::isfinite(u)) bound_row[j] = nrows++;
        } else if (std::isfinite(u)) {
            sf.kind[j] = StandardForm::kReflect;
        } else {
            sf.kind[j] = StandardForm::kFree;
            sf.neg[j] = next++;
        }
    }
    const Index nfree_end = next;
    sf.bound_rows = nrows - m;
    sf.m = nrows;
    sf.n = nfree_end + sf.bound_rows;
    sf.c.assign(sf.n, 0.0);
    sf.b.assign(nrows, 0.0);
    sf.col_ptrs.assign(static_cast<size_t>(sf.n) + 1, 0);
    // per standard-form column: its entries (rows ascending)
    std::vector<std::vector<std::pair<Index, Float>>> cols(sf.n);
    for (Index j = 0; j < n; ++j) {
        const Float l = lp.lb ? lp.lb[j] : 0.0, u = lp.ub ? lp.ub[j] : math::kInfinity;
        const Float sg = sf.kind[j] == StandardForm::kReflect ? -1.0 : 1.0;
        const Float fix = sf.kind[j] == StandardForm::kShift ? l : (sf.kind[j] == StandardForm::kReflect ? u : 0.0);
        for (Index q = lp.col_ptrs[j]; q < lp.col_ptrs[j + 1]; ++q) {
            const Index i = lp.row_idx[q];
            const Float a = lp.vals[q];
            if (i < 0 || i >= m || !std::isfinite(a)) throw std::invalid_argument("to_standard_form: bad matrix entry");
            cols[sf.pos[j]].push_back({i, sg * a});
            if (sf.kind[j] == StandardForm::kFree) cols[sf.neg[j]].push_back({i, -a});
            if (fix != 0.0) b[i] -= a * fix;
        }
        sf.c[sf.pos[j]] = sg * lp.c[j];
        if (sf.kind[j] == StandardForm::kFree) sf.c[sf.neg[j]] = -lp.c[j];
        sf.obj_offset += lp.c[j] * fix;
        if (bound_row[j] >= 0) {
            const Index r = bound_row[j], w = nfree_end + (r - m);
            cols[sf.pos[j]].push_back({r, 1.0});
            cols[w].push_back({r, 1.0});
            sf.b[r] = u - l;
        }
    }
    for (Index i = 0; i < m; ++i) sf.b[i] = b[i];
    for (Index k = 0; k < sf.n; ++k) {
        sf.col_ptrs[k + 1] = sf.col_ptrs[k] + static_cast<Index>(cols[k].size());
        for (const auto& e : cols[k]) {
            sf.row_idx.push_back(e.first);
            sf.vals.push_back(e.second);
        }
    }
    return sf;
}

Float recover_solution(const BoundedLp& lp, const StandardForm& sf, const Float* xs, const Float* ys, Float* x,
                       Float* y, Float* s) {
    const Index m = lp.m, n = lp.n;
    Float obj = 0.0;
    std::vector<Float> xv(n);
    for (Index j = 0; j < n; ++j) {
        const Float l = lp.lb ? lp.lb[j] : 0.0, u = lp.ub ? lp.ub[j] : math::kInfinity;
        switch (sf.kind[j]) {
            case StandardForm::kShift: xv[j] = l + xs[sf.pos[j]]; break;
            case StandardForm::kReflect: xv[j] = u - xs[sf.pos[j]]; break;
            default: xv[j] = xs[sf.pos[j]] - xs[sf.neg[j]]; break;
        }
        obj += lp.c[j] * xv[j];
    }
    if (x) for (Index j = 0; j < n; ++j) x[j] = xv[j];
    if (y) for (Index i = 0; i < m; ++i) y[i] = ys[i];
    if (s) {
        for (Index j = 0; j < n; ++j) {
            Float aty = 0.0;
            for (Index q = lp.col_ptrs[j]; q < lp.col_ptrs[j + 1]; ++q) aty += lp.vals[q] * ys[lp.row_idx[q]];
            s[j] = lp.c[j] - aty;
        }
    }
    return obj;
}

}  // namespace core
}  // namespace sankhya
