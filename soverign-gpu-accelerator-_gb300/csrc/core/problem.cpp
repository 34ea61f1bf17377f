// LP model container (reference behaviour: src/core/problem.cpp:16-132).
#include "core/problem.hpp"

#include <algorithm>
#include <numeric>

namespace sankhya {
namespace core {

Model::Model() = default;

void Model::add_variable(Float obj_coeff, Float lower, Float upper, VariableType vt) {
    obj.push_back(obj_coeff);
    lb.push_back(lower);
    ub.push_back(upper);
    vtype.push_back(vt);
}

static void check_row(const std::vector<Index>& cols, const std::vector<Float>& vals,
                      Index num_vars, const char* who) {
    if (cols.size() != vals.size())
        throw std::invalid_argument(std::string(who) + ": cols and vals must have the same size");
    for (Index c : cols)
        if (c < 0 || c >= num_vars)
            throw std::invalid_argument(std::string(who) + ": column index out of range");
}

void Model::add_constraint(const std::vector<Index>& cols, const std::vector<Float>& vals, Float b) {
    check_row(cols, vals, static_cast<Index>(vtype.size()), "add_constraint");
    constraint_cols_.push_back(cols);
    constraint_vals_.push_back(vals);
    rhs.push_back(b);
}

void Model::update_constraint(Index row, const std::vector<Index>& cols,
                              const std::vector<Float>& vals, Float b) {
    if (row < 0 || static_cast<size_t>(row) >= rhs.size())
        throw std::out_of_range("update_constraint: row index out of bounds");
    check_row(cols, vals, static_cast<Index>(vtype.size()), "update_constraint");
    constraint_cols_[static_cast<size_t>(row)] = cols;
    constraint_vals_[static_cast<size_t>(row)] = vals;
    rhs[static_cast<size_t>(row)] = b;
}

const std::vector<Index>& Model::get_constraint_cols(Index row) const {
    if (row < 0 || static_cast<size_t>(row) >= constraint_cols_.size())
        throw std::out_of_range("get_constraint_cols: row index out of bounds");
    return constraint_cols_[static_cast<size_t>(row)];
}

const std::vector<Float>& Model::get_constraint_vals(Index row) const {
    if (row < 0 || static_cast<size_t>(row) >= constraint_vals_.size())
        throw std::out_of_range("get_constraint_vals: row index out of bounds");
    return constraint_vals_[static_cast<size_t>(row)];
}

void Model::finalize() {
    const size_t nv = vtype.size();
    if (obj.size() != nv || lb.size() != nv || ub.size() != nv)
        throw std::invalid_argument("finalize: objective/bounds/type vectors differ in size");
    const Index m = static_cast<Index>(rhs.size());
    const Index n = static_cast<Index>(nv);
    // Rows are visited in increasing order, so each column's row list comes out sorted.
    std::vector<Index> ptr(static_cast<size_t>(n) + 1, 0);
    for (Index r = 0; r < m; ++r)
        for (Index c : constraint_cols_[static_cast<size_t>(r)]) ptr[static_cast<size_t>(c) + 1]++;
    for (Index c = 0; c < n; ++c) ptr[c + 1] += ptr[c];
    std::vector<Index> ri(static_cast<size_t>(ptr.back()));
    std::vector<Float> va(static_cast<size_t>(ptr.back()));
    std::vector<Index> next(ptr.begin(), ptr.end() - 1);
    for (Index r = 0; r < m; ++r) {
        const auto& cc = constraint_cols_[static_cast<size_t>(r)];
        const auto& vv = constraint_vals_[static_cast<size_t>(r)];
        for (size_t e = 0; e < cc.size(); ++e) {
            const Index dst = next[static_cast<size_t>(cc[e])]++;
            ri[dst] = r;
            va[dst] = vv[e];
        }
    }
    A = CSCMatrix(m, n, std::move(va), std::move(ri), std::move(ptr));
}

Model Model::from_csc(Index m, Index n, const Index* col_ptrs, const Index* row_idx,
                      const Float* vals, const Float* b, const Float* c) {
    if (m < 0 || n < 0) throw std::invalid_argument("from_csc: negative dimension");
    if (!col_ptrs || (n > 0 && (!c)) || (m > 0 && !b))
        throw std::invalid_argument("from_csc: null array");
    if (col_ptrs[0] != 0) throw std::invalid_argument("from_csc: col_ptrs[0] != 0");
    for (Index j = 0; j < n; ++j)
        if (col_ptrs[j + 1] < col_ptrs[j]) throw std::invalid_argument("from_csc: col_ptrs not monotone");
    const Index nz = col_ptrs[n];
    if (nz > 0 && (!row_idx || !vals)) throw std::invalid_argument("from_csc: null array");
    Model model;
    model.obj.assign(c, c + n);
    model.lb.assign(static_cast<size_t>(n), 0.0);
    model.ub.assign(static_cast<size_t>(n), math::kInfinity);
    model.vtype.assign(static_cast<size_t>(n), VariableType::Continuous);
    model.rhs.assign(b, b + m);
    std::vector<Index> ptr(col_ptrs, col_ptrs + n + 1);
    std::vector<Index> ri(row_idx, row_idx + nz);
    std::vector<Float> va(vals, vals + nz);
    for (Index k = 0; k < nz; ++k)
        if (ri[k] < 0 || ri[k] >= m) throw std::invalid_argument("from_csc: row index out of range");
    // Sort rows within each column (stable on equal rows; duplicates are rejected).
    std::vector<Index> order;
    for (Index j = 0; j < n; ++j) {
        const Index s = ptr[j], e = ptr[j + 1];
        bool sorted = true;
        for (Index k = s + 1; k < e; ++k)
            if (ri[k] <= ri[k - 1]) { sorted = false; break; }
        if (sorted) continue;
        order.resize(static_cast<size_t>(e - s));
        std::iota(order.begin(), order.end(), s);
        std::stable_sort(order.begin(), order.end(), [&](Index a, Index bb) { return ri[a] < ri[bb]; });
        std::vector<Index> r2(order.size());
        std::vector<Float> v2(order.size());
        for (size_t t = 0; t < order.size(); ++t) { r2[t] = ri[order[t]]; v2[t] = va[order[t]]; }
        for (size_t t = 0; t < order.size(); ++t) {
            if (t > 0 && r2[t] == r2[t - 1]) throw std::invalid_argument("from_csc: duplicate entry");
            ri[s + static_cast<Index>(t)] = r2[t];
            va[s + static_cast<Index>(t)] = v2[t];
        }
    }
    model.A = CSCMatrix(m, n, std::move(va), std::move(ri), std::move(ptr));
    return model;
}

}  // namespace core
}  // namespace sankhya
