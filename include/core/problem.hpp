// Equality-form LP data model:  min/max c^T x  s.t.  A x = b,  lb <= x <= ub.
// Public surface follows the reference's src/core/problem.hpp:40-119 (same member
// names obj / lb / ub / vtype / rhs / A, add_variable / add_constraint /
// update_constraint / finalize) so the reference's callers build unchanged.
// The device IPM solves the standard form min c^T x, Ax = b, x >= 0, exactly as
// the reference's device IPM does (it never reads lb / ub).
#pragma once

#include <array>
#include <stdexcept>
#include <vector>

#include "core/sparse_matrix.hpp"
#include "sankhya/types.hpp"

namespace sankhya {
namespace core {

struct BilinearTerm {
    Index x_col;
    Index y_col;
    Index w_col;
    std::array<Index, 4> mccormick_rows;
};

class Model {
public:
    OptimizationSense sense = OptimizationSense::Minimize;
    std::vector<Float> obj;
    std::vector<Float> lb;
    std::vector<Float> ub;
    std::vector<VariableType> vtype;
    std::vector<Float> rhs;
    CSCMatrix A;
    std::vector<BilinearTerm> bilinear_terms;
    std::vector<Float> row_scale;
    std::vector<Float> col_scale;

    Model();

    void add_variable(Float obj_coeff, Float lower = 0.0,
                      Float upper = math::kInfinity,
                      VariableType vt = VariableType::Continuous);
    void add_constraint(const std::vector<Index>& cols,
                        const std::vector<Float>& vals, Float b);
    void update_constraint(Index row, const std::vector<Index>& cols,
                           const std::vector<Float>& vals, Float b);
    const std::vector<Index>& get_constraint_cols(Index row) const;
    const std::vector<Float>& get_constraint_vals(Index row) const;

    // Builds A (CSC) from the accumulated rows. Throws std::invalid_argument when
    // obj / lb / ub / vtype differ in length.
    void finalize();

    // Direct construction from CSC arrays (the generators and the C ABI use it):
    // sets obj = c, rhs = b, lb = 0, ub = +inf, and A; rows within each column are
    // sorted on entry. Throws std::invalid_argument on inconsistent sizes or
    // out-of-range indices.
    static Model from_csc(Index m, Index n, const Index* col_ptrs,
                          const Index* row_idx, const Float* vals,
                          const Float* b, const Float* c);

private:
    std::vector<std::vector<Index>> constraint_cols_;
    std::vector<std::vector<Float>> constraint_vals_;
};

}  // namespace core
}  // namespace sankhya
