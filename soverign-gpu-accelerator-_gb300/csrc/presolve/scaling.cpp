// Ruiz equilibration of an LP model (presolve). Follows the reference's
// presolve::apply_ruiz_scaling (src/presolve/scaling.cpp:18-146): the same
// per-pass rule (row maxima, 1/sqrt; then column maxima of the row-scaled
// matrix, 1/sqrt; integer columns and empty rows / columns left alone), the
// same stopping test (all maxima within 1e-4 of 1) and the same final
// transformation of rhs, objective and bounds, with the floating-point
// operations in the same order, so the scaled model is bit-identical.
// The data layout differs: one pass walks the CSC arrays twice (row maxima,
// then column maxima fused with the column scaling) instead of building
// per-pass temporaries for each step.
#include "presolve/scaling.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

namespace sankhya {
namespace presolve {

namespace {
constexpr Float kZero = 1e-15;      // rows / columns whose largest |entry| is below this keep factor 1
constexpr Float kStop = 1e-4;       // stopping tolerance on |max - 1|
}  // namespace

int ruiz_scale_csc(Index m, Index n, const Index* cp, const Index* ri, Float* v, Float* rhs, Float* obj,
                   Float* lb, Float* ub, const unsigned char* integer_cols, int max_iterations, Float* row_scale,
                   Float* col_scale) {
    if (m < 0 || n < 0) throw std::invalid_argument("ruiz_scale_csc: negative size");
    if (m == 0 || n == 0) return 0;
    if (!cp || !row_scale || !col_scale) throw std::invalid_argument("ruiz_scale_csc: missing array");
    const Index nnz = cp[n];
    std::vector<Float> rmax(static_cast<size_t>(m)), rfac(static_cast<size_t>(m));
    int passes = 0;
    for (int it = 0; it < max_iterations; ++it) {
        ++passes;
        Float dev_r = 0.0, dev_c = 0.0;
        std::fill(rmax.begin(), rmax.end(), 0.0);
        for (Index q = 0; q < nnz; ++q) {
            const Float a = std::abs(v[q]);
            if (a > rmax[ri[q]]) rmax[ri[q]] = a;
        }
        for (Index i = 0; i < m; ++i) {
            rfac[i] = 1.0;
            if (rmax[i] > kZero) {
                rfac[i] = 1.0 / std::sqrt(rmax[i]);
                dev_r = std::max(dev_r, std::abs(rmax[i] - 1.0));
                row_scale[i] *= rfac[i];
            }
        }
        // column pass on the row-scaled values: scale each entry by its row factor,
        // take the column maximum, then scale the column
        for (Index j = 0; j < n; ++j) {
            Float cmax = 0.0;
            for (Index q = cp[j]; q < cp[j + 1]; ++q) {
                v[q] *= rfac[ri[q]];
                cmax = std::max(cmax, std::abs(v[q]));
            }
            if (integer_cols && integer_cols[j]) continue;
            if (cmax > kZero) {
                const Float f = 1.0 / std::sqrt(cmax);
                dev_c = std::max(dev_c, std::abs(cmax - 1.0));
                col_scale[j] *= f;
                for (Index q = cp[j]; q < cp[j + 1]; ++q) v[q] *= f;
            }
        }
        if (dev_r < kStop && dev_c < kStop) break;
    }
    if (rhs)
        for (Index i = 0; i < m; ++i) rhs[i] *= row_scale[i];
    for (Index j = 0; j < n; ++j) {
        if (obj) obj[j] *= col_scale[j];
        if (lb && lb[j] > -math::kInfinity) lb[j] /= col_scale[j];
        if (ub && ub[j] < math::kInfinity) ub[j] /= col_scale[j];
    }
    return passes;
}

void apply_ruiz_scaling(core::Model& model, int max_iterations) {
    const Index m = model.A.rows, n = model.A.cols;
    if (m == 0 || n == 0) return;
    if (model.row_scale.empty()) model.row_scale.assign(static_cast<size_t>(m), 1.0);
    if (model.col_scale.empty()) model.col_scale.assign(static_cast<size_t>(n), 1.0);
    if (static_cast<Index>(model.row_scale.size()) != m || static_cast<Index>(model.col_scale.size()) != n ||
        static_cast<Index>(model.rhs.size()) != m || static_cast<Index>(model.obj.size()) != n ||
        static_cast<Index>(model.lb.size()) != n || static_cast<Index>(model.ub.size()) != n)
        throw std::invalid_argument("apply_ruiz_scaling: model vectors do not match A");
    std::vector<unsigned char> integer(static_cast<size_t>(n), 0);
    for (Index j = 0; j < n; ++j)
        integer[j] = (static_cast<size_t>(j) < model.vtype.size() && model.vtype[j] != VariableType::Continuous);
    ruiz_scale_csc(m, n, model.A.col_ptrs.data(), model.A.row_indices.data(), model.A.values.data(),
                   model.rhs.data(), model.obj.data(), model.lb.data(), model.ub.data(), integer.data(),
                   max_iterations, model.row_scale.data(), model.col_scale.data());
}

}  // namespace presolve
}  // namespace sankhya
