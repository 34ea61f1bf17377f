// presolve::find_dependent_rows over the C ABI (sk_presolve_dependent_rows).
#include "presolve/dependent_rows.hpp"

#include <stdexcept>
#include <string>

#include "sankhya/sk_ipm.h"

namespace sankhya {
namespace presolve {

DependentRows find_dependent_rows(const core::Model& model) {
    const int m = model.A.rows, n = model.A.cols;
    if (m <= 0 || n <= 0 || model.rhs.size() != static_cast<size_t>(m) ||
        model.A.col_ptrs.size() != static_cast<size_t>(n) + 1)
        throw std::invalid_argument("find_dependent_rows: model dimensions inconsistent");
    std::vector<int> keep(static_cast<size_t>(m), 1);
    int count = 0;
    double inc = 0.0;
    const int rc = sk_presolve_dependent_rows(m, n, model.A.col_ptrs.data(), model.A.row_indices.data(),
                                              model.A.values.data(), model.rhs.data(), keep.data(), &count, &inc);
    if (rc == SK_ERR_INVALID) throw std::invalid_argument(std::string("find_dependent_rows: ") + sk_last_error());
    if (rc != SK_OK) throw std::runtime_error(std::string("find_dependent_rows: ") + sk_last_error());
    DependentRows out;
    out.inconsistency = inc;
    out.consistent = count == 0 || inc <= 1e-9;
    if (count > 0 && out.consistent)   // (with an inconsistent b the C ABI keeps, and names, no row)
        for (int i = 0; i < m; ++i)
            if (!keep[i]) out.rows.push_back(i);
    return out;
}

}  // namespace presolve
}  // namespace sankhya
