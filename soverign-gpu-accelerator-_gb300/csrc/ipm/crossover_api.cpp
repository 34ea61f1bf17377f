// ipm::generate_crossover_basis: the reference's C++ entry point (src/ipm/crossover.cuh:30-33)
// over the device crossover.
#include <stdexcept>
#include <string>

#include "cuda/crossover.hpp"
#include "ipm/crossover.hpp"

namespace sankhya {
namespace ipm {

simplex::Basis generate_crossover_basis(const core::Model& model, const std::vector<Float>& x_ipm) {
    const Index m = model.A.rows, n = model.A.cols;
    if (static_cast<Index>(x_ipm.size()) != n) throw std::invalid_argument("generate_crossover_basis: |x| != n");
    if (m > dev::kCrossoverMaxRows) throw std::length_error("generate_crossover_basis: too many rows");
    std::vector<int> basic(static_cast<size_t>(m)), status(static_cast<size_t>(n));
    const Float* lb = model.lb.size() == static_cast<size_t>(n) ? model.lb.data() : nullptr;
    const Float* ub = model.ub.size() == static_cast<size_t>(n) ? model.ub.data() : nullptr;
    std::string msg;
    const int rc = dev::crossover(m, n, model.A.col_ptrs.data(), model.A.row_indices.data(), model.A.values.data(),
                                  lb, ub, x_ipm.data(), basic.data(), status.data(), nullptr, &msg);
    if (rc != 0) throw std::runtime_error(msg.empty() ? std::string("Crossover failed") : msg);
    simplex::Basis b;
    b.basic_indices.assign(basic.begin(), basic.end());
    b.col_status.resize(static_cast<size_t>(n));
    for (Index j = 0; j < n; ++j)
        b.col_status[j] = status[j] == dev::kBasic ? simplex::BasisStatus::Basic
                          : status[j] == dev::kAtUpper ? simplex::BasisStatus::AtUpper
                                                       : simplex::BasisStatus::AtLower;
    return b;
}

}  // namespace ipm
}  // namespace sankhya
