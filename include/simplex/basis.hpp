// Basis of an LP min c^T x, A x = b (same names and members as the reference's
// src/simplex/basis.hpp:23-44, so callers of the crossover compile unchanged).
#pragma once

#include <vector>

#include "sankhya/types.hpp"

namespace sankhya {
namespace simplex {

enum class BasisStatus { Basic, AtLower, AtUpper, Superbasic };

// col_status: status of every column; basic_indices[i]: the basic column of row i.
struct Basis {
    std::vector<BasisStatus> col_status;
    std::vector<Index> basic_indices;
};

}  // namespace simplex
}  // namespace sankhya
