// CSC / CSR storage and the CSC -> CSR transpose
// (reference behaviour: src/core/sparse_matrix.cpp:49-85).
#include "core/sparse_matrix.hpp"

#include <algorithm>
#include <utility>

namespace sankhya {
namespace core {

CSCMatrix::CSCMatrix(Index r, Index c, std::vector<Float> vals,
                     std::vector<Index> rows_idx, std::vector<Index> ptrs)
    : rows(r), cols(c), col_ptrs(std::move(ptrs)),
      row_indices(std::move(rows_idx)), values(std::move(vals)) {}

Index CSCMatrix::nnz() const { return static_cast<Index>(values.size()); }

Float CSCMatrix::get(Index r, Index c) const {
    if (r < 0 || c < 0 || r >= rows || c >= cols) return 0.0;
    auto first = row_indices.begin() + col_ptrs[static_cast<size_t>(c)];
    auto last = row_indices.begin() + col_ptrs[static_cast<size_t>(c) + 1];
    auto it = std::lower_bound(first, last, r);
    if (it == last || *it != r) return 0.0;
    return values[static_cast<size_t>(it - row_indices.begin())];
}

CSRMatrix to_csr(const CSCMatrix& a) {
    CSRMatrix out;
    out.rows = a.rows;
    out.cols = a.cols;
    const size_t nz = static_cast<size_t>(a.col_ptrs.empty() ? 0 : a.col_ptrs.back());
    out.row_ptrs.assign(static_cast<size_t>(a.rows) + 1, 0);
    for (size_t k = 0; k < nz; ++k) out.row_ptrs[static_cast<size_t>(a.row_indices[k]) + 1]++;
    for (Index i = 0; i < a.rows; ++i) out.row_ptrs[i + 1] += out.row_ptrs[i];
    out.col_indices.resize(nz);
    out.values.resize(nz);
    std::vector<Index> next(out.row_ptrs.begin(), out.row_ptrs.end() - 1);
    for (Index j = 0; j < a.cols; ++j) {
        for (Index k = a.col_ptrs[j]; k < a.col_ptrs[j + 1]; ++k) {
            const Index dst = next[static_cast<size_t>(a.row_indices[k])]++;
            out.col_indices[dst] = j;
            out.values[dst] = a.values[k];
        }
    }
    return out;
}

}  // namespace core
}  // namespace sankhya
