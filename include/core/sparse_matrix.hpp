// Compressed sparse column / row matrices of the LP engine.
// Same layout and member names as the reference's src/core/sparse_matrix.hpp:28-75
// (col_ptrs / row_indices / values for CSC, row_ptrs / col_indices / values for
// CSR, int32 indices, FP64 values, indices sorted within each column / row).
#pragma once

#include <cstddef>
#include <vector>

#include "sankhya/types.hpp"

namespace sankhya {
namespace core {

struct CSCMatrix {
    Index rows = 0;
    Index cols = 0;
    std::vector<Index> col_ptrs;
    std::vector<Index> row_indices;
    std::vector<Float> values;

    CSCMatrix() : col_ptrs(1, 0) {}
    CSCMatrix(Index rows, Index cols, std::vector<Float> vals,
              std::vector<Index> rows_idx, std::vector<Index> col_ptrs);

    Index nnz() const;
    // A(r, c) by binary search within column c; 0 when absent or out of range.
    Float get(Index r, Index c) const;
};

struct CSRMatrix {
    Index rows = 0;
    Index cols = 0;
    std::vector<Index> row_ptrs;
    std::vector<Index> col_indices;
    std::vector<Float> values;
};

// O(nnz) counting-sort transpose of the storage; values are copied bit-exactly
// and the column indices of every row come out increasing.
CSRMatrix to_csr(const CSCMatrix& csc);

}  // namespace core
}  // namespace sankhya
