// Symbolic analysis of the normal matrix A A^T.
// The first two functions and SymbolicFactorization mirror the reference's
// src/ipm/symbolic.hpp:20-63 and give bit-identical results: exact minimum
// degree with lowest-index tie-break, and the elimination tree + strictly lower
// CSR pattern of P (A A^T) P^T. fill_reducing_ordering is the fast ordering used
// by the solver itself.
#pragma once

#include <vector>

#include "core/sparse_matrix.hpp"

namespace sankhya {
namespace ipm {

struct SymbolicFactorization {
    std::vector<Index> P;       // P[k] = original row eliminated k-th
    std::vector<Index> P_inv;   // P_inv[original] = k
    std::vector<Index> parent;  // elimination tree of the permuted matrix, -1 = root
    core::CSRMatrix L_pattern;  // strictly lower pattern of L, CSR, dummy values 1.0
};

std::vector<Index> compute_amd_ordering(const core::CSRMatrix& A);

void compute_symbolic_factorization(const core::CSRMatrix& A, const std::vector<Index>& P,
                                    SymbolicFactorization& out);

// Approximate minimum degree (quotient graph, element absorption, approximate
// external degrees) on the graph of A A^T; P[k] = original row eliminated k-th.
std::vector<Index> fill_reducing_ordering(const core::CSRMatrix& A);

// The same ordering on an explicit graph: Av[i] = sorted neighbours of vertex i
// (no self loops, symmetric). P[k] = vertex eliminated k-th. Vertices flagged in
// last_rows are eliminated after all others, in their index order.
std::vector<Index> min_degree_order(std::vector<std::vector<Index>> Av,
                                    const std::vector<char>* last_rows = nullptr);

// Sorted, duplicate-free adjacency of A A^T without self loops.
std::vector<std::vector<Index>> aat_graph(const core::CSRMatrix& A);

// Nested dissection of the graph of A A^T: recursive vertex separators from
// breadth-first level structures (a level, or the minimum vertex cut through a band
// of adjacent levels), separators ordered after both sides; parts whose best
// separator is larger than the smaller side, and parts of at most `leaf`
// vertices, are ordered by min_degree_order.
std::vector<Index> nested_dissection_ordering(const core::CSRMatrix& A, Index leaf = 1000);

// Lower adjacency of A A^T in CSR with rows / columns in the given order:
// row k lists j < k (increasing) such that rows P[k], P[j] of A share a column.
void permuted_lower_pattern(const core::CSRMatrix& A, const std::vector<Index>& P_inv,
                            std::vector<Index>& rowptr, std::vector<Index>& colidx);

// Elimination tree of a symmetric pattern given by its strict lower rows (Liu).
std::vector<Index> elimination_tree(Index m, const std::vector<Index>& rowptr,
                                    const std::vector<Index>& colidx);

}  // namespace ipm
}  // namespace sankhya
