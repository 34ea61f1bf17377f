// Launch-shape autotuner for the vector CSR SpMV (spmv.cuh).
//
// The reference hands every SpMV to cusparseSpMV with the default algorithm
// (src/ipm/mehrotra_device.cu:512,603,635,936). Here the kernel is this
// project's own, and its one shape parameter, the number of lanes G that share a
// row, is chosen per matrix by timing: short rows (A^T of a transportation LP,
// 4 entries) want few lanes, long rows (A of a dense batch member, 50+) want a
// warp. The choice is kept per matrix shape for the life of the process, so
// every solver built on the same shape uses the same width and gives the same
// bits.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sankhya {
namespace dev {

constexpr int kSpmvNumGroups = 5;
constexpr int kSpmvGroups[kSpmvNumGroups] = {2, 4, 8, 16, 32};

struct SpmvTuning {
    int group = 8;                         // lanes per row in use
    int heuristic = 8;                     // the row-length rule's width
    bool from_cache = false;               // an earlier tuning of the same shape was reused
    double ms[kSpmvNumGroups] = {};        // fastest event-timed launch per width (kSpmvGroups order)
};

// Row-length rule used before any timing: about one lane per average row entry,
// rounded to a power of two in [2, 32].
int spmv_heuristic_group(int64_t nnz, int rows);

// Times k_spmv (y = A x) on this CSR matrix for every width in kSpmvGroups: one
// warm-up launch and `reps` launches between CUDA events on `st` for each, the
// fastest launch counting. The winner is kept in a process-wide table under
// (device, rows, cols, nnz); a width replaces the heuristic's only when it is at
// least 3% faster, so near-ties keep a stable choice. With use_cache, a shape
// already in the table is not timed again. d_y (rows entries) is overwritten,
// d_x (cols entries) is read. Synchronises `st`.
SpmvTuning spmv_tune(int rows, int cols, int64_t nnz, const int* rp, const int* ci, const double* v,
                     const double* x, double* y, cudaStream_t st, bool use_cache = true, int reps = 5);

// The table's width for this shape, or the heuristic's if it was never tuned.
int spmv_tuned_group(int rows, int cols, int64_t nnz);

// y = alpha A x + beta y with `group` lanes per row, launched on `st`.
void spmv_axpby(int rows, int group, const int* rp, const int* ci, const double* v, const double* x, double alpha,
                double beta, double* y, cudaStream_t st);

}  // namespace dev
}  // namespace sankhya
