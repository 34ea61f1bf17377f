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

#include "cuda/spmv_shape.hpp"

namespace sankhya {
namespace dev {

constexpr int kSpmvNumGroups = 5;
constexpr int kSpmvGroups[kSpmvNumGroups] = {2, 4, 8, 16, 32};

struct SpmvTuning {
    int group = 8;                         // lanes per row in use
    bool windowed = false;                 // shared-memory windows (k_spmv_win) in use
    int heuristic = 8;                     // the row-length rule's width
    bool from_cache = false;               // an earlier tuning of the same shape was reused
    double ms[kSpmvNumGroups] = {};        // fastest event-timed launch per width, plain kernel
    double ms_win[kSpmvNumGroups] = {};    // the same for the windowed kernel (0: not timed)
};

// Chunk table of the windowed SpMV of one CSR matrix (device memory owned here).
// build() cuts the rows, in order, into chunks of at most target_nnz entries
// whose columns fit in kWinMaxCols; runs of rows wider than that form chunks that
// gather from global memory. It reads the row pointers and each row's column
// range back from the device and synchronises `st`.
class SpmvWindows {
public:
    SpmvWindows() = default;
    ~SpmvWindows();
    SpmvWindows(const SpmvWindows&) = delete;
    SpmvWindows& operator=(const SpmvWindows&) = delete;
    void build(int rows, const int* rp, const int* ci, cudaStream_t st, int64_t target_nnz = 49152);
    SpmvShape shape(int group, bool windowed) const;
    double staged_fraction() const { return staged_; }   // share of entries in shared-memory chunks
    int chunks() const { return nchunks_; }

private:
    int4* d_chunks_ = nullptr;
    int nchunks_ = 0;
    int max_cols_ = 0;
    double staged_ = 0.0;
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
// With `win` (built for this matrix) and at least half of the entries in
// shared-memory chunks, the windowed kernel is timed for every width as well.
SpmvTuning spmv_tune(int rows, int cols, int64_t nnz, const int* rp, const int* ci, const double* v,
                     const double* x, double* y, cudaStream_t st, const SpmvWindows* win = nullptr,
                     bool use_cache = true, int reps = 5);

// The table's width for this shape, or the heuristic's if it was never tuned.
int spmv_tuned_group(int rows, int cols, int64_t nnz);

// y = alpha A x + beta y as `shape` says, launched on `st`.
void spmv_axpby(int rows, const SpmvShape& shape, const int* rp, const int* ci, const double* v, const double* x,
                double alpha, double beta, double* y, cudaStream_t st);

}  // namespace dev
}  // namespace sankhya
