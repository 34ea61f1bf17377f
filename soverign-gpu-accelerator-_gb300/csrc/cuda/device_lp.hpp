// Device-resident batch LP (block-diagonal concatenation of the batch) and the
// segmented-reduction layout shared by the IPM kernels and the KKT engine.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace sankhya {
namespace dev {

struct DeviceLP {
    int nlp = 0;
    int M = 0, N = 0;
    int64_t nnz = 0;
    // A (scaled) in CSR and in CSC (= CSR of A^T); int32 indices, FP64 values
    int* a_rp = nullptr;  int* a_ci = nullptr;  double* a_v = nullptr;
    int* t_rp = nullptr;  int* t_ci = nullptr;  double* t_v = nullptr;
    double* b = nullptr;  double* c = nullptr;   // scaled
    double* R = nullptr;  double* C = nullptr;   // Ruiz row / column factors
    int* row_lp = nullptr; int* col_lp = nullptr;
    // reduction chunks: chunk q covers [start[q], end[q]) of one LP; chunks of LP k
    // are [ptr[k], ptr[k+1])
    int n_mchunks = 0, n_nchunks = 0;
    int* mc_start = nullptr; int* mc_end = nullptr; int* mc_ptr = nullptr;
    int* nc_start = nullptr; int* nc_end = nullptr; int* nc_ptr = nullptr;
    int spmv_group_A = 4, spmv_group_T = 4;      // lanes per row of the two SpMVs
};

// Chunking of [0, total) split at LP offsets into pieces of at most `chunk` entries.
inline void make_chunks(const std::vector<int>& off, int chunk, std::vector<int>& start, std::vector<int>& end,
                        std::vector<int>& ptr) {
    const int nlp = static_cast<int>(off.size()) - 1;
    start.clear();
    end.clear();
    ptr.assign(static_cast<size_t>(nlp) + 1, 0);
    for (int k = 0; k < nlp; ++k) {
        for (int s = off[k]; s < off[k + 1]; s += chunk) {
            start.push_back(s);
            end.push_back(s + chunk < off[k + 1] ? s + chunk : off[k + 1]);
        }
        if (off[k] == off[k + 1]) { start.push_back(off[k]); end.push_back(off[k]); }
        ptr[k + 1] = static_cast<int>(start.size());
    }
}

}  // namespace dev
}  // namespace sankhya
