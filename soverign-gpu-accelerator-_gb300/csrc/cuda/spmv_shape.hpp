// Launch description of the SpMV of one CSR matrix (host-side; see spmv.cuh).
#pragma once

#include <cuda_runtime.h>

namespace sankhya {
namespace dev {

constexpr int kWinThreads = 1024;          // threads per CTA of the windowed kernel
constexpr int kWinMaxCols = 24576;         // widest window: 192 KB of FP64 x per CTA

struct SpmvShape {
    int group = 8;                  // lanes per row
    bool windowed = false;          // k_spmv_win over `chunks`
    const int4* chunks = nullptr;   // device chunk table {row0, row1, col0, ncols}
    int nchunks = 0;
    int max_cols = 0;               // widest staged window (columns)
};

}  // namespace dev
}  // namespace sankhya
