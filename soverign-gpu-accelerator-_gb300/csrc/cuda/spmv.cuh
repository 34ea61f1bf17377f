// Vector CSR SpMV with a fused epilogue, shared by the IPM (A x, A^T y with the
// reference's residual / direction formulas fused in) and the public SpMV plans.
// Replaces the reference's cusparseSpMV CSR FP64 call sites
// (src/ipm/mehrotra_device.cu:512,603,635,936).
//
// G consecutive lanes own one row (G = 2..32, a power of two): lane l sums
// entries l, l + G, ... of the row, then the G partial sums are combined with
// xor shuffles and lane 0 hands the row's value to the epilogue. Consecutive
// rows are consecutive lane groups, so a warp reads 32 / G rows' index and value
// ranges, which are contiguous in CSR order. The best G depends on the row
// lengths and on how x is gathered; spmv_tune() (autotune.hpp) times them.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sankhya {
namespace dev {

template <int G, class Epi>
__global__ void __launch_bounds__(256) k_spmv(int rows, const int* __restrict__ rp, const int* __restrict__ ci,
                                              const double* __restrict__ v, const double* __restrict__ x, Epi epi) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = gid / G, lane = gid % G;
    const bool valid = row < rows;
    double acc = 0.0;
    if (valid)
        for (int q = rp[row] + lane; q < rp[row + 1]; q += G) acc += v[q] * x[ci[q]];
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
    if (valid && lane == 0) epi(row, acc);
}

inline int spmv_blocks(int64_t threads) { return static_cast<int>((threads + 255) / 256); }

// Launches the SpMV with `group` lanes per row (2, 4, 8, 16; anything else: 32).
template <class Epi>
void spmv(int rows, int group, const int* rp, const int* ci, const double* v, const double* x, Epi epi,
          cudaStream_t st) {
    if (rows <= 0) return;
    const int64_t threads = static_cast<int64_t>(rows) * group;
    switch (group) {
    case 2: k_spmv<2><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, epi); break;
    case 4: k_spmv<4><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, epi); break;
    case 8: k_spmv<8><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, epi); break;
    case 16: k_spmv<16><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, epi); break;
    default: k_spmv<32><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, epi); break;
    }
}

struct EpiAxpby {        // y = alpha d + beta y
    double alpha, beta;
    double* y;
    __device__ void operator()(int i, double d) const { y[i] = beta == 0.0 ? alpha * d : alpha * d + beta * y[i]; }
};

}  // namespace dev
}  // namespace sankhya
