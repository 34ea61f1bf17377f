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

#include <atomic>
#include <cstdint>

#include "cuda/spmv_shape.hpp"

namespace sankhya {
namespace dev {

// acc + sum over q = q0, q0 + G, ... < q1 of v[q] xs[ci[q] - off], in that order (so
// the sum is the same as a plain loop's), with four entries' index, value and
// gather loads in flight at a time.
template <int G>
__device__ __forceinline__ double spmv_row_part(int q0, int q1, const int* __restrict__ ci,
                                                const double* __restrict__ v, const double* __restrict__ xs,
                                                int off) {
    double acc = 0.0;
    int q = q0;
    for (; q + 3 * G < q1; q += 4 * G) {
        const int c0 = ci[q], c1 = ci[q + G], c2 = ci[q + 2 * G], c3 = ci[q + 3 * G];
        const double v0 = v[q], v1 = v[q + G], v2 = v[q + 2 * G], v3 = v[q + 3 * G];
        const double x0 = xs[c0 - off], x1 = xs[c1 - off], x2 = xs[c2 - off], x3 = xs[c3 - off];
        acc += v0 * x0;
        acc += v1 * x1;
        acc += v2 * x2;
        acc += v3 * x3;
    }
    for (; q < q1; q += G) acc += v[q] * xs[ci[q] - off];
    return acc;
}

template <int G, class Epi>
__global__ void __launch_bounds__(256) k_spmv(int rows, const int* __restrict__ rp, const int* __restrict__ ci,
                                              const double* __restrict__ v, const double* __restrict__ x, Epi epi) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = gid / G, lane = gid % G;
    const bool valid = row < rows;
    double acc = 0.0;
    if (valid) acc = spmv_row_part<G>(rp[row] + lane, rp[row + 1], ci, v, x, 0);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
    if (valid && lane == 0) epi(row, acc);
}

inline int spmv_blocks(int64_t threads) { return static_cast<int>((threads + 255) / 256); }

// k_spmv over the rows of the LPs whose entry of `on` is nonzero (lp_of: the LP of
// each row); the other rows are skipped without reading their entries, and their
// outputs are left as they are.
template <int G, class Epi>
__global__ void __launch_bounds__(256) k_spmv_masked(int rows, const int* __restrict__ rp, const int* __restrict__ ci,
                                                     const double* __restrict__ v, const double* __restrict__ x,
                                                     const int* __restrict__ lp_of, const double* __restrict__ on,
                                                     Epi epi) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = gid / G, lane = gid % G;
    const bool valid = row < rows && on[lp_of[row]] != 0.0;
    double acc = 0.0;
    if (valid) acc = spmv_row_part<G>(rp[row] + lane, rp[row + 1], ci, v, x, 0);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
    if (valid && lane == 0) epi(row, acc);
}

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

// Launches k_spmv_masked with `group` lanes per row (as spmv above).
template <class Epi>
void spmv_masked(int rows, int group, const int* rp, const int* ci, const double* v, const double* x,
                 const int* lp_of, const double* on, Epi epi, cudaStream_t st) {
    if (rows <= 0) return;
    const int64_t threads = static_cast<int64_t>(rows) * group;
    switch (group) {
    case 2: k_spmv_masked<2><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, lp_of, on, epi); break;
    case 4: k_spmv_masked<4><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, lp_of, on, epi); break;
    case 8: k_spmv_masked<8><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, lp_of, on, epi); break;
    case 16: k_spmv_masked<16><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, lp_of, on, epi); break;
    default: k_spmv_masked<32><<<spmv_blocks(threads), 256, 0, st>>>(rows, rp, ci, v, x, lp_of, on, epi); break;
    }
}

// ---- windowed variant: x staged in shared memory per chunk of rows ----
//
// Rows are cut into chunks (int4 {row0, row1, col0, ncols}) whose entries all lie
// in columns [col0, col0 + ncols); one CTA of kWinThreads threads copies that
// window of x into shared memory once and then runs the chunk's rows with G lanes
// per row, so the per-entry gathers of x hit shared memory instead of each
// taking its own L1 sector lookup. A chunk with ncols < 0 holds rows too wide for
// any window and gathers from global memory. Built by SpmvWindows (autotune.hpp).
template <int G, class Epi>
__global__ void __launch_bounds__(kWinThreads) k_spmv_win(const int4* __restrict__ chunks,
                                                           const int* __restrict__ rp, const int* __restrict__ ci,
                                                           const double* __restrict__ v,
                                                           const double* __restrict__ x, Epi epi) {
    extern __shared__ double xs[];
    const int4 ch = chunks[blockIdx.x];
    const bool staged = ch.w >= 0;
    if (staged)
        for (int t = threadIdx.x; t < ch.w; t += blockDim.x) xs[t] = x[ch.z + t];
    __syncthreads();
    const int groups = blockDim.x / G;
    const int g = threadIdx.x / G, lane = threadIdx.x % G;
    // the trip count depends on the chunk only, so every lane reaches the shuffles
    for (int base = ch.x; base < ch.y; base += groups) {
        const int row = base + g;
        const bool valid = row < ch.y;
        double acc = 0.0;
        if (valid) {
            const int q1 = rp[row + 1];
            if (staged) acc = spmv_row_part<G>(rp[row] + lane, q1, ci, v, xs, ch.z);
            else acc = spmv_row_part<G>(rp[row] + lane, q1, ci, v, x, 0);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
        if (valid && lane == 0) epi(row, acc);
    }
}

// Opts k_spmv_win<G, Epi> into kWinMaxCols doubles of dynamic shared memory on
// the current device (once per instantiation and device; devices 0..63).
// Returns false if the device refuses (the caller then runs the plain kernel).
template <int G, class Epi>
inline bool win_smem_attr() {
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load() & bit) return true;
    if (cudaFuncSetAttribute(k_spmv_win<G, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kWinMaxCols * static_cast<int>(sizeof(double))) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    done.fetch_or(bit);
    return true;
}

template <class Epi>
void spmv_win(int rows, const SpmvShape& sh, const int* rp, const int* ci, const double* v, const double* x, Epi epi,
              cudaStream_t st) {
    if (sh.nchunks <= 0) return;
    const int smem = sh.max_cols * static_cast<int>(sizeof(double));
    bool ok = false;
    switch (sh.group) {
    case 2: if ((ok = win_smem_attr<2, Epi>()))
            k_spmv_win<2><<<sh.nchunks, kWinThreads, smem, st>>>(sh.chunks, rp, ci, v, x, epi);
        break;
    case 4: if ((ok = win_smem_attr<4, Epi>()))
            k_spmv_win<4><<<sh.nchunks, kWinThreads, smem, st>>>(sh.chunks, rp, ci, v, x, epi);
        break;
    case 8: if ((ok = win_smem_attr<8, Epi>()))
            k_spmv_win<8><<<sh.nchunks, kWinThreads, smem, st>>>(sh.chunks, rp, ci, v, x, epi);
        break;
    case 16: if ((ok = win_smem_attr<16, Epi>()))
            k_spmv_win<16><<<sh.nchunks, kWinThreads, smem, st>>>(sh.chunks, rp, ci, v, x, epi);
        break;
    default: if ((ok = win_smem_attr<32, Epi>()))
            k_spmv_win<32><<<sh.nchunks, kWinThreads, smem, st>>>(sh.chunks, rp, ci, v, x, epi);
        break;
    }
    if (!ok) spmv(rows, sh.group, rp, ci, v, x, epi, st);
}

// The SpMV of a matrix as its shape says: windowed or plain, with its lane width.
template <class Epi>
void spmv(int rows, const SpmvShape& sh, const int* rp, const int* ci, const double* v, const double* x, Epi epi,
          cudaStream_t st) {
    if (sh.windowed) spmv_win(rows, sh, rp, ci, v, x, epi, st);
    else spmv(rows, sh.group, rp, ci, v, x, epi, st);
}

struct EpiAxpby {        // y = alpha d + beta y
    double alpha, beta;
    double* y;
    __device__ void operator()(int i, double d) const { y[i] = beta == 0.0 ? alpha * d : alpha * d + beta * y[i]; }
};

}  // namespace dev
}  // namespace sankhya
