// Allocation-free KKT solve for small systems: (A diag(theta) A^T) dy = rhs with
// m <= SK_KKT_NOALLOC_MAX_ROWS, entirely in one fixed device array.
//
// Why it exists: sk_kkt_create / sk_kkt_factorize_device / sk_kkt_solve_device
// reserve their fronts and vectors with cudaMalloc. Some callers cannot do that
// at the point where they need a solve: a host that has handed all device memory
// to its own pool (a framework's caching allocator), or one that must not let
// cudaMalloc / cudaFree synchronise the device while its other streams are busy.
// This entry point serves them for small normal-equation systems (a crossover
// step, a small LP's Newton system) with no allocation of any kind on the
// success path: the matrix, its factor and every work vector live in the
// file-scope array below, whose address is fetched once per device.
//
// Method (FP64 throughout, one thread block): M0 = A diag(theta) A^T formed by a
// sorted merge of row pairs; equilibration D = 1 / sqrt(max(|m_ii|, 1e-12)); dense
// Cholesky of D M0 D + delta I with the KKT engine's FP64 regularisation ladder
// (delta = 1e-9, x10, five tries); forward / backward substitution; iterative
// refinement against the unregularised M0 until ||rhs - M0 dy||_inf <= tol *
// max(1, ||rhs||_inf), stopping when a step no longer reduces the residual. The
// factor sits in the lower triangle of the scratch matrix and M0 in the strict
// upper triangle plus a diagonal vector, so both fit in one m x m block.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "api/sk_error.hpp"
#include "sankhya/sk_ipm.h"

namespace {

constexpr int kRows = SK_KKT_NOALLOC_MAX_ROWS;
constexpr int kVectors = 9;                 // d0, D, b0, x, bak, r, t1, t2, t3
constexpr int kTail = 32;                   // results read back by the host
constexpr size_t kScratchDoubles = static_cast<size_t>(kRows) * kRows + kVectors * kRows + kTail;
constexpr int kThreads = 512;
constexpr int kDeltaTries = 5;
constexpr int kMaxRefine = 10;
constexpr int kMaxDevices = 64;

// The one scratch area (542,976 bytes). Every call on a device shares it.
static __device__ __align__(256) double g_kkt_noalloc_scratch[kScratchDoubles];

// status codes written to tail[0] as (1 + code); 0 means the kernel never ran
enum : int { kOk = 0, kBadInput = 1, kNotPd = 2, kNotConverged = 3 };

__device__ double block_max(double v, double* red) {
    for (int s = 16; s > 0; s >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, s));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) r = fmax(r, red[w]);
    return r;
}

// out = D L^-T L^-1 D b (W holds L in its lower triangle, column-major, ld = m)
__device__ void chol_solve(int m, const double* W, const double* D, const double* b, double* out, double* z,
                           double* y) {
    const int tid = threadIdx.x;
    for (int i = tid; i < m; i += kThreads) z[i] = D[i] * b[i];
    __syncthreads();
    for (int k = 0; k < m; ++k) {           // L y = z; z[k] is final once column k - 1 is done
        const double yk = z[k] / W[k + static_cast<size_t>(k) * m];
        if (tid == 0) y[k] = yk;
        for (int r = k + 1 + tid; r < m; r += kThreads) z[r] -= W[r + static_cast<size_t>(k) * m] * yk;
        __syncthreads();
    }
    for (int k = m - 1; k >= 0; --k) {      // L^T w = y; w goes to z
        const double wk = y[k] / W[k + static_cast<size_t>(k) * m];
        if (tid == 0) z[k] = wk;
        for (int r = tid; r < k; r += kThreads) y[r] -= W[k + static_cast<size_t>(r) * m] * wk;
        __syncthreads();
    }
    for (int i = tid; i < m; i += kThreads) out[i] = D[i] * z[i];
    __syncthreads();
}

// r = b - M0 x with M0 = strict upper triangle of W plus diagonal d0; returns ||r||_inf
__device__ double residual(int m, const double* W, const double* d0, const double* b, const double* x, double* r,
                           double* red) {
    double mx = 0.0;
    for (int i = threadIdx.x; i < m; i += kThreads) {
        double s = d0[i] * x[i];
        for (int j = 0; j < i; ++j) s += W[j + static_cast<size_t>(i) * m] * x[j];
        for (int j = i + 1; j < m; ++j) s += W[i + static_cast<size_t>(j) * m] * x[j];
        r[i] = b[i] - s;
        mx = fmax(mx, fabs(r[i]));
    }
    return block_max(mx, red);
}

__global__ void __launch_bounds__(kThreads) k_kkt_noalloc(int m, int n, const int* __restrict__ rp,
                                                          const int* __restrict__ ci, const double* __restrict__ v,
                                                          const double* __restrict__ theta, double* rhs, double tol,
                                                          double* __restrict__ scratch) {
    __shared__ double red[kThreads / 32];
    __shared__ int bad;
    const int tid = threadIdx.x;
    double* W = scratch;
    double* d0 = W + static_cast<size_t>(kRows) * kRows;
    double* D = d0 + kRows;
    double* b0 = D + kRows;
    double* x = b0 + kRows;
    double* bak = x + kRows;
    double* r = bak + kRows;
    double* t1 = r + kRows;
    double* t2 = t1 + kRows;
    double* t3 = t2 + kRows;
    double* tail = t3 + kRows;
    if (tid == 0) bad = 0;
    __syncthreads();
    // input checks: CSR structure, sorted in-range columns, finite values
    if (tid == 0 && rp[0] != 0) bad = 1;
    for (int i = tid; i < m; i += kThreads) {
        const int q0 = rp[i], q1 = rp[i + 1];
        if (q0 < 0 || q1 < q0) { bad = 1; continue; }
        for (int q = q0; q < q1; ++q) {
            const int c = ci[q];
            if (c < 0 || c >= n || (q > q0 && c <= ci[q - 1]) || !isfinite(v[q])) { bad = 1; break; }
        }
        if (!isfinite(rhs[i])) bad = 1;
    }
    for (int j = tid; j < n; j += kThreads)
        if (!(theta[j] >= 0.0) || !isfinite(theta[j])) bad = 1;
    __syncthreads();
    if (bad) {
        if (tid == 0) { tail[0] = 1.0 + kBadInput; tail[1] = 0.0; tail[2] = 0.0; tail[3] = 0.0; }
        return;
    }
    // M0: strict upper triangle into W, diagonal into d0
    for (int p = tid; p < m * m; p += kThreads) {
        const int i = p % m, j = p / m;
        if (i > j) continue;
        double s = 0.0;
        int a = rp[i], b = rp[j];
        const int ae = rp[i + 1], be = rp[j + 1];
        while (a < ae && b < be) {
            const int ca = ci[a], cb = ci[b];
            if (ca == cb) { s += v[a] * theta[ca] * v[b]; ++a; ++b; }
            else if (ca < cb) ++a;
            else ++b;
        }
        if (i == j) d0[i] = s;
        else W[i + static_cast<size_t>(j) * m] = s;
    }
    __syncthreads();
    double bn = 0.0;
    for (int i = tid; i < m; i += kThreads) {
        D[i] = 1.0 / sqrt(fmax(fabs(d0[i]), 1e-12));
        b0[i] = rhs[i];
        bn = fmax(bn, fabs(rhs[i]));
    }
    bn = block_max(bn, red);
    // factor D M0 D + delta I, raising delta until every pivot is positive
    double delta = 1e-9;
    bool ok = false;
    for (int attempt = 0; attempt < kDeltaTries && !ok; ++attempt, delta *= 10.0) {
        for (int p = tid; p < m * m; p += kThreads) {
            const int i = p % m, j = p / m;
            if (i > j) W[p] = D[i] * W[j + static_cast<size_t>(i) * m] * D[j];
            else if (i == j) W[p] = D[i] * D[i] * d0[i] + delta;
        }
        __syncthreads();
        ok = true;
        for (int k = 0; k < m; ++k) {
            const double piv = W[k + static_cast<size_t>(k) * m];
            __syncthreads();                 // every thread has read the pivot
            if (!(piv > 0.0) || !isfinite(piv)) { ok = false; break; }   // uniform across the block
            const double lkk = sqrt(piv), inv = 1.0 / lkk;
            if (tid == 0) W[k + static_cast<size_t>(k) * m] = lkk;
            for (int i = k + 1 + tid; i < m; i += kThreads) W[i + static_cast<size_t>(k) * m] *= inv;
            __syncthreads();
            const int t = m - k - 1;
            for (int p = tid; p < t * t; p += kThreads) {
                const int i = k + 1 + p % t, j = k + 1 + p / t;
                if (i < j) continue;         // the strict upper triangle holds M0
                W[i + static_cast<size_t>(j) * m] -= W[i + static_cast<size_t>(k) * m] * W[j + static_cast<size_t>(k) * m];
            }
            __syncthreads();
        }
    }
    if (!ok) {
        if (tid == 0) { tail[0] = 1.0 + kNotPd; tail[1] = 0.0; tail[2] = bn; tail[3] = delta / 10.0; }
        return;
    }
    // solve and refine against M0
    const double target = tol * fmax(1.0, bn);
    chol_solve(m, W, D, b0, x, t1, t2);
    double rn = residual(m, W, d0, b0, x, r, red);
    for (int it = 0; it < kMaxRefine && rn > target; ++it) {
        for (int i = tid; i < m; i += kThreads) bak[i] = x[i];
        chol_solve(m, W, D, r, t3, t1, t2);   // correction into t3
        for (int i = tid; i < m; i += kThreads) x[i] += t3[i];
        __syncthreads();
        const double rn2 = residual(m, W, d0, b0, x, r, red);
        if (rn2 >= rn) {
            for (int i = tid; i < m; i += kThreads) x[i] = bak[i];
            __syncthreads();
            break;
        }
        rn = rn2;
    }
    for (int i = tid; i < m; i += kThreads) rhs[i] = x[i];
    if (tid == 0) {
        tail[0] = 1.0 + (rn <= target ? kOk : kNotConverged);
        tail[1] = rn;
        tail[2] = bn;
        tail[3] = delta / 10.0;
    }
}

std::mutex g_setup_mu;
double* g_scratch[kMaxDevices] = {};

// Address of the scratch array on the current device, fetched on the first call
// made with that device current. The same set-up also loads the kernel itself
// (with lazy module loading a kernel is otherwise loaded at its first launch,
// which may allocate), so later calls launch an already loaded kernel.
cudaError_t scratch_for_current_device(double** out) {
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return rc;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch[dev]) {
        cudaFuncAttributes attr;
        rc = cudaFuncGetAttributes(&attr, k_kkt_noalloc);
        if (rc != cudaSuccess) return rc;
        void* p = nullptr;
        rc = cudaGetSymbolAddress(&p, g_kkt_noalloc_scratch);
        if (rc != cudaSuccess) return rc;
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int sk_kkt_solve_noalloc(int m, int n, const int* d_row_ptrs, const int* d_col_idx, const double* d_vals,
                                    const double* d_theta, double* d_rhs, double tol, void* stream) {
    using sankhya::api::set_error;
    sankhya::api::clear_error();
    if (m <= 0 || n <= 0 || !d_row_ptrs || !d_col_idx || !d_vals || !d_theta || !d_rhs || !(tol > 0.0)) {
        set_error("sk_kkt_solve_noalloc: invalid argument");
        return SK_ERR_INVALID;
    }
    if (m > SK_KKT_NOALLOC_MAX_ROWS) {
        set_error("sk_kkt_solve_noalloc: m = " + std::to_string(m) + " exceeds the fixed scratch limit of " +
                  std::to_string(SK_KKT_NOALLOC_MAX_ROWS) + " rows; use sk_kkt_create / sk_kkt_solve_device");
        return SK_ERR_TOO_LARGE;
    }
    double* scratch = nullptr;
    cudaError_t rc = scratch_for_current_device(&scratch);
    if (rc != cudaSuccess) {
        set_error(std::string("sk_kkt_solve_noalloc: scratch set-up failed: ") + cudaGetErrorString(rc));
        return SK_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* tail = scratch + static_cast<size_t>(kRows) * kRows + kVectors * kRows;
    double h[4] = {0.0, 0.0, 0.0, 0.0};
    // the status word must start at zero so that a kernel that never ran reads as a failure
    rc = cudaMemsetAsync(tail, 0, sizeof(double) * 4, st);
    if (rc == cudaSuccess) {
        k_kkt_noalloc<<<1, kThreads, 0, st>>>(m, n, d_row_ptrs, d_col_idx, d_vals, d_theta, d_rhs, tol, scratch);
        rc = cudaGetLastError();
    }
    if (rc == cudaSuccess) rc = cudaMemcpyAsync(h, tail, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (rc == cudaSuccess) rc = cudaStreamSynchronize(st);
    if (rc != cudaSuccess) {
        set_error(std::string("sk_kkt_solve_noalloc: ") + cudaGetErrorString(rc));
        return SK_ERR_CUDA;
    }
    const int code = static_cast<int>(h[0]) - 1;
    switch (code) {
        case kOk: return SK_OK;
        case kBadInput:
            set_error("sk_kkt_solve_noalloc: bad input (CSR structure, unsorted or out-of-range columns, "
                      "negative or non-finite theta, non-finite values)");
            return SK_ERR_INVALID;
        case kNotPd:
            set_error("sk_kkt_solve_noalloc: not positive definite for any regularisation");
            return SK_ERR_NUMERICAL;
        case kNotConverged:
            set_error("sk_kkt_solve_noalloc: residual " + std::to_string(h[1]) + " above tolerance");
            return SK_ERR_NUMERICAL;
        default:
            set_error("sk_kkt_solve_noalloc: kernel did not report a status");
            return SK_ERR_INTERNAL;
    }
}
