// Crossover: Megiddo basis purification from an interior point to a basis, on the
// device. Follows the decisions of the reference's generate_crossover_basis
// (src/ipm/crossover.cu:322-460; purify_step_kernel :53-290, purify_bound_step_kernel
// :292-320), with its own data layout:
//
//  * the basis inverse is kept explicitly, dense and column-major in HBM (m x m
//    FP64), instead of an LU factor plus an eta file. B^-1 A_q is then a gather of
//    nnz(A_q) columns (one coalesced pass over m rows), and a basis change is one
//    rank-1 update of B^-1 (every column owned by one thread block, coalesced);
//  * the per-step decisions (largest artificial entry, the two ratio tests) are
//    single-block reductions that keep the reference's first-index tie rule, and the
//    host reads back one small status word per step;
//  * artificial columns n..n+m-1 start as the basis (B = I), as in the reference.
//
// Decisions kept from the reference: a column q is processed while it is not basic
// and lies more than 1e-6 inside its bounds; it first replaces the artificial of the
// row with the largest |(B^-1 A_q)_i| > 1e-7; otherwise x_q moves (increasing first)
// until q or a basic variable reaches a bound (|v_i| > 1e-9 in the ratio test), and a
// basic variable that reaches its bound leaves if its pivot exceeds 1e-7. The update
// of x after such a move runs over the basis after the exchange, as the reference's
// does (:253-260): the entering column's row adds -theta d_p to x_q and the leaving
// variable keeps its value. A second pass offers every non-basic column to the
// remaining artificial rows. An artificial left in the basis is rank deficiency.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cuda/crossover.hpp"

namespace sankhya {
namespace dev {

namespace {

constexpr double kAtBound = 1e-6;     // crossover.cu:68-70, 446
constexpr double kPivotTol = 1e-7;    // crossover.cu:100-109, 200, 205, 213, 218
constexpr double kDirTol = 1e-9;      // crossover.cu:165, 170
constexpr double kNoBound = 1e30;     // crossover.cu:137-140
constexpr int kDecideThreads = 1024;

#define XO_CUDA(call)                                                                             \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            throw std::runtime_error(std::string("crossover: ") + cudaGetErrorString(e_));       \
    } while (0)

// Step status written by the decision kernels and read by the host.
struct StepState {
    int pivoted;       // the step changed the basis or moved x_q
    int error;         // no admissible move (the reference's "invalid pivot")
    int update_row;    // row of B^-1 to pivot on, -1 = none
    int pad;
    double theta;
};

// d = B^-1 A_q: d_i = sum_k a_k Binv[i, r_k] (Binv column-major).
__global__ void k_ftran(int m, const double* __restrict__ Binv, const int* __restrict__ cp,
                        const int* __restrict__ ri, const double* __restrict__ v, int q, double* __restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    double s = 0.0;
    for (int k = cp[q]; k < cp[q + 1]; ++k) s += v[k] * Binv[static_cast<int64_t>(ri[k]) * m + i];
    d[i] = s;
}

// Pair reductions with the reference's tie rule (its loops run over rows in
// increasing order and replace only on a strict improvement: the first row wins).
struct MinPair { double v; int idx; };
__device__ __forceinline__ MinPair min_first(MinPair a, MinPair b) {
    if (b.v < a.v || (b.v == a.v && b.idx < a.idx)) return b;
    return a;
}
struct MaxPair { double v; int idx; };
__device__ __forceinline__ MaxPair max_first(MaxPair a, MaxPair b) {
    if (b.v > a.v || (b.v == a.v && b.idx >= 0 && (a.idx < 0 || b.idx < a.idx))) return b;
    return a;
}

template <class P, class F>
__device__ P block_reduce(P x, F op, P* sh) {
    const int t = threadIdx.x;
    sh[t] = x;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] = op(sh[t], sh[t + s]);
        __syncthreads();
    }
    P r = sh[0];
    __syncthreads();
    return r;
}

// Row of the largest |d_i| > kPivotTol among rows whose basic column is artificial.
__device__ int best_artificial_row(int m, int n, const int* basis, const double* d, MaxPair* sh) {
    MaxPair b{kPivotTol, -1};
    for (int i = threadIdx.x; i < m; i += blockDim.x)
        if (basis[i] >= n) {
            const double a = fabs(d[i]);
            if (a > b.v) b = MaxPair{a, i};
        }
    b = block_reduce(b, [](MaxPair x, MaxPair y) { return max_first(x, y); }, sh);
    return b.v > kPivotTol ? b.idx : -1;
}

// One purification step of column q (the reference's purify_step_kernel).
__global__ void __launch_bounds__(kDecideThreads) k_purify_decide(
    int m, int n, int q, const double* __restrict__ lb, const double* __restrict__ ub, double* __restrict__ x,
    int* __restrict__ basis, int* __restrict__ is_basic, const double* __restrict__ d, StepState* st) {
    __shared__ MaxPair shx[kDecideThreads];
    __shared__ MinPair shn[kDecideThreads];
    __shared__ int skip;
    const int t = threadIdx.x;
    if (t == 0) {
        st->pivoted = 0;
        st->update_row = -1;
        st->theta = 0.0;
        const double l = lb ? lb[q] : 0.0, u = ub ? ub[q] : INFINITY;
        skip = (x[q] <= l + kAtBound || x[q] >= u - kAtBound || is_basic[q]) ? 1 : 0;
    }
    __syncthreads();
    if (skip) return;
    // 1. an artificial row to replace
    const int art = best_artificial_row(m, n, basis, d, shx);
    if (art >= 0) {
        if (t == 0) {
            basis[art] = q;
            is_basic[q] = 1;
            st->update_row = art;
            st->pivoted = 1;
        }
        return;
    }
    // 2. ratio tests in both directions, seeded with q's own bound distances (q wins ties)
    const double lq = lb ? lb[q] : 0.0, uq = ub ? ub[q] : INFINITY;
    MinPair pos{kNoBound, -1}, neg{kNoBound, -1};   // idx: -2 = q itself, else the row
    if (uq - x[q] < kNoBound) pos = MinPair{uq - x[q], -2};
    if (x[q] - lq < kNoBound) neg = MinPair{x[q] - lq, -2};
    MinPair tp{kNoBound, 0x7fffffff}, tn{kNoBound, 0x7fffffff};
    for (int i = t; i < m; i += blockDim.x) {
        const int bv = basis[i];
        if (bv >= n) continue;
        const double vi = -d[i];
        const double l = lb ? lb[bv] : 0.0, u = ub ? ub[bv] : INFINITY;
        const double dub = u - x[bv], dlb = x[bv] - l;
        if (vi > kDirTol) {
            tp = min_first(tp, MinPair{dub / vi, i});
            tn = min_first(tn, MinPair{dlb / vi, i});
        } else if (vi < -kDirTol) {
            tp = min_first(tp, MinPair{dlb / (-vi), i});
            tn = min_first(tn, MinPair{dub / (-vi), i});
        }
    }
    tp = block_reduce(tp, [](MinPair a, MinPair b) { return min_first(a, b); }, shn);
    tn = block_reduce(tn, [](MinPair a, MinPair b) { return min_first(a, b); }, shn);
    if (t == 0) {
        if (tp.v < pos.v) pos = tp;   // a basic row must be strictly closer than q's own bound
        if (tn.v < neg.v) neg = tn;
        const int row1 = (pos.idx >= 0 && fabs(d[pos.idx]) > kPivotTol) ? pos.idx : -1;
        const int row2 = (neg.idx >= 0 && fabs(d[neg.idx]) > kPivotTol) ? neg.idx : -1;
        int row = -1;
        double theta = 0.0;
        bool ok = true;
        if (row1 >= 0) { row = row1; theta = pos.v; }
        else if (row2 >= 0) { row = row2; theta = -neg.v; }
        else if (pos.idx == -2) theta = pos.v;
        else if (neg.idx == -2) theta = -neg.v;
        else ok = false;
        if (!ok) {
            st->error = 1;
        } else {
            if (row >= 0) {
                is_basic[basis[row]] = 0;
                basis[row] = q;
                is_basic[q] = 1;
                st->update_row = row;
            }
            st->theta = theta;
            st->pivoted = 1;
            x[q] += theta;
        }
    }
    __syncthreads();
    if (st->pivoted == 0) return;
    // x_B moves by -theta d over the basis after the exchange (see the file comment)
    const double theta = st->theta;
    for (int i = t; i < m; i += blockDim.x) {
        const int bv = basis[i];
        if (bv < n && bv != q) x[bv] += theta * (-d[i]);
    }
    __syncthreads();
    if (t == 0 && st->update_row >= 0) x[q] += theta * (-d[st->update_row]);
}

// The second pass: a non-basic column q replaces the artificial of the row with the
// largest |d_i| > 1e-7 (the reference's purify_bound_step_kernel).
__global__ void __launch_bounds__(kDecideThreads) k_bound_decide(int m, int n, int q, int* __restrict__ basis,
                                                                 int* __restrict__ is_basic,
                                                                 const double* __restrict__ d, StepState* st) {
    __shared__ MaxPair shx[kDecideThreads];
    if (threadIdx.x == 0) st->update_row = -1;
    if (is_basic[q]) return;
    const int art = best_artificial_row(m, n, basis, d, shx);
    if (threadIdx.x == 0 && art >= 0) {
        basis[art] = q;
        is_basic[q] = 1;
        st->update_row = art;
    }
}

// B^-1 <- E B^-1 for a basis change in row p with entering column d = B^-1 A_q:
// row p is divided by d_p, every other row i loses d_i times the new row p. Column j
// of B^-1 is owned by block j.
__global__ void k_inverse_update(int m, double* __restrict__ Binv, const double* __restrict__ d,
                                 const StepState* __restrict__ st) {
    const int p = st->update_row;
    if (p < 0) return;
    const int j = blockIdx.x;
    double* col = Binv + static_cast<int64_t>(j) * m;
    __shared__ double rp;
    if (threadIdx.x == 0) rp = col[p] / d[p];
    __syncthreads();
    const double r = rp;
    for (int i = threadIdx.x; i < m; i += blockDim.x) col[i] = (i == p) ? r : col[i] - d[i] * r;
}

__global__ void k_identity(int m, double* __restrict__ Binv) {
    const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = static_cast<int64_t>(m) * m;
    for (int64_t e = k; e < total; e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        Binv[e] = (e % (m + 1) == 0) ? 1.0 : 0.0;
}

__global__ void k_init_basis(int m, int n, int* __restrict__ basis, int* __restrict__ is_basic) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) basis[i] = n + i;
    if (i < n) is_basic[i] = 0;
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    explicit DevBuf(size_t count) { XO_CUDA(cudaMalloc(&p, sizeof(T) * (count ? count : 1))); }
    ~DevBuf() { if (p) cudaFree(p); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
};

}  // namespace

int crossover(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, const double* lb,
              const double* ub, const double* x_ipm, int* basic, int* status, double* x_out, std::string* message) {
    if (m <= 0 || n <= 0 || !col_ptrs || !row_idx || !vals || !x_ipm || !basic || !status)
        throw std::invalid_argument("crossover: invalid arguments");
    if (m > kCrossoverMaxRows) return kCrossoverTooLarge;
    const int nnz = col_ptrs[n];
    for (int j = 0; j < n; ++j)
        if (col_ptrs[j + 1] < col_ptrs[j]) throw std::invalid_argument("crossover: column pointers decrease");
    for (int k = 0; k < nnz; ++k)
        if (row_idx[k] < 0 || row_idx[k] >= m) throw std::invalid_argument("crossover: row index out of range");
    cudaStream_t s;
    XO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{s};
    DevBuf<int> dcp(static_cast<size_t>(n) + 1), dri(nnz), dbasis(m), disb(n);
    DevBuf<double> dv(nnz), dlb(lb ? n : 0), dub(ub ? n : 0), dx(n), dd(m);
    DevBuf<double> binv(static_cast<size_t>(m) * m);
    DevBuf<StepState> dst(1);
    StepState* hst = nullptr;
    XO_CUDA(cudaMallocHost(&hst, sizeof(StepState)));
    struct HostGuard { StepState* p; ~HostGuard() { cudaFreeHost(p); } } hguard{hst};
    XO_CUDA(cudaMemcpyAsync(dcp.p, col_ptrs, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    XO_CUDA(cudaMemcpyAsync(dri.p, row_idx, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    XO_CUDA(cudaMemcpyAsync(dv.p, vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    if (lb) XO_CUDA(cudaMemcpyAsync(dlb.p, lb, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    if (ub) XO_CUDA(cudaMemcpyAsync(dub.p, ub, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    XO_CUDA(cudaMemcpyAsync(dx.p, x_ipm, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    XO_CUDA(cudaMemsetAsync(dst.p, 0, sizeof(StepState), s));
    k_identity<<<1216, 256, 0, s>>>(m, binv.p);
    k_init_basis<<<(std::max(m, n) + 255) / 256, 256, 0, s>>>(m, n, dbasis.p, disb.p);
    XO_CUDA(cudaGetLastError());
    const double* plb = lb ? dlb.p : nullptr;
    const double* pub = ub ? dub.p : nullptr;
    const int fgrid = (m + 255) / 256;
    bool failed = false;
    // pass 1: purification (a column is revisited while its step changes something)
    for (int q = 0; q < n && !failed; ++q) {
        for (int guard_steps = 0; guard_steps <= m + 1; ++guard_steps) {
            k_ftran<<<fgrid, 256, 0, s>>>(m, binv.p, dcp.p, dri.p, dv.p, q, dd.p);
            k_purify_decide<<<1, kDecideThreads, 0, s>>>(m, n, q, plb, pub, dx.p, dbasis.p, disb.p, dd.p, dst.p);
            k_inverse_update<<<m, 256, 0, s>>>(m, binv.p, dd.p, dst.p);
            XO_CUDA(cudaMemcpyAsync(hst, dst.p, sizeof(StepState), cudaMemcpyDeviceToHost, s));
            XO_CUDA(cudaStreamSynchronize(s));
            if (hst->error) { failed = true; break; }
            if (!hst->pivoted) break;
        }
    }
    // pass 2: non-basic columns fill the rows whose artificial is still basic
    if (!failed) {
        for (int q = 0; q < n; ++q) {
            k_ftran<<<fgrid, 256, 0, s>>>(m, binv.p, dcp.p, dri.p, dv.p, q, dd.p);
            k_bound_decide<<<1, kDecideThreads, 0, s>>>(m, n, q, dbasis.p, disb.p, dd.p, dst.p);
            k_inverse_update<<<m, 256, 0, s>>>(m, binv.p, dd.p, dst.p);
        }
        XO_CUDA(cudaGetLastError());
    }
    std::vector<double> hx(static_cast<size_t>(n));
    XO_CUDA(cudaMemcpyAsync(basic, dbasis.p, sizeof(int) * m, cudaMemcpyDeviceToHost, s));
    XO_CUDA(cudaMemcpyAsync(hx.data(), dx.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    XO_CUDA(cudaStreamSynchronize(s));
    // statuses as the reference assigns them (crossover.cu:433-449)
    bool deficient = false;
    for (int j = 0; j < n; ++j) status[j] = kAtLower;
    for (int i = 0; i < m; ++i) {
        if (basic[i] < n) status[basic[i]] = kBasic;
        else deficient = true;
    }
    for (int j = 0; j < n; ++j)
        if (status[j] != kBasic) {
            const double u = ub ? ub[j] : INFINITY;
            if (std::fabs(hx[j] - u) < kAtBound) status[j] = kAtUpper;
        }
    if (x_out) std::memcpy(x_out, hx.data(), sizeof(double) * n);
    if (failed) {
        if (message) *message = "Crossover failed: Invalid pivot encountered";
        return kCrossoverInvalidPivot;
    }
    if (deficient) {
        if (message) *message = "Crossover failed: Matrix is rank deficient";
        return kCrossoverRankDeficient;
    }
    return 0;
}

}  // namespace dev
}  // namespace sankhya
