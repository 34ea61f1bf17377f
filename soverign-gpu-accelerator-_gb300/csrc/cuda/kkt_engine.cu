// Device normal-equation engine (see kkt_engine.hpp).
//
// Kernels, in the order one factorisation + solve runs them:
//   assembly    k_asm_*          D (A Theta A^T) D + delta I into the fronts
//   factor      k_potrf          Cholesky of one 64x64 diagonal tile per front
//               k_trsm           panel rows below the tile: X L^T = B
//               k_update         trailing update C -= L_i L_j^T (tiles of 64x64)
//               k_extend_add     child update matrix into the parent front
//   solve       k_fwd_gather     frontal right-hand sides of one level
//               k_fwd_tasks      L z = r, dependency-driven 64-row block tasks
//               k_bwd_tasks      L^T x = z, same scheme in reverse
// Factorisation grids are lists of (front, tile) work items of one level / step,
// decoded with a binary search over a prefix of per-front tile counts.
#include "cuda/kkt_engine.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <type_traits>

namespace sankhya {
namespace dev {

struct PlanDev {
    const int* sn_first;
    const int* sn_ncols;
    const int* sn_nrows;
    const int* sn_lda;
    const int64_t* F_off;
    const int64_t* f_off;
    const int64_t* rows_off;
    const int* rows;
    const int64_t* ea_off;
    const int* ea_map;
    const int* ch_ptr;
    const int* ch_list;
    const int* sn_parent;
    const int* sn_lp;      // LP of each front (fronts never span LPs)
    const int* lp_on;      // 1 while an LP of the batch is still being solved; 0 skips its fronts
    int* lp_fail;          // per LP: set to 1 when one of its pivots was not positive
};

namespace {

constexpr int T64 = ipm::kTile;   // 64
constexpr int LDS = T64 + 1;      // padded leading dimension of shared tiles

struct StepArgs {
    int k;
    int item_off;
    int nitems;
    int tp_off;   // trsm prefix offset
    int up_off;   // update prefix offset (64x64 tiles)
    int up2_off;  // update prefix offset (128x128 blocks, tensor-core path)
    int up3_off;  // update prefix offset (128x64 blocks, emulated FP64 path)
    int dr_off;   // digit-row offsets of the items (emulated FP64 path)
};


// Largest i in [0, n) with prefix[i] <= b (prefix ascending, prefix[0] = 0 <= b). The
// whole warp searches (every lane must call it, converged, with the same arguments):
// each round probes 32 evenly spaced entries and keeps the segment after the last
// one <= b, so n <= 32 takes one dependent load and n <= 1024 two, where a binary
// search takes log2(n) (this sits at the head of every tile of a factorisation step).
__device__ __forceinline__ int find_item(const int* prefix, int n, int b) {
    const int lane = threadIdx.x & 31;
    int lo = 0, len = n;      // the answer lies in [lo, lo + len)
    while (len > 1) {
        const int step = (len + 31) >> 5;
        const int idx = lo + lane * step;
        const bool le = idx < lo + len && prefix[idx] <= b;
        const unsigned m = __ballot_sync(0xffffffffu, le);   // lane 0 probes lo: always set
        const int nlo = lo + (31 - __clz(m)) * step;
        len = min(step, lo + len - nlo);
        lo = nlo;
    }
    return lo;
}

__device__ __forceinline__ void tri_index(int lt, int& ti, int& tj) {
    int t = static_cast<int>((sqrtf(8.0f * static_cast<float>(lt) + 1.0f) - 1.0f) * 0.5f);
    while ((t + 1) * (t + 2) / 2 <= lt) ++t;
    while (t > 0 && t * (t + 1) / 2 > lt) --t;
    ti = t;
    tj = lt - t * (t + 1) / 2;
}

// ------------------------------------------------------------------ assembly

// Diagonal of A Theta A^T and the equilibration D = 1/sqrt(max(|m_ii|, 1e-12))
// (reference src/cuda/kkt.cu:65-94). Row i of W holds a_ik^2 for the entries of
// row i of A, so the rows have A's row lengths: G lanes share a row, G being the
// width the SpMV autotuner chose for A.
template <int G>
__global__ void __launch_bounds__(256) k_asm_diag_sparse(int M, const int64_t* __restrict__ w_ptr,
                                                         const int* __restrict__ w_col,
                                                         const double* __restrict__ w_val,
                                                         const double* __restrict__ theta,
                                                         double* __restrict__ Mdiag, double* __restrict__ D) {
    const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int i = static_cast<int>(gid / G), lane = static_cast<int>(gid % G);
    const bool valid = i < M;
    double acc = 0.0;
    if (valid) {
        int64_t t = w_ptr[i] + lane;
        const int64_t t1 = w_ptr[i + 1];
        for (; t + 3 * G < t1; t += 4 * G) {   // four entries' loads in flight; same summation order
            const int c0 = w_col[t], c1 = w_col[t + G], c2 = w_col[t + 2 * G], c3 = w_col[t + 3 * G];
            const double v0 = w_val[t], v1 = w_val[t + G], v2 = w_val[t + 2 * G], v3 = w_val[t + 3 * G];
            const double h0 = theta[c0], h1 = theta[c1], h2 = theta[c2], h3 = theta[c3];
            acc += v0 * h0;
            acc += v1 * h1;
            acc += v2 * h2;
            acc += v3 * h3;
        }
        for (; t < t1; t += G) acc += w_val[t] * theta[w_col[t]];
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
    if (valid && lane == 0) {
        Mdiag[i] = acc;
        D[i] = 1.0 / sqrt(fmax(fabs(acc), 1e-12));
    }
}

// Slots of LPs whose fronts are not being factored (lp_on 0) are left alone.
template <class T>
__global__ void k_asm_slots_sparse(int64_t nslots, int M, const int64_t* __restrict__ w_ptr,
                                   const int* __restrict__ w_col, const double* __restrict__ w_val,
                                   const double* __restrict__ theta, const int* __restrict__ si,
                                   const int* __restrict__ sj, const int64_t* __restrict__ pos,
                                   const double* __restrict__ Mdiag, const double* __restrict__ D,
                                   const double* __restrict__ params, const int* __restrict__ q_lp,
                                   const int* __restrict__ lp_on, T* __restrict__ F) {
    const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    // every load that depends only on s first, then the ones they index, so a slot
    // waits for three rounds of loads rather than one per link of the chain
    const bool diag = s < M;
    const int i = diag ? static_cast<int>(s) : si[s];
    const int j = diag ? static_cast<int>(s) : sj[s];
    const int64_t p = pos[s];
    const int64_t t0 = diag ? 0 : w_ptr[s], t1 = diag ? 0 : w_ptr[s + 1];
    const double di = D[i], dj = D[j];
    const int on = lp_on[q_lp[i]];
    double acc = 0.0;
    for (int64_t t = t0; t < t1; ++t) acc += w_val[t] * theta[w_col[t]];
    if (!on) return;
    const double v = diag ? Mdiag[s] * di * di + params[0] : acc * di * dj;
    F[p] = static_cast<T>(v);
}

template <int G>
__global__ void __launch_bounds__(256) k_asm_diag_dense(int M, const int* __restrict__ rp, const int* __restrict__ ci,
                                                        const double* __restrict__ av,
                                                        const double* __restrict__ theta,
                                                        double* __restrict__ Mdiag, double* __restrict__ D) {
    const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int i = static_cast<int>(gid / G), lane = static_cast<int>(gid % G);
    const bool valid = i < M;
    double acc = 0.0;
    if (valid)
        for (int q = rp[i] + lane; q < rp[i + 1]; q += G) acc += av[q] * av[q] * theta[ci[q]];
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, G);
    if (valid && lane == 0) {
        Mdiag[i] = acc;
        D[i] = 1.0 / sqrt(fmax(fabs(acc), 1e-12));
    }
}

// Launches a diagonal kernel K<G> with G lanes per row (2, 4, 8, 16; else 32).
template <template <int> class K, class... Args>
void launch_diag(int M, int group, cudaStream_t st, Args... args) {
    if (M <= 0) return;
    const int64_t threads = static_cast<int64_t>(M) * group;
    const int blocks = static_cast<int>((threads + 255) / 256);
    switch (group) {
    case 2: K<2>::launch(blocks, st, M, args...); break;
    case 4: K<4>::launch(blocks, st, M, args...); break;
    case 8: K<8>::launch(blocks, st, M, args...); break;
    case 16: K<16>::launch(blocks, st, M, args...); break;
    default: K<32>::launch(blocks, st, M, args...); break;
    }
}
template <int G>
struct DiagSparse {
    template <class... A>
    static void launch(int blocks, cudaStream_t st, A... a) { k_asm_diag_sparse<G><<<blocks, 256, 0, st>>>(a...); }
};
template <int G>
struct DiagDense {
    template <class... A>
    static void launch(int blocks, cudaStream_t st, A... a) { k_asm_diag_dense<G><<<blocks, 256, 0, st>>>(a...); }
};

// One warp per column j of M (dense mode: one front per LP, natural order).
// Column j below the diagonal is sum_k a_jk theta_k A(:,k); the k loop is
// sequential so every entry is summed in a fixed order. The column ranges and
// coefficients of 32 k at a time are loaded by the lanes together and broadcast,
// and the rows, values and D of the next k are loaded before the current k's
// read-modify-write, so the loop carries one dependent memory round trip per k
// (the update of the front column) instead of four.
template <class T>
__global__ void k_asm_cols_dense(int M, const int* __restrict__ rp, const int* __restrict__ ci,
                                 const double* __restrict__ av, const int* __restrict__ tp,
                                 const int* __restrict__ ti, const double* __restrict__ tv,
                                 const double* __restrict__ theta, const double* __restrict__ Mdiag,
                                 const double* __restrict__ D, const int* __restrict__ row_lp, PlanDev pd,
                                 const double* __restrict__ params, T* __restrict__ F) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= M) return;
    const int j = warp;
    const int s = row_lp[j];
    if (!pd.lp_on[s]) return;            // dense mode: front s is LP s
    const int first = pd.sn_first[s];
    T* col = F + pd.F_off[s] + static_cast<int64_t>(j - first) * pd.sn_lda[s] - first;
    const double dj = D[j];
    const int q0 = rp[j], q1 = rp[j + 1];
    for (int qb = q0; qb < q1; qb += 32) {
        int ts = 0, te = 0;
        double cf = 0.0;
        if (qb + lane < q1) {
            const int k = ci[qb + lane];
            ts = tp[k];
            te = tp[k + 1];
            cf = av[qb + lane] * theta[k] * dj;
        }
        const int nq = min(32, q1 - qb);
        // first chunk (32 rows) of k = qb: loaded ahead
        int s0 = __shfl_sync(0xffffffffu, ts, 0), e0 = __shfl_sync(0xffffffffu, te, 0);
        int i0 = -1;
        double v0 = 0.0, d0 = 0.0;
        if (s0 + lane < e0) {
            i0 = ti[s0 + lane];
            v0 = tv[s0 + lane];
            d0 = D[i0];
        }
        for (int u = 0; u < nq; ++u) {              // nq is the same for every lane
            const double coef = __shfl_sync(0xffffffffu, cf, u);
            const int s1 = s0, e1 = e0, i1 = i0;
            const double v1 = v0, d1 = d0;
            if (u + 1 < nq) {                        // next k's first chunk
                s0 = __shfl_sync(0xffffffffu, ts, u + 1);
                e0 = __shfl_sync(0xffffffffu, te, u + 1);
                i0 = -1;
                if (s0 + lane < e0) {
                    i0 = ti[s0 + lane];
                    v0 = tv[s0 + lane];
                    d0 = D[i0];
                }
            }
            if (i1 > j) col[i1] = static_cast<T>(static_cast<double>(col[i1]) + coef * v1 * d1);
            for (int t = s1 + 32 + lane; t < e1; t += 32) {   // columns longer than 32 rows
                const int i = ti[t];
                if (i > j) col[i] = static_cast<T>(static_cast<double>(col[i]) + coef * tv[t] * D[i]);
            }
            __syncwarp();
        }
    }
    if (lane == 0) col[j] = static_cast<T>(Mdiag[j] * dj * dj + params[0]);
}

// ------------------------------------------------------------------- factor

// Cholesky of the 64x64 diagonal tile of step k of one front, in the front's
// precision T, plus the explicit inverse of the factored tile (used by the panel
// solve and by both triangular solves), stored column-major in Linv.
// Blocked by 16 columns so that the block-wide barriers are few: warp 0 factors
// each 16x16 diagonal block (warp-synchronous), one thread per row solves the
// panel below it, and all threads apply the trailing update. The inverse: four
// warps invert the four diagonal blocks, then block rows of L^{-1} follow as
// X_ij = -X_ii (sum_k L_ik X_kj). A partial tile is padded with the identity.
template <class T>
__device__ __noinline__ void potrf_tile(int s, int kstep, PlanDev pd, T* F, T* __restrict__ Linv,
                           const int64_t* __restrict__ inv_off, int* err, unsigned char* smraw) {
    constexpr int B = 16;
    T* A = reinterpret_cast<T*>(smraw);   // A[r * LDS + c], lower triangle
    T* X = A + T64 * LDS;                 // L^{-1}, same layout
    T* rdiag = X + T64 * LDS;             // 1 / L(c, c)
    const int K = pd.sn_ncols[s];
    const int LD = pd.sn_lda[s];
    const int k0 = kstep * T64;
    const int w = min(T64, K - k0);
    T* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
#pragma unroll 4
    for (int it = 0; it < 16; ++it) {
        const int idx = tid + it * 256;
        const int r = idx & 63, c = idx >> 6;
        T x = T(0);
        if (r < w && c < w && c <= r) x = Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * LD];
        else if (r == c) x = T(1);
        A[r * LDS + c] = x;
        X[r * LDS + c] = T(0);
    }
    __syncthreads();
    for (int c0 = 0; c0 < T64; c0 += B) {
        if (wid == 0) {            // 16x16 diagonal block, lanes 0..15 own its rows
            const int rr = c0 + (lane & 15);
            for (int jj = 0; jj < B; ++jj) {
                const int c = c0 + jj;
                if (lane == 0) {
                    T p = A[c * LDS + c];
                    if (!(p > T(0))) {
                        if (atomicCAS(err, 0, 1) == 0) err[1] = s;
                        pd.lp_fail[pd.sn_lp[s]] = 1;
                        p = T(1);
                    }
                    const T d = sqrt(p);
                    A[c * LDS + c] = d;
                    rdiag[c] = T(1) / d;
                }
                __syncwarp();
                if (lane < B && rr > c) A[rr * LDS + c] *= rdiag[c];
                __syncwarp();
                if (rr > c) {
                    const T l = A[rr * LDS + c];
                    for (int cc = c + 1 + (lane >> 4); cc <= rr; cc += 2) A[rr * LDS + cc] -= l * A[cc * LDS + c];
                }
                __syncwarp();
            }
        }
        __syncthreads();
        const int t0 = c0 + B, nt = T64 - t0;
        if (tid < nt) {            // panel row r: X L_kk^T = A_r
            const int r = t0 + tid;
            T x[B];
#pragma unroll
            for (int jj = 0; jj < B; ++jj) {
                T v = A[r * LDS + c0 + jj];
#pragma unroll
                for (int q = 0; q < jj; ++q) v -= x[q] * A[(c0 + jj) * LDS + c0 + q];
                x[jj] = v * rdiag[c0 + jj];
            }
#pragma unroll
            for (int jj = 0; jj < B; ++jj) A[r * LDS + c0 + jj] = x[jj];
        }
        __syncthreads();
        for (int e = tid; e < nt * nt; e += 256) {   // trailing lower triangle
            const int r = t0 + e / nt, cc = t0 + e % nt;
            if (cc > r) continue;
            T v = A[r * LDS + cc];
#pragma unroll
            for (int q = 0; q < B; ++q) v -= A[r * LDS + c0 + q] * A[cc * LDS + c0 + q];
            A[r * LDS + cc] = v;
        }
        __syncthreads();
    }
#pragma unroll 4
    for (int it = 0; it < 16; ++it) {
        const int idx = tid + it * 256;
        const int r = idx & 63, c = idx >> 6;
        if (r < w && c < w && c <= r) Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * LD] = A[r * LDS + c];
    }
    // inverse of the diagonal blocks: warp b, lane = column of block b
    if (wid < T64 / B && lane < B) {
        const int c0 = wid * B, j = c0 + lane;
        for (int i = j; i < c0 + B; ++i) {
            T acc = (i == j) ? T(1) : T(0);
            for (int q = j; q < i; ++q) acc -= A[i * LDS + q] * X[q * LDS + j];
            X[i * LDS + j] = acc * rdiag[i];
        }
    }
    __syncthreads();
    // block rows 1..3: T_ij = sum_{q < r0} L(i, q) X(q, j), then X_ij = -X_ii T_ij
    for (int r0 = B; r0 < T64; r0 += B) {
        const int cnt = r0 * B;            // (r0 / B) blocks of 16x16
        for (int e = tid; e < cnt; e += 256) {
            const int i = r0 + (e % (B * B)) / B, j = (e / (B * B)) * B + e % B;
            T acc = T(0);
            for (int q = (e / (B * B)) * B; q < r0; ++q) acc += A[i * LDS + q] * X[q * LDS + j];
            X[i * LDS + j] = acc;
        }
        __syncthreads();
        T out[3];
#pragma unroll
        for (int u = 0; u < 3; ++u) {
            const int e = tid + u * 256;
            out[u] = T(0);
            if (e < cnt) {
                const int rr = (e % (B * B)) / B, i = r0 + rr, j = (e / (B * B)) * B + e % B;
                T acc = T(0);
                for (int q = 0; q <= rr; ++q) acc += X[i * LDS + r0 + q] * X[(r0 + q) * LDS + j];
                out[u] = -acc;
            }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 3; ++u) {
            const int e = tid + u * 256;
            if (e < cnt) {
                const int i = r0 + (e % (B * B)) / B, j = (e / (B * B)) * B + e % B;
                X[i * LDS + j] = out[u];
            }
        }
        __syncthreads();
    }
    T* Li = Linv + inv_off[s] + static_cast<int64_t>(kstep) * T64 * T64;
#pragma unroll 4
    for (int it = 0; it < 16; ++it) {
        const int idx = tid + it * 256;
        const int i = idx & 63, jj = idx >> 6;
        Li[i + jj * T64] = (i < w && jj < w) ? X[i * LDS + jj] : T(0);
    }
}

constexpr size_t potrf_smem(size_t elem) { return (2 * T64 * LDS + 2 * T64) * elem; }

// Diagonal-tile Cholesky of the first step of each front of a level (later steps
// are factored at the end of the previous step's update, see k_update).
template <class T>
__global__ void __launch_bounds__(256) k_potrf(StepArgs a, const int* __restrict__ items, PlanDev pd, T* F,
                                               T* __restrict__ Linv, const int64_t* __restrict__ inv_off,
                                               int* err) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int s = items[a.item_off + blockIdx.x];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    potrf_tile<T>(s, a.k, pd, F, Linv, inv_off, err, smraw);
}

// Panel rows below the diagonal tile: X = B L_kk^{-T} = B Linv^T (a small GEMM).
template <class T>
__global__ void __launch_bounds__(256) k_trsm(StepArgs a, const int* __restrict__ items,
                                              const int* __restrict__ prefix, PlanDev pd, T* F,
                                              const T* __restrict__ Linv, const int64_t* __restrict__ inv_off) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* Iv = reinterpret_cast<T*>(smraw);    // Linv column-major [q + c*64]
    T* B = Iv + T64 * T64;                   // B[c][r] (column-major)
    const int i = find_item(prefix + a.tp_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int r0 = k0 + w + lt * T64;
    const int nr = min(T64, N - r0);
    T* Fs = F + pd.F_off[s];
    const T* Li = Linv + inv_off[s] + static_cast<int64_t>(a.k) * T64 * T64;
    const int tid = threadIdx.x;
    for (int idx = tid; idx < T64 * T64; idx += blockDim.x) Iv[idx] = Li[idx];
    for (int idx = tid; idx < T64 * T64; idx += blockDim.x) {
        const int r = idx & 63, c = idx >> 6;
        B[c * T64 + r] = (r < nr && c < w) ? Fs[(r0 + r) + static_cast<int64_t>(k0 + c) * LD] : T(0);
    }
    __syncthreads();
    // X[r][c] = sum_{q <= c} B[r][q] Linv[c][q]; thread: row r, 16 columns
    const int r = tid & 63, cg = tid >> 6;
    T acc[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) acc[t] = T(0);
    for (int q = 0; q < w; ++q) {
        const T bq = B[q * T64 + r];
#pragma unroll
        for (int t = 0; t < 16; ++t) acc[t] += bq * Iv[(cg * 16 + t) + q * T64];   // Linv[c][q], 0 when q > c
    }
    if (r < nr)
#pragma unroll
        for (int t = 0; t < 16; ++t) {
            const int c = cg * 16 + t;
            if (c < w) Fs[(r0 + r) + static_cast<int64_t>(k0 + c) * LD] = acc[t];
        }
}

// C(64x64) -= A_i (64 x w) A_j^T; 256 threads, 4x4 outputs each. The C tile is
// read into registers and both panel tiles are staged with fully unrolled loads
// before any arithmetic, so every global load of a thread is in flight at once.
template <class T>
__global__ void __launch_bounds__(256) k_update(StepArgs a, const int* __restrict__ items,
                                                const int* __restrict__ prefix, PlanDev pd, T* F,
                                                T* __restrict__ Linv, const int64_t* __restrict__ inv_off,
                                                int* err) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* As = reinterpret_cast<T*>(smraw);     // [kk][r]
    T* Bs = As + T64 * T64;                  // [kk][c]
    const int i = find_item(prefix + a.up_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int lt = blockIdx.x - prefix[a.up_off + i];
    int ti, tj;
    tri_index(lt, ti, tj);
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int t0 = k0 + w;
    const int ri0 = t0 + ti * T64, cj0 = t0 + tj * T64;
    const int nri = min(T64, N - ri0), ncj = min(T64, N - cj0);
    T* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    T cv[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = ty * 4 + q, c = tx * 4 + p;
            const bool in = r < nri && c < ncj && (ti != tj || r >= c);
            cv[q][p] = in ? Fs[(ri0 + r) + static_cast<int64_t>(cj0 + c) * LD] : T(0);
        }
    T va[16], vb[16];
#pragma unroll
    for (int it = 0; it < 16; ++it) {
        const int idx = tid + it * 256;
        const int r = idx & (T64 - 1), kk = idx >> 6;
        const int64_t cofs = static_cast<int64_t>(k0 + kk) * LD;
        va[it] = (kk < w && r < nri) ? Fs[ri0 + r + cofs] : T(0);
        vb[it] = (kk < w && r < ncj) ? Fs[cj0 + r + cofs] : T(0);
    }
#pragma unroll
    for (int it = 0; it < 16; ++it) {
        const int idx = tid + it * 256;
        As[idx] = va[it];
        Bs[idx] = vb[it];
    }
    __syncthreads();
    T acc[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[q][p] = T(0);
#pragma unroll 4
    for (int kk = 0; kk < w; ++kk) {
        T av[4], bv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) { av[q] = As[kk * T64 + ty * 4 + q]; bv[q] = Bs[kk * T64 + tx * 4 + q]; }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int p = 0; p < 4; ++p) acc[q][p] += av[q] * bv[p];
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = ty * 4 + q, c = tx * 4 + p;
            if (r < nri && c < ncj && (ti != tj || r >= c))
                Fs[(ri0 + r) + static_cast<int64_t>(cj0 + c) * LD] = cv[q][p] - acc[q][p];
        }
    // The block that finished the first trailing diagonal tile factors it right away
    // (step k + 1's diagonal tile), overlapping the rest of this step's update.
    if (lt == 0 && t0 < K) {
        __syncthreads();
        potrf_tile<T>(s, a.k + 1, pd, F, Linv, inv_off, err, smraw);
    }
}

// ---- shared helpers of the tensor-core kernels (tcgen05) --------------------
// Shared-memory descriptors of the canonical K-major no-swizzle layout: 8-row x
// 16-byte core matrices, K-adjacent core matrices 128 B apart, 8-row groups 2048 B
// apart (64 four-byte elements per row).
constexpr uint32_t kTcLbo = 128;                     // bytes between K-adjacent core matrices
constexpr uint32_t kTcSbo = 2048;                    // bytes between 8-row groups (64 fp32 per row)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr) {
    uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(kTcLbo >> 4) << 16;
    d |= static_cast<uint64_t>(kTcSbo >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;             // descriptor version bits 46-48 = 0b001
    return d;                                        // base offset 0, no swizzle
}
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// ---- emulated FP64 trailing update on the tensor cores (BF16 digits) --------
// FP64 fronts of the late iterations of a mixed-precision solve. Each trailing
// row of the step's panel (its 64 L entries a_k) is written as
//     a_k = sum_{i=0..6} d_ik 2^(E - 7 - 8 i),   E = floor(log2 max_k |a_k|),
// with balanced base-256 digits (d_0 in [-256, 256], d_i in [-128, 127] for
// i >= 1): 56 bits, the row to 2^-56 of its largest entry. Every digit is an
// integer of at most 8 significant bits, exact in BF16 (k_oz_digits, once per
// panel row). C -= A B^T is then the sum over digit pairs (i, j); the pairs of
// one level L = i + j share the scale 2^(E_a + E_b - 14 - 8 L) and accumulate in
// one FP32 TMEM accumulator. With K <= 64 each level sum is an integer below
// 9 * 2^20 in magnitude (|d_0 e_0| <= 2^16, |d_0 e_j| <= 2^15, |d_i e_j| <= 2^14,
// at most L + 1 pairs of 64 products), so the tensor cores add it exactly. Levels
// 0..6 (28 pairs; the pairs beyond level 6 weigh below 2^-56 and are left out)
// are combined in 64-bit integers, hi = levels 0..2 and lo = levels 3..6, folded
// into u = hi 2^22 + round(lo 2^-10) (below 2^62 in magnitude) and applied with
// one conversion and one FP64 FMA per entry: C - u 2^(Ea+Eb-52) (GB300's FP64 pipe
// is the scarce resource of this epilogue).
// This is the error-free splitting of Ozaki, Ogita, Oishi and Rump (2012) with
// BF16 digits, exact FP32 tensor-core sums and an integer epilogue; the result
// agrees with an FP64 product to about 2^-53 of sum_k |a_k| |b_k|.
//
// Digit layout (global and shared alike): per digit plane i, K half h = k >> 5, row q
// and column k at byte i * plane + h * (plane / 2) + (q >> 3) * 512 + ((k & 31) >> 3) * 128
// + (q & 7) * 16 + (k & 7) * 2: within one half the canonical K-major no-swizzle layout
// of 8-row x 16-byte core matrices, so a block's 128 (32, 64) consecutive rows of one
// plane and half are one contiguous 8 KB (2 KB, 4 KB) bulk copy, and a block streams
// the two K halves through one buffer.

constexpr int kOzDigits = 7;
constexpr uint32_t kOzLbo = 128;                       // bytes between K-adjacent core matrices
constexpr uint32_t kOzSbo = 512;                       // bytes between 8-row groups (32 bf16 per row and half)
constexpr size_t kOzA = 128 * 64;                      // 128 rows of one plane and half: 8 KB
constexpr size_t kOzBu = 32 * 64;                      // 32 rows (update tiles): 2 KB
constexpr size_t kOzBt = 64 * 64;                      // 64 rows (Linv rows of the panel solve): 4 KB
constexpr size_t kOzSmemU = kOzDigits * (kOzA + kOzBu) + 64;   // 70 KB: two blocks per SM
constexpr size_t kOzSmemT = kOzDigits * (kOzA + kOzBt) + 64;   // 84 KB
constexpr int kOzSpin = 1 << 22;
// instruction descriptors (kind::f16): D = F32 (bits 4-5 = 1), A = B = BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28 (M = 128; N = 64 or 32)
constexpr uint32_t kOzIdesc64 = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t kOzIdesc32 = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint64_t oz_sdesc(uint32_t saddr) {
    uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(kOzLbo >> 4) << 16;
    d |= static_cast<uint64_t>(kOzSbo >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}
__device__ __forceinline__ double oz_pow2(int p) {       // 2^p, 0 below the normal range
    if (p < -1022) return 0.0;
    return __longlong_as_double(static_cast<long long>(p + 1023) << 52);
}
__device__ __forceinline__ uint32_t oz_bf16(int d) {     // |d| <= 256: exact
    return __float_as_uint(static_cast<float>(d)) >> 16;
}
__device__ __forceinline__ bool oz_wait(uint32_t bar, uint32_t parity = 0) {
    uint32_t done = 0;
    for (int spin = 0; spin < kOzSpin && !done; ++spin) {
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n" : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        // back-to-back polls first: a copy or an MMA batch of one tile completes within
        // microseconds, and a sleep per poll adds its own latency to every tile
        if (!done && spin >= 4096) __nanosleep(32);
    }
    return done != 0;
}

// The 7 balanced base-256 digits of 16 entries v of row q (columns 16 cg .. 16 cg + 15)
// with row exponent E, as BF16 into the digit planes (layout above).
__device__ __forceinline__ void oz_store_digits(const double* v, int E, int q, int cg, unsigned char* dig,
                                                int64_t plane) {
    const double mul = oz_pow2(55 - E);             // |v mul| < 2^56
    uint32_t pk[kOzDigits][8];                      // 16 BF16 digits per plane, packed in pairs
#pragma unroll
    for (int t = 0; t < 16; t += 2) {
        int d0[kOzDigits], d1[kOzDigits];
        long long f0 = llrint(v[t] * mul), f1 = llrint(v[t + 1] * mul);
#pragma unroll
        for (int j = kOzDigits - 1; j >= 1; --j) {
            int l0 = static_cast<int>(f0 & 255), l1 = static_cast<int>(f1 & 255);
            f0 >>= 8;
            f1 >>= 8;
            if (l0 >= 128) { l0 -= 256; f0 += 1; }
            if (l1 >= 128) { l1 -= 256; f1 += 1; }
            d0[j] = l0;
            d1[j] = l1;
        }
        d0[0] = static_cast<int>(f0);
        d1[0] = static_cast<int>(f1);
#pragma unroll
        for (int j = 0; j < kOzDigits; ++j) pk[j][t >> 1] = oz_bf16(d0[j]) | (oz_bf16(d1[j]) << 16);
    }
    unsigned char* base = dig + (cg >> 1) * (plane >> 1) + static_cast<int64_t>(q >> 3) * kOzSbo + (q & 7) * 16;
#pragma unroll
    for (int j = 0; j < kOzDigits; ++j)
#pragma unroll
        for (int h = 0; h < 2; ++h)
            *reinterpret_cast<uint4*>(base + j * plane + ((cg & 1) * 2 + h) * kOzLbo) =
                make_uint4(pk[j][4 * h], pk[j][4 * h + 1], pk[j][4 * h + 2], pk[j][4 * h + 3]);
}

// Thread 0 of a digit-product block: start the bulk copies of K half h of the 7
// planes of A (128 rows from row qa of adig) and B (32 rows from row qb of bdig)
// into As / Bs, completing on the mbarrier at b0.
__device__ __forceinline__ void oz_copy_half(int h, uint32_t b0, unsigned char* As, unsigned char* Bs,
                                             const unsigned char* adig, int64_t aplane, int qa,
                                             const unsigned char* bdig, int64_t bplane, int qb) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(b0), "r"(static_cast<uint32_t>(kOzDigits * (kOzA + kOzBu))) : "memory");
    for (int j = 0; j < kOzDigits; ++j) {
        const unsigned char* ga = adig + j * aplane + h * (aplane >> 1) + static_cast<int64_t>(qa >> 3) * kOzSbo;
        const unsigned char* gb = bdig + j * bplane + h * (bplane >> 1) + static_cast<int64_t>(qb >> 3) * kOzSbo;
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     :: "r"(smem_addr(As + j * kOzA)), "l"(ga), "r"(static_cast<uint32_t>(kOzA)), "r"(b0)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     :: "r"(smem_addr(Bs + j * kOzBu)), "l"(gb), "r"(static_cast<uint32_t>(kOzBu)), "r"(b0)
                     : "memory");
    }
}

// Thread 0, after oz_copy_half(0, ...): for each K half wait for its planes, issue
// the 28 digit pairs x 2 K-steps of MMAs (M=128, N=32, K=16; level L into TMEM
// columns 32L..32L+31), wait for them to finish with the buffer and start the next
// half's copies. bar[0] counts the copies (phase h), bar[1] the MMA batches. Every
// wait is bounded; on a time-out it waits once more for what is in flight and
// returns false.
__device__ __forceinline__ bool oz_products(uint64_t* bar, uint32_t tmem, unsigned char* As, unsigned char* Bs,
                                            const unsigned char* adig, int64_t aplane, int qa,
                                            const unsigned char* bdig, int64_t bplane, int qb) {
    const uint32_t b0 = smem_addr(bar), b1 = smem_addr(bar + 1);
    const uint32_t sa = smem_addr(As), sb = smem_addr(Bs);
    for (int h = 0; h < 2; ++h) {
        if (!oz_wait(b0, h)) {
            oz_wait(b0, h);                            // copies still in flight: a second bounded wait
            return false;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int L = 0; L < kOzDigits; ++L) {
            for (int da = 0; da <= L; ++da) {
                const int db = L - da;
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
                    const uint32_t acc = (h > 0 || da > 0 || ks > 0) ? 1u : 0u;
                    const uint64_t adesc = oz_sdesc(sa + da * static_cast<uint32_t>(kOzA) + ks * 2 * kOzLbo);
                    const uint64_t bdesc = oz_sdesc(sb + db * static_cast<uint32_t>(kOzBu) + ks * 2 * kOzLbo);
                    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                                 :: "r"(tmem + static_cast<uint32_t>(32 * L)), "l"(adesc), "l"(bdesc),
                                    "r"(kOzIdesc32), "r"(acc));
                }
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     :: "r"(b1) : "memory");
        if (!oz_wait(b1, h)) {
            oz_wait(b1, h);                            // a second bounded wait before TMEM is freed
            return false;
        }
        if (h == 0) oz_copy_half(1, b0, As, Bs, adig, aplane, qa, bdig, bplane, qb);
    }
    return true;
}

// Row accumulators of 8 TMEM columns (from column c) of the 7 levels for this
// thread's lane, combined into the integers u with sum = u 2^(Ea+Eb-52):
// hi 2^(E-30) + lo 2^(E-62) = 2^(E-52) (hi 2^22 + lo 2^-10), one integer below 2^62
// (lo rounded to 2^(E-53)).
__device__ __forceinline__ void oz_read8(uint32_t taddr, long long* u) {
    uint32_t v[kOzDigits][8];
#pragma unroll
    for (int L = 0; L < kOzDigits; ++L)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(v[L][0]), "=r"(v[L][1]), "=r"(v[L][2]), "=r"(v[L][3]), "=r"(v[L][4]),
                       "=r"(v[L][5]), "=r"(v[L][6]), "=r"(v[L][7])
                     : "r"(taddr + static_cast<uint32_t>(32 * L)));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        long long lv[kOzDigits];
#pragma unroll
        for (int L = 0; L < kOzDigits; ++L) lv[L] = __float2int_rn(__uint_as_float(v[L][q]));
        const long long hi = lv[0] * 65536LL + lv[1] * 256LL + lv[2];   // |hi| < 2^39.2
        const long long lo = lv[3] * 16777216LL + lv[4] * 65536LL + lv[5] * 256LL + lv[6];  // < 2^47.2
        u[q] = hi * 4194304LL + ((lo + 512) >> 10);
    }
}

// Digits of the step's trailing panel rows: one block per 64-row tile (the trsm
// tiles), four threads per row with 16 columns each.
// Row block bi of block lb in a list where row block bi holds 2 bi + 2 blocks
// (bi (bi + 1) <= lb < (bi + 1)(bi + 2)); FP32 estimate corrected in integers (the
// FP64 pipe is kept for the epilogues).
__device__ __forceinline__ int block_row_of(int lb) {
    int bi = static_cast<int>((sqrtf(4.0f * static_cast<float>(lb) + 1.0f) - 1.0f) * 0.5f);
    while ((bi + 1) * (bi + 2) <= lb) ++bi;
    while (bi > 0 && bi * (bi + 1) > lb) --bi;
    return bi;
}

__global__ void __launch_bounds__(256) k_oz_digits(StepArgs a, const int* __restrict__ items,
                                                   const int* __restrict__ prefix, PlanDev pd,
                                                   const double* __restrict__ F, unsigned char* __restrict__ dig,
                                                   int* __restrict__ dexp, int64_t plane) {
    __shared__ double smax[4][64];
    const int i = find_item(prefix + a.tp_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int t0 = k0 + w;
    const int r = threadIdx.x & 63, cg = threadIdx.x >> 6;
    const int row = t0 + lt * T64 + r;
    const bool rin = row < N;
    const double* Fs = F + pd.F_off[s];
    double v[16];
    double mx = 0.0;
#pragma unroll
    for (int t = 0; t < 16; ++t) {
        const int k = cg * 16 + t;
        v[t] = (rin && k < w) ? Fs[row + static_cast<int64_t>(k0 + k) * LD] : 0.0;
        mx = fmax(mx, fabs(v[t]));
    }
    smax[cg][r] = mx;
    __syncthreads();
    mx = fmax(fmax(smax[0][r], smax[1][r]), fmax(smax[2][r], smax[3][r]));
    // E is held at -968 or above so that 2^(55 - E) stays a normal double (rows whose
    // largest entry is below 2^-967 keep fewer digits; they do not matter next to 1)
    const int E = mx > 0.0 ? max(ilogb(mx), -968) : 0;
    const int q = prefix[a.dr_off + i] + lt * T64 + r;
    oz_store_digits(v, E, q, cg, dig, plane);
    if (cg == 0) dexp[q] = E;
}

// C(128 x 32) -= A B^T from the digit planes: two blocks per 128-row x 64-column
// block of the trailing lower part (row block bi holds column blocks 0..2bi+1), each
// taking 32 of its columns, so that two blocks fit an SM (70 KB of shared memory, 256
// TMEM columns, at most 128 registers). Thread 0 streams the two K halves of the 14
// planes through one buffer with bulk copies and issues 28 digit pairs x 2 K-steps of
// MMAs (M=128, N=32, K=16) per half; level L accumulates in TMEM columns 32L..32L+31.
// Every thread loads its 16 C values meanwhile, then reads its row's 7 accumulators
// and applies them. The diagonal tile of the next step lies in both blocks of the
// first 128 x 64 block: the one of the two that finishes second (a per-front counter,
// no waiting) factors it. Every wait is bounded: on a time-out the block records
// err[2], waits once more for what it issued, frees its TMEM and leaves C untouched.
__global__ void __launch_bounds__(256, 2) k_update_oz(StepArgs a, const int* __restrict__ items,
                                                      const int* __restrict__ prefix, PlanDev pd, double* F,
                                                      double* __restrict__ Linv, const int64_t* __restrict__ inv_off,
                                                      const unsigned char* __restrict__ dig,
                                                      const int* __restrict__ dexp, int64_t plane, int* cnt,
                                                      int* err) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char* As = smraw;
    unsigned char* Bs = smraw + kOzDigits * kOzA;
    uint64_t* bar = reinterpret_cast<uint64_t*>(Bs + kOzDigits * kOzBu);   // [0] planes loaded, [1] MMAs done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    int* fail = reinterpret_cast<int*>(bar + 3);
    int* last = fail + 1;
    const int unit = blockIdx.x >> 1, hc = blockIdx.x & 1;
    const int i = find_item(prefix + a.up3_off, a.nitems, unit);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int lb = unit - prefix[a.up3_off + i];
    const int bi = block_row_of(lb);
    const int bj = lb - bi * (bi + 1);
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int t0 = k0 + w;
    const int r0 = t0 + bi * 128, c0 = t0 + bj * T64 + hc * 32;
    if (c0 >= N) return;                              // the whole block: columns past the front
    const int nra = min(128, N - r0), ncb = min(32, N - c0);
    const int qa = prefix[a.dr_off + i] + bi * 128, qb = prefix[a.dr_off + i] + bj * T64 + hc * 32;
    double* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    // thread 0 starts the first half's copies; TMEM allocation and every thread's C
    // loads then overlap them
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar + 1)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *fail = 0;
        oz_copy_half(0, smem_addr(bar), As, Bs, dig, plane, qa, dig, plane, qb);
    }
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" :: "r"(smem_addr(tslot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // this thread's row (TMEM lane) and 16 columns, and its C values
    const int row = 32 * (wid & 3) + lane, ch = 16 * (wid >> 2);
    const bool rok = row < nra;
    double cv[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const int col = ch + j;
        const bool in = rok && col < ncb && r0 + row >= c0 + col;
        cv[j] = in ? Fs[(r0 + row) + static_cast<int64_t>(c0 + col) * LD] : 0.0;
    }
    const int ea = rok ? dexp[qa + row] : 0;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    if (tid == 0 && !oz_products(bar, tmem, As, Bs, dig, plane, qa, dig, plane, qb)) {
        *fail = 1;
        atomicExch(err + 2, 1);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool ok = *fail == 0;
    if (ok) {
#pragma unroll
        for (int c8 = 0; c8 < 2; ++c8) {
            long long u[8];
            oz_read8(tmem + (static_cast<uint32_t>(32 * (wid & 3)) << 16) + static_cast<uint32_t>(ch + 8 * c8), u);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int j = 8 * c8 + q, col = ch + j;
                // one conversion and one FP64 FMA on the slow FP64 pipe per entry
                if (rok && col < ncb && r0 + row >= c0 + col)
                    Fs[(r0 + row) + static_cast<int64_t>(c0 + col) * LD] =
                        fma(-static_cast<double>(u[q]), oz_pow2(ea + dexp[qb + col] - 52), cv[j]);
            }
        }
    }
    __threadfence();                                   // this block's C writes, before the counter below
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (wid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" :: "r"(tmem));
    }
    if (!ok) return;
    // the next diagonal tile spans both blocks of the first 128 x 64 block: the second
    // of the two to get here factors it (when the front ends within the first 32
    // columns the first block is alone) and resets the counter for the next step
    if (lb == 0 && t0 < K) {
        if (tid == 0) {
            if (t0 + 32 >= N) {
                *last = 1;
            } else {
                const int prev = atomicAdd(cnt + s, 1);
                *last = prev == 1;
                if (prev == 1) atomicExch(cnt + s, 0);
                __threadfence();
            }
        }
        __syncthreads();
        if (*last) potrf_tile<double>(s, a.k + 1, pd, F, Linv, inv_off, err, smraw);
    }
}

// ---- FP64 panel solve on the tensor cores (the same digit products) ----------
// X = B Linv^T for the step's panel rows below the diagonal tile (B = their current
// values, Linv = the inverse of the factored diagonal tile): k_oz_digits writes the
// digits of B before the solve, k_oz_linv_digits those of the 64 rows of Linv of
// every item of the step (one block per item, rows i * 64 .. in a buffer of its own),
// and k_trsm_oz forms X = u 2^(Ea+Eb-52) with the MMAs of k_update_oz and no C
// operand: two blocks per 128 panel rows, each taking 32 of the 64 Linv rows (N = 32).
__global__ void __launch_bounds__(256) k_oz_linv_digits(StepArgs a, const int* __restrict__ items, PlanDev pd,
                                                        const double* __restrict__ Linv,
                                                        const int64_t* __restrict__ inv_off,
                                                        unsigned char* __restrict__ dig, int* __restrict__ dexp,
                                                        int64_t plane) {
    __shared__ double smax[4][64];
    const int i = blockIdx.x;
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const double* Li = Linv + inv_off[s] + static_cast<int64_t>(a.k) * T64 * T64;   // column-major 64 x 64
    const int r = threadIdx.x & 63, cg = threadIdx.x >> 6;
    double v[16];
    double mx = 0.0;
#pragma unroll
    for (int t = 0; t < 16; ++t) {
        v[t] = Li[r + (cg * 16 + t) * T64];
        mx = fmax(mx, fabs(v[t]));
    }
    smax[cg][r] = mx;
    __syncthreads();
    mx = fmax(fmax(smax[0][r], smax[1][r]), fmax(smax[2][r], smax[3][r]));
    const int E = mx > 0.0 ? max(ilogb(mx), -968) : 0;
    const int q = i * T64 + r;
    oz_store_digits(v, E, q, cg, dig, plane);
    if (cg == 0) dexp[q] = E;
}

__global__ void __launch_bounds__(256, 2) k_trsm_oz(StepArgs a, const int* __restrict__ items,
                                                    const int* __restrict__ prefix, PlanDev pd, double* F,
                                                    const unsigned char* __restrict__ dig,
                                                    const int* __restrict__ dexp, int64_t plane,
                                                    const unsigned char* __restrict__ ldig,
                                                    const int* __restrict__ lexp, int64_t lplane, int* err) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char* As = smraw;
    unsigned char* Bs = smraw + kOzDigits * kOzA;
    uint64_t* bar = reinterpret_cast<uint64_t*>(Bs + kOzDigits * kOzBu);   // [0] planes loaded, [1] MMAs done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    int* fail = reinterpret_cast<int*>(bar + 3);
    const int unit = blockIdx.x >> 1, hc = blockIdx.x & 1;   // 128 panel rows, 32 of the 64 columns
    const int i = find_item(prefix + a.dr_off, a.nitems, unit * 128);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int blk = unit - prefix[a.dr_off + i] / 128;
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int r0 = k0 + w + blk * 128;
    if (r0 >= N || hc * 32 >= w) return;              // a padded block of the digit rows, or no columns
    const int nra = min(128, N - r0);
    const int qa = prefix[a.dr_off + i] + blk * 128, qb = i * T64 + hc * 32;
    double* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    if (tid == 0) {                                    // the copies first, then TMEM allocation
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar + 1)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *fail = 0;
        oz_copy_half(0, smem_addr(bar), As, Bs, dig, plane, qa, ldig, lplane, qb);
    }
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" :: "r"(smem_addr(tslot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    if (tid == 0 && !oz_products(bar, tmem, As, Bs, dig, plane, qa, ldig, lplane, qb)) {
        *fail = 1;
        atomicExch(err + 2, 1);
    }
    const int row = 32 * (wid & 3) + lane, ch = 16 * (wid >> 2);
    const bool rok = row < nra;
    const int ea = rok ? dexp[qa + row] : 0;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (*fail == 0) {
#pragma unroll
        for (int c8 = 0; c8 < 2; ++c8) {
            long long u[8];
            oz_read8(tmem + (static_cast<uint32_t>(32 * (wid & 3)) << 16) + static_cast<uint32_t>(ch + 8 * c8), u);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int col = hc * 32 + ch + 8 * c8 + q;
                if (rok && col < w)
                    Fs[(r0 + row) + static_cast<int64_t>(k0 + col) * LD] =
                        static_cast<double>(u[q]) * oz_pow2(ea + lexp[i * T64 + col] - 52);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (wid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" :: "r"(tmem));
    }
}

// ---- FP32 trailing update on the tensor cores from pre-split panels -----------
// The step's trailing panel rows (64 FP32 entries each) are split once per step
// into TF32 parts hi = tf32(x), lo = tf32(x - hi) (k_tc_split, one block per 64-row
// trsm tile) and written to the digit buffer in the canonical K-major no-swizzle
// layout of 8-row x 16-byte core matrices (K-adjacent core matrices 128 B apart,
// 8-row groups 2048 B apart): a block's 128 (A) or 64 (B) consecutive rows are one
// contiguous 32 KB / 16 KB bulk copy per part. k_update_tcs then computes C(128 x 64)
// -= A B^T as lo_A hi_B + hi_A lo_B + hi_A hi_B (TF32 x3, close to FP32 accuracy):
// one thread copies the four parts with cp.async.bulk and issues the 24 MMAs (M=128,
// N=64, K=8) into 64 TMEM columns while every thread loads its 32 C values; 96 KB of
// shared memory and at most 128 registers per thread leave room for two blocks per
// SM. Blocks follow the 128-row x 64-column lower-part list of the emulated FP64
// update (row block bi holds column blocks 0..2bi+1). Every wait is bounded: on a
// time-out the block records err[2], waits once more for what it issued, frees its
// TMEM and leaves C untouched.
constexpr uint32_t kTsLbo = 128;                       // bytes between K-adjacent core matrices
constexpr uint32_t kTsSbo = 2048;                      // bytes between 8-row groups (64 FP32 per row)
constexpr size_t kTsA = 128 * 256;                     // 128 rows x 64 FP32: 32 KB per part
constexpr size_t kTsB = 64 * 256;                      // 64 rows: 16 KB per part
constexpr size_t kTsSmem = 2 * (kTsA + kTsB) + 64;
// instruction descriptor: D = F32 (bits 4-5 = 1), A = B = TF32 (bits 7-9, 10-12 = 2), both
// K-major, N >> 3 at bits 17-22 (N = 64), M >> 4 at bits 24-28 (M = 128)
constexpr uint32_t kTsIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__global__ void __launch_bounds__(256) k_tc_split(StepArgs a, const int* __restrict__ items,
                                                  const int* __restrict__ prefix, PlanDev pd,
                                                  const float* __restrict__ F, unsigned char* __restrict__ dig,
                                                  int64_t plane) {
    const int i = find_item(prefix + a.tp_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int t0 = k0 + w;
    const int r = threadIdx.x & 63, cg = threadIdx.x >> 6;
    const int row = t0 + lt * T64 + r;
    const bool rin = row < N;
    const float* Fs = F + pd.F_off[s];
    const int q = prefix[a.dr_off + i] + lt * T64 + r;
    unsigned char* base = dig + static_cast<int64_t>(q >> 3) * kTsSbo + (q & 7) * 16;
#pragma unroll
    for (int h = 0; h < 4; ++h) {                      // one core matrix (4 columns) per pass
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int k = cg * 16 + h * 4 + u;
            const float v = (rin && k < w) ? Fs[row + static_cast<int64_t>(k0 + k) * LD] : 0.f;
            hi[u] = to_tf32(v);
            lo[u] = to_tf32(v - __uint_as_float(hi[u]));
        }
        const int kc = cg * 4 + h;
        *reinterpret_cast<uint4*>(base + kc * kTsLbo) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(base + plane + kc * kTsLbo) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
}

__global__ void __launch_bounds__(256, 2) k_update_tcs(StepArgs a, const int* __restrict__ items,
                                                       const int* __restrict__ prefix, PlanDev pd, float* F,
                                                       float* __restrict__ Linv, const int64_t* __restrict__ inv_off,
                                                       const unsigned char* __restrict__ dig, int64_t plane,
                                                       int* err) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char* Ah = smraw;
    unsigned char* Al = Ah + kTsA;
    unsigned char* Bh = Al + kTsA;
    unsigned char* Bl = Bh + kTsB;
    uint64_t* bar = reinterpret_cast<uint64_t*>(Bl + kTsB);   // [0] parts loaded, [1] MMAs done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    int* fail = reinterpret_cast<int*>(bar + 3);
    const int i = find_item(prefix + a.up3_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    const int lb = blockIdx.x - prefix[a.up3_off + i];
    int bi = block_row_of(lb);
    const int bj = lb - bi * (bi + 1);
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], LD = pd.sn_lda[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int t0 = k0 + w;
    const int r0 = t0 + bi * 128, c0 = t0 + bj * T64;
    if (c0 >= N) return;                              // the whole block: column block past the front
    const int nra = min(128, N - r0), ncb = min(T64, N - c0);
    const int qa = prefix[a.dr_off + i] + bi * 128, qb = prefix[a.dr_off + i] + bj * T64;
    float* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    // thread 0 starts the copies first; TMEM allocation and every thread's C loads
    // then overlap them
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(bar + 1)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *fail = 0;
        const uint32_t b0 = smem_addr(bar);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                     :: "r"(b0), "r"(static_cast<uint32_t>(2 * (kTsA + kTsB))) : "memory");
        const unsigned char* ga = dig + static_cast<int64_t>(qa >> 3) * kTsSbo;
        const unsigned char* gb = dig + static_cast<int64_t>(qb >> 3) * kTsSbo;
        const unsigned char* src[4] = {ga, ga + plane, gb, gb + plane};
        unsigned char* dst[4] = {Ah, Al, Bh, Bl};
        const uint32_t len[4] = {static_cast<uint32_t>(kTsA), static_cast<uint32_t>(kTsA),
                                 static_cast<uint32_t>(kTsB), static_cast<uint32_t>(kTsB)};
        for (int c = 0; c < 4; ++c)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         :: "r"(smem_addr(dst[c])), "l"(src[c]), "r"(len[c]), "r"(b0) : "memory");
    }
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" :: "r"(smem_addr(tslot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // this thread's row (TMEM lane) and 32 columns, and its C values
    const int row = 32 * (wid & 3) + lane, ch = 32 * (wid >> 2);
    const bool rok = row < nra;
    float cv[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int col = ch + j;
        const bool in = rok && col < ncb && r0 + row >= c0 + col;
        cv[j] = in ? Fs[(r0 + row) + static_cast<int64_t>(c0 + col) * LD] : 0.f;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        const uint32_t b0 = smem_addr(bar);
        bool ok = oz_wait(b0);
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ah = smem_addr(Ah), al = smem_addr(Al), bh = smem_addr(Bh), bl = smem_addr(Bl);
            uint32_t acc = 0;
            for (int ks = 0; ks < T64 / 8; ++ks) {
                const uint32_t ko = static_cast<uint32_t>(ks) * 2 * kTsLbo;
                const uint64_t da[3] = {tc_sdesc(al + ko), tc_sdesc(ah + ko), tc_sdesc(ah + ko)};
                const uint64_t db[3] = {tc_sdesc(bh + ko), tc_sdesc(bl + ko), tc_sdesc(bh + ko)};
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                                 :: "r"(tmem), "l"(da[q]), "l"(db[q]), "r"(kTsIdesc), "r"(acc));
                    acc = 1;
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(smem_addr(bar + 1)) : "memory");
            ok = oz_wait(smem_addr(bar + 1));
            if (!ok) oz_wait(smem_addr(bar + 1));     // a second bounded wait before TMEM is freed
        } else {
            oz_wait(b0);                               // copies still in flight: a second bounded wait
        }
        if (!ok) {
            *fail = 1;
            atomicExch(err + 2, 1);
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool ok = *fail == 0;
    if (ok) {
#pragma unroll
        for (int c16 = 0; c16 < 2; ++c16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + (static_cast<uint32_t>(32 * (wid & 3)) << 16) +
                                   static_cast<uint32_t>(ch + 16 * c16);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                           "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                           "=r"(v[14]), "=r"(v[15])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int j = 16 * c16 + q, col = ch + j;
                if (rok && col < ncb && r0 + row >= c0 + col)
                    Fs[(r0 + row) + static_cast<int64_t>(c0 + col) * LD] = cv[j] - __uint_as_float(v[q]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (wid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" :: "r"(tmem));
    }
    if (!ok) return;
    // the block holding the first trailing diagonal tile factors it (as in k_update)
    if (lb == 0 && t0 < K) {
        __syncthreads();
        potrf_tile<float>(s, a.k + 1, pd, F, Linv, inv_off, err, smraw);
    }
}

template <class T>
__global__ void k_extend_add(int item_off, int nitems, int prefix_off, const int* __restrict__ items,
                             const int* __restrict__ prefix, PlanDev pd, T* F) {
    const int i = find_item(prefix + prefix_off, nitems, blockIdx.x);
    const int c = items[item_off + i];
    if (!pd.lp_on[pd.sn_lp[c]]) return;
    const int lt = blockIdx.x - prefix[prefix_off + i];
    int ti, tj;
    tri_index(lt, ti, tj);
    const int Kc = pd.sn_ncols[c], Nc = pd.sn_nrows[c];
    const int u = Nc - Kc;
    const int p = pd.sn_parent[c];
    const T* Fc = F + pd.F_off[c];
    T* Fp = F + pd.F_off[p];
    const int* map = pd.ea_map + pd.ea_off[c];
    const int rr = ti * 32 + threadIdx.x;
    if (rr >= u) return;
    const int mr = map[rr];
    for (int cc = tj * 32 + threadIdx.y; cc < tj * 32 + 32 && cc < u; cc += blockDim.y) {
        if (rr < cc) continue;
        const T v = Fc[(Kc + rr) + static_cast<int64_t>(Kc + cc) * pd.sn_lda[c]];
        T* dst = Fp + mr + static_cast<int64_t>(map[cc]) * pd.sn_lda[p];
        *dst = *dst + v;
    }
}

// -------------------------------------------------------------------- solve
// Vectors of the solve are in the front precision T; the caller's vectors are FP64.

template <class T>
__global__ void k_permute_scale(int M, const int* __restrict__ perm, const double* __restrict__ D,
                                const double* __restrict__ src, T* __restrict__ zp) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < M) zp[q] = static_cast<T>(D[q] * src[perm[q]]);
}

// Rows of the LPs in `own` receive D xp; rows of the LPs in `other` (the set the
// other precision's pass serves; may be null) are left as they are; all other
// rows get 0.
template <class T>
__global__ void k_unpermute_scale(int M, const int* __restrict__ perm, const double* __restrict__ D,
                                  const T* __restrict__ xp, const int* __restrict__ row_lp,
                                  const int* __restrict__ own, const int* __restrict__ other,
                                  double* __restrict__ dst) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < M) {
        const int r = perm[q];
        const int k = row_lp[r];
        if (own[k]) dst[r] = D[q] * static_cast<double>(xp[q]);
        else if (!other || !other[k]) dst[r] = 0.0;
    }
}

// Zeroes the fronts of the LPs being factored, one chunk of a front per block
// (the fronts of other LPs keep their factors).
constexpr int kZeroChunk = 8192;
template <class T>
__global__ void __launch_bounds__(256) k_zero_fronts(const int* __restrict__ zc_sn, const int* __restrict__ zc_len,
                                                     const int64_t* __restrict__ zc_off, PlanDev pd,
                                                     T* __restrict__ F) {
    const int s = zc_sn[blockIdx.x];
    if (!pd.lp_on[pd.sn_lp[s]]) return;
    T* p = F + zc_off[blockIdx.x];
    const int len = zc_len[blockIdx.x];
    for (int i = threadIdx.x; i < len; i += blockDim.x) p[i] = T(0);
}

// Frontal right-hand sides of one level: one thread per front row, the row's own
// entry of the permuted rhs (or 0 outside the front's columns) plus the children's
// update-vector entries that map to it, added in child order.
template <class T>
__global__ void k_fwd_gather(int n, const int* __restrict__ dst, const int* __restrict__ zpi,
                             const int* __restrict__ ptr, const int* __restrict__ src, const T* __restrict__ zp,
                             T* __restrict__ fv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int z = zpi[t];
    T acc = z >= 0 ? zp[z] : T(0);
    for (int q = ptr[t]; q < ptr[t + 1]; ++q) acc += fv[src[q]];
    fv[dst[t]] = acc;
}

// ---- dependency-driven triangular solves -------------------------------------
// Each front's rows are split into 64-row blocks; block i of front s is one task.
// Tasks of a level are handed out in dependency order by an atomic counter, so a
// task only ever waits for tasks that have already started; results are
// published through per-block flags. Every wait is bounded: on time-out the task
// sets *err and returns (the host checks *err and reports an error).

constexpr int kSpinLimit = 1 << 24;

__device__ __forceinline__ bool wait_flag(const int* flag, int target, int* err, int* abort_sh) {
    int spins = 0;
    while (*reinterpret_cast<const volatile int*>(flag) < target) {
        if (*reinterpret_cast<const volatile int*>(err) != 0 || ++spins > kSpinLimit) {
            atomicExch(err, 1);
            *abort_sh = 1;
            return false;
        }
        // poll back to back first (the flag of the last dependency usually comes within
        // microseconds: this wait is on the solve's critical path), then back off
        if (spins > 512) __nanosleep(64);
    }
    __threadfence();
    return true;
}

template <class T>
__device__ __forceinline__ T ld_cg(const T* p) { return __ldcg(p); }

constexpr int kReadyBlocks = 16;   // column blocks taken per pass once their flags are set

__device__ __forceinline__ int flag_now(const int* flag) { return *reinterpret_cast<const volatile int*>(flag); }

// Forward: task (s, i). Own block i < nb covers rows [64 i, min(64 i + 64, K));
// external block i >= nb covers rows [K + 64 (i - nb), ...) < N. The task forms
// f_rows - sum_{j < min(i, nb)} L(rows, block j) z_j; an own block then stores
// z_i = Linv_i (..) in zsol and flags 1, an external block stores the parent's
// update vector in f. Column blocks whose flags are already set are taken
// together (up to kReadyBlocks per pass); the first block of each pass has its L
// values loaded before the wait, so the latency-critical last dependency only
// waits for its flag and z values.
template <class T>
__global__ void __launch_bounds__(256, 1) k_fwd_tasks(const int2* __restrict__ tasks, int ntasks, int* counter,
                                                   PlanDev pd, const T* __restrict__ F, const T* __restrict__ Linv,
                                                   const int64_t* __restrict__ inv_off,
                                                   const int* __restrict__ blk_off, int* flags, T* fv, T* zsol,
                                                   int* err) {
    __shared__ int task_sh, abort_sh, ready_sh;
    __shared__ T zs[kReadyBlocks * T64];
    __shared__ T red[4][T64];
    __shared__ T fb[T64];
    const int tid = threadIdx.x;
    if (tid == 0) {
        task_sh = atomicAdd(counter, 1);
        abort_sh = 0;
    }
    __syncthreads();
    const int t = task_sh;
    if (t >= ntasks) return;
    const int s = tasks[t].x, i = tasks[t].y;
    if (!pd.lp_on[pd.sn_lp[s]]) return;   // every task of the front's LP is skipped alike
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    const int LD = pd.sn_lda[s];
    const int nb = (K + T64 - 1) / T64;
    const T* Fs = F + pd.F_off[s];
    T* f = fv + pd.f_off[s];
    int* fl = flags + blk_off[s];
    const int r = tid & 63, cg = tid >> 6;
    const bool own = i < nb;
    const int row0 = own ? i * T64 : K + (i - nb) * T64;
    const int rend = own ? K : N;
    const int row = row0 + r;
    const bool rv = row < rend;
    // this thread's entries of the diagonal-tile inverse (own blocks), loaded up front
    const int w = own ? min(T64, K - i * T64) : 0;
    const int zc = tid >> 2, zpart = tid & 3;
    T li[16];
    if (own) {
        const T* Li = Linv + inv_off[s] + static_cast<int64_t>(i) * T64 * T64;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int q = zpart + 4 * k;
            li[k] = (zc < w && q <= zc) ? Li[zc + q * T64] : T(0);
        }
    }
    // this block's right-hand side (written by the gather before this kernel), loaded up front
    const T fown = (tid < T64 && row0 + tid < rend) ? f[row0 + tid] : T(0);
    T acc = T(0);
    const int jmax = own ? i : nb;
    for (int j = 0; j < jmax;) {
        T pre[16];
        const int colp = j * T64 + cg * 16;
#pragma unroll
        for (int c = 0; c < 16; ++c)
            pre[c] = (rv && colp + c < K) ? Fs[row + static_cast<int64_t>(colp + c) * LD] : T(0);
        if (tid == 0) {
            if (wait_flag(fl + j, 1, err, &abort_sh)) {
                int e = j + 1;
                while (e < jmax && e < j + kReadyBlocks && flag_now(fl + e) >= 1) ++e;
                __threadfence();
                ready_sh = e;
            }
        }
        __syncthreads();
        if (abort_sh) return;
        const int e = ready_sh;
        for (int q = tid; q < (e - j) * T64; q += 256) {
            const int col = j * T64 + q;
            zs[q] = col < K ? ld_cg(zsol + first + col) : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 16; ++c) acc += pre[c] * zs[cg * 16 + c];
        if (rv) {
            for (int jj = j + 1; jj < e; ++jj) {
                const T* Lc = Fs + row + static_cast<int64_t>(jj * T64 + cg * 16) * LD;
                const T* zz = zs + (jj - j) * T64 + cg * 16;
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    if (jj * T64 + cg * 16 + c < K) acc += Lc[static_cast<int64_t>(c) * LD] * zz[c];
            }
        }
        __syncthreads();
        j = e;
    }
    red[cg][r] = acc;
    __syncthreads();
    if (tid < T64) {
        const int rw = row0 + tid;
        fb[tid] = rw < rend ? fown - ((red[0][tid] + red[1][tid]) + (red[2][tid] + red[3][tid])) : T(0);
    }
    __syncthreads();
    if (own) {
        T z = T(0);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int q = zpart + 4 * k;
            if (q <= zc) z += li[k] * fb[q];
        }
        z += __shfl_xor_sync(0xffffffffu, z, 1);
        z += __shfl_xor_sync(0xffffffffu, z, 2);
        if (zpart == 0 && zc < w) zsol[first + i * T64 + zc] = z;
        __threadfence();
        __syncthreads();
        if (tid == 0) atomicExch(fl + i, 1);
    } else {
        if (tid < T64 && row0 + tid < N) f[row0 + tid] = fb[tid];
    }
}

// Backward: task (s, i), i descending: x_i = Linv_i^T (z_i - sum_{rows r below
// block i} L(r, block i)^T x_r); rows of own later blocks wait for their flag (2),
// rows outside the front's columns come from ancestors (earlier levels). Later
// blocks are taken oldest first (nb - 1 downwards), ready ones together, and the
// L values of the first block of each pass are loaded before its wait.
template <class T>
__global__ void __launch_bounds__(256, 2) k_bwd_tasks(const int2* __restrict__ tasks, int ntasks, int* counter,
                                                   PlanDev pd, const T* __restrict__ F, const T* __restrict__ Linv,
                                                   const int64_t* __restrict__ inv_off,
                                                   const int* __restrict__ blk_off, int* flags, T* xp,
                                                   const T* __restrict__ zsol, int* err) {
    __shared__ int task_sh, abort_sh, ready_sh;
    __shared__ T xb[kReadyBlocks * T64];   // x of ready own blocks, or of a chunk of outside rows
    __shared__ T tb[T64];
    const int tid = threadIdx.x;
    if (tid == 0) {
        task_sh = atomicAdd(counter, 1);
        abort_sh = 0;
    }
    __syncthreads();
    const int t = task_sh;
    if (t >= ntasks) return;
    const int s = tasks[t].x, i = tasks[t].y;
    if (!pd.lp_on[pd.sn_lp[s]]) return;   // every task of the front's LP is skipped alike
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    const int LD = pd.sn_lda[s];
    const int nb = (K + T64 - 1) / T64;
    const int w = min(T64, K - i * T64);
    const T* Fs = F + pd.F_off[s];
    const int* R = pd.rows + pd.rows_off[s];
    int* fl = flags + blk_off[s];
    const int lane = tid & 31, wid = tid >> 5;
    T part[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) part[q] = T(0);
    const int c0 = i * T64 + wid * 8;
    // rows outside the front's own columns (solved by ancestors): their x values are
    // gathered into shared memory a chunk at a time, then each warp runs down the rows
    constexpr int kOut = kReadyBlocks * T64;
    for (int r0 = K; r0 < N; r0 += kOut) {
        const int nr = min(kOut, N - r0);
        for (int q = tid; q < nr; q += 256) xb[q] = xp[R[r0 + q]];
        __syncthreads();
        // four rows per lane per pass: 32 independent loads in flight
        int q = lane;
        for (; q + 96 < nr; q += 128) {
            T fr[4][8];
#pragma unroll
            for (int h = 0; h < 4; ++h)
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    fr[h][u] = c0 + u < K ? Fs[(r0 + q + 32 * h) + static_cast<int64_t>(c0 + u) * LD] : T(0);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const T xr = xb[q + 32 * h];
#pragma unroll
                for (int u = 0; u < 8; ++u) part[u] += fr[h][u] * xr;
            }
        }
        for (; q < nr; q += 32) {
            const T xr = xb[q];
            const T* Fr = Fs + (r0 + q);
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (c0 + u < K) part[u] += Fr[static_cast<int64_t>(c0 + u) * LD] * xr;
        }
        __syncthreads();
    }
    // this thread's entries of the diagonal-tile inverse
    const int xc = tid >> 2, xpq = tid & 3;
    T li[16];
    {
        const T* Li = Linv + inv_off[s] + static_cast<int64_t>(i) * T64 * T64;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int q = xc + xpq + 4 * k;
            li[k] = (xc < w && q < w) ? Li[q + xc * T64] : T(0);
        }
    }
    // rows of own later blocks
    for (int j = nb - 1; j > i;) {
        T pre[16];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int rr = j * T64 + lane + 32 * h;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                pre[h * 8 + q] = (rr < K && c0 + q < K) ? Fs[rr + static_cast<int64_t>(c0 + q) * LD] : T(0);
        }
        if (tid == 0) {
            if (wait_flag(fl + j, 2, err, &abort_sh)) {
                int e = j - 1;
                while (e > i && e > j - kReadyBlocks && flag_now(fl + e) >= 2) --e;
                __threadfence();
                ready_sh = e;
            }
        }
        __syncthreads();
        if (abort_sh) return;
        const int e = ready_sh;   // blocks j, j - 1, ..., e + 1 are ready
        for (int q = tid; q < (j - e) * T64; q += 256) {
            const int blk = j - q / T64, rr = blk * T64 + q % T64;
            xb[q] = rr < K ? ld_cg(xp + first + rr) : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const T xr = xb[lane + 32 * h];
#pragma unroll
            for (int q = 0; q < 8; ++q) part[q] += pre[h * 8 + q] * xr;
        }
        for (int blk = j - 1; blk > e; --blk) {
            const T* xx = xb + (j - blk) * T64;
            for (int rr = lane; rr < T64; rr += 32) {
                const int r = blk * T64 + rr;
                if (r >= K) break;
                const T xr = xx[rr];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (c0 + q < K) part[q] += Fs[r + static_cast<int64_t>(c0 + q) * LD] * xr;
            }
        }
        __syncthreads();
        j = e;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        T v = part[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
            const int c = wid * 8 + q;
            tb[c] = c < w ? zsol[first + i * T64 + c] - v : T(0);
        }
    }
    __syncthreads();
    {
        T x = T(0);
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int q = xc + xpq + 4 * k;
            if (q < w) x += li[k] * tb[q];
        }
        x += __shfl_xor_sync(0xffffffffu, x, 1);
        x += __shfl_xor_sync(0xffffffffu, x, 2);
        if (xpq == 0 && xc < w) xp[first + i * T64 + xc] = x;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) atomicExch(fl + i, 2);
}

// ------------------------------------------------------- normal-matrix apply

__global__ void k_spmv_rows(int rows, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ v, const double* __restrict__ x,
                            const double* __restrict__ scale, double* __restrict__ y) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double acc = 0.0;
    for (int q = rp[r]; q < rp[r + 1]; ++q) acc += v[q] * x[ci[q]];
    y[r] = scale ? acc * scale[r] : acc;
}

inline int blocks_for(int64_t n, int t) { return static_cast<int>((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------ engine

struct KktEngine::Prof {
    cudaStream_t st;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev;
    double upd_flops = 0.0, upd_bytes = 0.0;
    double mma_flops = 0.0;   // flops the tensor cores execute in the update launches
    template <class F>
    void timed(int cls, F&& launch) {
        cudaEvent_t a, b;
        SK_CUDA(cudaEventCreate(&a));
        SK_CUDA(cudaEventCreate(&b));
        SK_CUDA(cudaEventRecord(a, st));
        launch();
        SK_CUDA(cudaEventRecord(b, st));
        ev.push_back({cls, {a, b}});
    }
};

template <class T>
static void set_smem_attrs() {
    if (std::is_same<T, float>::value)
        SK_CUDA(cudaFuncSetAttribute(k_update_tcs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(kTsSmem)));
    SK_CUDA(cudaFuncSetAttribute(k_potrf<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(potrf_smem(sizeof(T)))));
    SK_CUDA(cudaFuncSetAttribute(k_trsm<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(2 * T64 * T64 * sizeof(T))));
    SK_CUDA(cudaFuncSetAttribute(k_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(potrf_smem(sizeof(T)))));
    if (std::is_same<T, double>::value)
        SK_CUDA(cudaFuncSetAttribute(k_update_oz, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(kOzSmemU)));
    if (std::is_same<T, double>::value)
        SK_CUDA(cudaFuncSetAttribute(k_trsm_oz, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(kOzSmemU)));
}

KktEngine::KktEngine(const ipm::FrontPlan& plan, const DeviceLP& lp, cudaStream_t stream)
    : plan_(plan), lp_(lp), st_(stream) {
    const auto& p = plan_;
    // tile-inverse offsets and per-level column-block prefixes of the backward pass
    std::vector<int64_t> inv_off(static_cast<size_t>(p.ns), 0);
    inv_size_ = 0;
    for (int s = 0; s < p.ns; ++s) {
        inv_off[s] = inv_size_;
        inv_size_ += static_cast<int64_t>((p.sn_ncols[s] + T64 - 1) / T64) * T64 * T64;
    }
    // solve task lists per level (forward: row blocks ascending; backward: own
    // column blocks descending) and per-front flag offsets
    std::vector<int> blk_off(static_cast<size_t>(p.ns), 0);
    nflags_ = 0;
    for (int s = 0; s < p.ns; ++s) {
        blk_off[s] = nflags_;
        nflags_ += (p.sn_ncols[s] + T64 - 1) / T64;
    }
    // Within a level the tasks are ordered by their position in their front's chain
    // (forward: block index; backward: distance from the last own block), fronts
    // interleaved: blocks take tasks in list order, so the first tasks of every
    // front of a level (e.g. all LPs of a dense batch) run side by side instead of
    // a few fronts' chains at a time. A task only waits on tasks of smaller position
    // in its own front, which come earlier in the list, so the earliest unfinished
    // task can always proceed.
    std::vector<int2> ftask, btask;
    fwd_task_off_.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    bwd_task_off_.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    for (int l = 0; l < p.nlevels; ++l) {
        fwd_task_off_[l] = static_cast<int>(ftask.size());
        bwd_task_off_[l] = static_cast<int>(btask.size());
        std::vector<std::pair<int, int2>> fl, bl;   // (position, task)
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            const int s = p.level_sn[q];
            const int nb = (p.sn_ncols[s] + T64 - 1) / T64;
            const int neb = (p.sn_nrows[s] - p.sn_ncols[s] + T64 - 1) / T64;
            for (int i = 0; i < nb + neb; ++i) fl.push_back({i, make_int2(s, i)});
            for (int i = nb - 1; i >= 0; --i) bl.push_back({nb - 1 - i, make_int2(s, i)});
        }
        auto by_pos = [](const std::pair<int, int2>& a, const std::pair<int, int2>& b) { return a.first < b.first; };
        std::stable_sort(fl.begin(), fl.end(), by_pos);
        std::stable_sort(bl.begin(), bl.end(), by_pos);
        for (const auto& t : fl) ftask.push_back(t.second);
        for (const auto& t : bl) btask.push_back(t.second);
    }
    fwd_task_off_[p.nlevels] = static_cast<int>(ftask.size());
    bwd_task_off_[p.nlevels] = static_cast<int>(btask.size());
    // forward right-hand-side gather lists (one item per front row, level by level)
    if (p.f_size >= (int64_t(1) << 31)) throw std::runtime_error("front vectors exceed 2^31 entries");
    std::vector<int> g_dst, g_zp, g_ptr(1, 0), g_src;
    gather_off_.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    for (int l = 0; l < p.nlevels; ++l) {
        gather_off_[l] = static_cast<int>(g_dst.size());
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            const int s = p.level_sn[q];
            const int N = p.sn_nrows[s], K = p.sn_ncols[s];
            std::vector<int> cnt(static_cast<size_t>(N) + 1, 0);
            for (int e = p.ch_ptr[s]; e < p.ch_ptr[s + 1]; ++e) {
                const int c = p.ch_list[e], u = p.sn_nrows[c] - p.sn_ncols[c];
                for (int r = 0; r < u; ++r) cnt[p.ea_map[p.ea_off[c] + r] + 1]++;
            }
            for (int r = 0; r < N; ++r) cnt[r + 1] += cnt[r];
            std::vector<int> src(static_cast<size_t>(cnt[N])), pos(cnt.begin(), cnt.end() - 1);
            for (int e = p.ch_ptr[s]; e < p.ch_ptr[s + 1]; ++e) {
                const int c = p.ch_list[e], Kc = p.sn_ncols[c], u = p.sn_nrows[c] - Kc;
                for (int r = 0; r < u; ++r)
                    src[pos[p.ea_map[p.ea_off[c] + r]]++] = static_cast<int>(p.sn_f_off[c] + Kc + r);
            }
            for (int r = 0; r < N; ++r) {
                g_dst.push_back(static_cast<int>(p.sn_f_off[s] + r));
                g_zp.push_back(r < K ? p.sn_first[s] + r : -1);
                g_ptr.push_back(g_ptr.back() + cnt[r + 1] - cnt[r]);
            }
            g_src.insert(g_src.end(), src.begin(), src.end());
        }
    }
    gather_off_[p.nlevels] = static_cast<int>(g_dst.size());
    // LP of each front (from the batch row of its first column) and the all-on LP mask
    const std::vector<int> sn_lp = ipm::supernode_lps(p);
    sn_lp_h_ = sn_lp;
    on32_h_.assign(static_cast<size_t>(std::max(1, p.nlp)), 1);
    on64_h_ = on32_h_;
    // LP of each permuted row
    std::vector<int> q_lp(static_cast<size_t>(std::max<Index>(1, p.M)), 0);
    for (Index q = 0; q < p.M; ++q)
        q_lp[q] = static_cast<int>(std::upper_bound(p.row_off.begin(), p.row_off.end(), p.perm[q]) -
                                   p.row_off.begin()) - 1;
    // front-zeroing chunks (front, start, length), kZeroChunk entries at most
    std::vector<int> zc_sn, zc_len;
    std::vector<int64_t> zc_off;
    for (int s = 0; s < p.ns; ++s) {
        const int64_t size = static_cast<int64_t>(p.sn_lda[s]) * p.sn_nrows[s];
        for (int64_t o = 0; o < size; o += kZeroChunk) {
            zc_sn.push_back(s);
            zc_off.push_back(p.sn_F_off[s] + o);
            zc_len.push_back(static_cast<int>(std::min<int64_t>(kZeroChunk, size - o)));
        }
    }
    nzc_ = static_cast<int64_t>(zc_sn.size());
    if (zc_sn.empty()) { zc_sn.push_back(0); zc_off.push_back(0); zc_len.push_back(0); }
    auto rsv = [&](auto& slot, const auto& vec) { reserve(arena_, slot, vec.size()); };
    rsv(sn_first_, p.sn_first); rsv(sn_ncols_, p.sn_ncols); rsv(sn_nrows_, p.sn_nrows); rsv(sn_lda_, p.sn_lda); rsv(sn_parent_, p.sn_parent);
    rsv(rows_, p.rows); rsv(ea_map_, p.ea_map); rsv(ch_ptr_, p.ch_ptr); rsv(ch_list_, p.ch_list);
    rsv(perm_, p.perm); rsv(sn_F_off_, p.sn_F_off); rsv(sn_f_off_, p.sn_f_off); rsv(sn_rows_off_, p.sn_rows_off);
    rsv(ea_off_, p.ea_off); rsv(step_items_, p.step_items); rsv(step_prefix_, p.step_prefix);
    rsv(round_items_, p.round_items); rsv(round_prefix_, p.round_prefix); rsv(level_sn_, p.level_sn);
    rsv(slot_pos_, p.slot_pos); rsv(w_ptr_, p.w_ptr); rsv(slot_i_, p.slot_i); rsv(slot_j_, p.slot_j);
    rsv(w_col_, p.w_col); rsv(w_val_, p.w_val); rsv(inv_off_, inv_off); rsv(blk_off_, blk_off);
    rsv(fwd_tasks_, ftask); rsv(bwd_tasks_, btask);
    rsv(g_dst_, g_dst); rsv(g_zp_, g_zp); rsv(g_ptr_, g_ptr); rsv(g_src_, g_src);
    rsv(sn_lp_, sn_lp); rsv(on32_, on32_h_); rsv(on64_, on64_h_); rsv(q_lp_, q_lp);
    rsv(zc_sn_, zc_sn); rsv(zc_len_, zc_len); rsv(zc_off_, zc_off);
    reserve(arena_, flags_, static_cast<size_t>(std::max(1, nflags_)));
    reserve(arena_, counters_, static_cast<size_t>(2 * std::max(1, p.nlevels)));
    reserve(arena_, solve_err_, 1);
    reserve(arena_, D_, static_cast<size_t>(p.M));
    reserve(arena_, Mdiag_, static_cast<size_t>(p.M));
    reserve(arena_, zp_, static_cast<size_t>(p.M));
    reserve(arena_, xp_, static_cast<size_t>(p.M));
    reserve(arena_, zsol_, static_cast<size_t>(p.M));
    reserve(arena_, fvec_, static_cast<size_t>(p.f_size));
    reserve(arena_, tn_, static_cast<size_t>(std::max(1, p.N)));
    reserve(arena_, params_, 4);
    reserve(arena_, err_, 4);
    reserve(arena_, oz_cnt_, std::max<size_t>(1, p.sn_ncols.size()));
    reserve(arena_, lp_fail_, std::max<size_t>(1, static_cast<size_t>(p.nlp)));
    for (auto& sb : sub_) {
        reserve(arena_, sb.d_items, std::max<size_t>(1, p.step_items.size()));
        reserve(arena_, sb.d_prefix, std::max<size_t>(1, p.step_prefix.size()));
    }
    arena_.commit();
    auto bnd = [&](auto& slot) { bind(arena_, slot); };
    bnd(sn_first_); bnd(sn_ncols_); bnd(sn_nrows_); bnd(sn_lda_); bnd(sn_parent_); bnd(rows_); bnd(ea_map_); bnd(ch_ptr_);
    bnd(ch_list_); bnd(perm_); bnd(sn_F_off_); bnd(sn_f_off_); bnd(sn_rows_off_); bnd(ea_off_); bnd(step_items_);
    bnd(step_prefix_); bnd(round_items_); bnd(round_prefix_); bnd(level_sn_); bnd(slot_pos_); bnd(w_ptr_);
    bnd(slot_i_); bnd(slot_j_); bnd(w_col_); bnd(w_val_); bnd(inv_off_); bnd(blk_off_); bnd(fwd_tasks_);
    bnd(bwd_tasks_); bnd(g_dst_); bnd(g_zp_); bnd(g_ptr_); bnd(g_src_); bnd(sn_lp_); bnd(on32_); bnd(on64_); bnd(q_lp_); bnd(zc_sn_); bnd(zc_len_); bnd(zc_off_); bnd(flags_); bnd(counters_); bnd(solve_err_); bnd(D_); bnd(Mdiag_);
    bnd(zp_); bnd(xp_); bnd(zsol_); bnd(fvec_); bnd(tn_); bnd(params_); bnd(err_); bnd(lp_fail_); bnd(oz_cnt_);
    for (auto& sb : sub_) { bnd(sb.d_items); bnd(sb.d_prefix); }
    upload(sn_first_, p.sn_first, st_); upload(sn_ncols_, p.sn_ncols, st_); upload(sn_nrows_, p.sn_nrows, st_);
    upload(sn_lda_, p.sn_lda, st_);
    upload(sn_parent_, p.sn_parent, st_); upload(rows_, p.rows, st_); upload(ea_map_, p.ea_map, st_);
    upload(ch_ptr_, p.ch_ptr, st_); upload(ch_list_, p.ch_list, st_); upload(perm_, p.perm, st_);
    upload(sn_F_off_, p.sn_F_off, st_); upload(sn_f_off_, p.sn_f_off, st_); upload(sn_rows_off_, p.sn_rows_off, st_);
    upload(ea_off_, p.ea_off, st_); upload(step_items_, p.step_items, st_); upload(step_prefix_, p.step_prefix, st_);
    upload(round_items_, p.round_items, st_); upload(round_prefix_, p.round_prefix, st_);
    upload(level_sn_, p.level_sn, st_); upload(slot_pos_, p.slot_pos, st_); upload(w_ptr_, p.w_ptr, st_);
    upload(slot_i_, p.slot_i, st_); upload(slot_j_, p.slot_j, st_); upload(w_col_, p.w_col, st_);
    upload(w_val_, p.w_val, st_); upload(inv_off_, inv_off, st_); upload(blk_off_, blk_off, st_);
    upload(fwd_tasks_, ftask, st_); upload(bwd_tasks_, btask, st_);
    upload(g_dst_, g_dst, st_); upload(g_zp_, g_zp, st_); upload(g_ptr_, g_ptr, st_); upload(g_src_, g_src, st_);
    upload(sn_lp_, sn_lp, st_); upload(on32_, on32_h_, st_); upload(on64_, on64_h_, st_); upload(q_lp_, q_lp, st_);
    upload(zc_sn_, zc_sn, st_); upload(zc_len_, zc_len, st_); upload(zc_off_, zc_off, st_);
    SK_CUDA(cudaMemsetAsync(solve_err_.ptr, 0, sizeof(int), st_));
    SK_CUDA(cudaStreamSynchronize(st_));
    set_smem_attrs<float>();
    set_smem_attrs<double>();
    // per LP: the update blocks (plus the panel tiles) of one factorisation
    lp_work_.assign(sn_lp.empty() ? 0 : static_cast<size_t>(*std::max_element(sn_lp.begin(), sn_lp.end())) + 1, 0.0);
    for (const auto& st : p.steps)
        for (int i = 0; i < st.nitems; ++i) {
            const int s = p.step_items[st.item_off + i];
            const double w = p.step_prefix[st.upd3_prefix_off + i + 1] - p.step_prefix[st.upd3_prefix_off + i] +
                             p.step_prefix[st.trsm_prefix_off + i + 1] - p.step_prefix[st.trsm_prefix_off + i] + 1;
            lp_work_[sn_lp[s]] += w;
            total_work_ += w;
        }
}

KktEngine::~KktEngine() {
    for (int q = 0; q < 2; ++q)
        if (fev_[q]) cudaEventDestroy(fev_[q]);
    for (int q = 0; q < 4; ++q)
        if (gfac_[q]) cudaGraphExecDestroy(gfac_[q]);
    for (int q = 0; q < 2; ++q)
        if (gsol_[q]) cudaGraphExecDestroy(gsol_[q]);
}

PlanDev KktEngine::pd(bool fp32) const {
    return PlanDev{sn_first_.ptr, sn_ncols_.ptr, sn_nrows_.ptr, sn_lda_.ptr, sn_F_off_.ptr, sn_f_off_.ptr, sn_rows_off_.ptr,
                   rows_.ptr, ea_off_.ptr, ea_map_.ptr, ch_ptr_.ptr, ch_list_.ptr, sn_parent_.ptr, sn_lp_.ptr,
                   fp32 ? on32_.ptr : on64_.ptr, lp_fail_.ptr};
}

template <class T>
void KktEngine::launch_factor(T* F, T* Linv, Prof* prof, const SubSteps* sub) {
    auto run = [&](int cls, auto&& f) {
        if (prof) prof->timed(cls, f); else f();
    };
    const auto& p = plan_;
    const PlanDev pdv = pd(std::is_same<T, float>::value);
    if (nzc_ > 0)
        k_zero_fronts<T><<<static_cast<int>(nzc_), 256, 0, st_>>>(zc_sn_.ptr, zc_len_.ptr, zc_off_.ptr, pdv, F);
    SK_CUDA(cudaMemsetAsync(err_.ptr, 0, 4 * sizeof(int), st_));
    SK_CUDA(cudaMemsetAsync(lp_fail_.ptr, 0, lp_fail_.count * sizeof(int), st_));
    if (emulate64_ && std::is_same<T, double>::value)   // blocks of the first update tile that have finished
        SK_CUDA(cudaMemsetAsync(oz_cnt_.ptr, 0, oz_cnt_.count * sizeof(int), st_));
    const double* theta = theta_bound_;
    run(0, [&] {
        if (p.dense_mode) {
            launch_diag<DiagDense>(p.M, lp_.spmv_group_A, st_, lp_.a_rp, lp_.a_ci, lp_.a_v, theta, Mdiag_.ptr,
                                   D_.ptr);
            k_asm_cols_dense<T><<<blocks_for(static_cast<int64_t>(p.M) * 32, 256), 256, 0, st_>>>(
                p.M, lp_.a_rp, lp_.a_ci, lp_.a_v, lp_.t_rp, lp_.t_ci, lp_.t_v, theta, Mdiag_.ptr, D_.ptr, lp_.row_lp,
                pdv, params_.ptr, F);
        } else {
            launch_diag<DiagSparse>(p.M, lp_.spmv_group_A, st_, w_ptr_.ptr, w_col_.ptr, w_val_.ptr, theta,
                                    Mdiag_.ptr, D_.ptr);
            k_asm_slots_sparse<T><<<blocks_for(p.nslots, 256), 256, 0, st_>>>(
                p.nslots, p.M, w_ptr_.ptr, w_col_.ptr, w_val_.ptr, theta, slot_i_.ptr, slot_j_.ptr, slot_pos_.ptr,
                Mdiag_.ptr, D_.ptr, params_.ptr, q_lp_.ptr, pdv.lp_on, F);
        }
    });
    const std::vector<ipm::PlanStep>& steps = sub ? sub->rs.steps : p.steps;
    const std::vector<int>& level_ptr = sub ? sub->rs.level_ptr : p.step_level_ptr;
    const int* items = sub ? sub->d_items.ptr : step_items_.ptr;
    const int* prefix = sub ? sub->d_prefix.ptr : step_prefix_.ptr;
    for (int l = 0; l < p.nlevels; ++l) {
        for (int q = level_ptr[l]; q < level_ptr[l + 1]; ++q) {
            const auto& st = steps[q];
            StepArgs a{st.k,           st.item_off,         st.nitems,           st.trsm_prefix_off,
                       st.upd_prefix_off, st.upd2_prefix_off, st.upd3_prefix_off, st.digit_row_off};
            if (st.k == 0)   // later diagonal tiles are factored by the previous step's update
                run(1, [&] {
                    k_potrf<T><<<st.nitems, 256, potrf_smem(sizeof(T)), st_>>>(a, items, pdv, F, Linv,
                                                                               inv_off_.ptr, err_.ptr);
                });
            if (st.trsm_tiles > 0)
                run(2, [&] {
                    bool oz = false;
                    if constexpr (std::is_same<T, double>::value) {
                        if (emulate64_) {   // FP64-accurate panel solve on the tensor cores
                            oz = true;
                            const int64_t plane = plan_.max_digit_rows * 128, lplane = max_step_items_ * T64 * 128;
                            k_oz_digits<<<static_cast<int>(st.trsm_tiles), 256, 0, st_>>>(
                                a, items, prefix, pdv, F, dig_.ptr, dexp_.ptr, plane);
                            k_oz_linv_digits<<<st.nitems, 256, 0, st_>>>(a, items, pdv, Linv, inv_off_.ptr,
                                                                         ldig_.ptr, lexp_.ptr, lplane);
                            k_trsm_oz<<<static_cast<int>(st.digit_rows / 128) * 2, 256, kOzSmemU, st_>>>(
                                a, items, prefix, pdv, F, dig_.ptr, dexp_.ptr, plane, ldig_.ptr,
                                lexp_.ptr, lplane, err_.ptr);
                        }
                    }
                    if (!oz)
                        k_trsm<T><<<static_cast<int>(st.trsm_tiles), 256, 2 * T64 * T64 * sizeof(T), st_>>>(
                            a, items, prefix, pdv, F, Linv, inv_off_.ptr);
                });
            if (st.upd_tiles > 0) {
                run(3, [&] {
                    bool tc = false;
                    if constexpr (std::is_same<T, float>::value) {
                        if (tensor_) {
                            tc = true;
                            const int64_t plane = plan_.max_digit_rows * 256;
                            k_tc_split<<<static_cast<int>(st.trsm_tiles), 256, 0, st_>>>(
                                a, items, prefix, pdv, F, dig_.ptr, plane);
                            k_update_tcs<<<static_cast<int>(st.upd3_blocks), 256, kTsSmem, st_>>>(
                                a, items, prefix, pdv, F, Linv, inv_off_.ptr, dig_.ptr, plane,
                                err_.ptr);
                        }
                    } else {
                        if (emulate64_) {
                            tc = true;
                            const int64_t plane = plan_.max_digit_rows * 128;
                            k_oz_digits<<<static_cast<int>(st.trsm_tiles), 256, 0, st_>>>(
                                a, items, prefix, pdv, F, dig_.ptr, dexp_.ptr, plane);
                            k_update_oz<<<static_cast<int>(st.upd3_blocks) * 2, 256, kOzSmemU, st_>>>(
                                a, items, prefix, pdv, F, Linv, inv_off_.ptr, dig_.ptr,
                                dexp_.ptr, plane, oz_cnt_.ptr, err_.ptr);
                        }
                    }
                    if (!tc)
                        k_update<T><<<static_cast<int>(st.upd_tiles), 256, potrf_smem(sizeof(T)), st_>>>(
                            a, items, prefix, pdv, F, Linv, inv_off_.ptr, err_.ptr);
                });
                if (prof) {
                    for (int it = 0; it < st.nitems; ++it) {
                        const int s2 = (sub ? sub->rs.items : p.step_items)[st.item_off + it];
                        const double w = std::min<int64_t>(T64, p.sn_ncols[s2] - static_cast<int64_t>(st.k) * T64);
                        const double t = p.sn_nrows[s2] - static_cast<double>(st.k) * T64 - w;
                        prof->upd_flops += 2.0 * w * t * (t + 1.0) / 2.0;
                        prof->upd_bytes += sizeof(T) * (t * w + 2.0 * t * (t + 1.0) / 2.0);
                    }
                    // per 128 x 64 block of the lower part, K padded to 64: TF32 x3 runs
                    // three products, the emulated FP64 update 28 BF16 digit-pair products
                    const double blk = 2.0 * 128 * 64 * 64 * static_cast<double>(st.upd3_blocks);
                    if (std::is_same<T, float>::value && tensor_) prof->mma_flops += 3.0 * blk;
                    if (std::is_same<T, double>::value && emulate64_) prof->mma_flops += 28.0 * blk;
                }
            }
        }
        for (int q = p.round_level_ptr[l]; q < p.round_level_ptr[l + 1]; ++q) {
            const auto& rd = p.rounds[q];
            run(4, [&] {
                k_extend_add<T><<<static_cast<int>(rd.tiles), dim3(32, 8), 0, st_>>>(
                    rd.item_off, rd.nitems, rd.prefix_off, round_items_.ptr, round_prefix_.ptr, pdv, F);
            });
        }
    }
    SK_CUDA(cudaGetLastError());
}

template <class T>
void KktEngine::launch_solve(const T* F, const T* Linv, Prof* prof) {
    auto run = [&](int cls, auto&& f) {
        if (prof) prof->timed(cls, f); else f();
    };
    const auto& p = plan_;
    const PlanDev pdv = pd(std::is_same<T, float>::value);
    T* zp = reinterpret_cast<T*>(zp_.ptr);
    T* xp = reinterpret_cast<T*>(xp_.ptr);
    T* zs = reinterpret_cast<T*>(zsol_.ptr);
    T* fv = reinterpret_cast<T*>(fvec_.ptr);
    SK_CUDA(cudaMemsetAsync(flags_.ptr, 0, sizeof(int) * static_cast<size_t>(std::max(1, nflags_)), st_));
    SK_CUDA(cudaMemsetAsync(counters_.ptr, 0, sizeof(int) * 2 * static_cast<size_t>(std::max(1, p.nlevels)), st_));
    for (int l = 0; l < p.nlevels; ++l) {
        const int nt = fwd_task_off_[l + 1] - fwd_task_off_[l];
        const int g0 = gather_off_[l], ng = gather_off_[l + 1] - g0;
        run(5, [&] {
            if (ng > 0)
                k_fwd_gather<T><<<blocks_for(ng, 256), 256, 0, st_>>>(ng, g_dst_.ptr + g0, g_zp_.ptr + g0,
                                                                      g_ptr_.ptr + g0, g_src_.ptr, zp, fv);
            k_fwd_tasks<T><<<nt, 256, 0, st_>>>(fwd_tasks_.ptr + fwd_task_off_[l], nt, counters_.ptr + l, pdv, F,
                                                Linv, inv_off_.ptr, blk_off_.ptr, flags_.ptr, fv, zs,
                                                solve_err_.ptr);
        });
    }
    for (int l = p.nlevels - 1; l >= 0; --l) {
        const int nt = bwd_task_off_[l + 1] - bwd_task_off_[l];
        run(6, [&] {
            k_bwd_tasks<T><<<nt, 256, 0, st_>>>(bwd_tasks_.ptr + bwd_task_off_[l], nt, counters_.ptr + p.nlevels + l,
                                                pdv, F, Linv, inv_off_.ptr, blk_off_.ptr, flags_.ptr, xp, zs,
                                                solve_err_.ptr);
        });
    }
    SK_CUDA(cudaGetLastError());
}

int KktEngine::solve_error() {
    int h = 0;
    SK_CUDA(cudaMemcpyAsync(&h, solve_err_.ptr, sizeof(int), cudaMemcpyDeviceToHost, st_));
    SK_CUDA(cudaStreamSynchronize(st_));
    return h;
}

void KktEngine::ensure_fronts(bool fp32) {
    if (fp32 && !F32_.ptr) {
        f32_arena_.reset();
        reserve(f32_arena_, F32_, static_cast<size_t>(plan_.F_size));
        reserve(f32_arena_, Linv32_, static_cast<size_t>(std::max<int64_t>(1, inv_size_)));
        f32_arena_.commit();
        bind(f32_arena_, F32_);
        bind(f32_arena_, Linv32_);
    }
    if (!fp32 && !F64_.ptr) {
        f64_arena_.reset();
        reserve(f64_arena_, F64_, static_cast<size_t>(plan_.F_size));
        reserve(f64_arena_, Linv64_, static_cast<size_t>(std::max<int64_t>(1, inv_size_)));
        f64_arena_.commit();
        bind(f64_arena_, F64_);
        bind(f64_arena_, Linv64_);
    }
}

void KktEngine::ensure_digits() {
    if (dig_.ptr || plan_.max_digit_rows <= 0) return;
    max_step_items_ = 1;
    for (const auto& st : plan_.steps) max_step_items_ = std::max(max_step_items_, static_cast<int64_t>(st.nitems));
    dig_arena_.reset();
    reserve(dig_arena_, dig_, static_cast<size_t>(kOzDigits) * static_cast<size_t>(plan_.max_digit_rows) * 128);
    reserve(dig_arena_, dexp_, static_cast<size_t>(plan_.max_digit_rows));
    reserve(dig_arena_, ldig_, static_cast<size_t>(kOzDigits) * static_cast<size_t>(max_step_items_) * T64 * 128);
    reserve(dig_arena_, lexp_, static_cast<size_t>(max_step_items_) * T64);
    dig_arena_.commit();
    bind(dig_arena_, dig_);
    bind(dig_arena_, dexp_);
    bind(dig_arena_, ldig_);
    bind(dig_arena_, lexp_);
}

// The step lists for a factorisation of the LPs of this precision's mask: the
// plan's own (and its captured graph) while the LPs that are on hold at least 3/4
// of the batch's update blocks, else lists restricted to them (rebuilt and
// uploaded when the mask has changed since the last call).
const KktEngine::SubSteps* KktEngine::pick_steps(bool fp32) {
    const std::vector<int>& mask = fp32 ? on32_h_ : on64_h_;
    double on_work = 0.0;
    for (size_t k = 0; k < mask.size() && k < lp_work_.size(); ++k)
        if (mask[k]) on_work += lp_work_[k];
    if (on_work >= 0.75 * total_work_) return nullptr;
    SubSteps& sb = sub_[fp32 ? 0 : 1];
    if (sb.mask == mask && !sb.rs.level_ptr.empty()) return &sb;
    sb.mask = mask;
    ipm::restrict_steps(plan_, sn_lp_h_, mask, sb.rs);
    if (!sb.rs.items.empty())
        SK_CUDA(cudaMemcpyAsync(sb.d_items.ptr, sb.rs.items.data(), sizeof(int) * sb.rs.items.size(),
                                cudaMemcpyHostToDevice, st_));
    if (!sb.rs.prefix.empty())
        SK_CUDA(cudaMemcpyAsync(sb.d_prefix.ptr, sb.rs.prefix.data(), sizeof(int) * sb.rs.prefix.size(),
                                cudaMemcpyHostToDevice, st_));
    return &sb;
}

bool KktEngine::factor(const double* d_theta, double delta, bool fp32) {
    const int q = fp32 ? (tensor_ ? 2 : 1) : (emulate64_ ? 3 : 0);
    ensure_fronts(fp32);
    if ((!fp32 && emulate64_) || (fp32 && tensor_)) ensure_digits();
    fp32_ = fp32;
    double hp[4] = {delta, 0, 0, 0};
    SK_CUDA(cudaMemcpyAsync(params_.ptr, hp, sizeof(hp), cudaMemcpyHostToDevice, st_));
    if (!fev_[0]) {
        SK_CUDA(cudaEventCreate(&fev_[0]));
        SK_CUDA(cudaEventCreate(&fev_[1]));
    }
    const SubSteps* sub = pick_steps(fp32);
    if (sub) {   // a few LPs of the batch: their blocks only, launched directly
        theta_bound_ = d_theta;
        SK_CUDA(cudaEventRecord(fev_[0], st_));
        if (fp32) launch_factor<float>(F32_.ptr, Linv32_.ptr, nullptr, sub);
        else launch_factor<double>(F64_.ptr, Linv64_.ptr, nullptr, sub);
        SK_CUDA(cudaEventRecord(fev_[1], st_));
    } else {
        if (!gfac_[q] || gfac_theta_[q] != d_theta) {
            if (gfac_[q]) { cudaGraphExecDestroy(gfac_[q]); gfac_[q] = nullptr; }
            theta_bound_ = d_theta;
            cudaGraph_t g;
            SK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
            if (fp32) launch_factor<float>(F32_.ptr, Linv32_.ptr); else launch_factor<double>(F64_.ptr, Linv64_.ptr);
            SK_CUDA(cudaStreamEndCapture(st_, &g));
            SK_CUDA(cudaGraphInstantiate(&gfac_[q], g, 0));
            cudaGraphDestroy(g);
            gfac_theta_[q] = d_theta;
        }
        SK_CUDA(cudaEventRecord(fev_[0], st_));
        SK_CUDA(cudaGraphLaunch(gfac_[q], st_));
        SK_CUDA(cudaEventRecord(fev_[1], st_));
    }
    int herr[3];
    SK_CUDA(cudaMemcpyAsync(herr, err_.ptr, sizeof(herr), cudaMemcpyDeviceToHost, st_));
    SK_CUDA(cudaStreamSynchronize(st_));
    float fms = 0.f;
    SK_CUDA(cudaEventElapsedTime(&fms, fev_[0], fev_[1]));
    fact_ms_[fp32 ? 0 : 1] += fms;
    if (herr[2]) throw std::runtime_error("tensor-core update: a copy or an MMA did not complete in time");
    failed_sn_ = herr[0] ? herr[1] : -1;
    failed_lps_.clear();
    if (herr[0]) {
        std::vector<int> f(lp_fail_.count, 0);
        SK_CUDA(cudaMemcpy(f.data(), lp_fail_.ptr, sizeof(int) * f.size(), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < f.size(); ++k)
            if (f[k]) failed_lps_.push_back(static_cast<int>(k));
    }
    return herr[0] == 0;
}

// One precision's solve: permute and scale src, the level-scheduled triangular
// solves of that precision's fronts (graph `graph`), unscale and unpermute into
// dst. Rows of LPs in `other` keep their dst values (see k_unpermute_scale).
template <class T>
void KktEngine::solve_pass(const T* F, const T* Linv, const int* mask, bool keep, const double* d_src,
                           double* d_dst, int graph) {
    const auto& p = plan_;
    k_permute_scale<T><<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, perm_.ptr, D_.ptr, d_src,
                                                              reinterpret_cast<T*>(zp_.ptr));
    if (!gsol_[graph]) {
        cudaGraph_t g;
        SK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        launch_solve<T>(F, Linv);
        SK_CUDA(cudaStreamEndCapture(st_, &g));
        SK_CUDA(cudaGraphInstantiate(&gsol_[graph], g, 0));
        cudaGraphDestroy(g);
    }
    SK_CUDA(cudaGraphLaunch(gsol_[graph], st_));
    const int* other = keep ? (std::is_same<T, float>::value ? on64_.ptr : on32_.ptr) : nullptr;
    k_unpermute_scale<T><<<blocks_for(p.M, 256), 256, 0, st_>>>(
        p.M, perm_.ptr, D_.ptr, reinterpret_cast<const T*>(xp_.ptr), lp_.row_lp, mask, other, d_dst);
    SK_CUDA(cudaGetLastError());
}

void KktEngine::apply_inverse(const double* d_src, double* d_dst) {
    if (!mixed_) {
        if (fp32_) solve_pass<float>(F32_.ptr, Linv32_.ptr, on32_.ptr, false, d_src, d_dst, 1);
        else solve_pass<double>(F64_.ptr, Linv64_.ptr, on64_.ptr, false, d_src, d_dst, 0);
        return;
    }
    bool any32 = false, any64 = false;
    for (size_t k = 0; k < on32_h_.size(); ++k) { any32 |= on32_h_[k] != 0; any64 |= on64_h_[k] != 0; }
    // The FP32 pass writes only the rows of on32 (and zeroes the inactive ones); the FP64
    // pass then reads the rows of on64 from src, which the first pass left alone, so src
    // and dst may still alias.
    if (!any32 && !any64) {          // no LP left: every row is 0
        SK_CUDA(cudaMemsetAsync(d_dst, 0, sizeof(double) * static_cast<size_t>(plan_.M), st_));
        return;
    }
    if (any32) {
        ensure_fronts(true);
        solve_pass<float>(F32_.ptr, Linv32_.ptr, on32_.ptr, true, d_src, d_dst, 1);
    }
    if (any64) {
        ensure_fronts(false);
        solve_pass<double>(F64_.ptr, Linv64_.ptr, on64_.ptr, true, d_src, d_dst, 0);
    }
}

void KktEngine::upload_mask(Slot<int>& dev, std::vector<int>& host, const std::vector<char>& on) {
    if (on.size() != host.size()) throw std::invalid_argument("set_active: one flag per LP");
    bool same = true;
    for (size_t k = 0; same && k < on.size(); ++k) same = (on[k] != 0) == (host[k] != 0);
    if (same) return;
    for (size_t k = 0; k < on.size(); ++k) host[k] = on[k] ? 1 : 0;
    SK_CUDA(cudaMemcpyAsync(dev.ptr, host.data(), sizeof(int) * host.size(), cudaMemcpyHostToDevice, st_));
}

void KktEngine::set_active(const std::vector<char>& on) {
    restricted_ = false;
    mixed_ = false;
    upload_mask(on32_, on32_h_, on);
    upload_mask(on64_, on64_h_, on);
}

void KktEngine::set_masks(const std::vector<char>& on32, const std::vector<char>& on64) {
    for (size_t k = 0; k < on32.size() && k < on64.size(); ++k)
        if (on32[k] && on64[k]) throw std::invalid_argument("set_masks: an LP in both precisions");
    restricted_ = false;
    mixed_ = true;
    upload_mask(on32_, on32_h_, on32);
    upload_mask(on64_, on64_h_, on64);
}

void KktEngine::restrict_solves(const std::vector<char>& sub) {
    if (!restricted_) {
        full32_h_ = on32_h_;
        full64_h_ = on64_h_;
        restricted_ = true;
    }
    if (sub.size() != full32_h_.size()) throw std::invalid_argument("restrict_solves: one flag per LP");
    std::vector<char> a(sub.size()), b(sub.size());
    for (size_t k = 0; k < sub.size(); ++k) {
        a[k] = full32_h_[k] && sub[k];
        b[k] = full64_h_[k] && sub[k];
    }
    upload_mask(on32_, on32_h_, a);
    upload_mask(on64_, on64_h_, b);
}

void KktEngine::unrestrict_solves() {
    if (!restricted_) return;
    restricted_ = false;
    const std::vector<char> a(full32_h_.begin(), full32_h_.end()), b(full64_h_.begin(), full64_h_.end());
    upload_mask(on32_, on32_h_, a);
    upload_mask(on64_, on64_h_, b);
}

int KktEngine::failed_lp() const {
    return failed_sn_ >= 0 && failed_sn_ < static_cast<int>(sn_lp_h_.size()) ? sn_lp_h_[failed_sn_] : -1;
}

void KktEngine::apply_normal(const double* d_theta, const double* d_src, double* d_dst) {
    // t = theta .* (A^T src); dst = A t
    k_spmv_rows<<<blocks_for(lp_.N, 256), 256, 0, st_>>>(lp_.N, lp_.t_rp, lp_.t_ci, lp_.t_v, d_src, d_theta, tn_.ptr);
    k_spmv_rows<<<blocks_for(lp_.M, 256), 256, 0, st_>>>(lp_.M, lp_.a_rp, lp_.a_ci, lp_.a_v, tn_.ptr, nullptr, d_dst);
    SK_CUDA(cudaGetLastError());
}

void KktEngine::profile(const double* d_theta, double delta, bool fp32, const double* d_rhs, double* d_out,
                        double* out) {
    factor(d_theta, delta, fp32);   // allocates the fronts and sets D
    Prof pr;
    pr.st = st_;
    double hp[4] = {delta, 0, 0, 0};
    SK_CUDA(cudaMemcpyAsync(params_.ptr, hp, sizeof(hp), cudaMemcpyHostToDevice, st_));
    theta_bound_ = d_theta;
    if (fp32) launch_factor<float>(F32_.ptr, Linv32_.ptr, &pr);
    else launch_factor<double>(F64_.ptr, Linv64_.ptr, &pr);
    if (fp32) {
        k_permute_scale<float><<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, d_rhs,
                                                                          reinterpret_cast<float*>(zp_.ptr));
        launch_solve<float>(F32_.ptr, Linv32_.ptr, &pr);
        k_unpermute_scale<float><<<blocks_for(plan_.M, 256), 256, 0, st_>>>(
            plan_.M, perm_.ptr, D_.ptr, reinterpret_cast<const float*>(xp_.ptr), lp_.row_lp, on32_.ptr, nullptr,
            d_out);
    } else {
        k_permute_scale<double><<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, d_rhs, zp_.ptr);
        launch_solve<double>(F64_.ptr, Linv64_.ptr, &pr);
        k_unpermute_scale<double><<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, xp_.ptr,
                                                                             lp_.row_lp, on64_.ptr, nullptr, d_out);
    }
    SK_CUDA(cudaStreamSynchronize(st_));
    for (int q = 0; q < 16; ++q) out[q] = 0.0;
    for (auto& e : pr.ev) {
        float ms = 0.f;
        SK_CUDA(cudaEventElapsedTime(&ms, e.second.first, e.second.second));
        out[2 * e.first] += ms;
        out[2 * e.first + 1] += 1.0;
        cudaEventDestroy(e.second.first);
        cudaEventDestroy(e.second.second);
    }
    out[14] = pr.upd_flops;
    out[15] = pr.upd_bytes;
    out[16] = assembly_bytes(fp32 ? sizeof(float) : sizeof(double));
    out[17] = pr.mma_flops;
}

double KktEngine::assembly_bytes(size_t elem) const {
    const auto& p = plan_;
    const double M = p.M, N = p.N;
    const double diag_out = 16.0 * M;               // Mdiag and D
    if (p.dense_mode) {
        // A as CSR for the diagonal and as CSR + CSC for the columns (12 bytes per entry
        // and 4 per pointer each), Theta, and the lower triangle of every front written once
        double tri = 0.0;
        for (int s = 0; s < p.ns; ++s) tri += 0.5 * double(p.sn_nrows[s]) * (p.sn_nrows[s] + 1.0);
        return 3.0 * 12.0 * lp_.nnz + 8.0 * (M + 1) + 4.0 * (N + 1) + 8.0 * N + diag_out + elem * tri;
    }
    // Khatri-Rao map: 12 bytes per entry, 8 per row pointer; per off-diagonal slot its
    // two row indices (8), front position (8) and the front entry written; Theta once
    const double w = static_cast<double>(p.w_ptr.empty() ? 0 : p.w_ptr.back());
    const double offd = static_cast<double>(p.nslots) - M;
    return 12.0 * w + 8.0 * (p.nslots + 1.0) + 8.0 * N + diag_out + (16.0 + elem) * offd + elem * M;
}

namespace {
// L's diagonal entries of every front (one block per front, a thread per own column).
__global__ void k_pivots(const int* __restrict__ sn_first, const int* __restrict__ sn_ncols,
                         const int* __restrict__ sn_lda, const int64_t* __restrict__ F_off,
                         const double* __restrict__ F, double* __restrict__ out) {
    const int s = blockIdx.x;
    const int K = sn_ncols[s], LD = sn_lda[s], f = sn_first[s];
    for (int c = threadIdx.x; c < K; c += blockDim.x) out[f + c] = F[F_off[s] + c + static_cast<int64_t>(c) * LD];
}
}  // namespace

std::vector<double> KktEngine::pivots_host() {
    if (fp32_ || !F64_.ptr) throw std::logic_error("pivots_host: no FP64 factor");
    std::vector<double> out(static_cast<size_t>(plan_.M));
    Arena tmp;
    Slot<double> d;
    reserve(tmp, d, static_cast<size_t>(std::max<int64_t>(1, plan_.M)));
    tmp.commit();
    bind(tmp, d);
    if (plan_.ns > 0)
        k_pivots<<<plan_.ns, 128, 0, st_>>>(sn_first_.ptr, sn_ncols_.ptr, sn_lda_.ptr, sn_F_off_.ptr, F64_.ptr, d.ptr);
    SK_CUDA(cudaGetLastError());
    SK_CUDA(cudaMemcpyAsync(out.data(), d.ptr, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, st_));
    SK_CUDA(cudaStreamSynchronize(st_));
    return out;
}

std::vector<double> KktEngine::fronts_host() {
    std::vector<double> out(static_cast<size_t>(plan_.F_size));
    if (fp32_) {
        std::vector<float> tmp(out.size());
        SK_CUDA(cudaMemcpyAsync(tmp.data(), F32_.ptr, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost, st_));
        SK_CUDA(cudaStreamSynchronize(st_));
        for (size_t q = 0; q < out.size(); ++q) out[q] = tmp[q];
    } else {
        SK_CUDA(cudaMemcpyAsync(out.data(), F64_.ptr, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, st_));
        SK_CUDA(cudaStreamSynchronize(st_));
    }
    return out;
}

}  // namespace dev
}  // namespace sankhya

namespace sankhya {
namespace dev {

namespace {
__global__ void k_absmax_partial(int n, const double* __restrict__ a, double* __restrict__ part) {
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(a[i]));
    m = warp_max(m);
    __shared__ double sh[8];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) r = fmax(r, sh[w]);
        part[blockIdx.x] = r;
    }
}
__global__ void k_axpy_diff(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}
__global__ void k_add(int n, const double* __restrict__ a, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += a[i];
}
}  // namespace

double absmax_device(int n, const double* a, double* scratch64, cudaStream_t st) {
    k_absmax_partial<<<64, 256, 0, st>>>(n, a, scratch64);
    double h[64];
    SK_CUDA(cudaMemcpyAsync(h, scratch64, sizeof(h), cudaMemcpyDeviceToHost, st));
    SK_CUDA(cudaStreamSynchronize(st));
    double r = 0.0;
    for (double v : h) r = std::max(r, v);
    return r;
}

void vec_diff(int n, const double* a, const double* b, double* out, cudaStream_t st) {
    k_axpy_diff<<<(n + 255) / 256, 256, 0, st>>>(n, a, b, out);
    SK_CUDA(cudaGetLastError());
}

void vec_add(int n, const double* a, double* out, cudaStream_t st) {
    k_add<<<(n + 255) / 256, 256, 0, st>>>(n, a, out);
    SK_CUDA(cudaGetLastError());
}

}  // namespace dev
}  // namespace sankhya
