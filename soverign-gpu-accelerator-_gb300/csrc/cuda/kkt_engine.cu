// Device normal-equation engine (see kkt_engine.hpp).
//
// Kernels, in the order one factorisation + solve runs them:
//   assembly    k_asm_*          D (A Theta A^T) D + delta I into the fronts
//   factor      k_potrf          Cholesky of one 64x64 diagonal tile per front
//               k_trsm           panel rows below the tile: X L^T = B
//               k_update         trailing update C -= L_i L_j^T (tiles of 64x64)
//               k_extend_add     child update matrix into the parent front
//   solve       k_fwd_init / k_fwd_diag / k_fwd_gemv      L z = r, multifrontal
//               k_bwd_init / k_bwd_partial / k_bwd_diag   L^T x = z
// Every kernel's grid is a list of (front, tile) work items of one level / step,
// decoded with a binary search over a prefix of per-front tile counts.
#include "cuda/kkt_engine.hpp"

#include <algorithm>
#include <cmath>

namespace sankhya {
namespace dev {

struct PlanDev {
    const int* sn_first;
    const int* sn_ncols;
    const int* sn_nrows;
    const int64_t* F_off;
    const int64_t* f_off;
    const int64_t* rows_off;
    const int* rows;
    const int64_t* ea_off;
    const int* ea_map;
    const int* ch_ptr;
    const int* ch_list;
    const int* sn_parent;
};

namespace {

constexpr int T64 = ipm::kTile;   // 64
constexpr int LDS = T64 + 1;      // padded leading dimension of shared tiles

struct StepArgs {
    int k;
    int item_off;
    int nitems;
    int tp_off;   // trsm prefix offset
    int up_off;   // update prefix offset
};


__device__ __forceinline__ int find_item(const int* prefix, int n, int b) {
    int lo = 0, hi = n - 1;   // largest i with prefix[i] <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void tri_index(int lt, int& ti, int& tj) {
    int t = static_cast<int>((sqrt(8.0 * lt + 1.0) - 1.0) * 0.5);
    while ((t + 1) * (t + 2) / 2 <= lt) ++t;
    while (t * (t + 1) / 2 > lt) --t;
    ti = t;
    tj = lt - t * (t + 1) / 2;
}

// ------------------------------------------------------------------ assembly

__global__ void k_asm_diag_sparse(int M, const int64_t* __restrict__ w_ptr, const int* __restrict__ w_col,
                                  const double* __restrict__ w_val, const double* __restrict__ theta,
                                  double* __restrict__ Mdiag, double* __restrict__ D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    double acc = 0.0;
    for (int64_t t = w_ptr[i]; t < w_ptr[i + 1]; ++t) acc += w_val[t] * theta[w_col[t]];
    Mdiag[i] = acc;
    D[i] = 1.0 / sqrt(fmax(fabs(acc), 1e-12));
}

template <class T>
__global__ void k_asm_slots_sparse(int64_t nslots, int M, const int64_t* __restrict__ w_ptr,
                                   const int* __restrict__ w_col, const double* __restrict__ w_val,
                                   const double* __restrict__ theta, const int* __restrict__ si,
                                   const int* __restrict__ sj, const int64_t* __restrict__ pos,
                                   const double* __restrict__ Mdiag, const double* __restrict__ D,
                                   const double* __restrict__ params, T* __restrict__ F) {
    const int64_t s = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    double v;
    if (s < M) {
        v = Mdiag[s] * D[s] * D[s] + params[0];
    } else {
        double acc = 0.0;
        for (int64_t t = w_ptr[s]; t < w_ptr[s + 1]; ++t) acc += w_val[t] * theta[w_col[t]];
        v = acc * D[si[s]] * D[sj[s]];
    }
    F[pos[s]] = static_cast<T>(v);
}

__global__ void k_asm_diag_dense(int M, const int* __restrict__ rp, const int* __restrict__ ci,
                                 const double* __restrict__ av, const double* __restrict__ theta,
                                 double* __restrict__ Mdiag, double* __restrict__ D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M) return;
    double acc = 0.0;
    for (int q = rp[i]; q < rp[i + 1]; ++q) acc += av[q] * av[q] * theta[ci[q]];
    Mdiag[i] = acc;
    D[i] = 1.0 / sqrt(fmax(fabs(acc), 1e-12));
}

// One warp per column j of M (dense mode: one front per LP, natural order).
// Column j below the diagonal is sum_k a_jk theta_k A(:,k); the k loop is
// sequential so every entry is summed in a fixed order.
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
    const int first = pd.sn_first[s];
    const int N = pd.sn_nrows[s];
    T* col = F + pd.F_off[s] + static_cast<int64_t>(j - first) * N - first;
    const double dj = D[j];
    for (int q = rp[j]; q < rp[j + 1]; ++q) {
        const int k = ci[q];
        const double coef = av[q] * theta[k] * dj;
        for (int t = tp[k] + lane; t < tp[k + 1]; t += 32) {
            const int i = ti[t];
            if (i > j) col[i] = static_cast<T>(static_cast<double>(col[i]) + coef * tv[t] * D[i]);
        }
        __syncwarp();
    }
    if (lane == 0) col[j] = static_cast<T>(Mdiag[j] * dj * dj + params[0]);
}

// ------------------------------------------------------------------- factor

// Cholesky of the 64x64 diagonal tile of step k of one front, in the front's
// precision T, plus the explicit inverse of the factored tile (used by the panel
// solve and by both triangular solves), stored column-major in Linv. One warp:
// lane l owns rows l and l+32 during the factorisation and columns l and l+32 of
// the inverse, so no block-wide barrier is needed.
template <class T>
__global__ void __launch_bounds__(32) k_potrf(StepArgs a, const int* __restrict__ items, PlanDev pd, T* F,
                                              T* __restrict__ Linv, const int64_t* __restrict__ inv_off,
                                              int* err) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* A = reinterpret_cast<T*>(smraw);
    T* Iv = A + T64 * LDS;
    const int s = items[a.item_off + blockIdx.x];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    T* Fs = F + pd.F_off[s];
    const int lane = threadIdx.x;
    for (int c = 0; c < w; ++c)
        for (int r = lane; r < w; r += 32)
            A[r * LDS + c] = r >= c ? Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N] : T(0);
    __syncwarp();
    const int r0 = lane, r1 = lane + 32;
    for (int c = 0; c < w; ++c) {
        T piv = A[c * LDS + c];
        if (!(piv > T(0))) {
            if (lane == 0 && atomicCAS(err, 0, 1) == 0) err[1] = s;
            piv = T(1);
        }
        const T d = sqrt(piv);
        __syncwarp();
        if (r0 > c && r0 < w) A[r0 * LDS + c] /= d;
        if (r1 > c && r1 < w) A[r1 * LDS + c] /= d;
        if (lane == (c & 31)) A[c * LDS + c] = d;
        __syncwarp();
        const T l0 = (r0 > c && r0 < w) ? A[r0 * LDS + c] : T(0);
        const T l1 = (r1 > c && r1 < w) ? A[r1 * LDS + c] : T(0);
        for (int cc = c + 1; cc < w; ++cc) {
            const T lc = A[cc * LDS + c];
            if (r0 >= cc && r0 < w) A[r0 * LDS + cc] -= l0 * lc;
            if (r1 >= cc && r1 < w) A[r1 * LDS + cc] -= l1 * lc;
        }
        __syncwarp();
    }
    // inverse: lane owns columns j0 = lane, j1 = lane + 32 of X = L^{-1}
    for (int jj = 0; jj < 2; ++jj) {
        const int j = lane + 32 * jj;
        if (j >= w) continue;
        for (int i = j; i < w; ++i) {
            T acc = (i == j) ? T(1) : T(0);
            for (int q = j; q < i; ++q) acc -= A[i * LDS + q] * Iv[q * LDS + j];
            Iv[i * LDS + j] = acc / A[i * LDS + i];
        }
    }
    __syncwarp();
    T* Li = Linv + inv_off[s] + static_cast<int64_t>(a.k) * T64 * T64;
    for (int c = 0; c < T64; ++c)
        for (int r = lane; r < T64; r += 32) {
            const bool in = r < w && c < w && r >= c;
            if (in) Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N] = A[r * LDS + c];
            Li[r + c * T64] = in ? Iv[r * LDS + c] : T(0);
        }
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
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
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
        B[c * T64 + r] = (r < nr && c < w) ? Fs[(r0 + r) + static_cast<int64_t>(k0 + c) * N] : T(0);
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
            if (c < w) Fs[(r0 + r) + static_cast<int64_t>(k0 + c) * N] = acc[t];
        }
}

// C(64x64) -= A_i (64 x w) A_j^T; 256 threads, 4x4 outputs each.
template <class T>
__global__ void __launch_bounds__(256) k_update(StepArgs a, const int* __restrict__ items,
                                                const int* __restrict__ prefix, PlanDev pd, T* F) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* As = reinterpret_cast<T*>(smraw);     // [kk][r]
    T* Bs = As + T64 * T64;                  // [kk][c]
    const int i = find_item(prefix + a.up_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    const int lt = blockIdx.x - prefix[a.up_off + i];
    int ti, tj;
    tri_index(lt, ti, tj);
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int t0 = k0 + w;
    const int ri0 = t0 + ti * T64, cj0 = t0 + tj * T64;
    const int nri = min(T64, N - ri0), ncj = min(T64, N - cj0);
    T* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < T64 * T64; idx += blockDim.x) {
        const int r = idx & (T64 - 1), kk = idx >> 6;
        T va = T(0), vb = T(0);
        if (kk < w) {
            const int64_t cofs = static_cast<int64_t>(k0 + kk) * N;
            if (r < nri) va = Fs[ri0 + r + cofs];
            if (r < ncj) vb = Fs[cj0 + r + cofs];
        }
        As[kk * T64 + r] = va;
        Bs[kk * T64 + r] = vb;
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    T acc[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[q][p] = T(0);
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
    for (int p = 0; p < 4; ++p) {
        const int c = tx * 4 + p;
        if (c >= ncj) continue;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = ty * 4 + q;
            if (r >= nri) continue;
            if (ti == tj && r < c) continue;
            T* dst = Fs + (ri0 + r) + static_cast<int64_t>(cj0 + c) * N;
            *dst = *dst - acc[q][p];
        }
    }
}

template <class T>
__global__ void k_extend_add(int item_off, int nitems, int prefix_off, const int* __restrict__ items,
                             const int* __restrict__ prefix, PlanDev pd, T* F) {
    const int i = find_item(prefix + prefix_off, nitems, blockIdx.x);
    const int c = items[item_off + i];
    const int lt = blockIdx.x - prefix[prefix_off + i];
    int ti, tj;
    tri_index(lt, ti, tj);
    const int Kc = pd.sn_ncols[c], Nc = pd.sn_nrows[c];
    const int u = Nc - Kc;
    const int p = pd.sn_parent[c];
    const int Np = pd.sn_nrows[p];
    const T* Fc = F + pd.F_off[c];
    T* Fp = F + pd.F_off[p];
    const int* map = pd.ea_map + pd.ea_off[c];
    const int rr = ti * 32 + threadIdx.x;
    if (rr >= u) return;
    const int mr = map[rr];
    for (int cc = tj * 32 + threadIdx.y; cc < tj * 32 + 32 && cc < u; cc += blockDim.y) {
        if (rr < cc) continue;
        const T v = Fc[(Kc + rr) + static_cast<int64_t>(Kc + cc) * Nc];
        T* dst = Fp + mr + static_cast<int64_t>(map[cc]) * Np;
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

template <class T>
__global__ void k_unpermute_scale(int M, const int* __restrict__ perm, const double* __restrict__ D,
                                  const T* __restrict__ xp, double* __restrict__ dst) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < M) dst[perm[q]] = D[q] * static_cast<double>(xp[q]);
}

// Frontal right-hand side: own entries of the permuted rhs, then the children's
// update vectors added in a fixed order.
template <class T>
__global__ void k_fwd_init(const int* __restrict__ level_sn, PlanDev pd, const T* __restrict__ zp,
                           T* __restrict__ fv) {
    const int s = level_sn[blockIdx.x];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    T* f = fv + pd.f_off[s];
    for (int q = threadIdx.x; q < N; q += blockDim.x) f[q] = q < K ? zp[first + q] : T(0);
    __syncthreads();
    for (int e = pd.ch_ptr[s]; e < pd.ch_ptr[s + 1]; ++e) {
        const int c = pd.ch_list[e];
        const int Kc = pd.sn_ncols[c], u = pd.sn_nrows[c] - Kc;
        const T* uc = fv + pd.f_off[c] + Kc;
        const int* map = pd.ea_map + pd.ea_off[c];
        for (int t = threadIdx.x; t < u; t += blockDim.x) f[map[t]] += uc[t];
        __syncthreads();
    }
}

// Forward tile step: every block forms z = Linv f_blk; block 0 of a front stores
// z, the others subtract L(rows, blk) z from their 64 rows below the block.
template <class T>
__global__ void __launch_bounds__(256) k_fwd_step(StepArgs a, const int* __restrict__ items,
                                                  const int* __restrict__ prefix, PlanDev pd,
                                                  const T* __restrict__ F, const T* __restrict__ Linv,
                                                  const int64_t* __restrict__ inv_off, T* __restrict__ fv,
                                                  T* __restrict__ zsol) {
    __shared__ T fb[T64];
    __shared__ T z[T64];
    __shared__ T part[4][T64];
    // block b -> (item i, tile lt) with 1 + trsm tiles per item
    int lo = 0, hi = a.nitems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[a.tp_off + mid] + mid <= static_cast<int>(blockIdx.x)) lo = mid; else hi = mid - 1;
    }
    const int i = lo;
    const int lt = blockIdx.x - prefix[a.tp_off + i] - i;
    const int s = items[a.item_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const T* Fs = F + pd.F_off[s];
    const T* Li = Linv + inv_off[s] + static_cast<int64_t>(a.k) * T64 * T64;
    T* f = fv + pd.f_off[s];
    const int tid = threadIdx.x;
    if (tid < T64) fb[tid] = tid < w ? f[k0 + tid] : T(0);
    __syncthreads();
    {   // z[c] = sum_{q <= c} Linv[c][q] fb[q]; 4 threads per c
        const int c = tid >> 2, part4 = tid & 3;
        T acc = T(0);
        if (c < w)
            for (int q = part4; q <= c; q += 4) acc += Li[c + q * T64] * fb[q];
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (part4 == 0 && c < T64) z[c] = c < w ? acc : T(0);
    }
    __syncthreads();
    if (lt == 0) {
        if (tid < w) zsol[first + k0 + tid] = z[tid];
        return;
    }
    const int r0 = k0 + w + (lt - 1) * T64;
    const int nr = min(T64, N - r0);
    const int row = tid & 63, cg = tid >> 6;
    T acc = T(0);
    if (row < nr)
        for (int c = cg * 16; c < cg * 16 + 16 && c < w; ++c)
            acc += Fs[(r0 + row) + static_cast<int64_t>(k0 + c) * N] * z[c];
    part[cg][row] = acc;
    __syncthreads();
    if (tid < nr) f[r0 + tid] -= (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
}

// Backward, external rows: f[c] = z[c] - sum_{r >= K} L(r, c) x(R[r]) for the own
// columns c of one 64-column block (warp per 8 columns, lanes over rows).
template <class T>
__global__ void __launch_bounds__(256) k_bwd_ext(const int* __restrict__ level_sn, const int* __restrict__ cb_prefix,
                                                 int nsn, PlanDev pd, const T* __restrict__ F,
                                                 const T* __restrict__ xp, const T* __restrict__ zsol,
                                                 T* __restrict__ fv) {
    int lo = 0, hi = nsn - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cb_prefix[mid] <= static_cast<int>(blockIdx.x)) lo = mid; else hi = mid - 1;
    }
    const int s = level_sn[lo];
    const int kb = blockIdx.x - cb_prefix[lo];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    const T* Fs = F + pd.F_off[s];
    const int* R = pd.rows + pd.rows_off[s];
    T* f = fv + pd.f_off[s];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t = 0; t < 8; ++t) {
        const int c = kb * T64 + wid * 8 + t;
        if (c >= K) break;
        double acc = 0.0;
        for (int r = K + lane; r < N; r += 32)
            acc += static_cast<double>(Fs[r + static_cast<int64_t>(c) * N]) * static_cast<double>(xp[R[r]]);
        acc = warp_sum(acc);
        if (lane == 0) f[c] = static_cast<T>(static_cast<double>(zsol[first + c]) - acc);
    }
}

// Backward tile step k (descending): every block forms x = Linv^T f_blk; block 0
// stores x, block j >= 1 subtracts L(blk rows, column block j-1)^T x from f.
template <class T>
__global__ void __launch_bounds__(256) k_bwd_step(StepArgs a, const int* __restrict__ items, PlanDev pd,
                                                  const T* __restrict__ F, const T* __restrict__ Linv,
                                                  const int64_t* __restrict__ inv_off, T* __restrict__ fv,
                                                  T* __restrict__ xp) {
    __shared__ T fb[T64];
    __shared__ T x[T64];
    const int per = a.k + 1;
    const int i = blockIdx.x / per;
    const int j = blockIdx.x % per;
    const int s = items[a.item_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const T* Fs = F + pd.F_off[s];
    const T* Li = Linv + inv_off[s] + static_cast<int64_t>(a.k) * T64 * T64;
    T* f = fv + pd.f_off[s];
    const int tid = threadIdx.x;
    if (tid < T64) fb[tid] = tid < w ? f[k0 + tid] : T(0);
    __syncthreads();
    {   // x[c] = sum_{q >= c} Linv[q][c] fb[q]
        const int c = tid >> 2, part4 = tid & 3;
        T acc = T(0);
        if (c < w)
            for (int q = c + part4; q < w; q += 4) acc += Li[q + c * T64] * fb[q];
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (part4 == 0 && c < T64) x[c] = c < w ? acc : T(0);
    }
    __syncthreads();
    if (j == 0) {
        if (tid < w) xp[first + k0 + tid] = x[tid];
        return;
    }
    const int cb = j - 1;                       // column block < k
    const int lane = tid & 31, wid = tid >> 5;
    for (int t = 0; t < 8; ++t) {
        const int c = cb * T64 + wid * 8 + t;   // c < k0 <= K
        T acc = T(0);
        for (int r = lane; r < w; r += 32) acc += Fs[(k0 + r) + static_cast<int64_t>(c) * N] * x[r];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) f[c] -= acc;
    }
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
    SK_CUDA(cudaFuncSetAttribute(k_potrf<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(2 * T64 * LDS * sizeof(T))));
    SK_CUDA(cudaFuncSetAttribute(k_trsm<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(2 * T64 * T64 * sizeof(T))));
    SK_CUDA(cudaFuncSetAttribute(k_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(2 * T64 * T64 * sizeof(T))));
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
    std::vector<int> cbp;
    cb_level_off_.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    cb_level_tot_.assign(static_cast<size_t>(p.nlevels), 0);
    for (int l = 0; l < p.nlevels; ++l) {
        cb_level_off_[l] = static_cast<int>(cbp.size());
        int acc = 0;
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            cbp.push_back(acc);
            acc += (p.sn_ncols[p.level_sn[q]] + T64 - 1) / T64;
        }
        cbp.push_back(acc);
        cb_level_tot_[l] = acc;
    }
    cb_level_off_[p.nlevels] = static_cast<int>(cbp.size());
    auto rsv = [&](auto& slot, const auto& vec) { reserve(arena_, slot, vec.size()); };
    rsv(sn_first_, p.sn_first); rsv(sn_ncols_, p.sn_ncols); rsv(sn_nrows_, p.sn_nrows); rsv(sn_parent_, p.sn_parent);
    rsv(rows_, p.rows); rsv(ea_map_, p.ea_map); rsv(ch_ptr_, p.ch_ptr); rsv(ch_list_, p.ch_list);
    rsv(perm_, p.perm); rsv(sn_F_off_, p.sn_F_off); rsv(sn_f_off_, p.sn_f_off); rsv(sn_rows_off_, p.sn_rows_off);
    rsv(ea_off_, p.ea_off); rsv(step_items_, p.step_items); rsv(step_prefix_, p.step_prefix);
    rsv(round_items_, p.round_items); rsv(round_prefix_, p.round_prefix); rsv(level_sn_, p.level_sn);
    rsv(slot_pos_, p.slot_pos); rsv(w_ptr_, p.w_ptr); rsv(slot_i_, p.slot_i); rsv(slot_j_, p.slot_j);
    rsv(w_col_, p.w_col); rsv(w_val_, p.w_val); rsv(inv_off_, inv_off); rsv(cb_prefix_, cbp);
    reserve(arena_, D_, static_cast<size_t>(p.M));
    reserve(arena_, Mdiag_, static_cast<size_t>(p.M));
    reserve(arena_, zp_, static_cast<size_t>(p.M));
    reserve(arena_, xp_, static_cast<size_t>(p.M));
    reserve(arena_, zsol_, static_cast<size_t>(p.M));
    reserve(arena_, fvec_, static_cast<size_t>(p.f_size));
    reserve(arena_, tn_, static_cast<size_t>(std::max(1, p.N)));
    reserve(arena_, params_, 4);
    reserve(arena_, err_, 2);
    arena_.commit();
    auto bnd = [&](auto& slot) { bind(arena_, slot); };
    bnd(sn_first_); bnd(sn_ncols_); bnd(sn_nrows_); bnd(sn_parent_); bnd(rows_); bnd(ea_map_); bnd(ch_ptr_);
    bnd(ch_list_); bnd(perm_); bnd(sn_F_off_); bnd(sn_f_off_); bnd(sn_rows_off_); bnd(ea_off_); bnd(step_items_);
    bnd(step_prefix_); bnd(round_items_); bnd(round_prefix_); bnd(level_sn_); bnd(slot_pos_); bnd(w_ptr_);
    bnd(slot_i_); bnd(slot_j_); bnd(w_col_); bnd(w_val_); bnd(inv_off_); bnd(cb_prefix_); bnd(D_); bnd(Mdiag_);
    bnd(zp_); bnd(xp_); bnd(zsol_); bnd(fvec_); bnd(tn_); bnd(params_); bnd(err_);
    upload(sn_first_, p.sn_first, st_); upload(sn_ncols_, p.sn_ncols, st_); upload(sn_nrows_, p.sn_nrows, st_);
    upload(sn_parent_, p.sn_parent, st_); upload(rows_, p.rows, st_); upload(ea_map_, p.ea_map, st_);
    upload(ch_ptr_, p.ch_ptr, st_); upload(ch_list_, p.ch_list, st_); upload(perm_, p.perm, st_);
    upload(sn_F_off_, p.sn_F_off, st_); upload(sn_f_off_, p.sn_f_off, st_); upload(sn_rows_off_, p.sn_rows_off, st_);
    upload(ea_off_, p.ea_off, st_); upload(step_items_, p.step_items, st_); upload(step_prefix_, p.step_prefix, st_);
    upload(round_items_, p.round_items, st_); upload(round_prefix_, p.round_prefix, st_);
    upload(level_sn_, p.level_sn, st_); upload(slot_pos_, p.slot_pos, st_); upload(w_ptr_, p.w_ptr, st_);
    upload(slot_i_, p.slot_i, st_); upload(slot_j_, p.slot_j, st_); upload(w_col_, p.w_col, st_);
    upload(w_val_, p.w_val, st_); upload(inv_off_, inv_off, st_); upload(cb_prefix_, cbp, st_);
    SK_CUDA(cudaStreamSynchronize(st_));
    set_smem_attrs<float>();
    set_smem_attrs<double>();
}

KktEngine::~KktEngine() {
    for (int q = 0; q < 2; ++q) {
        if (gfac_[q]) cudaGraphExecDestroy(gfac_[q]);
        if (gsol_[q]) cudaGraphExecDestroy(gsol_[q]);
    }
}

PlanDev KktEngine::pd() const {
    return PlanDev{sn_first_.ptr, sn_ncols_.ptr, sn_nrows_.ptr, sn_F_off_.ptr, sn_f_off_.ptr, sn_rows_off_.ptr,
                   rows_.ptr, ea_off_.ptr, ea_map_.ptr, ch_ptr_.ptr, ch_list_.ptr, sn_parent_.ptr};
}

template <class T>
void KktEngine::launch_factor(T* F, T* Linv, Prof* prof) {
    auto run = [&](int cls, auto&& f) {
        if (prof) prof->timed(cls, f); else f();
    };
    const auto& p = plan_;
    const PlanDev pdv = pd();
    SK_CUDA(cudaMemsetAsync(F, 0, sizeof(T) * static_cast<size_t>(p.F_size), st_));
    SK_CUDA(cudaMemsetAsync(err_.ptr, 0, 2 * sizeof(int), st_));
    const double* theta = theta_bound_;
    run(0, [&] {
        if (p.dense_mode) {
            k_asm_diag_dense<<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, lp_.a_rp, lp_.a_ci, lp_.a_v, theta,
                                                                     Mdiag_.ptr, D_.ptr);
            k_asm_cols_dense<T><<<blocks_for(static_cast<int64_t>(p.M) * 32, 256), 256, 0, st_>>>(
                p.M, lp_.a_rp, lp_.a_ci, lp_.a_v, lp_.t_rp, lp_.t_ci, lp_.t_v, theta, Mdiag_.ptr, D_.ptr, lp_.row_lp,
                pdv, params_.ptr, F);
        } else {
            k_asm_diag_sparse<<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, w_ptr_.ptr, w_col_.ptr, w_val_.ptr, theta,
                                                                      Mdiag_.ptr, D_.ptr);
            k_asm_slots_sparse<T><<<blocks_for(p.nslots, 256), 256, 0, st_>>>(
                p.nslots, p.M, w_ptr_.ptr, w_col_.ptr, w_val_.ptr, theta, slot_i_.ptr, slot_j_.ptr, slot_pos_.ptr,
                Mdiag_.ptr, D_.ptr, params_.ptr, F);
        }
    });
    for (int l = 0; l < p.nlevels; ++l) {
        for (int q = p.step_level_ptr[l]; q < p.step_level_ptr[l + 1]; ++q) {
            const auto& st = p.steps[q];
            StepArgs a{st.k, st.item_off, st.nitems, st.trsm_prefix_off, st.upd_prefix_off};
            run(1, [&] {
                k_potrf<T><<<st.nitems, 32, 2 * T64 * LDS * sizeof(T), st_>>>(a, step_items_.ptr, pdv, F, Linv,
                                                                              inv_off_.ptr, err_.ptr);
            });
            if (st.trsm_tiles > 0)
                run(2, [&] {
                    k_trsm<T><<<static_cast<int>(st.trsm_tiles), 256, 2 * T64 * T64 * sizeof(T), st_>>>(
                        a, step_items_.ptr, step_prefix_.ptr, pdv, F, Linv, inv_off_.ptr);
                });
            if (st.upd_tiles > 0) {
                run(3, [&] {
                    k_update<T><<<static_cast<int>(st.upd_tiles), 256, 2 * T64 * T64 * sizeof(T), st_>>>(
                        a, step_items_.ptr, step_prefix_.ptr, pdv, F);
                });
                if (prof) {
                    for (int it = 0; it < st.nitems; ++it) {
                        const int s2 = p.step_items[st.item_off + it];
                        const double w = std::min<int64_t>(T64, p.sn_ncols[s2] - static_cast<int64_t>(st.k) * T64);
                        const double t = p.sn_nrows[s2] - static_cast<double>(st.k) * T64 - w;
                        prof->upd_flops += 2.0 * w * t * (t + 1.0) / 2.0;
                        prof->upd_bytes += sizeof(T) * (t * w + 2.0 * t * (t + 1.0) / 2.0);
                    }
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
    const PlanDev pdv = pd();
    T* zp = reinterpret_cast<T*>(zp_.ptr);
    T* xp = reinterpret_cast<T*>(xp_.ptr);
    T* zs = reinterpret_cast<T*>(zsol_.ptr);
    T* fv = reinterpret_cast<T*>(fvec_.ptr);
    for (int l = 0; l < p.nlevels; ++l) {
        const int nl = p.level_ptr[l + 1] - p.level_ptr[l];
        run(5, [&] { k_fwd_init<T><<<nl, 256, 0, st_>>>(level_sn_.ptr + p.level_ptr[l], pdv, zp, fv); });
        for (int q = p.step_level_ptr[l]; q < p.step_level_ptr[l + 1]; ++q) {
            const auto& st = p.steps[q];
            StepArgs a{st.k, st.item_off, st.nitems, st.trsm_prefix_off, st.upd_prefix_off};
            run(5, [&] {
                k_fwd_step<T><<<static_cast<int>(st.trsm_tiles) + st.nitems, 256, 0, st_>>>(
                    a, step_items_.ptr, step_prefix_.ptr, pdv, F, Linv, inv_off_.ptr, fv, zs);
            });
        }
    }
    for (int l = p.nlevels - 1; l >= 0; --l) {
        const int nl = p.level_ptr[l + 1] - p.level_ptr[l];
        run(6, [&] {
            k_bwd_ext<T><<<cb_level_tot_[l], 256, 0, st_>>>(level_sn_.ptr + p.level_ptr[l],
                                                            cb_prefix_.ptr + cb_level_off_[l], nl, pdv, F, xp, zs, fv);
        });
        for (int q = p.step_level_ptr[l + 1] - 1; q >= p.step_level_ptr[l]; --q) {
            const auto& st = p.steps[q];
            StepArgs a{st.k, st.item_off, st.nitems, st.trsm_prefix_off, st.upd_prefix_off};
            run(6, [&] {
                k_bwd_step<T><<<st.nitems * (st.k + 1), 256, 0, st_>>>(a, step_items_.ptr, pdv, F, Linv, inv_off_.ptr,
                                                                      fv, xp);
            });
        }
    }
    SK_CUDA(cudaGetLastError());
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

bool KktEngine::factor(const double* d_theta, double delta, bool fp32) {
    const int q = fp32 ? 1 : 0;
    ensure_fronts(fp32);
    fp32_ = fp32;
    double hp[4] = {delta, 0, 0, 0};
    SK_CUDA(cudaMemcpyAsync(params_.ptr, hp, sizeof(hp), cudaMemcpyHostToDevice, st_));
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
    SK_CUDA(cudaGraphLaunch(gfac_[q], st_));
    int herr[2];
    SK_CUDA(cudaMemcpyAsync(herr, err_.ptr, sizeof(herr), cudaMemcpyDeviceToHost, st_));
    SK_CUDA(cudaStreamSynchronize(st_));
    failed_sn_ = herr[0] ? herr[1] : -1;
    return herr[0] == 0;
}

void KktEngine::apply_inverse(const double* d_src, double* d_dst) {
    const auto& p = plan_;
    const int q = fp32_ ? 1 : 0;
    if (fp32_) k_permute_scale<float><<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, perm_.ptr, D_.ptr, d_src,
                                                                             reinterpret_cast<float*>(zp_.ptr));
    else k_permute_scale<double><<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, perm_.ptr, D_.ptr, d_src, zp_.ptr);
    if (!gsol_[q]) {
        cudaGraph_t g;
        SK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        if (fp32_) launch_solve<float>(F32_.ptr, Linv32_.ptr); else launch_solve<double>(F64_.ptr, Linv64_.ptr);
        SK_CUDA(cudaStreamEndCapture(st_, &g));
        SK_CUDA(cudaGraphInstantiate(&gsol_[q], g, 0));
        cudaGraphDestroy(g);
    }
    SK_CUDA(cudaGraphLaunch(gsol_[q], st_));
    if (fp32_) k_unpermute_scale<float><<<blocks_for(p.M, 256), 256, 0, st_>>>(
        p.M, perm_.ptr, D_.ptr, reinterpret_cast<const float*>(xp_.ptr), d_dst);
    else k_unpermute_scale<double><<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, perm_.ptr, D_.ptr, xp_.ptr, d_dst);
    SK_CUDA(cudaGetLastError());
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
            plan_.M, perm_.ptr, D_.ptr, reinterpret_cast<const float*>(xp_.ptr), d_out);
    } else {
        k_permute_scale<double><<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, d_rhs, zp_.ptr);
        launch_solve<double>(F64_.ptr, Linv64_.ptr, &pr);
        k_unpermute_scale<double><<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, xp_.ptr,
                                                                             d_out);
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
