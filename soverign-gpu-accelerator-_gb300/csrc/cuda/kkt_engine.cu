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

template <class T>
__global__ void __launch_bounds__(256) k_potrf(StepArgs a, const int* __restrict__ items, PlanDev pd, T* F,
                                               int* err) {
    __shared__ double A[T64 * LDS];
    const int s = items[a.item_off + blockIdx.x];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    T* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        if (r >= c) A[r * LDS + c] = static_cast<double>(Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N]);
    }
    __syncthreads();
    for (int c = 0; c < w; ++c) {
        if (tid == 0) {
            double piv = A[c * LDS + c];
            if (!(piv > 0.0)) {
                if (atomicCAS(err, 0, 1) == 0) err[1] = s;
                piv = 1.0;
            }
            A[c * LDS + c] = sqrt(piv);
        }
        __syncthreads();
        const double l = A[c * LDS + c];
        for (int r = c + 1 + tid; r < w; r += blockDim.x) A[r * LDS + c] /= l;
        __syncthreads();
        const int rem = w - c - 1;
        for (int idx = tid; idx < rem * rem; idx += blockDim.x) {
            const int r = c + 1 + idx % rem, cc = c + 1 + idx / rem;
            if (cc <= r) A[r * LDS + cc] -= A[r * LDS + c] * A[cc * LDS + c];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        if (r >= c) Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N] = static_cast<T>(A[r * LDS + c]);
    }
}

template <class T>
__global__ void __launch_bounds__(256) k_trsm(StepArgs a, const int* __restrict__ items,
                                              const int* __restrict__ prefix, PlanDev pd, T* F) {
    extern __shared__ double sm[];
    double* L = sm;               // w x w lower, row-major LDS
    double* X = sm + T64 * LDS;   // rows x w, row-major LDS
    const int i = find_item(prefix + a.tp_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int r0 = k0 + w + lt * T64;
    const int nr = min(T64, N - r0);
    T* Fs = F + pd.F_off[s];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        if (r >= c) L[r * LDS + c] = static_cast<double>(Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N]);
    }
    for (int idx = tid; idx < nr * w; idx += blockDim.x) {
        const int r = idx % nr, c = idx / nr;
        X[r * LDS + c] = static_cast<double>(Fs[(r0 + r) + static_cast<int64_t>(k0 + c) * N]);
    }
    __syncthreads();
    for (int c = 0; c < w; ++c) {
        const double d = L[c * LDS + c];
        for (int r = tid; r < nr; r += blockDim.x) X[r * LDS + c] /= d;
        __syncthreads();
        const int rem = w - c - 1;
        for (int idx = tid; idx < nr * rem; idx += blockDim.x) {
            const int r = idx % nr, cc = c + 1 + idx / nr;
            X[r * LDS + cc] -= X[r * LDS + c] * L[cc * LDS + c];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < nr * w; idx += blockDim.x) {
        const int r = idx % nr, c = idx / nr;
        Fs[(r0 + r) + static_cast<int64_t>(k0 + c) * N] = static_cast<T>(X[r * LDS + c]);
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

__global__ void k_permute_scale(int M, const int* __restrict__ perm, const double* __restrict__ D,
                                const double* __restrict__ src, double* __restrict__ zp) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < M) zp[q] = D[q] * src[perm[q]];
}

__global__ void k_unpermute_scale(int M, const int* __restrict__ perm, const double* __restrict__ D,
                                  const double* __restrict__ xp, double* __restrict__ dst) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < M) dst[perm[q]] = D[q] * xp[q];
}

__global__ void k_fwd_init(const int* __restrict__ level_sn, PlanDev pd, const double* __restrict__ zp,
                           double* __restrict__ fv) {
    const int s = level_sn[blockIdx.x];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    double* f = fv + pd.f_off[s];
    for (int q = threadIdx.x; q < N; q += blockDim.x) f[q] = q < K ? zp[first + q] : 0.0;
    __syncthreads();
    for (int e = pd.ch_ptr[s]; e < pd.ch_ptr[s + 1]; ++e) {
        const int c = pd.ch_list[e];
        const int Kc = pd.sn_ncols[c], u = pd.sn_nrows[c] - Kc;
        const double* uc = fv + pd.f_off[c] + Kc;
        const int* map = pd.ea_map + pd.ea_off[c];
        for (int t = threadIdx.x; t < u; t += blockDim.x) f[map[t]] += uc[t];
        __syncthreads();
    }
}

template <class T>
__global__ void k_fwd_diag(StepArgs a, const int* __restrict__ items, PlanDev pd, const T* __restrict__ F,
                           double* __restrict__ fv) {
    __shared__ double L[T64 * LDS];
    __shared__ double z[T64];
    const int s = items[a.item_off + blockIdx.x];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const T* Fs = F + pd.F_off[s];
    double* f = fv + pd.f_off[s];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        if (r >= c) L[r * LDS + c] = static_cast<double>(Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N]);
    }
    for (int c = tid; c < w; c += blockDim.x) z[c] = f[k0 + c];
    __syncthreads();
    for (int c = 0; c < w; ++c) {
        if (tid == 0) z[c] /= L[c * LDS + c];
        __syncthreads();
        for (int r = c + 1 + tid; r < w; r += blockDim.x) z[r] -= L[r * LDS + c] * z[c];
        __syncthreads();
    }
    for (int c = tid; c < w; c += blockDim.x) f[k0 + c] = z[c];
}

template <class T>
__global__ void __launch_bounds__(256) k_fwd_gemv(StepArgs a, const int* __restrict__ items,
                                                  const int* __restrict__ prefix, PlanDev pd,
                                                  const T* __restrict__ F, double* __restrict__ fv) {
    __shared__ double z[T64];
    __shared__ double part[4][T64];
    const int i = find_item(prefix + a.tp_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int r0 = k0 + w + lt * T64;
    const int nr = min(T64, N - r0);
    const T* Fs = F + pd.F_off[s];
    double* f = fv + pd.f_off[s];
    const int tid = threadIdx.x;
    if (tid < w) z[tid] = f[k0 + tid];
    __syncthreads();
    const int row = tid & 63, cg = tid >> 6;
    double acc = 0.0;
    if (row < nr)
        for (int c = cg * 16; c < cg * 16 + 16 && c < w; ++c)
            acc += static_cast<double>(Fs[(r0 + row) + static_cast<int64_t>(k0 + c) * N]) * z[c];
    part[cg][row] = acc;
    __syncthreads();
    if (tid < nr) f[r0 + tid] -= (part[0][tid] + part[1][tid]) + (part[2][tid] + part[3][tid]);
}

__global__ void k_bwd_init(const int* __restrict__ level_sn, PlanDev pd, const double* __restrict__ xp,
                           double* __restrict__ fv) {
    const int s = level_sn[blockIdx.x];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    double* f = fv + pd.f_off[s];
    const int* R = pd.rows + pd.rows_off[s];
    for (int q = K + threadIdx.x; q < N; q += blockDim.x) f[q] = xp[R[q]];
}

template <class T>
__global__ void __launch_bounds__(256) k_bwd_partial(StepArgs a, const int* __restrict__ items,
                                                     const int* __restrict__ prefix, PlanDev pd,
                                                     const T* __restrict__ F, const double* __restrict__ fv,
                                                     double* __restrict__ partial) {
    __shared__ double S[T64 * LDS];   // S[c][row]
    const int i = find_item(prefix + a.tp_off, a.nitems, blockIdx.x);
    const int s = items[a.item_off + i];
    const int lt = blockIdx.x - prefix[a.tp_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const int r0 = k0 + w + lt * T64;
    const int nr = min(T64, N - r0);
    const T* Fs = F + pd.F_off[s];
    const double* f = fv + pd.f_off[s];
    const int tid = threadIdx.x;
    const int row = tid & 63, cg = tid >> 6;
    const double fr = row < nr ? f[r0 + row] : 0.0;
    for (int c = cg * 16; c < cg * 16 + 16; ++c)
        S[c * LDS + row] = (row < nr && c < w) ? static_cast<double>(Fs[(r0 + row) + static_cast<int64_t>(k0 + c) * N]) * fr : 0.0;
    __syncthreads();
    if (tid < T64) {
        double acc = 0.0;
        for (int r = 0; r < nr; ++r) acc += S[tid * LDS + r];
        partial[static_cast<int64_t>(blockIdx.x) * T64 + tid] = acc;
    }
}

template <class T>
__global__ void k_bwd_diag(StepArgs a, const int* __restrict__ items, const int* __restrict__ prefix, PlanDev pd,
                           const T* __restrict__ F, const double* __restrict__ partial, double* __restrict__ fv,
                           double* __restrict__ xp) {
    __shared__ double L[T64 * LDS];
    __shared__ double t[T64];
    const int i = blockIdx.x;
    const int s = items[a.item_off + i];
    const int N = pd.sn_nrows[s], K = pd.sn_ncols[s], first = pd.sn_first[s];
    const int k0 = a.k * T64;
    const int w = min(T64, K - k0);
    const T* Fs = F + pd.F_off[s];
    double* f = fv + pd.f_off[s];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < w * w; idx += blockDim.x) {
        const int r = idx % w, c = idx / w;
        if (r >= c) L[r * LDS + c] = static_cast<double>(Fs[(k0 + r) + static_cast<int64_t>(k0 + c) * N]);
    }
    if (tid < w) {
        double v = f[k0 + tid];
        const int tb = prefix[a.tp_off + i], te = prefix[a.tp_off + i + 1];
        for (int q = tb; q < te; ++q) v -= partial[static_cast<int64_t>(q) * T64 + tid];
        t[tid] = v;
    }
    __syncthreads();
    for (int c = w - 1; c >= 0; --c) {
        if (tid == 0) t[c] /= L[c * LDS + c];
        __syncthreads();
        for (int r = tid; r < c; r += blockDim.x) t[r] -= L[c * LDS + r] * t[c];
        __syncthreads();
    }
    if (tid < w) {
        f[k0 + tid] = t[tid];
        xp[first + k0 + tid] = t[tid];
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


KktEngine::KktEngine(const ipm::FrontPlan& plan, const DeviceLP& lp, cudaStream_t stream)
    : plan_(plan), lp_(lp), st_(stream) {
    const auto& p = plan_;
    auto rsv = [&](auto& slot, const auto& vec) { reserve(arena_, slot, vec.size()); };
    rsv(sn_first_, p.sn_first); rsv(sn_ncols_, p.sn_ncols); rsv(sn_nrows_, p.sn_nrows);
    rsv(rows_, p.rows); rsv(ea_map_, p.ea_map); rsv(ch_ptr_, p.ch_ptr); rsv(ch_list_, p.ch_list);
    rsv(perm_, p.perm); rsv(sn_F_off_, p.sn_F_off); rsv(sn_f_off_, p.sn_f_off); rsv(sn_rows_off_, p.sn_rows_off);
    rsv(ea_off_, p.ea_off); rsv(step_items_, p.step_items); rsv(step_prefix_, p.step_prefix);
    rsv(round_items_, p.round_items); rsv(round_prefix_, p.round_prefix); rsv(level_sn_, p.level_sn);
    rsv(slot_pos_, p.slot_pos); rsv(w_ptr_, p.w_ptr); rsv(slot_i_, p.slot_i); rsv(slot_j_, p.slot_j);
    rsv(w_col_, p.w_col); rsv(w_val_, p.w_val);
    rsv(sn_parent_, p.sn_parent);
    reserve(arena_, D_, static_cast<size_t>(p.M));
    reserve(arena_, Mdiag_, static_cast<size_t>(p.M));
    reserve(arena_, zp_, static_cast<size_t>(p.M));
    reserve(arena_, xp_, static_cast<size_t>(p.M));
    reserve(arena_, fvec_, static_cast<size_t>(p.f_size));
    for (const auto& stp : p.steps) max_partial_ = std::max<int64_t>(max_partial_, stp.trsm_tiles);
    reserve(arena_, partial_, static_cast<size_t>(std::max<int64_t>(1, max_partial_) * T64));
    reserve(arena_, tn_, static_cast<size_t>(std::max(1, p.N)));
    reserve(arena_, params_, 4);
    reserve(arena_, err_, 2);
    arena_.commit();
    auto bnd = [&](auto& slot) { bind(arena_, slot); };
    bnd(sn_first_); bnd(sn_ncols_); bnd(sn_nrows_); bnd(rows_); bnd(ea_map_); bnd(ch_ptr_); bnd(ch_list_);
    bnd(perm_); bnd(sn_F_off_); bnd(sn_f_off_); bnd(sn_rows_off_); bnd(ea_off_); bnd(step_items_);
    bnd(step_prefix_); bnd(round_items_); bnd(round_prefix_); bnd(level_sn_); bnd(slot_pos_); bnd(w_ptr_);
    bnd(slot_i_); bnd(slot_j_); bnd(w_col_); bnd(w_val_); bnd(D_); bnd(Mdiag_); bnd(zp_); bnd(xp_);
    bnd(fvec_); bnd(partial_); bnd(tn_); bnd(params_); bnd(err_); bnd(sn_parent_);
    upload(sn_first_, p.sn_first, st_); upload(sn_ncols_, p.sn_ncols, st_); upload(sn_nrows_, p.sn_nrows, st_);
    upload(rows_, p.rows, st_); upload(ea_map_, p.ea_map, st_); upload(ch_ptr_, p.ch_ptr, st_);
    upload(ch_list_, p.ch_list, st_); upload(perm_, p.perm, st_); upload(sn_F_off_, p.sn_F_off, st_);
    upload(sn_f_off_, p.sn_f_off, st_); upload(sn_rows_off_, p.sn_rows_off, st_); upload(ea_off_, p.ea_off, st_);
    upload(step_items_, p.step_items, st_); upload(step_prefix_, p.step_prefix, st_);
    upload(round_items_, p.round_items, st_); upload(round_prefix_, p.round_prefix, st_);
    upload(level_sn_, p.level_sn, st_); upload(slot_pos_, p.slot_pos, st_); upload(w_ptr_, p.w_ptr, st_);
    upload(slot_i_, p.slot_i, st_); upload(slot_j_, p.slot_j, st_); upload(w_col_, p.w_col, st_);
    upload(w_val_, p.w_val, st_);
    upload(sn_parent_, p.sn_parent, st_);
    SK_CUDA(cudaStreamSynchronize(st_));
    SK_CUDA(cudaFuncSetAttribute(k_trsm<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * T64 * LDS * 8));
    SK_CUDA(cudaFuncSetAttribute(k_trsm<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * T64 * LDS * 8));
    SK_CUDA(cudaFuncSetAttribute(k_update<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * T64 * T64 * 8));
    SK_CUDA(cudaFuncSetAttribute(k_update<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * T64 * T64 * 4));
}

KktEngine::~KktEngine() {
    for (int q = 0; q < 2; ++q) {
        if (gfac_[q]) cudaGraphExecDestroy(gfac_[q]);
        if (gsol_[q]) cudaGraphExecDestroy(gsol_[q]);
    }
}

template <class T>
void KktEngine::launch_factor(T* F, Prof* prof) {
    auto run = [&](int cls, auto&& f) {
        if (prof) prof->timed(cls, f); else f();
    };
    const auto& p = plan_;
    PlanDev pd{sn_first_.ptr, sn_ncols_.ptr, sn_nrows_.ptr, sn_F_off_.ptr, sn_f_off_.ptr, sn_rows_off_.ptr,
               rows_.ptr, ea_off_.ptr, ea_map_.ptr, ch_ptr_.ptr, ch_list_.ptr, sn_parent_.ptr};
    SK_CUDA(cudaMemsetAsync(F, 0, sizeof(T) * static_cast<size_t>(p.F_size), st_));
    SK_CUDA(cudaMemsetAsync(err_.ptr, 0, 2 * sizeof(int), st_));
    const double* theta = theta_bound_;
    run(0, [&] {
        if (p.dense_mode) {
            k_asm_diag_dense<<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, lp_.a_rp, lp_.a_ci, lp_.a_v, theta,
                                                                     Mdiag_.ptr, D_.ptr);
            k_asm_cols_dense<T><<<blocks_for(static_cast<int64_t>(p.M) * 32, 256), 256, 0, st_>>>(
                p.M, lp_.a_rp, lp_.a_ci, lp_.a_v, lp_.t_rp, lp_.t_ci, lp_.t_v, theta, Mdiag_.ptr, D_.ptr, lp_.row_lp,
                pd, params_.ptr, F);
        } else {
            k_asm_diag_sparse<<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, w_ptr_.ptr, w_col_.ptr, w_val_.ptr, theta,
                                                                      Mdiag_.ptr, D_.ptr);
            k_asm_slots_sparse<T><<<blocks_for(p.nslots, 256), 256, 0, st_>>>(
                p.nslots, p.M, w_ptr_.ptr, w_col_.ptr, w_val_.ptr, theta, slot_i_.ptr, slot_j_.ptr, slot_pos_.ptr,
                Mdiag_.ptr, D_.ptr, params_.ptr, F);
        }
    });
    SK_CUDA(cudaGetLastError());
    for (int l = 0; l < p.nlevels; ++l) {
        for (int q = p.step_level_ptr[l]; q < p.step_level_ptr[l + 1]; ++q) {
            const auto& st = p.steps[q];
            StepArgs a{st.k, st.item_off, st.nitems, st.trsm_prefix_off, st.upd_prefix_off};
            run(1, [&] { k_potrf<T><<<st.nitems, 256, 0, st_>>>(a, step_items_.ptr, pd, F, err_.ptr); });
            if (st.trsm_tiles > 0)
                run(2, [&] {
                    k_trsm<T><<<static_cast<int>(st.trsm_tiles), 256, 2 * T64 * LDS * 8, st_>>>(
                        a, step_items_.ptr, step_prefix_.ptr, pd, F);
                });
            if (st.upd_tiles > 0) {
                run(3, [&] {
                    k_update<T><<<static_cast<int>(st.upd_tiles), 256, 2 * T64 * T64 * sizeof(T), st_>>>(
                        a, step_items_.ptr, step_prefix_.ptr, pd, F);
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
                    rd.item_off, rd.nitems, rd.prefix_off, round_items_.ptr, round_prefix_.ptr, pd, F);
            });
        }
    }
    SK_CUDA(cudaGetLastError());
}

template <class T>
void KktEngine::launch_solve(const T* F, Prof* prof) {
    auto run = [&](int cls, auto&& f) {
        if (prof) prof->timed(cls, f); else f();
    };
    const auto& p = plan_;
    PlanDev pd{sn_first_.ptr, sn_ncols_.ptr, sn_nrows_.ptr, sn_F_off_.ptr, sn_f_off_.ptr, sn_rows_off_.ptr,
               rows_.ptr, ea_off_.ptr, ea_map_.ptr, ch_ptr_.ptr, ch_list_.ptr, sn_parent_.ptr};
    for (int l = 0; l < p.nlevels; ++l) {
        const int nl = p.level_ptr[l + 1] - p.level_ptr[l];
        run(5, [&] { k_fwd_init<<<nl, 256, 0, st_>>>(level_sn_.ptr + p.level_ptr[l], pd, zp_.ptr, fvec_.ptr); });
        for (int q = p.step_level_ptr[l]; q < p.step_level_ptr[l + 1]; ++q) {
            const auto& st = p.steps[q];
            StepArgs a{st.k, st.item_off, st.nitems, st.trsm_prefix_off, st.upd_prefix_off};
            run(5, [&] { k_fwd_diag<T><<<st.nitems, 64, 0, st_>>>(a, step_items_.ptr, pd, F, fvec_.ptr); });
            if (st.trsm_tiles > 0)
                run(5, [&] {
                    k_fwd_gemv<T><<<static_cast<int>(st.trsm_tiles), 256, 0, st_>>>(a, step_items_.ptr,
                                                                                  step_prefix_.ptr, pd, F, fvec_.ptr);
                });
        }
    }
    for (int l = p.nlevels - 1; l >= 0; --l) {
        const int nl = p.level_ptr[l + 1] - p.level_ptr[l];
        run(6, [&] { k_bwd_init<<<nl, 256, 0, st_>>>(level_sn_.ptr + p.level_ptr[l], pd, xp_.ptr, fvec_.ptr); });
        for (int q = p.step_level_ptr[l + 1] - 1; q >= p.step_level_ptr[l]; --q) {
            const auto& st = p.steps[q];
            StepArgs a{st.k, st.item_off, st.nitems, st.trsm_prefix_off, st.upd_prefix_off};
            if (st.trsm_tiles > 0)
                run(6, [&] {
                    k_bwd_partial<T><<<static_cast<int>(st.trsm_tiles), 256, 0, st_>>>(
                        a, step_items_.ptr, step_prefix_.ptr, pd, F, fvec_.ptr, partial_.ptr);
                });
            run(6, [&] {
                k_bwd_diag<T><<<st.nitems, 64, 0, st_>>>(a, step_items_.ptr, step_prefix_.ptr, pd, F, partial_.ptr,
                                                         fvec_.ptr, xp_.ptr);
            });
        }
    }
    SK_CUDA(cudaGetLastError());
}

bool KktEngine::factor(const double* d_theta, double delta, bool fp32) {
    const int q = fp32 ? 1 : 0;
    if (fp32 && !F32_.ptr) {
        f32_arena_.reset();
        reserve(f32_arena_, F32_, static_cast<size_t>(plan_.F_size));
        f32_arena_.commit();
        bind(f32_arena_, F32_);
    }
    if (!fp32 && !F64_.ptr) {
        f64_arena_.reset();
        reserve(f64_arena_, F64_, static_cast<size_t>(plan_.F_size));
        f64_arena_.commit();
        bind(f64_arena_, F64_);
    }
    fp32_ = fp32;
    double hp[4] = {delta, 0, 0, 0};
    SK_CUDA(cudaMemcpyAsync(params_.ptr, hp, sizeof(hp), cudaMemcpyHostToDevice, st_));
    if (!gfac_[q] || gfac_theta_[q] != d_theta) {
        if (gfac_[q]) { cudaGraphExecDestroy(gfac_[q]); gfac_[q] = nullptr; }
        theta_bound_ = d_theta;
        cudaGraph_t g;
        SK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        if (fp32) launch_factor<float>(F32_.ptr); else launch_factor<double>(F64_.ptr);
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
    k_permute_scale<<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, perm_.ptr, D_.ptr, d_src, zp_.ptr);
    if (!gsol_[q]) {
        cudaGraph_t g;
        SK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        if (fp32_) launch_solve<float>(F32_.ptr); else launch_solve<double>(F64_.ptr);
        SK_CUDA(cudaStreamEndCapture(st_, &g));
        SK_CUDA(cudaGraphInstantiate(&gsol_[q], g, 0));
        cudaGraphDestroy(g);
    }
    SK_CUDA(cudaGraphLaunch(gsol_[q], st_));
    k_unpermute_scale<<<blocks_for(p.M, 256), 256, 0, st_>>>(p.M, perm_.ptr, D_.ptr, xp_.ptr, d_dst);
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
    if (fp32) launch_factor<float>(F32_.ptr, &pr); else launch_factor<double>(F64_.ptr, &pr);
    k_permute_scale<<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, d_rhs, zp_.ptr);
    if (fp32) launch_solve<float>(F32_.ptr, &pr); else launch_solve<double>(F64_.ptr, &pr);
    k_unpermute_scale<<<blocks_for(plan_.M, 256), 256, 0, st_>>>(plan_.M, perm_.ptr, D_.ptr, xp_.ptr, d_out);
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
