// Device Mehrotra predictor-corrector IPM (batch of LPs, lock-step iterations
// with per-LP masks). Follows the reference's MehrotraSolver::Impl
// (src/ipm/mehrotra_device.cu:276-1047):
//   * 10-pass inline Ruiz scaling (:289-323), unit start x = s = 1, y = 0 (:93-102)
//   * predictor: r_xs = -x s, v = -Theta rd - r_xs/s, rkkt = -rp + A v (:783-786)
//   * ds = -rd - A^T dy, dx = -Theta ds + r_xs/s (:799-802, :128-133)
//   * direction check e1, e2, e3 <= 1e-8 (:494-587)
//   * sigma = min(1, (mu_aff/mu)^3), corrector r_xs = -x s + sigma mu - dx_aff ds_aff (:839-843)
//   * eta = 0.995, Armijo 1e-4 backtracking on the normalised residual sum with up
//     to 15 halvings, then a centred direction (sigma_c = 1/2, common step, up to 30
//     halvings) (:873-996)
//   * normal-equation solves to ||r||_inf <= 1e-9 max(1, ||rp||_2) with up to 10
//     steps of FP64 iterative refinement and rollback on stagnation
//     (src/cuda/kkt.cu:620-870, src/ipm/mehrotra_device.cu:791)
// Differences by design: the normal matrix is factored once per iteration (the
// reference refactors on every solve), D (A Theta A^T) D + delta I with
// delta = 1e-9 x 10^retry is the only factorisation (the reference's extra
// unequilibrated factor is overwritten by its solve), reductions are
// deterministic per LP, and in mixed precision the factor is FP32 until mu drops
// below the switch threshold or an FP32 solve misses its tolerance.
#include "cuda/device_ipm.hpp"
#include "cuda/autotune.hpp"
#include "cuda/gnn.hpp"
#include "cuda/spmv.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <numeric>
#include <string>
#include <thread>

namespace sankhya {
namespace dev {

namespace {

constexpr int kChunk = 1024;   // entries per block of the segmented reductions
constexpr int kMaxR = 10;
constexpr double kLearnedSaturated = 0.99;   // learned start: upper bound on its distance to the stopping test
constexpr double kShortStep = 0.1;           // learned-start restart: a step shorter than this ...
constexpr int kShortSteps = 3;               // ... this many times ...
constexpr int kRestartWindow = 10;           // ... within the first iterations
// robust mode: a direction whose checks e1, e2, e3 stay below this is used (the merit
// line search then decides); tighter checks stalled a few LPs just short of 1e-8
constexpr double kUseDir = 1e-4;
constexpr double kTensorMu = 1e-4;           // FP32 fronts: tensor-core updates while mu >= this
constexpr int kLooseIters = 3;               // stall acceptance of the relative tests (see the stopping rule)
constexpr double kNearFeas = 0.1;            // near-optimal line-search rule: rel. pinf, dinf below this x tol
constexpr int kProgressIter = 12;            // learned-start restart: by this iteration the distance to the
constexpr double kProgress = 1e-3;           // stopping test must have fallen by this factor

enum { OP_SUM = 0, OP_MAX = 1, OP_MIN = 2 };

inline int nblk(int64_t n, int t = 256) { return static_cast<int>((n + t - 1) / t); }

// ---------------------------------------------------------------- SpMV
// k_spmv / spmv() / EpiAxpby: spmv.cuh; the lane-group width of A and A^T is
// chosen at set-up by spmv_tune() (autotune.hpp).

struct EpiSub {          // out = d - a
    const double* a;
    double* out;
    __device__ void operator()(int i, double d) const { out[i] = d - a[i]; }
};
struct EpiAdd {          // out = d + a
    const double* a;
    double* out;
    __device__ void operator()(int i, double d) const { out[i] = d + a[i]; }
};
struct EpiRd {           // rd = A^T y + s - c
    const double* s;
    const double* c;
    double* rd;
    __device__ void operator()(int j, double d) const { rd[j] = d + s[j] - c[j]; }
};
struct EpiRhsMinus {     // r = rhs - d
    const double* rhs;
    double* r;
    __device__ void operator()(int i, double d) const { r[i] = rhs[i] - d; }
};
struct EpiTheta {        // out = theta * d
    const double* theta;
    double* out;
    __device__ void operator()(int j, double d) const { out[j] = theta[j] * d; }
};
struct EpiDsDx {         // t = A^T dy: ds = -rd - t, dx = -theta ds + rxs / s, e2, e3
    const double *rd, *theta, *rxs, *x, *s;
    double *ds, *dx, *e2, *e3;
    __device__ void operator()(int j, double t) const {
        const double dsj = -rd[j] - t;
        const double dxj = -theta[j] * dsj + rxs[j] / s[j];
        ds[j] = dsj;
        dx[j] = dxj;
        e2[j] = rd[j] + dsj + t;
        e3[j] = s[j] * dxj + x[j] * dsj - rxs[j];
    }
};

// ------------------------------------------------------------ reductions

template <int R, class F>
__global__ void __launch_bounds__(256) k_reduce(const int* __restrict__ cstart, const int* __restrict__ cend, F f,
                                                double* __restrict__ partial) {
    __shared__ double sh[8][R];
    double acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = F::op(r) == OP_SUM ? 0.0 : (F::op(r) == OP_MAX ? -HUGE_VAL : HUGE_VAL);
    const int q = blockIdx.x;
    for (int i = cstart[q] + threadIdx.x; i < cend[q]; i += blockDim.x) {
        double v[R];
        f(i, v);
#pragma unroll
        for (int r = 0; r < R; ++r)
            acc[r] = F::op(r) == OP_SUM ? acc[r] + v[r] : (F::op(r) == OP_MAX ? fmax(acc[r], v[r]) : fmin(acc[r], v[r]));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        double a = acc[r];
        if (F::op(r) == OP_SUM) a = warp_sum(a);
        else if (F::op(r) == OP_MAX) a = warp_max(a);
        else a = warp_min(a);
        if (lane == 0) sh[wid][r] = a;
    }
    __syncthreads();
    if (threadIdx.x < R) {
        const int r = threadIdx.x;
        double a = sh[0][r];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w)
            a = F::op(r) == OP_SUM ? a + sh[w][r] : (F::op(r) == OP_MAX ? fmax(a, sh[w][r]) : fmin(a, sh[w][r]));
        partial[static_cast<int64_t>(q) * R + r] = a;
    }
}

template <int R, class F>
__global__ void k_reduce_final(int nlp, const int* __restrict__ cptr, const double* __restrict__ partial,
                               double* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nlp * R) return;
    const int k = t / R, r = t % R;
    double a = F::op(r) == OP_SUM ? 0.0 : (F::op(r) == OP_MAX ? -HUGE_VAL : HUGE_VAL);
    for (int q = cptr[k]; q < cptr[k + 1]; ++q) {
        const double v = partial[static_cast<int64_t>(q) * R + r];
        a = F::op(r) == OP_SUM ? a + v : (F::op(r) == OP_MAX ? fmax(a, v) : fmin(a, v));
    }
    out[k * R + r] = a;
}

struct RedResidM {       // [sum rp^2, max |rp/R|, sum b y]
    const double *rp, *R, *b, *y;
    __device__ static constexpr int op(int r) { return r == 1 ? OP_MAX : OP_SUM; }
    __device__ void operator()(int i, double* v) const {
        v[0] = rp[i] * rp[i];
        v[1] = fabs(rp[i] / R[i]);
        v[2] = b[i] * y[i];
    }
};
struct RedResidN {       // [sum rd^2, max |rd/C|, sum x s, sum c x]
    const double *rd, *C, *x, *s, *c;
    __device__ static constexpr int op(int r) { return r == 1 ? OP_MAX : OP_SUM; }
    __device__ void operator()(int j, double* v) const {
        v[0] = rd[j] * rd[j];
        v[1] = fabs(rd[j] / C[j]);
        v[2] = x[j] * s[j];
        v[3] = c[j] * x[j];
    }
};
struct RedSq {           // [sum a^2]
    const double* a;
    __device__ static constexpr int op(int) { return OP_SUM; }
    __device__ void operator()(int i, double* v) const { v[0] = a[i] * a[i]; }
};
struct RedAbsMax {       // [max |a|]
    const double* a;
    __device__ static constexpr int op(int) { return OP_MAX; }
    __device__ void operator()(int i, double* v) const { v[0] = fabs(a[i]); }
};
struct RedDir {          // [e2^2, e3^2, rxs^2, ratio x, ratio s, x s, x ds, dx s, dx ds]
    const double *e2, *e3, *rxs, *x, *s, *dx, *ds;
    __device__ static constexpr int op(int r) { return (r == 3 || r == 4) ? OP_MIN : OP_SUM; }
    __device__ void operator()(int j, double* v) const {
        v[0] = e2[j] * e2[j];
        v[1] = e3[j] * e3[j];
        v[2] = rxs[j] * rxs[j];
        v[3] = dx[j] < 0.0 ? -x[j] / dx[j] : 1.0e30;
        v[4] = ds[j] < 0.0 ? -s[j] / ds[j] : 1.0e30;
        v[5] = x[j] * s[j];
        v[6] = x[j] * ds[j];
        v[7] = dx[j] * s[j];
        v[8] = dx[j] * ds[j];
    }
};
struct RedTrialM {       // [sum rp^2, sum y^2, max |rp/R|, sum b y]
    const double *rp, *y, *R, *b;
    __device__ static constexpr int op(int r) { return r == 2 ? OP_MAX : OP_SUM; }
    __device__ void operator()(int i, double* v) const {
        v[0] = rp[i] * rp[i];
        v[1] = y[i] * y[i];
        v[2] = fabs(rp[i] / R[i]);
        v[3] = b[i] * y[i];
    }
};
struct RedTrialN {       // [sum rd^2, sum x s, min x, min s, max |rd/C|, sum c x]
    const double *rd, *x, *s, *C, *c;
    __device__ static constexpr int op(int r) { return (r == 2 || r == 3) ? OP_MIN : r == 4 ? OP_MAX : OP_SUM; }
    __device__ void operator()(int j, double* v) const {
        v[0] = rd[j] * rd[j];
        v[1] = x[j] * s[j];
        v[2] = x[j];
        v[3] = s[j];
        v[4] = fabs(rd[j] / C[j]);
        v[5] = c[j] * x[j];
    }
};

// --------------------------------------------------------- elementwise

__global__ void k_fill(int n, double* a, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void k_theta(int n, const double* __restrict__ x, const double* __restrict__ s,
                        const int* __restrict__ col_lp, const double* __restrict__ mask, double* __restrict__ th) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) th[j] = mask[col_lp[j]] != 0.0 ? x[j] / s[j] : 1.0;
}
// r_xs = -x s + target[lp] - (dxa ds a if given); v = -theta rd - r_xs / s
__global__ void k_rhs(int n, const double* __restrict__ x, const double* __restrict__ s,
                      const double* __restrict__ theta, const double* __restrict__ rd, const double* __restrict__ dxa,
                      const double* __restrict__ dsa, const double* __restrict__ target,
                      const int* __restrict__ col_lp, double* __restrict__ rxs, double* __restrict__ v) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double r = -x[j] * s[j] + (target ? target[col_lp[j]] : 0.0);
    if (dxa) r -= dxa[j] * dsa[j];
    rxs[j] = r;
    v[j] = -theta[j] * rd[j] - r / s[j];
}
// trial point: xt = x + ap dx ; st = s + ad ds (n) ; yt = y + ad dy (m)
__global__ void k_trial_n(int n, const double* __restrict__ x, const double* __restrict__ s,
                          const double* __restrict__ dx, const double* __restrict__ ds, const double* __restrict__ ap,
                          const double* __restrict__ ad, const int* __restrict__ col_lp, double* __restrict__ xt,
                          double* __restrict__ st) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int k = col_lp[j];
    xt[j] = x[j] + ap[k] * dx[j];
    st[j] = s[j] + ad[k] * ds[j];
}
__global__ void k_trial_m(int m, const double* __restrict__ y, const double* __restrict__ dy,
                          const double* __restrict__ ad, const int* __restrict__ row_lp, double* __restrict__ yt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) yt[i] = y[i] + ad[row_lp[i]] * dy[i];
}
// dst = mask[lp] ? src : dst
__global__ void k_masked_copy(int n, const double* __restrict__ src, const int* __restrict__ lp_of,
                              const double* __restrict__ mask, double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && mask[lp_of[i]] != 0.0) dst[i] = src[i];
}
// dst += mask[lp] * src
__global__ void k_masked_add(int n, const double* __restrict__ src, const int* __restrict__ lp_of,
                             const double* __restrict__ mask, double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && mask[lp_of[i]] != 0.0) dst[i] += src[i];
}

// s = c - t (t = A^T y); used by the heuristic start
__global__ void k_sub(int n, const double* __restrict__ c, const double* __restrict__ t, double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = c[j] - t[j];
}
// v = max(v + shift[lp], tiny) with the shift per LP
__global__ void k_shift_lp(int n, const double* __restrict__ shift, const int* __restrict__ lp_of,
                           double* __restrict__ v) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        const double t = v[j] + shift[lp_of[j]];
        v[j] = t > 1e-10 ? t : 1e-10;
    }
}
struct RedMin2 {         // [min a, min b]
    const double *a, *b;
    __device__ static constexpr int op(int) { return OP_MIN; }
    __device__ void operator()(int i, double* v) const {
        v[0] = a[i];
        v[1] = b[i];
    }
};
struct RedStart {        // [sum x s, sum x, sum s]
    const double *x, *s;
    __device__ static constexpr int op(int) { return OP_SUM; }
    __device__ void operator()(int j, double* v) const {
        v[0] = x[j] * s[j];
        v[1] = x[j];
        v[2] = s[j];
    }
};

// learned start: x = exp(lx), s = exp(ls), exponents clamped to [-20, 20]
__global__ void k_learned_point(int n, const double* __restrict__ lx, const double* __restrict__ ls,
                                double* __restrict__ x, double* __restrict__ s) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        const double a = lx[j], b = ls[j];
        x[j] = exp(isfinite(a) ? fmin(fmax(a, -20.0), 20.0) : 0.0);
        s[j] = exp(isfinite(b) ? fmin(fmax(b, -20.0), 20.0) : 0.0);
    }
}
// pairs with x_j s_j below floor[lp] are scaled up (both by the same factor) to the floor
__global__ void k_center_floor(int n, const double* __restrict__ floor_lp, const int* __restrict__ lp_of,
                               double* __restrict__ x, double* __restrict__ s) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        const double f = floor_lp[lp_of[j]], p = x[j] * s[j];
        if (p < f && p > 0.0) {
            const double g = sqrt(f / p);
            x[j] *= g;
            s[j] *= g;
        }
    }
}
struct RedRatioNeg {     // [max a with x - a dx >= 0, same for s - a ds]
    const double *x, *dx, *s, *ds;
    __device__ static constexpr int op(int) { return OP_MIN; }
    __device__ void operator()(int j, double* v) const {
        v[0] = dx[j] > 0.0 ? x[j] / dx[j] : 1.0e30;
        v[1] = ds[j] > 0.0 ? s[j] / ds[j] : 1.0e30;
    }
};
// out = a * b
__global__ void k_hadamard(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = a[j] * b[j];
}
// a = keep[lp] != 0 ? a : b
__global__ void k_pick_lp(int n, const double* __restrict__ keep, const int* __restrict__ lp_of,
                          double* __restrict__ a, const double* __restrict__ b) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n && keep[lp_of[j]] == 0.0) a[j] = b[j];
}
// out = log(max(v, 1e-300))
__global__ void k_log_floor(int n, const double* __restrict__ v, double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = log(fmax(v[j], 1e-300));
}

// y += a[lp] * x
__global__ void k_axpy_lp(int n, const double* __restrict__ a, const double* __restrict__ x,
                          const int* __restrict__ lp_of, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double al = a[lp_of[i]];
        if (al != 0.0) y[i] += al * x[i];
    }
}
// p = z + b[lp] * p
__global__ void k_xpby_lp(int n, const double* __restrict__ z, const double* __restrict__ b,
                          const int* __restrict__ lp_of, double* __restrict__ p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + b[lp_of[i]] * p[i];
}

struct RedRZ {           // [max |r|, sum r z]
    const double *r, *z;
    __device__ static constexpr int op(int k) { return k == 0 ? OP_MAX : OP_SUM; }
    __device__ void operator()(int i, double* v) const {
        v[0] = fabs(r[i]);
        v[1] = r[i] * z[i];
    }
};
struct RedDot {          // [sum a b]
    const double *a, *b;
    __device__ static constexpr int op(int) { return OP_SUM; }
    __device__ void operator()(int i, double* v) const { v[0] = a[i] * b[i]; }
};

}  // namespace

void spmv_csr(int rows, const int* rp, const int* ci, const double* v, const double* x, double alpha, double beta,
              double* y, cudaStream_t st) {
    spmv(rows, 8, rp, ci, v, x, EpiAxpby{alpha, beta, y}, st);
    SK_CUDA(cudaGetLastError());
}

// =====================================================================

struct DeviceIPM::Impl {
    sk_options opt;
    int nlp = 0, M = 0, N = 0;
    cudaStream_t st = nullptr;
    Arena arena;
    std::vector<int> m_of, n_of, row_off, col_off;
    std::vector<double> R_h, C_h;           // Ruiz factors (batch order)
    std::vector<double> binf, cinf;         // ||b||_inf, ||c||_inf of the unscaled LPs
    std::vector<int64_t> nnz_lp;            // entries of each LP's A
    int64_t nnz_total = 0;
    // device vectors
    Slot<int> a_rp, a_ci, t_rp, t_ci, row_lp, col_lp, mc_s, mc_e, mc_p, nc_s, nc_e, nc_p;
    Slot<double> a_v, t_v, b, c, R, C;
    Slot<double> x, y, s, rp, rd, theta, rxs, v, rkkt, dy, dx, ds, dxa, dya, dsa, e1, e2, e3;
    Slot<double> xt, yt, stt, rpt, rdt, r, corr, bak, tm, cdx, cdy, cds, crxs, pz, pp, pq;
    Slot<double> kdx, kdy, kds;             // directions kept while a direction is redone for some LPs
    Slot<double> scal;                      // per-LP scalars [8][nlp]
    Slot<double> partial, redout;
    int max_chunks = 0;
    // host per-LP state
    std::vector<LpResult> res;
    std::vector<char> active, user_start;
    std::vector<double> rp0, rd0, mu0;
    int factorizations = 0, solves = 0, refine_steps = 0, precision_path = 0, last_pcg = 0;
    bool switched = false, used_fp32 = false;
    // Per-LP precision of a mixed solve: sw[k] once LP k has moved to FP64 fronts for
    // good; sw_now[k] the fronts LP k uses in the current factorisation (a start-point
    // factorisation can fall back to FP64 without a permanent switch); pcg_k[k] the
    // most PCG steps of LP k's solves in the current iteration.
    std::vector<char> sw, sw_now;
    std::vector<int> pcg_k;
    double solve_ms = 0.0, device_ms = 0.0;
    double factor_ms32 = 0.0, factor_ms64 = 0.0;   // device time of the run's factorisations
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<double> hx0, hy0, hs0;      // user start (scaled)
    SpmvShape ga, gt;                       // SpMV launch shapes of A and A^T (autotuned at set-up)
    SpmvTuning tune_a, tune_t;
    SpmvWindows win_a, win_t;               // shared-memory chunk tables of A and A^T
    Gnn* gnn = nullptr;                     // network of SK_START_LEARNED (not owned)
    double capture_mu = 0.0;                // iterate capture for training targets
    std::vector<char> captured;
    double *cap_lx = nullptr, *cap_ls = nullptr, *cap_y = nullptr;
    double *mx0 = nullptr, *my0 = nullptr, *ms0 = nullptr;   // Mehrotra's start kept for learned-start restarts
    std::vector<int> short_steps, loose_count;
    std::vector<char> reinit;

    double* sc(int which) { return scal.ptr + static_cast<size_t>(which) * nlp; }
    double* tmpn() { return crxs.ptr; }   // scratch n-vector outside the backtracking phase
    void put_scalars(int which, const std::vector<double>& v) {
        SK_CUDA(cudaMemcpyAsync(sc(which), v.data(), sizeof(double) * nlp, cudaMemcpyHostToDevice, st));
    }

    template <int R, class F>
    void reduce_rows(F f, double* out_dev) {
        k_reduce<R><<<static_cast<int>(mc_s.count), 256, 0, st>>>(mc_s.ptr, mc_e.ptr, f, partial.ptr);
        k_reduce_final<R, F><<<nblk(static_cast<int64_t>(nlp) * R), 256, 0, st>>>(nlp, mc_p.ptr, partial.ptr, out_dev);
    }
    template <int R, class F>
    void reduce_cols(F f, double* out_dev) {
        k_reduce<R><<<static_cast<int>(nc_s.count), 256, 0, st>>>(nc_s.ptr, nc_e.ptr, f, partial.ptr);
        k_reduce_final<R, F><<<nblk(static_cast<int64_t>(nlp) * R), 256, 0, st>>>(nlp, nc_p.ptr, partial.ptr, out_dev);
    }
    // copies `count` doubles of redout to host (synchronising)
    std::vector<double> fetch(size_t count) {
        std::vector<double> h(count);
        SK_CUDA(cudaMemcpyAsync(h.data(), redout.ptr, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
        return h;
    }
};

DeviceIPM::DeviceIPM(const std::vector<ipm::LpView>& lps, const std::vector<const double*>& bvec,
                     const std::vector<const double*>& cvec, const sk_options& opt)
    : im_(new Impl) {
    auto t0 = std::chrono::steady_clock::now();
    Impl& I = *im_;
    I.opt = opt;
    nlp_ = I.nlp = static_cast<int>(lps.size());
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw api::sk_exception(SK_ERR_NO_DEVICE, "no CUDA device visible");
    SK_CUDA(cudaStreamCreateWithFlags(&I.st, cudaStreamNonBlocking));
    I.row_off.assign(I.nlp + 1, 0);
    I.col_off.assign(I.nlp + 1, 0);
    for (int k = 0; k < I.nlp; ++k) {
        if (lps[k].m <= 0 || lps[k].n <= 0) throw api::sk_exception(SK_ERR_INVALID, "every LP needs m, n >= 1");
        I.row_off[k + 1] = I.row_off[k] + lps[k].m;
        I.col_off[k + 1] = I.col_off[k] + lps[k].n;
    }
    I.M = I.row_off[I.nlp];
    I.N = I.col_off[I.nlp];
    const int M = I.M, N = I.N;
    // --- Ruiz scaling per LP (mehrotra_device.cu:289-323) and batch CSC / CSR. The LPs
    // are independent and own disjoint ranges of every array (LP k's entries sit at
    // [nz_off[k], nz_off[k + 1]) in the CSC and in the CSR order alike, A being block
    // diagonal), so they are processed on worker threads with the same results.
    std::vector<int64_t> nz_off(static_cast<size_t>(I.nlp) + 1, 0);
    for (int k = 0; k < I.nlp; ++k) nz_off[k + 1] = nz_off[k] + lps[k].col_ptrs[lps[k].n];
    const int64_t nnz = nz_off[I.nlp];
    if (nnz >= (int64_t(1) << 31)) throw api::sk_exception(SK_ERR_TOO_LARGE, "batch exceeds 2^31 nonzeros");
    std::vector<int> cp(static_cast<size_t>(N) + 1, 0), ri(static_cast<size_t>(nnz));
    std::vector<double> cv(static_cast<size_t>(nnz));
    std::vector<double> hb(M), hc(N);
    I.R_h.assign(M, 1.0);
    I.C_h.assign(N, 1.0);
    I.binf.assign(I.nlp, 0.0);
    I.cinf.assign(I.nlp, 0.0);
    core::CSRMatrix A;
    A.rows = M;
    A.cols = N;
    A.row_ptrs.assign(static_cast<size_t>(M) + 1, 0);
    A.col_indices.resize(static_cast<size_t>(nnz));
    A.values.resize(static_cast<size_t>(nnz));
    std::vector<ipm::LpView> sl(I.nlp);
    std::vector<std::vector<int>> lcp(I.nlp), lri(I.nlp);
    std::vector<std::string> bad(I.nlp);
    auto one_lp = [&](int k) {
        const auto& l = lps[k];
        const int ro = I.row_off[k], co = I.col_off[k];
        int64_t pos = nz_off[k];
        for (int j = 0; j < l.n; ++j) {
            cp[co + j] = static_cast<int>(pos);
            for (int q = l.col_ptrs[j]; q < l.col_ptrs[j + 1]; ++q) {
                if (l.row_idx[q] < 0 || l.row_idx[q] >= l.m) { bad[k] = "row index out of range"; return; }
                ri[pos] = ro + l.row_idx[q];
                cv[pos] = l.vals[q];
                ++pos;
            }
        }
        const int64_t end = pos;
        for (int i = 0; i < l.m; ++i) { hb[ro + i] = bvec[k][i]; I.binf[k] = std::max(I.binf[k], std::fabs(bvec[k][i])); }
        for (int j = 0; j < l.n; ++j) { hc[co + j] = cvec[k][j]; I.cinf[k] = std::max(I.cinf[k], std::fabs(cvec[k][j])); }
        std::vector<double> rmax, cmax;
        for (int pass = 0; pass < opt.ruiz_passes; ++pass) {
            rmax.assign(l.m, 0.0);
            cmax.assign(l.n, 0.0);
            for (int j = 0; j < l.n; ++j)
                for (int64_t q = cp[co + j]; q < (j + 1 < l.n ? cp[co + j + 1] : end); ++q) {
                    const double a = std::fabs(cv[q]);
                    rmax[ri[q] - ro] = std::max(rmax[ri[q] - ro], a);
                    cmax[j] = std::max(cmax[j], a);
                }
            for (int i = 0; i < l.m; ++i) {
                const double f = rmax[i] > 1e-8 ? 1.0 / std::sqrt(rmax[i]) : 1.0;
                I.R_h[ro + i] *= f; hb[ro + i] *= f; rmax[i] = f;
            }
            for (int j = 0; j < l.n; ++j) {
                const double f = cmax[j] > 1e-8 ? 1.0 / std::sqrt(cmax[j]) : 1.0;
                I.C_h[co + j] *= f; hc[co + j] *= f; cmax[j] = f;
            }
            for (int j = 0; j < l.n; ++j)
                for (int64_t q = cp[co + j]; q < (j + 1 < l.n ? cp[co + j + 1] : end); ++q)
                    cv[q] *= rmax[ri[q] - ro] * cmax[j];
        }
        for (int i = 0; i < l.m; ++i) if (!std::isfinite(hb[ro + i])) { bad[k] = "non-finite b"; return; }
        for (int j = 0; j < l.n; ++j) if (!std::isfinite(hc[co + j])) { bad[k] = "non-finite c"; return; }
        for (int64_t q = nz_off[k]; q < end; ++q) if (!std::isfinite(cv[q])) { bad[k] = "non-finite A"; return; }
        // this LP's rows of the batch CSR (its entries keep their range)
        std::vector<int> cnt(static_cast<size_t>(l.m) + 1, 0);
        for (int64_t q = nz_off[k]; q < end; ++q) cnt[ri[q] - ro + 1]++;
        for (int i = 0; i < l.m; ++i) cnt[i + 1] += cnt[i];
        for (int i = 0; i < l.m; ++i) A.row_ptrs[ro + i + 1] = static_cast<int>(nz_off[k] + cnt[i + 1]);
        std::vector<int64_t> nx(static_cast<size_t>(l.m));
        for (int i = 0; i < l.m; ++i) nx[i] = nz_off[k] + cnt[i];
        for (int j = 0; j < l.n; ++j)
            for (int q = cp[co + j]; q < (j + 1 < l.n ? cp[co + j + 1] : static_cast<int>(end)); ++q) {
                const int64_t d = nx[ri[q] - ro]++;
                A.col_indices[d] = co + j;
                A.values[d] = cv[q];
            }
        // this LP's scaled view (local indices) for the symbolic plan
        lcp[k].resize(l.n + 1);
        for (int j = 0; j < l.n; ++j) lcp[k][j] = static_cast<int>(cp[co + j] - nz_off[k]);
        lcp[k][l.n] = static_cast<int>(end - nz_off[k]);
        lri[k].resize(lcp[k].back());
        for (int64_t q = nz_off[k]; q < end; ++q) lri[k][q - nz_off[k]] = ri[q] - ro;
        sl[k].m = l.m;
        sl[k].n = l.n;
        sl[k].col_ptrs = lcp[k].data();
        sl[k].row_idx = lri[k].data();
        sl[k].vals = cv.data() + nz_off[k];
    };
    {
        const int nt = static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
        std::atomic<int> next{0};
        auto work = [&]() {
            for (int k = next++; k < I.nlp; k = next++) one_lp(k);
        };
        if (nt <= 1 || I.nlp <= 1 || nnz < 100000) {
            work();
        } else {
            std::vector<std::thread> pool;
            for (int t = 0; t < std::min(nt, I.nlp); ++t) pool.emplace_back(work);
            for (auto& th : pool) th.join();
        }
    }
    for (int k = 0; k < I.nlp; ++k)
        if (!bad[k].empty()) throw api::sk_exception(SK_ERR_INVALID, bad[k]);
    cp[N] = static_cast<int>(nnz);
    I.nnz_lp.assign(I.nlp, 0);
    for (int k = 0; k < I.nlp; ++k) I.nnz_lp[k] = static_cast<int64_t>(cp[I.col_off[k + 1]]) - cp[I.col_off[k]];
    I.nnz_total = static_cast<int64_t>(nnz);
    ipm::FrontPlan plan;
    ipm::build_front_plan(sl, A, opt.ordering, plan);
    lcp.clear();
    lri.clear();
    // --- device upload
    std::vector<int> h_row_lp(M), h_col_lp(N);
    for (int k = 0; k < I.nlp; ++k) {
        for (int i = I.row_off[k]; i < I.row_off[k + 1]; ++i) h_row_lp[i] = k;
        for (int j = I.col_off[k]; j < I.col_off[k + 1]; ++j) h_col_lp[j] = k;
    }
    std::vector<int> ms, me, mp, ns_, ne, np_;
    make_chunks(I.row_off, kChunk, ms, me, mp);
    make_chunks(I.col_off, kChunk, ns_, ne, np_);
    I.max_chunks = static_cast<int>(std::max(ms.size(), ns_.size()));
    Arena& ar = I.arena;
    reserve(ar, I.a_rp, M + 1); reserve(ar, I.a_ci, nnz); reserve(ar, I.a_v, nnz);
    reserve(ar, I.t_rp, N + 1); reserve(ar, I.t_ci, nnz); reserve(ar, I.t_v, nnz);
    reserve(ar, I.b, M); reserve(ar, I.c, N); reserve(ar, I.R, M); reserve(ar, I.C, N);
    reserve(ar, I.row_lp, M); reserve(ar, I.col_lp, N);
    reserve(ar, I.mc_s, ms.size()); reserve(ar, I.mc_e, me.size()); reserve(ar, I.mc_p, mp.size());
    reserve(ar, I.nc_s, ns_.size()); reserve(ar, I.nc_e, ne.size()); reserve(ar, I.nc_p, np_.size());
    for (auto* sl2 : {&I.x, &I.s, &I.rd, &I.theta, &I.rxs, &I.v, &I.dx, &I.ds, &I.dxa, &I.dsa, &I.e2, &I.e3, &I.xt,
                      &I.stt, &I.rdt, &I.cdx, &I.cds, &I.crxs, &I.kdx, &I.kds})
        reserve(ar, *sl2, N);
    for (auto* sl2 : {&I.y, &I.rp, &I.rkkt, &I.dy, &I.dya, &I.e1, &I.yt, &I.rpt, &I.r, &I.corr, &I.bak, &I.tm, &I.cdy,
                      &I.pz, &I.pp, &I.pq, &I.kdy})
        reserve(ar, *sl2, M);
    reserve(ar, I.scal, static_cast<size_t>(8) * I.nlp);
    reserve(ar, I.partial, static_cast<size_t>(I.max_chunks) * kMaxR);
    reserve(ar, I.redout, static_cast<size_t>(I.nlp) * 2 * kMaxR);
    ar.commit();
    for (auto* sl2 : {&I.a_rp, &I.a_ci, &I.t_rp, &I.t_ci, &I.row_lp, &I.col_lp, &I.mc_s, &I.mc_e, &I.mc_p, &I.nc_s,
                      &I.nc_e, &I.nc_p})
        bind(ar, *sl2);
    for (auto* sl2 : {&I.a_v, &I.t_v, &I.b, &I.c, &I.R, &I.C, &I.x, &I.s, &I.rd, &I.theta, &I.rxs, &I.v, &I.dx, &I.ds,
                      &I.dxa, &I.dsa, &I.e2, &I.e3, &I.xt, &I.stt, &I.rdt, &I.cdx, &I.cds, &I.crxs, &I.y, &I.rp,
                      &I.rkkt, &I.dy, &I.dya, &I.e1, &I.yt, &I.rpt, &I.r, &I.corr, &I.bak, &I.tm, &I.cdy, &I.scal,
                      &I.partial, &I.redout, &I.pz, &I.pp, &I.pq, &I.kdx, &I.kds, &I.kdy})
        bind(ar, *sl2);
    upload(I.a_rp, A.row_ptrs, I.st); upload(I.a_ci, A.col_indices, I.st); upload(I.a_v, A.values, I.st);
    upload(I.t_rp, cp, I.st); upload(I.t_ci, ri, I.st); upload(I.t_v, cv, I.st);
    upload(I.b, hb, I.st); upload(I.c, hc, I.st); upload(I.R, I.R_h, I.st); upload(I.C, I.C_h, I.st);
    upload(I.row_lp, h_row_lp, I.st); upload(I.col_lp, h_col_lp, I.st);
    upload(I.mc_s, ms, I.st); upload(I.mc_e, me, I.st); upload(I.mc_p, mp, I.st);
    upload(I.nc_s, ns_, I.st); upload(I.nc_e, ne, I.st); upload(I.nc_p, np_, I.st);
    // lane-group widths of A x and A^T y, timed on this batch (x and y zeroed first
    // so the timed launches read defined values)
    SK_CUDA(cudaMemsetAsync(I.x.ptr, 0, sizeof(double) * N, I.st));
    SK_CUDA(cudaMemsetAsync(I.y.ptr, 0, sizeof(double) * M, I.st));
    I.win_a.build(M, I.a_rp.ptr, I.a_ci.ptr, I.st);
    I.win_t.build(N, I.t_rp.ptr, I.t_ci.ptr, I.st);
    I.tune_a = spmv_tune(M, N, nnz, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, I.x.ptr, I.r.ptr, I.st, &I.win_a);
    I.tune_t = spmv_tune(N, M, nnz, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, I.y.ptr, I.v.ptr, I.st, &I.win_t);
    I.ga = I.win_a.shape(I.tune_a.group, I.tune_a.windowed);
    I.gt = I.win_t.shape(I.tune_t.group, I.tune_t.windowed);
    if (opt.verbose)
        std::fprintf(stderr, "[sankhya] SpMV: A %d lanes per row%s (rule %d), A^T %d%s (rule %d)\n", I.ga.group,
                     I.ga.windowed ? ", shared-memory windows" : "", I.tune_a.heuristic, I.gt.group,
                     I.gt.windowed ? ", shared-memory windows" : "", I.tune_t.heuristic);
    lp_.nlp = I.nlp; lp_.M = M; lp_.N = N; lp_.nnz = nnz;
    lp_.a_rp = I.a_rp.ptr; lp_.a_ci = I.a_ci.ptr; lp_.a_v = I.a_v.ptr;
    lp_.t_rp = I.t_rp.ptr; lp_.t_ci = I.t_ci.ptr; lp_.t_v = I.t_v.ptr;
    lp_.b = I.b.ptr; lp_.c = I.c.ptr; lp_.R = I.R.ptr; lp_.C = I.C.ptr;
    lp_.row_lp = I.row_lp.ptr; lp_.col_lp = I.col_lp.ptr;
    lp_.n_mchunks = static_cast<int>(ms.size()); lp_.n_nchunks = static_cast<int>(ns_.size());
    lp_.mc_start = I.mc_s.ptr; lp_.mc_end = I.mc_e.ptr; lp_.mc_ptr = I.mc_p.ptr;
    lp_.nc_start = I.nc_s.ptr; lp_.nc_end = I.nc_e.ptr; lp_.nc_ptr = I.nc_p.ptr;
    lp_.spmv_group_A = I.ga.group; lp_.spmv_group_T = I.gt.group;
    kkt_.reset(new KktEngine(plan, lp_, I.st));
    SK_CUDA(cudaStreamSynchronize(I.st));
    I.res.assign(I.nlp, LpResult());
    I.user_start.assign(I.nlp, 0);
    setup_ms_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void DeviceIPM::profile(bool fp32, bool tensor, double* out18) {
    Impl& I = *im_;
    std::vector<double> ones(I.nlp, 1.0);
    I.put_scalars(0, ones);
    k_theta<<<nblk(I.N), 256, 0, I.st>>>(I.N, I.x.ptr, I.s.ptr, I.col_lp.ptr, I.sc(0), I.theta.ptr);
    k_fill<<<nblk(I.M), 256, 0, I.st>>>(I.M, I.r.ptr, 1.0);
    kkt_->set_active(std::vector<char>(I.nlp, 1));   // every front, whatever the last run left on
    kkt_->set_tensor_update(tensor);
    kkt_->profile(I.theta.ptr, fp32 ? 1e-7 : 1e-9, fp32, I.r.ptr, I.corr.ptr, out18);
}

DeviceIPM::~DeviceIPM() {
    if (im_ && im_->ev0) { cudaEventDestroy(im_->ev0); cudaEventDestroy(im_->ev1); }
    if (im_) for (double* p : {im_->cap_lx, im_->cap_ls, im_->cap_y, im_->mx0, im_->my0, im_->ms0}) if (p) cudaFree(p);
    kkt_.reset();
    if (im_ && im_->st) cudaStreamDestroy(im_->st);
}

void DeviceIPM::set_start(int lp, const double* x, const double* y, const double* s) {
    Impl& I = *im_;
    if (lp < 0 || lp >= I.nlp || !x || !y || !s) throw api::sk_exception(SK_ERR_INVALID, "set_start: bad argument");
    if (I.hx0.empty()) { I.hx0.assign(I.N, 1.0); I.hy0.assign(I.M, 0.0); I.hs0.assign(I.N, 1.0); }
    const int ro = I.row_off[lp], co = I.col_off[lp];
    for (int j = 0; j < I.col_off[lp + 1] - co; ++j) {
        I.hx0[co + j] = x[j] / I.C_h[co + j];       // x_scaled = C^{-1} x
        I.hs0[co + j] = s[j] * I.C_h[co + j];       // s_scaled = C s
    }
    for (int i = 0; i < I.row_off[lp + 1] - ro; ++i) I.hy0[ro + i] = y[i] / I.R_h[ro + i];
    I.user_start[lp] = 1;
}

void DeviceIPM::set_gnn(Gnn* g) { im_->gnn = g; }

void DeviceIPM::set_capture(double mu) {
    Impl& I = *im_;
    if (!(mu >= 0.0)) throw api::sk_exception(SK_ERR_INVALID, "set_capture: mu must be >= 0");
    I.capture_mu = mu;
    if (mu > 0.0 && !I.cap_lx) {
        SK_CUDA(cudaMalloc(&I.cap_lx, sizeof(double) * I.N));
        SK_CUDA(cudaMalloc(&I.cap_ls, sizeof(double) * I.N));
        SK_CUDA(cudaMalloc(&I.cap_y, sizeof(double) * I.M));
    }
    I.captured.assign(I.nlp, 0);
}

bool DeviceIPM::capture_complete() const {
    const Impl& I = *im_;
    if (!(I.capture_mu > 0.0) || static_cast<int>(I.captured.size()) != I.nlp) return false;
    for (char c : I.captured) if (!c) return false;
    return true;
}
const double* DeviceIPM::capture_logx() const { return im_->cap_lx; }
const double* DeviceIPM::capture_logs() const { return im_->cap_ls; }
const double* DeviceIPM::capture_y() const { return im_->cap_y; }

void DeviceIPM::run() {
    Impl& I = *im_;
    KktEngine& K = *kkt_;
    const int M = I.M, N = I.N, nlp = I.nlp;
    cudaStream_t st = I.st;
    auto t0 = std::chrono::steady_clock::now();
    if (!I.ev0) {
        SK_CUDA(cudaEventCreate(&I.ev0));
        SK_CUDA(cudaEventCreate(&I.ev1));
    }
    SK_CUDA(cudaEventRecord(I.ev0, st));
    K.reset_factor_time();
    const auto& o = I.opt;
    if (o.start == SK_START_LEARNED && !I.gnn)
        throw api::sk_exception(SK_ERR_INVALID, "SK_START_LEARNED needs a network (sk_solver_set_gnn)");
    if (I.capture_mu > 0.0) I.captured.assign(nlp, 0);
    I.factorizations = I.solves = I.refine_steps = 0;
    I.switched = false;
    I.used_fp32 = false;
    I.res.assign(nlp, LpResult());
    I.active.assign(nlp, 1);
    I.sw.assign(nlp, o.precision == SK_PREC_FP64 ? 1 : 0);
    I.sw_now = I.sw;
    I.pcg_k.assign(nlp, 0);
    K.set_active(I.active);
    I.rp0.assign(nlp, 1.0);
    I.rd0.assign(nlp, 1.0);
    I.mu0.assign(nlp, 1.0);
    // start point
    k_fill<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, 1.0);
    k_fill<<<nblk(N), 256, 0, st>>>(N, I.s.ptr, 1.0);
    k_fill<<<nblk(M), 256, 0, st>>>(M, I.y.ptr, 0.0);
    if (o.start == SK_START_USER && !I.hx0.empty()) {
        SK_CUDA(cudaMemcpyAsync(I.x.ptr, I.hx0.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
        SK_CUDA(cudaMemcpyAsync(I.y.ptr, I.hy0.data(), sizeof(double) * M, cudaMemcpyHostToDevice, st));
        SK_CUDA(cudaMemcpyAsync(I.s.ptr, I.hs0.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
        for (int k = 0; k < nlp; ++k) I.res[k].learned_start = I.user_start[k];
    }
    std::vector<double> nrp(nlp, 1.0), nrd(nlp, 1.0), mu(nlp), nm(nlp), nn(nlp);
    for (int k = 0; k < nlp; ++k) {
        nm[k] = I.row_off[k + 1] - I.row_off[k];
        nn[k] = I.col_off[k + 1] - I.col_off[k];
    }
    std::vector<double> mask(nlp), ap(nlp), ad(nlp), tgt(nlp), tol(nlp);
    double* d_mask = I.sc(0);
    double* d_ap = I.sc(1);
    double* d_ad = I.sc(2);
    double* d_tgt = I.sc(3);
    double* d_rmask = I.sc(4);

    auto residuals = [&](const double* x, const double* y, const double* s, double* rp, double* rd) {
        spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, x, EpiSub{I.b.ptr, rp}, st);
        spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, y, EpiRd{s, I.c.ptr, rd}, st);
    };
    // unscaled measures of LP k from the residual reductions
    auto record = [&](int k, const double* hm, const double* hn) {
        LpResult& r = I.res[k];
        r.primal_residual = std::sqrt(hm[k * 3 + 0]);
        r.dual_residual = std::sqrt(hn[k * 4 + 0]);
        r.duality_gap = hn[k * 4 + 2] / nn[k];
        r.objective = hn[k * 4 + 3];
        const double by = hm[k * 3 + 2];
        r.rel_pinf = hm[k * 3 + 1] / (1.0 + I.binf[k]);
        r.rel_dinf = hn[k * 4 + 1] / (1.0 + I.cinf[k]);
        r.rel_gap = std::fabs(r.objective - by) / (1.0 + std::fabs(r.objective) + std::fabs(by));
    };
    // ---- normal-equation solve M0 dy = rhs, returns per-LP success (||r||_inf <= tol).
    // Strict mode: the reference's iterative refinement (up to 10 steps, rollback on
    // stagnation; src/cuda/kkt.cu:778-842). Default: preconditioned conjugate
    // gradients with the regularised factor as preconditioner (the iterative
    // refinement stalls once A Theta A^T is nearly singular), keeping each LP's best
    // iterate. Vectors and the operator are FP64 in both cases.
    auto normal_apply = [&](const double* xx, double* out) {   // out = A Theta A^T xx
        spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, xx, EpiTheta{I.theta.ptr, K.scratch_n()}, st);
        spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, K.scratch_n(), EpiAxpby{1.0, 0.0, out}, st);
    };
    // the same for the rows and columns of the LPs with a nonzero entry in d_on only
    // (the batch is block diagonal: their rows of out are exact, the others' are left
    // as they were)
    double* d_on = I.sc(5);
    auto normal_apply_some = [&](const double* xx, double* out) {
        spmv_masked(N, I.gt.group, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, xx, I.col_lp.ptr, d_on,
                    EpiTheta{I.theta.ptr, K.scratch_n()}, st);
        spmv_masked(M, I.ga.group, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, K.scratch_n(), I.row_lp.ptr, d_on,
                    EpiAxpby{1.0, 0.0, out}, st);
    };
    auto resid_norm = [&](const double* rhs, const double* xx) {   // I.r = rhs - M0 xx, returns max|r| per LP
        spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, xx, EpiTheta{I.theta.ptr, K.scratch_n()}, st);
        spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, K.scratch_n(), EpiRhsMinus{rhs, I.r.ptr}, st);
        I.reduce_rows<1>(RedAbsMax{I.r.ptr}, I.redout.ptr);
        return I.fetch(nlp);
    };
    // which (optional): solve for these LPs only; the others' rows of out are not
    // meaningful afterwards and their ok entries are left as they are
    auto solve = [&](const double* rhs, double* out, std::vector<char>& ok, const std::vector<char>* which = nullptr) {
        ++I.solves;
        // verbose >= 3: per-solve timing (the stream is drained first, so the time is this solve's)
        const bool trace = o.verbose >= 3;
        if (trace) SK_CUDA(cudaStreamSynchronize(st));
        const auto ts0 = std::chrono::steady_clock::now();
        const int steps0 = I.refine_steps;
        if (which) K.restrict_solves(*which);
        K.apply_inverse(rhs, out);
        if (which) K.unrestrict_solves();
        std::vector<double> rn = resid_norm(rhs, out);
        std::vector<char> done(nlp, 0), stag(nlp, 0);
        I.last_pcg = 0;
        std::vector<int> steps(nlp, 0);
        for (int k = 0; k < nlp; ++k) done[k] = !I.active[k] || (which && !(*which)[k]) || rn[k] <= tol[k];
        if (o.strict) {
            for (int it = 0; it < 10; ++it) {
                bool any = false;
                std::vector<double> rm(nlp);
                for (int k = 0; k < nlp; ++k) { rm[k] = (!done[k] && !stag[k]) ? 1.0 : 0.0; any |= rm[k] != 0.0; }
                if (!any) break;
                ++I.refine_steps;
                I.put_scalars(4, rm);
                SK_CUDA(cudaMemcpyAsync(I.bak.ptr, out, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
                K.apply_inverse(I.r.ptr, I.corr.ptr);
                k_masked_add<<<nblk(M), 256, 0, st>>>(M, I.corr.ptr, I.row_lp.ptr, d_rmask, out);
                std::vector<double> rn2 = resid_norm(rhs, out);
                std::vector<double> roll(nlp, 0.0);
                bool any_roll = false;
                for (int k = 0; k < nlp; ++k) {
                    if (rm[k] == 0.0) continue;
                    if (rn2[k] <= tol[k]) { done[k] = 1; rn[k] = rn2[k]; }
                    else if (rn2[k] >= rn[k]) { stag[k] = 1; roll[k] = 1.0; any_roll = true; }
                    else rn[k] = rn2[k];
                }
                if (any_roll) {
                    I.put_scalars(4, roll);
                    k_masked_copy<<<nblk(M), 256, 0, st>>>(M, I.bak.ptr, I.row_lp.ptr, d_rmask, out);
                }
            }
        } else {
            bool any = false;
            for (int k = 0; k < nlp; ++k) any |= !done[k];
            if (any) {
                // PCG steps per LP: 30 on FP32 fronts, 60 on FP64 fronts
                auto limit = [&](int k) { return I.sw_now[k] ? 60 : 30; };
                const int max_it = 60;
                std::vector<double> best = rn, rz(nlp, 0.0), al(nlp, 0.0), be(nlp, 0.0), imp(nlp, 0.0);
                SK_CUDA(cudaMemcpyAsync(I.bak.ptr, out, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
                // preconditioner applications cover only the LPs still iterating (the
                // others' rows come out 0, and their step sizes are 0)
                // and while their entries are under half of A's, A Theta A^T p is formed
                // for their rows alone
                std::vector<char> sub(nlp, 0);
                std::vector<double> subd(nlp, 0.0);
                bool few = false;
                auto restrict_to_running = [&]() {
                    int64_t nz = 0;
                    for (int k = 0; k < nlp; ++k) {
                        sub[k] = !done[k] && !stag[k];
                        subd[k] = sub[k] ? 1.0 : 0.0;
                        if (sub[k]) nz += I.nnz_lp[k];
                    }
                    K.restrict_solves(sub);
                    few = 2 * nz < I.nnz_total;
                    if (few) I.put_scalars(5, subd);
                };
                restrict_to_running();
                K.apply_inverse(I.r.ptr, I.pz.ptr);
                SK_CUDA(cudaMemcpyAsync(I.pp.ptr, I.pz.ptr, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
                I.reduce_rows<1>(RedDot{I.r.ptr, I.pz.ptr}, I.redout.ptr);
                rz = I.fetch(nlp);
                int last_best_it = 0;
                for (int it = 0; it < max_it; ++it) {
                    ++I.refine_steps;
                    if (few) normal_apply_some(I.pp.ptr, I.pq.ptr);
                    else normal_apply(I.pp.ptr, I.pq.ptr);
                    I.reduce_rows<1>(RedDot{I.pp.ptr, I.pq.ptr}, I.redout.ptr);
                    std::vector<double> pq = I.fetch(nlp);
                    bool run = false;
                    for (int k = 0; k < nlp; ++k) {
                        al[k] = 0.0;
                        if (done[k] || stag[k]) continue;
                        if (it >= limit(k)) { stag[k] = 1; continue; }
                        if (!(pq[k] > 0.0) || !(rz[k] > 0.0) || !std::isfinite(pq[k])) { stag[k] = 1; continue; }
                        steps[k] = it + 1;
                        al[k] = rz[k] / pq[k];
                        run = true;
                    }
                    if (!run) break;
                    I.put_scalars(1, al);
                    k_axpy_lp<<<nblk(M), 256, 0, st>>>(M, d_ap, I.pp.ptr, I.row_lp.ptr, out);
                    for (auto& v : al) v = -v;
                    I.put_scalars(1, al);
                    k_axpy_lp<<<nblk(M), 256, 0, st>>>(M, d_ap, I.pq.ptr, I.row_lp.ptr, I.r.ptr);
                    restrict_to_running();
                    K.apply_inverse(I.r.ptr, I.pz.ptr);
                    I.reduce_rows<2>(RedRZ{I.r.ptr, I.pz.ptr}, I.redout.ptr);
                    std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 2);
                    bool improved = false;
                    for (int k = 0; k < nlp; ++k) {
                        imp[k] = 0.0;
                        be[k] = 0.0;
                        if (done[k] || stag[k]) continue;
                        const double rnk = h[k * 2], rz2 = h[k * 2 + 1];
                        if (rnk < best[k]) { best[k] = rnk; imp[k] = 1.0; improved = true; }
                        if (rnk <= tol[k]) { done[k] = 1; continue; }
                        if (!(rz2 > 0.0) || !std::isfinite(rz2)) { stag[k] = 1; continue; }
                        be[k] = rz2 / rz[k];
                        rz[k] = rz2;
                    }
                    if (improved) {
                        last_best_it = it;
                        I.put_scalars(4, imp);
                        k_masked_copy<<<nblk(M), 256, 0, st>>>(M, out, I.row_lp.ptr, d_rmask, I.bak.ptr);
                    }
                    if (it - last_best_it > 8) break;   // no progress for a while
                    I.put_scalars(2, be);
                    k_xpby_lp<<<nblk(M), 256, 0, st>>>(M, I.pz.ptr, d_ad, I.row_lp.ptr, I.pp.ptr);
                }
                K.unrestrict_solves();
                SK_CUDA(cudaMemcpyAsync(out, I.bak.ptr, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
                rn = resid_norm(rhs, out);
                I.last_pcg = last_best_it + 1;
                for (int k = 0; k < nlp; ++k) I.pcg_k[k] = std::max(I.pcg_k[k], steps[k]);
                if (o.verbose > 1)
                    std::fprintf(stderr, "[sk]   pcg steps %d resid %.3e tol %.3e\n", last_best_it + 1, rn[0], tol[0]);
            }
        }
        if (K.solve_error())
            throw api::sk_exception(SK_ERR_CUDA, "triangular solve: a task timed out waiting for a dependency");
        if (trace) {
            int na = 0, nd = 0;
            for (int k = 0; k < nlp; ++k) { na += I.active[k] != 0; nd += I.active[k] && !done[k]; }
            std::fprintf(stderr, "[sk] solve: %d active LPs, %d needed refinement, %d steps, %.3f ms\n", na, nd,
                         I.refine_steps - steps0,
                         std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - ts0).count());
        }
        ok.resize(nlp, 0);
        for (int k = 0; k < nlp; ++k)
            if (!which || (*which)[k]) ok[k] = !I.active[k] || rn[k] <= tol[k];
    };
    // ---- factorisation with delta retries and the precision policy
    // delta: the reference's 1e-9 x10 ladder in strict mode (src/cuda/kkt.cu:35, 665-669);
    // otherwise 1e-12 x10 for FP64 fronts (a tighter preconditioner keeps PCG short
    // once A Theta A^T is nearly singular) and 1e-7 x10 for FP32 fronts.
    // FP32 trailing updates run on the tensor cores (TF32 x3) while mu >= kTensorMu; the
    // last FP32 iterations, whose directions decide the FP64 switch, use exact FP32.
    bool tensor_now = true;
    // One precision's fronts (the LPs of that precision's mask) through the delta
    // ladder. The LPs are independent blocks of one matrix: after a pass in which some
    // of them had a pivot that was not positive, only those are assembled and factored
    // again, with delta x10, while the others keep the factors they have. On failure
    // ladder_failed holds the LPs that failed every pass.
    const bool emulate64 = o.fp64_update == SK_FP64_UPDATE_TENSOR ||
                           (o.fp64_update == SK_FP64_UPDATE_AUTO && o.precision == SK_PREC_MIXED);
    std::vector<char> ladder_failed;
    auto ladder = [&](bool want_fp32) -> bool {
        K.set_tensor_update(tensor_now);
        K.set_fp64_emulation(emulate64);
        double delta = want_fp32 ? o.delta32 : (o.strict ? 1e-9 : o.delta64);
        const std::vector<char> m32(K.mask32().begin(), K.mask32().end());
        const std::vector<char> m64(K.mask64().begin(), K.mask64().end());
        std::vector<char> pend = want_fp32 ? m32 : m64;
        bool ok = false, narrowed = false;
        for (int retry = 0; retry < (o.strict ? 5 : 6); ++retry, delta *= 10.0) {
            ++I.factorizations;
            const double f0 = K.factor_ms(want_fp32);
            const bool fok = K.factor(I.theta.ptr, delta, want_fp32);
            if (o.verbose >= 3) {
                const std::vector<int>& on = want_fp32 ? K.mask32() : K.mask64();
                std::fprintf(stderr, "[sk] factor %s: %d LPs, delta %.0e, %.3f ms\n", want_fp32 ? "fp32" : "fp64",
                             static_cast<int>(std::count(on.begin(), on.end(), 1)), delta,
                             K.factor_ms(want_fp32) - f0);
            }
            if (fok) { ok = true; break; }
            std::vector<char> nf(nlp, 0);
            bool any = false;
            for (int k : K.failed_lps())
                if (k >= 0 && k < nlp && pend[k]) { nf[k] = 1; any = true; }
            if (!any) continue;          // no LP recorded: all of them again
            pend = nf;
            narrowed = true;
            if (want_fp32) K.set_masks(pend, m64);
            else K.set_masks(m32, pend);
        }
        if (narrowed) K.set_masks(m32, m64);
        if (ok && want_fp32) I.used_fp32 = true;
        ladder_failed = ok ? std::vector<char>(nlp, 0) : pend;
        return ok;
    };
    auto any_of = [&](const std::vector<char>& v) {
        for (char c : v) if (c) return true;
        return false;
    };
    auto masks_now = [&](std::vector<char>& on32, std::vector<char>& on64) {
        on32.assign(nlp, 0);
        on64.assign(nlp, 0);
        for (int k = 0; k < nlp; ++k) if (I.active[k]) (I.sw_now[k] ? on64 : on32)[k] = 1;
    };
    auto mark_switch = [&](int k, int it) {
        I.sw[k] = I.sw_now[k] = 1;
        I.switched = true;
        if (I.res[k].switch_iteration < 0) I.res[k].switch_iteration = it;
    };
    // Factors every active LP: FP32 fronts for the LPs not (yet) switched, FP64 fronts
    // for the others. The LPs whose FP32 pivots failed at every delta of the ladder
    // move to FP64 fronts (the other LPs keep their FP32 factors); with `sticky` false
    // that move lasts for this factorisation only (start points). Returns false when
    // the FP64 ladder fails.
    auto factor_all = [&](int it, bool sticky) -> bool {
        I.sw_now = I.sw;
        std::vector<char> on32, on64;
        masks_now(on32, on64);
        const std::vector<char> none(nlp, 0);
        if (any_of(on32)) {
            K.set_masks(on32, none);
            if (!ladder(true)) {
                const std::vector<char> move = any_of(ladder_failed) ? ladder_failed : on32;
                for (int q = 0; q < nlp; ++q) {
                    if (!move[q] || !on32[q]) continue;
                    if (o.verbose) std::fprintf(stderr, "[sk] lp %d: FP32 factorisation failed, FP64 fronts\n", q);
                    if (sticky) mark_switch(q, it);
                    else I.sw_now[q] = 1;
                }
            }
        }
        masks_now(on32, on64);
        if (any_of(on64)) {
            K.set_masks(on32, on64);
            if (!ladder(false)) return false;
        }
        K.set_masks(on32, on64);
        return true;
    };
    // Moves the LPs in `which` to FP64 fronts now and factors them alone (the other
    // LPs' factors stay as they are).
    auto switch_lps = [&](const std::vector<char>& which, int it) -> bool {
        for (int k = 0; k < nlp; ++k) if (which[k]) mark_switch(k, it);
        std::vector<char> on32, on64;
        masks_now(on32, on64);
        K.set_masks(on32, which);
        const bool ok = ladder(false);
        K.set_masks(on32, on64);
        return ok;
    };
    // ---- direction: solve for rkkt -> (dx, dy, ds) and check it (mehrotra_device.cu:494-587).
    // acc[k]: the solve met its tolerance and e1, e2, e3 <= 1e-8 (the reference's test);
    // use[k]: the direction may be used (strict: acc; otherwise finite with e1, e2, e3 <= 1e-6).
    struct DirStats { std::vector<double> e1, e2, e3, rx, rs, xs, xds, dxs, dxds; };
    std::vector<char> solved;   // per LP: the last direction's solve met its tolerance
    // which (optional): a direction redone for these LPs alone; the other LPs keep
    // the direction, statistics and flags of the previous call with the same outputs
    auto direction = [&](double* dxo, double* dyo, double* dso, const double* rxs, std::vector<char>& acc,
                         std::vector<char>& use, DirStats& ds_, const std::vector<char>* which = nullptr) {
        if (which) {
            SK_CUDA(cudaMemcpyAsync(I.kdx.ptr, dxo, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            SK_CUDA(cudaMemcpyAsync(I.kds.ptr, dso, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            SK_CUDA(cudaMemcpyAsync(I.kdy.ptr, dyo, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
        }
        spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, I.v.ptr, EpiSub{I.rp.ptr, I.rkkt.ptr}, st);
        solve(I.rkkt.ptr, dyo, solved, which);
        spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, dyo,
             EpiDsDx{I.rd.ptr, I.theta.ptr, rxs, I.x.ptr, I.s.ptr, dso, dxo, I.e2.ptr, I.e3.ptr}, st);
        spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, dxo, EpiAdd{I.rp.ptr, I.e1.ptr}, st);
        I.reduce_rows<1>(RedSq{I.e1.ptr}, I.redout.ptr);
        I.reduce_cols<9>(RedDir{I.e2.ptr, I.e3.ptr, rxs, I.x.ptr, I.s.ptr, dxo, dso}, I.redout.ptr + nlp);
        if (which) {
            std::vector<double> keep(nlp, 0.0);
            for (int k = 0; k < nlp; ++k) keep[k] = (*which)[k] ? 0.0 : 1.0;
            I.put_scalars(6, keep);
            k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.kdx.ptr, I.col_lp.ptr, I.sc(6), dxo);
            k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.kds.ptr, I.col_lp.ptr, I.sc(6), dso);
            k_masked_copy<<<nblk(M), 256, 0, st>>>(M, I.kdy.ptr, I.row_lp.ptr, I.sc(6), dyo);
        }
        std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 10);
        const DirStats old = ds_;
        ds_ = DirStats();
        for (int k = 0; k < nlp; ++k) {
            if (which && !(*which)[k] && k < static_cast<int>(old.e1.size())) {
                ds_.e1.push_back(old.e1[k]); ds_.e2.push_back(old.e2[k]); ds_.e3.push_back(old.e3[k]);
                ds_.rx.push_back(old.rx[k]); ds_.rs.push_back(old.rs[k]); ds_.xs.push_back(old.xs[k]);
                ds_.xds.push_back(old.xds[k]); ds_.dxs.push_back(old.dxs[k]); ds_.dxds.push_back(old.dxds[k]);
                continue;
            }
            const double* q = h.data() + nlp + k * 9;
            ds_.e1.push_back(std::sqrt(h[k]) / std::max(1.0, nrp[k]));
            ds_.e2.push_back(std::sqrt(q[0]) / std::max(1.0, nrd[k]));
            ds_.e3.push_back(std::sqrt(q[1]) / std::max(1.0, std::sqrt(q[2])));
            ds_.rx.push_back(q[3]);
            ds_.rs.push_back(q[4]);
            ds_.xs.push_back(q[5]);
            ds_.xds.push_back(q[6]);
            ds_.dxs.push_back(q[7]);
            ds_.dxds.push_back(q[8]);
        }
        const std::vector<char> acc0 = acc, use0 = use;
        acc.assign(nlp, 0);
        use.assign(nlp, 0);
        if (o.verbose > 1)
            for (int k = 0; k < nlp && k < 4; ++k)
                if (I.active[k])
                    std::fprintf(stderr, "[sk]   dir lp %d solved %d e1 %.2e e2 %.2e e3 %.2e ratio_x %.3e ratio_s %.3e tol %.2e %s\n",
                                 k, (int)solved[k], ds_.e1[k], ds_.e2[k], ds_.e3[k], ds_.rx[k], ds_.rs[k], tol[k],
                                 I.sw_now[k] ? "fp64" : "fp32");
        for (int k = 0; k < nlp; ++k) {
            if (which && !(*which)[k] && k < static_cast<int>(acc0.size()) && k < static_cast<int>(use0.size())) {
                acc[k] = acc0[k];
                use[k] = use0[k];
                continue;
            }
            const double e = std::max(ds_.e1[k], std::max(ds_.e2[k], ds_.e3[k]));
            const bool fin = std::isfinite(ds_.e1[k]) && std::isfinite(ds_.e2[k]) && std::isfinite(ds_.e3[k]) &&
                             std::isfinite(ds_.rx[k]) && std::isfinite(ds_.rs[k]);
            acc[k] = solved[k] && fin && e <= 1e-8;
            use[k] = o.strict ? acc[k] : (fin && e <= kUseDir);
        }
    };

    if (o.start == SK_START_MEHROTRA || o.start == SK_START_LEARNED) {
        // Mehrotra's heuristic start in the scaled space: x~ = A^T (A A^T)^{-1} b,
        // y = (A A^T)^{-1} A c, s~ = c - A^T y; x, s shifted to positivity by
        // max(-1.5 min, 0) and then by 1/2 x^T s / sum(s), 1/2 x^T s / sum(x).
        std::vector<double> one(nlp, 1.0);
        I.put_scalars(0, one);
        k_fill<<<nblk(N), 256, 0, st>>>(N, I.theta.ptr, 1.0);
        if (!factor_all(0, false))
            throw api::sk_exception(SK_ERR_NUMERICAL, "heuristic start: A A^T could not be factored");
        for (int k = 0; k < nlp; ++k) tol[k] = 1e-10;
        std::vector<char> ok;
        solve(I.b.ptr, I.dy.ptr, ok);
        spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, I.dy.ptr, EpiAxpby{1.0, 0.0, I.x.ptr}, st);
        spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, I.c.ptr, EpiAxpby{1.0, 0.0, I.rkkt.ptr}, st);
        solve(I.rkkt.ptr, I.y.ptr, ok);
        spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, I.y.ptr, EpiAxpby{1.0, 0.0, I.tmpn()}, st);
        k_sub<<<nblk(N), 256, 0, st>>>(N, I.c.ptr, I.tmpn(), I.s.ptr);
        I.reduce_cols<2>(RedMin2{I.x.ptr, I.s.ptr}, I.redout.ptr);
        std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 2);
        std::vector<double> sx(nlp), ss(nlp);
        for (int k = 0; k < nlp; ++k) { sx[k] = std::max(-1.5 * h[2 * k], 0.0); ss[k] = std::max(-1.5 * h[2 * k + 1], 0.0); }
        I.put_scalars(1, sx);
        I.put_scalars(2, ss);
        k_shift_lp<<<nblk(N), 256, 0, st>>>(N, d_ap, I.col_lp.ptr, I.x.ptr);
        k_shift_lp<<<nblk(N), 256, 0, st>>>(N, d_ad, I.col_lp.ptr, I.s.ptr);
        I.reduce_cols<3>(RedStart{I.x.ptr, I.s.ptr}, I.redout.ptr);
        h = I.fetch(static_cast<size_t>(nlp) * 3);
        for (int k = 0; k < nlp; ++k) {
            const double xs = h[3 * k], sumx = h[3 * k + 1], sums = h[3 * k + 2];
            sx[k] = std::isfinite(xs) && sums > 0 ? 0.5 * xs / sums : 1.0;
            ss[k] = std::isfinite(xs) && sumx > 0 ? 0.5 * xs / sumx : 1.0;
        }
        I.put_scalars(1, sx);
        I.put_scalars(2, ss);
        k_shift_lp<<<nblk(N), 256, 0, st>>>(N, d_ap, I.col_lp.ptr, I.x.ptr);
        k_shift_lp<<<nblk(N), 256, 0, st>>>(N, d_ad, I.col_lp.ptr, I.s.ptr);
        SK_CUDA(cudaGetLastError());
    }

    if (o.start == SK_START_LEARNED) {
        // Mehrotra's start (just computed) is the fallback; keep it in (dxa, dya, dsa).
        SK_CUDA(cudaMemcpyAsync(I.dxa.ptr, I.x.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        SK_CUDA(cudaMemcpyAsync(I.dya.ptr, I.y.ptr, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
        SK_CUDA(cudaMemcpyAsync(I.dsa.ptr, I.s.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        // the network's point in the scaled space: x = exp(log x), s = exp(log s), y
        I.gnn->forward(lp_, st, I.dx.ptr, I.ds.ptr, I.dy.ptr);
        k_learned_point<<<nblk(N), 256, 0, st>>>(N, I.dx.ptr, I.ds.ptr, I.x.ptr, I.s.ptr);
        SK_CUDA(cudaMemcpyAsync(I.y.ptr, I.dy.ptr, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
        // Projection towards Ax = b and A^T y + s = c (rp = Ax - b, rd = A^T y + s - c):
        // x -= a_p A^T w with (A A^T) w = rp; y -= a_d v, s -= a_d (rd - A^T v) with
        // (A A^T) v = A rd; a_p, a_d the longest steps (at most 1) that keep 10% of x and
        // s. A A^T is the matrix of Mehrotra's start, factored just above, so the
        // projection costs two solves and no factorisation of its own.
        {
            std::vector<double> one(nlp, 1.0);
            I.put_scalars(0, one);
            k_fill<<<nblk(N), 256, 0, st>>>(N, I.theta.ptr, 1.0);
            // the projection only has to move the point towards feasibility (the distance
            // test below decides whether it is used), so its solves stop at 1e-6
            for (int k = 0; k < nlp; ++k) tol[k] = 1e-6;
            std::vector<char> ok;
            residuals(I.x.ptr, I.y.ptr, I.s.ptr, I.rp.ptr, I.rd.ptr);
            solve(I.rp.ptr, I.dy.ptr, ok);
            spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, I.dy.ptr, EpiTheta{I.theta.ptr, I.dx.ptr}, st);
            k_hadamard<<<nblk(N), 256, 0, st>>>(N, I.theta.ptr, I.rd.ptr, I.tmpn());
            spmv(M, I.ga, I.a_rp.ptr, I.a_ci.ptr, I.a_v.ptr, I.tmpn(), EpiAxpby{1.0, 0.0, I.rkkt.ptr}, st);
            solve(I.rkkt.ptr, I.dy.ptr, ok);
            spmv(N, I.gt, I.t_rp.ptr, I.t_ci.ptr, I.t_v.ptr, I.dy.ptr, EpiAxpby{1.0, 0.0, I.tmpn()}, st);
            k_sub<<<nblk(N), 256, 0, st>>>(N, I.rd.ptr, I.tmpn(), I.ds.ptr);
            I.reduce_cols<2>(RedRatioNeg{I.x.ptr, I.dx.ptr, I.s.ptr, I.ds.ptr}, I.redout.ptr);
            std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 2), apv(nlp), adv(nlp);
            for (int k = 0; k < nlp; ++k) {
                apv[k] = std::isfinite(h[2 * k]) ? -std::min(1.0, 0.9 * h[2 * k]) : 0.0;
                adv[k] = std::isfinite(h[2 * k + 1]) ? -std::min(1.0, 0.9 * h[2 * k + 1]) : 0.0;
            }
            I.put_scalars(1, apv);
            k_axpy_lp<<<nblk(N), 256, 0, st>>>(N, d_ap, I.dx.ptr, I.col_lp.ptr, I.x.ptr);
            I.put_scalars(1, adv);
            k_axpy_lp<<<nblk(N), 256, 0, st>>>(N, d_ap, I.ds.ptr, I.col_lp.ptr, I.s.ptr);
            k_axpy_lp<<<nblk(M), 256, 0, st>>>(M, d_ap, I.dy.ptr, I.row_lp.ptr, I.y.ptr);
        }
        // centrality floor: x_j s_j >= 0.1 mean(x s) within each LP
        I.reduce_cols<3>(RedStart{I.x.ptr, I.s.ptr}, I.redout.ptr);
        std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 3), fl(nlp);
        for (int k = 0; k < nlp; ++k) fl[k] = std::isfinite(h[3 * k]) ? 0.1 * h[3 * k] / nn[k] : 0.0;
        I.put_scalars(1, fl);
        k_center_floor<<<nblk(N), 256, 0, st>>>(N, d_ap, I.col_lp.ptr, I.x.ptr, I.s.ptr);
        // distance to the stopping test, max(rel pinf, rel dinf, rel gap), of both candidates
        auto merit = [&](const double* xx, const double* yy, const double* ss) {
            residuals(xx, yy, ss, I.rp.ptr, I.rd.ptr);
            I.reduce_rows<3>(RedResidM{I.rp.ptr, I.R.ptr, I.b.ptr, yy}, I.redout.ptr);
            I.reduce_cols<4>(RedResidN{I.rd.ptr, I.C.ptr, xx, ss, I.c.ptr}, I.redout.ptr + nlp * 3);
            std::vector<double> hh = I.fetch(static_cast<size_t>(nlp) * 7), phi(nlp);
            const double* a = hh.data();
            const double* b = hh.data() + nlp * 3;
            for (int k = 0; k < nlp; ++k) {
                const double obj = b[k * 4 + 3], by = a[k * 3 + 2];
                const double v = std::max({a[k * 3 + 1] / (1.0 + I.binf[k]), b[k * 4 + 1] / (1.0 + I.cinf[k]),
                                           std::fabs(obj - by) / (1.0 + std::fabs(obj) + std::fabs(by))});
                phi[k] = std::isfinite(v) ? v : HUGE_VAL;
            }
            return phi;
        };
        const std::vector<double> phiL = merit(I.x.ptr, I.y.ptr, I.s.ptr);
        const std::vector<double> phiM = merit(I.dxa.ptr, I.dya.ptr, I.dsa.ptr);
        std::vector<double> keep(nlp);
        for (int k = 0; k < nlp; ++k) {
            // phi near 1 means c^T x and b^T y differ by orders of magnitude: not a usable start
            keep[k] = phiL[k] < o.learned_accept * phiM[k] && phiL[k] < kLearnedSaturated ? 1.0 : 0.0;
            I.res[k].learned_start = keep[k] != 0.0;
            I.res[k].start_merit = keep[k] != 0.0 ? phiL[k] : phiM[k];
            I.res[k].fallback_merit = phiM[k];
        }
        if (!I.mx0) {
            SK_CUDA(cudaMalloc(&I.mx0, sizeof(double) * N));
            SK_CUDA(cudaMalloc(&I.ms0, sizeof(double) * N));
            SK_CUDA(cudaMalloc(&I.my0, sizeof(double) * M));
        }
        SK_CUDA(cudaMemcpyAsync(I.mx0, I.dxa.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        SK_CUDA(cudaMemcpyAsync(I.ms0, I.dsa.ptr, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        SK_CUDA(cudaMemcpyAsync(I.my0, I.dya.ptr, sizeof(double) * M, cudaMemcpyDeviceToDevice, st));
        I.put_scalars(0, keep);
        k_pick_lp<<<nblk(N), 256, 0, st>>>(N, d_mask, I.col_lp.ptr, I.x.ptr, I.dxa.ptr);
        k_pick_lp<<<nblk(N), 256, 0, st>>>(N, d_mask, I.col_lp.ptr, I.s.ptr, I.dsa.ptr);
        k_pick_lp<<<nblk(M), 256, 0, st>>>(M, d_mask, I.row_lp.ptr, I.y.ptr, I.dya.ptr);
        SK_CUDA(cudaGetLastError());
    }

    I.short_steps.assign(nlp, 0);
    I.loose_count.assign(nlp, 0);
    I.reinit.assign(nlp, 0);
    // An LP started from the network's point goes back to Mehrotra's start (once)
    // instead of stopping on a numerical failure.
    std::vector<char> back_req(nlp, 0);
    auto learned_rescue = [&](int k) {
        if (o.start != SK_START_LEARNED || !I.res[k].learned_start) return false;
        back_req[k] = 1;
        I.active[k] = 0;    // sits out the rest of this iteration
        return true;
    };
    int iter = 0;
    std::vector<double> hm, hn;
    for (iter = 0; iter < o.max_iter; ++iter) {
        residuals(I.x.ptr, I.y.ptr, I.s.ptr, I.rp.ptr, I.rd.ptr);
        I.reduce_rows<3>(RedResidM{I.rp.ptr, I.R.ptr, I.b.ptr, I.y.ptr}, I.redout.ptr);
        I.reduce_cols<4>(RedResidN{I.rd.ptr, I.C.ptr, I.x.ptr, I.s.ptr, I.c.ptr}, I.redout.ptr + nlp * 3);
        std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 7);
        hm.assign(h.begin(), h.begin() + nlp * 3);
        hn.assign(h.begin() + nlp * 3, h.end());
        bool any = false;
        double mumax = 0.0;
        for (int k = 0; k < nlp; ++k) {
            if (!I.active[k]) continue;
            nrp[k] = std::sqrt(hm[k * 3]);
            nrd[k] = std::sqrt(hn[k * 4]);
            mu[k] = hn[k * 4 + 2] / nn[k];
            if (iter == 0 || I.reinit[k]) {
                I.reinit[k] = 0;
                I.rp0[k] = std::max(1.0, nrp[k]);
                I.rd0[k] = std::max(1.0, nrd[k]);
                I.mu0[k] = std::max(1.0, mu[k]);
            }
            record(k, hm.data(), hn.data());
            LpResult& r = I.res[k];
            r.iterations = iter;
            bool conv;
            if (o.criteria == SK_CRIT_REFERENCE) conv = nrp[k] < 1e-6 && nrd[k] < 1e-6 && mu[k] < 1e-6;
            else {   // the gap also within tol (1 + |c^T x|): the objective is then within tol of the optimum
                const bool loose = r.rel_pinf <= o.tol && r.rel_dinf <= o.tol && r.rel_gap <= o.tol;
                conv = loose && std::fabs(r.objective - hm[k * 3 + 2]) <= o.tol * (1.0 + std::fabs(r.objective));
                // an iterate that meets the three relative tests but cannot close the gap
                // further (numerical stall) is accepted after kLooseIters iterations
                I.loose_count[k] = loose && !conv ? I.loose_count[k] + 1 : 0;
                if (I.loose_count[k] >= kLooseIters) conv = true;
            }
            if (o.verbose)
                std::fprintf(stderr, "[sk] lp %d iter %d rp %.3e rd %.3e mu %.3e gap %.3e %s\n", k, iter, nrp[k],
                             nrd[k], mu[k], r.rel_gap, I.sw[k] ? "fp64" : "fp32");
            if (I.capture_mu > 0.0 && !I.captured[k] && (conv || mu[k] < I.capture_mu)) {
                const int co = I.col_off[k], nk = I.col_off[k + 1] - co;
                const int ro = I.row_off[k], mk = I.row_off[k + 1] - ro;
                k_log_floor<<<nblk(nk), 256, 0, st>>>(nk, I.x.ptr + co, I.cap_lx + co);
                k_log_floor<<<nblk(nk), 256, 0, st>>>(nk, I.s.ptr + co, I.cap_ls + co);
                SK_CUDA(cudaMemcpyAsync(I.cap_y + ro, I.y.ptr + ro, sizeof(double) * mk, cudaMemcpyDeviceToDevice, st));
                I.captured[k] = 1;
            }
            if (conv) { r.status = SK_STATUS_OPTIMAL; I.active[k] = 0; continue; }
            any = true;
            mumax = std::max(mumax, mu[k]);
        }
        if (!any) break;
        for (int k = 0; k < nlp; ++k) mask[k] = I.active[k] ? 1.0 : 0.0;
        I.put_scalars(0, mask);
        // converged LPs' fronts are no longer factored or solved (factor_all sets the masks)
        k_theta<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, I.s.ptr, I.col_lp.ptr, d_mask, I.theta.ptr);
        // precision of each LP for this iteration: FP64 fronts once its mu is below mu_switch
        (void)mumax;
        double mu32 = 0.0;
        for (int k = 0; k < nlp; ++k) {
            if (!I.active[k] || I.sw[k]) continue;
            if (mu[k] < o.mu_switch) {
                if (o.verbose) std::fprintf(stderr, "[sk] lp %d: FP64 fronts from iter %d (mu below mu_switch)\n", k, iter);
                mark_switch(k, iter);
                continue;
            }
            mu32 = std::max(mu32, mu[k]);
        }
        tensor_now = mu32 >= kTensorMu;
        std::fill(I.pcg_k.begin(), I.pcg_k.end(), 0);
        const bool ok_fac = factor_all(iter, true);
        if (!ok_fac) {   // the reference throws here (kkt.cu:600-602); report a numerical stop
            for (int k = 0; k < nlp; ++k) if (I.active[k]) { I.res[k].status = SK_STATUS_ITERATION_LIMIT; I.active[k] = 0; }
            break;
        }
        for (int k = 0; k < nlp; ++k) tol[k] = 1e-9 * std::max(1.0, nrp[k]);
        // ---------------- predictor
        DirStats pd;
        std::vector<char> acc_p, use_p;
        bool fac_ok = true;
        // An FP32 direction that misses the check is first recomputed with the same
        // factor and a 100x tighter PCG target; an LP whose direction misses again moves
        // to FP64 fronts (alone: the other LPs keep their precision). An LP whose PCG
        // did not reach its tolerance moves at once: PCG from the same start with the
        // same factor repeats the same steps, so a tighter target cannot be met.
        std::vector<char> tightened(nlp, 0);
        auto retry_fp32_misses = [&](const std::vector<char>& acc, const char* what,
                                     std::vector<char>& again) -> int {
            // returns 0: nothing to redo; 1: redo the direction of the LPs in `again`;
            // -1: FP64 factorisation failed
            std::vector<char> now(nlp, 0);
            bool redo = false, any_now = false;
            again.assign(nlp, 0);
            for (int k = 0; k < nlp; ++k) {
                if (!I.active[k] || I.sw[k] || acc[k]) continue;
                redo = true;
                again[k] = 1;
                if (!tightened[k] && solved[k]) { tightened[k] = 1; tol[k] *= 0.01; }
                else { now[k] = 1; any_now = true; }
            }
            if (any_now) {
                if (o.verbose)
                    for (int k = 0; k < nlp; ++k)
                        if (now[k])
                            std::fprintf(stderr, "[sk] lp %d: FP64 fronts from iter %d (FP32 %s missed the accuracy, "
                                         "pcg %d)\n", k, iter, what, I.pcg_k[k]);
                if (!switch_lps(now, iter)) return -1;
            }
            return redo ? 1 : 0;
        };
        // a repeated direction is solved for the LPs that retry alone
        std::vector<char> again;
        for (int attempt = 0; attempt < 3; ++attempt) {
            k_rhs<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, I.s.ptr, I.theta.ptr, I.rd.ptr, nullptr, nullptr, nullptr,
                                          I.col_lp.ptr, I.rxs.ptr, I.v.ptr);
            direction(I.dxa.ptr, I.dya.ptr, I.dsa.ptr, I.rxs.ptr, acc_p, use_p, pd, attempt > 0 ? &again : nullptr);
            if (attempt == 2) break;
            const int r = retry_fp32_misses(acc_p, "predictor", again);
            if (r < 0) { fac_ok = false; break; }
            if (r == 0) break;
        }
        if (!fac_ok) {
            for (int k = 0; k < nlp; ++k) if (I.active[k]) { I.res[k].status = SK_STATUS_ITERATION_LIMIT; I.active[k] = 0; }
            break;
        }
        std::vector<double> sigmu(nlp, 0.0);
        for (int k = 0; k < nlp; ++k) {
            if (!I.active[k]) continue;
            if (!use_p[k]) {
                if (!learned_rescue(k)) { I.res[k].status = SK_STATUS_ITERATION_LIMIT; I.active[k] = 0; }
                continue;
            }
            const double apa = std::min(1.0, pd.rx[k]), ada = std::min(1.0, pd.rs[k]);
            const double mua = (pd.xs[k] + ada * pd.xds[k] + apa * pd.dxs[k] + apa * ada * pd.dxds[k]) / nn[k];
            const double sigma = std::min(1.0, std::pow(std::max(0.0, mua) / std::max(1e-16, mu[k]), 3.0));
            sigmu[k] = sigma * mu[k];
        }
        // ---------------- corrector
        I.put_scalars(3, sigmu);
        DirStats cd;
        std::vector<char> acc_c, okc;
        for (int attempt = 0; attempt < 3; ++attempt) {
            k_rhs<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, I.s.ptr, I.theta.ptr, I.rd.ptr, I.dxa.ptr, I.dsa.ptr, d_tgt,
                                          I.col_lp.ptr, I.rxs.ptr, I.v.ptr);
            direction(I.dx.ptr, I.dy.ptr, I.ds.ptr, I.rxs.ptr, acc_c, okc, cd, attempt > 0 ? &again : nullptr);
            if (attempt == 2) break;
            const int r = retry_fp32_misses(acc_c, "corrector", again);
            if (r < 0) { okc.assign(nlp, 0); break; }
            if (r == 0) break;
        }
        // FP32 fronts that needed many PCG steps are not worth keeping: FP64 from the next iteration
        for (int k = 0; k < nlp; ++k) {
            if (!I.active[k] || I.sw[k] || I.pcg_k[k] <= 20) continue;
            if (o.verbose)
                std::fprintf(stderr, "[sk] lp %d: FP64 fronts from iter %d (%d PCG steps)\n", k, iter + 1, I.pcg_k[k]);
            mark_switch(k, iter + 1);
        }
        const double eta = 0.995, armijo = 1e-4;
        std::vector<int> dir(nlp, 0), bt(nlp, 0);
        std::vector<char> decided(nlp, 1), accepted(nlp, 0);
        std::vector<double> merit0(nlp, 0.0), dist0(nlp, 0.0);
        std::vector<char> near(nlp, 0);
        bool need_centred = false;
        for (int k = 0; k < nlp; ++k) {
            if (!I.active[k]) continue;
            decided[k] = 0;
            merit0[k] = nrp[k] / I.rp0[k] + nrd[k] / I.rd0[k] + mu[k] / I.mu0[k];
            // near-optimal: primal and dual infeasibility already well inside the relative
            // stopping test; progress may then also be judged by the test itself (below)
            const LpResult& r = I.res[k];
            near[k] = !o.strict && o.criteria == SK_CRIT_RELATIVE && r.rel_pinf <= kNearFeas * o.tol &&
                      r.rel_dinf <= kNearFeas * o.tol;
            dist0[k] = std::max({r.rel_pinf, r.rel_dinf,
                                 std::fabs(r.objective - hm[k * 3 + 2]) / (1.0 + std::fabs(r.objective))});
            dir[k] = okc[k] ? 0 : 1;
            ap[k] = std::min(1.0, eta * cd.rx[k]);
            ad[k] = std::min(1.0, eta * cd.rs[k]);
            if (dir[k] == 1) need_centred = true;
        }
        auto centred = [&]() {
            // centred safeguard direction sigma_c = 1/2 for the LPs in direction 1
            std::vector<double> half(nlp, 0.0), cm(nlp, 0.0);
            for (int k = 0; k < nlp; ++k) {
                half[k] = 0.5 * mu[k];
                cm[k] = (!decided[k] && dir[k] == 1) ? 1.0 : 0.0;
            }
            I.put_scalars(3, half);
            k_rhs<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, I.s.ptr, I.theta.ptr, I.rd.ptr, nullptr, nullptr, d_tgt,
                                          I.col_lp.ptr, I.crxs.ptr, I.v.ptr);
            DirStats cs;
            std::vector<char> accz, okz;
            direction(I.cdx.ptr, I.cdy.ptr, I.cds.ptr, I.crxs.ptr, accz, okz, cs);
            I.put_scalars(4, cm);
            k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.cdx.ptr, I.col_lp.ptr, d_rmask, I.dx.ptr);
            k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.cds.ptr, I.col_lp.ptr, d_rmask, I.ds.ptr);
            k_masked_copy<<<nblk(M), 256, 0, st>>>(M, I.cdy.ptr, I.row_lp.ptr, d_rmask, I.dy.ptr);
            for (int k = 0; k < nlp; ++k) {
                if (cm[k] == 0.0) continue;
                if (!okz[k]) { decided[k] = 1; continue; }   // failed safeguard solve: no step
                const double bnd = std::min(cs.rx[k], cs.rs[k]);
                ap[k] = ad[k] = std::min(1.0, eta * bnd);
                bt[k] = 0;
            }
        };
        if (need_centred) centred();
        for (int round = 0; round < 64; ++round) {
            bool pending = false;
            for (int k = 0; k < nlp; ++k) pending |= !decided[k];
            if (!pending) break;
            std::vector<double> tap(nlp, 0.0), tad(nlp, 0.0);
            for (int k = 0; k < nlp; ++k) if (!decided[k]) { tap[k] = ap[k]; tad[k] = ad[k]; }
            I.put_scalars(1, tap);
            I.put_scalars(2, tad);
            k_trial_n<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, I.s.ptr, I.dx.ptr, I.ds.ptr, d_ap, d_ad, I.col_lp.ptr,
                                              I.xt.ptr, I.stt.ptr);
            k_trial_m<<<nblk(M), 256, 0, st>>>(M, I.y.ptr, I.dy.ptr, d_ad, I.row_lp.ptr, I.yt.ptr);
            residuals(I.xt.ptr, I.yt.ptr, I.stt.ptr, I.rpt.ptr, I.rdt.ptr);
            I.reduce_rows<4>(RedTrialM{I.rpt.ptr, I.yt.ptr, I.R.ptr, I.b.ptr}, I.redout.ptr);
            I.reduce_cols<6>(RedTrialN{I.rdt.ptr, I.xt.ptr, I.stt.ptr, I.C.ptr, I.c.ptr}, I.redout.ptr + nlp * 4);
            std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 10);
            bool want_centred = false;
            for (int k = 0; k < nlp; ++k) {
                if (decided[k]) continue;
                const double rpn = std::sqrt(h[k * 4]), yn = std::sqrt(h[k * 4 + 1]);
                const double* q = h.data() + nlp * 4 + k * 6;
                const double rdn = std::sqrt(q[0]), mun = q[1] / nn[k], minx = q[2], mins = q[3];
                const double merit = rpn / I.rp0[k] + rdn / I.rd0[k] + mun / I.mu0[k];
                const double stp = std::min(ap[k], ad[k]);
                const bool finite = std::isfinite(rpn) && std::isfinite(rdn) && std::isfinite(mun) &&
                                    std::isfinite(merit) && std::isfinite(merit0[k]) && std::isfinite(minx) &&
                                    std::isfinite(mins) && std::isfinite(ap[k]) && std::isfinite(ad[k]) &&
                                    std::isfinite(yn);
                const bool positive = minx > 0.0 && mins > 0.0 && mun > 0.0 && stp > 0.0;
                bool progress = merit < merit0[k] && merit <= (1.0 - armijo * stp) * merit0[k];
                if (!progress && near[k] && finite && positive) {
                    // Near the optimum the merit's residual terms can outweigh its mu term
                    // although the step closes the gap: an inexact FP64 direction (normal
                    // equations beyond FP64's reach) adds primal infeasibility far below the
                    // tolerance and the merit rejects every step (an LP stalled at rel. gap
                    // 3e-8 that way). Such a trial is accepted when it stays near-feasible
                    // and its distance to the stopping test falls by the Armijo factor.
                    const double tp = h[k * 4 + 2] / (1.0 + I.binf[k]), td = q[4] / (1.0 + I.cinf[k]);
                    const double tobj = q[5], tby = h[k * 4 + 3];
                    const double tdist = std::max({tp, td, std::fabs(tobj - tby) / (1.0 + std::fabs(tobj))});
                    progress = tp <= kNearFeas * o.tol && td <= kNearFeas * o.tol && std::isfinite(tdist) &&
                               tdist <= (1.0 - armijo * stp) * dist0[k];
                }
                if (o.verbose > 1 && k < 4)
                    std::fprintf(stderr, "[sk]   trial lp %d dir %d bt %d ap %.3e ad %.3e merit %.6e -> %.6e minx %.2e mins %.2e %s\n",
                                 k, dir[k], bt[k], ap[k], ad[k], merit0[k], merit, minx, mins,
                                 !finite ? "non-finite" : !positive ? "positivity" : !progress ? "no-decrease" : "accept");
                if (finite && positive && progress) { decided[k] = 1; accepted[k] = 1; continue; }
                ap[k] *= 0.5;
                ad[k] *= 0.5;
                ++bt[k];
                if (bt[k] >= (dir[k] == 0 ? 15 : 30)) {
                    if (dir[k] == 0) { dir[k] = 1; want_centred = true; }
                    else decided[k] = 1;
                }
            }
            if (want_centred) centred();
        }
        std::vector<double> acc(nlp, 0.0);
        for (int k = 0; k < nlp; ++k) acc[k] = accepted[k] ? 1.0 : 0.0;
        I.put_scalars(4, acc);
        // re-evaluate the accepted trials (the last trial buffers hold only the
        // final round's points) and commit them
        {
            std::vector<double> tap(nlp, 0.0), tad(nlp, 0.0);
            for (int k = 0; k < nlp; ++k) if (accepted[k]) { tap[k] = ap[k]; tad[k] = ad[k]; }
            I.put_scalars(1, tap);
            I.put_scalars(2, tad);
            k_trial_n<<<nblk(N), 256, 0, st>>>(N, I.x.ptr, I.s.ptr, I.dx.ptr, I.ds.ptr, d_ap, d_ad, I.col_lp.ptr,
                                              I.xt.ptr, I.stt.ptr);
            k_trial_m<<<nblk(M), 256, 0, st>>>(M, I.y.ptr, I.dy.ptr, d_ad, I.row_lp.ptr, I.yt.ptr);
            k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.xt.ptr, I.col_lp.ptr, d_rmask, I.x.ptr);
            k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.stt.ptr, I.col_lp.ptr, d_rmask, I.s.ptr);
            k_masked_copy<<<nblk(M), 256, 0, st>>>(M, I.yt.ptr, I.row_lp.ptr, d_rmask, I.y.ptr);
        }
        for (int k = 0; k < nlp; ++k)
            if (I.active[k] && !accepted[k] && !learned_rescue(k)) {
                I.res[k].status = SK_STATUS_ITERATION_LIMIT;
                I.active[k] = 0;
            }
        // Learned-start safeguard: an LP started from the network's point that takes a
        // short step (min(a_p, a_d) < kShortStep) in kShortSteps of its first
        // kRestartWindow iterations, or that hit a numerical failure, goes back to
        // Mehrotra's start.
        if (o.start == SK_START_LEARNED) {
            std::vector<double> back(nlp, 0.0);
            bool any_back = false;
            for (int k = 0; k < nlp; ++k) {
                if (!I.res[k].learned_start) continue;
                bool go = back_req[k] != 0;
                if (!go && iter < kRestartWindow && I.active[k] && accepted[k] &&
                    std::min(ap[k], ad[k]) < kShortStep && ++I.short_steps[k] >= kShortSteps)
                    go = true;
                // too little progress: the distance to the stopping test has not fallen by
                // kProgress since the start after kProgressIter iterations
                const LpResult& rk = I.res[k];
                if (!go && iter == kProgressIter && I.active[k] &&
                    std::max({rk.rel_pinf, rk.rel_dinf, rk.rel_gap}) > kProgress * rk.start_merit)
                    go = true;
                if (!go) continue;
                back[k] = 1.0;
                any_back = true;
                back_req[k] = 0;
                I.active[k] = 1;
                I.res[k].learned_start = 0;
                I.reinit[k] = 1;
                if (o.verbose) std::fprintf(stderr, "[sk] lp %d: learned start abandoned, Mehrotra's start\n", k);
            }
            if (any_back) {
                I.put_scalars(4, back);
                k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.mx0, I.col_lp.ptr, d_rmask, I.x.ptr);
                k_masked_copy<<<nblk(N), 256, 0, st>>>(N, I.ms0, I.col_lp.ptr, d_rmask, I.s.ptr);
                k_masked_copy<<<nblk(M), 256, 0, st>>>(M, I.my0, I.row_lp.ptr, d_rmask, I.y.ptr);
            }
        }
    }
    // LPs still running at the iteration cap: final residuals (mehrotra_device.cu:1026-1035)
    bool any_left = false;
    for (int k = 0; k < nlp; ++k) any_left |= I.active[k] != 0;
    residuals(I.x.ptr, I.y.ptr, I.s.ptr, I.rp.ptr, I.rd.ptr);
    I.reduce_rows<3>(RedResidM{I.rp.ptr, I.R.ptr, I.b.ptr, I.y.ptr}, I.redout.ptr);
    I.reduce_cols<4>(RedResidN{I.rd.ptr, I.C.ptr, I.x.ptr, I.s.ptr, I.c.ptr}, I.redout.ptr + nlp * 3);
    std::vector<double> h = I.fetch(static_cast<size_t>(nlp) * 7);
    for (int k = 0; k < nlp; ++k) {
        if (I.res[k].status == SK_STATUS_OPTIMAL) continue;
        record(k, h.data(), h.data() + nlp * 3);
        if (I.active[k]) I.res[k].iterations = o.max_iter;
        I.res[k].status = SK_STATUS_ITERATION_LIMIT;
    }
    (void)any_left;
    I.precision_path = o.precision == SK_PREC_FP64 ? 0 : (I.switched ? (I.used_fp32 ? 2 : 0) : 1);
    SK_CUDA(cudaEventRecord(I.ev1, st));
    SK_CUDA(cudaStreamSynchronize(st));
    {
        float ms = 0.f;
        SK_CUDA(cudaEventElapsedTime(&ms, I.ev0, I.ev1));
        I.device_ms = ms;
    }
    I.factor_ms32 = K.factor_ms(true);
    I.factor_ms64 = K.factor_ms(false);
    I.solve_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void DeviceIPM::result(int lp, double* x, double* y, double* s, sk_info* info) const {
    const Impl& I = *im_;
    if (lp < 0 || lp >= I.nlp) throw api::sk_exception(SK_ERR_INVALID, "result: lp out of range");
    const int ro = I.row_off[lp], co = I.col_off[lp];
    const int m = I.row_off[lp + 1] - ro, n = I.col_off[lp + 1] - co;
    std::vector<double> hx(n), hy(m), hs(n);
    SK_CUDA(cudaMemcpyAsync(hx.data(), I.x.ptr + co, sizeof(double) * n, cudaMemcpyDeviceToHost, I.st));
    SK_CUDA(cudaMemcpyAsync(hy.data(), I.y.ptr + ro, sizeof(double) * m, cudaMemcpyDeviceToHost, I.st));
    SK_CUDA(cudaMemcpyAsync(hs.data(), I.s.ptr + co, sizeof(double) * n, cudaMemcpyDeviceToHost, I.st));
    SK_CUDA(cudaStreamSynchronize(I.st));
    if (x) for (int j = 0; j < n; ++j) x[j] = hx[j] * I.C_h[co + j];
    if (y) for (int i = 0; i < m; ++i) y[i] = hy[i] * I.R_h[ro + i];
    if (s) for (int j = 0; j < n; ++j) s[j] = hs[j] / I.C_h[co + j];
    if (info) {
        const LpResult& r = I.res[lp];
        const auto& p = kkt_->plan();
        info->status = r.status;
        info->iterations = r.iterations;
        info->objective = r.objective;
        info->primal_residual = r.primal_residual;
        info->dual_residual = r.dual_residual;
        info->duality_gap = r.duality_gap;
        info->rel_pinf = r.rel_pinf;
        info->rel_dinf = r.rel_dinf;
        info->rel_gap = r.rel_gap;
        info->precision_path = I.precision_path;
        info->switch_iteration = r.switch_iteration;
        info->factorizations = I.factorizations;
        info->solves = I.solves;
        info->refine_steps = I.refine_steps;
        info->learned_start = r.learned_start;
        info->setup_ms = setup_ms_;
        info->solve_ms = I.solve_ms;
        info->nnz_factor = p.nnz_factor;
        info->num_supernodes = p.ns;
        info->dense_front = p.dense_mode ? 1 : 0;
        info->device_ms = I.device_ms;
        info->flops_factor = p.flops_factor;
        info->start_merit = r.start_merit;
        info->fallback_merit = r.fallback_merit;
        info->factor_ms_fp32 = I.factor_ms32;
        info->factor_ms_fp64 = I.factor_ms64;
    }
}

}  // namespace dev
}  // namespace sankhya
