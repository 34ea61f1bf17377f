// Device convex QP iteration with a diagonal Hessian: the steps of the reference's
// qp::QPSolver::solve_with_diagnostics (src/qp/qp_solver.cpp:151-560) with every
// vector operation, reduction and the Schur-complement solve on the GPU.
//
// Per iteration (reference lines in brackets):
//   rp = A x - b, rd = h.x + c - A^T y - zl + zu, mu, objective        [:219-266]
//   stop / Infeasible / Unbounded tests on the host                    [:269-292]
//   D = zl/gap_l + zu/gap_u (floor 1e-12), theta = 1/(h + D)           [:295-325]
//   rhs_x = -rd + (sigma mu - z gap)/gap terms, sigma = 0.2            [:335-352]
//   S = A diag(theta) A^T: the multifrontal engine's FP64 factor of
//   D_S S D_S + delta I, then PCG with the exact operator to a 1e-13
//   relative residual; rhs_y = -A (theta rhs_x) - rp, S dy = rhs_y     [:354-418]
//   dx = theta (A^T dy + rhs_x), dzl, dzu                               [:420-446]
//   fraction to the boundary 0.995, separate primal / dual steps       [:448-477]
//   update, z floored at 1e-14 on finite bounds                        [:479-491]
// W = h + D is diagonal, so the reference's dense Cholesky of W fails exactly when
// some W_j <= 1e-14; its Cholesky of S fails when a pivot is <= 1e-14, of which
// S_ii <= 1e-14 is the part checked here (exact for one row); both give
// NumericalFailure, as does an engine factorisation that fails its delta ladder.
#include "cuda/device_qp.hpp"

#include <algorithm>
#include <cmath>
#include <memory>

#include "cuda/dev_common.cuh"
#include "cuda/device_lp.hpp"
#include "cuda/kkt_engine.hpp"
#include "cuda/spmv.cuh"
#include "ipm/front_plan.hpp"

namespace sankhya {
namespace dev {

namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 148;          // partial sums per reduction (fixed: deterministic results)
constexpr double kBoundInf = 1e15;    // |bound| beyond this is infinite (reference :196-197)

__device__ __forceinline__ bool has_lo(double lb) { return lb > -kBoundInf; }
__device__ __forceinline__ bool has_hi(double ub) { return ub < kBoundInf; }

// block partials of up to 4 values: op 0 sum, 1 max, 2 min
template <int R>
__device__ void block_partials(double (&v)[R], const int (&op)[R], double* part) {
    __shared__ double sh[kThreads / 32][R];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        double a = v[r];
        a = op[r] == 0 ? warp_sum(a) : (op[r] == 1 ? warp_max(a) : warp_min(a));
        if (lane == 0) sh[w][r] = a;
    }
    __syncthreads();
    if (threadIdx.x < R) {
        const int r = threadIdx.x;
        double a = sh[0][r];
        for (int q = 1; q < kThreads / 32; ++q)
            a = op[r] == 0 ? a + sh[q][r] : (op[r] == 1 ? fmax(a, sh[q][r]) : fmin(a, sh[q][r]));
        part[blockIdx.x * R + r] = a;
    }
}

// rd = h x + c - aty - zl + zu; partials [sum mu terms, max |rd|, sum objective]
__global__ void __launch_bounds__(kThreads) k_qp_dual(int n, const double* __restrict__ h, const double* __restrict__ x,
                                                      const double* __restrict__ c, const double* __restrict__ aty,
                                                      const double* __restrict__ zl, const double* __restrict__ zu,
                                                      const double* __restrict__ lb, const double* __restrict__ ub,
                                                      double* __restrict__ rd, double* __restrict__ part) {
    double v[3] = {0.0, 0.0, 0.0};
    const int op[3] = {0, 1, 0};
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const double hx = h[j] * x[j];
        const double r = hx + c[j] - aty[j] - zl[j] + zu[j];
        rd[j] = r;
        if (has_lo(lb[j])) v[0] += (x[j] - lb[j]) * zl[j];
        if (has_hi(ub[j])) v[0] += (ub[j] - x[j]) * zu[j];
        v[1] = fmax(v[1], fabs(r));
        v[2] += 0.5 * x[j] * hx + c[j] * x[j];
    }
    block_partials<3>(v, op, part);
}

// rp = ax - b; partials [max |rp|, max |y|]
__global__ void __launch_bounds__(kThreads) k_qp_primal(int m, const double* __restrict__ ax,
                                                        const double* __restrict__ b, const double* __restrict__ y,
                                                        double* __restrict__ rp, double* __restrict__ part) {
    double v[2] = {0.0, 0.0};
    const int op[2] = {1, 1};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double r = ax[i] - b[i];
        rp[i] = r;
        v[0] = fmax(v[0], fabs(r));
        v[1] = fmax(v[1], fabs(y[i]));
    }
    block_partials<2>(v, op, part);
}

template <int R>
__global__ void k_qp_final(const double* __restrict__ part, int nparts, int op0, int op1, int op2, int op3,
                           double* __restrict__ out) {
    const int r = threadIdx.x;
    if (r >= R) return;
    const int op = r == 0 ? op0 : r == 1 ? op1 : r == 2 ? op2 : op3;
    double a = part[r];
    for (int q = 1; q < nparts; ++q) {
        const double b = part[q * R + r];
        a = op == 0 ? a + b : (op == 1 ? fmax(a, b) : fmin(a, b));
    }
    out[r] = a;
}

// theta = 1 / (h + D), rhs_x = -rd + comp, wr = theta rhs_x; partial [min W]
__global__ void __launch_bounds__(kThreads) k_qp_prep(int n, const double* __restrict__ h, const double* __restrict__ x,
                                                      const double* __restrict__ zl, const double* __restrict__ zu,
                                                      const double* __restrict__ lb, const double* __restrict__ ub,
                                                      const double* __restrict__ rd, const double* __restrict__ scal,
                                                      double* __restrict__ theta, double* __restrict__ rhsx,
                                                      double* __restrict__ wr, double* __restrict__ part) {
    const double smu = scal[0];     // sigma mu
    double v[1] = {HUGE_VAL};
    const int op[1] = {2};
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double D = 0.0, comp = 0.0;
        if (has_lo(lb[j])) {
            const double g = fmax(x[j] - lb[j], 1e-12);
            D += zl[j] / g;
            comp += (smu - zl[j] * g) / g;
        }
        if (has_hi(ub[j])) {
            const double g = fmax(ub[j] - x[j], 1e-12);
            D += zu[j] / g;
            comp -= (smu - zu[j] * g) / g;
        }
        if (D < 1e-12) D = 1e-12;
        const double W = h[j] + D;
        v[0] = fmin(v[0], W);
        const double t = 1.0 / W;
        const double rx = -rd[j] + comp;
        theta[j] = t;
        rhsx[j] = rx;
        wr[j] = t * rx;
    }
    block_partials<1>(v, op, part);
}

// S_ii = sum_k a_ik^2 theta_k (one warp per row); partial [min S_ii]
__global__ void __launch_bounds__(kThreads) k_qp_sdiag(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                                                       const double* __restrict__ av,
                                                       const double* __restrict__ theta, double* __restrict__ part) {
    double v[1] = {HUGE_VAL};
    const int op[1] = {2};
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += (gridDim.x * blockDim.x) >> 5) {
        double s = 0.0;
        for (int q = rp[i] + lane; q < rp[i + 1]; q += 32) s += av[q] * av[q] * theta[ci[q]];
        s = warp_sum(s);
        v[0] = fmin(v[0], s);
    }
    block_partials<1>(v, op, part);
}

struct EpiNegSub {     // out = -d - a   (rhs_y = -A wr - rp)
    const double* a;
    double* out;
    __device__ void operator()(int i, double d) const { out[i] = -d - a[i]; }
};
struct EpiDx {         // dx = theta (d + rhs_x)
    const double *theta, *rhsx;
    double* dx;
    __device__ void operator()(int j, double d) const { dx[j] = theta[j] * (d + rhsx[j]); }
};
struct EpiStore {
    double* out;
    __device__ void operator()(int i, double d) const { out[i] = d; }
};

// dzl, dzu and the step-length ratios; partials [min primal ratio, min dual ratio]
__global__ void __launch_bounds__(kThreads) k_qp_dz(int n, const double* __restrict__ x, const double* __restrict__ dx,
                                                    const double* __restrict__ zl, const double* __restrict__ zu,
                                                    const double* __restrict__ lb, const double* __restrict__ ub,
                                                    const double* __restrict__ scal, double* __restrict__ dzl,
                                                    double* __restrict__ dzu, double* __restrict__ part) {
    const double smu = scal[0];
    double v[2] = {HUGE_VAL, HUGE_VAL};
    const int op[2] = {2, 2};
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double a = 0.0, b = 0.0;
        if (has_lo(lb[j])) {
            const double g = fmax(x[j] - lb[j], 1e-12);
            a = (smu - zl[j] * g - zl[j] * dx[j]) / g;
            if (dx[j] < 0.0) v[0] = fmin(v[0], -(x[j] - lb[j]) / dx[j]);
            if (a < 0.0 && zl[j] > 0.0) v[1] = fmin(v[1], -zl[j] / a);
        }
        if (has_hi(ub[j])) {
            const double g = fmax(ub[j] - x[j], 1e-12);
            b = (smu - zu[j] * g + zu[j] * dx[j]) / g;
            if (dx[j] > 0.0) v[0] = fmin(v[0], (ub[j] - x[j]) / dx[j]);
            if (b < 0.0 && zu[j] > 0.0) v[1] = fmin(v[1], -zu[j] / b);
        }
        dzl[j] = a;
        dzu[j] = b;
    }
    block_partials<2>(v, op, part);
}

__global__ void k_qp_update_n(int n, const double* __restrict__ dx, const double* __restrict__ dzl,
                              const double* __restrict__ dzu, const double* __restrict__ lb,
                              const double* __restrict__ ub, const double* __restrict__ steps, double* __restrict__ x,
                              double* __restrict__ zl, double* __restrict__ zu) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double ap = steps[0], ad = steps[1];
    x[j] += ap * dx[j];
    double a = zl[j] + ad * dzl[j], b = zu[j] + ad * dzu[j];
    if (has_lo(lb[j])) a = fmax(a, 1e-14);
    if (has_hi(ub[j])) b = fmax(b, 1e-14);
    zl[j] = a;
    zu[j] = b;
}

__global__ void k_qp_axpy(int m, const double* __restrict__ steps, int which, const double* __restrict__ d,
                          double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) y[i] += steps[which] * d[i];
}

__global__ void k_qp_start(int n, const double* __restrict__ lb, const double* __restrict__ ub, double* __restrict__ x,
                           double* __restrict__ zl, double* __restrict__ zu) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const bool l = has_lo(lb[j]), u = has_hi(ub[j]);
    x[j] = ((l ? lb[j] : -10.0) + (u ? ub[j] : 10.0)) / 2.0;
    zl[j] = l ? 1.0 : 0.0;
    zu[j] = u ? 1.0 : 0.0;
}

// PCG vector steps: x += a p, r -= a q; p = z + b p; r -= q
__global__ void k_qp_cg1(int m, double a, const double* __restrict__ p, const double* __restrict__ q,
                         double* __restrict__ x, double* __restrict__ r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) { x[i] += a * p[i]; r[i] -= a * q[i]; }
}
__global__ void k_qp_cg2(int m, double b, const double* __restrict__ z, double* __restrict__ p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) p[i] = z[i] + b * p[i];
}
__global__ void k_qp_sub(int m, const double* __restrict__ q, double* __restrict__ r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) r[i] -= q[i];
}
// partials of [sum a b, max |a|]
__global__ void __launch_bounds__(kThreads) k_qp_dot(int m, const double* __restrict__ a, const double* __restrict__ b,
                                                     double* __restrict__ part) {
    double v[2] = {0.0, 0.0};
    const int op[2] = {0, 1};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        v[0] += a[i] * b[i];
        v[1] = fmax(v[1], fabs(a[i]));
    }
    block_partials<2>(v, op, part);
}

inline int nb(int64_t n) { return static_cast<int>((n + kThreads - 1) / kThreads); }

}  // namespace

QpOutcome solve_qp_device(const QpProblem& qp, const QpSettings& s) {
    const int m = qp.m, n = qp.n;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw api::sk_exception(SK_ERR_NO_DEVICE, "no CUDA device visible");
    cudaStream_t st = nullptr;
    SK_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { if (s) cudaStreamDestroy(s); }
    } guard{st};
    const int nz = qp.col_ptrs[n];
    // CSR of A and CSR of A^T (= the CSC arrays)
    core::CSRMatrix A;
    A.rows = m;
    A.cols = n;
    A.row_ptrs.assign(static_cast<size_t>(m) + 1, 0);
    for (int q = 0; q < nz; ++q) A.row_ptrs[qp.row_idx[q] + 1]++;
    for (int i = 0; i < m; ++i) A.row_ptrs[i + 1] += A.row_ptrs[i];
    A.col_indices.resize(static_cast<size_t>(nz));
    A.values.resize(static_cast<size_t>(nz));
    {
        std::vector<int> nx(A.row_ptrs.begin(), A.row_ptrs.end() - 1);
        for (int j = 0; j < n; ++j)
            for (int q = qp.col_ptrs[j]; q < qp.col_ptrs[j + 1]; ++q) {
                const int d = nx[qp.row_idx[q]]++;
                A.col_indices[d] = j;
                A.values[d] = qp.vals[q];
            }
    }
    Arena ar;
    Slot<int> a_rp, a_ci, t_rp, t_ci, row_lp, col_lp;
    Slot<double> a_v, t_v, b, c, lb, ub, h, x, y, zl, zu, rd, rp, ax, aty, theta, rhsx, wr, rhsy, dy, dx, dzl, dzu;
    Slot<double> pr, pz, pp, pq, part, red, scal;
    const int mm = std::max(1, m);
    reserve(ar, a_rp, mm + 1); reserve(ar, a_ci, std::max(1, nz)); reserve(ar, a_v, std::max(1, nz));
    reserve(ar, t_rp, n + 1); reserve(ar, t_ci, std::max(1, nz)); reserve(ar, t_v, std::max(1, nz));
    reserve(ar, row_lp, mm); reserve(ar, col_lp, n);
    for (auto* sl : {&c, &lb, &ub, &h, &x, &zl, &zu, &rd, &aty, &theta, &rhsx, &wr, &dx, &dzl, &dzu}) reserve(ar, *sl, n);
    for (auto* sl : {&b, &y, &rp, &ax, &rhsy, &dy, &pr, &pz, &pp, &pq}) reserve(ar, *sl, mm);
    reserve(ar, part, kBlocks * 8);     // up to five partials per block (primal 2 + dual 3)
    reserve(ar, red, 8);
    reserve(ar, scal, 4);
    ar.commit();
    for (auto* sl : {&a_rp, &a_ci, &t_rp, &t_ci, &row_lp, &col_lp}) bind(ar, *sl);
    for (auto* sl : {&a_v, &t_v, &b, &c, &lb, &ub, &h, &x, &y, &zl, &zu, &rd, &rp, &ax, &aty, &theta, &rhsx, &wr,
                     &rhsy, &dy, &dx, &dzl, &dzu, &pr, &pz, &pp, &pq, &part, &red, &scal})
        bind(ar, *sl);
    if (m > 0) {
        upload(a_rp, A.row_ptrs, st); upload(a_ci, A.col_indices, st); upload(a_v, A.values, st);
        upload(b, qp.b, st);
    }
    upload(t_rp, qp.col_ptrs, st); upload(t_ci, qp.row_idx, st); upload(t_v, qp.vals, st);
    upload(c, qp.c, st); upload(lb, qp.lb, st); upload(ub, qp.ub, st); upload(h, qp.h, st);
    SK_CUDA(cudaMemsetAsync(row_lp.ptr, 0, sizeof(int) * mm, st));
    SK_CUDA(cudaMemsetAsync(col_lp.ptr, 0, sizeof(int) * n, st));
    SK_CUDA(cudaMemsetAsync(y.ptr, 0, sizeof(double) * mm, st));
    SK_CUDA(cudaMemsetAsync(aty.ptr, 0, sizeof(double) * n, st));
    std::unique_ptr<KktEngine> eng;
    DeviceLP dlp;
    if (m > 0) {
        ipm::LpView v;
        v.m = m; v.n = n; v.col_ptrs = qp.col_ptrs.data(); v.row_idx = qp.row_idx.data(); v.vals = qp.vals.data();
        ipm::FrontPlan plan;
        ipm::build_front_plan({v}, A, SK_ORDER_AUTO, plan);
        dlp.nlp = 1; dlp.M = m; dlp.N = n; dlp.nnz = nz;
        dlp.a_rp = a_rp.ptr; dlp.a_ci = a_ci.ptr; dlp.a_v = a_v.ptr;
        dlp.t_rp = t_rp.ptr; dlp.t_ci = t_ci.ptr; dlp.t_v = t_v.ptr;
        dlp.row_lp = row_lp.ptr; dlp.col_lp = col_lp.ptr;
        eng.reset(new KktEngine(plan, dlp, st));
    }
    k_qp_start<<<nb(n), kThreads, 0, st>>>(n, lb.ptr, ub.ptr, x.ptr, zl.ptr, zu.ptr);
    int ncomp = 0;
    for (int j = 0; j < n; ++j) ncomp += (qp.lb[j] > -kBoundInf) + (qp.ub[j] < kBoundInf);
    auto fetch = [&](int count) {
        std::vector<double> hv(static_cast<size_t>(count));
        SK_CUDA(cudaMemcpyAsync(hv.data(), red.ptr, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
        return hv;
    };
    QpOutcome out;
    out.status = 3;                     // iteration limit unless a test below decides otherwise
    const double sigma = 0.2, eta = 0.995;
    for (int it = 0; it < s.max_iter; ++it) {
        out.iterations = it;
        // residuals, mu, objective
        if (m > 0) {
            spmv(n, 8, t_rp.ptr, t_ci.ptr, t_v.ptr, y.ptr, EpiStore{aty.ptr}, st);
            spmv(m, 8, a_rp.ptr, a_ci.ptr, a_v.ptr, x.ptr, EpiStore{ax.ptr}, st);
            k_qp_primal<<<kBlocks, kThreads, 0, st>>>(m, ax.ptr, b.ptr, y.ptr, rp.ptr, part.ptr);
            k_qp_final<2><<<1, 32, 0, st>>>(part.ptr, kBlocks, 1, 1, 0, 0, red.ptr);
        }
        k_qp_dual<<<kBlocks, kThreads, 0, st>>>(n, h.ptr, x.ptr, c.ptr, aty.ptr, zl.ptr, zu.ptr, lb.ptr, ub.ptr,
                                                rd.ptr, part.ptr + 2 * kBlocks);
        k_qp_final<3><<<1, 32, 0, st>>>(part.ptr + 2 * kBlocks, kBlocks, 0, 1, 0, 0, red.ptr + 2);
        SK_CUDA(cudaGetLastError());
        std::vector<double> hv = fetch(5);
        const double nrp = m > 0 ? hv[0] : 0.0, ny = m > 0 ? hv[1] : 0.0;
        double mu = hv[2];
        if (ncomp > 0) mu /= ncomp;
        const double nrd = hv[3], obj = hv[4];
        out.primal_residual = nrp;
        out.dual_residual = nrd;
        out.complementarity = mu;
        out.objective = obj;
        if (nrp < s.feas_tol && nrd < s.dual_tol && mu < s.grad_tol) {
            out.status = 0;
            break;
        }
        if (ny > 1e15) { out.status = 1; return out; }
        if (obj < -1e15) { out.status = 2; return out; }
        // W = h + D, theta, rhs_x
        const double smu = sigma * mu;
        SK_CUDA(cudaMemcpyAsync(scal.ptr, &smu, sizeof(double), cudaMemcpyHostToDevice, st));
        k_qp_prep<<<kBlocks, kThreads, 0, st>>>(n, h.ptr, x.ptr, zl.ptr, zu.ptr, lb.ptr, ub.ptr, rd.ptr, scal.ptr,
                                                theta.ptr, rhsx.ptr, wr.ptr, part.ptr);
        k_qp_final<1><<<1, 32, 0, st>>>(part.ptr, kBlocks, 2, 0, 0, 0, red.ptr);
        if (m > 0) {
            k_qp_sdiag<<<kBlocks, kThreads, 0, st>>>(m, a_rp.ptr, a_ci.ptr, a_v.ptr, theta.ptr, part.ptr + kBlocks);
            k_qp_final<1><<<1, 32, 0, st>>>(part.ptr + kBlocks, kBlocks, 2, 0, 0, 0, red.ptr + 1);
        }
        hv = fetch(2);
        if (!(hv[0] > 1e-14) || (m > 0 && !(hv[1] > 1e-14))) { out.status = 4; return out; }
        if (m > 0) {
            // rhs_y = -A (theta rhs_x) - rp; S dy = rhs_y
            spmv(m, 8, a_rp.ptr, a_ci.ptr, a_v.ptr, wr.ptr, EpiNegSub{rp.ptr, rhsy.ptr}, st);
            bool ok = false;
            double delta = 1e-12;
            for (int r = 0; r < 6 && !ok; ++r, delta *= 10.0) ok = eng->factor(theta.ptr, delta, false);
            if (!ok) { out.status = 4; return out; }
            // PCG on S with the regularised factor as preconditioner; r = rhs_y - S dy with
            // S applied matrix-free in FP64
            eng->apply_inverse(rhsy.ptr, dy.ptr);
            eng->apply_normal(theta.ptr, dy.ptr, pq.ptr);
            SK_CUDA(cudaMemcpyAsync(pr.ptr, rhsy.ptr, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
            k_qp_sub<<<nb(m), kThreads, 0, st>>>(m, pq.ptr, pr.ptr);
            k_qp_dot<<<kBlocks, kThreads, 0, st>>>(m, rhsy.ptr, rhsy.ptr, part.ptr);
            k_qp_final<2><<<1, 32, 0, st>>>(part.ptr, kBlocks, 0, 1, 0, 0, red.ptr);
            const double bn = fetch(2)[1];
            const double target = 1e-13 * std::max(1.0, bn);
            eng->apply_inverse(pr.ptr, pz.ptr);
            SK_CUDA(cudaMemcpyAsync(pp.ptr, pz.ptr, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
            k_qp_dot<<<kBlocks, kThreads, 0, st>>>(m, pr.ptr, pz.ptr, part.ptr);
            k_qp_final<2><<<1, 32, 0, st>>>(part.ptr, kBlocks, 0, 1, 0, 0, red.ptr);
            std::vector<double> rz = fetch(2);
            double rzv = rz[0], rnorm = rz[1];
            for (int k = 0; k < 50 && rnorm > target && rzv > 0.0; ++k) {
                eng->apply_normal(theta.ptr, pp.ptr, pq.ptr);
                k_qp_dot<<<kBlocks, kThreads, 0, st>>>(m, pp.ptr, pq.ptr, part.ptr);
                k_qp_final<2><<<1, 32, 0, st>>>(part.ptr, kBlocks, 0, 1, 0, 0, red.ptr);
                const double pqv = fetch(2)[0];
                if (!(pqv > 0.0)) break;
                const double a = rzv / pqv;
                k_qp_cg1<<<nb(m), kThreads, 0, st>>>(m, a, pp.ptr, pq.ptr, dy.ptr, pr.ptr);
                eng->apply_inverse(pr.ptr, pz.ptr);
                k_qp_dot<<<kBlocks, kThreads, 0, st>>>(m, pr.ptr, pz.ptr, part.ptr);
                k_qp_final<2><<<1, 32, 0, st>>>(part.ptr, kBlocks, 0, 1, 0, 0, red.ptr);
                rz = fetch(2);
                rnorm = rz[1];
                if (!(rz[0] > 0.0)) break;
                k_qp_cg2<<<nb(m), kThreads, 0, st>>>(m, rz[0] / rzv, pz.ptr, pp.ptr);
                rzv = rz[0];
            }
            // dx = theta (A^T dy + rhs_x)
            spmv(n, 8, t_rp.ptr, t_ci.ptr, t_v.ptr, dy.ptr, EpiDx{theta.ptr, rhsx.ptr, dx.ptr}, st);
        } else {
            SK_CUDA(cudaMemcpyAsync(dx.ptr, wr.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        }
        // dzl, dzu, step lengths
        k_qp_dz<<<kBlocks, kThreads, 0, st>>>(n, x.ptr, dx.ptr, zl.ptr, zu.ptr, lb.ptr, ub.ptr, scal.ptr, dzl.ptr,
                                              dzu.ptr, part.ptr);
        k_qp_final<2><<<1, 32, 0, st>>>(part.ptr, kBlocks, 2, 2, 0, 0, red.ptr);
        hv = fetch(2);
        const double steps[2] = {std::min(1.0, eta * std::min(1.0, hv[0])), std::min(1.0, eta * std::min(1.0, hv[1]))};
        SK_CUDA(cudaMemcpyAsync(scal.ptr + 1, steps, sizeof(steps), cudaMemcpyHostToDevice, st));
        k_qp_update_n<<<nb(n), kThreads, 0, st>>>(n, dx.ptr, dzl.ptr, dzu.ptr, lb.ptr, ub.ptr, scal.ptr + 1, x.ptr,
                                                  zl.ptr, zu.ptr);
        if (m > 0) k_qp_axpy<<<nb(m), kThreads, 0, st>>>(m, scal.ptr + 1, 1, dy.ptr, y.ptr);
        SK_CUDA(cudaGetLastError());
    }
    if (out.status == 3) out.iterations = s.max_iter;
    if (out.status == 0 || out.status == 3) {
        out.x.resize(static_cast<size_t>(n));
        out.y.resize(static_cast<size_t>(m));
        std::vector<double> hl(static_cast<size_t>(n)), hu(static_cast<size_t>(n));
        SK_CUDA(cudaMemcpyAsync(out.x.data(), x.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if (m > 0) SK_CUDA(cudaMemcpyAsync(out.y.data(), y.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaMemcpyAsync(hl.data(), zl.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaMemcpyAsync(hu.data(), zu.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
        out.z.resize(static_cast<size_t>(n));
        for (int j = 0; j < n; ++j) out.z[j] = hl[j] - hu[j];
    }
    return out;
}

}  // namespace dev
}  // namespace sankhya
