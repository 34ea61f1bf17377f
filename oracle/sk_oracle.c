/*
 * CPU oracle for the device Mehrotra IPM path -- TEST INFRASTRUCTURE ONLY.
 * Plain-C restatement of the reference's algorithm; see sk_oracle.h for the
 * reference file:line each function follows. Only tests/, the smoke check and
 * the benchmark's CPU-baseline leg use it, and only as the checker.
 */
#include "sk_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- helpers */

static unsigned char* adjacency_aat(int m, int n, const int* rp, const int* ci) {
    /* Dense boolean graph of A A^T (no self loops) from CSR A. */
    unsigned char* adj = (unsigned char*)calloc((size_t)m * (size_t)m, 1);
    int* cnt = (int*)calloc((size_t)n + 1, sizeof(int));
    int nz = rp[m];
    int* crow = (int*)malloc(sizeof(int) * (size_t)(nz > 0 ? nz : 1));
    for (int k = 0; k < nz; ++k) cnt[ci[k] + 1]++;
    for (int j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
    int* pos = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int j = 0; j < n; ++j) pos[j] = cnt[j];
    for (int i = 0; i < m; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) crow[pos[ci[k]]++] = i;
    for (int j = 0; j < n; ++j)
        for (int a = cnt[j]; a < cnt[j + 1]; ++a)
            for (int b = a + 1; b < cnt[j + 1]; ++b) {
                int u = crow[a], v = crow[b];
                if (u == v) continue;
                adj[(size_t)u * m + v] = 1;
                adj[(size_t)v * m + u] = 1;
            }
    free(cnt); free(crow); free(pos);
    return adj;
}

/* ------------------------------------------- ordering: symbolic.cpp:11-98 */

int oracle_min_degree(int m, int n, const int* rp, const int* ci, int* P) {
    unsigned char* adj = adjacency_aat(m, n, rp, ci);
    unsigned char* gone = (unsigned char*)calloc((size_t)m + 1, 1);
    int* deg = (int*)calloc((size_t)m + 1, sizeof(int));
    int* nb = (int*)malloc(sizeof(int) * (size_t)(m + 1));
    for (int i = 0; i < m; ++i) {
        int d = 0;
        for (int j = 0; j < m; ++j) d += adj[(size_t)i * m + j];
        deg[i] = d;
    }
    for (int step = 0; step < m; ++step) {
        int u = -1, best = m + 1;
        for (int i = 0; i < m; ++i)           /* strict '<': lowest index wins ties */
            if (!gone[i] && deg[i] < best) { best = deg[i]; u = i; }
        if (u < 0) { free(adj); free(gone); free(deg); free(nb); return -1; }
        gone[u] = 1;
        P[step] = u;
        int k = 0;
        for (int v = 0; v < m; ++v)
            if (adj[(size_t)u * m + v]) nb[k++] = v;
        for (int a = 0; a < k; ++a) {         /* neighbours lose u and gain the clique */
            int v = nb[a];
            if (adj[(size_t)v * m + u]) { adj[(size_t)v * m + u] = 0; deg[v]--; }
            for (int b = 0; b < k; ++b) {
                int w = nb[b];
                if (w == v) continue;
                if (!adj[(size_t)v * m + w]) { adj[(size_t)v * m + w] = 1; deg[v]++; }
            }
        }
    }
    free(adj); free(gone); free(deg); free(nb);
    return 0;
}

/* ------------------------------------ symbolic pass: symbolic.cpp:100-218 */

int oracle_symbolic(int m, int n, const int* rp, const int* ci, const int* P,
                    int* P_inv, int* parent, int* L_row_ptrs, int* L_cols, int L_cap) {
    unsigned char* adj = adjacency_aat(m, n, rp, ci);
    for (int i = 0; i < m; ++i) P_inv[P[i]] = i;
    /* Lstr[j*m + i] = 1 iff L(i, j) != 0 for i > j (permuted numbering). */
    unsigned char* Lstr = (unsigned char*)calloc((size_t)m * (size_t)m + 1, 1);
    for (int u = 0; u < m; ++u)
        for (int v = 0; v < m; ++v)
            if (adj[(size_t)u * m + v]) {
                int pu = P_inv[u], pv = P_inv[v];
                if (pu > pv) Lstr[(size_t)pv * m + pu] = 1;
            }
    for (int j = 0; j < m; ++j) {
        for (int i = 0; i < j; ++i)
            if (parent[i] == j)
                for (int r = j + 1; r < m; ++r)
                    if (Lstr[(size_t)i * m + r]) Lstr[(size_t)j * m + r] = 1;
        parent[j] = -1;
        for (int r = j + 1; r < m; ++r)
            if (Lstr[(size_t)j * m + r]) { parent[j] = r; break; }
    }
    int nnz = 0;
    L_row_ptrs[0] = 0;
    for (int i = 0; i < m; ++i) {
        for (int j = 0; j < i; ++j)
            if (Lstr[(size_t)j * m + i]) {
                if (nnz >= L_cap) { free(adj); free(Lstr); return -1; }
                L_cols[nnz++] = j;
            }
        L_row_ptrs[i + 1] = nnz;
    }
    free(adj); free(Lstr);
    return nnz;
}

/* ---------------------------------------------------- dense linear algebra */

/* M0 = A diag(theta) A^T (dense, row-major m x m) from CSR A. */
static void form_normal_matrix(int m, const int* rp, const int* ci, const double* v,
                               const double* theta, double* M) {
    memset(M, 0, sizeof(double) * (size_t)m * (size_t)m);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j <= i; ++j) {
            double acc = 0.0;
            int a = rp[i], ae = rp[i + 1], b = rp[j], be = rp[j + 1];
            while (a < ae && b < be) {
                if (ci[a] == ci[b]) { acc += v[a] * theta[ci[a]] * v[b]; ++a; ++b; }
                else if (ci[a] < ci[b]) ++a;
                else ++b;
            }
            M[(size_t)i * m + j] = acc;
            M[(size_t)j * m + i] = acc;
        }
}

/* Up-looking row Cholesky of the dense SPD matrix (lower part of M, row-major),
 * L stored row-major lower. Returns 0 if a pivot is not positive. */
static int dense_cholesky(int m, const double* M, double* L) {
    for (int i = 0; i < m; ++i) {
        double* Li = L + (size_t)i * m;
        for (int j = 0; j < i; ++j) {
            const double* Lj = L + (size_t)j * m;
            double s = M[(size_t)i * m + j];
            for (int k = 0; k < j; ++k) s -= Li[k] * Lj[k];
            Li[j] = s / Lj[j];
        }
        double d = M[(size_t)i * m + i];
        for (int k = 0; k < i; ++k) d -= Li[k] * Li[k];
        if (!(d > 0.0)) return 0;
        Li[i] = sqrt(d);
        for (int k = i + 1; k < m; ++k) Li[k] = 0.0;
    }
    return 1;
}

static void chol_solve(int m, const double* L, double* x) {
    for (int i = 0; i < m; ++i) {
        double s = x[i];
        const double* Li = L + (size_t)i * m;
        for (int k = 0; k < i; ++k) s -= Li[k] * x[k];
        x[i] = s / Li[i];
    }
    for (int i = m - 1; i >= 0; --i) {
        double s = x[i];
        for (int k = i + 1; k < m; ++k) s -= L[(size_t)k * m + i] * x[k];
        x[i] = s / L[(size_t)i * m + i];
    }
}

static double norm_inf(int n, const double* v) {
    double r = 0.0;
    for (int i = 0; i < n; ++i) { double a = fabs(v[i]); if (a > r) r = a; }
    return r;
}

static double norm2(int n, const double* v) {
    double r = 0.0;
    for (int i = 0; i < n; ++i) r += v[i] * v[i];
    return sqrt(r);
}

/* --------------------------------------------- KKT solve: kkt.cu:620-870 */

typedef struct kkt_ctx {
    int m;
    double* M0;   /* permuted, dense row-major */
    double* Md;   /* D M0 D + delta I */
    double* L;
    double* D;
    double* w1; double* w2; double* w3; double* w4;
} kkt_ctx;

static void kkt_init(kkt_ctx* k, int m) {
    k->m = m;
    size_t mm = (size_t)m * (size_t)m;
    k->M0 = (double*)malloc(sizeof(double) * (mm + 1));
    k->Md = (double*)malloc(sizeof(double) * (mm + 1));
    k->L = (double*)malloc(sizeof(double) * (mm + 1));
    k->D = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    k->w1 = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    k->w2 = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    k->w3 = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    k->w4 = (double*)malloc(sizeof(double) * ((size_t)m + 1));
}

static void kkt_free(kkt_ctx* k) {
    free(k->M0); free(k->Md); free(k->L); free(k->D);
    free(k->w1); free(k->w2); free(k->w3); free(k->w4);
}

static void m0_residual(const kkt_ctx* k, const double* dy, const double* rhs, double* r) {
    int m = k->m;
    for (int i = 0; i < m; ++i) {
        double s = 0.0;
        const double* Mi = k->M0 + (size_t)i * m;
        for (int j = 0; j < m; ++j) s += Mi[j] * dy[j];
        r[i] = rhs[i] - s;
    }
}

/* rhs_p and dy_p are in permuted order. Returns 1 on success. */
static int kkt_solve_permuted(kkt_ctx* k, const double* rhs_p, double tol, double* dy_p) {
    int m = k->m;
    double* r = k->w1; double* t = k->w2; double* backup = k->w3;
    for (int i = 0; i < m; ++i) {
        double a = fabs(k->M0[(size_t)i * m + i]);
        if (a < 1e-12) a = 1e-12;
        k->D[i] = 1.0 / sqrt(a);
    }
    double delta = 1e-9;
    int success = 0;
    for (int retry = 0; retry < 5; ++retry) {
        if (retry > 0) delta *= 10.0;
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j)
                k->Md[(size_t)i * m + j] = k->M0[(size_t)i * m + j] * k->D[i] * k->D[j] + (i == j ? delta : 0.0);
        if (!dense_cholesky(m, k->Md, k->L)) continue;
        for (int i = 0; i < m; ++i) t[i] = rhs_p[i] * k->D[i];
        chol_solve(m, k->L, t);
        for (int i = 0; i < m; ++i) dy_p[i] = t[i] * k->D[i];
        m0_residual(k, dy_p, rhs_p, r);
        double before = norm_inf(m, r);
        if (before <= tol) { success = 1; break; }
        int converged = 0;
        for (int it = 0; it < 10; ++it) {
            memcpy(backup, dy_p, sizeof(double) * (size_t)m);
            for (int i = 0; i < m; ++i) t[i] = r[i] * k->D[i];
            chol_solve(m, k->L, t);
            for (int i = 0; i < m; ++i) dy_p[i] += t[i] * k->D[i];
            m0_residual(k, dy_p, rhs_p, r);
            double after = norm_inf(m, r);
            if (after <= tol) { converged = 1; break; }
            if (after >= before) {
                memcpy(dy_p, backup, sizeof(double) * (size_t)m);
                m0_residual(k, dy_p, rhs_p, r);
                break;
            }
            before = after;
        }
        success = converged;
        break;
    }
    return success;
}

/* Robust-mode solve: preconditioned conjugate gradients on M0 dy = rhs with the
 * preconditioner D (L L^T)^{-1} D of the regularised factor (delta raised x10 up to
 * 5 times while a pivot is not positive), up to `maxit` iterations; returns the
 * best iterate by true residual. Returns 1 when ||rhs - M0 dy||_inf <= tol. */
static int kkt_solve_pcg(kkt_ctx* k, const double* rhs, double tol, double* x, int maxit) {
    int m = k->m;
    for (int i = 0; i < m; ++i) {
        double a = fabs(k->M0[(size_t)i * m + i]);
        if (a < 1e-12) a = 1e-12;
        k->D[i] = 1.0 / sqrt(a);
    }
    double delta = 1e-9;
    int factored = 0;
    for (int retry = 0; retry < 5 && !factored; ++retry, delta *= 10.0) {
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < m; ++j)
                k->Md[(size_t)i * m + j] = k->M0[(size_t)i * m + j] * k->D[i] * k->D[j] + (i == j ? delta : 0.0);
        factored = dense_cholesky(m, k->Md, k->L);
    }
    if (!factored) return 0;
    double* r = k->w1; double* z = k->w2; double* pv = k->w3; double* q = k->w4;
    double* best = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    /* x = B rhs */
    for (int i = 0; i < m; ++i) x[i] = rhs[i] * k->D[i];
    chol_solve(m, k->L, x);
    for (int i = 0; i < m; ++i) x[i] *= k->D[i];
    m0_residual(k, x, rhs, r);
    double bestn = norm_inf(m, r);
    memcpy(best, x, sizeof(double) * (size_t)m);
    if (bestn > tol) {
        for (int i = 0; i < m; ++i) z[i] = r[i] * k->D[i];
        chol_solve(m, k->L, z);
        for (int i = 0; i < m; ++i) { z[i] *= k->D[i]; pv[i] = z[i]; }
        double rz = 0.0;
        for (int i = 0; i < m; ++i) rz += r[i] * z[i];
        for (int it = 0; it < maxit; ++it) {
            for (int i = 0; i < m; ++i) {
                double s = 0.0;
                const double* Mi = k->M0 + (size_t)i * m;
                for (int j = 0; j < m; ++j) s += Mi[j] * pv[j];
                q[i] = s;
            }
            double pq = 0.0;
            for (int i = 0; i < m; ++i) pq += pv[i] * q[i];
            if (!(pq > 0.0) || !(rz > 0.0)) break;
            const double alpha = rz / pq;
            for (int i = 0; i < m; ++i) { x[i] += alpha * pv[i]; r[i] -= alpha * q[i]; }
            const double rn = norm_inf(m, r);
            if (rn < bestn) { bestn = rn; memcpy(best, x, sizeof(double) * (size_t)m); }
            if (rn <= tol) break;
            for (int i = 0; i < m; ++i) z[i] = r[i] * k->D[i];
            chol_solve(m, k->L, z);
            double rz2 = 0.0;
            for (int i = 0; i < m; ++i) { z[i] *= k->D[i]; rz2 += r[i] * z[i]; }
            const double beta = rz2 / rz;
            rz = rz2;
            for (int i = 0; i < m; ++i) pv[i] = z[i] + beta * pv[i];
        }
    }
    memcpy(x, best, sizeof(double) * (size_t)m);
    m0_residual(k, x, rhs, r);
    bestn = norm_inf(m, r);
    free(best);
    return bestn <= tol;
}

int oracle_kkt_solve(int m, int n, const int* rp, const int* ci, const double* v,
                     const double* theta, const int* P, const double* rhs, double tol, int rel,
                     double* dy) {
    (void)n;
    kkt_ctx k;
    kkt_init(&k, m);
    double* M = (double*)malloc(sizeof(double) * ((size_t)m * m + 1));
    form_normal_matrix(m, rp, ci, v, theta, M);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            int pi = P ? P[i] : i, pj = P ? P[j] : j;
            k.M0[(size_t)i * m + j] = M[(size_t)pi * m + pj];
        }
    double* rp_ = (double*)calloc((size_t)m + 1, sizeof(double));
    double* dp = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    for (int i = 0; i < m; ++i) rp_[i] = rhs[P ? P[i] : i];
    double t = tol;
    if (rel) { double nr = norm_inf(m, rhs); t = tol * (nr > 1.0 ? nr : 1.0); }
    int ok = kkt_solve_permuted(&k, rp_, t, dp);
    for (int i = 0; i < m; ++i) dy[P ? P[i] : i] = dp[i];
    free(M); free(rp_); free(dp);
    kkt_free(&k);
    return ok;
}

/* ------------------------------------------- IPM: mehrotra_device.cu */

typedef struct lp_s {
    int m, n;
    const int* cp; const int* ri; double* va;   /* scaled CSC values */
    int* rp; int* ci; double* rv;               /* scaled CSR */
} lp_s;

static void spmv_A(const lp_s* p, const double* x, double* out) {  /* out = A x */
    for (int i = 0; i < p->m; ++i) {
        double s = 0.0;
        for (int k = p->rp[i]; k < p->rp[i + 1]; ++k) s += p->rv[k] * x[p->ci[k]];
        out[i] = s;
    }
}

static void spmv_At(const lp_s* p, const double* y, double* out) { /* out = A^T y */
    for (int j = 0; j < p->n; ++j) {
        double s = 0.0;
        for (int k = p->cp[j]; k < p->cp[j + 1]; ++k) s += p->va[k] * y[p->ri[k]];
        out[j] = s;
    }
}

static double step_length(int n, const double* v, const double* dv) {
    double r = 1.0e30;
    for (int i = 0; i < n; ++i)
        if (dv[i] < 0.0) { double t = -v[i] / dv[i]; if (t < r) r = t; }
    return r;
}

static double dot(int n, const double* a, const double* b) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

typedef struct ipm_ws {
    double *rp, *rd, *theta, *rxs, *v, *rkkt, *dy, *dx, *ds, *dx_aff, *ds_aff, *dy_aff;
    double *tx, *ts, *bx, *by, *bs, *brp, *brd, *t1, *t2, *t3, *rk_p, *dy_p;
    double* M;
} ipm_ws;

/* Solve the normal equations for rkkt -> dy with the reference's KKT rules. */
static int g_verbose = 0;
static int g_strict = 0;

static int normal_solve(const lp_s* p, kkt_ctx* k, const double* theta, const double* rkkt,
                        double tol, double* dy, int* nsolves) {
    (void)theta;
    (void)p;
    ++*nsolves;
    /* M0 was formed for this iteration by the caller; identity permutation (the
     * reference's ordering only changes fill and rounding, not the operator). */
    int ok = g_strict ? kkt_solve_permuted(k, rkkt, tol, dy) : kkt_solve_pcg(k, rkkt, tol, dy, 50);
    if (g_verbose) {
        m0_residual(k, dy, rkkt, k->w4);
        fprintf(stderr, "  solve ok=%d resid_inf %.3e tol %.3e rhs_inf %.3e\n", ok, norm_inf(k->m, k->w4), tol,
                norm_inf(k->m, rkkt));
    }
    return ok;
}

static int verify_direction(const lp_s* p, ipm_ws* w, const double* x, const double* s,
                            const double* dx, const double* dy, const double* ds, const double* rxs,
                            double nrp, double nrd, double limit) {
    int m = p->m, n = p->n;
    spmv_A(p, dx, w->t1);
    for (int i = 0; i < m; ++i) w->t1[i] += w->rp[i];
    spmv_At(p, dy, w->t2);
    for (int j = 0; j < n; ++j) w->t2[j] += w->rd[j] + ds[j];
    for (int j = 0; j < n; ++j) w->t3[j] = s[j] * dx[j] + x[j] * ds[j] - rxs[j];
    double e1 = norm2(m, w->t1) / fmax(1.0, nrp);
    double e2 = norm2(n, w->t2) / fmax(1.0, nrd);
    double e3 = norm2(n, w->t3) / fmax(1.0, norm2(n, rxs));
    if (g_verbose) fprintf(stderr, "  verify e1 %.3e e2 %.3e e3 %.3e\n", e1, e2, e3);
    if (!(isfinite(e1) && isfinite(e2) && isfinite(e3))) return 0;
    return !(e1 > limit || e2 > limit || e3 > limit);
}

static void residuals(const lp_s* p, const double* b, const double* c, const double* x,
                      const double* y, const double* s, double* rp, double* rd) {
    spmv_A(p, x, rp);
    for (int i = 0; i < p->m; ++i) rp[i] -= b[i];
    spmv_At(p, y, rd);
    for (int j = 0; j < p->n; ++j) rd[j] += s[j] - c[j];
}

void oracle_kkt_measures(int m, int n, const int* cp, const int* ri, const double* va,
                         const double* b, const double* c, const double* x, const double* y,
                         const double* s, double* out) {
    double* ax = (double*)calloc((size_t)m + 1, sizeof(double));
    double pinf = 0.0, dinf = 0.0, cx = 0.0, by = 0.0, minx = 1e300, mins = 1e300;
    for (int j = 0; j < n; ++j) {
        double aty = 0.0;
        for (int k = cp[j]; k < cp[j + 1]; ++k) { ax[ri[k]] += va[k] * x[j]; aty += va[k] * y[ri[k]]; }
        double r = fabs(aty + s[j] - c[j]);
        if (r > dinf) dinf = r;
        cx += c[j] * x[j];
        if (x[j] < minx) minx = x[j];
        if (s[j] < mins) mins = s[j];
    }
    for (int i = 0; i < m; ++i) { double r = fabs(ax[i] - b[i]); if (r > pinf) pinf = r; by += b[i] * y[i]; }
    out[0] = pinf / (1.0 + norm_inf(m, b));
    out[1] = dinf / (1.0 + norm_inf(n, c));
    out[2] = fabs(cx - by) / (1.0 + fabs(cx) + fabs(by));
    out[3] = cx;
    out[4] = minx;
    out[5] = mins;
    free(ax);
}

int oracle_ipm_solve(int m, int n, const int* cp, const int* ri, const double* va0,
                     const double* b0, const double* c0, const oracle_ipm_opts* o,
                     double* x_out, double* y_out, double* s_out, oracle_ipm_result* res) {
    oracle_ipm_opts opts = {0, 1e-8, 200, 0, 0, 0};
    if (o) opts = *o;
    g_verbose = opts.verbose > 1;
    g_strict = opts.strict;
    lp_s p;
    p.m = m; p.n = n; p.cp = cp; p.ri = ri;
    int nz = cp[n];
    p.va = (double*)malloc(sizeof(double) * ((size_t)nz + 1));
    memcpy(p.va, va0, sizeof(double) * (size_t)nz);
    /* CSR mirror (scaled in place together with the CSC values). */
    p.rp = (int*)calloc((size_t)m + 1, sizeof(int));
    p.ci = (int*)malloc(sizeof(int) * ((size_t)nz + 1));
    p.rv = (double*)malloc(sizeof(double) * ((size_t)nz + 1));
    int* csr_of = (int*)malloc(sizeof(int) * ((size_t)nz + 1)); /* CSR slot -> CSC slot */
    for (int k = 0; k < nz; ++k) p.rp[ri[k] + 1]++;
    for (int i = 0; i < m; ++i) p.rp[i + 1] += p.rp[i];
    int* nx = (int*)malloc(sizeof(int) * ((size_t)m + 1));
    for (int i = 0; i < m; ++i) nx[i] = p.rp[i];
    for (int j = 0; j < n; ++j)
        for (int k = cp[j]; k < cp[j + 1]; ++k) { int d = nx[ri[k]]++; p.ci[d] = j; csr_of[d] = k; }
    free(nx);

    /* 10-pass inline Ruiz (mehrotra_device.cu:289-323). */
    double* R = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    double* C = (double*)malloc(sizeof(double) * ((size_t)n + 1));
    double* b = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    double* c = (double*)malloc(sizeof(double) * ((size_t)n + 1));
    double* rmax = (double*)malloc(sizeof(double) * ((size_t)m + 1));
    double* cmax = (double*)malloc(sizeof(double) * ((size_t)n + 1));
    for (int i = 0; i < m; ++i) { R[i] = 1.0; b[i] = b0[i]; }
    for (int j = 0; j < n; ++j) { C[j] = 1.0; c[j] = c0[j]; }
    for (int pass = 0; pass < 10; ++pass) {
        for (int i = 0; i < m; ++i) rmax[i] = 0.0;
        for (int j = 0; j < n; ++j) cmax[j] = 0.0;
        for (int j = 0; j < n; ++j)
            for (int k = cp[j]; k < cp[j + 1]; ++k) {
                double a = fabs(p.va[k]);
                if (a > rmax[ri[k]]) rmax[ri[k]] = a;
                if (a > cmax[j]) cmax[j] = a;
            }
        for (int i = 0; i < m; ++i) { double f = rmax[i] > 1e-8 ? 1.0 / sqrt(rmax[i]) : 1.0; R[i] *= f; b[i] *= f; rmax[i] = f; }
        for (int j = 0; j < n; ++j) { double f = cmax[j] > 1e-8 ? 1.0 / sqrt(cmax[j]) : 1.0; C[j] *= f; c[j] *= f; cmax[j] = f; }
        for (int j = 0; j < n; ++j)
            for (int k = cp[j]; k < cp[j + 1]; ++k) p.va[k] *= rmax[ri[k]] * cmax[j];
    }
    for (int d = 0; d < nz; ++d) p.rv[d] = p.va[csr_of[d]];
    free(rmax); free(cmax); free(csr_of);

    ipm_ws w;
    double** vecs_n[] = {&w.rd, &w.theta, &w.rxs, &w.v, &w.dx, &w.ds, &w.dx_aff, &w.ds_aff,
                         &w.tx, &w.ts, &w.bx, &w.bs, &w.brd, &w.t2, &w.t3};
    double** vecs_m[] = {&w.rp, &w.rkkt, &w.dy, &w.dy_aff, &w.by, &w.brp, &w.t1, &w.rk_p, &w.dy_p};
    for (size_t q = 0; q < sizeof(vecs_n) / sizeof(vecs_n[0]); ++q) *vecs_n[q] = (double*)calloc((size_t)n + 1, sizeof(double));
    for (size_t q = 0; q < sizeof(vecs_m) / sizeof(vecs_m[0]); ++q) *vecs_m[q] = (double*)calloc((size_t)m + 1, sizeof(double));
    double* x = (double*)malloc(sizeof(double) * ((size_t)n + 1));
    double* s = (double*)malloc(sizeof(double) * ((size_t)n + 1));
    double* y = (double*)calloc((size_t)m + 1, sizeof(double));
    for (int j = 0; j < n; ++j) { x[j] = 1.0; s[j] = 1.0; }
    kkt_ctx k;
    kkt_init(&k, m);
    if (opts.start == 1) {
        /* Mehrotra's start (Mehrotra 1992): x~ = A^T (A A^T)^{-1} b, y = (A A^T)^{-1} A c,
         * s~ = c - A^T y, shifted to positivity and then balanced by x^T s. */
        for (int j = 0; j < n; ++j) w.theta[j] = 1.0;
        form_normal_matrix(m, p.rp, p.ci, p.rv, w.theta, k.M0);
        int dummy = 0;
        normal_solve(&p, &k, w.theta, b, 1e-12 * (1.0 + norm_inf(m, b)), w.dy, &dummy);
        spmv_At(&p, w.dy, x);
        spmv_A(&p, c, w.rkkt);
        normal_solve(&p, &k, w.theta, w.rkkt, 1e-12 * (1.0 + norm_inf(m, w.rkkt)), y, &dummy);
        spmv_At(&p, y, s);
        for (int j = 0; j < n; ++j) s[j] = c[j] - s[j];
        double mx = 1e300, ms = 1e300;
        for (int j = 0; j < n; ++j) { if (x[j] < mx) mx = x[j]; if (s[j] < ms) ms = s[j]; }
        const double dx = fmax(-1.5 * mx, 0.0), dsv = fmax(-1.5 * ms, 0.0);
        double xs = 0.0, sx = 0.0, ss = 0.0;
        for (int j = 0; j < n; ++j) { x[j] += dx; s[j] += dsv; xs += x[j] * s[j]; sx += x[j]; ss += s[j]; }
        const double hx = 0.5 * xs / ss, hs = 0.5 * xs / sx;
        for (int j = 0; j < n; ++j) { x[j] += hx; s[j] += hs; if (!(x[j] > 0.0)) x[j] = 1.0; if (!(s[j] > 0.0)) s[j] = 1.0; }
    }

    oracle_ipm_result r;
    memset(&r, 0, sizeof(r));
    r.status = 0;
    double rp0 = 1.0, rd0 = 1.0, mu0 = 1.0;
    double unscale_b = 1.0 + norm_inf(m, b0), unscale_c = 1.0 + norm_inf(n, c0);
    int iter;
    int done = 0, loose_count = 0;
    for (iter = 0; iter < opts.max_iter && !done; ++iter) {
        residuals(&p, b, c, x, y, s, w.rp, w.rd);
        double nrp = norm2(m, w.rp), nrd = norm2(n, w.rd), mu = dot(n, x, s) / n;
        if (iter == 0) { rp0 = fmax(1.0, nrp); rd0 = fmax(1.0, nrd); mu0 = fmax(1.0, mu); }
        int converged;
        double pinf = 0.0, dinf = 0.0, cx = 0.0, by = 0.0;
        if (opts.criteria == 1) {
            converged = nrp < 1e-6 && nrd < 1e-6 && mu < 1e-6;
        } else {
            for (int i = 0; i < m; ++i) { double a = fabs(w.rp[i] / R[i]); if (a > pinf) pinf = a; }
            for (int j = 0; j < n; ++j) { double a = fabs(w.rd[j] / C[j]); if (a > dinf) dinf = a; }
            cx = dot(n, c, x);
            by = dot(m, b, y);
            double gap = fabs(cx - by) / (1.0 + fabs(cx) + fabs(by));
            /* the gap is also held to tol (1 + |c^T x|): with the optimum between the primal
             * and dual objectives, c^T x is then within tol of it in relative terms */
            const int loose = pinf / unscale_b <= opts.tol && dinf / unscale_c <= opts.tol && gap <= opts.tol;
            converged = loose && fabs(cx - by) <= opts.tol * (1.0 + fabs(cx));
            /* the three relative tests met for 3 iterations without the gap closing: accepted */
            loose_count = loose && !converged ? loose_count + 1 : 0;
            if (loose_count >= 3) converged = 1;
        }
        if (opts.verbose)
            fprintf(stderr, "oracle iter %d rp %.3e rd %.3e mu %.3e\n", iter, nrp, nrd, mu);
        if (converged) { r.status = 0; done = 1; break; }

        for (int j = 0; j < n; ++j) w.theta[j] = x[j] / s[j];
        {   /* M0 = A Theta A^T for this iteration (dense) */
            form_normal_matrix(m, p.rp, p.ci, p.rv, w.theta, k.M0);
        }
        double tol = 1e-9 * fmax(1.0, nrp);
        /* predictor */
        for (int j = 0; j < n; ++j) { w.rxs[j] = -x[j] * s[j]; w.v[j] = -w.theta[j] * w.rd[j] - w.rxs[j] / s[j]; }
        spmv_A(&p, w.v, w.rkkt);
        for (int i = 0; i < m; ++i) w.rkkt[i] -= w.rp[i];
        const double vlim = opts.strict ? 1e-8 : 1e-4;
        if (!normal_solve(&p, &k, w.theta, w.rkkt, tol, w.dy_aff, &r.solves) && opts.strict) { r.status = 3; break; }
        spmv_At(&p, w.dy_aff, w.ds_aff);
        for (int j = 0; j < n; ++j) { w.ds_aff[j] = -w.rd[j] - w.ds_aff[j]; w.dx_aff[j] = -w.theta[j] * w.ds_aff[j] + w.rxs[j] / s[j]; }
        if (!verify_direction(&p, &w, x, s, w.dx_aff, w.dy_aff, w.ds_aff, w.rxs, nrp, nrd, vlim)) { r.status = 3; break; }
        double ap_aff = fmin(1.0, step_length(n, x, w.dx_aff));
        double ad_aff = fmin(1.0, step_length(n, s, w.ds_aff));
        for (int j = 0; j < n; ++j) { w.tx[j] = x[j] + ap_aff * w.dx_aff[j]; w.ts[j] = s[j] + ad_aff * w.ds_aff[j]; }
        double mu_aff = dot(n, w.tx, w.ts) / n;
        double sigma = fmin(1.0, pow(fmax(0.0, mu_aff) / fmax(1e-16, mu), 3.0));
        /* corrector */
        for (int j = 0; j < n; ++j) {
            w.rxs[j] = -x[j] * s[j] + sigma * mu - w.dx_aff[j] * w.ds_aff[j];
            w.v[j] = -w.theta[j] * w.rd[j] - w.rxs[j] / s[j];
        }
        spmv_A(&p, w.v, w.rkkt);
        for (int i = 0; i < m; ++i) w.rkkt[i] -= w.rp[i];
        if (!normal_solve(&p, &k, w.theta, w.rkkt, tol, w.dy, &r.solves) && opts.strict) { r.status = 3; break; }
        spmv_At(&p, w.dy, w.ds);
        for (int j = 0; j < n; ++j) { w.ds[j] = -w.rd[j] - w.ds[j]; w.dx[j] = -w.theta[j] * w.ds[j] + w.rxs[j] / s[j]; }
        int corrector_valid = verify_direction(&p, &w, x, s, w.dx, w.dy, w.ds, w.rxs, nrp, nrd, vlim);
        const double eta = 0.995, armijo = 1e-4;
        double cap = fmin(1.0, eta * step_length(n, x, w.dx));
        double cad = fmin(1.0, eta * step_length(n, s, w.ds));
        double orig_merit = nrp / rp0 + nrd / rd0 + mu / mu0;
        /* near-optimal (robust mode, relative criteria): primal and dual infeasibility within
         * 0.1 tol; a trial that stays so and whose distance to the stopping test falls by the
         * Armijo factor is accepted even when the merit rises (an inexact direction can add
         * infeasibility far below the tolerance while it closes the gap) */
        const int near = !opts.strict && opts.criteria != 1 && pinf / unscale_b <= 0.1 * opts.tol &&
                         dinf / unscale_c <= 0.1 * opts.tol;
        const double dist0 = fmax(fmax(pinf / unscale_b, dinf / unscale_c), fabs(cx - by) / (1.0 + fabs(cx)));
        int accepted = 0;
        for (int dir = corrector_valid ? 0 : 1; dir < 2 && !accepted; ++dir) {
            if (dir == 1) {
                for (int j = 0; j < n; ++j) {
                    w.rxs[j] = -x[j] * s[j] + 0.5 * mu;
                    w.v[j] = -w.theta[j] * w.rd[j] - w.rxs[j] / s[j];
                }
                spmv_A(&p, w.v, w.rkkt);
                for (int i = 0; i < m; ++i) w.rkkt[i] -= w.rp[i];
                if (!normal_solve(&p, &k, w.theta, w.rkkt, tol, w.dy, &r.solves) && opts.strict) break;
                spmv_At(&p, w.dy, w.ds);
                for (int j = 0; j < n; ++j) { w.ds[j] = -w.rd[j] - w.ds[j]; w.dx[j] = -w.theta[j] * w.ds[j] + w.rxs[j] / s[j]; }
                if (!verify_direction(&p, &w, x, s, w.dx, w.dy, w.ds, w.rxs, nrp, nrd, vlim)) break;
                double bnd = fmin(step_length(n, x, w.dx), step_length(n, s, w.ds));
                cap = cad = fmin(1.0, eta * bnd);
            }
            int maxbt = dir == 0 ? 15 : 30;
            for (int bt = 0; bt < maxbt; ++bt) {
                for (int j = 0; j < n; ++j) { w.bx[j] = x[j] + cap * w.dx[j]; w.bs[j] = s[j] + cad * w.ds[j]; }
                for (int i = 0; i < m; ++i) w.by[i] = y[i] + cad * w.dy[i];
                residuals(&p, b, c, w.bx, w.by, w.bs, w.brp, w.brd);
                double nrp2 = norm2(m, w.brp), nrd2 = norm2(n, w.brd), mu2 = dot(n, w.bx, w.bs) / n;
                double minx = 1e30, mins = 1e30;
                for (int j = 0; j < n; ++j) { if (w.bx[j] < minx) minx = w.bx[j]; if (w.bs[j] < mins) mins = w.bs[j]; }
                double merit = nrp2 / rp0 + nrd2 / rd0 + mu2 / mu0;
                double step = fmin(cap, cad);
                int finite = isfinite(nrp2) && isfinite(nrd2) && isfinite(mu2) && isfinite(merit) &&
                             isfinite(orig_merit) && isfinite(minx) && isfinite(mins) && isfinite(cap) &&
                             isfinite(cad) && isfinite(norm2(m, w.by));
                int positive = minx > 0.0 && mins > 0.0 && mu2 > 0.0 && step > 0.0;
                int progress = merit < orig_merit && merit <= (1.0 - armijo * step) * orig_merit;
                if (!progress && near && finite && positive) {
                    double tp = 0.0, td = 0.0;
                    for (int i = 0; i < m; ++i) { double a = fabs(w.brp[i] / R[i]); if (a > tp) tp = a; }
                    for (int j = 0; j < n; ++j) { double a = fabs(w.brd[j] / C[j]); if (a > td) td = a; }
                    tp /= unscale_b;
                    td /= unscale_c;
                    const double tcx = dot(n, c, w.bx), tby = dot(m, b, w.by);
                    const double tdist = fmax(fmax(tp, td), fabs(tcx - tby) / (1.0 + fabs(tcx)));
                    progress = tp <= 0.1 * opts.tol && td <= 0.1 * opts.tol && isfinite(tdist) &&
                               tdist <= (1.0 - armijo * step) * dist0;
                }
                if (finite && positive && progress) { accepted = 1; break; }
                cap *= 0.5;
                cad *= 0.5;
            }
        }
        if (!accepted) { r.status = 3; break; }
        memcpy(x, w.bx, sizeof(double) * (size_t)n);
        memcpy(y, w.by, sizeof(double) * (size_t)m);
        memcpy(s, w.bs, sizeof(double) * (size_t)n);
    }
    if (!done && r.status == 0) { r.status = 3; iter = opts.max_iter; }
    r.iterations = iter;
    residuals(&p, b, c, x, y, s, w.rp, w.rd);
    r.primal_residual = norm2(m, w.rp);
    r.dual_residual = norm2(n, w.rd);
    r.duality_gap = dot(n, x, s) / n;
    r.objective = dot(n, c, x);
    for (int j = 0; j < n; ++j) { x_out[j] = x[j] * C[j]; if (s_out) s_out[j] = s[j] / C[j]; }
    for (int i = 0; i < m; ++i) y_out[i] = y[i] * R[i];
    {
        double meas[6];
        double* sv = (double*)malloc(sizeof(double) * ((size_t)n + 1));
        for (int j = 0; j < n; ++j) sv[j] = s[j] / C[j];
        oracle_kkt_measures(m, n, cp, ri, va0, b0, c0, x_out, y_out, sv, meas);
        r.rel_pinf = meas[0]; r.rel_dinf = meas[1]; r.rel_gap = meas[2];
        free(sv);
    }
    if (res) *res = r;
    for (size_t q = 0; q < sizeof(vecs_n) / sizeof(vecs_n[0]); ++q) free(*vecs_n[q]);
    for (size_t q = 0; q < sizeof(vecs_m) / sizeof(vecs_m[0]); ++q) free(*vecs_m[q]);
    free(x); free(s); free(y); free(R); free(C); free(b); free(c);
    free(p.va); free(p.rp); free(p.ci); free(p.rv);
    kkt_free(&k);
    return 0;
}
