/*
 * CPU oracle for the device Mehrotra IPM path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithm, used by tests/, by the
 * smoke check and by the benchmark's CPU-baseline leg as the checker. The
 * product library never links, loads or calls anything in this directory.
 *
 * Pinned against the reference: tests/test_oracle_pins.py checks these
 * functions against the golden vectors of the reference's own tests
 * (tests/unit/test_ipm_symbolic.cpp:46,66-77,109,133-150,
 *  tests/unit/test_gpu_kkt.cu:35-46,104-121,168-194,
 *  tests/unit/test_mehrotra.cu:29-67) and against the reference's own CPU code
 * compiled from its sources into oracle/_ref (symbolic analysis and the CPU
 * simplex objective) by oracle/Makefile.
 *
 * All matrices are CSR or CSC with int32 indices and FP64 values.
 */
#ifndef SK_ORACLE_H
#define SK_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Exact minimum-degree ordering on the graph of A A^T with explicit fill cliques
 * and lowest-index tie-break; P[k] = original row eliminated k-th.
 * Restates src/ipm/symbolic.cpp:11-98. Returns 0 on success. */
int oracle_min_degree(int m, int n, const int* row_ptrs, const int* col_idx, int* P);

/* Elimination tree and strictly-lower L pattern (CSR, row-major, columns
 * increasing) of P (A A^T) P^T. Restates src/ipm/symbolic.cpp:100-218.
 * L_row_ptrs has m+1 entries; L_cols must hold L_cap entries.
 * Returns nnz(L) (>= 0), or -1 if L_cap is too small. */
int oracle_symbolic(int m, int n, const int* row_ptrs, const int* col_idx, const int* P,
                    int* P_inv, int* parent, int* L_row_ptrs, int* L_cols, int L_cap);

/* Normal-equation solve M0 dy = rhs with M0 = A diag(theta) A^T (A in CSR,
 * rows permuted by P for the factorisation; P may be NULL for identity).
 * Restates src/cuda/kkt.cu:620-870: diagonal equilibration D = 1/sqrt(max(|m_ii|,1e-12)),
 * factor of D M0 D + delta I with delta = 1e-9 raised x10 up to 5 times on a
 * non-positive pivot, up to 10 steps of FP64 iterative refinement against M0 with
 * rollback on stagnation. Success when ||rhs - M0 dy||_inf <= tol * max(1, rel ? ||rhs||_inf : 1).
 * dy receives the solution (also on failure). Returns 1 on success, 0 on failure. */
int oracle_kkt_solve(int m, int n, const int* row_ptrs, const int* col_idx, const double* vals,
                     const double* theta, const int* P, const double* rhs, double tol, int rel,
                     double* dy);

typedef struct oracle_ipm_opts {
    int criteria;      /* 0: relative 1e-8-style on unscaled data (tol); 1: reference absolute 1e-6 scaled 2-norms */
    double tol;        /* tolerance of criteria 0 */
    int max_iter;      /* reference: 200 */
    int verbose;
    int start;         /* 0: x = s = 1, y = 0 (reference :93-102); 1: Mehrotra's heuristic start */
    int strict;        /* 1: a missed solve tolerance or direction check ends the solve with
                        * IterationLimit (reference :793-797, :814-822); 0: the direction is
                        * used when finite with e1, e2, e3 <= 1e-4 (the stopping test and the
                        * merit line search still decide progress) */
} oracle_ipm_opts;

typedef struct oracle_ipm_result {
    int status;        /* 0 Optimal, 3 IterationLimit (reference SimplexStatus numbering) */
    int iterations;
    double objective;  /* c^T x, unscaled */
    double primal_residual, dual_residual, duality_gap; /* reference quantities: scaled ||rp||_2, ||rd||_2, mu */
    double rel_pinf, rel_dinf, rel_gap;                 /* unscaled relative criteria */
    int solves;        /* number of normal-equation solves */
} oracle_ipm_result;

/* Mehrotra predictor-corrector IPM on min c^T x, Ax = b, x >= 0 (A in CSC, rows
 * sorted within columns). Restates src/ipm/mehrotra_device.cu:276-330 (10-pass
 * inline Ruiz), :695-1047 (x = s = 1, y = 0 start; sigma = (mu_aff/mu)^3; eta = 0.995;
 * Newton-direction verification at 1e-8; Armijo 1e-4 merit backtracking with up
 * to 15 halvings, then a centred direction sigma_c = 1/2 with a common step and up
 * to 30 halvings) using a dense FP64 Cholesky (sizes up to a few thousand rows).
 * x (n), y (m), s (n) receive the unscaled solution. Returns 0 on success. */
int oracle_ipm_solve(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                     const double* b, const double* c, const oracle_ipm_opts* opts,
                     double* x, double* y, double* s, oracle_ipm_result* res);

/* Unscaled relative optimality measures of (x, y, s):
 * rel_pinf = ||Ax-b||_inf/(1+||b||_inf), rel_dinf = ||A^T y + s - c||_inf/(1+||c||_inf),
 * rel_gap = |c^T x - b^T y| / (1 + |c^T x| + |b^T y|). out[0..2] = these, out[3] = c^T x,
 * out[4] = min(x), out[5] = min(s). */
void oracle_kkt_measures(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                         const double* b, const double* c, const double* x, const double* y,
                         const double* s, double* out);

/* A generated LP in standard form (CSC with rows increasing in each column). */
typedef struct oracle_lp {
    int m, n, nnz;
    int* col_ptrs;     /* n + 1 */
    int* row_idx;      /* nnz */
    double* vals;      /* nnz */
    double* b;         /* m */
    double* c;         /* n */
} oracle_lp;

/* Seeded LP families of the benchmark (lpgen_oracle.c): the same arrays as the
 * product's generator for the same seed, built without it, so that the CPU
 * baselines load nothing of the product. Return 0 on success; release with
 * oracle_lp_free. family: 0, 1 or 3. */
int oracle_lp_family(int family, int instance, oracle_lp* lp);
int oracle_lp_random(int m, int n, double density, unsigned long long seed, oracle_lp* lp);
int oracle_lp_block_angular(unsigned long long seed, int blocks, int block_rows, int block_cols, int link_rows,
                            int nnz_per_block_col, oracle_lp* lp);
void oracle_lp_free(oracle_lp* lp);
/* Rows, columns and density of family-3 member `instance` without building it. */
int oracle_lp_family3_shape(int instance, int* m, int* n, double* density);

#ifdef __cplusplus
}
#endif
#endif
