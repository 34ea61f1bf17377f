/*
 * sk_ipm.h -- C ABI of the GB300 device Mehrotra interior-point LP engine.
 *
 * Plain pointers and sizes only (int32 indices, FP64 values). No exception
 * crosses this boundary: every function returns an SK_* status code. Each entry
 * point names the reference interface it replaces (paths inside the reference
 * project). Device pointers are marked d_*; everything else is host memory.
 */
#ifndef SK_IPM_H
#define SK_IPM_H

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (0 = ok). */
#define SK_OK 0
#define SK_ERR_INVALID 1       /* bad argument / inconsistent sizes */
#define SK_ERR_CUDA 2          /* CUDA runtime error (std::runtime_error in the reference, src/ipm/mehrotra_device.cu:26-43) */
#define SK_ERR_NUMERICAL 3     /* factorisation failed for every regularisation (src/cuda/kkt.cu:600-602, 862-864) */
#define SK_ERR_NO_DEVICE 4     /* no CUDA device visible */
#define SK_ERR_ALLOC 5         /* device allocation failed (std::bad_alloc in src/gpu/vram_arena.cu:58-60) */
#define SK_ERR_INTERNAL 6
#define SK_ERR_TOO_LARGE 7     /* request exceeds a stated maximum size */
#define SK_ERR_RANK_DEFICIENT 8 /* crossover: an artificial column stays in the basis ("Crossover failed:
                                   Matrix is rank deficient", src/ipm/crossover.cu:455-457) */

/* Solver status, numbered as the reference's simplex::SimplexStatus (src/simplex/primal.hpp:26-31). */
#define SK_STATUS_OPTIMAL 0
#define SK_STATUS_INFEASIBLE 1
#define SK_STATUS_UNBOUNDED 2
#define SK_STATUS_ITERATION_LIMIT 3

/* Precision of the normal-equation factorisation. */
#define SK_PREC_FP64 0         /* plain FP64 factor (reference arithmetic) */
#define SK_PREC_MIXED 1        /* FP32 factor + FP64 residuals / refinement, FP64 switch near convergence */

/* Starting point. */
#define SK_START_UNIT 0        /* x = s = 1, y = 0 (src/ipm/mehrotra_device.cu:93-102) */
#define SK_START_MEHROTRA 1    /* Mehrotra's standard heuristic start */
#define SK_START_USER 2        /* x, y, s given in sk_solver_set_start (scaled space of the caller's LP) */
#define SK_START_LEARNED 3     /* bipartite network's prediction (sk_solver_set_gnn); per LP, Mehrotra's start
                                  when the prediction is not at least twice as close to the stopping test */

/* Stopping rule. */
#define SK_CRIT_RELATIVE 0     /* rel_pinf, rel_dinf, rel_gap <= tol and |c^T x - b^T y| <= tol (1 + |c^T x|), unscaled;
                                  the first three alone for 3 iterations in a row also stop */
#define SK_CRIT_REFERENCE 1    /* ||rp||_2, ||rd||_2, mu < 1e-6 on the scaled LP (src/ipm/mehrotra_device.cu:746-748) */

/* Fill-reducing ordering of A A^T. */
#define SK_ORDER_AUTO 0        /* one dense front when A A^T is dense; else approximate minimum degree; for
                                  LPs of >= 50000 rows the given row order or nested dissection, whichever
                                  needs fewer factorisation flops */
#define SK_ORDER_REFERENCE 1   /* exact minimum degree, lowest index wins ties (src/ipm/symbolic.cpp:11-98) */
#define SK_ORDER_NATURAL 2
#define SK_ORDER_MINDEG 3      /* approximate minimum degree */
#define SK_ORDER_DISSECTION 4  /* nested dissection (level-structure separators, minimum vertex covers) */

typedef struct sk_options {
    int precision;        /* SK_PREC_* (default SK_PREC_MIXED) */
    int start;            /* SK_START_* (default SK_START_UNIT) */
    int criteria;         /* SK_CRIT_* (default SK_CRIT_RELATIVE) */
    double tol;           /* default 1e-8 */
    int max_iter;         /* default 200 (src/ipm/mehrotra_device.cu:703) */
    int ordering;         /* SK_ORDER_* (default SK_ORDER_AUTO) */
    int verbose;          /* 0 = silent; >0 prints per-iteration lines on stderr */
    double mu_switch;     /* mixed precision: switch the factor to FP64 once mu < mu_switch (default 1e-4) */
    int ruiz_passes;      /* default 10 (src/ipm/mehrotra_device.cu:293) */
    int strict;           /* 1: a normal-equation solve that misses 1e-9 max(1, ||rp||_2) or a direction
                           * with e1, e2 or e3 > 1e-8 ends the LP with IterationLimit, as the reference
                           * does (src/ipm/mehrotra_device.cu:793-797, 814-822). 0 (default): such a
                           * miss first switches a mixed-precision solve to the FP64 factor; an FP64
                           * direction is then used when it is finite with e1, e2, e3 <= 1e-4, and the
                           * merit line search plus the exact stopping test decide progress. */
    double delta32;       /* first regularisation of FP32 fronts (default 1e-8); x10 per failed attempt */
    double delta64;       /* first regularisation of FP64 fronts (default 1e-14; strict mode uses 1e-9) */
    double learned_accept;/* SK_START_LEARNED: the network's start is used for an LP when its distance to
                           * the stopping test is below learned_accept x that of Mehrotra's start
                           * (default 0.5); otherwise that LP starts from Mehrotra's start */
    int fp64_update;      /* trailing updates of FP64 fronts: SK_FP64_UPDATE_AUTO (default: FP64-accurate
                           * products on the tensor cores in SK_PREC_MIXED, the FP64 pipe in SK_PREC_FP64),
                           * SK_FP64_UPDATE_NATIVE (FP64 pipe) or SK_FP64_UPDATE_TENSOR (tensor cores:
                           * BF16 digits of the FP64 panel, exact FP32 sums, results within about
                           * 2^-53 of sum |a||b|) */
    int dependent_rows;   /* 0 (default, as the reference): every row of A is kept (a rank-deficient A is
                           * absorbed by the delta regularisation); 1: rows of A that are linearly
                           * dependent on the others are found (sk_presolve_dependent_rows) and, when b
                           * is consistent, dropped before the solve; their y is returned as 0 and
                           * sk_info.rel_pinf includes their residuals at x */
} sk_options;
#define SK_FP64_UPDATE_AUTO 0
#define SK_FP64_UPDATE_NATIVE 1
#define SK_FP64_UPDATE_TENSOR 2

typedef struct sk_info {
    int status;               /* SK_STATUS_* */
    int iterations;
    double objective;         /* c^T x, unscaled */
    double primal_residual;   /* reference quantities: scaled ||Ax-b||_2 */
    double dual_residual;     /* scaled ||A^T y + s - c||_2 */
    double duality_gap;       /* scaled mu = x^T s / n */
    double rel_pinf, rel_dinf, rel_gap;  /* unscaled relative measures */
    int precision_path;       /* 0 FP64 throughout, 1 FP32 throughout, 2 FP32 then FP64 */
    int switch_iteration;     /* first FP64 iteration in mixed mode, -1 if none */
    int factorizations;
    int solves;
    int refine_steps;
    int learned_start;        /* 1 if a user / learned start was accepted */
    double setup_ms;          /* host analysis + upload */
    double solve_ms;          /* IPM iterations */
    long long nnz_factor;     /* stored factor entries */
    int num_supernodes;
    int dense_front;          /* 1 if A A^T was treated as one dense front */
    double device_ms;         /* last sk_solver_run measured with CUDA events on the solver stream */
    double flops_factor;      /* algorithmic flops of one factorisation: sum_j c_j^2 over factor columns */
    double start_merit;       /* max(rel pinf, rel dinf, rel gap) at the start point used */
    double fallback_merit;    /* the same for Mehrotra's start (SK_START_LEARNED runs), else 0 */
    int dependent_rows;       /* rows dropped as linearly dependent (sk_options.dependent_rows), else 0 */
    double factor_ms_fp32;    /* device time of the last run's factorisations with FP32 fronts (batch-wide) */
    double factor_ms_fp64;    /* the same with FP64 fronts */
} sk_info;

/* Fills the defaults listed above. */
void sk_options_default(sk_options* opt);

/* One-shot solve of min c^T x, Ax = b, x >= 0 from host CSC arrays (rows sorted or
 * not, no duplicates). x (n), y (m), s (n) receive the unscaled primal / dual /
 * reduced-cost solution; any may be NULL. info may be NULL.
 * Replaces: sankhya::ipm::MehrotraSolver(const core::Model&) + solve()
 *           (src/ipm/mehrotra.hpp:21-31, src/ipm/mehrotra_device.cu:1049-1059). */
int sk_ipm_solve_csc(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                     const double* b, const double* c, const sk_options* opt,
                     double* x, double* y, double* s, sk_info* info);

/* As sk_ipm_solve_csc for min c^T x, A x = b, lb <= x <= ub (lb / ub may be NULL:
 * 0 / +infinity; +-HUGE_VAL = unbounded). The LP is brought to standard form on the
 * host (shifts, reflections, free-variable splits, one extra row per finite upper
 * bound), solved on the device and mapped back: x (n) in the original variables, y
 * (m) for the original rows, s = c - A^T y; info->objective is c^T x, the relative
 * measures refer to the standard-form LP. No reference counterpart: the reference's
 * device IPM ignores lb / ub (parsers::read_mps sets them, mps_reader.cpp:259-298). */
int sk_ipm_solve_bounded(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                         const double* b, const double* c, const double* lb, const double* ub,
                         const sk_options* opt, double* x, double* y, double* s, sk_info* info);

/* Persistent solver over a batch of independent LPs (num_lps >= 1), all resident in
 * device memory after creation. The batch is solved as one block-diagonal problem
 * with per-LP step lengths, merit and convergence.
 * Replaces: MehrotraSolver::Impl::Impl (src/ipm/mehrotra_device.cu:276-465) for
 *           each LP; the reference has no batch entry point. */
typedef struct sk_solver sk_solver;
int sk_solver_create(int num_lps, const int* m, const int* n, const int* const* col_ptrs,
                     const int* const* row_idx, const double* const* vals, const double* const* b,
                     const double* const* c, const sk_options* opt, sk_solver** out);
/* Optional starting point for LP `lp` (unscaled x, y, s); used when opt.start == SK_START_USER. */
int sk_solver_set_start(sk_solver* h, int lp, const double* x, const double* y, const double* s);
/* Runs the IPM from the start point on the resident data (Impl::solve, :695-1047). */
int sk_solver_run(sk_solver* h);
int sk_solver_result(sk_solver* h, int lp, double* x, double* y, double* s, sk_info* info);
void sk_solver_destroy(sk_solver* h);
/* Kernel-class breakdown of one factorisation + one solve at the current iterate,
 * replayed without graphs with CUDA events around every launch (diagnostics;
 * not part of a solve). out[2*c] = total ms, out[2*c+1] = launches, for classes
 * c = 0 assembly, 1 potrf, 2 trsm, 3 update, 4 extend-add, 5 forward solve,
 * 6 backward solve; out[14] = algorithmic flops of the update launches, out[15] =
 * bytes the update launches must move at least (each input tile read once, each
 * output tile read and written once); with cap >= 17, out[16] = algorithmic bytes
 * of the assembly launches (A or the Khatri-Rao map read once, Theta read once,
 * each normal-matrix entry written once, the diagonal and D written once); with
 * cap >= 18, out[17] = flops the tensor cores execute in the update launches (per
 * 128 x 64 block of the lower part with K padded to 64: three TF32 products for FP32
 * fronts, 28 BF16 digit-pair products for FP64 fronts on the tensor cores; 0 for
 * SIMT updates). fp32: 0 = FP64 fronts, 1 = FP32 fronts with tensor-core (tcgen05)
 * updates, 2 = FP32 fronts with SIMT updates. Returns the number of values written
 * (16, 17 or 18).
 * No reference counterpart. */
int sk_solver_profile(sk_solver* h, int fp32, double* out, int cap);

/* ---- Learned start: bipartite row / column message-passing network ----
 * No reference counterpart. 3 layers, hidden width 64, BF16 weights with FP32
 * accumulation, FP32 master weights for Adam. Input: a Ruiz-scaled LP (column
 * features c_j, log(1 + nnz_j), ||A_.j||_2; row features b_i, log(1 + nnz_i),
 * ||A_i.||_2; edge weights a_ij). Output: log x_j, log s_j per column and y_i per
 * row, in the scaled space. Loss: (1 / 2n) sum_j [(log x_j - t_j)^2 + (log s_j -
 * u_j)^2] + (1 / m) sum_i (y_i - w_i)^2, log targets clamped to [-30, 30]. */
typedef struct sk_gnn sk_gnn;
typedef struct sk_gnn_batch sk_gnn_batch;
int sk_gnn_create(unsigned long long seed, sk_gnn** out);   /* Glorot-uniform weights, biases 0 (0.01 in the input layers) */
void sk_gnn_destroy(sk_gnn* g);
int sk_gnn_num_params(const sk_gnn* g);
int sk_gnn_get_params(const sk_gnn* g, float* out);         /* FP32 master weights */
int sk_gnn_set_params(sk_gnn* g, const float* in);          /* also refreshes the BF16 copy */
/* One graph from host CSR arrays (m x n, already scaled as the caller wants it
 * seen); targets t_logx, t_logs (n) and t_y (m) may be NULL (inference only). */
int sk_gnn_batch_create(int m, int n, const int* row_ptrs, const int* col_idx, const double* vals,
                        const double* b, const double* c, const double* t_logx, const double* t_logs,
                        const double* t_y, sk_gnn_batch** out);
/* Device copy of a solver's scaled batch LP and of the iterate captured during its
 * last run (sk_solver_set_capture); SK_ERR_INVALID if some LP was not captured. */
int sk_gnn_batch_from_solver(sk_solver* h, sk_gnn_batch** out);
int sk_gnn_batch_dims(const sk_gnn_batch* bt, int* m, int* n);
/* Host copies of the batch's targets (log x, log s: n; y: m); any may be NULL. */
int sk_gnn_batch_targets(const sk_gnn_batch* bt, double* logx, double* logs, double* y);
void sk_gnn_batch_destroy(sk_gnn_batch* bt);
/* Host outputs: logx, logs (n), y (m); any may be NULL. */
int sk_gnn_predict(sk_gnn* g, sk_gnn_batch* bt, double* logx, double* logs, double* y);
/* Loss on the batch's targets and its gradient w.r.t. every parameter (grad: num_params floats). */
int sk_gnn_loss_grad(sk_gnn* g, sk_gnn_batch* bt, double* loss, float* grad);
/* Forward + backward + one Adam step (beta1 0.9, beta2 0.999, eps 1e-8, gradient
 * entries clipped to [-10, 10]) at learning rate lr; loss before the step. */
int sk_gnn_train_step(sk_gnn* g, sk_gnn_batch* bt, float lr, double* loss);
/* Network for SK_START_LEARNED (not owned: keep it alive while the solver runs). */
int sk_solver_set_gnn(sk_solver* h, sk_gnn* g);
/* Keep each LP's iterate the first time its mu drops below mu_threshold (or the
 * final iterate), as training targets; 0 turns capture off. */
int sk_solver_set_capture(sk_solver* h, double mu_threshold);

/* ---- KKT normal-equation engine (device pointers) ----
 * Replaces: gpu::GPUKKTCholeskySolver (src/cuda/kkt.cuh:28-71). A is CSR (m x n).
 * P: elimination order (P[k] = original row), NULL = choose per opt.ordering. */
typedef struct sk_kkt sk_kkt;
int sk_kkt_create(int m, int n, const int* row_ptrs, const int* col_idx, const double* vals,
                  const int* P, int precision, sk_kkt** out);                /* kkt.cuh:38-43 */
int sk_kkt_factorize_device(sk_kkt* k, const double* d_theta);              /* kkt.cuh:67 */
/* Solves M0 dy = rhs in place (M0 = A diag(theta) A^T); returns SK_OK when
 * ||rhs - M0 dy||_inf <= tol * max(1, ||rhs||_inf), SK_ERR_NUMERICAL otherwise. */
int sk_kkt_solve_device(sk_kkt* k, double* d_rhs, double tol);              /* kkt.cuh:68 */
int sk_kkt_factorize(sk_kkt* k, const double* theta);                       /* kkt.cuh:53 */
int sk_kkt_solve(sk_kkt* k, double* rhs, double tol);                        /* kkt.cuh:61 */
/* Copies the factor of D (P M0 P^T) D + delta I as a dense lower-triangular m x m
 * row-major matrix in the elimination order, plus D (m), for inspection. */
int sk_kkt_get_factor(sk_kkt* k, double* L_dense, double* D);
/* Trailing updates of the FP64 factorisation (sk_kkt_create with SK_PREC_FP64):
 * SK_FP64_UPDATE_NATIVE / _AUTO (FP64 pipe, default) or SK_FP64_UPDATE_TENSOR
 * (FP64-accurate products on the tensor cores). No counterpart in the reference
 * (its factorisation is scalar FP64). Applies from the next factorisation. */
int sk_kkt_set_fp64_update(sk_kkt* k, int mode);
void sk_kkt_destroy(sk_kkt* k);

/* ---- Symbolic analysis (host) ----
 * Replaces: ipm::compute_amd_ordering (src/ipm/symbolic.hpp:50) -- exact minimum
 * degree with lowest-index tie-break, bit-exact with the reference. */
int sk_compute_amd_ordering(int m, int n, const int* row_ptrs, const int* col_idx, int* P);
/* Replaces: ipm::compute_symbolic_factorization (src/ipm/symbolic.hpp:59-63):
 * P_inv, elimination tree parent (-1 = root) and strictly lower L pattern in CSR
 * (L_row_ptrs: m+1, L_cols: capacity cap). Returns nnz(L) >= 0, -1 if cap is too small. */
int sk_compute_symbolic(int m, int n, const int* row_ptrs, const int* col_idx, const int* P,
                        int* P_inv, int* parent, int* L_row_ptrs, int* L_cols, int cap);
/* Fill-reducing approximate minimum degree order of A A^T used by the solver (no
 * reference counterpart beyond compute_amd_ordering's role). */
int sk_fill_ordering(int m, int n, const int* row_ptrs, const int* col_idx, int* P);
/* Nested dissection order of A A^T (SK_ORDER_DISSECTION; no reference counterpart):
 * separators from breadth-first level structures narrowed to minimum vertex covers,
 * each ordered after the two parts it splits. */
int sk_dissection_ordering(int m, int n, const int* row_ptrs, const int* col_idx, int* P);

/* Host-only analysis of one LP's normal matrix (no device needed): builds the
 * multifrontal plan the solver would use and writes out[0..15] =
 * {supernodes, levels, tile steps, extend-add rounds, stored factor entries,
 *  factorisation flops (sum c_j^2), front storage entries, largest front rows,
 *  supernodes with <= 64 columns, assembly slots, Khatri-Rao map entries,
 *  dense front (0/1), ordering used, consistency check (1 = every normal-matrix
 *  entry maps into its front and every front lists its own columns first),
 *  solve launches per triangular solve, factor launches per factorisation}.
 * Returns 16. No reference counterpart. */
int sk_plan_stats(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, int ordering,
                  double* out, int cap);

/* ---- Crossover (basis purification) ----
 * Replaces: ipm::generate_crossover_basis (src/ipm/crossover.cuh:30-33, crossover.cu:322-460),
 * same decisions. From a point x (n) with A x = b and lb <= x <= ub (lb / ub NULL: 0 / +inf),
 * strictly interior columns are pivoted into the basis or moved to a bound, then the
 * remaining artificial rows are filled. Outputs: basic (m) = the column of each basis
 * row (>= n: artificial), status (n) = SK_BASIS_* per column, x_out (n, may be NULL) =
 * x after the moves. Returns SK_OK; SK_ERR_NUMERICAL when a column has no admissible
 * move ("Crossover failed: Invalid pivot encountered"); SK_ERR_RANK_DEFICIENT; and
 * SK_ERR_TOO_LARGE for m > SK_CROSSOVER_MAX_ROWS (the basis inverse is a dense m x m
 * FP64 matrix on the device). Outputs are filled in every case but SK_ERR_TOO_LARGE. */
#define SK_CROSSOVER_MAX_ROWS 32768
#define SK_BASIS_BASIC 0
#define SK_BASIS_AT_LOWER 1
#define SK_BASIS_AT_UPPER 2
int sk_crossover(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, const double* lb,
                 const double* ub, const double* x, int* basic, int* status, double* x_out);

/* ---- Allocation-free small KKT solve ----
 * No counterpart in the reference. Solves (A diag(theta) A^T) dy = rhs in place
 * (FP64, same regularisation ladder, refinement and return contract as
 * sk_kkt_factorize_device + sk_kkt_solve_device) for a device CSR matrix A
 * (m x n, column indices sorted within each row) without allocating: it is for
 * callers that cannot call cudaMalloc / cudaFree where they need the solve
 * (all device memory handed to their own pool, or no device-wide
 * synchronisation allowed). All work lives in one fixed device array of
 * 542,976 bytes, which limits m to SK_KKT_NOALLOC_MAX_ROWS; a larger m returns
 * SK_ERR_TOO_LARGE. The first call on each device fetches that array's address
 * and loads the kernel (set-up; loading the module may allocate driver memory),
 * so make it before any stream capture. Every call on a device uses
 * the same array: calls that overlap in time (two host threads, or two streams
 * without ordering between them) race and corrupt each other's results. The
 * call synchronises `stream` (NULL = legacy default stream) before it returns.
 * d_row_ptrs[m] must equal the length of d_col_idx and d_vals: the kernel reads
 * up to that entry and cannot check it against the arrays' sizes. Malformed
 * row pointers, unsorted or out-of-range columns, a negative or non-finite theta
 * and non-finite values of A or rhs return SK_ERR_INVALID with d_rhs untouched;
 * a solve that misses tol (for example a row of A without entries) returns
 * SK_ERR_NUMERICAL with d_rhs holding the last iterate. */
#define SK_KKT_NOALLOC_MAX_ROWS 256
int sk_kkt_solve_noalloc(int m, int n, const int* d_row_ptrs, const int* d_col_idx, const double* d_vals,
                         const double* d_theta, double* d_rhs, double tol, void* stream);

/* ---- Convex QP on the device ----
 * Replaces: qp::QPSolver::solve_with_diagnostics (src/qp/qp_solver.hpp:47-66,
 * src/qp/qp_solver.cpp:151-560; C++ interface kept in include/qp/qp_solver.hpp).
 * min 1/2 x^T H x + c^T x subject to A x = b and lb <= x <= ub. A is m x n in CSC
 * (m may be 0); H is n x n given by its lower triangle (diagonal included) in CSC;
 * lb / ub may be NULL (0 and +inf); a bound beyond 1e15 in magnitude is absent.
 * convexity: SK_QP_CONVEX_PSD solves; SK_QP_CONVEXITY_UNKNOWN and SK_QP_NONCONVEX
 * give status UnsupportedNonconvex, as the reference does. opts may be NULL
 * (sk_qp_options_default: 1e-6, 1e-6, 1e-6, 200). The reference's iteration runs
 * on the GPU with W = H + D diagonal (a non-diagonal H is lifted through a
 * pivoted Cholesky H = F^T F into free variables w = F x; dense, n <= 4096).
 * *status receives the QPSolverStatus (SK_QP_OPTIMAL ...); x (n), y (m) and
 * z = zl - zu (n) are written when it is Optimal or IterationLimit; info (may be
 * NULL) receives {objective, iterations, primal_residual, dual_residual,
 * complementarity}. Returns SK_OK, SK_ERR_INVALID (bad pointers or entries, an
 * entry of H above the diagonal), SK_ERR_NO_DEVICE or SK_ERR_CUDA. */
#define SK_QP_CONVEXITY_UNKNOWN 0
#define SK_QP_CONVEX_PSD 1
#define SK_QP_NONCONVEX 2
#define SK_QP_OPTIMAL 0
#define SK_QP_INFEASIBLE 1
#define SK_QP_UNBOUNDED 2
#define SK_QP_ITERATION_LIMIT 3
#define SK_QP_NUMERICAL_FAILURE 4
#define SK_QP_UNSUPPORTED_NONCONVEX 5
#define SK_QP_INVALID_MODEL 6
typedef struct sk_qp_options {
    double feasibility_tol;   /* ||A x - b||_inf below this */
    double dual_tol;          /* ||H x + c - A^T y - zl + zu||_inf below this */
    double grad_tol;          /* complementarity mu below this */
    int max_iterations;
} sk_qp_options;
void sk_qp_options_default(sk_qp_options* opts);
int sk_qp_solve(int m, int n, const int* a_col_ptrs, const int* a_row_idx, const double* a_vals, const double* b,
                const double* c, const double* lb, const double* ub, const int* h_col_ptrs, const int* h_row_idx,
                const double* h_vals, int convexity, const sk_qp_options* opts, double* x, double* y, double* z,
                int* status, double* info);

/* ---- Presolve: linearly dependent rows of A (device) ----
 * No counterpart in the reference (its presolve is the Ruiz scaling below; its IPM
 * absorbs a rank-deficient A through the delta regularisation). A (m x n, CSC) and b.
 * A A^T is factored in FP64 on the device (equilibrated to a unit diagonal, delta from
 * 1e-12) in a fill-reducing order; a row whose pivot L_kk^2 (its squared distance from
 * the span of the rows eliminated before it, rows normalised) is at most 1e-6 counts as
 * linearly dependent on them (FP64 rounding through the normal equations leaves about
 * 1e-9 on an exact dependency). b is consistent when the residual of
 * A A^T w = b, iteratively refined on that factor, vanishes: *inconsistency (may be NULL)
 * receives ||b - A A^T w||_inf / (1 + ||b||_inf). keep (m) receives 0 for the dependent
 * rows when the inconsistency is at most 1e-9 (their equations then follow from the
 * kept rows) and 1 for every row otherwise; *num_dependent receives the number of
 * dependent rows found. Returns SK_OK, SK_ERR_INVALID, SK_ERR_NO_DEVICE,
 * SK_ERR_NUMERICAL or SK_ERR_CUDA. */
int sk_presolve_dependent_rows(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals,
                               const double* b, int* keep, int* num_dependent, double* inconsistency);

/* ---- Presolve: Ruiz equilibration of a model (host) ----
 * Replaces: presolve::apply_ruiz_scaling(core::Model&, int max_iterations)
 * (src/presolve/scaling.hpp:25, src/presolve/scaling.cpp:18-146), with the
 * same arithmetic (bit-identical results). Up to max_iterations passes (the
 * reference's default is 10) scale A's rows, then its columns, by
 * 1/sqrt(largest |entry|), stopping once all those maxima were within 1e-4 of 1;
 * columns with integer_cols[j] != 0 are never scaled (integer_cols may be NULL:
 * all continuous). vals (CSC, in place) is scaled; row_scale (m) and col_scale
 * (n) hold the model's scale vectors on entry (ones for a model not scaled
 * before) and the accumulated ones on return; then b <- row_scale .* b,
 * c <- col_scale .* c, finite lb / ub <- bound ./ col_scale (b, c, lb, ub may be
 * NULL). Host only: needs no device. */
int sk_presolve_ruiz(int m, int n, const int* col_ptrs, const int* row_idx, double* vals, double* b, double* c,
                     double* lb, double* ub, const unsigned char* integer_cols, int max_iterations,
                     double* row_scale, double* col_scale);

/* ---- Device kernels exposed for parity tests (device pointers, stream may be NULL) ---- */
/* y = alpha * A x + beta * y for CSR A (rows x ?). Replaces cusparseSpMV CSR FP64
 * (src/ipm/mehrotra_device.cu:512,603,635,936). */
int sk_spmv_csr(int rows, const int* d_row_ptrs, const int* d_col_idx, const double* d_vals,
                const double* d_x, double alpha, double beta, double* d_y, void* stream);

/* ---- Autotuned SpMV plans ----
 * Replaces the reference's descriptor-based cuSPARSE SpMV (cusparseCreateCsr at
 * src/ipm/mehrotra_device.cu:424-428, cusparseSpMV_bufferSize + cusparseSpMV at
 * :508-530 and :596-624) for one CSR matrix kept on the device by the caller
 * (rows x cols, nnz entries, int32 indices, FP64 values; the arrays must outlive
 * the plan). sk_spmv_plan_create cuts the rows into chunks whose columns fit a
 * shared-memory window of x (up to 24576 columns), then times the project's two
 * vector CSR kernels (x gathered from global memory, or staged per chunk in
 * shared memory) for 2, 4, 8, 16 and 32 lanes per row on this matrix and keeps
 * the fastest. It allocates and frees its own x / y scratch, keeps the chunk
 * table in device memory until sk_spmv_plan_destroy, and synchronises `stream`.
 * The choice is remembered for the process under (device, rows, cols, nnz), so
 * later plans and solvers on the same shape reuse it without timing.
 * sk_spmv_plan_execute computes y = alpha A x + beta y asynchronously on `stream`
 * (NULL = legacy default stream). sk_spmv_plan_info reports the width in use,
 * whether shared-memory windows are in use, the row-length rule's width, and
 * the fastest timed launch of each width in milliseconds for the plain and the
 * windowed kernel (5 entries each in the order 2, 4, 8, 16, 32; zero when not
 * timed or when the choice came from an earlier plan); any output may be NULL. */
typedef struct sk_spmv_plan sk_spmv_plan;
int sk_spmv_plan_create(int rows, int cols, long long nnz, const int* d_row_ptrs, const int* d_col_idx,
                        const double* d_vals, void* stream, sk_spmv_plan** out);
int sk_spmv_plan_execute(const sk_spmv_plan* plan, const double* d_x, double alpha, double beta, double* d_y,
                         void* stream);
int sk_spmv_plan_info(const sk_spmv_plan* plan, int* group, int* windowed, int* heuristic_group,
                      double* ms_per_group, double* ms_windowed_per_group);
/* Overrides the plan's choice: `group` lanes per row (2, 4, 8, 16 or 32) and
 * windowed 0 (global gathers) or 1 (shared-memory windows); other values give
 * SK_ERR_INVALID. Every choice computes the same products; only the order of
 * the additions within a row depends on `group` (windowed or not gives the same
 * bits for the same group). */
int sk_spmv_plan_set_group(sk_spmv_plan* plan, int group, int windowed);
void sk_spmv_plan_destroy(sk_spmv_plan* plan);

/* ---- Model input ----
 * Replaces: parsers::read_mps (src/parsers/mps_reader.hpp:20) and the seeded
 * generators (no reference counterpart). An sk_lp owns CSC arrays + b + c. */
typedef struct sk_lp sk_lp;
int sk_lp_read_mps(const char* path, sk_lp** out);
int sk_lp_generate(int family, int instance, sk_lp** out);
int sk_lp_random(int m, int n, double density, unsigned long long seed, sk_lp** out);
/* Block-angular member of family 1 with a chosen shape (family 1 itself is
 * blocks=40, block_rows=500, block_cols=1200, link_rows=2000, nnz_per_col=5). */
int sk_lp_block_angular(unsigned long long seed, int blocks, int block_rows, int block_cols, int link_rows,
                        int nnz_per_col, sk_lp** out);
/* Staircase transportation member of family 2 with a chosen shape (family 2 itself is
 * stages=50, supply=demand=1000, cap=2000, arcs=8000: m = stages (supply + demand + cap),
 * n = stages (arcs + cap)). */
int sk_lp_staircase(unsigned long long seed, int stages, int supply, int demand, int cap, int arcs, sk_lp** out);
int sk_lp_dims(const sk_lp* lp, int* m, int* n, int* nnz);
/* Pointers into the LP's own storage (valid until sk_lp_free). lb / ub may be NULL. */
int sk_lp_arrays(const sk_lp* lp, const int** col_ptrs, const int** row_idx, const double** vals,
                 const double** b, const double** c);
int sk_lp_bounds(const sk_lp* lp, const double** lb, const double** ub);
/* Host standard form of min c^T x, A x = b, lb <= x <= ub (see sk_ipm_solve_bounded):
 * a new sk_lp with x' >= 0 and c^T x = c'^T x' + *obj_offset. Original column j is
 * standard-form column j (negated when only ub is finite); free columns add one
 * column each (after the n originals), finite upper bounds one row (after the m
 * originals) and one slack column (last). */
int sk_lp_standard_form(int m, int n, const int* col_ptrs, const int* row_idx, const double* vals, const double* b,
                        const double* c, const double* lb, const double* ub, sk_lp** out, double* obj_offset);
void sk_lp_free(sk_lp* lp);

/* Last error message of the calling thread ("" if none). */
const char* sk_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
