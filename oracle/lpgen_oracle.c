/*
 * Seeded LP families restated in plain C -- TEST INFRASTRUCTURE ONLY.
 *
 * The benchmark's reference arm and the CPU baseline time the CPU restatement of
 * the reference's algorithm on the same LPs the device path solves, without
 * loading the product library. These functions rebuild those LPs from their
 * seeds: the same xoshiro256** stream (seeded through splitmix64), the same draw
 * order and the same arithmetic as the product's generator, so the arrays are
 * identical (tests/test_oracle_lpgen.py compares them element for element).
 *
 *   family 0: random sparse LP, m=500, n=1000, 1 % density, seed 0xC0 + instance
 *   family 1: block-angular LP, 40 blocks of 500x1200 + 2000 linking rows, 5 + 1
 *             nonzeros per column, seed 0xC1 + instance
 *   family 3: member `instance` of the 512-LP uneven batch: m ~ logUniform[200, 5000],
 *             n = ceil(m U[2, 3]), density U[0.5 %, 2 %], seed 0xC3 * 10^6 + instance
 *
 * b = A x0 with x0 ~ U[0.5, 2]; c = A^T y0 + s0 with y0 ~ N(0, 1), s0 ~ U[0.1, 1].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sk_oracle.h"

typedef struct {
    uint64_t s[4];
    int have_spare;
    double spare;
} rng_t;

static uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t rotl64(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }

static void rng_init(rng_t* g, uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) g->s[i] = splitmix64(&x);
    g->have_spare = 0;
    g->spare = 0.0;
}

static uint64_t rng_next(rng_t* g) {
    uint64_t* s = g->s;
    const uint64_t r = rotl64(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return r;
}

static double rng_unit(rng_t* g) { return (double)(rng_next(g) >> 11) * (1.0 / 9007199254740992.0); }
static double rng_range(rng_t* g, double lo, double hi) { return lo + (hi - lo) * rng_unit(g); }

static uint64_t rng_below(rng_t* g, uint64_t bound) {
    const uint64_t limit = UINT64_MAX - (UINT64_MAX % bound);
    uint64_t r;
    do { r = rng_next(g); } while (r >= limit);
    return r % bound;
}

static double rng_normal(rng_t* g) {
    if (g->have_spare) { g->have_spare = 0; return g->spare; }
    double u1;
    do { u1 = rng_unit(g); } while (u1 <= 0.0);
    const double u2 = rng_unit(g);
    const double r = sqrt(-2.0 * log(u1));
    const double a = 6.283185307179586 * u2;
    g->spare = r * sin(a);
    g->have_spare = 1;
    return r * cos(a);
}

static double signed_value(rng_t* g) {
    const double v = rng_range(g, 0.1, 10.0);
    return (rng_next(g) >> 63) ? -v : v;
}

/* Column lists: entries of column j are (row, value) pairs appended in draw order. */
typedef struct { int row; double val; } entry_t;
typedef struct { entry_t* e; int len, cap; } column_t;

static int col_push(column_t* c, int row, double val) {
    if (c->len == c->cap) {
        int nc = c->cap ? 2 * c->cap : 8;
        entry_t* ne = (entry_t*)realloc(c->e, (size_t)nc * sizeof(entry_t));
        if (!ne) return -1;
        c->e = ne;
        c->cap = nc;
    }
    c->e[c->len].row = row;
    c->e[c->len].val = val;
    c->len++;
    return 0;
}

static int by_row(const void* a, const void* b) {
    const int ra = ((const entry_t*)a)->row, rb = ((const entry_t*)b)->row;
    return (ra > rb) - (ra < rb);
}

static void free_columns(column_t* cols, int n) {
    for (int j = 0; j < n; ++j) free(cols[j].e);
    free(cols);
}

/* Rows within a column are distinct, so sorting by row alone fixes the order. */
static int pack(oracle_lp* lp, column_t* cols) {
    size_t nz = 0;
    for (int j = 0; j < lp->n; ++j) nz += (size_t)cols[j].len;
    lp->col_ptrs = (int*)malloc(((size_t)lp->n + 1) * sizeof(int));
    lp->row_idx = (int*)malloc((nz ? nz : 1) * sizeof(int));
    lp->vals = (double*)malloc((nz ? nz : 1) * sizeof(double));
    if (!lp->col_ptrs || !lp->row_idx || !lp->vals) return -1;
    size_t k = 0;
    lp->col_ptrs[0] = 0;
    for (int j = 0; j < lp->n; ++j) {
        qsort(cols[j].e, (size_t)cols[j].len, sizeof(entry_t), by_row);
        for (int q = 0; q < cols[j].len; ++q, ++k) {
            lp->row_idx[k] = cols[j].e[q].row;
            lp->vals[k] = cols[j].e[q].val;
        }
        lp->col_ptrs[j + 1] = (int)k;
    }
    lp->nnz = (int)nz;
    return 0;
}

static int interior_rhs_and_cost(oracle_lp* lp, rng_t* g) {
    const int m = lp->m, n = lp->n;
    double* x0 = (double*)malloc((size_t)n * sizeof(double));
    double* y0 = (double*)malloc((size_t)m * sizeof(double));
    double* s0 = (double*)malloc((size_t)n * sizeof(double));
    lp->b = (double*)calloc((size_t)m, sizeof(double));
    lp->c = (double*)calloc((size_t)n, sizeof(double));
    if (!x0 || !y0 || !s0 || !lp->b || !lp->c) { free(x0); free(y0); free(s0); return -1; }
    for (int j = 0; j < n; ++j) x0[j] = rng_range(g, 0.5, 2.0);
    for (int i = 0; i < m; ++i) y0[i] = rng_normal(g);
    for (int j = 0; j < n; ++j) s0[j] = rng_range(g, 0.1, 1.0);
    for (int j = 0; j < n; ++j) {
        double acc = 0.0;
        for (int k = lp->col_ptrs[j]; k < lp->col_ptrs[j + 1]; ++k) {
            double t = lp->vals[k] * x0[j];
            lp->b[lp->row_idx[k]] += t;
            double u = lp->vals[k] * y0[lp->row_idx[k]];
            acc += u;
        }
        lp->c[j] = acc + s0[j];
    }
    free(x0); free(y0); free(s0);
    return 0;
}

/* k distinct rows out of [0, m) by Floyd's sampling, in draw order. */
static void distinct_rows(rng_t* g, int m, int k, int* out, int* len) {
    *len = 0;
    for (int j = m - k; j < m; ++j) {
        const int t = (int)rng_below(g, (uint64_t)j + 1);
        int seen = 0;
        for (int q = 0; q < *len; ++q) seen |= (out[q] == t);
        out[(*len)++] = seen ? j : t;
    }
}

static int random_sparse(oracle_lp* lp, int m, int n, double density, uint64_t seed) {
    if (m < 2 || n < 2) return -1;
    rng_t g;
    rng_init(&g, seed);
    lp->m = m;
    lp->n = n;
    long kk = lround(density * m);
    if (kk < 2) kk = 2;
    const int k = (int)(kk < m ? kk : m);
    column_t* cols = (column_t*)calloc((size_t)n, sizeof(column_t));
    int* rows = (int*)malloc((size_t)k * sizeof(int));
    int* count = (int*)calloc((size_t)m, sizeof(int));
    int rc = (!cols || !rows || !count) ? -1 : 0;
    for (int j = 0; j < n && rc == 0; ++j) {
        int len;
        distinct_rows(&g, m, k, rows, &len);
        for (int q = 0; q < len && rc == 0; ++q) {
            const double v = signed_value(&g);
            rc = col_push(&cols[j], rows[q], v);
            count[rows[q]]++;
        }
    }
    for (int r = 0; r < m && rc == 0; ++r) {
        if (count[r] > 0) continue;
        const int j = (int)rng_below(&g, (uint64_t)n);
        const double v = signed_value(&g);
        rc = col_push(&cols[j], r, v);
        count[r]++;
    }
    if (rc == 0) rc = pack(lp, cols);
    if (rc == 0) rc = interior_rhs_and_cost(lp, &g);
    if (cols) free_columns(cols, n);
    free(rows);
    free(count);
    return rc;
}

static int block_angular(oracle_lp* lp, uint64_t seed, int blocks, int brows, int bcols, int lrows, int per_col) {
    rng_t g;
    rng_init(&g, seed);
    lp->m = blocks * brows + lrows;
    lp->n = blocks * bcols;
    column_t* cols = (column_t*)calloc((size_t)lp->n, sizeof(column_t));
    int* rows = (int*)malloc((size_t)per_col * sizeof(int));
    int* count = (int*)calloc((size_t)lp->m, sizeof(int));
    int rc = (!cols || !rows || !count) ? -1 : 0;
    for (int bk = 0; bk < blocks && rc == 0; ++bk) {
        for (int jj = 0; jj < bcols && rc == 0; ++jj) {
            const int j = bk * bcols + jj;
            int len;
            distinct_rows(&g, brows, per_col, rows, &len);
            for (int q = 0; q < len && rc == 0; ++q) {
                const double v = signed_value(&g);
                rc = col_push(&cols[j], bk * brows + rows[q], v);
                count[bk * brows + rows[q]]++;
            }
            if (lrows > 0 && rc == 0) {
                const int lr = blocks * brows + (int)rng_below(&g, (uint64_t)lrows);
                const double v = signed_value(&g);
                rc = col_push(&cols[j], lr, v);
                count[lr]++;
            }
        }
    }
    for (int r = 0; r < lp->m && rc == 0; ++r) {
        if (count[r] > 0) continue;
        int j;
        if (r < blocks * brows) {
            const int bk = r / brows;
            j = bk * bcols + (int)rng_below(&g, (uint64_t)bcols);
            int present = 0;
            for (int q = 0; q < cols[j].len; ++q) present |= (cols[j].e[q].row == r);
            if (present) continue;
        } else {
            j = (int)rng_below(&g, (uint64_t)lp->n);
        }
        const double v = signed_value(&g);
        rc = col_push(&cols[j], r, v);
        count[r]++;
    }
    if (rc == 0) rc = pack(lp, cols);
    if (rc == 0) rc = interior_rhs_and_cost(lp, &g);
    if (cols) free_columns(cols, lp->n);
    free(rows);
    free(count);
    return rc;
}

void oracle_lp_free(oracle_lp* lp) {
    if (!lp) return;
    free(lp->col_ptrs);
    free(lp->row_idx);
    free(lp->vals);
    free(lp->b);
    free(lp->c);
    memset(lp, 0, sizeof(*lp));
}

int oracle_lp_random(int m, int n, double density, unsigned long long seed, oracle_lp* lp) {
    memset(lp, 0, sizeof(*lp));
    int rc = random_sparse(lp, m, n, density, (uint64_t)seed);
    if (rc != 0) oracle_lp_free(lp);
    return rc;
}

int oracle_lp_block_angular(unsigned long long seed, int blocks, int block_rows, int block_cols, int link_rows,
                            int nnz_per_block_col, oracle_lp* lp) {
    memset(lp, 0, sizeof(*lp));
    if (blocks <= 0 || block_rows <= 0 || block_cols <= 0 || link_rows < 0 || nnz_per_block_col <= 0 ||
        nnz_per_block_col > block_rows)
        return -1;
    int rc = block_angular(lp, (uint64_t)seed, blocks, block_rows, block_cols, link_rows, nnz_per_block_col);
    if (rc != 0) oracle_lp_free(lp);
    return rc;
}

/* Shape of family-3 member `instance`: its own stream, drawn before the LP's. */
static uint64_t family3_shape(int instance, int* m_out, int* n_out, double* density_out) {
    const uint64_t seed = 0xC3ull * 1000000ull + (uint64_t)instance;
    rng_t g;
    rng_init(&g, seed ^ 0x5DEECE66Dull);
    const double lm = rng_range(&g, log(200.0), log(5000.0));
    int m = (int)floor(exp(lm));
    if (m > 5000) m = 5000;
    if (m < 200) m = 200;
    *m_out = m;
    *n_out = (int)ceil(m * rng_range(&g, 2.0, 3.0));
    *density_out = rng_range(&g, 0.005, 0.02);
    return seed;
}

int oracle_lp_family3_shape(int instance, int* m, int* n, double* density) {
    family3_shape(instance, m, n, density);
    return 0;
}

int oracle_lp_family(int family, int instance, oracle_lp* lp) {
    memset(lp, 0, sizeof(*lp));
    int rc = -1;
    if (family == 0) {
        rc = random_sparse(lp, 500, 1000, 0.01, 0xC0ull + (uint64_t)instance);
    } else if (family == 1) {
        rc = block_angular(lp, 0xC1ull + (uint64_t)instance, 40, 500, 1200, 2000, 5);
    } else if (family == 3) {
        int m, n;
        double density;
        const uint64_t seed = family3_shape(instance, &m, &n, &density);
        rc = random_sparse(lp, m, n, density, seed);
    }
    if (rc != 0) oracle_lp_free(lp);
    return rc;
}
