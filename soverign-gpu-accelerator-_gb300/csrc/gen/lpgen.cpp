#include "gen/lpgen.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace sankhya {
namespace gen {

static uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }

Rng::Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto& w : s_) w = splitmix64(x);
}

uint64_t Rng::next() {
    const uint64_t result = rotl(s_[1] * 5, 7) * 9;
    const uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return result;
}

double Rng::uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
double Rng::uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }

uint64_t Rng::below(uint64_t bound) {
    // Lemire-free rejection: unbiased and portable.
    const uint64_t limit = UINT64_MAX - (UINT64_MAX % bound);
    uint64_t r;
    do { r = next(); } while (r >= limit);
    return r % bound;
}

double Rng::normal() {
    if (have_spare_) { have_spare_ = false; return spare_; }
    double u1;
    do { u1 = uniform(); } while (u1 <= 0.0);
    const double u2 = uniform();
    const double r = std::sqrt(-2.0 * std::log(u1));
    const double a = 6.283185307179586 * u2;
    spare_ = r * std::sin(a);
    have_spare_ = true;
    return r * std::cos(a);
}

static double signed_value(Rng& g) {
    const double v = g.uniform(0.1, 10.0);
    return (g.next() >> 63) ? -v : v;
}

// Builds CSC from per-column (row, value) lists, sorting rows within each column.
static void pack_columns(GeneratedLP& lp, std::vector<std::vector<std::pair<Index, Float>>>& colv) {
    lp.col_ptrs.assign(static_cast<size_t>(lp.n) + 1, 0);
    size_t nz = 0;
    for (auto& cv : colv) nz += cv.size();
    lp.row_idx.clear();
    lp.vals.clear();
    lp.row_idx.reserve(nz);
    lp.vals.reserve(nz);
    for (Index j = 0; j < lp.n; ++j) {
        auto& cv = colv[static_cast<size_t>(j)];
        std::sort(cv.begin(), cv.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        for (auto& e : cv) { lp.row_idx.push_back(e.first); lp.vals.push_back(e.second); }
        lp.col_ptrs[static_cast<size_t>(j) + 1] = static_cast<Index>(lp.row_idx.size());
    }
}

// b = A x0 with x0 ~ U[0.5,2]; c = A^T y0 + s0 with y0 ~ N(0,1), s0 ~ U[0.1,1].
static void interior_rhs_and_cost(GeneratedLP& lp, Rng& g) {
    std::vector<double> x0(static_cast<size_t>(lp.n)), y0(static_cast<size_t>(lp.m)), s0(static_cast<size_t>(lp.n));
    for (auto& v : x0) v = g.uniform(0.5, 2.0);
    for (auto& v : y0) v = g.normal();
    for (auto& v : s0) v = g.uniform(0.1, 1.0);
    lp.b.assign(static_cast<size_t>(lp.m), 0.0);
    lp.c.assign(static_cast<size_t>(lp.n), 0.0);
    for (Index j = 0; j < lp.n; ++j) {
        double acc = 0.0;
        for (Index k = lp.col_ptrs[j]; k < lp.col_ptrs[j + 1]; ++k) {
            lp.b[static_cast<size_t>(lp.row_idx[k])] += lp.vals[k] * x0[static_cast<size_t>(j)];
            acc += lp.vals[k] * y0[static_cast<size_t>(lp.row_idx[k])];
        }
        lp.c[static_cast<size_t>(j)] = acc + s0[static_cast<size_t>(j)];
    }
}

// k distinct rows out of [0, m) by Floyd's sampling.
static void distinct_rows(Rng& g, Index m, Index k, std::vector<Index>& out) {
    out.clear();
    for (Index j = m - k; j < m; ++j) {
        const Index t = static_cast<Index>(g.below(static_cast<uint64_t>(j) + 1));
        if (std::find(out.begin(), out.end(), t) == out.end()) out.push_back(t);
        else out.push_back(j);
    }
}

GeneratedLP random_sparse_lp(Index m, Index n, double density, uint64_t seed) {
    if (m < 2 || n < 2) throw std::invalid_argument("random_sparse_lp: m, n must be >= 2");
    Rng g(seed);
    GeneratedLP lp;
    lp.m = m;
    lp.n = n;
    const Index k = std::min<Index>(m, std::max<Index>(2, static_cast<Index>(std::lround(density * m))));
    std::vector<std::vector<std::pair<Index, Float>>> colv(static_cast<size_t>(n));
    std::vector<Index> rows;
    std::vector<Index> row_count(static_cast<size_t>(m), 0);
    for (Index j = 0; j < n; ++j) {
        distinct_rows(g, m, k, rows);
        for (Index r : rows) {
            colv[static_cast<size_t>(j)].push_back({r, signed_value(g)});
            row_count[static_cast<size_t>(r)]++;
        }
    }
    // Every row gets at least one entry: an empty row receives one entry in a
    // uniformly drawn column that does not hold it yet.
    for (Index r = 0; r < m; ++r) {
        if (row_count[static_cast<size_t>(r)] > 0) continue;
        const Index j = static_cast<Index>(g.below(static_cast<uint64_t>(n)));
        colv[static_cast<size_t>(j)].push_back({r, signed_value(g)});
        row_count[static_cast<size_t>(r)]++;
    }
    pack_columns(lp, colv);
    interior_rhs_and_cost(lp, g);
    return lp;
}

GeneratedLP block_angular_lp(uint64_t seed, Index blocks, Index block_rows, Index block_cols,
                             Index link_rows, Index nnz_per_block_col) {
    Rng g(seed);
    GeneratedLP lp;
    lp.m = blocks * block_rows + link_rows;
    lp.n = blocks * block_cols;
    std::vector<std::vector<std::pair<Index, Float>>> colv(static_cast<size_t>(lp.n));
    std::vector<Index> rows;
    std::vector<Index> row_count(static_cast<size_t>(lp.m), 0);
    for (Index bk = 0; bk < blocks; ++bk) {
        for (Index jj = 0; jj < block_cols; ++jj) {
            const Index j = bk * block_cols + jj;
            distinct_rows(g, block_rows, nnz_per_block_col, rows);
            for (Index r : rows) {
                colv[static_cast<size_t>(j)].push_back({bk * block_rows + r, signed_value(g)});
                row_count[static_cast<size_t>(bk * block_rows + r)]++;
            }
            if (link_rows > 0) {
                const Index lr = blocks * block_rows + static_cast<Index>(g.below(static_cast<uint64_t>(link_rows)));
                colv[static_cast<size_t>(j)].push_back({lr, signed_value(g)});
                row_count[static_cast<size_t>(lr)]++;
            }
        }
    }
    for (Index r = 0; r < lp.m; ++r) {
        if (row_count[static_cast<size_t>(r)] > 0) continue;
        Index j;
        if (r < blocks * block_rows) {
            const Index bk = r / block_rows;
            j = bk * block_cols + static_cast<Index>(g.below(static_cast<uint64_t>(block_cols)));
            bool present = false;
            for (auto& e : colv[static_cast<size_t>(j)]) present |= (e.first == r);
            if (present) continue;
        } else {
            j = static_cast<Index>(g.below(static_cast<uint64_t>(lp.n)));
        }
        colv[static_cast<size_t>(j)].push_back({r, signed_value(g)});
        row_count[static_cast<size_t>(r)]++;
    }
    pack_columns(lp, colv);
    interior_rhs_and_cost(lp, g);
    return lp;
}

GeneratedLP staircase_transport_lp(uint64_t seed, Index stages, Index kSupply, Index kDemand, Index kCap,
                                   Index kArcs) {
    if (stages <= 0 || kSupply <= 0 || kDemand <= 0 || kCap <= 1 || kArcs < std::max(kSupply, kDemand))
        throw std::invalid_argument("staircase_transport_lp: bad shape");
    const Index kRowsPerStage = kSupply + kDemand + kCap;
    const Index kColsPerStage = kArcs + kCap;
    Rng g(seed);
    GeneratedLP lp;
    lp.m = stages * kRowsPerStage;
    lp.n = stages * kColsPerStage;
    std::vector<std::vector<std::pair<Index, Float>>> colv(static_cast<size_t>(lp.n));
    std::vector<double> flow(static_cast<size_t>(lp.n), 0.0);
    std::vector<double> rowsum(static_cast<size_t>(lp.m), 0.0);
    lp.c.assign(static_cast<size_t>(lp.n), 0.0);
    std::vector<Index> perm_s(kSupply), perm_d(kDemand);
    for (Index t = 0; t < stages; ++t) {
        const Index r0 = t * kRowsPerStage;
        const Index cap0 = r0 + kSupply + kDemand;
        const Index next_cap0 = (t + 1 < stages) ? (t + 1) * kRowsPerStage + kSupply + kDemand : cap0;
        std::iota(perm_s.begin(), perm_s.end(), 0);
        std::iota(perm_d.begin(), perm_d.end(), 0);
        for (Index i = kSupply - 1; i > 0; --i) std::swap(perm_s[i], perm_s[g.below(static_cast<uint64_t>(i) + 1)]);
        for (Index i = kDemand - 1; i > 0; --i) std::swap(perm_d[i], perm_d[g.below(static_cast<uint64_t>(i) + 1)]);
        for (Index a = 0; a < kArcs; ++a) {
            const Index j = t * kColsPerStage + a;
            // The first kSupply arcs cover every supply and demand node once.
            const Index s = a < kSupply ? perm_s[a] : static_cast<Index>(g.below(kSupply));
            const Index d = a < kDemand ? perm_d[a] : static_cast<Index>(g.below(kDemand));
            const Index cr = static_cast<Index>(g.below(kCap));
            Index nr = static_cast<Index>(g.below(kCap));
            if (next_cap0 == cap0 && nr == cr) nr = (nr + 1) % kCap;
            auto& cv = colv[static_cast<size_t>(j)];
            cv.push_back({r0 + s, 1.0});
            cv.push_back({r0 + kSupply + d, 1.0});
            cv.push_back({cap0 + cr, g.uniform(0.5, 2.0)});
            cv.push_back({next_cap0 + nr, g.uniform(0.5, 2.0)});
            flow[static_cast<size_t>(j)] = static_cast<double>(1 + g.below(90));
            lp.c[static_cast<size_t>(j)] = g.uniform(1.0, 100.0);
        }
        for (Index r = 0; r < kCap; ++r) {
            const Index j = t * kColsPerStage + kArcs + r;
            colv[static_cast<size_t>(j)].push_back({cap0 + r, 1.0});
            flow[static_cast<size_t>(j)] = g.uniform(1.0, 10.0);
        }
    }
    pack_columns(lp, colv);
    for (Index j = 0; j < lp.n; ++j)
        for (Index k = lp.col_ptrs[j]; k < lp.col_ptrs[j + 1]; ++k)
            rowsum[static_cast<size_t>(lp.row_idx[k])] += lp.vals[k] * flow[static_cast<size_t>(j)];
    lp.b.assign(rowsum.begin(), rowsum.end());
    return lp;
}

GeneratedLP family_lp(int family, int instance) {
    switch (family) {
    case 0:
        return random_sparse_lp(500, 1000, 0.01, 0xC0ull + static_cast<uint64_t>(instance));
    case 1:
        return block_angular_lp(0xC1ull + static_cast<uint64_t>(instance));
    case 2:
        return staircase_transport_lp(0xC2ull + static_cast<uint64_t>(instance));
    case 3: {
        const uint64_t seed = 0xC3ull * 1000000ull + static_cast<uint64_t>(instance);
        Rng g(seed ^ 0x5DEECE66Dull);
        const double lm = g.uniform(std::log(200.0), std::log(5000.0));
        const Index m = std::max<Index>(200, std::min<Index>(5000, static_cast<Index>(std::floor(std::exp(lm)))));
        const Index n = static_cast<Index>(std::ceil(m * g.uniform(2.0, 3.0)));
        const double density = g.uniform(0.005, 0.02);
        return random_sparse_lp(m, n, density, seed);
    }
    default:
        throw std::invalid_argument("family_lp: family must be 0..3");
    }
}

}  // namespace gen
}  // namespace sankhya
