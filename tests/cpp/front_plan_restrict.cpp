// Host check of ipm::restrict_steps, the step lists with which a factorisation of
// some LPs of a batch launches only their fronts' blocks. Builds the front plan of
// two batches of seeded random LPs (one in dense-front mode, one in sparse
// multifrontal mode), restricts it with several LP masks and checks, step by step,
// that the kept items are the plan's items of the LPs that are on (in order), that
// every prefix array holds the kept items' own counts summed from 0, that the totals
// match and that steps without items are dropped. Prints one JSON line; exit code 0
// when every check holds.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "core/problem.hpp"
#include "ipm/front_plan.hpp"

using namespace sankhya;

namespace {

struct Lcg {
    uint64_t s;
    explicit Lcg(uint64_t seed) : s(seed * 6364136223846793005ull + 1442695040888963407ull) {}
    uint32_t next() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return static_cast<uint32_t>(s >> 33);
    }
    int below(int n) { return static_cast<int>(next() % static_cast<uint32_t>(n)); }
};

struct Lp {
    int m = 0, n = 0;
    std::vector<int> cp, ri;
    std::vector<double> v;
};

// n = 2m columns with `per_col` distinct rows each; column j < m also touches row j
// so that every row has an entry
Lp random_lp(int m, int per_col, uint64_t seed) {
    Lcg g(seed);
    Lp lp;
    lp.m = m;
    lp.n = 2 * m;
    lp.cp.push_back(0);
    for (int j = 0; j < lp.n; ++j) {
        std::vector<int> rows;
        if (j < m) rows.push_back(j);
        while (static_cast<int>(rows.size()) < per_col) {
            const int r = g.below(m);
            bool seen = false;
            for (int q : rows) seen = seen || q == r;
            if (!seen) rows.push_back(r);
        }
        for (size_t a = 1; a < rows.size(); ++a)      // sorted rows within the column
            for (size_t b = a; b > 0 && rows[b] < rows[b - 1]; --b) std::swap(rows[b], rows[b - 1]);
        for (int r : rows) {
            lp.ri.push_back(r);
            lp.v.push_back(0.5 + (g.below(1000) + 1) / 1000.0);
        }
        lp.cp.push_back(static_cast<int>(lp.ri.size()));
    }
    return lp;
}

int g_checks = 0, g_fail = 0;
void check(bool ok, const char* what, int a, int b) {
    ++g_checks;
    if (!ok && g_fail++ < 10) std::fprintf(stderr, "check failed: %s (%d, %d)\n", what, a, b);
}

void check_restriction(const ipm::FrontPlan& p, const std::vector<int>& sn_lp, const std::vector<int>& on) {
    ipm::RestrictedSteps r;
    ipm::restrict_steps(p, sn_lp, on, r);
    check(static_cast<int>(r.level_ptr.size()) == p.nlevels + 1, "level_ptr size", 0, 0);
    for (int l = 0; l < p.nlevels; ++l) {
        int q2 = r.level_ptr[l];
        for (int q = p.step_level_ptr[l]; q < p.step_level_ptr[l + 1]; ++q) {
            const ipm::PlanStep& st = p.steps[q];
            std::vector<int> keep;
            for (int i = 0; i < st.nitems; ++i)
                if (on[sn_lp[p.step_items[st.item_off + i]]]) keep.push_back(i);
            if (keep.empty()) continue;                // dropped: no restricted step for it
            check(q2 < r.level_ptr[l + 1], "step present", l, q);
            if (q2 >= r.level_ptr[l + 1]) return;
            const ipm::PlanStep& c = r.steps[q2++];
            check(c.k == st.k && c.level == st.level, "same tile step", c.k, st.k);
            check(c.nitems == static_cast<int>(keep.size()), "item count", c.nitems, static_cast<int>(keep.size()));
            for (size_t t = 0; t < keep.size(); ++t)
                check(r.items[c.item_off + t] == p.step_items[st.item_off + keep[t]], "item order", q,
                      static_cast<int>(t));
            const int offs[5][2] = {{st.trsm_prefix_off, c.trsm_prefix_off}, {st.upd_prefix_off, c.upd_prefix_off},
                                    {st.upd2_prefix_off, c.upd2_prefix_off}, {st.upd3_prefix_off, c.upd3_prefix_off},
                                    {st.digit_row_off, c.digit_row_off}};
            const int64_t totals[5] = {c.trsm_tiles, c.upd_tiles, c.upd2_blocks, c.upd3_blocks, c.digit_rows};
            for (int kind = 0; kind < 5; ++kind) {
                const int o = offs[kind][0], o2 = offs[kind][1];
                check(r.prefix[o2] == 0, "prefix starts at 0", kind, r.prefix[o2]);
                for (size_t t = 0; t < keep.size(); ++t) {
                    const int own = p.step_prefix[o + keep[t] + 1] - p.step_prefix[o + keep[t]];
                    const int got = r.prefix[o2 + t + 1] - r.prefix[o2 + t];
                    check(own == got, "item count kept", own, got);
                }
                check(totals[kind] == r.prefix[o2 + keep.size()], "step total", kind, static_cast<int>(totals[kind]));
            }
        }
        check(q2 == r.level_ptr[l + 1], "no extra steps", q2, r.level_ptr[l + 1]);
    }
}

bool run_batch(const std::vector<Lp>& lps, int* dense_mode, int* nlevels, int* nsteps) {
    std::vector<int> cp{0}, ri;
    std::vector<double> v;
    int M = 0, N = 0;
    for (const Lp& lp : lps) {
        for (int j = 0; j < lp.n; ++j) {
            for (int q = lp.cp[j]; q < lp.cp[j + 1]; ++q) {
                ri.push_back(M + lp.ri[q]);
                v.push_back(lp.v[q]);
            }
            cp.push_back(static_cast<int>(ri.size()));
        }
        M += lp.m;
        N += lp.n;
    }
    const core::Model md = core::Model::from_csc(M, N, cp.data(), ri.data(), v.data(),
                                                 std::vector<double>(M, 1.0).data(), std::vector<double>(N, 1.0).data());
    const core::CSRMatrix A = core::to_csr(md.A);
    std::vector<ipm::LpView> views;
    for (const Lp& lp : lps) {
        ipm::LpView w;
        w.m = lp.m;
        w.n = lp.n;
        w.col_ptrs = lp.cp.data();
        w.row_idx = lp.ri.data();
        w.vals = lp.v.data();
        views.push_back(w);
    }
    ipm::FrontPlan p;
    ipm::build_front_plan(views, A, 0, p);
    *dense_mode = p.dense_mode ? 1 : 0;
    *nlevels = p.nlevels;
    *nsteps = static_cast<int>(p.steps.size());
    const std::vector<int> sn_lp = ipm::supernode_lps(p);
    // every front's own rows belong to its LP
    for (int s = 0; s < p.ns; ++s)
        for (int q = 0; q < p.sn_ncols[s]; ++q) {
            const int r = p.perm[p.sn_first[s] + q];
            check(r >= p.row_off[sn_lp[s]] && r < p.row_off[sn_lp[s] + 1], "front rows in its LP", s, r);
        }
    const int k = static_cast<int>(lps.size());
    std::vector<std::vector<int>> masks;
    masks.push_back(std::vector<int>(k, 1));
    masks.push_back(std::vector<int>(k, 0));
    for (int a = 0; a < k; ++a) {
        std::vector<int> one(k, 0);
        one[a] = 1;
        masks.push_back(one);
    }
    std::vector<int> alt(k, 0);
    for (int a = 0; a < k; a += 2) alt[a] = 1;
    masks.push_back(alt);
    for (const auto& mk : masks) check_restriction(p, sn_lp, mk);
    // all on: the plan's own lists
    ipm::RestrictedSteps all;
    ipm::restrict_steps(p, sn_lp, masks[0], all);
    check(all.items == p.step_items, "all on keeps every item", static_cast<int>(all.items.size()),
          static_cast<int>(p.step_items.size()));
    check(all.steps.size() == p.steps.size(), "all on keeps every step", static_cast<int>(all.steps.size()),
          static_cast<int>(p.steps.size()));
    ipm::RestrictedSteps none;
    ipm::restrict_steps(p, sn_lp, masks[1], none);
    check(none.steps.empty() && none.items.empty(), "none on leaves no step", static_cast<int>(none.steps.size()), 0);
    return true;
}

}  // namespace

int main() {
    // dense-front batch: small LPs whose A A^T is dense (many entries per column)
    std::vector<Lp> dense;
    const int dm[5] = {70, 150, 90, 200, 130};
    for (int a = 0; a < 5; ++a) dense.push_back(random_lp(dm[a], dm[a] / 3, 11 + a));
    // sparse batch: three entries per column, multifrontal levels
    std::vector<Lp> sparse;
    const int sm[6] = {400, 250, 600, 300, 500, 350};
    for (int a = 0; a < 6; ++a) sparse.push_back(random_lp(sm[a], 3, 101 + a));
    int d_mode = 0, d_lv = 0, d_st = 0, s_mode = 0, s_lv = 0, s_st = 0;
    run_batch(dense, &d_mode, &d_lv, &d_st);
    run_batch(sparse, &s_mode, &s_lv, &s_st);
    std::printf("{\"checks\": %d, \"failed\": %d, \"dense\": {\"dense_mode\": %d, \"levels\": %d, \"steps\": %d}, "
                "\"sparse\": {\"dense_mode\": %d, \"levels\": %d, \"steps\": %d}}\n",
                g_checks, g_fail, d_mode, d_lv, d_st, s_mode, s_lv, s_st);
    return g_fail == 0 ? 0 : 1;
}
