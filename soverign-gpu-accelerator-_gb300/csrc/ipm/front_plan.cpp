// Multifrontal plan construction (see front_plan.hpp).
#include "ipm/front_plan.hpp"

#include <algorithm>
#include <functional>
#include <future>
#include <thread>
#include <numeric>
#include <stdexcept>

#include "ipm/symbolic.hpp"

namespace sankhya {
namespace ipm {

bool prefer_dense_front(const LpView& lp) {
    if (lp.m <= 256) return true;
    double pairs = 0.0;
    for (Index j = 0; j < lp.n; ++j) {
        const double c = lp.col_ptrs[j + 1] - lp.col_ptrs[j];
        pairs += c * (c - 1.0);
    }
    return pairs >= 0.05 * static_cast<double>(lp.m) * (lp.m - 1.0);
}

namespace {

int64_t tri(int64_t t) { return t * (t + 1) / 2; }
int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Postorder of a forest: roots in increasing order, children in increasing order.
std::vector<Index> postorder(const std::vector<Index>& parent) {
    const Index m = static_cast<Index>(parent.size());
    std::vector<Index> head(static_cast<size_t>(m), -1), next(static_cast<size_t>(m), -1);
    for (Index j = m - 1; j >= 0; --j) {  // push in reverse so lists come out increasing
        const Index p = parent[j];
        if (p >= 0) { next[j] = head[p]; head[p] = j; }
    }
    std::vector<Index> post;
    post.reserve(static_cast<size_t>(m));
    std::vector<Index> stack;
    std::vector<Index> it(static_cast<size_t>(m), -2);
    for (Index r = 0; r < m; ++r) {
        if (parent[r] >= 0) continue;
        stack.push_back(r);
        it[r] = head[r];
        while (!stack.empty()) {
            const Index v = stack.back();
            const Index c = it[v];
            if (c >= 0) {
                it[v] = next[c];
                stack.push_back(c);
                it[c] = head[c];
            } else {
                post.push_back(v);
                stack.pop_back();
            }
        }
    }
    return post;
}

}  // namespace

static void build_schedule(FrontPlan& p) {
    // levels
    p.sn_level.assign(static_cast<size_t>(p.ns), 0);
    for (int s = 0; s < p.ns; ++s) {  // children precede parents (postorder)
        const int par = p.sn_parent[s];
        if (par >= 0) p.sn_level[par] = std::max(p.sn_level[par], p.sn_level[s] + 1);
    }
    p.nlevels = 0;
    for (int s = 0; s < p.ns; ++s) p.nlevels = std::max(p.nlevels, p.sn_level[s] + 1);
    p.level_ptr.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    for (int s = 0; s < p.ns; ++s) p.level_ptr[p.sn_level[s] + 1]++;
    for (int l = 0; l < p.nlevels; ++l) p.level_ptr[l + 1] += p.level_ptr[l];
    p.level_sn.assign(static_cast<size_t>(p.ns), 0);
    {
        std::vector<int> nx(p.level_ptr.begin(), p.level_ptr.end() - 1);
        for (int s = 0; s < p.ns; ++s) p.level_sn[nx[p.sn_level[s]]++] = s;
    }
    // tile steps
    p.steps.clear();
    p.step_items.clear();
    p.step_prefix.clear();
    p.max_digit_rows = 0;
    p.step_level_ptr.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    for (int l = 0; l < p.nlevels; ++l) {
        int kmax = 0;
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) kmax = std::max(kmax, p.sn_ncols[p.level_sn[q]]);
        const int nsteps = static_cast<int>(ceil_div(kmax, kTile));
        for (int k = 0; k < nsteps; ++k) {
            PlanStep st;
            st.level = l;
            st.k = k;
            st.item_off = static_cast<int>(p.step_items.size());
            std::vector<int> items;
            for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
                const int s = p.level_sn[q];
                if (p.sn_ncols[s] > k * kTile) items.push_back(s);
            }
            st.nitems = static_cast<int>(items.size());
            p.step_items.insert(p.step_items.end(), items.begin(), items.end());
            st.trsm_prefix_off = static_cast<int>(p.step_prefix.size());
            int64_t acc = 0;
            p.step_prefix.push_back(0);
            for (int s : items) {
                const int64_t w = std::min<int64_t>(kTile, p.sn_ncols[s] - static_cast<int64_t>(k) * kTile);
                const int64_t below = p.sn_nrows[s] - static_cast<int64_t>(k) * kTile - w;
                acc += ceil_div(below, kTile);
                p.step_prefix.push_back(static_cast<int>(acc));
            }
            st.trsm_tiles = acc;
            st.upd_prefix_off = static_cast<int>(p.step_prefix.size());
            acc = 0;
            p.step_prefix.push_back(0);
            for (int s : items) {
                const int64_t w = std::min<int64_t>(kTile, p.sn_ncols[s] - static_cast<int64_t>(k) * kTile);
                const int64_t t = p.sn_nrows[s] - static_cast<int64_t>(k) * kTile - w;
                acc += tri(ceil_div(t, kTile));
                if (acc > INT32_MAX) throw std::runtime_error("front plan: too many tiles in one step");
                p.step_prefix.push_back(static_cast<int>(acc));
            }
            st.upd_tiles = acc;
            st.upd2_prefix_off = static_cast<int>(p.step_prefix.size());
            acc = 0;
            p.step_prefix.push_back(0);
            for (int s : items) {
                const int64_t w = std::min<int64_t>(kTile, p.sn_ncols[s] - static_cast<int64_t>(k) * kTile);
                const int64_t t = p.sn_nrows[s] - static_cast<int64_t>(k) * kTile - w;
                acc += tri(ceil_div(t, 2 * kTile));
                p.step_prefix.push_back(static_cast<int>(acc));
            }
            st.upd2_blocks = acc;
            st.upd3_prefix_off = static_cast<int>(p.step_prefix.size());
            acc = 0;
            p.step_prefix.push_back(0);
            for (int s : items) {
                const int64_t w = std::min<int64_t>(kTile, p.sn_ncols[s] - static_cast<int64_t>(k) * kTile);
                const int64_t t = p.sn_nrows[s] - static_cast<int64_t>(k) * kTile - w;
                const int64_t nbr = ceil_div(t, 2 * kTile);
                acc += nbr * (nbr + 1);
                if (acc > INT32_MAX) throw std::runtime_error("front plan: too many blocks in one step");
                p.step_prefix.push_back(static_cast<int>(acc));
            }
            st.upd3_blocks = acc;
            st.digit_row_off = static_cast<int>(p.step_prefix.size());
            acc = 0;
            p.step_prefix.push_back(0);
            for (int s : items) {
                const int64_t w = std::min<int64_t>(kTile, p.sn_ncols[s] - static_cast<int64_t>(k) * kTile);
                const int64_t t = p.sn_nrows[s] - static_cast<int64_t>(k) * kTile - w;
                acc += ceil_div(t, 2 * kTile) * 2 * kTile;
                if (acc > INT32_MAX) throw std::runtime_error("front plan: too many digit rows in one step");
                p.step_prefix.push_back(static_cast<int>(acc));
            }
            st.digit_rows = acc;
            p.max_digit_rows = std::max(p.max_digit_rows, acc);
            p.steps.push_back(st);
        }
        p.step_level_ptr[l + 1] = static_cast<int>(p.steps.size());
    }
    // extend-add rounds and children lists
    std::vector<int> rank(static_cast<size_t>(p.ns), 0), nseen(static_cast<size_t>(p.ns), 0);
    std::vector<std::vector<int>> kids(static_cast<size_t>(p.ns));
    for (int l = 0; l < p.nlevels; ++l) {
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            const int s = p.level_sn[q];
            const int par = p.sn_parent[s];
            if (par < 0) continue;
            kids[par].push_back(s);
        }
        // per-level ranks: reset counters of parents touched at this level
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            const int par = p.sn_parent[p.level_sn[q]];
            if (par >= 0) nseen[par] = 0;
        }
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            const int s = p.level_sn[q];
            const int par = p.sn_parent[s];
            if (par >= 0) rank[s] = nseen[par]++;
        }
    }
    p.ch_ptr.assign(static_cast<size_t>(p.ns) + 1, 0);
    p.ch_list.clear();
    for (int s = 0; s < p.ns; ++s) {
        p.ch_list.insert(p.ch_list.end(), kids[s].begin(), kids[s].end());
        p.ch_ptr[s + 1] = static_cast<Index>(p.ch_list.size());
    }
    p.rounds.clear();
    p.round_items.clear();
    p.round_prefix.clear();
    p.round_level_ptr.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    for (int l = 0; l < p.nlevels; ++l) {
        int maxr = -1;
        for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
            const int s = p.level_sn[q];
            if (p.sn_parent[s] >= 0 && p.sn_nrows[s] > p.sn_ncols[s]) maxr = std::max(maxr, rank[s]);
        }
        for (int r = 0; r <= maxr; ++r) {
            PlanRound rd;
            rd.level = l;
            rd.item_off = static_cast<int>(p.round_items.size());
            rd.prefix_off = static_cast<int>(p.round_prefix.size());
            p.round_prefix.push_back(0);
            int64_t acc = 0;
            for (int q = p.level_ptr[l]; q < p.level_ptr[l + 1]; ++q) {
                const int s = p.level_sn[q];
                if (p.sn_parent[s] < 0 || rank[s] != r) continue;
                const int64_t u = p.sn_nrows[s] - p.sn_ncols[s];
                if (u <= 0) continue;
                p.round_items.push_back(s);
                acc += tri(ceil_div(u, 32));
                if (acc > INT32_MAX) throw std::runtime_error("front plan: too many extend-add tiles");
                p.round_prefix.push_back(static_cast<int>(acc));
            }
            rd.nitems = static_cast<int>(p.round_items.size()) - rd.item_off;
            rd.tiles = acc;
            if (rd.nitems > 0) p.rounds.push_back(rd);
            else p.round_prefix.pop_back();
        }
        p.round_level_ptr[l + 1] = static_cast<int>(p.rounds.size());
    }
}

static void finish_offsets(FrontPlan& p) {
    p.sn_F_off.assign(static_cast<size_t>(p.ns), 0);
    p.sn_f_off.assign(static_cast<size_t>(p.ns), 0);
    p.sn_lda.assign(static_cast<size_t>(p.ns), 0);
    p.F_size = 0;
    p.f_size = 0;
    p.nnz_factor = 0;
    p.flops_factor = 0.0;
    for (int s = 0; s < p.ns; ++s) {
        const int64_t N = p.sn_nrows[s], K = p.sn_ncols[s];
        const int64_t lda = (N + 3) & ~int64_t(3);
        p.sn_lda[s] = static_cast<Index>(lda);
        p.sn_F_off[s] = p.F_size;
        p.F_size += lda * N;                      // multiple of 4 entries: fronts stay 16-byte aligned
        p.sn_f_off[s] = p.f_size;
        p.f_size += N;
        p.nnz_factor += N * K - K * (K - 1) / 2;
        for (int64_t c = 0; c < K; ++c) {
            const double len = static_cast<double>(N - c);
            p.flops_factor += len * len;
        }
    }
}

namespace {

// Automatic ordering from this many rows (of the largest LP) on: the given row
// order or nested dissection, whichever needs fewer factorisation flops. Minimum
// degree is left out there: its quotient-graph elimination (no supervariables)
// takes minutes at 200000 rows.
constexpr Index kLargeRows = 50000;

// Factorisation flops sum_j c_j^2 (c_j = column count of L incl. the diagonal)
// of the normal matrix in elimination order perm.
double factor_flops(const core::CSRMatrix& A, const std::vector<Index>& perm) {
    const Index M = A.rows;
    std::vector<Index> iperm(static_cast<size_t>(M));
    for (Index k = 0; k < M; ++k) iperm[perm[k]] = k;
    std::vector<Index> rp, ci;
    permuted_lower_pattern(A, iperm, rp, ci);
    const std::vector<Index> parent = elimination_tree(M, rp, ci);
    std::vector<int64_t> cc(static_cast<size_t>(M), 1);
    auto count_rows = [&](Index i0, Index i1, std::vector<int64_t>& out) {
        std::vector<Index> mark(static_cast<size_t>(M), -1);
        for (Index i = i0; i < i1; ++i) {
            mark[i] = i;
            for (Index q = rp[i]; q < rp[i + 1]; ++q)
                for (Index j = ci[q]; j != -1 && mark[j] != i; j = parent[j]) {
                    mark[j] = i;
                    out[j]++;
                }
        }
    };
    const int nt = M >= 16384 ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency()))) : 1;
    if (nt == 1) {
        count_rows(0, M, cc);
    } else {      // per-thread integer counts, summed: the same counts as one sweep
        std::vector<std::vector<int64_t>> part(static_cast<size_t>(nt), std::vector<int64_t>(static_cast<size_t>(M), 0));
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back(count_rows, static_cast<Index>(static_cast<int64_t>(M) * t / nt),
                              static_cast<Index>(static_cast<int64_t>(M) * (t + 1) / nt), std::ref(part[t]));
        for (auto& th : pool) th.join();
        for (const auto& c : part)
            for (Index j = 0; j < M; ++j) cc[j] += c[j];
    }
    double f = 0.0;
    for (Index j = 0; j < M; ++j) f += static_cast<double>(cc[j]) * static_cast<double>(cc[j]);
    return f;
}

}  // namespace

void build_front_plan(const std::vector<LpView>& lps, const core::CSRMatrix& A, int ordering, FrontPlan& p,
                      const std::vector<Index>* explicit_perm) {
    p = FrontPlan();
    p.nlp = static_cast<int>(lps.size());
    p.row_off.assign(static_cast<size_t>(p.nlp) + 1, 0);
    p.col_off.assign(static_cast<size_t>(p.nlp) + 1, 0);
    // A batch runs in dense mode when its LPs prefer dense fronts, or when the LPs that
    // do not are a negligible part of the batch's dense factorisation work (their
    // sum of m^3 at most 2% of the batch's): one dense front each then costs little
    // extra and spares the whole batch the sparse analysis.
    double cube_all = 0.0, cube_sparse = 0.0;
    for (int k = 0; k < p.nlp; ++k) {
        p.row_off[k + 1] = p.row_off[k] + lps[k].m;
        p.col_off[k + 1] = p.col_off[k] + lps[k].n;
        const double c = static_cast<double>(lps[k].m) * lps[k].m * lps[k].m;
        cube_all += c;
        if (!prefer_dense_front(lps[k])) cube_sparse += c;
    }
    const bool all_dense = cube_sparse == 0.0 || (p.nlp > 1 && cube_sparse <= 0.02 * cube_all);
    p.M = p.row_off[p.nlp];
    p.N = p.col_off[p.nlp];
    p.nnzA = A.row_ptrs.empty() ? 0 : A.row_ptrs.back();
    p.dense_mode = !explicit_perm && (ordering == 0 || ordering == 2) && all_dense;

    if (p.dense_mode) {
        p.ordering_used = 2;
        p.perm.resize(static_cast<size_t>(p.M));
        std::iota(p.perm.begin(), p.perm.end(), 0);
        p.iperm = p.perm;
        p.ns = p.nlp;
        for (int k = 0; k < p.nlp; ++k) {
            p.sn_first.push_back(p.row_off[k]);
            p.sn_ncols.push_back(lps[k].m);
            p.sn_nrows.push_back(lps[k].m);
            p.sn_parent.push_back(-1);
            p.sn_lp.push_back(k);
            p.sn_rows_off.push_back(static_cast<int64_t>(p.rows.size()));
            for (Index i = 0; i < lps[k].m; ++i) p.rows.push_back(p.row_off[k] + i);
            p.ea_off.push_back(static_cast<int64_t>(p.ea_map.size()));
        }
        p.sn_of_col.resize(static_cast<size_t>(p.M));
        for (int k = 0; k < p.nlp; ++k)
            for (Index i = p.row_off[k]; i < p.row_off[k + 1]; ++i) p.sn_of_col[i] = k;
        finish_offsets(p);
        build_schedule(p);
        return;
    }

    // 1. ordering
    std::vector<Index> perm0;
    if (explicit_perm) {
        if (static_cast<Index>(explicit_perm->size()) != p.M) throw std::invalid_argument("front plan: |P| != m");
        perm0 = *explicit_perm;
        std::vector<char> seen(static_cast<size_t>(p.M), 0);
        for (Index v : perm0) {
            if (v < 0 || v >= p.M || seen[v]) throw std::invalid_argument("front plan: P is not a permutation");
            seen[v] = 1;
        }
        p.ordering_used = 3;
    } else if (ordering == 1) {
        perm0 = compute_amd_ordering(A);
        p.ordering_used = 1;
    } else if (ordering == 2) {
        perm0.resize(static_cast<size_t>(p.M));
        std::iota(perm0.begin(), perm0.end(), 0);
        p.ordering_used = 2;
    } else if (ordering == 4) {
        perm0 = nested_dissection_ordering(A);
        p.ordering_used = 4;
    } else {
        Index largest = 0;
        for (const auto& v : lps) largest = std::max(largest, v.m);
        if (ordering == 0 && largest >= kLargeRows) {
            // the given row order (stage-major models are nearly banded) or nested
            // dissection, whichever needs fewer flops
            perm0.resize(static_cast<size_t>(p.M));
            std::iota(perm0.begin(), perm0.end(), 0);
            p.ordering_used = 2;
            auto natural = std::async(std::launch::async, [&]() { return factor_flops(A, perm0); });
            std::vector<Index> nd = nested_dissection_ordering(A);
            const double natural_flops = natural.get();
            if (factor_flops(A, nd) < natural_flops) {
                perm0.swap(nd);
                p.ordering_used = 4;
            }
        } else {
            perm0 = fill_reducing_ordering(A);
            p.ordering_used = 0;
        }
    }
    std::vector<Index> iperm0(static_cast<size_t>(p.M));
    for (Index k = 0; k < p.M; ++k) iperm0[perm0[k]] = k;
    std::vector<Index> rp, ci;
    permuted_lower_pattern(A, iperm0, rp, ci);
    std::vector<Index> parent0 = elimination_tree(p.M, rp, ci);
    // 2. postorder relabel (kept off for an explicit order)
    std::vector<Index> post = postorder(parent0);
    if (explicit_perm) std::iota(post.begin(), post.end(), 0);
    std::vector<Index> ipost(static_cast<size_t>(p.M));
    for (Index k = 0; k < p.M; ++k) ipost[post[k]] = k;
    p.perm.resize(static_cast<size_t>(p.M));
    p.iperm.resize(static_cast<size_t>(p.M));
    for (Index k = 0; k < p.M; ++k) p.perm[k] = perm0[post[k]];
    for (Index k = 0; k < p.M; ++k) p.iperm[p.perm[k]] = k;
    std::vector<Index> parent(static_cast<size_t>(p.M), -1);
    for (Index k = 0; k < p.M; ++k) {
        const Index q = parent0[post[k]];
        parent[k] = q >= 0 ? ipost[q] : -1;
    }
    permuted_lower_pattern(A, p.iperm, rp, ci);
    // 3. column counts by row-subtree traversal
    std::vector<int64_t> colcount(static_cast<size_t>(p.M), 1);
    {
        // row i adds one to every column on the paths from its entries up the tree; the
        // rows split into ranges on worker threads with their own marks and counts,
        // summed afterwards (integer counts: the same result in any order)
        auto count_rows = [&](Index i0, Index i1, std::vector<int64_t>& cc) {
            std::vector<Index> mark(static_cast<size_t>(p.M), -1);
            for (Index i = i0; i < i1; ++i) {
                mark[i] = i;
                for (Index q = rp[i]; q < rp[i + 1]; ++q)
                    for (Index j = ci[q]; j != -1 && mark[j] != i; j = parent[j]) {
                        mark[j] = i;
                        cc[j]++;
                    }
            }
        };
        const int nt = p.M >= 16384 ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())))
                                    : 1;
        if (nt == 1) {
            count_rows(0, p.M, colcount);
        } else {
            std::vector<std::vector<int64_t>> part(static_cast<size_t>(nt),
                                                   std::vector<int64_t>(static_cast<size_t>(p.M), 0));
            std::vector<std::thread> pool;
            for (int t = 0; t < nt; ++t)
                pool.emplace_back(count_rows, static_cast<Index>(static_cast<int64_t>(p.M) * t / nt),
                                  static_cast<Index>(static_cast<int64_t>(p.M) * (t + 1) / nt), std::ref(part[t]));
            for (auto& th : pool) th.join();
            for (const auto& cc : part)
                for (Index j = 0; j < p.M; ++j) colcount[j] += cc[j];
        }
    }
    std::vector<Index> nchild(static_cast<size_t>(p.M), 0);
    for (Index j = 0; j < p.M; ++j) if (parent[j] >= 0) nchild[parent[j]]++;
    // 4. fundamental supernodes
    std::vector<Index> sfirst;
    for (Index j = 0; j < p.M; ++j) {
        const bool extend = j > 0 && parent[j - 1] == j && colcount[j - 1] == colcount[j] + 1 && nchild[j] == 1;
        if (!extend) sfirst.push_back(j);
    }
    const Index nfund = static_cast<Index>(sfirst.size());
    std::vector<Index> fsn(static_cast<size_t>(p.M));
    for (Index s = 0; s < nfund; ++s) {
        const Index e = s + 1 < nfund ? sfirst[s + 1] : p.M;
        for (Index j = sfirst[s]; j < e; ++j) fsn[j] = s;
    }
    // 5. relaxed amalgamation of a supernode into its parent when it is the
    //    parent's last child (its columns end right before the parent's).
    std::vector<int64_t> s_ncols(static_cast<size_t>(nfund)), s_nrows(static_cast<size_t>(nfund)),
        s_zeros(static_cast<size_t>(nfund), 0);
    std::vector<Index> s_first(sfirst), s_par(static_cast<size_t>(nfund), -1);
    for (Index s = 0; s < nfund; ++s) {
        const Index e = s + 1 < nfund ? sfirst[s + 1] : p.M;
        s_ncols[s] = e - sfirst[s];
        s_nrows[s] = colcount[sfirst[s]];
        const Index last = e - 1;
        s_par[s] = parent[last] >= 0 ? fsn[parent[last]] : -1;
    }
    std::vector<Index> merged_into(static_cast<size_t>(nfund), -1);
    auto find = [&](Index s) {
        while (merged_into[s] >= 0) s = merged_into[s];
        return s;
    };
    for (Index s = 0; s < nfund; ++s) {  // postorder: children first
        const Index par0 = s_par[s];
        if (par0 < 0) continue;
        const Index par = find(par0);
        const int64_t lastc = s_first[s] + s_ncols[s];
        if (lastc != s_first[par]) continue;  // not the parent's last child
        const int64_t nc = s_ncols[s] + s_ncols[par];
        const int64_t nr = s_ncols[s] + s_nrows[par];
        const int64_t z = s_zeros[s] + s_zeros[par] + s_ncols[s] * (s_ncols[s] + s_nrows[par] - s_nrows[s]);
        const int64_t total = nc * nr - nc * (nc - 1) / 2;
        const double frac = static_cast<double>(z) / static_cast<double>(total);
        const bool merge = nc <= 16 || (nc <= 48 && frac < 0.5) || (nc <= 160 && frac < 0.2) || frac < 0.06;
        if (!merge) continue;
        merged_into[s] = par;
        s_first[par] = s_first[s];
        s_ncols[par] = nc;
        s_nrows[par] = nr;
        s_zeros[par] = z;
    }
    // final supernodes in column order
    std::vector<Index> final_id(static_cast<size_t>(nfund), -1);
    for (Index s = 0; s < nfund; ++s) {
        if (merged_into[s] >= 0) continue;
        final_id[s] = 0;
    }
    std::vector<std::pair<Index, Index>> roots;  // (first col, fund id)
    for (Index s = 0; s < nfund; ++s) if (merged_into[s] < 0) roots.push_back({s_first[s], s});
    std::sort(roots.begin(), roots.end());
    p.ns = static_cast<int>(roots.size());
    for (int t = 0; t < p.ns; ++t) final_id[roots[t].second] = t;
    p.sn_first.resize(static_cast<size_t>(p.ns));
    p.sn_ncols.resize(static_cast<size_t>(p.ns));
    p.sn_parent.assign(static_cast<size_t>(p.ns), -1);
    p.sn_lp.assign(static_cast<size_t>(p.ns), 0);
    p.sn_of_col.assign(static_cast<size_t>(p.M), -1);
    for (int t = 0; t < p.ns; ++t) {
        const Index s = roots[t].second;
        p.sn_first[t] = s_first[s];
        p.sn_ncols[t] = static_cast<Index>(s_ncols[s]);
        for (Index j = s_first[s]; j < s_first[s] + s_ncols[s]; ++j) p.sn_of_col[j] = t;
    }
    for (int t = 0; t < p.ns; ++t) {
        const Index last = p.sn_first[t] + p.sn_ncols[t] - 1;
        p.sn_parent[t] = parent[last] >= 0 ? p.sn_of_col[parent[last]] : -1;
        const Index row = p.perm[p.sn_first[t]];
        p.sn_lp[t] = static_cast<Index>(std::upper_bound(p.row_off.begin(), p.row_off.end(), row) - p.row_off.begin() - 1);
    }
    // 6. row structures (children precede parents in column order)
    std::vector<Index> cp(static_cast<size_t>(p.M) + 1, 0), crow(ci.size());
    for (Index q : ci) cp[static_cast<size_t>(q) + 1]++;
    for (Index j = 0; j < p.M; ++j) cp[j + 1] += cp[j];
    {
        std::vector<Index> nx(cp.begin(), cp.end() - 1);
        for (Index i = 0; i < p.M; ++i)
            for (Index q = rp[i]; q < rp[i + 1]; ++q) crow[nx[ci[q]]++] = i;
    }
    std::vector<std::vector<Index>> kids(static_cast<size_t>(p.ns));
    for (int t = 0; t < p.ns; ++t) if (p.sn_parent[t] >= 0) kids[p.sn_parent[t]].push_back(t);
    std::vector<Index> mark(static_cast<size_t>(p.M), -1);
    std::vector<Index> buf;
    p.sn_rows_off.assign(static_cast<size_t>(p.ns), 0);
    p.sn_nrows.assign(static_cast<size_t>(p.ns), 0);
    for (int t = 0; t < p.ns; ++t) {
        const Index f = p.sn_first[t], l = f + p.sn_ncols[t];
        buf.clear();
        for (Index j = f; j < l; ++j) { mark[j] = t; buf.push_back(j); }
        for (Index j = f; j < l; ++j)
            for (Index q = cp[j]; q < cp[j + 1]; ++q) {
                const Index i = crow[q];
                if (i >= l && mark[i] != t) { mark[i] = t; buf.push_back(i); }
            }
        for (int c : kids[t]) {
            const int64_t o = p.sn_rows_off[c];
            for (Index q = p.sn_ncols[c]; q < p.sn_nrows[c]; ++q) {
                const Index i = p.rows[o + q];
                if (i >= l && mark[i] != t) { mark[i] = t; buf.push_back(i); }
            }
        }
        std::sort(buf.begin() + (l - f), buf.end());
        p.sn_rows_off[t] = static_cast<int64_t>(p.rows.size());
        p.sn_nrows[t] = static_cast<Index>(buf.size());
        p.rows.insert(p.rows.end(), buf.begin(), buf.end());
    }
    // 7. extend-add maps
    p.ea_off.assign(static_cast<size_t>(p.ns), 0);
    std::vector<Index> pos(static_cast<size_t>(p.M), -1);
    for (int t = 0; t < p.ns; ++t) {
        p.ea_off[t] = static_cast<int64_t>(p.ea_map.size());
        const int par = p.sn_parent[t];
        if (par < 0) continue;
        const int64_t po = p.sn_rows_off[par];
        for (Index q = 0; q < p.sn_nrows[par]; ++q) pos[p.rows[po + q]] = q;
        const int64_t o = p.sn_rows_off[t];
        for (Index q = p.sn_ncols[t]; q < p.sn_nrows[t]; ++q) {
            const Index r = pos[p.rows[o + q]];
            if (r < 0) throw std::runtime_error("front plan: child row missing from parent structure");
            p.ea_map.push_back(r);
        }
        for (Index q = 0; q < p.sn_nrows[par]; ++q) pos[p.rows[po + q]] = -1;
    }
    finish_offsets(p);
    build_schedule(p);
    // 8. Khatri-Rao assembly map W. Slots: the M diagonal entries of A A^T first (slot i),
    // then its strictly lower entries in front-position order: the assembly runs one
    // thread per slot, so consecutive threads store consecutive entries of a front
    // column. Columns j are visited in order (fronts are laid out in column order, and
    // a front's rows are sorted), so the positions come out sorted without a sort.
    const int64_t noff = static_cast<int64_t>(ci.size());
    p.nslots = p.M + noff;
    p.slot_pos.resize(static_cast<size_t>(p.nslots));
    p.slot_i.resize(static_cast<size_t>(p.nslots));
    p.slot_j.resize(static_cast<size_t>(p.nslots));
    // column view of the strictly lower pattern (rows ascending within a column)
    std::vector<int64_t> lcp(static_cast<size_t>(p.M) + 1, 0);
    for (int64_t q = 0; q < noff; ++q) lcp[ci[q] + 1]++;
    for (Index j = 0; j < p.M; ++j) lcp[j + 1] += lcp[j];
    std::vector<Index> lrow(static_cast<size_t>(noff));
    {
        std::vector<int64_t> cur(lcp.begin(), lcp.end() - 1);
        for (Index i = 0; i < p.M; ++i)
            for (Index q = rp[i]; q < rp[i + 1]; ++q) lrow[cur[ci[q]]++] = i;
    }
    std::vector<int64_t> sid_row(static_cast<size_t>(noff));   // slot of row-view entry q
    {
        std::vector<Index> rowpos(static_cast<size_t>(p.M), -1);
        std::vector<int64_t> rcur(rp.begin(), rp.end() - 1);
        int64_t next = p.M, last_pos = -1;
        bool sorted = true;
        int tprev = -1;
        for (Index j = 0; j < p.M; ++j) {
            const int t = p.sn_of_col[j];
            const int64_t o = p.sn_rows_off[t];
            if (t != tprev) {
                for (Index q = 0; q < p.sn_nrows[t]; ++q) rowpos[p.rows[o + q]] = q;
                tprev = t;
            }
            auto fpos = [&](Index i) -> int64_t {
                const Index q = rowpos[i];
                if (q < 0 || q >= p.sn_nrows[t] || p.rows[o + q] != i)
                    throw std::runtime_error("front plan: M entry outside the factor structure");
                return p.sn_F_off[t] + q + static_cast<int64_t>(j - p.sn_first[t]) * p.sn_lda[t];
            };
            p.slot_i[j] = j;
            p.slot_j[j] = j;
            p.slot_pos[j] = fpos(j);
            for (int64_t e = lcp[j]; e < lcp[j + 1]; ++e) {
                const Index i = lrow[e];
                const int64_t sl = next++;
                p.slot_i[sl] = i;
                p.slot_j[sl] = j;
                p.slot_pos[sl] = fpos(i);
                if (p.slot_pos[sl] <= last_pos) sorted = false;
                last_pos = p.slot_pos[sl];
                sid_row[rcur[i]++] = sl;
            }
        }
        if (!sorted) throw std::runtime_error("front plan: front positions out of column order");
    }
    // W entries of each slot, row by row: row i of the permuted A A^T meets row j <= i in
    // every column k holding both; the entries of a slot follow in increasing k, as a
    // column-by-column sweep of A would give them.
    std::vector<int> col_lp(static_cast<size_t>(p.N), 0);
    for (int L = 0; L < p.nlp; ++L)
        for (Index k = p.col_off[L]; k < p.col_off[L + 1]; ++k) col_lp[k] = L;
    // Rows only touch their own slots (slot (i, j) belongs to row i), so both sweeps split
    // over row ranges on worker threads, each with its own column-to-slot scratch.
    auto sweep_rows = [&](Index i0, Index i1, std::vector<int64_t>& slot_of_col, auto&& visit) {
        for (Index i = i0; i < i1; ++i) {
            for (Index q = rp[i]; q < rp[i + 1]; ++q) slot_of_col[ci[q]] = sid_row[q];
            slot_of_col[i] = i;
            const Index r = p.perm[i];
            for (Index kk = A.row_ptrs[r]; kk < A.row_ptrs[r + 1]; ++kk) {
                const Index k = A.col_indices[kk];
                const int L = col_lp[k];
                const LpView& v = lps[L];
                const Index jl = k - p.col_off[L], ro = p.row_off[L];
                Float ar = 0.0;
                for (Index e = v.col_ptrs[jl]; e < v.col_ptrs[jl + 1]; ++e)
                    if (ro + v.row_idx[e] == r) { ar = v.vals[e]; break; }
                for (Index e = v.col_ptrs[jl]; e < v.col_ptrs[jl + 1]; ++e) {
                    const Index j2 = p.iperm[ro + v.row_idx[e]];
                    if (j2 <= i) visit(slot_of_col[j2], k, ar * v.vals[e]);
                }
            }
        }
    };
    const int nthreads = p.M >= 4096 ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())))
                                     : 1;
    auto parallel_rows = [&](auto&& visit) {
        auto body = [&](int t) {
            std::vector<int64_t> slot_of_col(static_cast<size_t>(p.M), -1);
            const Index i0 = static_cast<Index>(static_cast<int64_t>(p.M) * t / nthreads);
            const Index i1 = static_cast<Index>(static_cast<int64_t>(p.M) * (t + 1) / nthreads);
            sweep_rows(i0, i1, slot_of_col, visit);
        };
        if (nthreads == 1) { body(0); return; }
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t) pool.emplace_back(body, t);
        for (auto& th : pool) th.join();
    };
    std::vector<int64_t> cnt(static_cast<size_t>(p.nslots) + 1, 0);
    parallel_rows([&](int64_t sl, Index, Float) { cnt[sl + 1]++; });
    for (int64_t sl = 0; sl < p.nslots; ++sl) cnt[sl + 1] += cnt[sl];
    p.w_col.resize(static_cast<size_t>(cnt.back()));
    p.w_val.resize(static_cast<size_t>(cnt.back()));
    {
        std::vector<int64_t> nx(cnt.begin(), cnt.end() - 1);
        parallel_rows([&](int64_t sl, Index k, Float w) {
            const int64_t d = nx[sl]++;
            p.w_col[d] = k;
            p.w_val[d] = w;
        });
    }
    p.w_ptr.swap(cnt);
}

std::vector<int> supernode_lps(const FrontPlan& p) {
    std::vector<int> sn_lp(static_cast<size_t>(p.ns), 0);
    for (int s = 0; s < p.ns; ++s) {
        const Index r = p.perm[p.sn_first[s]];
        sn_lp[s] = static_cast<int>(std::upper_bound(p.row_off.begin(), p.row_off.end(), r) - p.row_off.begin()) - 1;
    }
    return sn_lp;
}

void restrict_steps(const FrontPlan& p, const std::vector<int>& sn_lp, const std::vector<int>& on,
                    RestrictedSteps& out) {
    out.steps.clear();
    out.items.clear();
    out.prefix.clear();
    out.level_ptr.assign(static_cast<size_t>(p.nlevels) + 1, 0);
    std::vector<int> keep;
    for (int l = 0; l < p.nlevels; ++l) {
        for (int q = p.step_level_ptr[l]; q < p.step_level_ptr[l + 1]; ++q) {
            const PlanStep& st = p.steps[q];
            keep.clear();
            for (int i = 0; i < st.nitems; ++i) {
                const int lp = sn_lp[p.step_items[st.item_off + i]];
                if (lp >= 0 && lp < static_cast<int>(on.size()) && on[lp]) keep.push_back(i);
            }
            if (keep.empty()) continue;
            PlanStep c = st;
            c.item_off = static_cast<int>(out.items.size());
            c.nitems = static_cast<int>(keep.size());
            for (int i : keep) out.items.push_back(p.step_items[st.item_off + i]);
            auto remap = [&](int off, int64_t& total) {
                const int at = static_cast<int>(out.prefix.size());
                int64_t acc = 0;
                out.prefix.push_back(0);
                for (int i : keep) {
                    acc += p.step_prefix[off + i + 1] - p.step_prefix[off + i];
                    out.prefix.push_back(static_cast<int>(acc));
                }
                total = acc;
                return at;
            };
            c.trsm_prefix_off = remap(st.trsm_prefix_off, c.trsm_tiles);
            c.upd_prefix_off = remap(st.upd_prefix_off, c.upd_tiles);
            c.upd2_prefix_off = remap(st.upd2_prefix_off, c.upd2_blocks);
            c.upd3_prefix_off = remap(st.upd3_prefix_off, c.upd3_blocks);
            c.digit_row_off = remap(st.digit_row_off, c.digit_rows);
            out.steps.push_back(c);
        }
        out.level_ptr[l + 1] = static_cast<int>(out.steps.size());
    }
}

}  // namespace ipm
}  // namespace sankhya
