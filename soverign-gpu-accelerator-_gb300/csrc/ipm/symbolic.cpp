// Symbolic analysis: exact minimum degree (reference ordering), elimination
// tree, L pattern, and the approximate minimum degree ordering of the solver.
#include "ipm/symbolic.hpp"

#include <algorithm>
#include <numeric>
#include <stdexcept>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace sankhya {
namespace ipm {

namespace {

// Rows of each column of CSR A (transpose of the pattern).
void column_rows(const core::CSRMatrix& A, std::vector<Index>& cptr, std::vector<Index>& crow) {
    cptr.assign(static_cast<size_t>(A.cols) + 1, 0);
    const Index nz = A.row_ptrs[static_cast<size_t>(A.rows)];
    for (Index k = 0; k < nz; ++k) cptr[static_cast<size_t>(A.col_indices[k]) + 1]++;
    for (Index j = 0; j < A.cols; ++j) cptr[j + 1] += cptr[j];
    crow.resize(static_cast<size_t>(nz));
    std::vector<Index> next(cptr.begin(), cptr.end() - 1);
    for (Index i = 0; i < A.rows; ++i)
        for (Index k = A.row_ptrs[i]; k < A.row_ptrs[i + 1]; ++k) crow[next[A.col_indices[k]]++] = i;
}

}  // namespace

// Sorted, duplicate-free adjacency of A A^T without self loops.
std::vector<std::vector<Index>> aat_graph(const core::CSRMatrix& A) {
    std::vector<Index> cptr, crow;
    column_rows(A, cptr, crow);
    std::vector<std::vector<Index>> adj(static_cast<size_t>(A.rows));
    // rows are independent: ranges of rows on worker threads, each with its own marks
    auto rows = [&](Index i0, Index i1) {
        std::vector<Index> mark(static_cast<size_t>(A.rows), -1);
        for (Index i = i0; i < i1; ++i) {
            auto& ai = adj[static_cast<size_t>(i)];
            mark[i] = i;
            for (Index k = A.row_ptrs[i]; k < A.row_ptrs[i + 1]; ++k) {
                const Index j = A.col_indices[k];
                for (Index q = cptr[j]; q < cptr[j + 1]; ++q) {
                    const Index r = crow[q];
                    if (mark[r] != i) { mark[r] = i; ai.push_back(r); }
                }
            }
            std::sort(ai.begin(), ai.end());
        }
    };
    const int nt = A.rows >= 4096 ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())))
                                  : 1;
    if (nt == 1) {
        rows(0, A.rows);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back(rows, static_cast<Index>(static_cast<int64_t>(A.rows) * t / nt),
                              static_cast<Index>(static_cast<int64_t>(A.rows) * (t + 1) / nt));
        for (auto& th : pool) th.join();
    }
    return adj;
}

std::vector<Index> compute_amd_ordering(const core::CSRMatrix& A) {
    const Index m = A.rows;
    auto adj = aat_graph(A);
    std::vector<char> done(static_cast<size_t>(m), 0);
    std::vector<Index> P;
    P.reserve(static_cast<size_t>(m));
    std::vector<Index> merged;
    for (Index step = 0; step < m; ++step) {
        Index u = -1;
        size_t best = static_cast<size_t>(m) + 1;
        for (Index i = 0; i < m; ++i)  // lowest index wins ties
            if (!done[i] && adj[i].size() < best) { best = adj[i].size(); u = i; }
        if (u < 0) throw std::runtime_error("compute_amd_ordering: Disconnected graph or invalid state");
        done[u] = 1;
        P.push_back(u);
        const std::vector<Index> nb = adj[u];
        for (Index v : nb) {
            // adj[v] <- (adj[v] \ {u}) U (nb \ {v})
            auto& av = adj[v];
            merged.clear();
            merged.reserve(av.size() + nb.size());
            std::set_union(av.begin(), av.end(), nb.begin(), nb.end(), std::back_inserter(merged));
            merged.erase(std::remove_if(merged.begin(), merged.end(), [&](Index w) { return w == u || w == v; }),
                         merged.end());
            av.swap(merged);
        }
    }
    return P;
}

void permuted_lower_pattern(const core::CSRMatrix& A, const std::vector<Index>& P_inv,
                            std::vector<Index>& rowptr, std::vector<Index>& colidx) {
    const Index m = A.rows;
    std::vector<Index> cptr, crow;
    column_rows(A, cptr, crow);
    std::vector<Index> P(static_cast<size_t>(m));
    for (Index i = 0; i < m; ++i) P[P_inv[i]] = i;
    rowptr.assign(static_cast<size_t>(m) + 1, 0);
    colidx.clear();
    // rows are independent: contiguous ranges of permuted rows on worker threads, each
    // building its part of the pattern, joined in row order
    struct Part { std::vector<Index> ci; };
    auto rows = [&](Index k0, Index k1, Part& out) {
        std::vector<Index> mark(static_cast<size_t>(m), -1);
        std::vector<Index> row;
        for (Index k = k0; k < k1; ++k) {
            const Index i = P[k];
            mark[i] = k;
            row.clear();
            for (Index q = A.row_ptrs[i]; q < A.row_ptrs[i + 1]; ++q) {
                const Index j = A.col_indices[q];
                for (Index t = cptr[j]; t < cptr[j + 1]; ++t) {
                    const Index r = crow[t];
                    if (mark[r] != k) {
                        mark[r] = k;
                        const Index pr = P_inv[r];
                        if (pr < k) row.push_back(pr);
                    }
                }
            }
            std::sort(row.begin(), row.end());
            out.ci.insert(out.ci.end(), row.begin(), row.end());
            rowptr[k + 1] = static_cast<Index>(row.size());
        }
    };
    const int nt = m >= 4096 ? static_cast<int>(std::max(1u, std::min(16u, std::thread::hardware_concurrency()))) : 1;
    std::vector<Part> parts(static_cast<size_t>(nt));
    if (nt == 1) {
        rows(0, m, parts[0]);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back(rows, static_cast<Index>(static_cast<int64_t>(m) * t / nt),
                              static_cast<Index>(static_cast<int64_t>(m) * (t + 1) / nt), std::ref(parts[t]));
        for (auto& th : pool) th.join();
    }
    for (Index k = 0; k < m; ++k) rowptr[k + 1] += rowptr[k];
    colidx.reserve(static_cast<size_t>(rowptr[m]));
    for (auto& pt : parts) colidx.insert(colidx.end(), pt.ci.begin(), pt.ci.end());
}

std::vector<Index> elimination_tree(Index m, const std::vector<Index>& rowptr,
                                    const std::vector<Index>& colidx) {
    std::vector<Index> parent(static_cast<size_t>(m), -1), anc(static_cast<size_t>(m), -1);
    for (Index i = 0; i < m; ++i) {
        for (Index q = rowptr[i]; q < rowptr[i + 1]; ++q) {
            Index j = colidx[q];
            while (j != -1 && j < i) {  // climb with path compression towards i
                const Index next = anc[j];
                anc[j] = i;
                if (next == -1) { parent[j] = i; break; }
                j = next;
            }
        }
    }
    return parent;
}

void compute_symbolic_factorization(const core::CSRMatrix& A, const std::vector<Index>& P,
                                    SymbolicFactorization& out) {
    const Index m = A.rows;
    if (static_cast<Index>(P.size()) != m) throw std::invalid_argument("compute_symbolic_factorization: |P| != m");
    out.P = P;
    out.P_inv.assign(static_cast<size_t>(m), 0);
    for (Index k = 0; k < m; ++k) out.P_inv[P[k]] = k;
    std::vector<Index> rp, ci;
    permuted_lower_pattern(A, out.P_inv, rp, ci);
    out.parent = elimination_tree(m, rp, ci);
    // Row i of L = union of etree paths from each j in row i of M up to i
    // (row-subtree traversal), listed in increasing column order.
    out.L_pattern.rows = m;
    out.L_pattern.cols = m;
    out.L_pattern.row_ptrs.assign(static_cast<size_t>(m) + 1, 0);
    out.L_pattern.col_indices.clear();
    std::vector<Index> mark(static_cast<size_t>(m), -1), row;
    for (Index i = 0; i < m; ++i) {
        mark[i] = i;
        row.clear();
        for (Index q = rp[i]; q < rp[i + 1]; ++q) {
            for (Index j = ci[q]; j != -1 && mark[j] != i; j = out.parent[j]) {
                mark[j] = i;
                row.push_back(j);
            }
        }
        std::sort(row.begin(), row.end());
        out.L_pattern.col_indices.insert(out.L_pattern.col_indices.end(), row.begin(), row.end());
        out.L_pattern.row_ptrs[i + 1] = static_cast<Index>(out.L_pattern.col_indices.size());
    }
    out.L_pattern.values.assign(out.L_pattern.col_indices.size(), 1.0);
}

// ---------------------------------------------------------------------------
// Approximate minimum degree on the quotient graph (Amestoy, Davis & Duff 1996):
// eliminated pivots become elements (cliques); each variable keeps its adjacent
// elements E_i and remaining variable neighbours A_i; the external degree of a
// variable touched by pivot p is bounded by
//   min(n_live - 1, d_old + |L_p \ i|, |A_i \ i| + |L_p \ i| + sum_{e in E_i, e != p} |L_e \ L_p|).
// Elements whose members all lie in L_p are absorbed (aggressive absorption).
// A_i is pruned of neighbours covered by the new element only on every 16th time
// i is touched (and always before i is eliminated): between prunings |A_i| is an
// over-count, which keeps the degree an upper bound, and variables touched by
// many pivots (rows linking many blocks) stop costing O(|A_i|) per pivot.
// Variables whose degree exceeds four times the current minimum are updated
// lazily: between refreshes (every 16th touch) they skip the |L_e \ L_p| scan and
// keep their degree; skipped decrements only over-estimate the other degrees.
// A lazily kept variable popped as pivot is re-scored first.
// Ties go to the most recently inserted variable of the minimum-degree bucket.
//
// Rows of A whose columns span more than a quarter of all columns (the linking
// rows of a block-angular LP) are ordered last when they are at most a quarter
// of the rows: they are never pivots while other rows remain, their own degrees
// are not maintained, and they follow in their given order. They still count in
// the degrees of the other rows, so the blocks are ordered as the full graph
// would order them, at a fraction of the cost (family 1: 0.13 s instead of
// 0.6 s). This is the constrained form of minimum degree that keeps dense or
// linking rows for the last front.
std::vector<Index> fill_reducing_ordering(const core::CSRMatrix& A) {
    const Index m = A.rows, n = A.cols;
    std::vector<char> last(static_cast<size_t>(m), 0);
    Index nlast = 0;
    for (Index i = 0; i < m; ++i) {
        const Index a = A.row_ptrs[i], b = A.row_ptrs[i + 1];
        if (b <= a) continue;
        Index lo = A.col_indices[a], hi = lo;
        for (Index q = a + 1; q < b; ++q) {
            lo = std::min(lo, A.col_indices[q]);
            hi = std::max(hi, A.col_indices[q]);
        }
        if (static_cast<int64_t>(hi - lo + 1) * 4 > n) { last[i] = 1; ++nlast; }
    }
    if (nlast == 0 || static_cast<int64_t>(nlast) * 4 > m) return min_degree_order(aat_graph(A));
    std::vector<std::vector<Index>> adj = aat_graph(A);
    // Once the linking rows are constrained to the end, the other rows fall apart into
    // the connected components of the graph without them (the blocks): pivots of one
    // component never change the degrees in another (elements of a component hold only
    // its own rows and linking rows, whose degrees are not kept). Each component is
    // ordered on its own subgraph (its rows plus the linking rows next to them), in
    // parallel; the components follow one another and the linking rows come last.
    std::vector<Index> comp(static_cast<size_t>(m), -1), stack;
    Index ncomp = 0;
    for (Index r = 0; r < m; ++r) {
        if (last[r] || comp[r] >= 0) continue;
        comp[r] = ncomp;
        stack.assign(1, r);
        while (!stack.empty()) {
            const Index u = stack.back();
            stack.pop_back();
            for (Index v : adj[u])
                if (!last[v] && comp[v] < 0) { comp[v] = ncomp; stack.push_back(v); }
        }
        ++ncomp;
    }
    if (ncomp <= 1) return min_degree_order(std::move(adj), &last);
    std::vector<std::vector<Index>> members(static_cast<size_t>(ncomp));
    for (Index r = 0; r < m; ++r)
        if (!last[r]) members[comp[r]].push_back(r);
    std::vector<std::vector<Index>> part(static_cast<size_t>(ncomp));
    // local numbering of a component's subgraph: a dense map per worker thread (reset
    // after each component), rows first in index order, then linking rows as met
    auto order_component = [&](Index c, std::vector<Index>& local) {
        const auto& rows = members[c];
        std::vector<Index> verts(rows.begin(), rows.end());
        for (size_t q = 0; q < rows.size(); ++q) local[rows[q]] = static_cast<Index>(q);
        const Index nrows = static_cast<Index>(rows.size());
        for (Index r : rows)
            for (Index v : adj[r])
                if (last[v] && local[v] < 0) {
                    local[v] = static_cast<Index>(verts.size());
                    verts.push_back(v);
                }
        std::vector<std::vector<Index>> g(verts.size());
        for (Index q = 0; q < nrows; ++q) {
            g[q].reserve(adj[rows[q]].size());
            for (Index v : adj[rows[q]]) {
                const Index lv = local[v];
                g[q].push_back(lv);
                if (lv >= nrows) g[lv].push_back(q);
            }
        }
        for (Index v : verts) local[v] = -1;
        for (auto& nb : g) std::sort(nb.begin(), nb.end());
        std::vector<char> lastl(verts.size(), 0);
        for (size_t q = static_cast<size_t>(nrows); q < verts.size(); ++q) lastl[q] = 1;
        const std::vector<Index> lo = min_degree_order(std::move(g), &lastl);
        auto& out = part[c];
        out.reserve(static_cast<size_t>(nrows));
        for (Index q = 0; q < nrows; ++q) out.push_back(verts[lo[q]]);
    };
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const Index nthreads = std::min<Index>(static_cast<Index>(hw), ncomp);
    std::vector<std::thread> pool;
    std::exception_ptr err;
    std::mutex err_mu;
    for (Index t = 0; t < nthreads; ++t)
        pool.emplace_back([&, t]() {
            try {
                std::vector<Index> local(static_cast<size_t>(m), -1);
                for (Index c = t; c < ncomp; c += nthreads) order_component(c, local);
            } catch (...) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (!err) err = std::current_exception();
            }
        });
    for (auto& th : pool) th.join();
    if (err) std::rethrow_exception(err);
    std::vector<Index> order;
    order.reserve(static_cast<size_t>(m));
    for (Index c = 0; c < ncomp; ++c) order.insert(order.end(), part[c].begin(), part[c].end());
    for (Index r = 0; r < m; ++r)
        if (last[r]) order.push_back(r);
    return order;
}

std::vector<Index> min_degree_order(std::vector<std::vector<Index>> Av, const std::vector<char>* last_rows) {
    const Index m = static_cast<Index>(Av.size());
    std::vector<Index> order;
    order.reserve(static_cast<size_t>(m));
    if (m == 0) return order;
    std::vector<std::vector<Index>> Ev(static_cast<size_t>(m));   // adjacent elements
    std::vector<std::vector<Index>> Le(static_cast<size_t>(m));   // element members (live variables)
    std::vector<char> eliminated(static_cast<size_t>(m), 0), dead_elem(static_cast<size_t>(m), 0);
    std::vector<Index> deg(static_cast<size_t>(m));
    for (Index i = 0; i < m; ++i) deg[i] = static_cast<Index>(Av[i].size());
    // Degree buckets as ordered sets of (degree, index) via a simple bucket array
    // of doubly linked lists; the minimum-degree search scans upward from the last
    // known minimum.
    std::vector<Index> head(static_cast<size_t>(m) + 1, -1), nxt(static_cast<size_t>(m), -1),
        prv(static_cast<size_t>(m), -1);
    auto insert = [&](Index i) {
        const Index d = deg[i];
        nxt[i] = head[d];
        prv[i] = -1;
        if (head[d] != -1) prv[head[d]] = i;
        head[d] = i;
    };
    auto remove = [&](Index i) {
        const Index d = deg[i];
        if (prv[i] != -1) nxt[prv[i]] = nxt[i]; else head[d] = nxt[i];
        if (nxt[i] != -1) prv[nxt[i]] = prv[i];
    };
    auto is_last = [&](Index i) { return last_rows && (*last_rows)[i]; };
    Index npivots = m;
    for (Index i = m - 1; i >= 0; --i) {
        if (is_last(i)) { --npivots; continue; }
        insert(i);
    }
    std::vector<Index> w(static_cast<size_t>(m), -1);   // |L_e \ L_p| scratch, -1 = unset
    std::vector<unsigned char> touches(static_cast<size_t>(m), 0), lazy_count(static_cast<size_t>(m), 0);
    std::vector<char> lazy(static_cast<size_t>(m), 0), stale(static_cast<size_t>(m), 0);
    std::vector<Index> inLp(static_cast<size_t>(m), -1);
    std::vector<Index> touched;
    Index mindeg = 0;
    Index live = m;
    for (Index k = 0; k < npivots; ++k) {
        Index p;
        for (;;) {
            while (mindeg <= m && head[mindeg] == -1) ++mindeg;
            p = head[mindeg];   // most recently inserted of the minimum bucket
            if (!stale[p]) break;
            // lazily kept degree: recompute the bound |A_p| + sum_e (|L_e| - 1)
            stale[p] = 0;
            Index d = 0;
            auto& Ep = Ev[p];
            size_t o = 0;
            for (Index e : Ep) if (!dead_elem[e]) { Ep[o++] = e; d += static_cast<Index>(Le[e].size()) - 1; }
            Ep.resize(o);
            d += static_cast<Index>(Av[p].size());
            d = std::max<Index>(0, std::min<Index>(d, live - 1));
            if (d <= mindeg) break;
            remove(p);
            deg[p] = d;
            insert(p);
        }
        remove(p);
        eliminated[p] = 1;
        order.push_back(p);
        --live;
        // L_p = A_p U (U_{e in E_p} L_e) \ {p}
        auto& Lp = Le[p];
        Lp.clear();
        inLp[p] = p;
        for (Index v : Av[p]) if (!eliminated[v] && inLp[v] != p) { inLp[v] = p; Lp.push_back(v); }
        // (A_p may still hold covered neighbours; they are de-duplicated by inLp)
        for (Index e : Ev[p]) {
            if (dead_elem[e]) continue;
            for (Index v : Le[e]) if (!eliminated[v] && inLp[v] != p) { inLp[v] = p; Lp.push_back(v); }
            dead_elem[e] = 1;               // absorbed into p
            Le[e].clear();
            Le[e].shrink_to_fit();
        }
        Av[p].clear(); Av[p].shrink_to_fit();
        Ev[p].clear(); Ev[p].shrink_to_fit();
        const Index lp_size = static_cast<Index>(Lp.size());
        // Update E_i, prune A_i, compute |L_e \ L_p|.
        touched.clear();
        const Index lazy_thr = std::max<Index>(64, 4 * std::max<Index>(1, mindeg));
        for (Index i : Lp) {
            auto& Ei = Ev[i];
            lazy[i] = is_last(i) || (deg[i] > lazy_thr && (++lazy_count[i] & 15) != 0);
            if (lazy[i]) { Ei.push_back(p); stale[i] = 1; continue; }
            size_t o = 0;
            for (Index e : Ei) if (!dead_elem[e] && e != p) Ei[o++] = e;
            Ei.resize(o);
            for (Index e : Ei) {
                if (w[e] < 0) { w[e] = static_cast<Index>(Le[e].size()); touched.push_back(e); }
                w[e] -= 1;
            }
            Ei.push_back(p);
            if (++touches[i] >= 16) {
                touches[i] = 0;
                auto& Ai = Av[i];
                size_t t = 0;
                for (Index v : Ai) if (!eliminated[v] && inLp[v] != p) Ai[t++] = v;
                Ai.resize(t);
            }
        }
        // Aggressive absorption of elements entirely inside L_p.
        for (Index e : touched)
            if (w[e] == 0) { dead_elem[e] = 1; Le[e].clear(); }
        for (Index i : Lp) {
            if (lazy[i] || is_last(i)) continue;
            stale[i] = 0;
            Index ext = 0;
            Index d = static_cast<Index>(Av[i].size()) + (lp_size - 1);
            auto& Ei = Ev[i];
            size_t o = 0;
            for (Index e : Ei) {
                if (dead_elem[e]) continue;
                Ei[o++] = e;
                if (e != p) ext += w[e];
            }
            Ei.resize(o);
            d += ext;
            const Index bound = std::min<Index>(live - 1, deg[i] + lp_size - 1);
            if (d > bound) d = bound;
            if (d < 0) d = 0;
            remove(i);
            deg[i] = d;
            insert(i);
            if (d < mindeg) mindeg = d;
        }
        for (Index e : touched) w[e] = -1;
    }
    if (npivots < m)
        for (Index i = 0; i < m; ++i)
            if (is_last(i)) order.push_back(i);
    return order;
}

}  // namespace ipm
}  // namespace sankhya
