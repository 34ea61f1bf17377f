// Nested dissection ordering of the graph of A A^T (declared in ipm/symbolic.hpp).
//
// The reference orders only by exact minimum degree (src/ipm/symbolic.cpp:11-98).
// On staircase LPs (stages coupled to the next stage only) greedy minimum degree
// interleaves the stages and fills far more than a stage-by-stage elimination;
// nested dissection finds the coupling rows as separators instead.
//
// A part (a connected vertex set) is split with a breadth-first level structure
// from a pseudo-peripheral vertex. Every level L_k separates the levels before it
// from the levels after it; narrower separators come from a band of kBand adjacent
// levels: the minimum vertex cut between the levels before the band and the levels
// after it, through the band (unit vertex capacities, Dinic's max-flow on the
// vertex-split graph). The narrowest balanced candidate becomes the separator; both
// sides are dissected further and the separator is ordered after them. Parts of at
// most `leaf` vertices, and parts whose best separator is larger than the smaller
// side, are ordered by minimum degree on their induced graph.
#include <algorithm>
#include <atomic>
#include <future>
#include <numeric>
#include <utility>

#include "ipm/symbolic.hpp"

namespace sankhya {
namespace ipm {

namespace {

constexpr Index kUnset = -1;

constexpr int kMinSideDiv = 5;      // each side of a separator holds at least 1/5 of the part
constexpr Index kSlackNum = 11, kSlackDen = 10;   // a separator up to 10% wider wins when better balanced
constexpr int kNoGain = 2;          // ball radii tried after the last narrower cut
constexpr int kParallelDepth = 4;   // separators whose sides are dissected concurrently: 2^4 threads at most
constexpr Index kParallelRows = 20000;

// Minimum vertex cut through a band of vertices 0..nb-1 (adjacency inside the band
// in CSR ptr/adj, both directions listed) between the vertices outside the band
// before it (touched where src[b] = 1) and after it (touched where snk[b] = 1):
// Dinic's max-flow on the split graph (in(b) -> out(b) capacity 1, every other
// arc unbounded). side[b]: 0 before the cut, 1 in the cut, 2 after it. Returns
// the cut size.
class BandCut {
public:
    Index run(Index nb, const std::vector<Index>& ptr, const std::vector<Index>& adj, const std::vector<char>& src,
              const std::vector<char>& snk, std::vector<char>& side) {
        const Index N = 2 * nb + 2, S = 2 * nb, T = 2 * nb + 1;
        // arcs in CSR form (each with its reverse residual arc): count, place, fill
        off_.assign(static_cast<size_t>(N) + 1, 0);
        auto count = [&](Index u, Index v) { off_[u + 1]++; off_[v + 1]++; };
        for (Index b = 0; b < nb; ++b) {
            count(2 * b, 2 * b + 1);
            for (Index q = ptr[b]; q < ptr[b + 1]; ++q) count(2 * b + 1, 2 * adj[q]);
            if (src[b]) count(S, 2 * b);
            if (snk[b]) count(2 * b + 1, T);
        }
        for (Index u = 0; u < N; ++u) off_[u + 1] += off_[u];
        const Index E = off_[N];
        to_.resize(static_cast<size_t>(E));
        cap_.resize(static_cast<size_t>(E));
        rev_.resize(static_cast<size_t>(E));
        it_.assign(off_.begin(), off_.end() - 1);
        auto arc = [&](Index u, Index v, Index c) {
            const Index e = it_[u]++, r = it_[v]++;
            to_[e] = v; cap_[e] = c; rev_[e] = r;
            to_[r] = u; cap_[r] = 0; rev_[r] = e;
        };
        for (Index b = 0; b < nb; ++b) {
            arc(2 * b, 2 * b + 1, 1);
            for (Index q = ptr[b]; q < ptr[b + 1]; ++q) arc(2 * b + 1, 2 * adj[q], kBig);
            if (src[b]) arc(S, 2 * b, kBig);
            if (snk[b]) arc(2 * b + 1, T, kBig);
        }
        lvl_.resize(static_cast<size_t>(N));
        it_.resize(static_cast<size_t>(N));
        Index flow = 0;
        while (levels(S, T, N)) {
            std::copy(off_.begin(), off_.end() - 1, it_.begin());
            while (augment(S, T)) ++flow;
        }
        // reachability from S in the final residual graph: the source side of the
        // minimum cut closest to S, the same for every maximum flow
        levels(S, T, N);
        side.resize(static_cast<size_t>(nb));
        for (Index b = 0; b < nb; ++b)
            side[b] = lvl_[2 * b] < 0 ? 2 : (lvl_[2 * b + 1] < 0 ? 1 : 0);
        return flow;
    }

private:
    static constexpr Index kBig = 0x3fffffff;
    std::vector<Index> off_, to_, cap_, rev_, lvl_, it_, queue_, path_;

    // Breadth-first distances from S over arcs with residual capacity; true if T is reached.
    bool levels(Index S, Index T, Index N) {
        std::fill(lvl_.begin(), lvl_.begin() + N, kUnset);
        queue_.clear();
        queue_.push_back(S);
        lvl_[S] = 0;
        for (size_t h = 0; h < queue_.size(); ++h) {
            const Index u = queue_[h];
            for (Index e = off_[u]; e < off_[u + 1]; ++e)
                if (cap_[e] > 0 && lvl_[to_[e]] < 0) { lvl_[to_[e]] = lvl_[u] + 1; queue_.push_back(to_[e]); }
        }
        return lvl_[T] >= 0;
    }

    // One augmenting path along increasing distances (current-arc depth-first
    // search); every path crosses a split arc, so it carries one unit.
    bool augment(Index S, Index T) {
        path_.clear();
        Index u = S;
        for (;;) {
            if (u == T) {
                for (Index e : path_) { cap_[e] -= 1; cap_[rev_[e]] += 1; }
                return true;
            }
            Index& e = it_[u];
            while (e < off_[u + 1] && !(cap_[e] > 0 && lvl_[to_[e]] == lvl_[u] + 1)) ++e;
            if (e >= off_[u + 1]) {
                lvl_[u] = kUnset;            // dead end for this phase
                if (path_.empty()) return false;
                const Index back = path_.back();
                path_.pop_back();
                u = to_[rev_[back]];
                ++it_[u];
                continue;
            }
            path_.push_back(e);
            u = to_[e];
        }
    }
};

// Per-thread scratch of the separator search.
struct Scratch {
    BandCut cut;
    std::vector<Index> ptr, adj;
    std::vector<char> src, snk, side;
};

// Parts are disjoint vertex sets, so the two sides of a separator are dissected
// concurrently (large parts only). Every per-vertex array is written only for the
// vertices of the part that owns them; labels of other parts may change while a
// part reads them, but never to its own label, so labels are relaxed atomics.
class Dissector {
public:
    Dissector(std::vector<std::vector<Index>>&& g, Index leaf)
        : g_(std::move(g)), leaf_(std::max<Index>(leaf, 8)), label_(g_.size()) {
        const Index m = static_cast<Index>(g_.size());
        for (auto& l : label_) l.store(0, std::memory_order_relaxed);
        level_.assign(static_cast<size_t>(m), kUnset);
        loc_.assign(static_cast<size_t>(m), kUnset);
    }

    std::vector<Index> run() {
        const Index m = static_cast<Index>(g_.size());
        std::vector<Index> all(static_cast<size_t>(m));
        std::iota(all.begin(), all.end(), 0);
        next_label_.store(1);
        Scratch sc;
        return dissect(std::move(all), 0, 0, sc);
    }

private:
    std::vector<std::vector<Index>> g_;
    Index leaf_;
    std::vector<std::atomic<Index>> label_;
    std::vector<Index> level_, loc_;
    std::atomic<Index> next_label_{0};

    Index lab_of(Index v) const { return label_[v].load(std::memory_order_relaxed); }
    void set_lab(Index v, Index l) { label_[v].store(l, std::memory_order_relaxed); }
    Index fresh() { return next_label_.fetch_add(1, std::memory_order_relaxed); }

    // Order of the part V (all labelled lab): its sub-parts, then its separator.
    std::vector<Index> dissect(std::vector<Index> V, Index lab, int depth, Scratch& sc) {
        std::vector<Index> out;
        out.reserve(V.size());
        if (static_cast<Index>(V.size()) <= leaf_) { order_min_degree(V, lab, out); return out; }
        std::vector<std::vector<Index>> comps = components(V, lab);
        if (comps.size() > 1) {
            V.clear();
            V.shrink_to_fit();
            for (auto& c : comps) {
                const Index cl = lab_of(c[0]);
                const std::vector<Index> o = dissect(std::move(c), cl, depth, sc);
                out.insert(out.end(), o.begin(), o.end());
            }
            return out;
        }
        lab = lab_of(V[0]);   // the single component's fresh label
        std::vector<Index> S, A, B;
        if (!separate(V, lab, S, A, B, sc)) { order_min_degree(V, lab, out); return out; }
        V.clear();
        V.shrink_to_fit();
        const Index la = fresh(), lb = fresh(), ls = fresh();
        for (Index v : A) set_lab(v, la);
        for (Index v : B) set_lab(v, lb);
        for (Index v : S) set_lab(v, ls);
        std::vector<Index> oa, ob;
        if (depth < kParallelDepth && static_cast<Index>(A.size() + B.size()) >= kParallelRows) {
            auto fa = std::async(std::launch::async, [&]() {
                Scratch s2;
                return dissect(std::move(A), la, depth + 1, s2);
            });
            ob = dissect(std::move(B), lb, depth + 1, sc);
            oa = fa.get();
        } else {
            oa = dissect(std::move(A), la, depth + 1, sc);
            ob = dissect(std::move(B), lb, depth + 1, sc);
        }
        out.insert(out.end(), oa.begin(), oa.end());
        out.insert(out.end(), ob.begin(), ob.end());
        order_min_degree(S, ls, out);
        return out;
    }

    // Connected components of the part; each gets a fresh label.
    std::vector<std::vector<Index>> components(const std::vector<Index>& V, Index lab) {
        std::vector<std::vector<Index>> comps;
        for (Index s : V) {
            if (lab_of(s) != lab) continue;
            const Index cl = fresh();
            std::vector<Index> c{s};
            set_lab(s, cl);
            for (size_t h = 0; h < c.size(); ++h)
                for (Index w : g_[c[h]])
                    if (lab_of(w) == lab) { set_lab(w, cl); c.push_back(w); }
            comps.push_back(std::move(c));
        }
        return comps;
    }

    // Breadth-first levels of the part from r; `order` lists the part by level and
    // start[k] is where level k begins (start has levels+1 entries).
    void bfs(Index r, Index lab, std::vector<Index>& order, std::vector<Index>& start) {
        order.clear();
        start.clear();
        order.push_back(r);
        level_[r] = 0;
        start.push_back(0);
        for (size_t h = 0; h < order.size(); ++h) {
            const Index u = order[h];
            if (static_cast<Index>(start.size()) - 1 < level_[u]) start.push_back(static_cast<Index>(h));
            for (Index w : g_[u])
                if (lab_of(w) == lab && level_[w] == kUnset) { level_[w] = level_[u] + 1; order.push_back(w); }
        }
        start.push_back(static_cast<Index>(order.size()));
        for (Index v : order) level_[v] = kUnset;
    }

    bool separate(const std::vector<Index>& V, Index lab, std::vector<Index>& S, std::vector<Index>& A,
                  std::vector<Index>& B, Scratch& sc) {
        const Index n = static_cast<Index>(V.size());
        std::vector<Index> order, start, order_v, start_v;
        // pseudo-peripheral pair: restart from a lowest-degree vertex of the last
        // level while the eccentricity grows
        Index r = V[0];
        for (Index v : V) if (g_[v].size() < g_[r].size()) r = v;
        Index ecc = -1;
        for (int it = 0; it < 8; ++it) {
            bfs(r, lab, order, start);
            const Index e = static_cast<Index>(start.size()) - 2;
            if (e <= ecc) break;
            ecc = e;
            Index best = order[start[e]];
            for (Index q = start[e]; q < start[e + 1]; ++q)
                if (g_[order[q]].size() < g_[best].size()) best = order[q];
            if (best == r) break;
            r = best;
        }
        bfs(r, lab, order, start);
        const Index e = static_cast<Index>(start.size()) - 2;
        if (e < 2) return false;
        Index far = order[start[e]];
        for (Index q = start[e]; q < start[e + 1]; ++q)
            if (g_[order[q]].size() < g_[far].size()) far = order[q];
        bfs(far, lab, order_v, start_v);
        const Index min_side = std::max<Index>(1, n / kMinSideDiv);
        struct Cand { std::vector<Index> a, s, b; };
        std::vector<Cand> cands;
        auto consider = [&](Cand&& c) {
            if (static_cast<Index>(std::min(c.a.size(), c.b.size())) >= min_side) cands.push_back(std::move(c));
        };
        // single levels of the first structure
        for (Index k = 1; k < e; ++k) {
            if (std::min(start[k], n - start[k + 1]) < min_side) continue;
            Cand c;
            c.a.assign(order.begin(), order.begin() + start[k]);
            c.s.assign(order.begin() + start[k], order.begin() + start[k + 1]);
            c.b.assign(order.begin() + start[k + 1], order.end());
            consider(std::move(c));
        }
        // minimum cuts between the balls of radius k around both ends of the pair,
        // from the largest radius at which the balls are apart downwards while the
        // cut stays balanced (smaller balls leave the cut more room)
        // (stops after kNoGain radii without a narrower cut)
        const Index ev = static_cast<Index>(start_v.size()) - 2;
        int no_gain = 0;
        int narrowest = -1;
        for (Index k = std::min(e, ev) / 2; k >= 0 && no_gain < kNoGain; --k) {
            Cand c;
            const int rc = ball_cut(order, order_v, start[k + 1], start_v[k + 1], lab, c.a, c.s, c.b, sc);
            if (rc < 0) continue;   // balls touch: shrink them
            if (static_cast<Index>(std::min(c.a.size(), c.b.size())) < min_side) break;
            if (narrowest < 0 || rc < narrowest) { narrowest = rc; no_gain = 0; } else ++no_gain;
            consider(std::move(c));
        }
        if (cands.empty()) return false;
        // the best balanced candidate among those at most 10% wider than the narrowest
        size_t narrow = cands[0].s.size();
        for (const auto& c : cands) narrow = std::min(narrow, c.s.size());
        size_t pick = cands.size(), bal = 0;
        for (size_t i = 0; i < cands.size(); ++i) {
            const size_t bl = std::min(cands[i].a.size(), cands[i].b.size());
            if (cands[i].s.size() * kSlackDen <= narrow * kSlackNum && (pick == cands.size() || bl > bal)) {
                pick = i;
                bal = bl;
            }
        }
        Cand& c = cands[pick];
        A.swap(c.a); S.swap(c.s); B.swap(c.b);
        return S.size() <= std::min(A.size(), B.size());
    }

    // X = the first nx vertices of order_u, Y = the first ny of order_v outside X;
    // the minimum vertex cut between them through the rest of the part. Returns -1
    // when X and Y touch (no cut exists), else the cut size.
    int ball_cut(const std::vector<Index>& order_u, const std::vector<Index>& order_v, Index nx, Index ny,
                  Index lab, std::vector<Index>& a_set, std::vector<Index>& s_set, std::vector<Index>& b_set,
                  Scratch& sc) {
        const Index n = static_cast<Index>(order_u.size());
        constexpr Index kX = -2, kY = -3;
        for (Index q = 0; q < nx; ++q) loc_[order_u[q]] = kX;
        Index taken = 0;
        for (Index q = 0; q < n && taken < ny; ++q)
            if (loc_[order_v[q]] != kX) { loc_[order_v[q]] = kY; ++taken; }
        bool adjacent = false;
        std::vector<Index> band;
        for (Index v : order_u) {
            if (loc_[v] == kY) { for (Index w : g_[v]) adjacent |= (lab_of(w) == lab && loc_[w] == kX); }
            else if (loc_[v] != kX) band.push_back(v);
        }
        const Index nb = static_cast<Index>(band.size());
        const bool ok = !adjacent && nb > 0;
        if (ok) {
            for (Index q = 0; q < nb; ++q) loc_[band[q]] = q;
            sc.ptr.assign(static_cast<size_t>(nb) + 1, 0);
            sc.adj.clear();
            sc.src.assign(static_cast<size_t>(nb), 0);
            sc.snk.assign(static_cast<size_t>(nb), 0);
            for (Index q = 0; q < nb; ++q) {
                for (Index w : g_[band[q]]) {
                    if (lab_of(w) != lab) continue;
                    if (loc_[w] == kX) sc.src[q] = 1;
                    else if (loc_[w] == kY) sc.snk[q] = 1;
                    else sc.adj.push_back(loc_[w]);
                }
                sc.ptr[q + 1] = static_cast<Index>(sc.adj.size());
            }
            sc.cut.run(nb, sc.ptr, sc.adj, sc.src, sc.snk, sc.side);
            a_set.clear(); s_set.clear(); b_set.clear();
            for (Index v : order_u) {
                const Index l = loc_[v];
                if (l == kX) a_set.push_back(v);
                else if (l == kY) b_set.push_back(v);
                else (sc.side[l] == 0 ? a_set : sc.side[l] == 1 ? s_set : b_set).push_back(v);
            }
        }
        for (Index v : order_u) loc_[v] = kUnset;
        return ok ? static_cast<int>(s_set.size()) : -1;
    }

    // Minimum degree on the part's induced graph; appends the part to out.
    void order_min_degree(const std::vector<Index>& V, Index lab, std::vector<Index>& out) {
        const Index n = static_cast<Index>(V.size());
        if (n == 0) return;
        for (Index q = 0; q < n; ++q) loc_[V[q]] = q;
        std::vector<std::vector<Index>> sub(static_cast<size_t>(n));
        for (Index q = 0; q < n; ++q) {
            for (Index w : g_[V[q]])
                if (lab_of(w) == lab) sub[q].push_back(loc_[w]);
            std::sort(sub[q].begin(), sub[q].end());
        }
        for (Index q = 0; q < n; ++q) loc_[V[q]] = kUnset;
        const std::vector<Index> p = min_degree_order(std::move(sub));
        for (Index q : p) {
            out.push_back(V[q]);
            set_lab(V[q], kUnset);
        }
    }
};

}  // namespace

std::vector<Index> nested_dissection_ordering(const core::CSRMatrix& A, Index leaf) {
    Dissector d(aat_graph(A), leaf);
    return d.run();
}

}  // namespace ipm
}  // namespace sankhya
