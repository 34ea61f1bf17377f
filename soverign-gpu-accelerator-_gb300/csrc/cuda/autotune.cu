// SpMV launch-shape autotuner (see autotune.hpp).
#include "cuda/autotune.hpp"

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "cuda/dev_common.cuh"
#include "cuda/spmv.cuh"

namespace sankhya {
namespace dev {

namespace {

using Key = std::tuple<int, int, int, int64_t>;   // device, rows, cols, nnz

std::mutex& table_mutex() {
    static std::mutex m;
    return m;
}
std::map<Key, SpmvTuning>& table() {
    static std::map<Key, SpmvTuning> t;
    return t;
}

int current_device() {
    int d = 0;
    SK_CUDA(cudaGetDevice(&d));
    return d;
}

// Owns the two events of the timing loop so that an exception frees them.
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        SK_CUDA(cudaEventCreate(&a));
        SK_CUDA(cudaEventCreate(&b));
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

}  // namespace

int spmv_heuristic_group(int64_t nnz, int rows) {
    const double avg = rows > 0 ? static_cast<double>(nnz) / rows : 0.0;
    if (avg <= 3) return 2;
    if (avg <= 6) return 4;
    if (avg <= 12) return 8;
    if (avg <= 24) return 16;
    return 32;
}

void spmv_axpby(int rows, int group, const int* rp, const int* ci, const double* v, const double* x, double alpha,
                double beta, double* y, cudaStream_t st) {
    spmv(rows, group, rp, ci, v, x, EpiAxpby{alpha, beta, y}, st);
    SK_CUDA(cudaGetLastError());
}

int spmv_tuned_group(int rows, int cols, int64_t nnz) {
    const Key key{current_device(), rows, cols, nnz};
    std::lock_guard<std::mutex> lk(table_mutex());
    auto it = table().find(key);
    return it != table().end() ? it->second.group : spmv_heuristic_group(nnz, rows);
}

SpmvTuning spmv_tune(int rows, int cols, int64_t nnz, const int* rp, const int* ci, const double* v,
                     const double* x, double* y, cudaStream_t st, bool use_cache, int reps) {
    const Key key{current_device(), rows, cols, nnz};
    if (use_cache) {
        std::lock_guard<std::mutex> lk(table_mutex());
        auto it = table().find(key);
        if (it != table().end()) {
            SpmvTuning t = it->second;
            t.from_cache = true;
            return t;
        }
    }
    SpmvTuning t;
    t.heuristic = spmv_heuristic_group(nnz, rows);
    t.group = t.heuristic;
    if (rows <= 0 || nnz <= 0) return t;
    reps = std::max(1, reps);
    EventPair ev;
    double best = 0.0, heur_ms = 0.0;
    int best_g = t.heuristic;
    for (int k = 0; k < kSpmvNumGroups; ++k) {
        const int g = kSpmvGroups[k];
        spmv_axpby(rows, g, rp, ci, v, x, 1.0, 0.0, y, st);     // warm-up
        float fastest = 0.0f;
        for (int r = 0; r < reps; ++r) {
            SK_CUDA(cudaEventRecord(ev.a, st));
            spmv_axpby(rows, g, rp, ci, v, x, 1.0, 0.0, y, st);
            SK_CUDA(cudaEventRecord(ev.b, st));
            SK_CUDA(cudaEventSynchronize(ev.b));
            float ms = 0.0f;
            SK_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            fastest = r == 0 ? ms : std::min(fastest, ms);
        }
        t.ms[k] = fastest;
        if (g == t.heuristic) heur_ms = fastest;
        if (k == 0 || fastest < best) {
            best = fastest;
            best_g = g;
        }
    }
    t.group = (best < 0.97 * heur_ms) ? best_g : t.heuristic;
    std::lock_guard<std::mutex> lk(table_mutex());
    if (!use_cache) {             // an explicit re-tune replaces the kept width
        table()[key] = t;
        return t;
    }
    auto ins = table().emplace(key, t);
    if (!ins.second) {            // another thread tuned the same shape first: keep its choice
        SpmvTuning kept = ins.first->second;
        kept.from_cache = true;
        return kept;
    }
    return t;
}

}  // namespace dev
}  // namespace sankhya
