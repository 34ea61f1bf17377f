// SpMV launch-shape autotuner (see autotune.hpp).
#include "cuda/autotune.hpp"

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

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

// Column range of each row ({INT_MAX, -1} for an empty row).
__global__ void k_row_span(int rows, const int* __restrict__ rp, const int* __restrict__ ci, int2* __restrict__ span) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int lo = 0x7fffffff, hi = -1;
    for (int q = rp[r]; q < rp[r + 1]; ++q) {
        lo = min(lo, ci[q]);
        hi = max(hi, ci[q]);
    }
    span[r] = make_int2(lo, hi);
}

}  // namespace

SpmvWindows::~SpmvWindows() {
    if (d_chunks_) cudaFree(d_chunks_);
}

void SpmvWindows::build(int rows, const int* rp, const int* ci, cudaStream_t st, int64_t target_nnz) {
    if (d_chunks_) {
        SK_CUDA(cudaFree(d_chunks_));
        d_chunks_ = nullptr;
    }
    nchunks_ = 0;
    max_cols_ = 0;
    staged_ = 0.0;
    if (rows <= 0) return;
    int2* d_span = nullptr;
    SK_CUDA(cudaMalloc(&d_span, sizeof(int2) * static_cast<size_t>(rows)));
    std::vector<int2> span(static_cast<size_t>(rows));
    std::vector<int> hrp(static_cast<size_t>(rows) + 1);
    try {
        k_row_span<<<(rows + 255) / 256, 256, 0, st>>>(rows, rp, ci, d_span);
        SK_CUDA(cudaGetLastError());
        SK_CUDA(cudaMemcpyAsync(span.data(), d_span, sizeof(int2) * span.size(), cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaMemcpyAsync(hrp.data(), rp, sizeof(int) * hrp.size(), cudaMemcpyDeviceToHost, st));
        SK_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        cudaFree(d_span);
        throw;
    }
    SK_CUDA(cudaFree(d_span));
    // greedy cut in row order: a chunk grows while its column window stays within
    // kWinMaxCols and its entries within target_nnz; rows wider than any window
    // are grouped into global-gather chunks of at most target_nnz entries
    std::vector<int4> ch;
    int64_t staged_nnz = 0;
    const int64_t total = hrp[rows] - hrp[0];
    auto wide = [&](int r) { return span[r].y >= 0 && span[r].y - span[r].x + 1 > kWinMaxCols; };
    int r = 0;
    while (r < rows) {
        const int r0 = r;
        int64_t nz = 0;
        if (wide(r)) {
            while (r < rows && wide(r) && (r == r0 || nz + (hrp[r + 1] - hrp[r]) <= target_nnz)) {
                nz += hrp[r + 1] - hrp[r];
                ++r;
            }
            ch.push_back(make_int4(r0, r, 0, -1));
            continue;
        }
        int lo = 0x7fffffff, hi = -1;
        while (r < rows && !wide(r)) {
            const int len = hrp[r + 1] - hrp[r];
            const int nlo = std::min(lo, span[r].x), nhi = std::max(hi, span[r].y);
            if (r > r0 && ((nhi >= 0 && nhi - nlo + 1 > kWinMaxCols) || nz + len > target_nnz)) break;
            lo = nlo;
            hi = nhi;
            nz += len;
            ++r;
        }
        const int ncols = hi >= 0 ? hi - lo + 1 : 0;
        ch.push_back(make_int4(r0, r, hi >= 0 ? lo : 0, ncols));
        max_cols_ = std::max(max_cols_, ncols);
        staged_nnz += nz;
    }
    staged_ = total > 0 ? static_cast<double>(staged_nnz) / total : 0.0;
    nchunks_ = static_cast<int>(ch.size());
    SK_CUDA(cudaMalloc(&d_chunks_, sizeof(int4) * ch.size()));
    SK_CUDA(cudaMemcpyAsync(d_chunks_, ch.data(), sizeof(int4) * ch.size(), cudaMemcpyHostToDevice, st));
    SK_CUDA(cudaStreamSynchronize(st));
}

SpmvShape SpmvWindows::shape(int group, bool windowed) const {
    SpmvShape sh;
    sh.group = group;
    sh.windowed = windowed && d_chunks_ != nullptr;
    sh.chunks = d_chunks_;
    sh.nchunks = nchunks_;
    sh.max_cols = max_cols_;
    return sh;
}

int spmv_heuristic_group(int64_t nnz, int rows) {
    const double avg = rows > 0 ? static_cast<double>(nnz) / rows : 0.0;
    if (avg <= 3) return 2;
    if (avg <= 6) return 4;
    if (avg <= 12) return 8;
    if (avg <= 24) return 16;
    return 32;
}

void spmv_axpby(int rows, const SpmvShape& shape, const int* rp, const int* ci, const double* v, const double* x,
                double alpha, double beta, double* y, cudaStream_t st) {
    spmv(rows, shape, rp, ci, v, x, EpiAxpby{alpha, beta, y}, st);
    SK_CUDA(cudaGetLastError());
}

int spmv_tuned_group(int rows, int cols, int64_t nnz) {
    const Key key{current_device(), rows, cols, nnz};
    std::lock_guard<std::mutex> lk(table_mutex());
    auto it = table().find(key);
    return it != table().end() ? it->second.group : spmv_heuristic_group(nnz, rows);
}

SpmvTuning spmv_tune(int rows, int cols, int64_t nnz, const int* rp, const int* ci, const double* v,
                     const double* x, double* y, cudaStream_t st, const SpmvWindows* win, bool use_cache, int reps) {
    const Key key{current_device(), rows, cols, nnz};
    if (use_cache) {
        std::lock_guard<std::mutex> lk(table_mutex());
        auto it = table().find(key);
        if (it != table().end()) {
            SpmvTuning t = it->second;
            t.from_cache = true;
            if (!win) t.windowed = false;
            return t;
        }
    }
    SpmvTuning t;
    t.heuristic = spmv_heuristic_group(nnz, rows);
    t.group = t.heuristic;
    if (rows <= 0 || nnz <= 0) return t;
    reps = std::max(1, reps);
    const bool try_win = win && win->chunks() > 0 && win->staged_fraction() >= 0.5;
    EventPair ev;
    double best = 0.0, heur_ms = 0.0;
    int best_g = t.heuristic;
    bool best_w = false, first = true;
    for (int w = 0; w < (try_win ? 2 : 1); ++w) {
        for (int k = 0; k < kSpmvNumGroups; ++k) {
            const int g = kSpmvGroups[k];
            SpmvShape sh = w ? win->shape(g, true) : SpmvShape{};
            sh.group = g;
            spmv_axpby(rows, sh, rp, ci, v, x, 1.0, 0.0, y, st);     // warm-up
            float fastest = 0.0f;
            for (int r = 0; r < reps; ++r) {
                SK_CUDA(cudaEventRecord(ev.a, st));
                spmv_axpby(rows, sh, rp, ci, v, x, 1.0, 0.0, y, st);
                SK_CUDA(cudaEventRecord(ev.b, st));
                SK_CUDA(cudaEventSynchronize(ev.b));
                float ms = 0.0f;
                SK_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
                fastest = r == 0 ? ms : std::min(fastest, ms);
            }
            (w ? t.ms_win : t.ms)[k] = fastest;
            if (!w && g == t.heuristic) heur_ms = fastest;
            if (first || fastest < best) {
                best = fastest;
                best_g = g;
                best_w = w != 0;
                first = false;
            }
        }
    }
    if (best < 0.97 * heur_ms) {
        t.group = best_g;
        t.windowed = best_w;
    }
    std::lock_guard<std::mutex> lk(table_mutex());
    if (!use_cache) {             // an explicit re-tune replaces the kept choice
        table()[key] = t;
        return t;
    }
    auto ins = table().emplace(key, t);
    if (!ins.second) {            // another thread tuned the same shape first: keep its choice
        SpmvTuning kept = ins.first->second;
        kept.from_cache = true;
        if (!win) kept.windowed = false;
        return kept;
    }
    return t;
}

}  // namespace dev
}  // namespace sankhya
