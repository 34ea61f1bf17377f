// Shared device-side helpers: error checks, a bump arena for device memory,
// warp / block reductions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "api/sk_error.hpp"
#include "sankhya/sk_ipm.h"

#define SK_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            throw ::sankhya::api::sk_exception(                                                    \
                (e_ == cudaErrorMemoryAllocation) ? SK_ERR_ALLOC : SK_ERR_CUDA,                    \
                std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " + __FILE__ + ":" +   \
                    std::to_string(__LINE__));                                                     \
    } while (0)

namespace sankhya {
namespace dev {

// One cudaMalloc per owner, carved into 256-byte aligned pieces. Replaces the
// reference's first-fit VRAMArena (src/gpu/vram_arena.cu:27-153): sizes are all
// known after the symbolic phase, so a single reservation with no free list and
// no per-allocation memset is enough.
class Arena {
public:
    Arena() = default;
    ~Arena() { release(); }
    Arena(const Arena&) = delete;
    Arena& operator=(const Arena&) = delete;

    // Phase 1: reserve sizes; phase 2: commit() allocates; pointers are then valid.
    size_t reserve(size_t bytes) {
        const size_t off = size_;
        size_ += (bytes + 255) & ~size_t(255);
        return off;
    }
    void commit() {
        release();
        if (size_ == 0) size_ = 256;
        SK_CUDA(cudaMalloc(&base_, size_));
    }
    template <class T>
    T* at(size_t off) const { return reinterpret_cast<T*>(static_cast<char*>(base_) + off); }
    size_t size() const { return size_; }
    void release() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
    }
    void reset() { release(); size_ = 0; }

private:
    void* base_ = nullptr;
    size_t size_ = 0;
};

template <class T>
struct Slot {       // typed handle into an Arena
    size_t off = 0;
    size_t count = 0;
    T* ptr = nullptr;
};

template <class T>
void reserve(Arena& a, Slot<T>& s, size_t count) {
    s.count = count;
    s.off = a.reserve(sizeof(T) * (count ? count : 1));
}

template <class T>
void bind(Arena& a, Slot<T>& s) { s.ptr = a.at<T>(s.off); }

template <class T>
void upload(Slot<T>& s, const std::vector<T>& v, cudaStream_t st) {
    if (!v.empty()) SK_CUDA(cudaMemcpyAsync(s.ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
}

#ifdef __CUDACC__
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
#endif

}  // namespace dev
}  // namespace sankhya
