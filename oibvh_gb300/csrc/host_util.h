// Host-side helpers shared by the library's translation units: error
// reporting, checked CUDA calls, device/pinned buffers, and the tree object.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/oibvh_gb300.h"
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh_host {

// Last error message of the calling thread (oibvh_last_error).
extern thread_local std::string g_last_error;

// Allocation-failure injection (oibvh_debug_fail_alloc_after): -1 = off;
// n >= 0: the allocation attempt n places ahead (0 = the next one) reports
// cudaErrorMemoryAllocation without calling CUDA, then the hook is off again.
extern std::atomic<int64_t> g_fail_alloc;
extern std::atomic<uint64_t> g_alloc_attempts;  // device + pinned allocation attempts
inline bool injected_alloc_failure()
{
    g_alloc_attempts.fetch_add(1, std::memory_order_relaxed);
    int64_t c = g_fail_alloc.load(std::memory_order_relaxed);
    while (c >= 0)
        if (g_fail_alloc.compare_exchange_weak(c, c - 1, std::memory_order_relaxed)) return c == 0;
    return false;
}

inline int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

inline int cuda_fail(cudaError_t e, const char* what)
{
    const int code = (e == cudaErrorMemoryAllocation) ? OIBVH_ERR_OOM : OIBVH_ERR_CUDA;
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return code;
}

#define CUDA_TRY(expr)                                   \
    do {                                                 \
        cudaError_t _e = (expr);                         \
        if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
    } while (0)

#define OK_TRY(expr)              \
    do {                          \
        int _s = (expr);          \
        if (_s != OIBVH_OK) return _s; \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

inline int sm_count(int dev)
{
    static int cache[64] = {};
    if (dev >= 0 && dev < 64 && cache[dev]) return cache[dev];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    if (dev >= 0 && dev < 64) cache[dev] = n;
    return n;
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // grow to at least `want` elements; contents are not kept
    int ensure(size_t want, const char* what)
    {
        if (want <= n && p) return OIBVH_OK;
        release();
        if (want == 0) want = 1;
        cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation : cudaMalloc(&p, want * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return cuda_fail(e, what);
        }
        n = want;
        return OIBVH_OK;
    }
    // grow keeping the first `keep` elements (stream-ordered copy)
    int grow_keep(size_t want, size_t keep, cudaStream_t s, const char* what)
    {
        if (want <= n && p) return OIBVH_OK;
        T* q = nullptr;
        cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation : cudaMalloc(&q, want * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cuda_fail(e, what);
        }
        if (p && keep) {
            e = cudaMemcpyAsync(q, p, std::min(keep, n) * sizeof(T), cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) {
                cudaFree(q);
                return cuda_fail(e, what);
            }
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                cudaFree(q);
                return cuda_fail(e, what);
            }
        }
        release();
        p = q;
        n = want;
        return OIBVH_OK;
    }
};

template <class T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf()
    {
        if (p) cudaFreeHost(p);
    }
    int ensure(size_t want, const char* what)
    {
        if (want <= n && p) return OIBVH_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (want == 0) want = 1;
        cudaError_t e = injected_alloc_failure() ? cudaErrorMemoryAllocation : cudaMallocHost(&p, want * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return cuda_fail(e, what);
        }
        n = want;
        return OIBVH_OK;
    }
};

}  // namespace oibvh_host

using namespace oibvh_host;
using namespace oibvh;

// ============================================================================
// Tree
// ============================================================================
struct oibvh_tree_s {
    int device = 0;
    uint32_t nV = 0, nT = 0;
    TreeShape shape{};
    DevBuf<float> xyz;          // staging for positions given as xyz (3 * nV)
    DevBuf<float4> pos4;        // positions in the device layout (x, y, z, 0), in the tree's vertex order
    const float4* cur_pos = nullptr;  // positions the refit and detect read (pos4)
    const float4* borrowed = nullptr; // caller's (x, y, z, w) positions, caller's order: copied into pos4 before each refit
    DevBuf<uint32_t> vperm;     // tree vertex v is the caller's vertex vperm[v] (set by the first build)
    bool reordered = false;     // vperm holds the map (before the first build: the caller's order)
    DevBuf<uint32_t> tri;       // faces (3 * nT) in the tree's vertex numbering
    DevBuf<uint4> face;         // Morton-ordered faces (v0, v1, v2, original index)
    DevBuf<float4> box;         // 2 * (size - nT): internal nodes only
    DevBuf<uint32_t> counters;  // refit climbing counters
    bool built = false;
    uint32_t morton_bits = 30;  // 30 (the reference's key) or 63 (21 bits per axis)

    const uint32_t* vmap() const { return reordered ? vperm.p : nullptr; }

    RefitJob job() const
    {
        RefitJob j{};
        j.box = box.p;
        j.face = face.p;
        j.pos = cur_pos;
        j.shape = shape;
        j.block_begin = 0;
        j.n_blocks = refit_blocks_for(nT);
        j.counters = counters.p;
        return j;
    }
};

