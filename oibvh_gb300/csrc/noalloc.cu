// oibvh_pair_detect_noalloc: collision detection for one mesh pair that
// allocates no memory at all, neither on the device nor pinned on the host.
//
// Who needs it: callers that must not allocate while they run. A physics or
// robotics step with a hard frame budget cannot afford cudaMalloc, which may
// synchronise the whole device and take an unbounded time; an application
// whose device memory is owned by an outside pool allocator (all of it
// reserved up front) may not create allocations of its own.
// oibvh_scene_detect grows its queues on demand; this entry point instead
// runs the same traversal kernels over a fixed scratch area that lives in
// this file.
//
// The scratch is a file-scope __device__ array: every GPU that loads the
// library holds it (kNoAllocBytes, about 4 MB) until the process exits. Host
// code cannot use the array's name as a device address, so the first call on
// a device (with that device current) resolves the address with
// cudaGetSymbolAddress and caches it together with the id of the device's
// context; make that first call at start-up. A later call in a
// new context (after cudaDeviceReset) resolves it again. Every call shares
// the one array: the counters are cleared at the start of each call, and
// calls whose GPU work overlaps (several host threads, or several streams)
// race on it and must be serialised by the caller.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/oibvh_gb300.h"
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh {

// Fixed capacity of each of the two traversal work lists (BVTT node pairs).
constexpr uint32_t kNoAllocItems = 1u << 18;
// Header: the two tree views, the pair view and the counters, rounded up.
constexpr size_t kNoAllocHeader = 4096;
constexpr size_t kNoAllocBytes = kNoAllocHeader + 2 * (size_t)kNoAllocItems * sizeof(uint64_t);

struct NoAllocHeader {
    TreeView trees[2];
    PairView pair;
    uint32_t counts[kCountTotal];
};
static_assert(sizeof(NoAllocHeader) <= kNoAllocHeader, "header fits");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Defined in host.cu: the device view of a tree handle.
int tree_device_view(oibvh_tree_t t, TreeView* out, int* device, bool* built);
int noalloc_fail(int code, const std::string& msg);

namespace {

std::mutex g_scratch_mu;
unsigned char* g_scratch_addr[64] = {};
unsigned long long g_scratch_ctx[64] = {};  // id of the context the address belongs to

// cuCtxGetId through the runtime's driver entry point (no link to libcuda).
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);

// Id of the current context (0 when it cannot be read).
unsigned long long current_context_id()
{
    static CtxGetIdFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (CtxGetIdFn) nullptr;
        return (CtxGetIdFn)f;
    }();
    unsigned long long id = 0;
    if (!fn || fn(nullptr, &id) != 0) return 0;
    return id;
}

// Device address of g_noalloc_scratch on `dev` (the current device, its
// context already initialised by the caller).
int scratch_address(int dev, unsigned char** out)
{
    if (dev < 0 || dev >= 64) return noalloc_fail(OIBVH_ERR_UNSUPPORTED, "device index above 63");
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev] || ctx != g_scratch_ctx[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return noalloc_fail(OIBVH_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = (unsigned char*)p;
        g_scratch_ctx[dev] = current_context_id();
    }
    *out = g_scratch_addr[dev];
    return OIBVH_OK;
}

#define NA_CUDA(expr)                                                                                   \
    do {                                                                                                \
        const cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) return noalloc_fail(OIBVH_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

}  // namespace

}  // namespace oibvh

using namespace oibvh;

extern "C" __attribute__((visibility("default"))) int oibvh_pair_detect_noalloc(
    oibvh_tree_t a, oibvh_tree_t b, uint32_t entry_level, uint32_t* d_out4, uint32_t out_cap, uint32_t* n_hits,
    void* stream)
{
    try {
        if (!a || !b || !n_hits) return noalloc_fail(OIBVH_ERR_ARG, "a, b or n_hits is NULL");
        if (out_cap && !d_out4) return noalloc_fail(OIBVH_ERR_ARG, "d_out4 is NULL");
        if (((uintptr_t)d_out4) % 16)
            return noalloc_fail(OIBVH_ERR_ARG, "d_out4 must be 16-byte aligned (the kernels store 16-byte records)");
        *n_hits = 0;
        NoAllocHeader h;
        std::memset(&h, 0, sizeof(h));
        int dev_a = -1, dev_b = -1;
        bool built_a = false, built_b = false;
        int st = tree_device_view(a, &h.trees[0], &dev_a, &built_a);
        if (st == OIBVH_OK) st = tree_device_view(b, &h.trees[1], &dev_b, &built_b);
        if (st != OIBVH_OK) return st;
        if (!built_a || !built_b) return noalloc_fail(OIBVH_ERR_STATE, "both trees must be built");
        if (dev_a != dev_b) return noalloc_fail(OIBVH_ERR_ARG, "the trees live on different devices");
        int cur = -1;
        NA_CUDA(cudaGetDevice(&cur));
        if (cur != dev_a) NA_CUDA(cudaSetDevice(dev_a));
        struct Restore {
            int d, c;
            ~Restore()
            {
                if (d != c) cudaSetDevice(c);
            }
        } restore{dev_a, cur};

        unsigned char* base = nullptr;
        st = scratch_address(dev_a, &base);
        if (st != OIBVH_OK) return st;

        // start level: the entry level, deepened to a ~2^16-pair cross product (as oibvh_scene_detect)
        const TreeShape& A = h.trees[0].shape;
        const TreeShape& B = h.trees[1].shape;
        const uint32_t start = entry_level > 8u ? entry_level : 8u;
        h.pair.a = 0;
        h.pair.b = 1;
        h.pair.ta = h.trees[0];
        h.pair.tb = h.trees[1];
        h.pair.front_off = 0;
        h.pair.entry_a = start < A.L ? start : A.L;
        h.pair.entry_b = start < B.L ? start : B.L;
        h.pair.front_cnt_a = A.level_count(h.pair.entry_a);
        h.pair.front_cnt_b = B.level_count(h.pair.entry_b);
        const uint64_t total0 = (uint64_t)h.pair.front_cnt_a * h.pair.front_cnt_b;
        if (total0 > (uint64_t)64 * kNoAllocItems)
            return noalloc_fail(OIBVH_ERR_ARG, "entry level " + std::to_string(entry_level) + " starts from " +
                                                   std::to_string(total0) + " node pairs; the fixed scratch allows " +
                                                   std::to_string((uint64_t)64 * kNoAllocItems));

        cudaStream_t s = (cudaStream_t)stream;
        NoAllocHeader* dh = (NoAllocHeader*)base;
        // header (views, pair, zeroed counters): the previous call's contents are overwritten
        NA_CUDA(cudaMemcpyAsync(dh, &h, sizeof(h), cudaMemcpyHostToDevice, s));

        DetectArgs args{};
        args.trees = dh->trees;
        args.pairs = &dh->pair;
        args.n_pairs = 1;
        args.expand_levels = 1;
        args.work[0] = (uint64_t*)(base + kNoAllocHeader);
        args.work[1] = args.work[0] + kNoAllocItems;
        args.work_cap = kNoAllocItems;
        args.hits = (uint4*)d_out4;
        args.hit_cap = out_cap;
        args.counts = dh->counts;
        args.fuse_narrow = 1;
        int sms = 1, per_sm = walk_blocks_per_sm();
        NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_a));
        args.grid = sms * per_sm;

        NA_CUDA(launch_init_front(args, (uint32_t)total0, s));
        NA_CUDA(launch_top(args, s));
        uint32_t counts[kCountTotal];
        uint32_t rounds = 1;
        for (;;) {
            const uint32_t upto = rounds == 1 ? 3u : rounds + 1;
            for (; rounds < upto && rounds < kMaxRounds; ++rounds) NA_CUDA(launch_walk(args, rounds, s));
            NA_CUDA(cudaMemcpyAsync(counts, dh->counts, sizeof(counts), cudaMemcpyDeviceToHost, s));
            NA_CUDA(cudaStreamSynchronize(s));
            if (counts[kCountFlags] || counts[kCountWork0 + rounds] == 0) break;
            if (rounds >= kMaxRounds) return noalloc_fail(OIBVH_ERR_OVERFLOW, "traversal needed too many rounds");
        }
        *n_hits = counts[kCountHits];
        if (counts[kCountFlags] & kFlagFrontOverflow)
            return noalloc_fail(OIBVH_ERR_OVERFLOW, "the pair needs more than " + std::to_string(kNoAllocItems) +
                                                        " queued node pairs, the fixed scratch; use oibvh_scene_detect");
        if (counts[kCountFlags] & kFlagHitOverflow)
            return noalloc_fail(OIBVH_ERR_OVERFLOW, "out_cap is too small: " + std::to_string(counts[kCountHits]) +
                                                        " colliding pairs (in *n_hits)");
        if (counts[kCountFlags]) return noalloc_fail(OIBVH_ERR_STATE, "unexpected device flag");
        return OIBVH_OK;
    } catch (...) {
        return noalloc_fail(OIBVH_ERR_CUDA, "unexpected C++ exception");
    }
}
