// Serving: a request loop over a pool of device-resident meshes with
// continuous batching. This has no counterpart in the reference, whose
// Scene detects one fixed set of meshes per call (src/cuda/scene.cu:157-185);
// it reuses the reference's per-query steps (Mesh::transform +
// OibvhTree::refit + Scene::detectCollision) on the library's kernels.
//
// A query names two pool meshes A and B and a rigid transform M of B. On
// admission it gets a slot in a fixed device arena (the memory budget): B's
// transformed positions and B's tree boxes, refit in place; A is read at
// rest from the pool. The loop runs on its own host thread:
//
//   * arrivals queue FIFO; whenever a lane (a CUDA stream with its own work
//     lists) is idle and queries are waiting, all waiting queries whose slots
//     fit in the arena (up to max_batch) form a batch and are launched at
//     once: one transform launch for all slots, one refit launch for all
//     slots, one detect (start front, top walk, walk rounds) for all pairs,
//     and the counters copied back; so queries that arrive while earlier
//     batches are on the GPU are admitted as lanes and memory free up, and
//     batches on different lanes overlap on the device;
//   * the batch's hits are grouped by query on the device; it completes in
//     two stream-ordered steps (counters and per-query offsets, then exactly
//     the grouped pairs, 8 B each) tracked by events, each query's pairs then
//     one block copy on the host; the loop never waits on the device while
//     other work can be launched;
//   * a batch whose queues were too small (flags, or spill beyond the
//     launched walk rounds) is redone on its lane with larger queues, so
//     results are never truncated.
//
// A query's pair set does not depend on what it was batched with: the
// traversal and the triangle test of a pair read only that pair's trees.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host_util.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr size_t kArenaAlign = 256;
static_assert(kArenaAlign % 32 == 0, "node arrays in the arena must be 32-byte aligned (256-bit node loads)");
constexpr uint32_t kServeWalkRoundsInit = 8;

size_t align_up(size_t x) { return (x + kArenaAlign - 1) / kArenaAlign * kArenaAlign; }

// First-fit allocator over the arena's byte range (host-side bookkeeping).
struct Arena {
    std::map<size_t, size_t> free_blocks;  // offset -> size
    size_t size = 0, used = 0, peak = 0;

    void reset(size_t n)
    {
        free_blocks.clear();
        free_blocks[0] = n;
        size = n;
        used = peak = 0;
    }
    bool alloc(size_t bytes, size_t& off)
    {
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            const size_t rest = it->second - bytes;
            free_blocks.erase(it);
            if (rest) free_blocks[off + bytes] = rest;
            used += bytes;
            peak = std::max(peak, used);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        used -= bytes;
        auto it = free_blocks.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_blocks.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_blocks.erase(next);
        }
        if (it != free_blocks.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_blocks.erase(it);
            }
        }
    }
};

struct Query {
    uint64_t ticket = 0;
    uint32_t a = 0, b = 0;
    float mat[12] = {};
    Clock::time_point t_submit, t_launch, t_done;
    int status = OIBVH_QUERY_QUEUED;
    int error = OIBVH_OK;
    std::string message;
    size_t slot_off = 0, slot_bytes = 0;
    float4* pos = nullptr;  // B transformed (slot)
    float4* box = nullptr;  // B's internal nodes (slot)
    std::vector<uint32_t> pairs;  // (triA, triB), original face indices
    uint32_t lane = 0, batch_size = 0;
};

struct Lane {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    int phase = 0;  // 0 idle, 1 detect in flight, 2 hit copy in flight
    std::vector<Query*> batch;
    PinnedBuf<TreeView> h_views;
    DevBuf<TreeView> views;
    PinnedBuf<PairView> h_pairs;
    DevBuf<PairView> pairv;
    PinnedBuf<BuildJob> h_jobs;
    DevBuf<BuildJob> jobs;
    PinnedBuf<RefitJob> h_rjobs;
    DevBuf<RefitJob> rjobs;
    PinnedBuf<float> h_mats;
    DevBuf<float> mats;
    DevBuf<uint32_t> rcount;
    DevBuf<uint64_t> front0, front1;
    DevBuf<uint4> hits;
    DevBuf<uint32_t> counts;
    PinnedBuf<uint32_t> h_counts;
    DevBuf<uint32_t> qcount, qcursor, qoff;  // per query of the batch: hit count, scatter cursor, offset
    PinnedBuf<uint32_t> h_qoff;
    DevBuf<uint2> out;     // the batch's (triA, triB) grouped by query
    PinnedBuf<uint2> h_out;
    uint32_t front_cap = 0, hit_cap = 0;  // set from the server's capacities at the first batch
    uint32_t cap_gen = ~0u;  // queue capacities follow the server's settings of this generation
    uint32_t rounds = kServeWalkRoundsInit;
    uint64_t front0_count = 0;
    uint32_t n_pairs = 0;
    uint64_t n_hits = 0;

    ~Lane()
    {
        if (ev) cudaEventDestroy(ev);
        if (st) cudaStreamDestroy(st);
    }
};

// Staging buffers grow to powers of two: allocating (cudaMallocHost,
// cudaMalloc/cudaFree) stalls the device, so it must stay rare in the loop.
template <class Buf>
int ensure_pow2(Buf& b, size_t want, const char* what)
{
    size_t n = 64;
    while (n < want) n <<= 1;
    return b.ensure(n, what);
}

uint32_t grow(uint64_t need, uint32_t cur)
{
    uint64_t c = std::max<uint64_t>(need + need / 4 + 1024, (uint64_t)cur * 2);
    return (uint32_t)std::min<uint64_t>(c, 0x7fffffffull);
}

// A batch's hit records {view a = 2i, view b = 2i + 1, triA, triB} grouped
// by query i on the device, so that the host takes each query's pairs as one
// block (a copy) instead of sorting every record into its query: count per
// query, exclusive scan, scatter of the (triA, triB) words. Lanes of a warp
// on the same query combine their atomics (__match_any_sync). The order of
// pairs within a query is not specified.
constexpr uint32_t kNoQuery = 0xffffffffu;
__global__ void k_bucket_count(const uint4* __restrict__ hits, const uint32_t* __restrict__ counts, uint32_t hit_cap,
                               uint32_t* __restrict__ qcount)
{
    const uint32_t n = min(counts[kCountHits], hit_cap);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t k = base + lane;
        const uint32_t q = k < n ? __ldg(&hits[k].x) >> 1 : kNoQuery;
        const uint32_t peers = __match_any_sync(0xffffffffu, q);
        if (q != kNoQuery && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(qcount + q, (uint32_t)__popc(peers));
    }
}
// One block: qoff[i] = sum of qcount[0..i), qoff[n] = the total; cursor = qoff.
__global__ void __launch_bounds__(1024) k_bucket_scan(const uint32_t* __restrict__ qcount, uint32_t n,
                                                      uint32_t* __restrict__ qoff, uint32_t* __restrict__ cursor)
{
    __shared__ uint32_t warp_sum[32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t b = min(n, threadIdx.x * per), e = min(n, b + per);
    uint32_t mine = 0;
    for (uint32_t i = b; i < e; ++i) mine += qcount[i];
    uint32_t x = mine;  // inclusive scan within the warp
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < n_warps ? warp_sum[lane] : 0u;
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        warp_sum[lane] = v;  // inclusive over warps
    }
    __syncthreads();
    uint32_t run = x - mine + (warp ? warp_sum[warp - 1] : 0u);
    for (uint32_t i = b; i < e; ++i) {
        qoff[i] = run;
        cursor[i] = run;
        run += qcount[i];
    }
    if (threadIdx.x == 0) qoff[n] = warp_sum[n_warps - 1];
}
__global__ void k_bucket_scatter(const uint4* __restrict__ hits, const uint32_t* __restrict__ counts, uint32_t hit_cap,
                                 uint32_t* __restrict__ cursor, uint2* __restrict__ out)
{
    const uint32_t n = min(counts[kCountHits], hit_cap);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t k = base + lane;
        const uint4 h = k < n ? hits[k] : make_uint4(0, 0, 0, 0);
        const uint32_t q = k < n ? h.x >> 1 : kNoQuery;
        const uint32_t peers = __match_any_sync(0xffffffffu, q);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t pos = 0;
        if (q != kNoQuery && lane == leader) pos = atomicAdd(cursor + q, (uint32_t)__popc(peers));
        pos = __shfl_sync(0xffffffffu, pos, leader) + __popc(peers & ((1u << lane) - 1u));
        if (q != kNoQuery) out[pos] = make_uint2(h.z, h.w);
    }
}
constexpr uint32_t kBucketThreads = 256;

}  // namespace

struct oibvh_server_s {
    int device = 0;
    uint64_t budget = 0;
    uint32_t max_batch = 0;
    uint32_t entry_level = 4;
    uint32_t start_log2 = 16;
    // lane queue capacities: generous from the start (a regrowth redoes a
    // batch synchronously), and shared: a lane that had to grow raises them
    // for every lane before its next batch
    uint32_t init_front_cap = 1u << 22, init_hit_cap = 1u << 21, cap_gen = 0;
    uint64_t max_batch_cost = 32ull << 20;  // triangles (A + B) per batch, 0 = no limit
    std::vector<oibvh_tree_t> pool;
    DevBuf<uint8_t> arena_mem;
    Arena arena;
    std::vector<std::unique_ptr<Lane>> lanes;

    std::mutex mu;
    std::condition_variable cv_submit, cv_done;
    std::deque<Query*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Query>> queries;
    uint64_t next_ticket = 1;
    bool running = false, stop = false;
    std::thread worker;
    oibvh_server_stats stats{};

    ~oibvh_server_s();
    void loop();
    int reserve_lanes();
    int launch(Lane& L, std::vector<Query*>& batch);
    int enqueue_detect(Lane& L);
    int advance(Lane& L);
    void finish(Lane& L, int status, const std::string& msg);
    size_t slot_bytes(uint32_t b) const
    {
        const oibvh_tree_t t = pool[b];
        return align_up((size_t)t->nV * sizeof(float4)) +
               align_up(2 * (size_t)std::max(1u, t->shape.size - t->nT) * sizeof(float4));
    }
};

oibvh_server_s::~oibvh_server_s()
{
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
    }
    cv_submit.notify_all();
    if (worker.joinable()) worker.join();
}

// Every lane's staging tables (for max_batch queries), work lists, hit
// queue and its pinned copy, allocated before the loop starts: a lane's first
// batch, or the first batch larger than any before it, would otherwise
// allocate in the loop (pinned host memory and cudaFree stall every lane for
// milliseconds). Only a redo with larger queues allocates afterwards.
int oibvh_server_s::reserve_lanes()
{
    const uint32_t per = refit_counters_per_tree();
    const size_t n = max_batch;
    for (auto& Lp : lanes) {
        Lane& L = *Lp;
        OK_TRY(ensure_pow2(L.h_views, 2 * n, "cudaMallocHost(views)"));
        OK_TRY(ensure_pow2(L.views, 2 * n, "cudaMalloc(views)"));
        OK_TRY(ensure_pow2(L.h_pairs, n, "cudaMallocHost(pairs)"));
        OK_TRY(ensure_pow2(L.pairv, n, "cudaMalloc(pairs)"));
        OK_TRY(ensure_pow2(L.h_jobs, n, "cudaMallocHost(jobs)"));
        OK_TRY(ensure_pow2(L.jobs, n, "cudaMalloc(jobs)"));
        OK_TRY(ensure_pow2(L.h_rjobs, n, "cudaMallocHost(refit jobs)"));
        OK_TRY(ensure_pow2(L.rjobs, n, "cudaMalloc(refit jobs)"));
        OK_TRY(ensure_pow2(L.h_mats, 12 * n, "cudaMallocHost(matrices)"));
        OK_TRY(ensure_pow2(L.mats, 12 * n, "cudaMalloc(matrices)"));
        OK_TRY(ensure_pow2(L.rcount, (size_t)per * n, "cudaMalloc(refit counters)"));
        OK_TRY(L.counts.ensure(kCountTotal, "cudaMalloc(counts)"));
        OK_TRY(L.h_counts.ensure(kCountTotal, "cudaMallocHost(counts)"));
        L.front_cap = init_front_cap;
        L.hit_cap = init_hit_cap;
        L.cap_gen = cap_gen;
        OK_TRY(L.front0.ensure(L.front_cap, "cudaMalloc(work list)"));
        OK_TRY(L.front1.ensure(L.front_cap, "cudaMalloc(work list)"));
        OK_TRY(L.hits.ensure(L.hit_cap, "cudaMalloc(hits)"));
        OK_TRY(L.qcount.ensure(n + 1, "cudaMalloc(query counts)"));
        OK_TRY(L.qcursor.ensure(n + 1, "cudaMalloc(query cursors)"));
        OK_TRY(L.qoff.ensure(n + 1, "cudaMalloc(query offsets)"));
        OK_TRY(L.h_qoff.ensure(n + 1, "cudaMallocHost(query offsets)"));
        OK_TRY(L.out.ensure(L.hit_cap, "cudaMalloc(grouped pairs)"));
        OK_TRY(ensure_pow2(L.h_out, L.hit_cap, "cudaMallocHost(grouped pairs)"));
    }
    return OIBVH_OK;
}

// One batch: tables, transform, refit, then the detect.
int oibvh_server_s::launch(Lane& L, std::vector<Query*>& batch)
{
    const uint32_t n = (uint32_t)batch.size();
    const uint32_t per = refit_counters_per_tree();
    OK_TRY(ensure_pow2(L.h_views, 2 * n, "cudaMallocHost(views)"));
    OK_TRY(ensure_pow2(L.views, 2 * n, "cudaMalloc(views)"));
    OK_TRY(ensure_pow2(L.h_pairs, n, "cudaMallocHost(pairs)"));
    OK_TRY(ensure_pow2(L.pairv, n, "cudaMalloc(pairs)"));
    OK_TRY(ensure_pow2(L.h_jobs, n, "cudaMallocHost(jobs)"));
    OK_TRY(ensure_pow2(L.jobs, n, "cudaMalloc(jobs)"));
    OK_TRY(ensure_pow2(L.h_rjobs, n, "cudaMallocHost(refit jobs)"));
    OK_TRY(ensure_pow2(L.rjobs, n, "cudaMalloc(refit jobs)"));
    OK_TRY(ensure_pow2(L.h_mats, 12 * (size_t)n, "cudaMallocHost(matrices)"));
    OK_TRY(ensure_pow2(L.mats, 12 * (size_t)n, "cudaMalloc(matrices)"));
    OK_TRY(ensure_pow2(L.rcount, (size_t)per * n, "cudaMalloc(refit counters)"));
    OK_TRY(L.counts.ensure(kCountTotal, "cudaMalloc(counts)"));
    OK_TRY(L.h_counts.ensure(kCountTotal, "cudaMallocHost(counts)"));
    OK_TRY(L.qcount.ensure((size_t)n + 1, "cudaMalloc(query counts)"));
    OK_TRY(L.qcursor.ensure((size_t)n + 1, "cudaMalloc(query cursors)"));
    OK_TRY(L.qoff.ensure((size_t)n + 1, "cudaMalloc(query offsets)"));
    OK_TRY(L.h_qoff.ensure((size_t)n + 1, "cudaMallocHost(query offsets)"));

    // start level: the entry level, deepened so the batch's start cross
    // product holds about 2^start_log2 node pairs
    const uint32_t lg = ilog2(std::max(1u, n));
    const uint32_t auto_level = lg >= start_log2 ? 0u : (start_log2 - lg) / 2u;
    uint64_t front0 = 0;
    uint32_t vblocks = 0, rblocks = 0;
    for (uint32_t i = 0; i < n; ++i) {
        Query* q = batch[i];
        const oibvh_tree_t A = pool[q->a];
        const oibvh_tree_t B = pool[q->b];
        TreeView va{};
        va.box = A->box.p;
        va.face = A->face.p;
        va.pos = A->cur_pos;
        va.shape = A->shape;
        va.nV = A->nV;
        TreeView vb{};
        vb.box = q->box;
        vb.face = B->face.p;
        vb.pos = q->pos;
        vb.shape = B->shape;
        vb.nV = B->nV;
        L.h_views.p[2 * i] = va;
        L.h_views.p[2 * i + 1] = vb;
        PairView pv{};
        pv.a = 2 * i;
        pv.b = 2 * i + 1;
        pv.ta = va;
        pv.tb = vb;
        const uint32_t start = std::max(entry_level, auto_level);
        pv.entry_a = std::min(start, A->shape.L);
        pv.entry_b = std::min(start, B->shape.L);
        pv.front_cnt_a = A->shape.level_count(pv.entry_a);
        pv.front_cnt_b = B->shape.level_count(pv.entry_b);
        pv.front_off = (uint32_t)front0;
        front0 += (uint64_t)pv.front_cnt_a * pv.front_cnt_b;
        L.h_pairs.p[i] = pv;
        BuildJob j{};
        j.pos = B->cur_pos;  // B at rest
        j.pos_out = q->pos;
        j.nV = B->nV;
        j.nT = B->nT;
        j.vblock_begin = vblocks;
        vblocks += (B->nV + 255) / 256;
        L.h_jobs.p[i] = j;
        std::memcpy(L.h_mats.p + 12 * (size_t)i, q->mat, 12 * sizeof(float));
        RefitJob r{};
        r.box = q->box;
        r.face = B->face.p;
        r.pos = q->pos;
        r.shape = B->shape;
        r.block_begin = rblocks;
        r.n_blocks = refit_blocks_for(B->nT);
        rblocks += r.n_blocks;
        r.counters = L.rcount.p + (size_t)per * i;
        L.h_rjobs.p[i] = r;
    }
    if (front0 > 0x7fffffffull) return fail(OIBVH_ERR_ARG, "batch start front exceeds 2^31 node pairs");
    L.front0_count = front0;
    L.n_pairs = n;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (L.cap_gen != cap_gen) {
            // adopt the server's capacities (set by the caller, or raised by a lane that grew)
            if (L.front_cap != init_front_cap) {
                L.front0.release();
                L.front1.release();
            }
            if (L.hit_cap != init_hit_cap) L.hits.release();
            L.front_cap = init_front_cap;
            L.hit_cap = init_hit_cap;
            L.cap_gen = cap_gen;
        }
    }
    cudaStream_t st = L.st;
    CUDA_TRY(cudaMemcpyAsync(L.views.p, L.h_views.p, 2 * n * sizeof(TreeView), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(L.pairv.p, L.h_pairs.p, n * sizeof(PairView), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(L.jobs.p, L.h_jobs.p, n * sizeof(BuildJob), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(L.rjobs.p, L.h_rjobs.p, n * sizeof(RefitJob), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(L.mats.p, L.h_mats.p, 12 * n * sizeof(float), cudaMemcpyHostToDevice, st));
    // a batch has few jobs: the kernels binary-search them (no block maps)
    CUDA_TRY(launch_transform_multi(L.jobs.p, n, vblocks, nullptr, nullptr, L.mats.p, false, st));
    CUDA_TRY(launch_refit(L.rjobs.p, n, rblocks, nullptr, L.rcount.p, (size_t)per * n, 0, st));
    L.batch = batch;
    const auto now = Clock::now();
    for (uint32_t i = 0; i < n; ++i) {
        batch[i]->t_launch = now;
        batch[i]->status = OIBVH_QUERY_RUNNING;
        batch[i]->batch_size = n;
    }
    return enqueue_detect(L);
}

// Broad + fused narrow phase of the lane's batch; counters copied back.
int oibvh_server_s::enqueue_detect(Lane& L)
{
    cudaStream_t st = L.st;
    OK_TRY(L.front0.ensure(L.front_cap, "cudaMalloc(work list)"));
    OK_TRY(L.front1.ensure(L.front_cap, "cudaMalloc(work list)"));
    OK_TRY(L.hits.ensure(L.hit_cap, "cudaMalloc(hits)"));
    OK_TRY(L.out.ensure(L.hit_cap, "cudaMalloc(grouped pairs)"));
    CUDA_TRY(cudaMemsetAsync(L.counts.p, 0, kCountTotal * sizeof(uint32_t), st));
    CUDA_TRY(cudaMemsetAsync(L.qcount.p, 0, L.n_pairs * sizeof(uint32_t), st));
    DetectArgs a{};
    a.trees = L.views.p;
    a.pairs = L.pairv.p;
    a.n_pairs = L.n_pairs;
    a.expand_levels = 1;
    a.work[0] = L.front0.p;
    a.work[1] = L.front1.p;
    a.work_cap = L.front_cap;
    a.hits = L.hits.p;
    a.hit_cap = L.hit_cap;
    a.counts = L.counts.p;
    a.fuse_narrow = 1;
    a.grid = sm_count(device) * walk_blocks_per_sm();
    a.handoff = 0;
    CUDA_TRY(launch_init_front(a, (uint32_t)L.front0_count, st));
    CUDA_TRY(launch_top(a, st));
    for (uint32_t r = 1; r <= L.rounds; ++r) CUDA_TRY(launch_walk(a, r, st));
    // the hits grouped by query (discarded if the batch is redone)
    const uint32_t bgrid = (uint32_t)sm_count(device) * 2;
    k_bucket_count<<<bgrid, kBucketThreads, 0, st>>>(L.hits.p, L.counts.p, L.hit_cap, L.qcount.p);
    k_bucket_scan<<<1, 1024, 0, st>>>(L.qcount.p, L.n_pairs, L.qoff.p, L.qcursor.p);
    k_bucket_scatter<<<bgrid, kBucketThreads, 0, st>>>(L.hits.p, L.counts.p, L.hit_cap, L.qcursor.p, L.out.p);
    CUDA_TRY(cudaGetLastError());
    note_launches(3);
    CUDA_TRY(cudaMemcpyAsync(L.h_counts.p, L.counts.p, kCountTotal * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(L.h_qoff.p, L.qoff.p, ((size_t)L.n_pairs + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaEventRecord(L.ev, st));
    L.phase = 1;
    return OIBVH_OK;
}

void oibvh_server_s::finish(Lane& L, int status, const std::string& msg)
{
    const auto now = Clock::now();
    std::lock_guard<std::mutex> lk(mu);
    for (Query* q : L.batch) {
        q->t_done = now;
        q->status = status == OIBVH_OK ? OIBVH_QUERY_DONE : OIBVH_QUERY_FAILED;
        q->error = status;
        q->message = msg;
        arena.release(q->slot_off, q->slot_bytes);
        q->pos = nullptr;
        q->box = nullptr;
        if (status == OIBVH_OK) stats.completed++;
        else stats.failed++;
    }
    L.batch.clear();
    L.phase = 0;
    cv_done.notify_all();
}

// The lane's event fired: validate the counters, then fetch the hits.
int oibvh_server_s::advance(Lane& L)
{
    if (L.phase == 1) {
        const uint32_t* c = L.h_counts.p;
        const bool spill = c[kCountWork0 + L.rounds + 1] != 0;
        if (c[kCountFlags] || spill) {
            // queues too small or more walk rounds needed: grow and redo the detect
            uint64_t peak = 0;
            for (uint32_t k = 0; k <= L.rounds + 1; ++k) peak = std::max<uint64_t>(peak, c[kCountWork0 + k]);
            if (c[kCountFlags] & kFlagFrontOverflow) L.front_cap = grow(peak, L.front_cap);
            if (c[kCountFlags] & kFlagHitOverflow) L.hit_cap = grow(c[kCountHits], L.hit_cap);
            if (spill) L.rounds = std::min(kMaxRounds - 1, L.rounds + 4);
            if (c[kCountFlags] & ~(uint32_t)(kFlagFrontOverflow | kFlagHitOverflow))
                return fail(OIBVH_ERR_CUDA, "unexpected traversal flags");
            if (L.front_cap == 0x7fffffffu && (c[kCountFlags] & kFlagFrontOverflow))
                return fail(OIBVH_ERR_OVERFLOW, "BVTT front beyond 2^31 entries");
            {
                std::lock_guard<std::mutex> lk(mu);
                stats.redos++;
                // the other lanes take the grown capacities before their next batch
                if (L.front_cap > init_front_cap || L.hit_cap > init_hit_cap) {
                    init_front_cap = std::max(init_front_cap, L.front_cap);
                    init_hit_cap = std::max(init_hit_cap, L.hit_cap);
                    cap_gen++;
                    L.cap_gen = cap_gen;
                }
            }
            return enqueue_detect(L);
        }
        L.n_hits = c[kCountHits];
        {
            std::lock_guard<std::mutex> lk(mu);
            stats.candidates += c[kCountCands];
            stats.hits += L.n_hits;
        }
        OK_TRY(ensure_pow2(L.h_out, std::max<uint64_t>(L.n_hits, L.hit_cap), "cudaMallocHost(grouped pairs)"));
        if (L.n_hits)
            CUDA_TRY(cudaMemcpyAsync(L.h_out.p, L.out.p, L.n_hits * sizeof(uint2), cudaMemcpyDeviceToHost, L.st));
        CUDA_TRY(cudaEventRecord(L.ev, L.st));
        L.phase = 2;
        return OIBVH_OK;
    }
    // phase 2: query i's (triA, triB) words are h_out[qoff[i] .. qoff[i + 1])
    const uint32_t* words = (const uint32_t*)L.h_out.p;
    for (size_t i = 0; i < L.batch.size(); ++i)
        L.batch[i]->pairs.assign(words + 2 * (size_t)L.h_qoff.p[i], words + 2 * (size_t)L.h_qoff.p[i + 1]);
    finish(L, OIBVH_OK, "");
    return OIBVH_OK;
}

void oibvh_server_s::loop()
{
    cudaSetDevice(device);
    for (;;) {
        bool progress = false;
        for (auto& Lp : lanes) {
            Lane& L = *Lp;
            if (!L.phase) continue;
            const cudaError_t e = cudaEventQuery(L.ev);
            if (e == cudaErrorNotReady) continue;
            progress = true;
            int st = e == cudaSuccess ? advance(L) : cuda_fail(e, "batch on the device");
            if (st != OIBVH_OK) {
                // a failed batch: its queries report the error, the lane starts clean
                const std::string msg = g_last_error;
                cudaStreamSynchronize(L.st);
                cudaGetLastError();
                finish(L, st, msg);
            }
        }
        // admission: an idle lane takes every waiting query whose slot fits
        for (auto& Lp : lanes) {
            Lane& L = *Lp;
            if (L.phase) continue;
            std::vector<Query*> batch;
            {
                std::lock_guard<std::mutex> lk(mu);
                uint64_t cost = 0;
                while (!pending.empty() && batch.size() < max_batch) {
                    Query* q = pending.front();
                    // a batch completes as a whole: bound its work (the first query always goes)
                    const uint64_t qc = (uint64_t)pool[q->a]->nT + pool[q->b]->nT;
                    if (!batch.empty() && max_batch_cost && cost + qc > max_batch_cost) break;
                    size_t off = 0;
                    if (!arena.alloc(q->slot_bytes, off)) break;  // FIFO: the head waits for memory
                    cost += qc;
                    q->slot_off = off;
                    q->pos = (float4*)(arena_mem.p + off);
                    q->box = (float4*)(arena_mem.p + off + align_up((size_t)pool[q->b]->nV * sizeof(float4)));
                    q->lane = (uint32_t)(&Lp - &lanes[0]);
                    pending.pop_front();
                    batch.push_back(q);
                }
                if (!batch.empty()) {
                    stats.batches++;
                    stats.max_batch_seen = std::max<uint64_t>(stats.max_batch_seen, batch.size());
                    stats.arena_peak_bytes = arena.peak;
                }
            }
            if (batch.empty()) break;
            progress = true;
            int st = launch(L, batch);
            if (st != OIBVH_OK) {
                const std::string msg = g_last_error;
                L.batch = batch;
                cudaStreamSynchronize(L.st);
                cudaGetLastError();
                finish(L, st, msg);
            }
        }
        if (progress) continue;
        bool busy = false;
        for (auto& Lp : lanes) busy |= Lp->phase != 0;
        std::unique_lock<std::mutex> lk(mu);
        if (stop && pending.empty() && !busy) break;
        if (busy) {
            lk.unlock();
            std::this_thread::yield();  // the device is working: poll its events
        } else if (pending.empty()) {
            cv_submit.wait_for(lk, std::chrono::milliseconds(2));
        } else {
            // waiting queries, idle lanes, no memory: only a completion frees memory
            cv_submit.wait_for(lk, std::chrono::microseconds(200));
        }
    }
}

#define API extern "C" __attribute__((visibility("default")))
#define GUARD_BEGIN try {
#define GUARD_END                                                   \
    }                                                               \
    catch (const std::bad_alloc&)                                   \
    {                                                               \
        return fail(OIBVH_ERR_OOM, "host allocation failed");       \
    }                                                               \
    catch (const std::exception& ex)                                \
    {                                                               \
        return fail(OIBVH_ERR_CUDA, ex.what());                     \
    }

API int oibvh_server_create(int device, uint64_t memory_budget_bytes, uint32_t max_batch, uint32_t n_lanes,
                            oibvh_server_t* out)
{
    GUARD_BEGIN
    if (!out) return fail(OIBVH_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (memory_budget_bytes < (1u << 20)) return fail(OIBVH_ERR_ARG, "memory budget below 1 MiB");
    if (max_batch == 0 || max_batch > kMaxPairsPerPass) return fail(OIBVH_ERR_ARG, "max_batch must be in 1..16384");
    if (n_lanes == 0 || n_lanes > 16) return fail(OIBVH_ERR_ARG, "lanes must be in 1..16");
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(OIBVH_ERR_ARG, "no such device");
    DeviceGuard g(device);
    std::unique_ptr<oibvh_server_s> s(new oibvh_server_s());
    s->device = device;
    s->budget = align_up(memory_budget_bytes);
    s->max_batch = max_batch;
    OK_TRY(s->arena_mem.ensure(s->budget, "cudaMalloc(server arena)"));
    s->arena.reset(s->budget);
    s->stats.arena_bytes = s->budget;
    for (uint32_t i = 0; i < n_lanes; ++i) {
        std::unique_ptr<Lane> L(new Lane());
        CUDA_TRY(cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&L->ev, cudaEventDisableTiming));
        s->lanes.push_back(std::move(L));
    }
    *out = s.release();
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_server_set_entry_level(oibvh_server_t s, uint32_t entry_level)
{
    if (!s) return fail(OIBVH_ERR_ARG, "server is NULL");
    if (entry_level > kMaxLeafLevel) return fail(OIBVH_ERR_ARG, "entry level above the deepest leaf level");
    std::lock_guard<std::mutex> lk(s->mu);
    s->entry_level = entry_level;
    return OIBVH_OK;
}

API int oibvh_server_set_queue_capacity(oibvh_server_t s, uint32_t front, uint32_t hits)
{
    if (!s) return fail(OIBVH_ERR_ARG, "server is NULL");
    if (front > 0x7fffffffu || hits > 0x7fffffffu) return fail(OIBVH_ERR_ARG, "capacity above 2^31");
    std::lock_guard<std::mutex> lk(s->mu);
    if (front) s->init_front_cap = front;
    if (hits) s->init_hit_cap = hits;
    s->cap_gen++;
    return OIBVH_OK;
}

API int oibvh_server_set_batch_cost(oibvh_server_t s, uint64_t max_triangles)
{
    if (!s) return fail(OIBVH_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    s->max_batch_cost = max_triangles;
    return OIBVH_OK;
}

API int oibvh_server_add_mesh(oibvh_server_t s, oibvh_tree_t t, uint32_t* id)
{
    GUARD_BEGIN
    if (!s || !t) return fail(OIBVH_ERR_ARG, "server or tree is NULL");
    if (!t->built) return fail(OIBVH_ERR_STATE, "pool meshes must be built");
    if (t->device != s->device) return fail(OIBVH_ERR_ARG, "tree lives on another device");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(OIBVH_ERR_STATE, "add pool meshes before oibvh_server_start");
    s->pool.push_back(t);
    if (id) *id = (uint32_t)(s->pool.size() - 1);
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_server_start(oibvh_server_t s)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return OIBVH_OK;
    if (s->pool.empty()) return fail(OIBVH_ERR_STATE, "the pool is empty");
    DeviceGuard g(s->device);
    OK_TRY(s->reserve_lanes());
    s->running = true;
    s->worker = std::thread([s] { s->loop(); });
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_server_submit(oibvh_server_t s, uint32_t mesh_a, uint32_t mesh_b, const float* mat_b, uint64_t* ticket)
{
    GUARD_BEGIN
    if (!s || !mat_b || !ticket) return fail(OIBVH_ERR_ARG, "server, mat_b or ticket is NULL");
    const auto now = Clock::now();
    std::unique_ptr<Query> q(new Query());
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->running || s->stop) return fail(OIBVH_ERR_STATE, "server is not running");
        if (mesh_a >= s->pool.size() || mesh_b >= s->pool.size()) return fail(OIBVH_ERR_ARG, "no such pool mesh");
        q->slot_bytes = s->slot_bytes(mesh_b);
        if (q->slot_bytes > s->arena.size)
            return fail(OIBVH_ERR_OOM, "the query's slot is larger than the whole memory budget");
        q->ticket = s->next_ticket++;
        q->a = mesh_a;
        q->b = mesh_b;
        std::memcpy(q->mat, mat_b, sizeof(q->mat));
        q->t_submit = now;
        *ticket = q->ticket;
        s->pending.push_back(q.get());
        s->stats.submitted++;
        s->queries.emplace(q->ticket, std::move(q));
    }
    s->cv_submit.notify_one();
    return OIBVH_OK;
    GUARD_END
}

static void fill_result(const Query* q, oibvh_query_result* out)
{
    out->status = q->status;
    out->error = q->error;
    out->lane = q->lane;
    out->batch_size = q->batch_size;
    out->n_pairs = q->pairs.size() / 2;
    using us = std::chrono::duration<double, std::micro>;
    const bool launched = q->status == OIBVH_QUERY_RUNNING || q->status == OIBVH_QUERY_DONE ||
                          q->status == OIBVH_QUERY_FAILED;
    const bool done = q->status == OIBVH_QUERY_DONE || q->status == OIBVH_QUERY_FAILED;
    out->queue_us = launched ? us(q->t_launch - q->t_submit).count() : 0.0;
    out->service_us = done ? us(q->t_done - q->t_launch).count() : 0.0;
}

API int oibvh_server_wait(oibvh_server_t s, uint64_t ticket, uint32_t timeout_ms, oibvh_query_result* out)
{
    GUARD_BEGIN
    if (!s || !out) return fail(OIBVH_ERR_ARG, "server or out is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(OIBVH_ERR_ARG, "unknown ticket");
    Query* q = it->second.get();
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [q] {
        return q->status == OIBVH_QUERY_DONE || q->status == OIBVH_QUERY_FAILED;
    });
    fill_result(q, out);
    if (!ok) return fail(OIBVH_ERR_TIMEOUT, "query not finished within the timeout");
    if (q->status == OIBVH_QUERY_FAILED) return fail(q->error, q->message);
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_server_get_pairs(oibvh_server_t s, uint64_t ticket, uint32_t* out2, uint64_t cap, uint64_t* n)
{
    GUARD_BEGIN
    if (!s || !n) return fail(OIBVH_ERR_ARG, "server or n is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(OIBVH_ERR_ARG, "unknown ticket");
    const Query* q = it->second.get();
    if (q->status != OIBVH_QUERY_DONE) return fail(OIBVH_ERR_STATE, "query not done");
    *n = q->pairs.size() / 2;
    const size_t m = std::min<uint64_t>(cap, *n);
    if (m && !out2) return fail(OIBVH_ERR_ARG, "out2 is NULL");
    if (m) std::memcpy(out2, q->pairs.data(), 2 * m * sizeof(uint32_t));
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_server_release(oibvh_server_t s, uint64_t ticket)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(OIBVH_ERR_ARG, "unknown ticket");
    const int st = it->second->status;
    if (st != OIBVH_QUERY_DONE && st != OIBVH_QUERY_FAILED) return fail(OIBVH_ERR_STATE, "query still in flight");
    s->queries.erase(it);
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_server_get_stats(oibvh_server_t s, oibvh_server_stats* out)
{
    if (!s || !out) return fail(OIBVH_ERR_ARG, "server or out is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->arena_used_bytes = s->arena.used;
    out->arena_peak_bytes = s->arena.peak;
    out->queued = s->pending.size();
    return OIBVH_OK;
}

API int oibvh_server_destroy(oibvh_server_t s)
{
    if (!s) return OIBVH_OK;
    delete s;  // stops the loop after the queries already submitted finish
    return OIBVH_OK;
}
