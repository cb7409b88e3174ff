// Single-launch bottom-up construction / refit of oibvh trees.
//
// Reference: oibvh_tree_construction_kernel{,2} (src/cuda/oibvh.cu:80-219)
// launched once per level group by OibvhTree::build/refit
// (src/cuda/oibvhTree.cu:193-235,338-357) after calculate_aabb_kernel
// (src/cuda/oibvh.cu:24-40). Here one kernel does all of it, for any number
// of trees at once:
//   * a CTA owns 2048 consecutive Morton-ordered leaves: it loads their face
//     records (16 B, coalesced), gathers the vertices, and reduces the leaf
//     boxes 11 levels up through shared memory, writing every level's nodes
//     to HBM as it goes (coalesced float4 stores);
//   * the CTA finishing last among the 2048-node groups of the level above
//     (one atomic counter per group, threadfence-reduction pattern) loads the
//     group's roots and climbs the next 11 levels the same way, until the root.
// No CTA ever waits for another, so there is no spin loop.
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh {

constexpr int kRefitThreads = 512;
constexpr int kRefitLog = 11;
constexpr int kRefitChunk = 1 << kRefitLog;  // leaves per CTA, and nodes per climbing group
constexpr int kStageCounters = 16;           // counters per climbing stage and tree
constexpr int kRefitSmemBytes = 6 * kRefitChunk * (int)sizeof(float);

struct SmemBoxes {
    float* v;  // SoA: [6][kRefitChunk] = mnx, mny, mnz, mxx, mxy, mxz
    __device__ __forceinline__ void put(int i, const float b[6])
    {
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k * kRefitChunk + i] = b[k];
    }
    __device__ __forceinline__ void get(int i, float b[6]) const
    {
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] = v[k * kRefitChunk + i];
    }
};

__device__ __forceinline__ void store_box(float4* box, uint32_t real, const float b[6])
{
    box[2 * (size_t)real] = make_float4(b[0], b[1], b[2], 0.0f);
    box[2 * (size_t)real + 1] = make_float4(b[3], b[4], b[5], 0.0f);
}

__device__ __forceinline__ void merge_children(const SmemBoxes& sm, uint32_t j, uint32_t cnt, float m[6])
{
    float lb[6];
    sm.get(2 * j, lb);
    if (2 * j + 1 < cnt) {
        float rb[6];
        sm.get(2 * j + 1, rb);
        // merge_aabb (src/cuda/oibvh.cu:72-78): glm::min(left, right), glm::max(left, right)
        m[0] = gmin(lb[0], rb[0]);
        m[1] = gmin(lb[1], rb[1]);
        m[2] = gmin(lb[2], rb[2]);
        m[3] = gmax(lb[3], rb[3]);
        m[4] = gmax(lb[4], rb[4]);
        m[5] = gmax(lb[5], rb[5]);
    } else {
#pragma unroll
        for (int k = 0; k < 6; ++k) m[k] = lb[k];
    }
}

// Reduce `levels` levels in shared memory. On entry entries [0, cnt) hold the
// nodes of level `lvl` with global indices [base, base + cnt); each level's
// nodes are written to HBM. Returns with entry 0 = the subtree root.
__device__ __forceinline__ void reduce_levels(SmemBoxes sm, float4* box, const TreeShape& S, uint32_t lvl,
                                              uint32_t base, uint32_t cnt, uint32_t levels)
{
    // A level above 2048 nodes has at most 1024 nodes: two per thread.
    static_assert(kRefitChunk / 2 <= 2 * kRefitThreads, "two nodes per thread per level");
    for (uint32_t lev = 1; lev <= levels; ++lev) {
        const uint32_t l = lvl - lev;
        const uint32_t nc = (cnt + 1) >> 1;
        const uint32_t off = S.level_offset(l) + (base >> lev);
        const uint32_t j0 = threadIdx.x, j1 = threadIdx.x + kRefitThreads;
        float m0[6], m1[6];
        if (j0 < nc) merge_children(sm, j0, cnt, m0);
        if (j1 < nc) merge_children(sm, j1, cnt, m1);
        __syncthreads();
        if (j0 < nc) {
            sm.put(j0, m0);
            store_box(box, off + j0, m0);
        }
        if (j1 < nc) {
            sm.put(j1, m1);
            store_box(box, off + j1, m1);
        }
        __syncthreads();
        cnt = nc;
    }
}

// `jobs` == nullptr: a single tree passed by value in `one`.
__global__ void __launch_bounds__(kRefitThreads) k_refit(const RefitJob* __restrict__ jobs, uint32_t n_jobs,
                                                         const RefitJob one)
{
    extern __shared__ float smem_raw[];
    __shared__ uint32_t s_last;
    SmemBoxes sm{smem_raw};

    RefitJob job = one;
    if (jobs != nullptr) {
        // job lookup: largest block_begin <= blockIdx.x
        uint32_t lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (jobs[mid].block_begin <= blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        job = jobs[lo];
    }
    const TreeShape S = job.shape;
    const uint32_t chunk = blockIdx.x - job.block_begin;

    // ---- leaves: calculate_aabb_kernel (src/cuda/oibvh.cu:24-40) ----
    const uint32_t leaf0 = chunk << kRefitLog;
    const uint32_t nl = min((uint32_t)kRefitChunk, S.nT - leaf0);
    const uint32_t leaf_off = S.level_offset(S.L) + leaf0;
    for (uint32_t i = threadIdx.x; i < nl; i += kRefitThreads) {
        const uint4 f = __ldg(job.face + leaf0 + i);
        float b[6];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = __ldg(job.xyz + 3 * (size_t)f.x + k);
            const float c = __ldg(job.xyz + 3 * (size_t)f.y + k);
            const float d = __ldg(job.xyz + 3 * (size_t)f.z + k);
            b[k] = gmin(gmin(a, c), d);
            b[3 + k] = gmax(gmax(a, c), d);
        }
        sm.put(i, b);
        store_box(job.box, leaf_off + i, b);
    }
    __syncthreads();

    const uint32_t lv0 = min((uint32_t)kRefitLog, S.L);
    reduce_levels(sm, job.box, S, S.L, leaf0, nl, lv0);
    if (S.L <= (uint32_t)kRefitLog) return;  // this CTA wrote the root

    // ---- climb: the last CTA of each 2048-node group continues upward ----
    uint32_t lvl = S.L - kRefitLog;  // level of the node this CTA just finished
    uint32_t idx = chunk;            // its index in that level
    for (int stage = 0;; ++stage) {
        const uint32_t g = idx >> kRefitLog;
        const uint32_t gcnt = min((uint32_t)kRefitChunk, S.level_count(lvl) - (g << kRefitLog));
        if (threadIdx.x == 0) {
            __threadfence();
            const uint32_t old = atomicAdd(job.counters + stage * kStageCounters + g, 1u);
            s_last = (old == gcnt - 1) ? 1u : 0u;
        }
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        const uint32_t off = S.level_offset(lvl) + (g << kRefitLog);
        for (uint32_t j = threadIdx.x; j < gcnt; j += kRefitThreads) {
            const float4 a = __ldcg(job.box + 2 * (size_t)(off + j));
            const float4 c = __ldcg(job.box + 2 * (size_t)(off + j) + 1);
            const float b[6] = {a.x, a.y, a.z, c.x, c.y, c.z};
            sm.put(j, b);
        }
        __syncthreads();
        const uint32_t levels = min((uint32_t)kRefitLog, lvl);
        reduce_levels(sm, job.box, S, lvl, g << kRefitLog, gcnt, levels);
        lvl -= levels;
        if (lvl == 0) return;
        idx = g;
    }
}

uint32_t refit_blocks_for(uint32_t nT) { return (nT + kRefitChunk - 1) / kRefitChunk; }
uint32_t refit_counters_per_tree() { return 4 * kStageCounters; }

static cudaError_t configure_refit()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    static bool configured[64] = {};
    if (dev >= 0 && dev < 64 && configured[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_refit, cudaFuncAttributeMaxDynamicSharedMemorySize, kRefitSmemBytes);
    if (e == cudaSuccess && dev >= 0 && dev < 64) configured[dev] = true;
    return e;
}

cudaError_t launch_refit_one(const RefitJob& job, cudaStream_t s)
{
    cudaError_t e = configure_refit();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(job.counters, 0, refit_counters_per_tree() * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    note_launches(1);
    k_refit<<<job.n_blocks, kRefitThreads, kRefitSmemBytes, s>>>(nullptr, 1, job);
    return cudaGetLastError();
}

cudaError_t launch_refit(const RefitJob* d_jobs, uint32_t n_jobs, uint32_t total_blocks, uint32_t* d_counters,
                         size_t n_counters, cudaStream_t s)
{
    cudaError_t e = configure_refit();
    if (e != cudaSuccess) return e;
    if (n_jobs == 0 || total_blocks == 0) return cudaSuccess;
    e = cudaMemsetAsync(d_counters, 0, n_counters * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    RefitJob none{};
    note_launches(1);
    k_refit<<<total_blocks, kRefitThreads, kRefitSmemBytes, s>>>(d_jobs, n_jobs, none);
    return cudaGetLastError();
}

} // namespace oibvh
