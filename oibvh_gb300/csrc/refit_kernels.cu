// Single-launch bottom-up construction / refit of oibvh trees.
//
// Reference: oibvh_tree_construction_kernel{,2} (src/cuda/oibvh.cu:80-219)
// launched once per level group by OibvhTree::build/refit
// (src/cuda/oibvhTree.cu:193-235,338-357) after calculate_aabb_kernel
// (src/cuda/oibvh.cu:24-40). Here one kernel does all of it, for any number
// of trees at once:
//   * a CTA owns 2^g consecutive Morton-ordered leaves (a level group of g
//     levels, g = 9, 10 or 11, chosen by the tuning; 2^g / 4 threads), four
//     per thread: it loads the four 16-byte face records and the twelve
//     vertices with independent loads, builds the leaf boxes in registers,
//     reduces two levels inside the thread, five across the warp (shuffles)
//     and g - 7 across the CTA (one box per warp through shared memory),
//     writing every internal node it produces;
//   * the CTA finishing last among a group of 2^g sibling subtree roots (one
//     atomic counter per group, threadfence-reduction pattern) loads the
//     group and climbs the next g levels the same way, up to the root.
// No CTA waits for another (no spin loop).
//
// Leaf boxes are not stored: a leaf's box is min/max of its three vertices
// and is recomputed where it is needed (broad-phase tests at the leaf level,
// oibvh_tree_get_aabbs), which removes half of the node writes per refit.
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh {

// Level groups: a CTA reduces 2^kLog nodes by kLog levels (four nodes per
// thread), kLog = 9, 10 (default) or 11; the group depth is a tuning knob.
constexpr uint32_t kRefitLogDefault = 10;
constexpr int kStageCounters = 64;  // counters per climbing stage and tree (groups of the widest stage, kLog 9)

__device__ __forceinline__ Box shfl_down(const Box& b, int d)
{
    return Box{__shfl_down_sync(0xffffffffu, b.nx, d), __shfl_down_sync(0xffffffffu, b.ny, d),
               __shfl_down_sync(0xffffffffu, b.nz, d), __shfl_down_sync(0xffffffffu, b.xx, d),
               __shfl_down_sync(0xffffffffu, b.xy, d), __shfl_down_sync(0xffffffffu, b.xz, d)};
}

__device__ __forceinline__ void store_node(float4* box, uint32_t real, const Box& b)
{
    store_node_v8(box + 2 * (size_t)real, b);
}

// Reduce the 2^kLog-node block whose four nodes per thread are v[0..3]
// (level `lvl`, global indices base + 4*tid + k, real when < level_count(lvl))
// by `levels` levels, writing each produced node. Thread 0 ends holding the
// block root (level lvl - levels, index base >> levels).
template <int kLog>
__device__ __forceinline__ void reduce_block(Box v[4], const TreeShape& S, float4* box, uint32_t lvl, uint32_t base,
                                             uint32_t levels, Box* sm8)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t cnt = S.level_count(lvl);
    uint32_t idx = base + 4 * tid;  // index of v[0]
    uint32_t done = 0;
    // two levels inside the thread
    if (done < levels) {
        const uint32_t off = S.level_offset(lvl - 1);
        const Box n0 = (idx + 1 < cnt) ? merge(v[0], v[1]) : v[0];
        const Box n1 = (idx + 3 < cnt) ? merge(v[2], v[3]) : v[2];
        if (idx < cnt) store_node(box, off + (idx >> 1), n0);
        if (idx + 2 < cnt) store_node(box, off + (idx >> 1) + 1, n1);
        v[0] = n0;
        v[1] = n1;
        cnt = (cnt + 1) >> 1;
        idx >>= 1;
        --lvl;
        ++done;
    }
    if (done < levels) {
        const uint32_t off = S.level_offset(lvl - 1);
        const Box n0 = (idx + 1 < cnt) ? merge(v[0], v[1]) : v[0];
        if (idx < cnt) store_node(box, off + (idx >> 1), n0);
        v[0] = n0;
        cnt = (cnt + 1) >> 1;
        --lvl;
        ++done;
    }
    // five levels across the warp: lane holds node idx0 + lane (idx0 = base/4 + 32*warp)
    const uint32_t idx0 = (base >> 2) + 32 * warp;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        if (done < levels) {  // uniform over the CTA
            const Box r = shfl_down(v[0], 1 << s);
            const uint32_t j = (idx0 + lane) >> s;  // this lane's node (when lane % 2^(s+1) == 0)
            if ((lane & ((2u << s) - 1u)) == 0) {
                if (j + 1 < cnt) v[0] = merge(v[0], r);
                if (j < cnt) store_node(box, S.level_offset(lvl - 1) + (j >> 1), v[0]);
            }
            cnt = (cnt + 1) >> 1;
            --lvl;
            ++done;
        }
    }
    // the last kLog - 7 levels across the CTA: one root per warp
    constexpr int kWarpLog = kLog - 7, kWarps = 1 << kWarpLog;
    if (done < levels) {
        if (lane == 0) sm8[warp] = v[0];
        __syncthreads();
        if (warp == 0) {
            if (lane < kWarps) v[0] = sm8[lane];
            const uint32_t b0 = base >> 7;  // index of warp 0's root
#pragma unroll
            for (int s = 0; s < kWarpLog; ++s) {
                if (done < levels) {
                    const Box r = shfl_down(v[0], 1 << s);
                    const uint32_t j = (b0 + lane) >> s;
                    if (lane < kWarps && (lane & ((2u << s) - 1u)) == 0) {
                        if (j + 1 < cnt) v[0] = merge(v[0], r);
                        if (j < cnt) store_node(box, S.level_offset(lvl - 1) + (j >> 1), v[0]);
                    }
                    cnt = (cnt + 1) >> 1;
                    --lvl;
                    ++done;
                }
            }
        }
    }
}

// `jobs` == nullptr: a single tree passed by value in `one`.
template <int kLog>
__global__ void __launch_bounds__((1 << kLog) / 4, 1536 / ((1 << kLog) / 4))
    k_refit(const RefitJob* __restrict__ jobs, uint32_t n_jobs, const uint32_t* __restrict__ block_job,
            const RefitJob one)
{
    constexpr uint32_t kRefitLog = kLog, kRefitChunk = 1u << kLog;
    __shared__ Box sm8[(1 << kLog) / 128];
    __shared__ uint32_t s_last;

    RefitJob job = one;
    if (jobs != nullptr && block_job != nullptr) {
        job = jobs[__ldg(block_job + blockIdx.x)];
    } else if (jobs != nullptr) {
        uint32_t lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (jobs[mid].block_begin <= blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        job = jobs[lo];
    }
    const TreeShape S = job.shape;
    if (S.L == 0) return;  // a single leaf: no internal node
    const uint32_t chunk = blockIdx.x - job.block_begin;

    // ---- leaves: calculate_aabb_kernel (src/cuda/oibvh.cu:24-40), in registers ----
    const uint32_t leaf0 = (chunk << kRefitLog) + 4 * threadIdx.x;
    uint4 f[4];
    if (leaf0 + 3 < S.nT) {  // leaf0 is a multiple of 4: 64-byte aligned, two 256-bit loads
        load_face_pair(job.face + leaf0, f[0], f[1]);
        load_face_pair(job.face + leaf0 + 2, f[2], f[3]);
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) f[k] = (leaf0 + k < S.nT) ? __ldg(job.face + leaf0 + k) : make_uint4(0, 0, 0, 0);
    }
    Box v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = leaf_box(job.pos, f[k]);

    uint32_t levels = min((uint32_t)kRefitLog, S.L);
    reduce_block<kLog>(v, S, job.box, S.L, chunk << kRefitLog, levels, sm8);
    uint32_t lvl = S.L - levels;
    if (lvl == 0) return;

    // ---- climb: the last CTA of each 1024-node group continues upward ----
    uint32_t idx = chunk;
    for (int stage = 0;; ++stage) {
        const uint32_t g = idx >> kRefitLog;
        const uint32_t gcnt = min(kRefitChunk, S.level_count(lvl) - (g << kRefitLog));
        if (threadIdx.x == 0) {
            __threadfence();
            const uint32_t old = atomicAdd(job.counters + stage * kStageCounters + g, 1u);
            s_last = (old == gcnt - 1) ? 1u : 0u;
        }
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        const uint32_t base = g << kRefitLog;
        const uint32_t off = S.level_offset(lvl);
        const uint32_t cnt = S.level_count(lvl);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t j = base + 4 * threadIdx.x + k;
            v[k] = (j < cnt) ? load_node_cg(job.box + 2 * (size_t)(off + j)) : Box{0, 0, 0, 0, 0, 0};
        }
        levels = min((uint32_t)kRefitLog, lvl);
        reduce_block<kLog>(v, S, job.box, lvl, base, levels, sm8);
        lvl -= levels;
        if (lvl == 0) return;
        idx = g;
        __syncthreads();  // s_last and sm8 are reused by the next stage
    }
}

// Leaf boxes of one tree as float4 pairs (for oibvh_tree_get_aabbs).
__global__ void __launch_bounds__(256) k_leaf_boxes(const uint4* __restrict__ face, const float4* __restrict__ xyz,
                                                    uint32_t nT, float4* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nT) return;
    const Box b = leaf_box(xyz, __ldg(face + i));
    out[2 * (size_t)i] = make_float4(b.nx, b.ny, b.nz, 0.0f);
    out[2 * (size_t)i + 1] = make_float4(b.xx, b.xy, b.xz, 0.0f);
}

uint32_t refit_blocks_for(uint32_t nT, uint32_t group_log2)
{
    const uint32_t g = group_log2 ? group_log2 : kRefitLogDefault;
    return (nT + (1u << g) - 1) >> g;
}
uint32_t refit_counters_per_tree() { return 4 * kStageCounters; }

template <int kLog>
static void refit_launch(uint32_t blocks, const RefitJob* jobs, uint32_t n_jobs, const uint32_t* block_job,
                         const RefitJob& one, cudaStream_t s)
{
    k_refit<kLog><<<blocks, (1 << kLog) / 4, 0, s>>>(jobs, n_jobs, block_job, one);
}

static cudaError_t refit_dispatch(uint32_t group_log2, uint32_t blocks, const RefitJob* jobs, uint32_t n_jobs,
                                  const uint32_t* block_job, const RefitJob& one, cudaStream_t s)
{
    switch (group_log2 ? group_log2 : kRefitLogDefault) {
    case 9: refit_launch<9>(blocks, jobs, n_jobs, block_job, one, s); break;
    case 10: refit_launch<10>(blocks, jobs, n_jobs, block_job, one, s); break;
    case 11: refit_launch<11>(blocks, jobs, n_jobs, block_job, one, s); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_refit_one(const RefitJob& job, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(job.counters, 0, refit_counters_per_tree() * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    note_launches(1);
    return refit_dispatch(kRefitLogDefault, job.n_blocks, nullptr, 1, nullptr, job, s);
}

cudaError_t launch_refit(const RefitJob* d_jobs, uint32_t n_jobs, uint32_t total_blocks, const uint32_t* block_job,
                         uint32_t* d_counters, size_t n_counters, uint32_t group_log2, cudaStream_t s)
{
    if (n_jobs == 0 || total_blocks == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counters, 0, n_counters * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    RefitJob none{};
    note_launches(1);
    return refit_dispatch(group_log2, total_blocks, d_jobs, n_jobs, block_job, none, s);
}

cudaError_t launch_leaf_boxes(const uint4* face, const float4* xyz, uint32_t nT, float4* out, cudaStream_t s)
{
    note_launches(1);
    k_leaf_boxes<<<(nT + 255) / 256, 256, 0, s>>>(face, xyz, nT, out);
    return cudaGetLastError();
}

} // namespace oibvh
