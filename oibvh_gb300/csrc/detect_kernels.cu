// Broad phase (BVTT front expansion) and narrow phase (17-axis SAT).
//
// Reference: Scene::expandBvttNodes (src/cuda/scene.cu:192-223),
// traversal_kernel (src/cuda/collide.cu:76-246) driven by the host loop of
// Scene::detectCollisionOnGPU (src/cuda/scene.cu:270-311), and
// triangle_intersect_kernel (src/cuda/collide.cu:248-299) with
// triangleIntersection2 (third/gProximity/cuda_intersect_tritri.h:350-434).
//
// Every BVTT level is one grid-stride launch that reads its front size from
// device memory, so the host enqueues all levels without reading anything
// back. Appends (next front, candidates, hits) are warp-aggregated: one
// atomicAdd per warp, positions from ballot/shuffle prefix sums.
//
// The triangle test reproduces the reference's CPU arithmetic
// (src/utils/utils.cpp:71-169, glm scalar dot/cross): every product, sum and
// difference is rounded on its own (__fmul_rn/__fadd_rn/__fsub_rn, never
// contracted to FMA), so the GPU pair set is the CPU pair set bit for bit.
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh {

constexpr int kDetectThreads = 256;

__device__ __forceinline__ bool box_overlap(const float4& a0, const float4& a1, const float4& b0, const float4& b1)
{
    // aabb_box_t::overlap (include/utils/utils.h:39-44; src/cuda/collide.cu:12-17)
    return (a0.x <= b1.x && a1.x >= b0.x) && (a0.y <= b1.y && a1.y >= b0.y) && (a0.z <= b1.z && a1.z >= b0.z);
}

// ---------------------------------------------------------------------------
// Exact-rounding SAT
// ---------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 vsub(const V3& a, const V3& b)
{
    return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
// glm::cross: (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
__device__ __forceinline__ V3 vcross(const V3& x, const V3& y)
{
    return V3{__fsub_rn(__fmul_rn(x.y, y.z), __fmul_rn(y.y, x.z)), __fsub_rn(__fmul_rn(x.z, y.x), __fmul_rn(y.z, x.x)),
              __fsub_rn(__fmul_rn(x.x, y.y), __fmul_rn(y.x, x.y))};
}
// glm::dot: (a.x*b.x + a.y*b.y) + a.z*b.z, each op rounded
__device__ __forceinline__ float vdot(const V3& a, const V3& b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// project6 (src/utils/utils.cpp:71-95)
__device__ __forceinline__ bool project6(const V3& ax, const V3& p1, const V3& p2, const V3& p3, const V3& q1,
                                         const V3& q2, const V3& q3)
{
    const float P1 = vdot(ax, p1), P2 = vdot(ax, p2), P3 = vdot(ax, p3);
    const float Q1 = vdot(ax, q1), Q2 = vdot(ax, q2), Q3 = vdot(ax, q3);
    const float mx1 = fmaxf(fmaxf(P1, P2), P3), mn1 = fminf(fminf(P1, P2), P3);
    const float mx2 = fmaxf(fmaxf(Q1, Q2), Q3), mn2 = fminf(fminf(Q1, Q2), Q3);
    if (mn1 > mx2) return false;
    if (mn2 > mx1) return false;
    return true;
}
// triangleIntersect (src/utils/utils.cpp:97-169); the 17 tests are a
// conjunction, so evaluating the axes lazily does not change the result.
__device__ __forceinline__ bool tri_intersect_exact(const V3& P1, const V3& P2, const V3& P3, const V3& Q1,
                                                    const V3& Q2, const V3& Q3)
{
    const V3 p1{0.0f, 0.0f, 0.0f};
    const V3 p2 = vsub(P2, P1), p3 = vsub(P3, P1);
    const V3 q1 = vsub(Q1, P1), q2 = vsub(Q2, P1), q3 = vsub(Q3, P1);
    const V3 e1 = vsub(p2, p1), e2 = vsub(p3, p2), e3 = vsub(p1, p3);
    const V3 f1 = vsub(q2, q1), f2 = vsub(q3, q2), f3 = vsub(q1, q3);
    const V3 n1 = vcross(e1, e2);
    if (!project6(n1, p1, p2, p3, q1, q2, q3)) return false;
    const V3 m1 = vcross(f1, f2);
    if (!project6(m1, p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e1, f1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e1, f2), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e1, f3), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e2, f1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e2, f2), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e2, f3), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e3, f1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e3, f2), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e3, f3), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e1, n1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e2, n1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(e3, n1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(f1, m1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(f2, m1), p1, p2, p3, q1, q2, q3)) return false;
    if (!project6(vcross(f3, m1), p1, p2, p3, q1, q2, q3)) return false;
    return true;
}

__device__ __forceinline__ V3 load_vertex(const float* __restrict__ xyz, uint32_t v)
{
    return V3{__ldg(xyz + 3 * (size_t)v), __ldg(xyz + 3 * (size_t)v + 1), __ldg(xyz + 3 * (size_t)v + 2)};
}

// ---------------------------------------------------------------------------
// Counters: [0] hits, [1] flags, [2] candidates, [3 + it] front size at step it
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred, uint32_t lane)
{
    const uint32_t mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return 0;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// Initial front: for every pair, all real nodes of A at its entry level x all
// real nodes of B at its entry level (Scene::expandBvttNodes).
__global__ void __launch_bounds__(kDetectThreads) k_init_front(DetectArgs a, uint32_t total)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) a.counts[3] = total;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = a.n_pairs - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (a.pairs[mid].front_off <= i) lo = mid;
            else hi = mid - 1;
        }
        const PairView pv = a.pairs[lo];
        const uint32_t k = i - pv.front_off;
        const uint32_t x = k / pv.front_cnt_b, y = k - x * pv.front_cnt_b;
        a.front[0][i] = bvtt_pack(lo, (1u << pv.entry_a) - 1u + x, (1u << pv.entry_b) - 1u + y);
    }
}

// Children of implicit node `ia` (level la) `e` levels down, clamped at the
// leaf level: the first child and the count of real ones
// (src/cuda/collide.cu:165-176).
__device__ __forceinline__ void expand_side(const TreeShape& S, uint32_t ia, uint32_t la, uint32_t e,
                                            uint32_t& first, uint32_t& count)
{
    if (la == S.L) {
        first = ia;
        count = 1;
        return;
    }
    const uint32_t nl = min(S.L, la + e);
    const uint32_t d = nl - la;
    first = ((ia + 1u) << d) - 1u;
    const uint32_t right_valid = (2u << nl) - 2u - (S.vl >> (S.L - nl));
    count = min(1u << d, right_valid - first + 1u);
}

__global__ void __launch_bounds__(kDetectThreads) k_bvtt_step(DetectArgs a, uint32_t it)
{
    const uint32_t n = min(a.counts[3 + it], a.front_cap);
    const uint64_t* __restrict__ src = (it & 1) ? a.front[1] : a.front[0];
    uint64_t* __restrict__ dst = (it & 1) ? a.front[0] : a.front[1];
    uint32_t* dst_count = a.counts + 3 + it + 1;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp * 32; base < n; base += n_warps * 32) {
        const uint32_t i = base + lane;
        bool cand = false;
        uint64_t cval = 0;
        uint32_t pair = 0, firstA = 0, firstB = 0, ncA = 0, ncB = 0;
        if (i < n) {
            const uint64_t node = src[i];
            pair = bvtt_pair(node);
            const uint32_t ia = bvtt_a(node), ib = bvtt_b(node);
            const PairView pv = a.pairs[pair];
            const TreeView& TA = a.trees[pv.a];
            const TreeView& TB = a.trees[pv.b];
            const TreeShape SA = TA.shape, SB = TB.shape;
            const uint32_t la = ilog2(ia + 1u), lb = ilog2(ib + 1u);
            const uint32_t ra = SA.real_index(ia), rb = SB.real_index(ib);
            const float4* ba = TA.box + 2 * (size_t)ra;
            const float4* bb = TB.box + 2 * (size_t)rb;
            const float4 a0 = __ldg(ba), a1 = __ldg(ba + 1), b0 = __ldg(bb), b1 = __ldg(bb + 1);
            if (box_overlap(a0, a1, b0, b1)) {
                if (la == SA.L && lb == SB.L) {
                    cand = true;
                    cval = bvtt_pack(pair, ia - ((1u << SA.L) - 1u), ib - ((1u << SB.L) - 1u));
                } else {
                    expand_side(SA, ia, la, a.expand_levels, firstA, ncA);
                    expand_side(SB, ib, lb, a.expand_levels, firstB, ncB);
                }
            }
        }
        const uint32_t cpos = warp_append(a.counts + 2, cand, lane);
        if (cand) {
            if (cpos < a.cand_cap) a.cand[cpos] = cval;
            else atomicOr(a.counts + 1, (uint32_t)kFlagCandOverflow);
        }
        // next front: warp inclusive scan of the child counts
        const uint32_t nch = ncA * ncB;
        uint32_t incl = nch;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, s);
            if ((int)lane >= s) incl += y;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        if (total) {
            uint32_t wbase = 0;
            if (lane == 31) wbase = atomicAdd(dst_count, total);
            wbase = __shfl_sync(0xffffffffu, wbase, 31);
            uint32_t pos = wbase + incl - nch;
            bool overflow = false;
            for (uint32_t x = 0; x < ncA; ++x)
                for (uint32_t y = 0; y < ncB; ++y, ++pos) {
                    if (pos < a.front_cap) dst[pos] = bvtt_pack(pair, firstA + x, firstB + y);
                    else overflow = true;
                }
            if (overflow) atomicOr(a.counts + 1, (uint32_t)kFlagFrontOverflow);
        }
    }
}

__global__ void __launch_bounds__(kDetectThreads) k_narrow(DetectArgs a)
{
    const uint32_t n = min(a.counts[2], a.cand_cap);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp * 32; base < n; base += n_warps * 32) {
        const uint32_t i = base + lane;
        bool hit = false;
        uint4 rec = make_uint4(0, 0, 0, 0);
        if (i < n) {
            const uint64_t c = a.cand[i];
            const PairView pv = a.pairs[bvtt_pair(c)];
            const TreeView& TA = a.trees[pv.a];
            const TreeView& TB = a.trees[pv.b];
            const uint4 fa = __ldg(TA.face + bvtt_a(c));
            const uint4 fb = __ldg(TB.face + bvtt_b(c));
            const float* xa = TA.xyz;
            const float* xb = TB.xyz;
            hit = tri_intersect_exact(load_vertex(xa, fa.x), load_vertex(xa, fa.y), load_vertex(xa, fa.z),
                                      load_vertex(xb, fb.x), load_vertex(xb, fb.y), load_vertex(xb, fb.z));
            rec = make_uint4(pv.a, pv.b, fa.w, fb.w);
        }
        const uint32_t pos = warp_append(a.counts + 0, hit, lane);
        if (hit) {
            if (pos < a.hit_cap) a.hits[pos] = rec;
            else atomicOr(a.counts + 1, (uint32_t)kFlagHitOverflow);
        }
    }
}

cudaError_t launch_init_front(const DetectArgs& a, uint32_t total, cudaStream_t s)
{
    uint32_t blocks = (total + kDetectThreads - 1) / kDetectThreads;
    if (blocks > (uint32_t)a.grid) blocks = (uint32_t)a.grid;
    if (blocks == 0) blocks = 1;
    note_launches(1);
    k_init_front<<<blocks, kDetectThreads, 0, s>>>(a, total);
    return cudaGetLastError();
}

cudaError_t launch_bvtt_step(const DetectArgs& a, uint32_t it, cudaStream_t s)
{
    note_launches(1);
    k_bvtt_step<<<a.grid, kDetectThreads, 0, s>>>(a, it);
    return cudaGetLastError();
}

cudaError_t launch_narrow(const DetectArgs& a, cudaStream_t s)
{
    note_launches(1);
    k_narrow<<<a.grid, kDetectThreads, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace oibvh
