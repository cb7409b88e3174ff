// Host orchestration and the C ABI (include/oibvh_gb300.h).
//
// oibvh_tree_s mirrors OibvhTree (include/cuda/oibvhTree.cuh:50-93,
// src/cuda/oibvhTree.cu) and oibvh_scene_s mirrors Scene
// (include/cuda/scene.cuh:44-61, src/cuda/scene.cu). Differences by design:
//   * the tree stays resident in device memory; nothing is copied back to
//     the host after build or refit unless asked (oibvh_tree_get_aabbs);
//   * the BVTT loop is enqueued whole: each level reads its front size on
//     the device, so detect reads counters back once per pass, not once per
//     level (the reference reads after every level, src/cuda/scene.cu:302);
//   * queues are sized by demand: an overflow is detected, the queue grows,
//     and the pass reruns (the reference writes past fixed 10M-entry buffers
//     unchecked, src/cuda/scene.cu:15-21, src/cuda/collide.cu:160-161);
//   * every CUDA status is checked and returned.
#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/oibvh_gb300.h"
#include "host_util.h"
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

using namespace oibvh;

namespace oibvh {
static std::atomic<uint64_t> g_launches{0};
void note_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace oibvh

namespace oibvh_host {
thread_local std::string g_last_error;
std::atomic<int64_t> g_fail_alloc{-1};
std::atomic<uint64_t> g_alloc_attempts{0};
}  // namespace oibvh_host

static int tree_alloc(oibvh_tree_t t)
{
    OK_TRY(t->xyz.ensure(3 * (size_t)t->nV, "cudaMalloc(positions)"));
    OK_TRY(t->pos4.ensure((size_t)t->nV, "cudaMalloc(positions)"));
    OK_TRY(t->tri.ensure(3 * (size_t)t->nT, "cudaMalloc(faces)"));
    // one record more than the faces: traversal reads two sibling leaves' faces as one
    // 32-byte load, and the last leaf's sibling may be virtual (past the end)
    OK_TRY(t->face.ensure((size_t)t->nT + 1, "cudaMalloc(sorted faces)"));
    OK_TRY(t->vperm.ensure(t->nV, "cudaMalloc(vertex order)"));
    OK_TRY(t->box.ensure(2 * (size_t)std::max(1u, t->shape.size - t->nT), "cudaMalloc(tree)"));
    OK_TRY(t->counters.ensure(refit_counters_per_tree(), "cudaMalloc(counters)"));
    return OIBVH_OK;
}

static int tree_create_impl(const float* xyz, uint32_t nV, const uint32_t* tri, uint32_t nT, int device,
                            oibvh_tree_t* out)
{
    if (!out) return fail(OIBVH_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!xyz || !tri) return fail(OIBVH_ERR_ARG, "xyz or tri is NULL");
    if (nT == 0) return fail(OIBVH_ERR_ARG, "a mesh needs at least one triangle");
    if (nT > (1u << kMaxLeafLevel)) return fail(OIBVH_ERR_ARG, "more than 2^23 triangles");
    if (nV == 0) return fail(OIBVH_ERR_ARG, "no vertices");
    for (size_t i = 0; i < 3 * (size_t)nT; ++i)
        if (tri[i] >= nV)
            return fail(OIBVH_ERR_ARG, "face " + std::to_string(i / 3) + " refers to vertex " +
                                           std::to_string(tri[i]) + " >= " + std::to_string(nV));
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(OIBVH_ERR_ARG, "no such device");
    DeviceGuard g(device);
    if (!g.ok) return fail(OIBVH_ERR_CUDA, "cudaSetDevice failed");
    oibvh_tree_t t = new oibvh_tree_s();
    t->device = device;
    t->nV = nV;
    t->nT = nT;
    t->shape = TreeShape::of(nT);
    int st = tree_alloc(t);
    if (st == OIBVH_OK) {
        cudaError_t e = cudaMemcpy(t->xyz.p, xyz, 3 * (size_t)nV * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(t->tri.p, tri, 3 * (size_t)nT * sizeof(uint32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launch_xyz_to_pos4(t->xyz.p, nullptr, nV, t->pos4.p, 0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpy(mesh)");
    }
    if (st != OIBVH_OK) {
        delete t;
        return st;
    }
    t->cur_pos = t->pos4.p;
    *out = t;
    return OIBVH_OK;
}

// Borrowed positions (caller's order) into the tree's own buffer, in the
// tree's vertex order.
static int sync_positions(oibvh_tree_t t, cudaStream_t s)
{
    if (t->borrowed) CUDA_TRY(launch_gather_pos4(t->borrowed, t->vmap(), t->nV, t->pos4.p, s));
    t->cur_pos = t->pos4.p;
    return OIBVH_OK;
}

// After the faces are sorted: vertices renumbered in the order the sorted
// faces first use them (faces, `tri`, positions and the caller-order map).
// `scratch` (reorder_scratch_bytes(nV) or more) may be shared by trees
// renumbered one after another on the same stream; nullptr: a private one.
static int reorder_vertices(oibvh_tree_t t, cudaStream_t s, void* scratch = nullptr)
{
    DevBuf<uint8_t> own;
    if (!scratch) {
        OK_TRY(own.ensure(reorder_scratch_bytes(t->nV), "cudaMalloc(reorder scratch)"));
        scratch = own.p;
    }
    OK_TRY(t->vperm.ensure(t->nV, "cudaMalloc(vertex order)"));
    CUDA_TRY(launch_reorder_vertices(t->face.p, t->tri.p, t->nT, t->nV, t->pos4.p, t->vperm.p, t->reordered,
                                     scratch, s));
    if (own.p) CUDA_TRY(cudaStreamSynchronize(s));  // the private scratch is freed on return
    t->reordered = true;
    return OIBVH_OK;
}

static int tree_build_impl(oibvh_tree_t t, cudaStream_t s)
{
    if (!t) return fail(OIBVH_ERR_ARG, "tree is NULL");
    DeviceGuard g(t->device);
    const uint32_t nT = t->nT;
    // scratch: bounds keys, codes, indices, sort buffers
    DevBuf<uint8_t> scratch;
    const bool wide = t->morton_bits == 63;
    const size_t sort_bytes = radix_sort_scratch_bytes(nT);
    const size_t arr = ((size_t)nT * 4 + 255) / 256 * 256;
    const size_t codes_off = 256, idx_off = codes_off + arr, hi_off = idx_off + arr, gath_off = hi_off + arr;
    const size_t sort_off = gath_off + arr;
    OK_TRY(scratch.ensure(sort_off + sort_bytes, "cudaMalloc(build scratch)"));
    uint32_t* keys6 = (uint32_t*)scratch.p;
    uint32_t* codes = (uint32_t*)(scratch.p + codes_off);
    uint32_t* idx = (uint32_t*)(scratch.p + idx_off);
    uint32_t* hi = (uint32_t*)(scratch.p + hi_off);
    uint32_t* hi_sorted = (uint32_t*)(scratch.p + gath_off);
    OK_TRY(sync_positions(t, s));
    CUDA_TRY(launch_mesh_bounds(t->cur_pos, t->nV, keys6, sm_count(t->device), s));
    CUDA_TRY(launch_leaf_morton(t->tri.p, t->cur_pos, nT, keys6, codes, idx, wide ? hi : nullptr, s));
    // stable LSD order by (key, original index): low key bits first, then the high ones
    CUDA_TRY(launch_radix_sort(codes, idx, nT, wide ? 32 : 30, scratch.p + sort_off, s));
    if (wide) {
        CUDA_TRY(launch_gather_u32(hi, idx, nT, hi_sorted, s));
        CUDA_TRY(launch_radix_sort(hi_sorted, idx, nT, 31, scratch.p + sort_off, s));
    }
    CUDA_TRY(launch_gather_faces(t->tri.p, idx, nT, t->face.p, s));
    OK_TRY(reorder_vertices(t, s));
    CUDA_TRY(launch_refit_one(t->job(), s));
    CUDA_TRY(cudaStreamSynchronize(s));
    t->built = true;
    return OIBVH_OK;
}

// ============================================================================
// Scene
// ============================================================================
struct oibvh_scene_s {
    int device = 0;
    std::vector<oibvh_tree_t> trees;
    bool all_pairs = true;
    std::vector<uint32_t> pairs;  // flattened (a, b)

    DevBuf<TreeView> views;
    DevBuf<PairView> pairv;
    DevBuf<uint64_t> front0, front1, cand;
    DevBuf<uint4> hits;
    DevBuf<uint32_t> counts;
    DevBuf<uint32_t> prec_lists;  // precision narrow phase: float-hit, recheck and FP64 lists (4 x cand_cap)
    DevBuf<double> fp64_tri;      // precision narrow phase: FP64 setups (kFp64TriRows x fp64_tri_cap)
    uint32_t fp64_tri_cap = 0;
    PinnedBuf<TreeView> h_views;
    PinnedBuf<PairView> h_pairs;
    PinnedBuf<uint32_t> h_counts;

    uint32_t front_cap = 1u << 20;
    uint32_t cand_cap = 1u << 20;
    uint32_t hit_cap = 1u << 18;

    // multi-tree refit: job table as last uploaded
    DevBuf<RefitJob> refit_jobs;
    DevBuf<uint32_t> refit_block_job;  // refit CTA -> job
    DevBuf<uint32_t> refit_counters;
    PinnedBuf<RefitJob> h_refit_jobs;
    std::vector<RefitJob> refit_cache;
    uint32_t refit_blocks = 0;

    // multi-tree build / transform: job table for the current tree list
    DevBuf<BuildJob> build_jobs;
    DevBuf<uint32_t> vblock_job, fblock_job;  // 256-vertex / 256-face block -> job
    DevBuf<uint32_t> bound_keys;
    std::vector<BuildJob> build_cache;
    uint32_t v_blocks = 0, f_blocks = 0, n_faces = 0, n_verts = 0;

    // tuning (oibvh_scene_set_tuning / oibvh_scene_autotune)
    uint32_t tune_start_log2 = 16;  // start cross product ~ 2^this node pairs per pass
    uint32_t tune_handoff = 2048;   // front width at which k_top hands over to the walkers
    uint32_t precision = 0;         // OIBVH_PRECISION_*
    uint32_t tune_walk_per_sm = 0;  // walker CTAs per SM, 0 = as many as fit
    uint32_t tune_walk_cap = 128;   // per-warp front entries of the walkers
    uint32_t tune_refit_log = 10;   // refit level-group depth (levels per CTA: 9, 10 or 11)
    uint32_t tune_descend = 16;     // both sides descend while the boxes' squared diagonals are within it
    uint32_t tune_claim = 1;        // walkers claim list items dynamically from this many per warp

    // captured frame (CUDA graph): [transform] + refit + detect
    cudaGraphExec_t frame_exec = nullptr;
    bool frame_stale = true;
    uint32_t frame_entry = 0, frame_expand = 1, frame_rounds = 3, frame_kernels = 0, frame_redos = 0;
    bool frame_refit = true;
    const float4* frame_rest = nullptr;
    DevBuf<float4> frame_rest_tree;  // frame_rest in each tree's vertex order (gathered at capture)
    const float* frame_mats = nullptr;
    PinnedBuf<uint32_t> h_frame_counts;
    cudaStream_t capture_stream = nullptr;  // private stream the frame is captured on
    DetectArgs frame_args{};                // the captured detect's arguments
    uint32_t frame_front0 = 0;              // its start cross product

    uint64_t hit_count = 0;
    uint64_t cand_count = 0;
    bool cands_valid = false;    // candidates of a single pass are on the device
    std::vector<PairView> last_pairs;
    oibvh_detect_stats stats{};

    ~oibvh_scene_s()
    {
        if (frame_exec) cudaGraphExecDestroy(frame_exec);
        if (capture_stream) cudaStreamDestroy(capture_stream);
    }
};

namespace {

struct PassPlan {
    std::vector<PairView> pv;
    uint64_t front0 = 0;
};

void list_pairs(const oibvh_scene_s* s, std::vector<uint32_t>& out)
{
    out.clear();
    if (s->all_pairs) {
        const uint32_t n = (uint32_t)s->trees.size();
        for (uint32_t i = 0; i < n; ++i)
            for (uint32_t j = i + 1; j < n; ++j) {
                out.push_back(i);
                out.push_back(j);
            }
    } else {
        out = s->pairs;
    }
}

TreeView view_of(const oibvh_tree_t t)
{
    TreeView v{};
    v.box = t->box.p;
    v.face = t->face.p;
    v.pos = t->cur_pos;
    v.shape = t->shape;
    v.nV = t->nV;
    return v;
}

// Start level of each pair: the reference's entry level, deepened so that
// the start cross products hold about 2^tune_start_log2 (default 2^16) node
// pairs over the pass, shared out in proportion to the pairs' triangle counts
// (the pair set does not depend on it; a deeper start gives the traversal
// enough independent work for every SM, and starting large pairs deeper
// keeps the work items of similar size).
int plan_pass(const oibvh_scene_s* s, const uint32_t* pr, uint32_t n, uint32_t entry, PassPlan& plan)
{
    plan.pv.resize(n);
    plan.front0 = 0;
    // the pass's start budget of 2^tune_start_log2 node pairs, shared out in
    // proportion to each pair's triangles: a large pair starts deeper, so the
    // work items handed to the walkers cover subtrees of similar size
    double total = 0.0;
    for (uint32_t p = 0; p < n; ++p)
        total += (double)s->trees[pr[2 * p]]->nT + (double)s->trees[pr[2 * p + 1]]->nT;
    const double budget = std::ldexp(1.0, (int)s->tune_start_log2);
    for (uint32_t p = 0; p < n; ++p) {
        const TreeShape& A = s->trees[pr[2 * p]]->shape;
        const TreeShape& B = s->trees[pr[2 * p + 1]]->shape;
        PairView v{};
        v.a = pr[2 * p];
        v.b = pr[2 * p + 1];
        v.ta = view_of(s->trees[v.a]);
        v.tb = view_of(s->trees[v.b]);
        const double share = budget * ((double)A.nT + (double)B.nT) / total;  // start pairs for this pair
        const uint32_t auto_level = share >= 4.0 ? (uint32_t)std::floor(std::log2(share) / 2.0) : 0u;
        const uint32_t start = std::max(entry, std::min(auto_level, kMaxLeafLevel));
        v.entry_a = std::min(start, A.L);
        v.entry_b = std::min(start, B.L);
        v.front_cnt_a = A.level_count(v.entry_a);
        v.front_cnt_b = B.level_count(v.entry_b);
        if (plan.front0 > 0x7fffffffull) return fail(OIBVH_ERR_ARG, "initial BVTT front exceeds 2^31 nodes");
        v.front_off = (uint32_t)plan.front0;
        plan.front0 += (uint64_t)v.front_cnt_a * v.front_cnt_b;
        plan.pv[p] = v;
    }
    if (plan.front0 > 0x7fffffffull) return fail(OIBVH_ERR_ARG, "initial BVTT front exceeds 2^31 nodes");
    return OIBVH_OK;
}

uint32_t grow_cap(uint64_t need, uint32_t cur)
{
    uint64_t c = std::max<uint64_t>(need + need / 4 + 1024, (uint64_t)cur * 2);
    if (c > 0x7fffffffull) c = 0x7fffffffull;
    return (uint32_t)c;
}

int upload_views(oibvh_scene_s* s, cudaStream_t st)
{
    const size_t n = s->trees.size();
    OK_TRY(s->h_views.ensure(n, "cudaMallocHost(views)"));
    OK_TRY(s->views.ensure(n, "cudaMalloc(views)"));
    CUDA_TRY(cudaStreamSynchronize(st));  // the pinned staging buffer may still feed an earlier copy
    for (size_t i = 0; i < n; ++i) {
        const oibvh_tree_t t = s->trees[i];
        TreeView v{};
        v.box = t->box.p;
        v.face = t->face.p;
        v.pos = t->cur_pos;
        v.shape = t->shape;
        v.nV = t->nV;
        s->h_views.p[i] = v;
    }
    CUDA_TRY(cudaMemcpyAsync(s->views.p, s->h_views.p, n * sizeof(TreeView), cudaMemcpyHostToDevice, st));
    return OIBVH_OK;
}

int walk_grid(const oibvh_scene_s* s, bool fused = true)
{
    const int fit = walk_blocks_per_sm(s->tune_walk_cap, fused);
    const int per = s->tune_walk_per_sm ? std::min<int>(fit, (int)s->tune_walk_per_sm) : fit;
    return sm_count(s->device) * std::max(1, per);
}

int narrow_pass(oibvh_scene_s* s, uint32_t np, uint64_t hits_before, cudaStream_t st);

// How detect_impl runs the narrow phase: fused into the traversal (float
// test), not at all (broad phase only, candidates kept), or as a separate
// kernel over each pass's candidates (precision mode: the filtered test
// runs at its own occupancy instead of holding the traversal's registers).
enum DetectMode { kDetectFused = 0, kDetectBroad = 1, kDetectSplit = 2 };
inline int full_detect_mode(const oibvh_scene_s* s) { return s->precision ? kDetectSplit : kDetectFused; }

// Broad phase (+ narrow phase unless kDetectBroad) over every pair, pass by pass.
int detect_impl(oibvh_scene_s* s, int device_type, uint32_t entry, uint32_t expand, int mode, cudaStream_t st)
{
    const bool narrow = mode == kDetectFused;  // narrow phase inside the traversal kernels
    if (device_type < 0)
        return fail(OIBVH_ERR_UNSUPPORTED,
                    "device type CPU: the reference's detectCollisionOnCPU is empty; this library has no CPU path");
    if (device_type != s->device) return fail(OIBVH_ERR_ARG, "device type does not match the scene's device");
    if (expand < 1 || expand > 16) return fail(OIBVH_ERR_ARG, "expand_levels must be in 1..16");
    for (auto t : s->trees)
        if (!t->built) return fail(OIBVH_ERR_STATE, "every tree must be built before detect");
    DeviceGuard g(s->device);
    struct StaleIfMoved {
        oibvh_scene_s* s;
        const void* p[6];
        explicit StaleIfMoved(oibvh_scene_s* sc)
            : s(sc), p{sc->front0.p, sc->front1.p, sc->hits.p, sc->counts.p, sc->pairv.p, sc->views.p}
        {
        }
        ~StaleIfMoved()
        {
            const void* q[6] = {s->front0.p, s->front1.p, s->hits.p, s->counts.p, s->pairv.p, s->views.p};
            for (int i = 0; i < 6; ++i)
                if (p[i] != q[i]) s->frame_stale = true;
        }
    } stale_guard(s);
    s->stats = oibvh_detect_stats{};
    s->hit_count = 0;
    s->cand_count = 0;
    s->cands_valid = false;
    std::vector<uint32_t> pr;
    list_pairs(s, pr);
    const uint32_t n_pairs = (uint32_t)(pr.size() / 2);
    for (uint32_t i = 0; i < n_pairs; ++i)
        if (pr[2 * i] >= s->trees.size() || pr[2 * i + 1] >= s->trees.size() || pr[2 * i] == pr[2 * i + 1])
            return fail(OIBVH_ERR_ARG, "pair list refers to a missing tree or pairs a tree with itself");
    if (n_pairs == 0) return OIBVH_OK;
    OK_TRY(upload_views(s, st));
    OK_TRY(s->hits.ensure(s->hit_cap, "cudaMalloc(hits)"));

    const int grid = walk_grid(s, narrow);
    for (uint32_t p0 = 0; p0 < n_pairs; p0 += kMaxPairsPerPass) {
        const uint32_t np = std::min(kMaxPairsPerPass, n_pairs - p0);
        PassPlan plan;
        OK_TRY(plan_pass(s, pr.data() + 2 * (size_t)p0, np, entry, plan));
        OK_TRY(s->counts.ensure(kCountTotal, "cudaMalloc(counts)"));
        OK_TRY(s->h_counts.ensure(kCountTotal, "cudaMallocHost(counts)"));
        OK_TRY(s->h_pairs.ensure(np, "cudaMallocHost(pairs)"));
        OK_TRY(s->pairv.ensure(np, "cudaMalloc(pairs)"));
        CUDA_TRY(cudaStreamSynchronize(st));
        std::memcpy(s->h_pairs.p, plan.pv.data(), np * sizeof(PairView));
        CUDA_TRY(cudaMemcpyAsync(s->pairv.p, s->h_pairs.p, np * sizeof(PairView), cudaMemcpyHostToDevice, st));
        const uint64_t hits_before = s->hit_count;
        for (int attempt = 0;; ++attempt) {
            if (attempt > 12) return fail(OIBVH_ERR_OVERFLOW, "BVTT queues kept overflowing after regrowing");
            OK_TRY(s->front0.ensure(s->front_cap, "cudaMalloc(work list)"));
            OK_TRY(s->front1.ensure(s->front_cap, "cudaMalloc(work list)"));
            if (!narrow) OK_TRY(s->cand.ensure(s->cand_cap, "cudaMalloc(candidates)"));
            CUDA_TRY(cudaMemsetAsync(s->counts.p, 0, kCountTotal * sizeof(uint32_t), st));
            if (hits_before) {
                s->h_counts.p[0] = (uint32_t)hits_before;
                CUDA_TRY(cudaMemcpyAsync(s->counts.p, s->h_counts.p, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            }
            DetectArgs a{};
            a.trees = s->views.p;
            a.pairs = s->pairv.p;
            a.n_pairs = np;
            a.expand_levels = 1;
            a.work[0] = s->front0.p;
            a.work[1] = s->front1.p;
            a.work_cap = s->front_cap;
            a.cand = narrow ? nullptr : s->cand.p;
            a.cand_cap = narrow ? 0 : s->cand_cap;
            a.hits = s->hits.p;
            a.hit_cap = s->hit_cap;
            a.counts = s->counts.p;
            a.fuse_narrow = narrow ? 1u : 0u;
            a.grid = grid;
            a.handoff = s->tune_handoff;
            a.walk_cap = s->tune_walk_cap;
            a.precision = s->precision;
            a.descend_ratio = (float)s->tune_descend;
            a.claim_min = s->tune_claim;
            CUDA_TRY(launch_init_front(a, (uint32_t)plan.front0, st));
            CUDA_TRY(launch_top(a, st));
            uint32_t rounds = 1;  // list 1 is the first walk round's input
            for (;;) {
                // two walk rounds go out with the first read-back; later ones one by one
                const uint32_t upto = std::min(kMaxRounds, rounds == 1 ? 3u : rounds + 1);
                for (; rounds < upto; ++rounds) CUDA_TRY(launch_walk(a, rounds, st));
                CUDA_TRY(cudaMemcpyAsync(s->h_counts.p, s->counts.p, kCountTotal * sizeof(uint32_t),
                                         cudaMemcpyDeviceToHost, st));
                CUDA_TRY(cudaStreamSynchronize(st));
                const uint32_t* c = s->h_counts.p;
                if (c[kCountFlags] || c[kCountWork0 + rounds] == 0) break;
                if (rounds >= kMaxRounds) return fail(OIBVH_ERR_OVERFLOW, "BVTT traversal needed too many rounds");
            }
            const uint32_t* c = s->h_counts.p;
            const uint32_t flags = c[kCountFlags];
            uint64_t peak = 0;
            for (uint32_t k = 0; k <= rounds; ++k) peak = std::max<uint64_t>(peak, c[kCountWork0 + k]);
            if (flags) {
                s->stats.retries++;
                if (flags & kFlagFrontOverflow) s->front_cap = grow_cap(peak, s->front_cap);
                if (flags & kFlagCandOverflow) s->cand_cap = grow_cap(c[kCountCandSlots], s->cand_cap);
                if (flags & kFlagHitOverflow) {
                    const uint32_t want = grow_cap(c[kCountHits], s->hit_cap);
                    OK_TRY(s->hits.grow_keep(want, hits_before, st, "cudaMalloc(hits)"));
                    s->hit_cap = want;
                }
                continue;
            }
            s->stats.nodes_tested += c[kCountTested];
            s->stats.fp64_axes += c[kCountFp64Axes];
            s->stats.fp64_candidates += c[kCountFp64Cands];
            s->stats.fp32_disagreements += c[kCountDisagree];
            s->stats.front_peak = std::max(s->stats.front_peak, peak);
            s->stats.steps = rounds;
            s->cand_count += c[kCountCands];
            if (narrow) s->hit_count = c[kCountHits];
            break;
        }
        s->stats.passes++;
        if (mode == kDetectSplit) {
            OK_TRY(narrow_pass(s, np, hits_before, st));
        } else if (!narrow) {
            if (n_pairs > kMaxPairsPerPass)
                return fail(OIBVH_ERR_UNSUPPORTED, "the split broad phase handles at most 16384 pairs");
            s->last_pairs = plan.pv;
            s->cands_valid = true;
        }
    }
    s->stats.candidates = s->cand_count;
    s->stats.hits = s->hit_count;
    return OIBVH_OK;
}

// Room for the FP64 setups of the next passes: twice the list the
// double-float pass left to FP64 this time (the first pass forms every setup
// where it is used). A captured frame that used the old buffer is captured
// again.
int size_fp64_setups(oibvh_scene_s* s, uint32_t fp64_list)
{
    const uint64_t want = std::min<uint64_t>(2ull * fp64_list, s->cand_cap);
    if (want <= s->fp64_tri_cap) return OIBVH_OK;
    const uint32_t cap = grow_cap((uint32_t)want, s->fp64_tri_cap);
    OK_TRY(s->fp64_tri.ensure((size_t)kFp64TriRows * cap, "cudaMalloc(FP64 setups)"));
    s->fp64_tri_cap = cap;
    s->frame_stale = true;
    return OIBVH_OK;
}

// Narrow phase over the stored candidates of the last broad pass (pairv holds
// that pass's pair table); hits are appended after the first `hits_before`.
int narrow_pass(oibvh_scene_s* s, uint32_t np, uint64_t hits_before, cudaStream_t st)
{
    for (int attempt = 0;; ++attempt) {
        if (attempt > 12) return fail(OIBVH_ERR_OVERFLOW, "hit queue kept overflowing");
        // counts[kCountCandSlots] still holds the candidate count of the broad phase;
        // hits (from hits_before), flags and the precision-mode counters are reset
        std::memset(s->h_counts.p, 0, kCountWork0 * sizeof(uint32_t));
        s->h_counts.p[kCountHits] = (uint32_t)hits_before;
        CUDA_TRY(cudaMemcpyAsync(s->counts.p, s->h_counts.p, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(s->counts.p + kCountFp64Axes, s->h_counts.p + kCountFp64Axes,
                                 (kCountWork0 - kCountFp64Axes) * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        const void* lists_before = s->prec_lists.p;
        if (s->precision) OK_TRY(s->prec_lists.ensure(4 * (size_t)s->cand_cap, "cudaMalloc(precision lists)"));
        if (s->prec_lists.p != lists_before) s->frame_stale = true;  // a captured frame used the old lists
        DetectArgs a{};
        a.precision = s->precision;
        a.prec_lists = s->precision ? s->prec_lists.p : nullptr;
        a.trees = s->views.p;
        a.pairs = s->pairv.p;
        a.n_pairs = np;
        a.cand = s->cand.p;
        a.cand_cap = s->cand_cap;
        a.hits = s->hits.p;
        a.hit_cap = s->hit_cap;
        a.counts = s->counts.p;
        a.grid = sm_count(s->device) * 8;
        a.fuse_narrow = 1;
        if (s->precision) {
            a.fp64_tri = s->fp64_tri.p;
            a.fp64_tri_cap = s->fp64_tri_cap;
        }
        CUDA_TRY(launch_narrow(a, st));
        CUDA_TRY(cudaMemcpyAsync(s->h_counts.p, s->counts.p, kCountTotal * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                 st));
        CUDA_TRY(cudaStreamSynchronize(st));
        const uint32_t* c = s->h_counts.p;
        if (c[kCountFlags] & kFlagHitOverflow) {
            const uint32_t want = grow_cap(c[kCountHits], s->hit_cap);
            OK_TRY(s->hits.grow_keep(want, hits_before, st, "cudaMalloc(hits)"));
            s->hit_cap = want;
            continue;
        }
        s->hit_count = c[kCountHits];
        s->stats.hits = s->hit_count;
        s->stats.fp64_axes += c[kCountFp64Axes];
        s->stats.fp64_candidates += c[kCountFp64Cands];
        s->stats.fp32_disagreements += c[kCountDisagree];
        s->stats.bounded_candidates += (uint64_t)c[kCountPrecHits] + c[kCountPrecRecheck];
        if (s->precision) OK_TRY(size_fp64_setups(s, c[kCountPrecLeft]));
        return OIBVH_OK;
    }
}

int narrow_impl(oibvh_scene_s* s, cudaStream_t st)
{
    if (!s->cands_valid) return fail(OIBVH_ERR_STATE, "narrow phase needs a broad phase first");
    DeviceGuard g(s->device);
    s->stats.fp64_axes = s->stats.fp64_candidates = s->stats.fp32_disagreements = s->stats.bounded_candidates = 0;
    return narrow_pass(s, (uint32_t)s->last_pairs.size(), 0, st);
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
#define API extern "C" __attribute__((visibility("default")))

#define GUARD_BEGIN try {
#define GUARD_END                                                   \
    }                                                               \
    catch (const std::bad_alloc&)                                   \
    {                                                               \
        return fail(OIBVH_ERR_OOM, "host allocation failed");       \
    }                                                               \
    catch (...)                                                     \
    {                                                               \
        return fail(OIBVH_ERR_CUDA, "unexpected C++ exception");    \
    }

API const char* oibvh_status_string(int status)
{
    switch (status) {
    case OIBVH_OK: return "ok";
    case OIBVH_ERR_ARG: return "invalid argument";
    case OIBVH_ERR_OOM: return "out of memory";
    case OIBVH_ERR_CUDA: return "CUDA error";
    case OIBVH_ERR_OVERFLOW: return "queue overflow";
    case OIBVH_ERR_STATE: return "invalid state";
    case OIBVH_ERR_UNSUPPORTED: return "unsupported";
    case OIBVH_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

API const char* oibvh_last_error(void) { return g_last_error.c_str(); }

API int oibvh_version(void) { return 100; }

API uint64_t oibvh_get_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

API int oibvh_debug_fail_alloc_after(int64_t n)
{
    g_fail_alloc.store(n < 0 ? -1 : n, std::memory_order_relaxed);
    return OIBVH_OK;
}

API uint64_t oibvh_debug_alloc_attempts(void) { return g_alloc_attempts.load(std::memory_order_relaxed); }

API int oibvh_tree_create(const float* xyz, uint32_t n_vertices, const uint32_t* tri, uint32_t n_triangles, int device,
                          oibvh_tree_t* out)
{
    GUARD_BEGIN
    return tree_create_impl(xyz, n_vertices, tri, n_triangles, device, out);
    GUARD_END
}

API int oibvh_tree_create_copy(oibvh_tree_t other, const float* xyz, uint32_t n_vertices, oibvh_tree_t* out)
{
    GUARD_BEGIN
    if (!out) return fail(OIBVH_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!other || !xyz) return fail(OIBVH_ERR_ARG, "other or xyz is NULL");
    if (!other->built) return fail(OIBVH_ERR_STATE, "the source tree is not built");
    if (n_vertices != other->nV) return fail(OIBVH_ERR_ARG, "vertex count differs from the source mesh");
    DeviceGuard g(other->device);
    oibvh_tree_t t = new oibvh_tree_s();
    t->device = other->device;
    t->nV = other->nV;
    t->nT = other->nT;
    t->shape = other->shape;
    int st = tree_alloc(t);
    if (st == OIBVH_OK) {
        cudaError_t e = cudaSuccess;
        if (other->reordered) {
            e = t->vperm.ensure(t->nV, "cudaMalloc(vertex order)") == OIBVH_OK ? cudaSuccess : cudaErrorMemoryAllocation;
            if (e == cudaSuccess)
                e = cudaMemcpy(t->vperm.p, other->vperm.p, (size_t)t->nV * sizeof(uint32_t), cudaMemcpyDeviceToDevice);
            t->reordered = true;
        }
        if (e == cudaSuccess) e = cudaMemcpy(t->xyz.p, xyz, 3 * (size_t)t->nV * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launch_xyz_to_pos4(t->xyz.p, t->vmap(), t->nV, t->pos4.p, 0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);
        if (e == cudaSuccess)
            e = cudaMemcpy(t->tri.p, other->tri.p, 3 * (size_t)t->nT * sizeof(uint32_t), cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(t->face.p, other->face.p, (size_t)t->nT * sizeof(uint4), cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(t->box.p, other->box.p, 2 * (size_t)(t->shape.size - t->nT) * sizeof(float4),
                           cudaMemcpyDeviceToDevice);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpy(copy tree)");
    }
    if (st != OIBVH_OK) {
        delete t;
        return st;
    }
    t->cur_pos = t->pos4.p;
    t->built = true;  // the copied boxes describe `other`'s positions until refit
    *out = t;
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_tree_build(oibvh_tree_t t, void* stream)
{
    GUARD_BEGIN
    return tree_build_impl(t, (cudaStream_t)stream);
    GUARD_END
}

// Positions as given (xyz, host or device) into the tree's own device layout.
static int stage_xyz(oibvh_tree_t t, const float* xyz, bool on_device, cudaStream_t s)
{
    const float* src = xyz;
    if (!on_device) {
        CUDA_TRY(cudaMemcpyAsync(t->xyz.p, xyz, 3 * (size_t)t->nV * sizeof(float), cudaMemcpyHostToDevice, s));
        src = t->xyz.p;
    }
    CUDA_TRY(launch_xyz_to_pos4(src, t->vmap(), t->nV, t->pos4.p, s));
    t->cur_pos = t->pos4.p;
    t->borrowed = nullptr;
    return OIBVH_OK;
}

static int check_device_ptr(const void* p, size_t align)
{
    cudaPointerAttributes attr{};
    CUDA_TRY(cudaPointerGetAttributes(&attr, p));
    if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
        return fail(OIBVH_ERR_ARG, "pointer is not device memory");
    if (((uintptr_t)p) % align) return fail(OIBVH_ERR_ARG, "pointer is not aligned to " + std::to_string(align));
    return OIBVH_OK;
}

API int oibvh_tree_refit(oibvh_tree_t t, const float* xyz, void* stream)
{
    GUARD_BEGIN
    if (!t) return fail(OIBVH_ERR_ARG, "tree is NULL");
    if (!t->built) return fail(OIBVH_ERR_STATE, "refit before build");
    DeviceGuard g(t->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (xyz) OK_TRY(stage_xyz(t, xyz, false, s));
    else OK_TRY(sync_positions(t, s));
    CUDA_TRY(launch_refit_one(t->job(), s));
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_tree_refit_device(oibvh_tree_t t, const float* d_xyz, void* stream)
{
    GUARD_BEGIN
    if (!t || !d_xyz) return fail(OIBVH_ERR_ARG, "tree or d_xyz is NULL");
    if (!t->built) return fail(OIBVH_ERR_STATE, "refit before build");
    DeviceGuard g(t->device);
    OK_TRY(check_device_ptr(d_xyz, 4));
    OK_TRY(stage_xyz(t, d_xyz, true, (cudaStream_t)stream));
    CUDA_TRY(launch_refit_one(t->job(), (cudaStream_t)stream));
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_tree_set_positions(oibvh_tree_t t, const float* xyz, void* stream)
{
    GUARD_BEGIN
    if (!t || !xyz) return fail(OIBVH_ERR_ARG, "tree or xyz is NULL");
    DeviceGuard g(t->device);
    return stage_xyz(t, xyz, false, (cudaStream_t)stream);
    GUARD_END
}

API int oibvh_tree_set_positions_device(oibvh_tree_t t, const float* d_xyz, void* stream)
{
    GUARD_BEGIN
    if (!t || !d_xyz) return fail(OIBVH_ERR_ARG, "tree or d_xyz is NULL");
    DeviceGuard g(t->device);
    OK_TRY(check_device_ptr(d_xyz, 4));
    return stage_xyz(t, d_xyz, true, (cudaStream_t)stream);
    GUARD_END
}

API int oibvh_tree_set_positions4_device(oibvh_tree_t t, const float* d_xyzw)
{
    GUARD_BEGIN
    if (!t || !d_xyzw) return fail(OIBVH_ERR_ARG, "tree or d_xyzw is NULL");
    DeviceGuard g(t->device);
    OK_TRY(check_device_ptr(d_xyzw, 16));
    t->borrowed = (const float4*)d_xyzw;  // read (in the tree's vertex order) by every following refit
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_tree_set_morton_bits(oibvh_tree_t t, uint32_t bits)
{
    if (!t) return fail(OIBVH_ERR_ARG, "tree is NULL");
    if (bits != 30 && bits != 63) return fail(OIBVH_ERR_ARG, "Morton key width must be 30 or 63 bits");
    t->morton_bits = bits;
    return OIBVH_OK;
}

API uint32_t oibvh_tree_get_morton_bits(oibvh_tree_t t) { return t ? t->morton_bits : 0; }

API uint32_t oibvh_tree_get_depth(oibvh_tree_t t) { return t ? ilog2(t->shape.size) : 0; }
API uint32_t oibvh_tree_get_prim_count(oibvh_tree_t t) { return t ? t->nT : 0; }
API uint32_t oibvh_tree_get_size(oibvh_tree_t t) { return t ? t->shape.size : 0; }

API int oibvh_tree_get_aabbs(oibvh_tree_t t, float* out6, uint64_t cap_nodes)
{
    GUARD_BEGIN
    if (!t || !out6) return fail(OIBVH_ERR_ARG, "tree or out6 is NULL");
    if (!t->built) return fail(OIBVH_ERR_STATE, "tree not built");
    DeviceGuard g(t->device);
    const size_t internal = t->shape.size - t->nT;
    const size_t n = std::min<uint64_t>(cap_nodes, t->shape.size);
    std::vector<float4> tmp(2 * (size_t)t->shape.size);
    CUDA_TRY(cudaDeviceSynchronize());
    if (internal)
        CUDA_TRY(cudaMemcpy(tmp.data(), t->box.p, 2 * internal * sizeof(float4), cudaMemcpyDeviceToHost));
    {
        // leaves are not stored: rebuild them from the faces and positions
        DevBuf<float4> leaves;
        OK_TRY(leaves.ensure(2 * (size_t)t->nT, "cudaMalloc(leaf boxes)"));
        CUDA_TRY(launch_leaf_boxes(t->face.p, t->cur_pos, t->nT, leaves.p, 0));
        CUDA_TRY(cudaMemcpy(tmp.data() + 2 * internal, leaves.p, 2 * (size_t)t->nT * sizeof(float4),
                            cudaMemcpyDeviceToHost));
    }
    for (size_t i = 0; i < n; ++i) {
        out6[6 * i + 0] = tmp[2 * i].x;
        out6[6 * i + 1] = tmp[2 * i].y;
        out6[6 * i + 2] = tmp[2 * i].z;
        out6[6 * i + 3] = tmp[2 * i + 1].x;
        out6[6 * i + 4] = tmp[2 * i + 1].y;
        out6[6 * i + 5] = tmp[2 * i + 1].z;
    }
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_tree_get_sorted_faces(oibvh_tree_t t, uint32_t* out3, uint32_t* perm, uint64_t cap)
{
    GUARD_BEGIN
    if (!t) return fail(OIBVH_ERR_ARG, "tree is NULL");
    if (!t->built) return fail(OIBVH_ERR_STATE, "tree not built");
    DeviceGuard g(t->device);
    const size_t n = std::min<uint64_t>(cap, t->nT);
    std::vector<uint4> tmp(n);
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemcpy(tmp.data(), t->face.p, n * sizeof(uint4), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> vp;  // the tree's vertex numbering back to the caller's
    if (out3 && t->reordered) {
        vp.resize(t->nV);
        CUDA_TRY(cudaMemcpy(vp.data(), t->vperm.p, (size_t)t->nV * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    }
    auto caller = [&](uint32_t v) { return vp.empty() ? v : vp[v]; };
    for (size_t i = 0; i < n; ++i) {
        if (out3) {
            out3[3 * i] = caller(tmp[i].x);
            out3[3 * i + 1] = caller(tmp[i].y);
            out3[3 * i + 2] = caller(tmp[i].z);
        }
        if (perm) perm[i] = tmp[i].w;
    }
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_tree_destroy(oibvh_tree_t t)
{
    if (!t) return OIBVH_OK;
    {
        DeviceGuard g(t->device);
        delete t;
    }
    return OIBVH_OK;
}

API int oibvh_scene_create(int device, oibvh_scene_t* out)
{
    GUARD_BEGIN
    if (!out) return fail(OIBVH_ERR_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(OIBVH_ERR_ARG, "no such device");
    oibvh_scene_t s = new oibvh_scene_s();
    s->device = device;
    *out = s;
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_add_tree(oibvh_scene_t s, oibvh_tree_t t, uint32_t* id)
{
    GUARD_BEGIN
    if (!s || !t) return fail(OIBVH_ERR_ARG, "scene or tree is NULL");
    if (t->device != s->device) return fail(OIBVH_ERR_ARG, "tree lives on another device");
    // the reference asserts a built tree (src/cuda/scene.cu:97); here a tree may
    // also be added unbuilt and built with the others by oibvh_scene_build
    s->trees.push_back(t);
    s->frame_stale = true;
    if (id) *id = (uint32_t)(s->trees.size() - 1);
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_set_pairs(oibvh_scene_t s, const uint32_t* pairs, uint32_t n_pairs)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (!pairs) {
        s->all_pairs = true;
        s->pairs.clear();
        s->frame_stale = true;
        return OIBVH_OK;
    }
    for (uint32_t i = 0; i < n_pairs; ++i)
        if (pairs[2 * i] >= s->trees.size() || pairs[2 * i + 1] >= s->trees.size() || pairs[2 * i] == pairs[2 * i + 1])
            return fail(OIBVH_ERR_ARG, "pair " + std::to_string(i) + " is not two distinct trees of this scene");
    s->all_pairs = false;
    s->pairs.assign(pairs, pairs + 2 * (size_t)n_pairs);
    s->frame_stale = true;
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_detect(oibvh_scene_t s, int device_type, uint32_t entry_level, uint32_t expand_levels,
                           void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    return detect_impl(s, device_type, entry_level, expand_levels, full_detect_mode(s), (cudaStream_t)stream);
    GUARD_END
}

API int oibvh_scene_broad(oibvh_scene_t s, int device_type, uint32_t entry_level, uint32_t expand_levels, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    return detect_impl(s, device_type, entry_level, expand_levels, kDetectBroad, (cudaStream_t)stream);
    GUARD_END
}

API int oibvh_scene_narrow(oibvh_scene_t s, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    return narrow_impl(s, (cudaStream_t)stream);
    GUARD_END
}

API int oibvh_scene_refit(oibvh_scene_t s, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = s->trees.size();
    if (n == 0) return OIBVH_OK;
    std::vector<RefitJob> jobs(n);
    uint32_t blocks = 0;
    for (size_t i = 0; i < n; ++i) {
        const oibvh_tree_t t = s->trees[i];
        if (!t->built) return fail(OIBVH_ERR_STATE, "every tree must be built before refit");
        OK_TRY(sync_positions(t, st));
        RefitJob j = t->job();
        j.n_blocks = refit_blocks_for(t->nT, s->tune_refit_log);
        j.block_begin = blocks;
        j.counters = nullptr;  // filled below
        blocks += j.n_blocks;
        jobs[i] = j;
    }
    const size_t per = refit_counters_per_tree();
    OK_TRY(s->refit_counters.ensure(per * n, "cudaMalloc(refit counters)"));
    for (size_t i = 0; i < n; ++i) jobs[i].counters = s->refit_counters.p + per * i;
    bool same = s->refit_cache.size() == n && s->refit_jobs.p;
    for (size_t i = 0; same && i < n; ++i) same = std::memcmp(&jobs[i], &s->refit_cache[i], sizeof(RefitJob)) == 0;
    if (!same) {
        OK_TRY(s->refit_jobs.ensure(n, "cudaMalloc(refit jobs)"));
        OK_TRY(s->h_refit_jobs.ensure(n, "cudaMallocHost(refit jobs)"));
        OK_TRY(s->refit_block_job.ensure(std::max(1u, blocks), "cudaMalloc(refit block map)"));
        CUDA_TRY(cudaStreamSynchronize(st));  // the staging buffer may feed an earlier copy
        std::memcpy(s->h_refit_jobs.p, jobs.data(), n * sizeof(RefitJob));
        CUDA_TRY(cudaMemcpyAsync(s->refit_jobs.p, s->h_refit_jobs.p, n * sizeof(RefitJob), cudaMemcpyHostToDevice, st));
        std::vector<uint32_t> map(blocks);
        for (size_t i = 0; i < n; ++i)
            std::fill(map.begin() + jobs[i].block_begin, map.begin() + jobs[i].block_begin + jobs[i].n_blocks,
                      (uint32_t)i);
        CUDA_TRY(cudaMemcpyAsync(s->refit_block_job.p, map.data(), blocks * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                 st));
        CUDA_TRY(cudaStreamSynchronize(st));  // map is a pageable host vector
        s->refit_cache = jobs;
    }
    s->refit_blocks = blocks;
    CUDA_TRY(launch_refit(s->refit_jobs.p, (uint32_t)n, blocks, s->refit_block_job.p, s->refit_counters.p, per * n,
                          s->tune_refit_log, st));
    return OIBVH_OK;
    GUARD_END
}

API uint32_t oibvh_scene_get_int_tri_pair_count(oibvh_scene_t s) { return s ? (uint32_t)s->hit_count : 0; }
API uint64_t oibvh_scene_get_candidate_count(oibvh_scene_t s) { return s ? s->cand_count : 0; }

API int oibvh_scene_get_int_tri_pairs(oibvh_scene_t s, uint32_t* out4, uint64_t cap, uint64_t* n)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (n) *n = s->hit_count;
    const uint64_t k = std::min(cap, s->hit_count);
    if (k == 0) return OIBVH_OK;
    if (!out4) return fail(OIBVH_ERR_ARG, "out4 is NULL");
    DeviceGuard g(s->device);
    CUDA_TRY(cudaMemcpy(out4, s->hits.p, k * sizeof(uint4), cudaMemcpyDeviceToHost));
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_get_candidates(oibvh_scene_t s, uint32_t* out4, uint64_t cap, uint64_t* n)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (!s->cands_valid) return fail(OIBVH_ERR_STATE, "no broad phase result (use oibvh_scene_broad)");
    if (n) *n = s->cand_count;
    const uint64_t k = std::min(cap, s->cand_count);
    if (k == 0) return OIBVH_OK;
    if (!out4) return fail(OIBVH_ERR_ARG, "out4 is NULL");
    DeviceGuard g(s->device);
    std::vector<uint64_t> tmp(k);
    CUDA_TRY(cudaMemcpy(tmp.data(), s->cand.p, k * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < k; ++i) {
        const PairView& pv = s->last_pairs[bvtt_pair(tmp[i])];
        out4[4 * i + 0] = pv.a;
        out4[4 * i + 1] = pv.b;
        out4[4 * i + 2] = bvtt_a(tmp[i]);
        out4[4 * i + 3] = bvtt_b(tmp[i]);
    }
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_set_queue_capacity(oibvh_scene_t s, uint32_t front, uint32_t candidates, uint32_t hits)
{
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (front > 0x7fffffffu || candidates > 0x7fffffffu || hits > 0x7fffffffu)
        return fail(OIBVH_ERR_ARG, "capacity above 2^31");
    // shrinking the hit queue would drop hits of the last detect
    if (front) {
        s->front_cap = front;
        s->front0.release();
        s->front1.release();
    }
    if (candidates) {
        s->cand_cap = candidates;
        s->cand.release();
        s->cands_valid = false;
    }
    if (hits) {
        s->hit_cap = hits;
        s->hits.release();
        s->hit_count = 0;
    }
    s->frame_stale = true;  // a captured frame points at the released buffers
    return OIBVH_OK;
}

API int oibvh_scene_set_precision(oibvh_scene_t s, int mode)
{
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (mode != OIBVH_PRECISION_FP32 && mode != OIBVH_PRECISION_FP64_FILTERED)
        return fail(OIBVH_ERR_ARG, "unknown precision mode");
    if ((uint32_t)mode != s->precision) s->frame_stale = true;
    s->precision = (uint32_t)mode;
    return OIBVH_OK;
}

API int oibvh_scene_get_precision(oibvh_scene_t s) { return s ? (int)s->precision : -1; }

API int oibvh_scene_get_stats(oibvh_scene_t s, oibvh_detect_stats* out)
{
    if (!s || !out) return fail(OIBVH_ERR_ARG, "scene or out is NULL");
    *out = s->stats;
    out->frame_redos = s->frame_redos;
    return OIBVH_OK;
}

API int oibvh_scene_destroy(oibvh_scene_t s)
{
    if (!s) return OIBVH_OK;
    {
        DeviceGuard g(s->device);
        delete s;
    }
    return OIBVH_OK;
}

// ============================================================================
// Used by oibvh_pair_detect_noalloc (noalloc.cu)
// ============================================================================
namespace oibvh {

int tree_device_view(oibvh_tree_t t, TreeView* out, int* device, bool* built)
{
    TreeView v{};
    v.box = t->box.p;
    v.face = t->face.p;
    v.pos = t->cur_pos;
    v.shape = t->shape;
    v.nV = t->nV;
    *out = v;
    *device = t->device;
    *built = t->built;
    return OIBVH_OK;
}

int noalloc_fail(int code, const std::string& msg) { return fail(code, msg); }

}  // namespace oibvh

// ============================================================================
// Multi-tree build, transforms, tuning and the captured frame
// ============================================================================
namespace {

// (Re)build the job table of the multi-tree build / transform launches.
int ensure_build_jobs(oibvh_scene_s* s, cudaStream_t st)
{
    const size_t n = s->trees.size();
    std::vector<BuildJob> jobs(n);
    uint32_t vb = 0, fb = 0, fo = 0, vo = 0;
    OK_TRY(s->bound_keys.ensure(6 * std::max<size_t>(n, 1), "cudaMalloc(bounds)"));
    for (size_t i = 0; i < n; ++i) {
        const oibvh_tree_t t = s->trees[i];
        BuildJob j{};
        j.pos = t->cur_pos;
        j.tri = t->tri.p;
        j.face_out = t->face.p;
        j.bound_keys = s->bound_keys.p + 6 * i;
        j.pos_out = t->pos4.p;
        j.nV = t->nV;
        j.nT = t->nT;
        j.vblock_begin = vb;
        j.fblock_begin = fb;
        j.face_off = fo;
        j.vert_off = vo;
        j.vperm = t->vmap();
        j.vperm_out = t->vperm.p;
        j.tri_rw = t->tri.p;
        vb += (t->nV + 255) / 256;
        fb += (t->nT + 255) / 256;
        if ((uint64_t)fo + t->nT > 0xffffffffull || (uint64_t)vo + t->nV > 0xffffffffull)
            return fail(OIBVH_ERR_ARG, "the scene holds more than 2^32 faces or vertices");
        fo += t->nT;
        vo += t->nV;
        jobs[i] = j;
    }
    s->v_blocks = vb;
    s->f_blocks = fb;
    s->n_faces = fo;
    s->n_verts = vo;
    bool same = s->build_cache.size() == n && s->build_jobs.p;
    for (size_t i = 0; same && i < n; ++i) same = std::memcmp(&jobs[i], &s->build_cache[i], sizeof(BuildJob)) == 0;
    if (!same) {
        OK_TRY(s->build_jobs.ensure(std::max<size_t>(n, 1), "cudaMalloc(build jobs)"));
        OK_TRY(s->vblock_job.ensure(std::max(1u, vb), "cudaMalloc(vertex block map)"));
        OK_TRY(s->fblock_job.ensure(std::max(1u, fb), "cudaMalloc(face block map)"));
        std::vector<uint32_t> vmap(vb), fmap(fb);
        for (size_t i = 0; i < n; ++i) {
            const oibvh_tree_t t = s->trees[i];
            std::fill(vmap.begin() + jobs[i].vblock_begin, vmap.begin() + jobs[i].vblock_begin + (t->nV + 255) / 256,
                      (uint32_t)i);
            std::fill(fmap.begin() + jobs[i].fblock_begin, fmap.begin() + jobs[i].fblock_begin + (t->nT + 255) / 256,
                      (uint32_t)i);
        }
        CUDA_TRY(cudaMemcpyAsync(s->build_jobs.p, jobs.data(), n * sizeof(BuildJob), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(s->vblock_job.p, vmap.data(), vb * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(s->fblock_job.p, fmap.data(), fb * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));  // jobs and the maps are pageable host vectors
        s->build_cache = jobs;
    }
    return OIBVH_OK;
}

}  // namespace

API int oibvh_scene_build(oibvh_scene_t s, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (s->trees.empty()) return OIBVH_OK;
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    for (auto t : s->trees) OK_TRY(sync_positions(t, st));
    OK_TRY(ensure_build_jobs(s, st));
    DevBuf<uint8_t> scratch;  // the build stages, then (in stream order) the renumbering
    OK_TRY(scratch.ensure(std::max(build_multi_scratch_bytes(s->n_faces),
                                   reorder_multi_scratch_bytes(s->n_verts, s->v_blocks, s->f_blocks)),
                          "cudaMalloc(build scratch)"));
    const uint32_t n = (uint32_t)s->trees.size();
    const uint32_t tree_bits = n <= 1 ? 0u : ilog2(next_pow2(n));
    const bool wide = s->trees[0]->morton_bits == 63;
    for (auto t : s->trees)
        if ((t->morton_bits == 63) != wide)
            return fail(OIBVH_ERR_UNSUPPORTED, "a scene build needs the same Morton key width for every tree");
    CUDA_TRY(launch_build_multi(s->build_jobs.p, n, s->v_blocks, s->f_blocks, s->vblock_job.p, s->fblock_job.p,
                                s->n_faces, tree_bits, wide, scratch.p, st));
    // every tree's vertices renumbered in the order its sorted faces first use
    // them: six launches for all trees
    CUDA_TRY(launch_reorder_vertices_multi(s->build_jobs.p, n, s->v_blocks, s->f_blocks, s->vblock_job.p,
                                           s->fblock_job.p, s->n_verts, scratch.p, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (auto t : s->trees) {
        t->reordered = true;
        t->built = true;
    }
    const int r = oibvh_scene_refit(s, stream);
    if (r != OIBVH_OK) return r;
    CUDA_TRY(cudaStreamSynchronize(st));
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_transform(oibvh_scene_t s, const float* d_rest_xyzw, const float* d_mats, void* stream)
{
    GUARD_BEGIN
    if (!s || !d_rest_xyzw || !d_mats) return fail(OIBVH_ERR_ARG, "scene, rest or mats is NULL");
    if (s->trees.empty()) return OIBVH_OK;
    if (((uintptr_t)d_rest_xyzw) % 16) return fail(OIBVH_ERR_ARG, "rest positions must be 16-byte aligned");
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    for (auto t : s->trees) {  // the transform writes each tree's own positions
        t->cur_pos = t->pos4.p;
        t->borrowed = nullptr;
    }
    OK_TRY(ensure_build_jobs(s, st));
    CUDA_TRY(launch_transform_multi(s->build_jobs.p, (uint32_t)s->trees.size(), s->v_blocks, s->vblock_job.p,
                                    (const float4*)d_rest_xyzw, d_mats, false, st));
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_set_tuning(oibvh_scene_t s, const oibvh_tuning* t)
{
    if (!s || !t) return fail(OIBVH_ERR_ARG, "scene or tuning is NULL");
    if (t->start_pairs_log2 < 8 || t->start_pairs_log2 > 24) return fail(OIBVH_ERR_ARG, "start_pairs_log2 in 8..24");
    if (t->handoff < 32 || t->handoff > 8192) return fail(OIBVH_ERR_ARG, "handoff in 32..8192");
    if (t->walk_front && (t->walk_front % 32 || t->walk_front > 512))
        return fail(OIBVH_ERR_ARG, "walk_front: a multiple of 32 up to 512 (0 keeps the value)");
    if (t->walk_front) s->tune_walk_cap = t->walk_front;
    if (t->refit_group_log2 && (t->refit_group_log2 < 9 || t->refit_group_log2 > 11))
        return fail(OIBVH_ERR_ARG, "refit_group_log2: 9, 10 or 11 (0 keeps the value)");
    if (t->refit_group_log2) s->tune_refit_log = t->refit_group_log2;
    if (t->descend_ratio > (1u << 30)) return fail(OIBVH_ERR_ARG, "descend_ratio: 1..2^30 (0 keeps the value)");
    if (t->descend_ratio) s->tune_descend = t->descend_ratio;
    if (t->claim_min > (1u << 20)) return fail(OIBVH_ERR_ARG, "claim_min: 1..2^20 (0 keeps the value)");
    if (t->claim_min) s->tune_claim = t->claim_min;
    s->tune_start_log2 = t->start_pairs_log2;
    s->tune_handoff = t->handoff;
    s->tune_walk_per_sm = t->walk_blocks_per_sm;
    if (t->front_capacity) s->front_cap = std::min<uint32_t>(t->front_capacity, 0x7fffffffu);
    if (t->hit_capacity) s->hit_cap = std::min<uint32_t>(t->hit_capacity, 0x7fffffffu);
    s->frame_stale = true;
    return OIBVH_OK;
}

API int oibvh_scene_get_tuning(oibvh_scene_t s, oibvh_tuning* t)
{
    if (!s || !t) return fail(OIBVH_ERR_ARG, "scene or tuning is NULL");
    t->start_pairs_log2 = s->tune_start_log2;
    t->handoff = s->tune_handoff;
    t->walk_blocks_per_sm = s->tune_walk_per_sm;
    t->walk_front = s->tune_walk_cap;
    t->refit_group_log2 = s->tune_refit_log;
    t->descend_ratio = s->tune_descend;
    t->claim_min = s->tune_claim;
    t->front_capacity = s->front_cap;
    t->hit_capacity = s->hit_cap;
    return OIBVH_OK;
}

// Times `reps` detects per candidate setting with CUDA events and keeps the
// fastest. Coordinate descent: the start size x handoff grid first, then the
// walkers' front capacity, then walker CTAs per SM, each with the others at
// their best so far.
API int oibvh_scene_autotune(oibvh_scene_t s, uint32_t entry_level, uint32_t reps, oibvh_tuning* chosen)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (reps == 0) reps = 3;
    DeviceGuard g(s->device);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    int st = OIBVH_OK;
    // one setting: a warm-up detect (sizes the queues), then `reps` timed ones
    auto time_setting = [&](float& ms_out) {
        st = detect_impl(s, s->device, entry_level, 1, full_detect_mode(s), 0);
        float tot = 0.0f;
        for (uint32_t r = 0; r < reps && st == OIBVH_OK; ++r) {
            cudaEventRecord(e0, 0);
            st = detect_impl(s, s->device, entry_level, 1, full_detect_mode(s), 0);
            cudaEventRecord(e1, 0);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            tot += ms;
        }
        ms_out = tot;
        return st == OIBVH_OK;
    };
    // the refit's level-group depth: the scene refit timed alone
    uint32_t b_group = s->tune_refit_log;
    {
        float best_refit = 1e30f;
        for (uint32_t gl : {9u, 10u, 11u}) {
            s->tune_refit_log = gl;
            st = oibvh_scene_refit(s, 0);  // warm-up (uploads the job table)
            float tot = 0.0f;
            for (uint32_t r = 0; r < reps && st == OIBVH_OK; ++r) {
                cudaEventRecord(e0, 0);
                st = oibvh_scene_refit(s, 0);
                cudaEventRecord(e1, 0);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                tot += ms;
            }
            if (st != OIBVH_OK) break;
            if (tot < best_refit) best_refit = tot, b_group = gl;
        }
        s->tune_refit_log = b_group;
        if (st == OIBVH_OK) st = oibvh_scene_refit(s, 0);
    }
    float best = 1e30f;
    uint32_t b_start = s->tune_start_log2, b_handoff = s->tune_handoff, b_cap = 128, b_per = 0;
    uint32_t b_desc = 16, b_claim = 1;
    s->tune_walk_cap = 128;
    s->tune_walk_per_sm = 0;
    s->tune_descend = 16;
    s->tune_claim = 1;
    for (uint32_t sl : {12u, 14u, 16u, 18u, 20u})
        for (uint32_t h : {512u, 2048u, 8192u}) {
            s->tune_start_log2 = sl;
            s->tune_handoff = h;
            float ms;
            if (!time_setting(ms)) break;
            if (ms < best) best = ms, b_start = sl, b_handoff = h;
        }
    s->tune_start_log2 = b_start;
    s->tune_handoff = b_handoff;
    for (uint32_t cap : {64u, 256u, 512u}) {
        if (st != OIBVH_OK) break;
        s->tune_walk_cap = cap;
        float ms;
        if (!time_setting(ms)) break;
        if (ms < best) best = ms, b_cap = cap;
    }
    s->tune_walk_cap = b_cap;
    for (uint32_t r : {4u, 64u, 1u << 30}) {
        if (st != OIBVH_OK) break;
        s->tune_descend = r;
        float ms;
        if (!time_setting(ms)) break;
        if (ms < best) best = ms, b_desc = r;
    }
    s->tune_descend = b_desc;
    for (uint32_t c : {4u, 32u}) {
        if (st != OIBVH_OK) break;
        s->tune_claim = c;
        float ms;
        if (!time_setting(ms)) break;
        if (ms < best) best = ms, b_claim = c;
    }
    s->tune_claim = b_claim;
    const int fit = walk_blocks_per_sm(b_cap);
    for (int per = 1; per < fit && st == OIBVH_OK; ++per) {
        s->tune_walk_per_sm = (uint32_t)per;
        float ms;
        if (!time_setting(ms)) break;
        if (ms < best) best = ms, b_per = (uint32_t)per;
    }
    s->tune_walk_per_sm = b_per;
    // confirmation: the descent follows noisy timings, so the chosen detect
    // setting is timed again against the defaults (twice the repetitions)
    // and the faster one is kept
    if (st == OIBVH_OK) {
        const uint32_t reps0 = reps;
        reps = 2 * reps0;
        float ms_chosen = 0.0f, ms_default = 0.0f;
        if (time_setting(ms_chosen)) {
            s->tune_start_log2 = 16;
            s->tune_handoff = 2048;
            s->tune_walk_cap = 128;
            s->tune_walk_per_sm = 0;
            s->tune_descend = 16;
            s->tune_claim = 1;
            if (time_setting(ms_default) && ms_default < ms_chosen) {
                b_start = 16, b_handoff = 2048, b_cap = 128, b_per = 0, b_desc = 16, b_claim = 1;
            }
        }
        reps = reps0;
        s->tune_start_log2 = b_start;
        s->tune_handoff = b_handoff;
        s->tune_walk_cap = b_cap;
        s->tune_walk_per_sm = b_per;
        s->tune_descend = b_desc;
        s->tune_claim = b_claim;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != OIBVH_OK) return st;
    oibvh_tuning bt{};
    bt.start_pairs_log2 = b_start;
    bt.handoff = b_handoff;
    bt.walk_blocks_per_sm = b_per ? b_per : (uint32_t)walk_blocks_per_sm(b_cap);
    bt.walk_front = b_cap;
    bt.refit_group_log2 = b_group;
    bt.descend_ratio = b_desc;
    bt.claim_min = b_claim;
    // capacities: the largest work list and hit count seen, doubled
    st = detect_impl(s, s->device, entry_level, 1, full_detect_mode(s), 0);
    if (st != OIBVH_OK) return st;
    s->front_cap = grow_cap(2 * s->stats.front_peak, s->front_cap);
    if (s->hit_count * 2 > s->hit_cap) {
        const uint32_t want = grow_cap(2 * s->hit_count, s->hit_cap);
        OK_TRY(s->hits.ensure(want, "cudaMalloc(hits)"));
        s->hit_cap = want;
    }
    bt.front_capacity = s->front_cap;
    bt.hit_capacity = s->hit_cap;
    s->frame_stale = true;
    if (chosen) *chosen = bt;
    return OIBVH_OK;
    GUARD_END
}

namespace {

// The frame's work on `st`, as captured: [transform of every tree], [refit
// of every tree], the detect of every pair (start front, top walk, the
// captured walk rounds), [the precision narrow phase], the counters to the
// host. `ev` (optional, 6 events) brackets the stages for per-stage times:
// ev[0] | transform | ev[1] | refit | ev[2] | start + top | ev[3] | walk
// rounds | ev[4] | narrow | ev[5].
cudaError_t enqueue_frame(oibvh_scene_s* s, cudaStream_t st, cudaEvent_t* ev, uint32_t* kernels)
{
    const DetectArgs& a = s->frame_args;
    uint32_t k = 0;
    cudaError_t e = cudaSuccess;
    auto mark = [&](int i) {
        if (ev && e == cudaSuccess) e = cudaEventRecord(ev[i], st);
    };
    mark(0);
    if (s->frame_rest && e == cudaSuccess) {
        e = launch_transform_multi(s->build_jobs.p, (uint32_t)s->trees.size(), s->v_blocks, s->vblock_job.p,
                                   s->frame_rest_tree.p, s->frame_mats, true, st);
        ++k;
    }
    mark(1);
    if (s->frame_refit && e == cudaSuccess) {
        e = launch_refit(s->refit_jobs.p, (uint32_t)s->trees.size(), s->refit_blocks, s->refit_block_job.p,
                         s->refit_counters.p, refit_counters_per_tree() * s->trees.size(), s->tune_refit_log, st);
        ++k;
    }
    mark(2);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->counts.p, 0, kCountTotal * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = launch_init_front(a, s->frame_front0, st);
    if (e == cudaSuccess) e = launch_top(a, st);
    k += 2;
    mark(3);
    for (uint32_t r = 1; r <= s->frame_rounds && e == cudaSuccess; ++r) {
        e = launch_walk(a, r, st);
        ++k;
    }
    mark(4);
    if (s->precision && e == cudaSuccess) {
        DetectArgs n = a;
        n.fuse_narrow = 1;
        n.grid = sm_count(s->device) * 8;
        e = launch_narrow(n, st);
        k += narrow_kernels(n);
    }
    mark(5);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->h_frame_counts.p, s->counts.p, kCountTotal * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            st);
    if (kernels) *kernels = k;
    return e;
}

// Capture [transform] + refit + detect of every pair (one pass) into a graph.
int capture_frame_impl(oibvh_scene_s* s, cudaStream_t st)
{
    if (s->frame_exec) {
        cudaGraphExecDestroy(s->frame_exec);
        s->frame_exec = nullptr;
    }
    std::vector<uint32_t> pr;
    list_pairs(s, pr);
    const uint32_t np = (uint32_t)(pr.size() / 2);
    if (np == 0) return fail(OIBVH_ERR_STATE, "no pairs to detect");
    if (np > kMaxPairsPerPass) return fail(OIBVH_ERR_UNSUPPORTED, "a captured frame handles at most 16384 pairs");
    // warm-up frame outside the capture: sizes every buffer and uploads the tables
    if (s->frame_rest) OK_TRY(oibvh_scene_transform(s, (const float*)s->frame_rest, s->frame_mats, st));
    if (s->frame_refit) OK_TRY(oibvh_scene_refit(s, st));
    OK_TRY(detect_impl(s, s->device, s->frame_entry, s->frame_expand, full_detect_mode(s), st));
    // walk rounds: the warm-up frame used steps - 1 of them; two more for headroom
    // (a round with an empty input list returns at once)
    s->frame_rounds = std::min(kMaxRounds - 1, std::max(3u, s->stats.steps + 1));
    // headroom, then the exact tables the graph will read
    s->front_cap = std::max(s->front_cap, grow_cap(2 * s->stats.front_peak, s->front_cap));
    OK_TRY(s->front0.ensure(s->front_cap, "cudaMalloc(work list)"));
    OK_TRY(s->front1.ensure(s->front_cap, "cudaMalloc(work list)"));
    if (s->hit_count * 2 > s->hit_cap) {
        const uint32_t want = grow_cap(2 * s->hit_count, s->hit_cap);
        OK_TRY(s->hits.ensure(want, "cudaMalloc(hits)"));
        s->hit_cap = want;
    }
    if (s->precision) {
        // split narrow phase: the candidates of the whole frame are stored
        s->cand_cap = std::max(s->cand_cap, grow_cap(2 * s->cand_count, s->cand_cap));
        OK_TRY(s->cand.ensure(s->cand_cap, "cudaMalloc(candidates)"));
        OK_TRY(s->prec_lists.ensure(4 * (size_t)s->cand_cap, "cudaMalloc(precision lists)"));
    }
    OK_TRY(s->h_frame_counts.ensure(kCountTotal, "cudaMallocHost(frame counts)"));
    PassPlan plan;
    OK_TRY(plan_pass(s, pr.data(), np, s->frame_entry, plan));
    CUDA_TRY(cudaStreamSynchronize(st));
    std::memcpy(s->h_pairs.p, plan.pv.data(), np * sizeof(PairView));
    CUDA_TRY(cudaMemcpyAsync(s->pairv.p, s->h_pairs.p, np * sizeof(PairView), cudaMemcpyHostToDevice, st));
    OK_TRY(upload_views(s, st));
    if (s->frame_rest) {
        OK_TRY(ensure_build_jobs(s, st));
        // the graph reads the rest positions in each tree's vertex order: one
        // gathered copy now, so that every frame's transform reads them in order
        OK_TRY(s->frame_rest_tree.ensure(std::max<size_t>(s->n_verts, 1), "cudaMalloc(rest positions)"));
        CUDA_TRY(launch_gather_rest_multi(s->build_jobs.p, (uint32_t)s->trees.size(), s->v_blocks, s->vblock_job.p,
                                          s->frame_rest, s->frame_rest_tree.p, st));
    }
    if (s->frame_refit) OK_TRY(oibvh_scene_refit(s, st));  // refreshes the refit job table
    CUDA_TRY(cudaStreamSynchronize(st));

    DetectArgs a{};
    a.trees = s->views.p;
    a.pairs = s->pairv.p;
    a.n_pairs = np;
    a.expand_levels = 1;
    a.work[0] = s->front0.p;
    a.work[1] = s->front1.p;
    a.work_cap = s->front_cap;
    a.hits = s->hits.p;
    a.hit_cap = s->hit_cap;
    a.counts = s->counts.p;
    a.fuse_narrow = s->precision ? 0u : 1u;
    a.cand = s->precision ? s->cand.p : nullptr;
    a.cand_cap = s->precision ? s->cand_cap : 0u;
    a.prec_lists = s->precision ? s->prec_lists.p : nullptr;
    a.fp64_tri = s->precision ? s->fp64_tri.p : nullptr;
    a.fp64_tri_cap = s->precision ? s->fp64_tri_cap : 0u;
    a.grid = walk_grid(s, !s->precision);
    a.handoff = s->tune_handoff;
    a.walk_cap = s->tune_walk_cap;
    a.precision = s->precision;
    a.descend_ratio = (float)s->tune_descend;
    a.claim_min = s->tune_claim;

    s->frame_args = a;
    s->frame_front0 = (uint32_t)plan.front0;

    // capture on a private non-blocking stream (the legacy default stream
    // cannot be captured); the graph is launched on the caller's stream
    if (!s->capture_stream) CUDA_TRY(cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking));
    st = s->capture_stream;
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    uint32_t kernels = 0;
    cudaError_t e = enqueue_frame(s, st, nullptr, &kernels);
    const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(e, "capturing the frame");
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&s->frame_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        s->frame_exec = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    s->frame_kernels = kernels;
    s->frame_stale = false;
    s->last_pairs = plan.pv;
    return OIBVH_OK;
}

}  // namespace

API int oibvh_scene_capture_frame(oibvh_scene_t s, uint32_t entry_level, uint32_t expand_levels, int refit,
                                  const float* d_rest_xyzw, const float* d_mats, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    if (expand_levels < 1 || expand_levels > 16) return fail(OIBVH_ERR_ARG, "expand_levels must be in 1..16");
    if ((d_rest_xyzw == nullptr) != (d_mats == nullptr)) return fail(OIBVH_ERR_ARG, "give both rest and mats, or neither");
    for (auto t : s->trees)
        if (!t->built) return fail(OIBVH_ERR_STATE, "every tree must be built before a frame is captured");
    DeviceGuard g(s->device);
    s->frame_entry = entry_level;
    s->frame_expand = expand_levels;
    s->frame_refit = refit != 0;
    s->frame_rest = (const float4*)d_rest_xyzw;
    s->frame_mats = d_mats;
    return capture_frame_impl(s, (cudaStream_t)stream);
    GUARD_END
}

API int oibvh_scene_launch_frame(oibvh_scene_t s, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    DeviceGuard g(s->device);
    if (s->frame_stale || !s->frame_exec) OK_TRY(capture_frame_impl(s, (cudaStream_t)stream));
    CUDA_TRY(cudaGraphLaunch(s->frame_exec, (cudaStream_t)stream));
    note_launches(s->frame_kernels);
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_finish_frame(oibvh_scene_t s, void* stream)
{
    GUARD_BEGIN
    if (!s) return fail(OIBVH_ERR_ARG, "scene is NULL");
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaStreamSynchronize(st));
    const uint32_t* c = s->h_frame_counts.p;
    if (!c) return fail(OIBVH_ERR_STATE, "no frame was launched");
    if (c[kCountFlags] || c[kCountWork0 + s->frame_rounds + 1] != 0) {
        // the captured queues were too small for this frame: redo the detect the
        // synchronous way (the refit already ran) and capture again next frame
        s->frame_stale = true;
        s->frame_redos++;
        OK_TRY(detect_impl(s, s->device, s->frame_entry, s->frame_expand, full_detect_mode(s), st));
        s->stats.retries++;
        return OIBVH_OK;
    }
    s->stats = oibvh_detect_stats{};
    s->stats.passes = 1;
    s->stats.steps = s->frame_rounds;
    s->stats.nodes_tested = c[kCountTested];
    s->stats.fp64_axes = c[kCountFp64Axes];
    s->stats.fp64_candidates = c[kCountFp64Cands];
    s->stats.fp32_disagreements = c[kCountDisagree];
    s->stats.bounded_candidates = (uint64_t)c[kCountPrecHits] + c[kCountPrecRecheck];
    uint64_t peak = 0;
    for (uint32_t k = 0; k <= s->frame_rounds + 1; ++k) peak = std::max<uint64_t>(peak, c[kCountWork0 + k]);
    s->stats.front_peak = peak;
    s->hit_count = c[kCountHits];
    s->cand_count = c[kCountCands];
    s->stats.candidates = s->cand_count;
    s->stats.hits = s->hit_count;
    s->cands_valid = false;
    return OIBVH_OK;
    GUARD_END
}

API int oibvh_scene_profile_frame(oibvh_scene_t s, void* stream, oibvh_frame_profile* out)
{
    GUARD_BEGIN
    if (!s || !out) return fail(OIBVH_ERR_ARG, "scene or out is NULL");
    DeviceGuard g(s->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (s->frame_stale || !s->frame_exec) OK_TRY(capture_frame_impl(s, st));
    struct Events {
        cudaEvent_t e[6] = {};
        ~Events()
        {
            for (auto& x : e)
                if (x) cudaEventDestroy(x);
        }
    } ev;
    for (auto& x : ev.e) CUDA_TRY(cudaEventCreate(&x));
    uint32_t kernels = 0;
    CUDA_TRY(enqueue_frame(s, st, ev.e, &kernels));
    CUDA_TRY(cudaStreamSynchronize(st));
    float ms[5] = {};
    for (int i = 0; i < 5; ++i) CUDA_TRY(cudaEventElapsedTime(&ms[i], ev.e[i], ev.e[i + 1]));
    *out = oibvh_frame_profile{};
    out->transform_ms = ms[0];
    out->refit_ms = ms[1];
    out->start_ms = ms[2];
    out->walk_ms = ms[3];
    out->narrow_ms = ms[4];
    out->walk_rounds = s->frame_rounds;
    out->kernels = kernels;
    return oibvh_scene_finish_frame(s, stream);
    GUARD_END
}
