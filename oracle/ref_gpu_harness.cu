/*
 * ORACLE — test infrastructure only; never part of the product library.
 *
 * Headless driver of the reference's own GPU kernels, compiled unmodified
 * with nvcc from src/cuda/oibvh.cu (leaf boxes, Morton codes, level-group
 * construction) and src/cuda/collide.cu (BVTT traversal, triangle test) by
 * build_ref.sh. The reference drives them from OibvhTree and Scene, whose
 * constructors create OpenGL objects (src/cuda/oibvhTree.cu:9-15,
 * src/cuda/scene.cu:12-33); no graphics stack exists here, so this file
 * restates their host sequences instead:
 *   OibvhTree::build   src/cuda/oibvhTree.cu:237-388
 *   OibvhTree::refit   src/cuda/oibvhTree.cu:193-235
 *   OibvhTree::schedulingParameters  src/cuda/oibvhTree.cu:126-155
 *   Scene::expandBvttNodes           src/cuda/scene.cu:192-223
 *   Scene::detectCollisionOnGPU      src/cuda/scene.cu:225-446
 * with the same launches, the same block sizes and thrust's stable sorts.
 *
 * Two hazards of the reference are ruled out on the host before a kernel runs
 * (nothing unsafe is ever launched; the call returns a refusal code instead):
 *   - the construction kernels return early for threads past the level's real
 *     node count and then reach __syncthreads (src/cuda/oibvh.cu:87-88,
 *     :122): a schedule is only launched when every one of its blocks is
 *     full, so no thread returns before the barrier;
 *   - the traversal appends to fixed 10,000,000-entry buffers without a
 *     bound check (src/cuda/scene.cu:15-21, src/cuda/collide.cu:160-161,
 *     :296-297): the traversal is simulated on the host over the trees just
 *     built (the same boxes, the same expansion rule) and only launched when
 *     every front and the candidate list fit.
 * Buffers are allocated to the sizes the input needs (the reference's own
 * capacities are only checked against).
 */
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include <thrust/device_ptr.h>
#include <thrust/sort.h>

#include "cuda/collide.cuh"
#include "cuda/oibvh.cuh"

namespace {

constexpr size_t kRefCapacity = 10000000;  // the reference's fixed buffer entries

enum RefStatus : int {
    kRefOk = 0,
    kRefCuda = -1,
    kRefUnsafeSchedule = -2,  // a construction launch would have a partial block
    kRefUnsafeCapacity = -3,  // a traversal buffer would overflow the reference's capacity
    kRefArg = -4,
};

struct Schedule {
    unsigned int entry, real, threads, group;
};

struct RefTree {
    std::vector<glm::uvec3> faces;      // m_faces (Morton order after build)
    std::vector<glm::vec3> positions;   // m_positions
    std::vector<aabb_box_t> tree;       // m_aabbTree
    std::vector<Schedule> schedule;     // m_scheduleParams
    aabb_box_t mesh_box;                // Mesh::m_aabb (src/utils/mesh.cpp:91-98)
    bool built = false;
};

// OibvhTree::schedulingParameters restated.
std::vector<Schedule> make_schedule(unsigned int entry, unsigned int real, unsigned int per_group)
{
    std::vector<Schedule> out;
    unsigned int l = entry, r = real;
    unsigned int g = std::min(per_group, next_power_of_two(r));
    unsigned int t = (r + g - 1) / g * g;
    for (;;) {
        out.push_back({l, r, t, g});
        if (l >= ilog2(g) + 1) l = l - ilog2(g) - 1;
        else break;
        r = (t / g + 1) / 2;
        const unsigned int gl = g;
        g = std::min(gl, next_power_of_two(r));
        t = (r + g - 1) / g * g;
    }
    return out;
}

// Every launch runs full blocks (threads == real nodes): no early return
// before the construction kernels' barrier.
bool schedule_safe(const std::vector<Schedule>& s)
{
    for (const auto& e : s)
        if (e.threads != e.real) return false;
    return true;
}

struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    Events()
    {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~Events()
    {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    float ms() const
    {
        float v = 0.0f;
        cudaEventElapsedTime(&v, a, b);
        return v;
    }
};

template <class T>
struct Dev {
    T* p = nullptr;
    explicit Dev(size_t n) { cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
    ~Dev() { cudaFree(p); }
};

int run_construction(const RefTree& t, unsigned int n_prim, aabb_box_t* d_aabbs, bool refit_kernel)
{
    for (const auto& s : t.schedule) {
        const dim3 block(s.group), grid(s.threads / s.group);
        if (refit_kernel) oibvh_tree_construction_kernel<<<grid, block>>>(s.entry, s.real, n_prim, s.group, d_aabbs);
        else oibvh_tree_construction_kernel2<<<grid, block>>>(s.entry, s.real, n_prim, s.group, d_aabbs);
    }
    return cudaGetLastError() == cudaSuccess ? kRefOk : kRefCuda;
}

// Traversal of detectCollisionOnGPU simulated on the host (collide.cu:76-246:
// a front node whose boxes overlap is a candidate when both are leaves, else
// every real child 'expand' levels down on both sides joins the next front).
// Returns false as soon as a front or the candidates exceed the capacity.
struct SimTree {
    const aabb_box_t* box;
    unsigned int offset, prims, leaf_lev, vl;
};

bool traversal_fits(const std::vector<SimTree>& trees, const std::vector<bvtt_node_t>& start, unsigned int expand,
                    uint64_t* candidates, uint64_t* peak)
{
    auto tree_of = [&](unsigned int g) {
        size_t i = trees.size() - 1;
        while (trees[i].offset > g) --i;
        return i;
    };
    std::vector<bvtt_node_t> cur = start, next;
    uint64_t cands = 0, most = cur.size();
    if (cur.size() > kRefCapacity) return false;
    while (!cur.empty()) {
        next.clear();
        for (const auto& n : cur) {
            const SimTree& A = trees[tree_of(n.m_aabbIndex[0])];
            const SimTree& B = trees[tree_of(n.m_aabbIndex[1])];
            const unsigned int ra = n.m_aabbIndex[0] - A.offset, rb = n.m_aabbIndex[1] - B.offset;
            aabb_box_t ba = A.box[ra];
            if (!ba.overlap(B.box[rb])) continue;
            const unsigned int ia = oibvh_real_to_implicit(ra, A.leaf_lev, A.vl);
            const unsigned int ib = oibvh_real_to_implicit(rb, B.leaf_lev, B.vl);
            const unsigned int la = ilog2(ia + 1), lb = ilog2(ib + 1);
            if (la == A.leaf_lev && lb == B.leaf_lev) {
                if (++cands > kRefCapacity) return false;
                continue;
            }
            const unsigned int na_l = std::min(A.leaf_lev, la + expand), nb_l = std::min(B.leaf_lev, lb + expand);
            const unsigned int sa = oibvh_get_most_left_descendant_implicitIdx(ia, na_l - la);
            const unsigned int sb = oibvh_get_most_left_descendant_implicitIdx(ib, nb_l - lb);
            const unsigned int ea = oibvh_get_most_right_valid_implicitIdx(na_l, A.leaf_lev, A.vl);
            const unsigned int eb = oibvh_get_most_right_valid_implicitIdx(nb_l, B.leaf_lev, B.vl);
            const unsigned int ca = std::min(1u << (na_l - la), ea - sa + 1);
            const unsigned int cb = std::min(1u << (nb_l - lb), eb - sb + 1);
            if (next.size() + (uint64_t)ca * cb > kRefCapacity) return false;
            for (unsigned int x = 0; x < ca; ++x)
                for (unsigned int y = 0; y < cb; ++y)
                    next.push_back(bvtt_node_t{oibvh_implicit_to_real(sa + x, A.leaf_lev, A.vl) + A.offset,
                                               oibvh_implicit_to_real(sb + y, B.leaf_lev, B.vl) + B.offset});
        }
        most = std::max<uint64_t>(most, next.size());
        cur.swap(next);
    }
    *candidates = cands;
    *peak = most;
    return true;
}

}  // namespace

#define REF_API extern "C" __attribute__((visibility("default")))

REF_API void* refgpu_tree_create(const float* xyz, unsigned int n_vertices, const unsigned int* tri,
                                 unsigned int n_triangles)
{
    if (!xyz || !tri || n_triangles < 2) return nullptr;  // the reference's build needs a leaf level >= 1
    auto* t = new RefTree();
    t->positions.resize(n_vertices);
    for (unsigned int v = 0; v < n_vertices; ++v) {
        t->positions[v] = glm::vec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
        t->mesh_box.m_maximum = glm::max(t->positions[v], t->mesh_box.m_maximum);
        t->mesh_box.m_minimum = glm::min(t->positions[v], t->mesh_box.m_minimum);
    }
    t->faces.resize(n_triangles);
    for (unsigned int f = 0; f < n_triangles; ++f) t->faces[f] = glm::uvec3(tri[3 * f], tri[3 * f + 1], tri[3 * f + 2]);
    return t;
}

REF_API void refgpu_tree_destroy(void* h) { delete static_cast<RefTree*>(h); }

// OibvhTree::build. With construct == 0 (or when the schedule has a partial
// block, return kRefUnsafeSchedule) only the leaf boxes, Morton codes and the
// two stable sorts run: the sorted faces are then valid, the tree is not.
// ms[0] = device time of the whole sequence (events), ms[1] = its kernels
// and sorts alone.
REF_API int refgpu_tree_build(void* h, int construct, float* ms)
{
    auto* t = static_cast<RefTree*>(h);
    if (!t) return kRefArg;
    const unsigned int prims = (unsigned int)t->faces.size(), verts = (unsigned int)t->positions.size();
    const unsigned int size = oibvh_get_size(prims), internal = size - prims;
    const unsigned int p2 = next_power_of_two(prims), leaf_lev = ilog2(p2), vl = p2 - prims;
    t->schedule = make_schedule(leaf_lev - 1, oibvh_level_real_node_count(leaf_lev - 1, leaf_lev, vl), THREADS_PER_BLOCK);
    const bool safe = schedule_safe(t->schedule);
    Events all, work;
    Dev<glm::vec3> d_pos(verts);
    Dev<glm::uvec3> d_faces(prims);
    Dev<aabb_box_t> d_aabbs(size);
    Dev<unsigned int> d_morton(prims), d_morton2(prims);
    cudaEventRecord(all.a);
    cudaMemcpy(d_pos.p, t->positions.data(), verts * sizeof(glm::vec3), cudaMemcpyHostToDevice);
    cudaMemcpy(d_faces.p, t->faces.data(), prims * sizeof(glm::uvec3), cudaMemcpyHostToDevice);
    cudaEventRecord(work.a);
    calculate_aabb_and_morton_kernel<<<(prims + 255) / 256, 256>>>(d_faces.p, d_pos.p, prims, t->mesh_box,
                                                                   d_aabbs.p + internal, d_morton.p);
    cudaMemcpy(d_morton2.p, d_morton.p, prims * sizeof(unsigned int), cudaMemcpyDeviceToDevice);
    thrust::device_ptr<unsigned int> k1(d_morton.p), k2(d_morton2.p);
    thrust::stable_sort_by_key(k1, k1 + prims, thrust::device_ptr<glm::uvec3>(d_faces.p));
    thrust::stable_sort_by_key(k2, k2 + prims, thrust::device_ptr<aabb_box_t>(d_aabbs.p + internal));
    int st = kRefOk;
    if (construct && safe) st = run_construction(*t, prims, d_aabbs.p, false);
    cudaEventRecord(work.b);
    t->tree.assign(size, aabb_box_t{});
    cudaMemcpy(t->tree.data(), d_aabbs.p, size * sizeof(aabb_box_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(t->faces.data(), d_faces.p, prims * sizeof(glm::uvec3), cudaMemcpyDeviceToHost);
    cudaEventRecord(all.b);
    cudaEventSynchronize(all.b);
    if (cudaGetLastError() != cudaSuccess) return kRefCuda;
    if (ms) {
        ms[0] = all.ms();
        ms[1] = work.ms();
    }
    t->built = construct && safe && st == kRefOk;
    if (st != kRefOk) return st;
    return (construct && !safe) ? kRefUnsafeSchedule : kRefOk;
}

// OibvhTree::refit after the mesh's positions moved (xyz in the mesh's own
// vertex order; the sorted faces index it).
REF_API int refgpu_tree_refit(void* h, const float* xyz, float* ms)
{
    auto* t = static_cast<RefTree*>(h);
    if (!t || !t->built) return kRefArg;
    for (size_t v = 0; v < t->positions.size(); ++v) t->positions[v] = glm::vec3(xyz[3 * v], xyz[3 * v + 1], xyz[3 * v + 2]);
    const unsigned int prims = (unsigned int)t->faces.size(), verts = (unsigned int)t->positions.size();
    const unsigned int size = oibvh_get_size(prims), internal = size - prims;
    Events all, work;
    Dev<glm::vec3> d_pos(verts);
    Dev<glm::uvec3> d_faces(prims);
    Dev<aabb_box_t> d_aabbs(size);
    cudaEventRecord(all.a);
    cudaMemcpy(d_pos.p, t->positions.data(), verts * sizeof(glm::vec3), cudaMemcpyHostToDevice);
    cudaMemcpy(d_faces.p, t->faces.data(), prims * sizeof(glm::uvec3), cudaMemcpyHostToDevice);
    cudaEventRecord(work.a);
    calculate_aabb_kernel<<<(prims + 255) / 256, 256>>>(d_faces.p, d_pos.p, prims, d_aabbs.p + internal);
    const int st = run_construction(*t, prims, d_aabbs.p, true);
    cudaEventRecord(work.b);
    cudaMemcpy(t->tree.data(), d_aabbs.p, size * sizeof(aabb_box_t), cudaMemcpyDeviceToHost);
    cudaEventRecord(all.b);
    cudaEventSynchronize(all.b);
    if (cudaGetLastError() != cudaSuccess) return kRefCuda;
    if (ms) {
        ms[0] = all.ms();
        ms[1] = work.ms();
    }
    return st;
}

// Node boxes (size * 6 floats: min xyz, max xyz) and Morton-ordered faces (3 each).
REF_API int refgpu_tree_get(void* h, float* boxes6, unsigned int* faces3)
{
    auto* t = static_cast<RefTree*>(h);
    if (!t) return kRefArg;
    if (boxes6)
        for (size_t i = 0; i < t->tree.size(); ++i) {
            const aabb_box_t& b = t->tree[i];
            const float v[6] = {b.m_minimum.x, b.m_minimum.y, b.m_minimum.z, b.m_maximum.x, b.m_maximum.y, b.m_maximum.z};
            std::memcpy(boxes6 + 6 * i, v, sizeof(v));
        }
    if (faces3)
        for (size_t i = 0; i < t->faces.size(); ++i) {
            faces3[3 * i] = t->faces[i].x;
            faces3[3 * i + 1] = t->faces[i].y;
            faces3[3 * i + 2] = t->faces[i].z;
        }
    return kRefOk;
}

REF_API unsigned int refgpu_tree_size(void* h)
{
    auto* t = static_cast<RefTree*>(h);
    return t ? (unsigned int)t->tree.size() : 0u;
}

// Scene::detectCollisionOnGPU over built trees (every i < j pair). Writes up
// to cap records {bvhA, bvhB, triA, triB} (Morton-order triangle indices, as
// the reference reports them) and returns the number of colliding pairs, or
// a negative RefStatus. ms[0] = the whole call (events: uploads, traversal
// rounds with their read-backs, narrow phase, result download), ms[1] = the
// traversal kernels, ms[2] = the triangle kernel. *n_candidates gets the
// candidate count.
REF_API long long refgpu_detect(void** handles, int n_trees, unsigned int entry, unsigned int expand,
                                unsigned int* out4, long long cap, long long* n_candidates, float* ms)
{
    if (!handles || n_trees < 2 || expand < 1 || expand > 3) return kRefArg;
    std::vector<RefTree*> trees(n_trees);
    std::vector<unsigned int> aabb_off, prim_off, prim_cnt, vert_off;
    unsigned int n_aabb = 0, n_prim = 0, n_vert = 0;
    for (int i = 0; i < n_trees; ++i) {
        trees[i] = static_cast<RefTree*>(handles[i]);
        if (!trees[i] || !trees[i]->built) return kRefArg;
        aabb_off.push_back(n_aabb);
        prim_off.push_back(n_prim);
        vert_off.push_back(n_vert);
        prim_cnt.push_back((unsigned int)trees[i]->faces.size());
        n_aabb += (unsigned int)trees[i]->tree.size();
        n_prim += (unsigned int)trees[i]->faces.size();
        n_vert += (unsigned int)trees[i]->positions.size();
    }
    if (n_aabb > kRefCapacity || n_prim > kRefCapacity || n_vert > kRefCapacity || n_trees > 256)
        return kRefUnsafeCapacity;
    // Scene::expandBvttNodes
    std::vector<bvtt_node_t> start;
    std::vector<SimTree> sim;
    for (int i = 0; i < n_trees; ++i) {
        const unsigned int p2 = next_power_of_two(prim_cnt[i]);
        sim.push_back(SimTree{trees[i]->tree.data(), aabb_off[i], prim_cnt[i], ilog2(p2), p2 - prim_cnt[i]});
    }
    for (int i = 0; i < n_trees; ++i)
        for (int j = i + 1; j < n_trees; ++j) {
            const SimTree &A = sim[i], &B = sim[j];
            const unsigned int ea = std::min(A.leaf_lev, entry), eb = std::min(B.leaf_lev, entry);
            const unsigned int sa = oibvh_get_most_left_descendant_implicitIdx(0, ea);
            const unsigned int sb = oibvh_get_most_left_descendant_implicitIdx(0, eb);
            const unsigned int ra0 = oibvh_implicit_to_real(sa, A.leaf_lev, A.vl);
            const unsigned int ra1 = oibvh_implicit_to_real(oibvh_get_most_right_valid_implicitIdx(ea, A.leaf_lev, A.vl), A.leaf_lev, A.vl);
            const unsigned int rb0 = oibvh_implicit_to_real(sb, B.leaf_lev, B.vl);
            const unsigned int rb1 = oibvh_implicit_to_real(oibvh_get_most_right_valid_implicitIdx(eb, B.leaf_lev, B.vl), B.leaf_lev, B.vl);
            for (unsigned int p = ra0; p <= ra1; ++p)
                for (unsigned int q = rb0; q <= rb1; ++q) start.push_back(bvtt_node_t{p + A.offset, q + B.offset});
        }
    if (start.empty()) return kRefArg;
    uint64_t sim_cands = 0, sim_peak = 0;
    if (!traversal_fits(sim, start, expand, &sim_cands, &sim_peak)) return kRefUnsafeCapacity;

    Dev<bvtt_node_t> d_src(std::max<uint64_t>(sim_peak, start.size())), d_dst(std::max<uint64_t>(sim_peak, start.size()));
    Dev<aabb_box_t> d_aabbs(n_aabb);
    Dev<tri_pair_node_t> d_tri(sim_cands);
    Dev<glm::uvec3> d_prims(n_prim);
    Dev<glm::vec3> d_verts(n_vert);
    Dev<int_tri_pair_node_t> d_hits(sim_cands);
    Dev<unsigned int> d_aoff(n_trees), d_poff(n_trees), d_pcnt(n_trees), d_voff(n_trees), d_next(1), d_tcnt(1),
        d_hcnt(1);
    Events all, trav, narrow;
    cudaEventRecord(all.a);
    cudaMemcpy(d_src.p, start.data(), start.size() * sizeof(bvtt_node_t), cudaMemcpyHostToDevice);
    cudaMemcpy(d_aoff.p, aabb_off.data(), n_trees * sizeof(unsigned int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_poff.p, prim_off.data(), n_trees * sizeof(unsigned int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_pcnt.p, prim_cnt.data(), n_trees * sizeof(unsigned int), cudaMemcpyHostToDevice);
    cudaMemset(d_tcnt.p, 0, sizeof(unsigned int));
    for (int i = 0; i < n_trees; ++i)
        cudaMemcpy(d_aabbs.p + aabb_off[i], trees[i]->tree.data(), trees[i]->tree.size() * sizeof(aabb_box_t),
                   cudaMemcpyHostToDevice);
    // broad phase: one launch per front, its size read back each time
    unsigned int size = (unsigned int)start.size();
    bvtt_node_t *src = d_src.p, *dst = d_dst.p;
    float trav_ms = 0.0f;
    while (size) {
        cudaMemset(d_next.p, 0, sizeof(unsigned int));
        const dim3 block(std::min(256u, std::max(next_power_of_two((unsigned int)n_trees), next_power_of_two(size))));
        cudaEventRecord(trav.a);
        traversal_kernel<<<(size + block.x - 1) / block.x, block>>>(src, dst, d_aabbs.p, d_tri.p, d_aoff.p, d_poff.p,
                                                                    d_pcnt.p, d_next.p, d_tcnt.p, (unsigned int)n_trees,
                                                                    size, expand);
        cudaEventRecord(trav.b);
        cudaMemcpy(&size, d_next.p, sizeof(unsigned int), cudaMemcpyDeviceToHost);
        trav_ms += trav.ms();
        std::swap(src, dst);
    }
    unsigned int cands = 0, hits = 0;
    cudaMemcpy(&cands, d_tcnt.p, sizeof(unsigned int), cudaMemcpyDeviceToHost);
    // narrow phase
    for (int i = 0; i < n_trees; ++i) {
        cudaMemcpy(d_prims.p + prim_off[i], trees[i]->faces.data(), trees[i]->faces.size() * sizeof(glm::uvec3),
                   cudaMemcpyHostToDevice);
        cudaMemcpy(d_verts.p + vert_off[i], trees[i]->positions.data(), trees[i]->positions.size() * sizeof(glm::vec3),
                   cudaMemcpyHostToDevice);
    }
    cudaMemcpy(d_voff.p, vert_off.data(), n_trees * sizeof(unsigned int), cudaMemcpyHostToDevice);
    cudaMemset(d_hcnt.p, 0, sizeof(unsigned int));
    if (cands) {
        const dim3 block(std::min(256u, std::max(next_power_of_two((unsigned int)n_trees), next_power_of_two(cands))));
        cudaEventRecord(narrow.a);
        triangle_intersect_kernel<<<(cands + block.x - 1) / block.x, block>>>(
            d_tri.p, d_prims.p, d_verts.p, d_poff.p, d_voff.p, d_hits.p, d_hcnt.p, (unsigned int)n_trees, cands);
        cudaEventRecord(narrow.b);
    }
    cudaMemcpy(&hits, d_hcnt.p, sizeof(unsigned int), cudaMemcpyDeviceToHost);
    std::vector<int_tri_pair_node_t> h(hits);
    if (hits) cudaMemcpy(h.data(), d_hits.p, hits * sizeof(int_tri_pair_node_t), cudaMemcpyDeviceToHost);
    cudaEventRecord(all.b);
    cudaEventSynchronize(all.b);
    if (cudaGetLastError() != cudaSuccess) return kRefCuda;
    if (cands != sim_cands) return kRefCuda;  // the host simulation and the kernels disagree
    for (long long k = 0; k < std::min<long long>(cap, hits); ++k) {
        out4[4 * k] = h[k].m_bvhIndex[0];
        out4[4 * k + 1] = h[k].m_bvhIndex[1];
        out4[4 * k + 2] = h[k].m_triIndex[0];
        out4[4 * k + 3] = h[k].m_triIndex[1];
    }
    if (n_candidates) *n_candidates = cands;
    if (ms) {
        ms[0] = all.ms();
        ms[1] = trav_ms;
        ms[2] = cands ? narrow.ms() : 0.0f;
    }
    return hits;
}
