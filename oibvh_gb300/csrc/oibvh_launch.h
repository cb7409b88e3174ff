// Host-side launchers of the device kernels (one translation unit per stage).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "oibvh_common.cuh"

namespace oibvh {

// Count of this library's kernel launches (all devices), for benchmarks.
void note_launches(uint64_t n);

// One tree of a (possibly multi-tree) refit launch.
struct RefitJob {
    float4* box;           // internal nodes
    const uint4* face;
    const float4* pos;
    TreeShape shape;
    uint32_t block_begin;  // first CTA of this tree in the launch
    uint32_t n_blocks;
    uint32_t* counters;    // refit_counters_per_tree() zeroed words
    uint32_t pad0;
};

// One tree of a multi-tree build / transform launch.
struct BuildJob {
    const float4* pos;      // positions to build from (transform source when no packed rest array is given)
    const uint32_t* tri;    // faces as given (3 * nT)
    uint4* face_out;        // Morton-ordered face records
    uint32_t* bound_keys;   // 6 words of scratch (mesh bounds)
    float4* pos_out;        // transform target (the tree's own positions)
    uint32_t nV, nT;
    uint32_t vblock_begin;  // first CTA of this tree in vertex-chunk launches (256 vertices per CTA)
    uint32_t fblock_begin;  // first CTA of this tree in face-chunk launches (256 faces per CTA)
    uint32_t face_off;      // first face of this tree in the global face numbering
    uint32_t vert_off;      // first vertex of this tree in packed rest positions
    const uint32_t* vperm;  // tree vertex v is the caller's vertex vperm[v] (nullptr: the same order)
    uint32_t* vperm_out;    // the tree's map buffer (nV entries), rewritten by the renumbering
    uint32_t* tri_rw;       // the tree's faces (3 * nT), rewritten by the renumbering (tri, writable)
};

// build_kernels.cu
size_t radix_sort_scratch_bytes(uint32_t n);
size_t build_multi_scratch_bytes(uint32_t n_faces);
// vjob / fjob: optional host-built maps from a 256-vertex / 256-face block
// to its job (nullptr: each CTA binary-searches the job table).
// wide: 63-bit Morton keys (21 bits per axis) instead of the reference's 30.
cudaError_t launch_build_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks, uint32_t f_blocks,
                               const uint32_t* vjob, const uint32_t* fjob, uint32_t n_faces, uint32_t tree_bits,
                               bool wide, void* scratch, cudaStream_t s);
// rest: packed positions of all jobs in each caller's vertex order (read
// through the jobs' vperm), or in each tree's order (rest_tree_order), or
// nullptr (each job's own pos). Writes each job's pos_out.
cudaError_t launch_transform_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks, const uint32_t* vjob,
                                   const float4* rest, const float* mats, bool rest_tree_order, cudaStream_t s);
cudaError_t launch_gather_rest_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks, const uint32_t* vjob,
                                     const float4* rest, float4* out, cudaStream_t s);
// pos[v] = (xyz of the caller's vertex vperm[v], 0); vperm == nullptr: the same order
cudaError_t launch_xyz_to_pos4(const float* xyz, const uint32_t* vperm, uint32_t nV, float4* pos, cudaStream_t s);
// pos[v] = src[vperm[v]] (vperm == nullptr: a copy)
cudaError_t launch_gather_pos4(const float4* src, const uint32_t* vperm, uint32_t nV, float4* pos, cudaStream_t s);
// Renumber a built tree's vertices in the order its sorted faces first use
// them: face records and `tri` get the new indices, `pos` the new order and
// vperm (nV entries; read first when has_vperm) the new caller-order map.
size_t reorder_scratch_bytes(uint32_t nV);
cudaError_t launch_reorder_vertices(uint4* face, uint32_t* tri, uint32_t nT, uint32_t nV, float4* pos,
                                    uint32_t* vperm, bool has_vperm, void* scratch, cudaStream_t s);
// The same renumbering for every tree of a multi-tree build, in a fixed
// number of launches: each job's face_out, tri_rw, pos_out (the positions,
// read and rewritten) and vperm_out (from vperm, or the identity when nullptr).
size_t reorder_multi_scratch_bytes(uint32_t n_verts, uint32_t v_blocks, uint32_t f_blocks);
cudaError_t launch_reorder_vertices_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks,
                                          uint32_t f_blocks, const uint32_t* vjob, const uint32_t* fjob,
                                          uint32_t n_verts, void* scratch, cudaStream_t s);
cudaError_t launch_mesh_bounds(const float4* pos, uint32_t nV, uint32_t* bound_keys, int num_sms, cudaStream_t s);
// codes_hi != nullptr: 63-bit keys, low 32 bits in codes and high 31 in codes_hi
cudaError_t launch_leaf_morton(const uint32_t* tri, const float4* pos, uint32_t nT, const uint32_t* bound_keys,
                               uint32_t* codes, uint32_t* idx, uint32_t* codes_hi, cudaStream_t s);
cudaError_t launch_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int key_bits, void* scratch,
                              cudaStream_t s);
// out[i] = src[idx[i]]
cudaError_t launch_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t n, uint32_t* out, cudaStream_t s);
cudaError_t launch_gather_faces(const uint32_t* tri, const uint32_t* perm, uint32_t nT, uint4* out, cudaStream_t s);

// refit_kernels.cu
// refit CTAs of a tree of nT leaves with level groups of group_log2 levels
// (9, 10 or 11; 0 = 10, the single-tree refit's)
uint32_t refit_blocks_for(uint32_t nT, uint32_t group_log2 = 0);
uint32_t refit_counters_per_tree();
cudaError_t launch_refit_one(const RefitJob& job, cudaStream_t s);
cudaError_t launch_leaf_boxes(const uint4* face, const float4* pos, uint32_t nT, float4* out, cudaStream_t s);
// block_job: optional host-built map from a refit CTA to its job (nullptr:
// each CTA binary-searches the job table).
cudaError_t launch_refit(const RefitJob* d_jobs, uint32_t n_jobs, uint32_t total_blocks, const uint32_t* block_job,
                         uint32_t* d_counters, size_t n_counters, uint32_t group_log2, cudaStream_t s);

// detect_kernels.cu
struct DetectArgs {
    const TreeView* trees;
    const PairView* pairs;
    uint32_t n_pairs;
    uint32_t expand_levels;
    uint64_t* work[2];     // traversal work lists (ping-pong between rounds)
    uint32_t work_cap;
    uint64_t* cand;        // broad-only mode: candidate leaf pairs
    uint32_t cand_cap;
    uint4* hits;
    uint32_t hit_cap;
    uint32_t* counts;      // see kCount* below
    uint32_t* prec_lists;  // precision mode, 4 x cand_cap words: float-hit list, recheck list (candidate
                           // indices), then the FP64 list ((candidate index, axis mask) pairs)
    double* fp64_tri;      // precision mode: the FP64 list's setups, kFp64TriRows rows of fp64_tri_cap
                           // (structure of arrays; nullptr: each is formed where it is used)
    uint32_t fp64_tri_cap;
    uint32_t fuse_narrow;  // 1: test candidates in the traversal; 0: store them
    int grid;              // CTAs of the grid-stride / persistent kernels
    uint32_t handoff;      // front width at which k_top hands over to the walkers (<= 8192)
    uint32_t precision;    // 0: float triangle test (reference arithmetic); 1: FP64-filtered
    uint32_t walk_cap;     // per-warp front entries of the walkers (multiple of 32, <= 512; 0: 128)
    float descend_ratio = kDescendRatio;  // both sides descend while the boxes' squared diagonals are within it
    uint32_t claim_min = 1;  // walkers claim list items dynamically from this many items per warp
};
cudaError_t launch_init_front(const DetectArgs& a, uint32_t total0, cudaStream_t s);
cudaError_t launch_top(const DetectArgs& a, cudaStream_t s);
cudaError_t launch_walk(const DetectArgs& a, uint32_t round, cudaStream_t s);
// walker CTAs that fit on one SM with fronts of `walk_cap` entries (0:
// default), for the fused (narrow phase inside) or the broad-only walker
int walk_blocks_per_sm(uint32_t walk_cap = 0, bool fused = true);
cudaError_t launch_narrow(const DetectArgs& a, cudaStream_t s);
uint32_t narrow_kernels(const DetectArgs& a);  // kernels launch_narrow launches
// Rows of a precision-mode FP64 setup: the relative vertices p2, p3, q1, q2,
// q3 and the normals n1, m1 (x, y, z each), then the hit record (2 words).
constexpr uint32_t kFp64TriRows = 23;

// counts[]: hits, flags, candidates found, candidate slots used (broad-only),
// BVTT pairs tested, (precision mode) axes evaluated in FP64, candidates with
// at least one such axis, candidates whose float and FP64 answers differ,
// the sizes of the float-hit, recheck and FP64 lists of the precision narrow phase
// and of the list its double-float pass leaves to FP64,
// then the work-list size of each traversal round (list
// 0: the overlapping start pairs; list 1: the front k_top hands over; list
// r+1: what walk round r spilled), then how many items of each list the
// walkers have claimed.
constexpr uint32_t kMaxRounds = 16;
constexpr uint32_t kCountHits = 0, kCountFlags = 1, kCountCands = 2, kCountCandSlots = 3, kCountTested = 4,
                   kCountFp64Axes = 5, kCountFp64Cands = 6, kCountDisagree = 7, kCountPrecHits = 8,
                   kCountPrecRecheck = 9, kCountPrecFp64 = 10, kCountPrecLeft = 11, kCountWork0 = 12,
                   kCountClaim0 = kCountWork0 + kMaxRounds + 1,  // items of list r claimed so far
                   kCountTotal = kCountClaim0 + kMaxRounds + 1;

} // namespace oibvh
