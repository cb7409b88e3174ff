/*
 * oibvh_gb300 — C ABI of the GB300 (sm_103a) oibvh collision pipeline.
 *
 * The reference (hhhcbw/oibvh) exposes this path only as C++ classes:
 * OibvhTree (include/cuda/oibvhTree.cuh:50-93) and Scene
 * (include/cuda/scene.cuh:44-61). Each entry point below replaces one of
 * their members; the comment names the member it stands for (file:line in
 * the reference). Plain pointers and sizes only: positions are float xyz
 * triples (the Vertex::m_position field of include/utils/mesh.h:23-53),
 * faces are uint32 index triples (Mesh::m_indices, include/utils/mesh.h:183).
 *
 * Conventions (the reference ignores every CUDA error, include/cuda/utils.cuh:
 * 6-34; here nothing is ignored):
 *   - every call returns an OIBVH_* status; 0 is success; oibvh_last_error()
 *     gives a one-line reason for the last failure on the calling thread;
 *   - a handle is used by one host thread at a time;
 *   - `stream` is a cudaStream_t (NULL = the legacy default stream); calls
 *     documented as blocking synchronise that stream before returning,
 *     the others only enqueue work on it;
 *   - there is no CPU fallback: a device type of CPU is refused
 *     (the reference's detectCollisionOnCPU is an empty TODO,
 *     src/cuda/scene.cu:187-190).
 *
 * Limits: 1 <= triangles per mesh <= 2^23; at most 2^14 mesh pairs are
 * traversed per pass (more are processed in several passes).
 */
#ifndef OIBVH_GB300_H
#define OIBVH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum oibvh_status {
    OIBVH_OK = 0,
    OIBVH_ERR_ARG = 1,         /* invalid argument (null, size, index out of range) */
    OIBVH_ERR_OOM = 2,         /* device or pinned host allocation failed */
    OIBVH_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    OIBVH_ERR_OVERFLOW = 4,    /* a work queue stayed too small after regrowing */
    OIBVH_ERR_STATE = 5,       /* call out of order (e.g. detect before build) */
    OIBVH_ERR_UNSUPPORTED = 6, /* e.g. the CPU device type */
    OIBVH_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up (the context stays usable) */
};

/* DeviceType (include/cuda/scene.cuh:12-24): CPU = -1, GPU0..GPU8 = 0..8. */
#define OIBVH_DEVICE_CPU (-1)
#define OIBVH_DEVICE_GPU0 0

typedef struct oibvh_tree_s* oibvh_tree_t;
typedef struct oibvh_scene_s* oibvh_scene_t;

/* Text of a status code, and the last failure reason on this thread. */
const char* oibvh_status_string(int status);
const char* oibvh_last_error(void);
/* Library version: major * 10000 + minor * 100 + patch. */
int oibvh_version(void);
/* Kernels this library has launched so far in this process (all devices). */
uint64_t oibvh_get_launch_count(void);

/* Test hook for the out-of-memory paths (no counterpart in the reference,
 * which ignores every CUDA error, include/cuda/utils.cuh:6-34): the n-th
 * device or pinned-host allocation this library attempts from now on (n = 0:
 * the next one) fails as cudaMalloc would with cudaErrorMemoryAllocation, but
 * without calling CUDA, so OIBVH_ERR_OOM can be driven on a healthy device;
 * the hook is then off again. n < 0 switches it off. Process-wide; inert
 * unless called. */
int oibvh_debug_fail_alloc_after(int64_t n);
/* Device and pinned-host allocations attempted so far (process-wide). */
uint64_t oibvh_debug_alloc_attempts(void);

/* ------------------------------------------------------------------ tree */

/* OibvhTree::OibvhTree(std::shared_ptr<Mesh>) + setup()
 * (src/cuda/oibvhTree.cu:9-15,157-191): copies the mesh's positions and
 * faces to `device`. Face indices are checked against n_vertices. */
int oibvh_tree_create(const float* xyz, uint32_t n_vertices, const uint32_t* tri, uint32_t n_triangles, int device,
                      oibvh_tree_t* out);

/* OibvhTree::OibvhTree(std::shared_ptr<OibvhTree>, std::shared_ptr<Mesh>)
 * (src/cuda/oibvhTree.cu:17-33): a tree over a copy of `other`'s mesh with
 * new positions. It keeps `other`'s Morton order (the reference never
 * rebuilds a copied tree, src/main.cpp:132-135); call oibvh_tree_refit next.
 * `other` must be built. */
int oibvh_tree_create_copy(oibvh_tree_t other, const float* xyz, uint32_t n_vertices, oibvh_tree_t* out);

/* OibvhTree::build() (src/cuda/oibvhTree.cu:237-388): mesh bounds, Morton
 * codes, stable radix sort, then every tree level. The tree then keeps its
 * vertices numbered in the order the sorted faces first use them (so that
 * consecutive leaves gather nearby positions); this is internal: every call
 * takes and returns vertices in the caller's numbering. Blocking. */
int oibvh_tree_build(oibvh_tree_t t, void* stream);

/* OibvhTree::refit() (src/cuda/oibvhTree.cu:193-235): new leaf boxes from the
 * mesh's current positions, then every level. `xyz` is a host array of
 * 3 * n_vertices floats copied to the device first, or NULL to refit to the
 * positions already held. Stream-ordered (not blocking). */
int oibvh_tree_refit(oibvh_tree_t t, const float* xyz, void* stream);

/* Same as oibvh_tree_refit with the xyz positions already in device memory
 * (4-byte aligned); they are converted into the tree's own device layout,
 * stream-ordered, so `d_xyz` may be reused once the stream has passed. */
int oibvh_tree_refit_device(oibvh_tree_t t, const float* d_xyz, void* stream);

/* Set the positions the next refit (of this tree, or of its scene) and the
 * next detect use, without refitting. The reference moves vertices through
 * Mesh::transform and reads them back in OibvhTree::refit
 * (src/utils/mesh.cpp:187-214, src/cuda/oibvhTree.cu:196-199).
 *   _set_positions:          host xyz, copied (stream-ordered);
 *   _set_positions_device:   device xyz, converted (stream-ordered);
 *   _set_positions4_device:  device xyzw, 16 bytes per vertex,
 *                            16-byte aligned, kept by reference: every
 *                            following refit (of this tree or of its scene)
 *                            first reads it into the tree's own buffer (one
 *                            gather pass, in the tree's vertex order), until
 *                            other positions are set; the caller keeps it
 *                            alive and unchanged while those refits run. A
 *                            detect reads the positions of the last refit.
 * Inside the library every vertex is a 16-byte (x, y, z, unused) record, so
 * each vertex gather is one vector load. */
int oibvh_tree_set_positions(oibvh_tree_t t, const float* xyz, void* stream);
int oibvh_tree_set_positions_device(oibvh_tree_t t, const float* d_xyz, void* stream);
int oibvh_tree_set_positions4_device(oibvh_tree_t t, const float* d_xyzw);

/* OibvhTree::getDepth() (src/cuda/oibvhTree.cu:46-49) = floor(log2(size)). */
/* Morton key width of the next build (OibvhTree::build, src/cuda/oibvh.cu:17-22
 * uses 30 bits: 10 per axis). 63 (21 bits per axis) orders the leaves of
 * large meshes more finely; the pair set does not depend on it. Default 30;
 * a scene build needs the same width for all its trees. */
int oibvh_tree_set_morton_bits(oibvh_tree_t t, uint32_t bits);
uint32_t oibvh_tree_get_morton_bits(oibvh_tree_t t);
uint32_t oibvh_tree_get_depth(oibvh_tree_t t);
/* OibvhTree::getPrimCount() (src/cuda/oibvhTree.cu:51-54). */
uint32_t oibvh_tree_get_prim_count(oibvh_tree_t t);
/* m_aabbTree.size() (src/cuda/oibvhTree.cu:375): oibvh_get_size(T). */
uint32_t oibvh_tree_get_size(oibvh_tree_t t);

/* m_aabbTree (src/cuda/oibvhTree.cu:232,375-376): the level-ordered real
 * nodes, root first, 6 floats each (min xyz, max xyz). Blocking. */
int oibvh_tree_get_aabbs(oibvh_tree_t t, float* out6, uint64_t cap_nodes);

/* m_faces after build (src/cuda/oibvhTree.cu:377): the faces in Morton
 * order (vertex indices in the caller's numbering), and perm[i] = original
 * index of sorted face i (either output may be NULL). Blocking. */
int oibvh_tree_get_sorted_faces(oibvh_tree_t t, uint32_t* out3, uint32_t* perm, uint64_t cap);

int oibvh_tree_destroy(oibvh_tree_t t);

/* ----------------------------------------------------------------- scene */

/* Scene::Scene() (src/cuda/scene.cu:12-34) on a device. */
int oibvh_scene_create(int device, oibvh_scene_t* out);

/* Scene::addOibvhTree (src/cuda/scene.cu:95-129). The scene refers to the
 * tree (no copy); *id is its index, reported as bvhIndex in the pairs. */
int oibvh_scene_add_tree(oibvh_scene_t s, oibvh_tree_t t, uint32_t* id);

/* Which tree pairs are tested. pairs = NULL (the default) means every i < j,
 * the reference's behaviour (src/cuda/scene.cu:195-196); otherwise n_pairs
 * (a, b) id pairs, a != b. */
int oibvh_scene_set_pairs(oibvh_scene_t s, const uint32_t* pairs, uint32_t n_pairs);

/* Scene::detectCollision(deviceType, entryLevel, expandLevels)
 * (src/cuda/scene.cu:157-185,225-446): BVTT broad phase from the cross
 * product of the nodes at entry_level (clamped to each tree's leaf level),
 * with the triangle test fused into the traversal. The pair set does not
 * depend on entry_level or expand_levels (they only shape the reference's
 * work): entry_level sets the initial front as in the reference.
 * expand_levels is validated (1..16) and otherwise has NO effect here: not on
 * the result, not on the work done. The reference expands 2^e x 2^e children
 * of every front pair unconditionally (src/cuda/collide.cu:165-176); this
 * traversal always descends one level per step and tests each child pair
 * before queueing it, which visits a subset of the pairs the reference
 * visits, so a caller porting detectCollision(GPU0, 4, 3) gets no tuning
 * from it (oibvh_scene_set_tuning / oibvh_scene_autotune shape the work
 * instead). Blocking: returns once the pair count is known. */
int oibvh_scene_detect(oibvh_scene_t s, int device_type, uint32_t entry_level, uint32_t expand_levels, void* stream);

/* The two halves of detect (src/cuda/scene.cu:270-311 and :382-423):
 * broad leaves the candidate leaf pairs on the device (blocking, it reads
 * their count); narrow tests them (blocking). */
int oibvh_scene_broad(oibvh_scene_t s, int device_type, uint32_t entry_level, uint32_t expand_levels, void* stream);
int oibvh_scene_narrow(oibvh_scene_t s, void* stream);

/* OibvhTree::refit() for every tree of the scene in ONE kernel launch, each
 * to its current positions (oibvh_tree_set_positions*). Stream-ordered. The
 * reference refits tree by tree with a host round trip each
 * (src/main.cpp:210-214,247-251, src/cuda/oibvhTree.cu:193-235). */
int oibvh_scene_refit(oibvh_scene_t s, void* stream);

/* Scene::getIntTriPairCount() (src/cuda/scene.cu:50-53). */
uint32_t oibvh_scene_get_int_tri_pair_count(oibvh_scene_t s);
/* Candidate (overlapping leaf box) pairs of the last broad phase
 * (printed by the reference at src/cuda/scene.cu:316-322). */
uint64_t oibvh_scene_get_candidate_count(oibvh_scene_t s);

/* m_intTriPairs (include/cuda/scene.cuh:133; private in the reference):
 * records {bvhA, bvhB, triA, triB}, 4 uint32 each, tri indices are the
 * ORIGINAL face indices of each mesh, in no particular order. Writes
 * min(cap, count) records, *n = count. Blocking. */
int oibvh_scene_get_int_tri_pairs(oibvh_scene_t s, uint32_t* out4, uint64_t cap, uint64_t* n);

/* Candidate leaf pairs of the last broad phase as {bvhA, bvhB, sortedA,
 * sortedB} records (Morton-order leaf indices, the reference GPU path's
 * tri_pair_node_t). Blocking. */
int oibvh_scene_get_candidates(oibvh_scene_t s, uint32_t* out4, uint64_t cap, uint64_t* n);

/* Starting capacities (entries) of the BVTT front, candidate and hit queues.
 * They grow on demand (an overflow is detected on the device and the pass
 * reruns), so this only trades memory against reruns. 0 keeps a value. */
int oibvh_scene_set_queue_capacity(oibvh_scene_t s, uint32_t front, uint32_t candidates, uint32_t hits);

/* Build every tree of the scene with one launch per build stage, whatever
 * the number of trees (bounds, Morton codes, one stable sort by code and then
 * by tree, gather, one refit for all): the batched form of
 * OibvhTree::build() (src/cuda/oibvhTree.cu:237-388). Trees may be added
 * unbuilt for this. Blocking. */
int oibvh_scene_build(oibvh_scene_t s, void* stream);

/* Rigid transforms of every tree on the device, one launch (the reference
 * transforms on the host and round-trips through Transform::transformVec4,
 * src/cuda/transform.cu:18-41, src/utils/mesh.cpp:187-214): tree i's
 * positions become M_i * rest_i, with d_rest_xyzw the rest positions of all
 * trees packed in tree order (16 B per vertex, 16-byte aligned) and d_mats
 * 12 floats per tree (row-major 3x4; x' = ((m0 x + m1 y) + m2 z) + m3, each
 * operation rounded on its own). Stream-ordered; follow with oibvh_scene_refit. */
int oibvh_scene_transform(oibvh_scene_t s, const float* d_rest_xyzw, const float* d_mats, void* stream);

/* Traversal tuning (also chosen by oibvh_scene_autotune). */
typedef struct oibvh_tuning {
    uint32_t start_pairs_log2;    /* start cross product ~ 2^this node pairs per pass (8..24, default 16) */
    uint32_t handoff;             /* front width at which one CTA hands the walk to all warps (32..8192, 2048) */
    uint32_t walk_blocks_per_sm;  /* walker CTAs per SM, 0 = as many as fit */
    uint32_t front_capacity;      /* starting work-list capacity (entries), 0 = keep */
    uint32_t hit_capacity;        /* starting hit-queue capacity (records), 0 = keep */
    uint32_t walk_front;          /* per-warp queue of the walkers, node pairs (multiple of 32, <= 512, at least 64 used; 128; 0 = keep) */
    uint32_t refit_group_log2;    /* refit level-group depth: levels one CTA reduces (9, 10, 11; 10; 0 = keep) */
    uint32_t descend_ratio;       /* a node pair's two sides descend together while their boxes' squared
                                     diagonals are within this factor, else only the larger (1..2^30, 16;
                                     2^30: always together; 0 = keep) */
    uint32_t claim_min;           /* walkers claim work-list items dynamically (up to 32 at a time) when a
                                     list holds at least this many items per warp, else each takes a
                                     static interleaved share (1..2^20, 1; 0 = keep) */
} oibvh_tuning;
int oibvh_scene_set_tuning(oibvh_scene_t s, const oibvh_tuning* t);
int oibvh_scene_get_tuning(oibvh_scene_t s, oibvh_tuning* t);
/* Project-written autotuner: times `reps` scene refits per refit level-group
 * depth, then `reps` detects of the scene's current state per setting, by
 * coordinate descent (start size x handoff, then the walkers' per-warp queue
 * capacity, then the descend ratio, then the claim threshold, then walker
 * CTAs per SM), keeps the fastest, and sizes the queues
 * from the observed peaks with 2x headroom. Blocking; *chosen may be NULL. */
int oibvh_scene_autotune(oibvh_scene_t s, uint32_t entry_level, uint32_t reps, oibvh_tuning* chosen);

/* A whole frame as one CUDA graph: [oibvh_scene_transform(d_rest, d_mats)]
 * + [oibvh_scene_refit] (when refit != 0) + the detect of every pair (at most
 * 16384 pairs, fixed number of traversal rounds, results to pinned memory).
 * capture_frame runs one ordinary frame first (it sizes the queues with 2x
 * headroom and uploads the tables), then captures. launch_frame replays the
 * graph (re-capturing first if the scene or tuning changed); finish_frame
 * waits for it and validates: if a queue overflowed, it reruns the detect the
 * synchronous way and marks the graph for re-capture, so results are always
 * complete. Matrix contents at d_mats may change between launches; the rest
 * positions are copied at capture (in each tree's vertex order), so capture
 * again after changing them. */
int oibvh_scene_capture_frame(oibvh_scene_t s, uint32_t entry_level, uint32_t expand_levels, int refit,
                              const float* d_rest_xyzw, const float* d_mats, void* stream);
int oibvh_scene_launch_frame(oibvh_scene_t s, void* stream);
int oibvh_scene_finish_frame(oibvh_scene_t s, void* stream);

/* Per-stage device times of one frame (milliseconds, CUDA events on the
 * caller's stream between the stages). */
typedef struct oibvh_frame_profile {
    float transform_ms;    /* rigid transforms of every tree (0 without) */
    float refit_ms;        /* the one refit launch (0 without) */
    float start_ms;        /* start front + top walk */
    float walk_ms;         /* every captured walk round */
    float narrow_ms;       /* precision mode's narrow phase (0 in float mode) */
    uint32_t walk_rounds;  /* walk rounds launched */
    uint32_t kernels;      /* kernels launched */
} oibvh_frame_profile;
/* One frame of the captured work (oibvh_scene_capture_frame) enqueued stage
 * by stage instead of as the graph, with CUDA events between the stages, so
 * that each stage's device time can be read; the same kernels with the same
 * arguments. Blocking; afterwards the results are those of the frame, as
 * after oibvh_scene_finish_frame. No counterpart in the reference, whose
 * stages print their own timers (src/cuda/scene.cu:299,320,419). */
int oibvh_scene_profile_frame(oibvh_scene_t s, void* stream, oibvh_frame_profile* out);

/* Arithmetic of the triangle test. OIBVH_PRECISION_FP32 (the default) is
 * the reference's float test, operation for operation (src/utils/utils.cpp:71-169):
 * the pair set is the reference's bit for bit. OIBVH_PRECISION_FP64_FILTERED
 * has no counterpart in the reference: every axis test is evaluated in float
 * with a forward error bound on its two margins, and an axis whose margins
 * lie within the bound of zero is evaluated again in FP64; the pair set then
 * equals that of the same 17-axis test evaluated entirely in FP64 over the
 * same float inputs. In that mode the stats also count the FP64 work and the
 * candidates on which the float test and the FP64 test disagree. Takes
 * effect at the next detect (a captured frame is re-captured). */
enum {
    OIBVH_PRECISION_FP32 = 0,
    OIBVH_PRECISION_FP64_FILTERED = 1,
};
int oibvh_scene_set_precision(oibvh_scene_t s, int mode);
int oibvh_scene_get_precision(oibvh_scene_t s);

/* Per-detect diagnostics: passes, BVTT steps, queue regrowths, nodes tested. */
typedef struct oibvh_detect_stats {
    uint32_t passes;         /* pair batches */
    uint32_t steps;          /* BVTT steps of the last pass */
    uint32_t retries;        /* queue regrowths */
    uint32_t frame_redos;    /* captured frames redone synchronously, since the scene was created */
    uint64_t nodes_tested;   /* BVTT nodes tested, all passes */
    uint64_t candidates;
    uint64_t hits;
    uint64_t front_peak;     /* largest front */
    uint64_t fp64_axes;      /* precision mode: axis tests evaluated again in FP64 */
    uint64_t fp64_candidates;     /* precision mode: candidates with at least one such axis */
    uint64_t fp32_disagreements;  /* precision mode: candidates where float and FP64 answers differ */
    uint64_t bounded_candidates;  /* precision mode: candidates the plain float test and its margin bound
                                     left open, which took the bounded float pass */
} oibvh_detect_stats;
int oibvh_scene_get_stats(oibvh_scene_t s, oibvh_detect_stats* out);

int oibvh_scene_destroy(oibvh_scene_t s);

/* ------------------------------------------------------------ serving */

/* A request loop over a pool of resident meshes with continuous batching.
 * No counterpart in the reference (its Scene detects a fixed set of meshes
 * per call, src/cuda/scene.cu:157-185); each query runs the reference's
 * steps for one pair: B transformed by a rigid transform (Mesh::transform),
 * B's tree refit (OibvhTree::refit), broad + narrow phase against A at rest
 * (Scene::detectCollision).
 *
 * create: a device arena of memory_budget_bytes holds one slot per admitted
 * query (B's transformed positions and tree boxes, 16 B per vertex + 32 B per
 * internal node), allocated up front; n_lanes CUDA streams each carry one
 * batch at a time (at most max_batch queries). add_mesh registers built
 * trees (their current positions are the rest positions; the trees must
 * outlive the server); start allocates every lane's staging tables (for
 * max_batch queries), BVTT work lists and hit queue with its pinned host
 * copy, then launches the loop thread, so that the loop allocates only when
 * a batch is redone with larger queues. submit is
 * thread-safe and returns at once; a query waits until its slot fits in the
 * arena (FIFO) and a lane is idle, then runs with every query admitted at
 * that moment. wait blocks until the query is done (OIBVH_ERR_TIMEOUT after
 * timeout_ms); get_pairs returns its (triA, triB) pairs, original face
 * indices, 2 uint32 each; release frees its record. A query's pair set does
 * not depend on what it was batched with. destroy finishes the queries
 * already submitted, then stops. */
typedef struct oibvh_server_s* oibvh_server_t;
enum {
    OIBVH_QUERY_QUEUED = 0,
    OIBVH_QUERY_RUNNING = 1,
    OIBVH_QUERY_DONE = 2,
    OIBVH_QUERY_FAILED = 3,
};
typedef struct oibvh_query_result {
    int status;           /* OIBVH_QUERY_* */
    int error;            /* OIBVH_OK, or the status of its failed batch */
    uint32_t lane;        /* lane (stream) it ran on */
    uint32_t batch_size;  /* queries launched with it */
    uint64_t n_pairs;     /* colliding triangle pairs */
    double queue_us;      /* submit -> launch */
    double service_us;    /* launch -> results on the host */
} oibvh_query_result;
typedef struct oibvh_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t batches, max_batch_seen;
    uint64_t redos;              /* batches redone with larger queues */
    uint64_t candidates, hits;
    uint64_t arena_bytes, arena_used_bytes, arena_peak_bytes;
    uint64_t queued;             /* waiting for admission */
} oibvh_server_stats;
/* max_batch: queries per batch, 1..16384 (one traversal pass); n_lanes:
 * 1..16; the memory budget (>= 1 MiB) is allocated at once. */
int oibvh_server_create(int device, uint64_t memory_budget_bytes, uint32_t max_batch, uint32_t n_lanes,
                        oibvh_server_t* out);
int oibvh_server_set_entry_level(oibvh_server_t s, uint32_t entry_level);
/* Starting capacities (entries) of each lane's BVTT work lists and hit
 * queue; they grow on demand (the batch is redone). 0 keeps a value. */
int oibvh_server_set_queue_capacity(oibvh_server_t s, uint32_t front, uint32_t hits);
/* Largest batch, in triangles of A + B summed over its queries (default
 * 32 Mi; 0 = no limit). A batch completes as a whole, so this bounds how
 * long one query can wait for the others of its batch; a single query
 * larger than the limit still runs, alone. */
int oibvh_server_set_batch_cost(oibvh_server_t s, uint64_t max_triangles);
int oibvh_server_add_mesh(oibvh_server_t s, oibvh_tree_t t, uint32_t* id);
int oibvh_server_start(oibvh_server_t s);
int oibvh_server_submit(oibvh_server_t s, uint32_t mesh_a, uint32_t mesh_b, const float* mat_b, uint64_t* ticket);
int oibvh_server_wait(oibvh_server_t s, uint64_t ticket, uint32_t timeout_ms, oibvh_query_result* out);
int oibvh_server_get_pairs(oibvh_server_t s, uint64_t ticket, uint32_t* out2, uint64_t cap, uint64_t* n);
int oibvh_server_release(oibvh_server_t s, uint64_t ticket);
int oibvh_server_get_stats(oibvh_server_t s, oibvh_server_stats* out);
int oibvh_server_destroy(oibvh_server_t s);

/* ------------------------------------------------------- no allocation */

/* Collision detection for ONE mesh pair (tree a against tree b) that
 * allocates nothing: no device memory, no pinned host memory. This entry
 * point has no counterpart in the reference; it exists for callers that must
 * not allocate while they run: a frame loop with a hard time budget (cudaMalloc
 * may synchronise the whole device and take an unbounded time), or an
 * application whose device memory is all reserved up front by an outside pool
 * allocator, so that a library may not make allocations of its own.
 *
 * The traversal runs the same kernels as oibvh_scene_detect over a fixed
 * scratch area compiled into the library: about 4 MB of device memory held on
 * every GPU that loads the library until the process exits, with room for
 * 262,144 queued node pairs per work list. A pair that needs more returns
 * OIBVH_ERR_OVERFLOW (use oibvh_scene_detect, which grows its queues); an
 * entry_level whose starting cross product exceeds 64 x 262,144 node pairs is
 * rejected with OIBVH_ERR_ARG.
 *
 * Inputs: two built trees on the same device (created beforehand). Output:
 * up to out_cap records {0, 1, triA, triB} (original face indices; 0 and 1
 * name a and b) written to the DEVICE buffer d_out4, which must be 16-byte
 * aligned (else OIBVH_ERR_ARG); *n_hits receives the number of colliding
 * pairs, also when it exceeds out_cap (then the call returns
 * OIBVH_ERR_OVERFLOW). Blocking.
 *
 * The first call on a device resolves the scratch address (cudaGetSymbolAddress
 * with that device current) and caches it with the id of the device's
 * context: make that first call at start-up. A call in a new
 * context (after cudaDeviceReset) resolves it again. All calls share the one
 * scratch area and overwrite it (the counters are cleared at the start of
 * each call); calls whose GPU work overlaps (different host threads or
 * streams) race and must be serialised by the caller. */
int oibvh_pair_detect_noalloc(oibvh_tree_t a, oibvh_tree_t b, uint32_t entry_level, uint32_t* d_out4,
                              uint32_t out_cap, uint32_t* n_hits, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OIBVH_GB300_H */
