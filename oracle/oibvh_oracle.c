/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the oibvh reference's CPU collision path and of its
 * GPU tree layout, used as the checker for the CUDA library in oibvh_gb300/.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this code; the product path never links or calls it.
 *
 * Parity pin: every function below is cross-checked against the reference's
 * own C++ sources compiled unmodified into oracle/_ref/ (see ref_harness.cpp
 * and build_ref.sh) on seeded meshes; the resulting pair sets are committed
 * as golden fixtures under tests/golden/.
 *
 * Floating point: this file must be compiled with -ffp-contract=off so that
 * every product and sum is rounded on its own, exactly as the reference's
 * scalar glm code does (third/glm/detail/func_geometric.inl:48-55,68-79 with
 * GLM SIMD off, third/glm/detail/setup.hpp:804-808).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_API __attribute__((visibility("default")))

ORACLE_API int oracle_oibvh_refit(const float *xyz, const uint32_t *sorted_tri, uint32_t nT, float *aabbs);

/* ------------------------------------------------------------------------ */
/* glm scalar min/max: third/glm/detail/func_common.inl:17-29                */
/* ------------------------------------------------------------------------ */
static inline float glm_min(float x, float y) { return (y < x) ? y : x; }
static inline float glm_max(float x, float y) { return (x < y) ? y : x; }

typedef struct {
    float mn[3];
    float mx[3];
} box_t;

/* aabb_box_t default: min = +FLT_MAX, max = -FLT_MAX (include/utils/utils.h:17-18) */
static inline void box_default(box_t *b)
{
    for (int k = 0; k < 3; ++k) {
        b->mn[k] = FLT_MAX;
        b->mx[k] = -FLT_MAX;
    }
}

/* aabb_box_t::merge (include/utils/utils.h:33-37): m = min(m, o.min), M = max(M, o.max) */
static inline void box_merge(box_t *b, const box_t *o)
{
    for (int k = 0; k < 3; ++k) {
        b->mn[k] = glm_min(b->mn[k], o->mn[k]);
        b->mx[k] = glm_max(b->mx[k], o->mx[k]);
    }
}

static inline void box_merge_point(box_t *b, const float *p)
{
    for (int k = 0; k < 3; ++k) {
        b->mn[k] = glm_min(b->mn[k], p[k]);
        b->mx[k] = glm_max(b->mx[k], p[k]);
    }
}

/* aabb_box_t::overlap (include/utils/utils.h:39-44), inclusive on all axes */
static inline int box_overlap(const box_t *a, const box_t *b)
{
    return (a->mn[0] <= b->mx[0] && a->mx[0] >= b->mn[0]) &&
           (a->mn[1] <= b->mx[1] && a->mx[1] >= b->mn[1]) &&
           (a->mn[2] <= b->mx[2] && a->mx[2] >= b->mn[2]);
}

/* ------------------------------------------------------------------------ */
/* Triangle-triangle SAT: src/utils/utils.cpp:71-169                         */
/* ------------------------------------------------------------------------ */

/* glm::dot for vec3: tmp = a*b (three rounded products); (tmp.x + tmp.y) + tmp.z */
static inline float dot3(const float *a, const float *b)
{
    float t0 = a[0] * b[0];
    float t1 = a[1] * b[1];
    float t2 = a[2] * b[2];
    return (t0 + t1) + t2;
}

/* glm::cross: (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y) */
static inline void cross3(float *r, const float *x, const float *y)
{
    float r0 = x[1] * y[2] - y[1] * x[2];
    float r1 = x[2] * y[0] - y[2] * x[0];
    float r2 = x[0] * y[1] - y[0] * x[1];
    r[0] = r0;
    r[1] = r1;
    r[2] = r2;
}

static inline void sub3(float *r, const float *a, const float *b)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}

/* project6 (src/utils/utils.cpp:71-95): strict '>' separation */
static inline int project6(const float *ax, const float *p1, const float *p2, const float *p3,
                           const float *q1, const float *q2, const float *q3)
{
    float P1 = dot3(ax, p1), P2 = dot3(ax, p2), P3 = dot3(ax, p3);
    float Q1 = dot3(ax, q1), Q2 = dot3(ax, q2), Q3 = dot3(ax, q3);
    float mx1 = fmaxf(fmaxf(P1, P2), P3);
    float mn1 = fminf(fminf(P1, P2), P3);
    float mx2 = fmaxf(fmaxf(Q1, Q2), Q3);
    float mn2 = fminf(fminf(Q1, Q2), Q3);
    if (mn1 > mx2) return 0;
    if (mn2 > mx1) return 0;
    return 1;
}

/* triangleIntersect (src/utils/utils.cpp:97-169): 17 candidate axes */
ORACLE_API int oracle_tri_intersect(const float *P1, const float *P2, const float *P3,
                                    const float *Q1, const float *Q2, const float *Q3)
{
    float p1[3] = {0.0f, 0.0f, 0.0f}, p2[3], p3[3], q1[3], q2[3], q3[3];
    sub3(p2, P2, P1);
    sub3(p3, P3, P1);
    sub3(q1, Q1, P1);
    sub3(q2, Q2, P1);
    sub3(q3, Q3, P1);
    float e1[3], e2[3], e3[3], f1[3], f2[3], f3[3];
    sub3(e1, p2, p1);
    sub3(e2, p3, p2);
    sub3(e3, p1, p3);
    sub3(f1, q2, q1);
    sub3(f2, q3, q2);
    sub3(f3, q1, q3);
    float n1[3], m1[3];
    cross3(n1, e1, e2);
    cross3(m1, f1, f2);
    float ax[15][3];
    cross3(ax[0], e1, f1);
    cross3(ax[1], e1, f2);
    cross3(ax[2], e1, f3);
    cross3(ax[3], e2, f1);
    cross3(ax[4], e2, f2);
    cross3(ax[5], e2, f3);
    cross3(ax[6], e3, f1);
    cross3(ax[7], e3, f2);
    cross3(ax[8], e3, f3);
    cross3(ax[9], e1, n1);
    cross3(ax[10], e2, n1);
    cross3(ax[11], e3, n1);
    cross3(ax[12], f1, m1);
    cross3(ax[13], f2, m1);
    cross3(ax[14], f3, m1);
    if (!project6(n1, p1, p2, p3, q1, q2, q3)) return 0;
    if (!project6(m1, p1, p2, p3, q1, q2, q3)) return 0;
    for (int k = 0; k < 15; ++k)
        if (!project6(ax[k], p1, p2, p3, q1, q2, q3)) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* The same SAT evaluated in double precision over the same float inputs.   */
/* The reference has no FP64 path; this is the precision oracle for the     */
/* sheet-stress workload (project-written, same axes and same tests).       */
/* ------------------------------------------------------------------------ */
static inline double dot3d(const double *a, const double *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static inline void cross3d(double *r, const double *x, const double *y)
{
    double r0 = x[1] * y[2] - y[1] * x[2];
    double r1 = x[2] * y[0] - y[2] * x[0];
    double r2 = x[0] * y[1] - y[0] * x[1];
    r[0] = r0;
    r[1] = r1;
    r[2] = r2;
}
static inline void sub3d(double *r, const double *a, const double *b)
{
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
static inline int project6d(const double *ax, const double *p1, const double *p2, const double *p3,
                            const double *q1, const double *q2, const double *q3)
{
    double P1 = dot3d(ax, p1), P2 = dot3d(ax, p2), P3 = dot3d(ax, p3);
    double Q1 = dot3d(ax, q1), Q2 = dot3d(ax, q2), Q3 = dot3d(ax, q3);
    double mx1 = fmax(fmax(P1, P2), P3), mn1 = fmin(fmin(P1, P2), P3);
    double mx2 = fmax(fmax(Q1, Q2), Q3), mn2 = fmin(fmin(Q1, Q2), Q3);
    if (mn1 > mx2) return 0;
    if (mn2 > mx1) return 0;
    return 1;
}
ORACLE_API int oracle_tri_intersect_f64(const float *P1f, const float *P2f, const float *P3f,
                                        const float *Q1f, const float *Q2f, const float *Q3f)
{
    double P1[3], P2[3], P3[3], Q1[3], Q2[3], Q3[3];
    for (int k = 0; k < 3; ++k) {
        P1[k] = P1f[k]; P2[k] = P2f[k]; P3[k] = P3f[k];
        Q1[k] = Q1f[k]; Q2[k] = Q2f[k]; Q3[k] = Q3f[k];
    }
    double p1[3] = {0, 0, 0}, p2[3], p3[3], q1[3], q2[3], q3[3];
    sub3d(p2, P2, P1); sub3d(p3, P3, P1);
    sub3d(q1, Q1, P1); sub3d(q2, Q2, P1); sub3d(q3, Q3, P1);
    double e1[3], e2[3], e3[3], f1[3], f2[3], f3[3];
    sub3d(e1, p2, p1); sub3d(e2, p3, p2); sub3d(e3, p1, p3);
    sub3d(f1, q2, q1); sub3d(f2, q3, q2); sub3d(f3, q1, q3);
    double n1[3], m1[3], ax[15][3];
    cross3d(n1, e1, e2); cross3d(m1, f1, f2);
    cross3d(ax[0], e1, f1); cross3d(ax[1], e1, f2); cross3d(ax[2], e1, f3);
    cross3d(ax[3], e2, f1); cross3d(ax[4], e2, f2); cross3d(ax[5], e2, f3);
    cross3d(ax[6], e3, f1); cross3d(ax[7], e3, f2); cross3d(ax[8], e3, f3);
    cross3d(ax[9], e1, n1); cross3d(ax[10], e2, n1); cross3d(ax[11], e3, n1);
    cross3d(ax[12], f1, m1); cross3d(ax[13], f2, m1); cross3d(ax[14], f3, m1);
    if (!project6d(n1, p1, p2, p3, q1, q2, q3)) return 0;
    if (!project6d(m1, p1, p2, p3, q1, q2, q3)) return 0;
    for (int k = 0; k < 15; ++k)
        if (!project6d(ax[k], p1, p2, p3, q1, q2, q3)) return 0;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* SimpleBVH: src/cpu/simpleBVH.cpp:41-160 as a flat node array             */
/* ------------------------------------------------------------------------ */
typedef struct {
    box_t box;
    int32_t left, right; /* -1 when absent */
    int32_t tri;         /* -1 for internal nodes */
} sbvh_node_t;

typedef struct {
    sbvh_node_t *nodes;
    int64_t count, cap;
    int32_t root;
    uint32_t depth;
    const float *xyz;
    const uint32_t *tri;
} sbvh_t;

static uint32_t next_pow2_u32(uint32_t x)
{
    x--;
    x |= x >> 1; x |= x >> 2; x |= x >> 4; x |= x >> 8; x |= x >> 16;
    x++;
    return x;
}

static uint32_t ilog2_u32(uint32_t x) { return 31u - (uint32_t)__builtin_clz(x); }

static int32_t sbvh_new(sbvh_t *b)
{
    if (b->count == b->cap) {
        int64_t nc = b->cap ? b->cap * 2 : 1024;
        sbvh_node_t *nn = (sbvh_node_t *)realloc(b->nodes, (size_t)nc * sizeof(sbvh_node_t));
        if (!nn) return -1;
        b->nodes = nn;
        b->cap = nc;
    }
    int32_t id = (int32_t)b->count++;
    box_default(&b->nodes[id].box);
    b->nodes[id].left = b->nodes[id].right = -1;
    b->nodes[id].tri = -1;
    return id;
}

/* recursiveBuild (src/cpu/simpleBVH.cpp:122-160). Written with an explicit
 * stack so that million-triangle meshes do not exhaust the C stack; the
 * visiting order and the split rule are the reference's. */
typedef struct { int32_t lo, hi, depth, node, stage; } sbvh_frame_t;

static int sbvh_build(sbvh_t *b, uint32_t nT)
{
    b->count = 0;
    b->depth = ilog2_u32(next_pow2_u32(nT));
    int64_t scap = 64 + 4 * (int64_t)b->depth;
    sbvh_frame_t *st = (sbvh_frame_t *)malloc((size_t)scap * sizeof(sbvh_frame_t));
    if (!st) return -1;
    int64_t sp = 0;
    int32_t root = sbvh_new(b);
    if (root < 0) { free(st); return -1; }
    st[sp++] = (sbvh_frame_t){0, (int32_t)nT - 1, 0, root, 0};
    while (sp > 0) {
        sbvh_frame_t *f = &st[sp - 1];
        sbvh_node_t *nd;
        const int32_t lo = f->lo, hi = f->hi, depth = f->depth;
        const int32_t count = hi - lo + 1;
        const int chain = (lo == hi) ? (depth < (int32_t)b->depth)
                                     : (count <= (1 << (b->depth - (uint32_t)depth - 1)));
        if (lo == hi && !chain) {
            /* leaf: default box merged with the three vertices (:135-139) */
            nd = &b->nodes[f->node];
            const uint32_t *fc = b->tri + 3 * (size_t)lo;
            box_merge_point(&nd->box, b->xyz + 3 * (size_t)fc[0]);
            box_merge_point(&nd->box, b->xyz + 3 * (size_t)fc[1]);
            box_merge_point(&nd->box, b->xyz + 3 * (size_t)fc[2]);
            nd->tri = lo;
            sp--;
            continue;
        }
        if (f->stage == 0) {
            int32_t c = sbvh_new(b);
            if (c < 0) { free(st); return -1; }
            b->nodes[f->node].left = c;
            f->stage = 1;
            if (sp + 2 > scap) {
                scap *= 2;
                sbvh_frame_t *ns = (sbvh_frame_t *)realloc(st, (size_t)scap * sizeof(sbvh_frame_t));
                if (!ns) { free(st); return -1; }
                st = ns;
                f = &st[sp - 1];
            }
            if (chain)
                st[sp++] = (sbvh_frame_t){lo, hi, depth + 1, c, 0};
            else {
                int32_t mid = lo + (int32_t)(next_pow2_u32((uint32_t)count) / 2) - 1;
                st[sp++] = (sbvh_frame_t){lo, mid, depth + 1, c, 0};
            }
            continue;
        }
        if (f->stage == 1 && !chain) {
            int32_t c = sbvh_new(b);
            if (c < 0) { free(st); return -1; }
            b->nodes[f->node].right = c;
            f->stage = 2;
            int32_t mid = lo + (int32_t)(next_pow2_u32((uint32_t)count) / 2) - 1;
            if (sp + 2 > scap) {
                scap *= 2;
                sbvh_frame_t *ns = (sbvh_frame_t *)realloc(st, (size_t)scap * sizeof(sbvh_frame_t));
                if (!ns) { free(st); return -1; }
                st = ns;
                f = &st[sp - 1];
            }
            st[sp++] = (sbvh_frame_t){mid + 1, hi, depth + 1, c, 0};
            continue;
        }
        /* all children built: default box merged with left then right (:152,157-158) */
        nd = &b->nodes[f->node];
        box_merge(&nd->box, &b->nodes[nd->left].box);
        if (nd->right >= 0) box_merge(&nd->box, &b->nodes[nd->right].box);
        sp--;
    }
    free(st);
    b->root = root;
    return 0;
}

/* recursiveRefit (src/cpu/simpleBVH.cpp:96-115): leaves use init(p0,p0) then
 * merge p1, p2; internal nodes init(left) then merge(right). Children are
 * always created after their parent, so a reverse sweep over the node array
 * visits every child before its parent. */
static void sbvh_refit(sbvh_t *b, const float *xyz)
{
    b->xyz = xyz;
    for (int64_t i = b->count - 1; i >= 0; --i) {
        sbvh_node_t *nd = &b->nodes[i];
        if (nd->tri >= 0) {
            const uint32_t *fc = b->tri + 3 * (size_t)nd->tri;
            const float *p0 = xyz + 3 * (size_t)fc[0];
            for (int k = 0; k < 3; ++k) nd->box.mn[k] = nd->box.mx[k] = p0[k];
            box_merge_point(&nd->box, xyz + 3 * (size_t)fc[1]);
            box_merge_point(&nd->box, xyz + 3 * (size_t)fc[2]);
        } else {
            nd->box = b->nodes[nd->left].box;
            if (nd->right >= 0) box_merge(&nd->box, &b->nodes[nd->right].box);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Public oracle objects: a CPU "scene" of SimpleBVHs and the DFS detect.   */
/* ------------------------------------------------------------------------ */
typedef struct {
    sbvh_t *bvh;
    int n, cap;
} oracle_scene_t;

ORACLE_API void *oracle_scene_create(void)
{
    oracle_scene_t *s = (oracle_scene_t *)calloc(1, sizeof(oracle_scene_t));
    return s;
}

ORACLE_API void oracle_scene_destroy(void *h)
{
    oracle_scene_t *s = (oracle_scene_t *)h;
    if (!s) return;
    for (int i = 0; i < s->n; ++i) free(s->bvh[i].nodes);
    free(s->bvh);
    free(s);
}

/* SimpleBVH(mesh) + build() + SimpleCollide::addSimpleBVH. The caller keeps
 * xyz/tri alive for the life of the scene (the reference copies them; this
 * port only points at them). Returns the BVH id or -1. */
ORACLE_API int oracle_scene_add_mesh(void *h, const float *xyz, uint32_t nV, const uint32_t *tri, uint32_t nT)
{
    (void)nV;
    oracle_scene_t *s = (oracle_scene_t *)h;
    if (!s || nT == 0) return -1;
    if (s->n == s->cap) {
        int nc = s->cap ? s->cap * 2 : 4;
        sbvh_t *nb = (sbvh_t *)realloc(s->bvh, (size_t)nc * sizeof(sbvh_t));
        if (!nb) return -1;
        s->bvh = nb;
        s->cap = nc;
    }
    sbvh_t *b = &s->bvh[s->n];
    memset(b, 0, sizeof(*b));
    b->xyz = xyz;
    b->tri = tri;
    if (sbvh_build(b, nT) != 0) return -1;
    return s->n++;
}

/* SimpleBVH::refit() with new positions for mesh `id`. */
ORACLE_API int oracle_scene_refit(void *h, int id, const float *xyz)
{
    oracle_scene_t *s = (oracle_scene_t *)h;
    if (!s || id < 0 || id >= s->n) return -1;
    sbvh_refit(&s->bvh[id], xyz);
    return 0;
}

typedef struct { int32_t a, b; uint32_t ia, ib; } dfs_item_t;

/* SimpleCollide::detect (src/cpu/simpleCollide.cpp:47-161) over the listed
 * mesh pairs (the reference lists every i<j; pass pairs=NULL for that).
 * Writes int_tri_pair records {bvhA, bvhB, triA, triB} with ORIGINAL face
 * indices; returns the number of hits (records beyond `cap` are counted but
 * not written). *n_candidates receives the number of leaf pairs tested. */
ORACLE_API int64_t oracle_scene_detect(void *h, const uint32_t *pairs, int n_pairs, uint32_t *out4, int64_t cap,
                                       int64_t *n_candidates)
{
    oracle_scene_t *s = (oracle_scene_t *)h;
    if (!s) return -1;
    int64_t scap = 1 << 16, sp = 0, hits = 0, cands = 0;
    dfs_item_t *st = (dfs_item_t *)malloc((size_t)scap * sizeof(dfs_item_t));
    if (!st) return -1;
    int np = pairs ? n_pairs : s->n * (s->n - 1) / 2;
    for (int p = 0, i = 0, j = 1; p < np; ++p) {
        uint32_t A, B;
        if (pairs) {
            A = pairs[2 * p];
            B = pairs[2 * p + 1];
        } else {
            A = (uint32_t)i;
            B = (uint32_t)j;
            if (++j == s->n) { ++i; j = i + 1; }
        }
        if (A >= (uint32_t)s->n || B >= (uint32_t)s->n) { free(st); return -1; }
        st[sp++] = (dfs_item_t){s->bvh[A].root, s->bvh[B].root, A, B};
        while (sp > 0) {
            dfs_item_t it = st[--sp];
            const sbvh_t *ba = &s->bvh[it.ia], *bb = &s->bvh[it.ib];
            const sbvh_node_t *na = &ba->nodes[it.a], *nb = &bb->nodes[it.b];
            if (!box_overlap(&na->box, &nb->box)) continue;
            if (na->tri >= 0 && nb->tri >= 0) {
                cands++;
                const uint32_t *fa = ba->tri + 3 * (size_t)na->tri, *fb = bb->tri + 3 * (size_t)nb->tri;
                if (oracle_tri_intersect(ba->xyz + 3 * (size_t)fa[0], ba->xyz + 3 * (size_t)fa[1],
                                         ba->xyz + 3 * (size_t)fa[2], bb->xyz + 3 * (size_t)fb[0],
                                         bb->xyz + 3 * (size_t)fb[1], bb->xyz + 3 * (size_t)fb[2])) {
                    if (hits < cap && out4) {
                        out4[4 * hits + 0] = it.ia;
                        out4[4 * hits + 1] = it.ib;
                        out4[4 * hits + 2] = (uint32_t)na->tri;
                        out4[4 * hits + 3] = (uint32_t)nb->tri;
                    }
                    hits++;
                }
                continue;
            }
            int32_t ca[2], cb[2];
            int nca = 0, ncb = 0;
            if (na->tri >= 0) ca[nca++] = it.a;
            else {
                ca[nca++] = na->left;
                if (na->right >= 0) ca[nca++] = na->right;
            }
            if (nb->tri >= 0) cb[ncb++] = it.b;
            else {
                cb[ncb++] = nb->left;
                if (nb->right >= 0) cb[ncb++] = nb->right;
            }
            if (sp + 4 > scap) {
                scap *= 2;
                dfs_item_t *ns = (dfs_item_t *)realloc(st, (size_t)scap * sizeof(dfs_item_t));
                if (!ns) { free(st); return -1; }
                st = ns;
            }
            for (int x = 0; x < nca; ++x)
                for (int y = 0; y < ncb; ++y) st[sp++] = (dfs_item_t){ca[x], cb[y], it.ia, it.ib};
        }
    }
    free(st);
    if (n_candidates) *n_candidates = cands;
    return hits;
}

/* Brute force over all leaf pairs of two meshes with an FP64 SAT. This is
 * the all-FP64 oracle pair set for the precision workload: the candidate
 * set is the same exact-AABB set, the triangle test runs in double. */
ORACLE_API int64_t oracle_scene_detect_f64(void *h, const uint32_t *pairs, int n_pairs, uint32_t *out4, int64_t cap)
{
    oracle_scene_t *s = (oracle_scene_t *)h;
    if (!s) return -1;
    int64_t scap = 1 << 16, sp = 0, hits = 0;
    dfs_item_t *st = (dfs_item_t *)malloc((size_t)scap * sizeof(dfs_item_t));
    if (!st) return -1;
    int np = pairs ? n_pairs : s->n * (s->n - 1) / 2;
    for (int p = 0, i = 0, j = 1; p < np; ++p) {
        uint32_t A, B;
        if (pairs) { A = pairs[2 * p]; B = pairs[2 * p + 1]; }
        else { A = (uint32_t)i; B = (uint32_t)j; if (++j == s->n) { ++i; j = i + 1; } }
        if (A >= (uint32_t)s->n || B >= (uint32_t)s->n) { free(st); return -1; }
        st[sp++] = (dfs_item_t){s->bvh[A].root, s->bvh[B].root, A, B};
        while (sp > 0) {
            dfs_item_t it = st[--sp];
            const sbvh_t *ba = &s->bvh[it.ia], *bb = &s->bvh[it.ib];
            const sbvh_node_t *na = &ba->nodes[it.a], *nb = &bb->nodes[it.b];
            if (!box_overlap(&na->box, &nb->box)) continue;
            if (na->tri >= 0 && nb->tri >= 0) {
                const uint32_t *fa = ba->tri + 3 * (size_t)na->tri, *fb = bb->tri + 3 * (size_t)nb->tri;
                if (oracle_tri_intersect_f64(ba->xyz + 3 * (size_t)fa[0], ba->xyz + 3 * (size_t)fa[1],
                                             ba->xyz + 3 * (size_t)fa[2], bb->xyz + 3 * (size_t)fb[0],
                                             bb->xyz + 3 * (size_t)fb[1], bb->xyz + 3 * (size_t)fb[2])) {
                    if (hits < cap && out4) {
                        out4[4 * hits + 0] = it.ia; out4[4 * hits + 1] = it.ib;
                        out4[4 * hits + 2] = (uint32_t)na->tri; out4[4 * hits + 3] = (uint32_t)nb->tri;
                    }
                    hits++;
                }
                continue;
            }
            int32_t ca[2], cb[2];
            int nca = 0, ncb = 0;
            if (na->tri >= 0) ca[nca++] = it.a;
            else { ca[nca++] = na->left; if (na->right >= 0) ca[nca++] = na->right; }
            if (nb->tri >= 0) cb[ncb++] = it.b;
            else { cb[ncb++] = nb->left; if (nb->right >= 0) cb[ncb++] = nb->right; }
            if (sp + 4 > scap) {
                scap *= 2;
                dfs_item_t *ns = (dfs_item_t *)realloc(st, (size_t)scap * sizeof(dfs_item_t));
                if (!ns) { free(st); return -1; }
                st = ns;
            }
            for (int x = 0; x < nca; ++x)
                for (int y = 0; y < ncb; ++y) st[sp++] = (dfs_item_t){ca[x], cb[y], it.ia, it.ib};
        }
    }
    free(st);
    return hits;
}

/* Leaf boxes of a built SimpleBVH in original face order (for checks). */
ORACLE_API int oracle_scene_leaf_boxes(void *h, int id, float *out6)
{
    oracle_scene_t *s = (oracle_scene_t *)h;
    if (!s || id < 0 || id >= s->n) return -1;
    const sbvh_t *b = &s->bvh[id];
    for (int64_t i = 0; i < b->count; ++i) {
        const sbvh_node_t *nd = &b->nodes[i];
        if (nd->tri >= 0) {
            memcpy(out6 + 6 * (size_t)nd->tri, nd->box.mn, 3 * sizeof(float));
            memcpy(out6 + 6 * (size_t)nd->tri + 3, nd->box.mx, 3 * sizeof(float));
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* oibvh (GPU path) restatement: src/cuda/oibvh.cu, src/cuda/oibvhTree.cu    */
/* ------------------------------------------------------------------------ */

/* oibvh_get_size (include/cuda/oibvh.cuh:56-59) */
ORACLE_API uint32_t oracle_oibvh_size(uint32_t t)
{
    if (t == 1) return 1;
    return 2u * t + (uint32_t)__builtin_popcount(next_pow2_u32(t) - t) - 1u;
}

/* strech_by_3 / morton3D (src/cuda/oibvh.cu:6-22). The clamp is thrust's
 * max(a,b)=a<b?b:a then min(a,b)=b<a?b:a; the float->unsigned conversion
 * truncates toward zero and maps NaN to 0, which is what the device's
 * cvt.rzi.u32.f32 does. */
static inline uint32_t stretch3(uint32_t x)
{
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x30000ffu;
    x = (x | (x << 8)) & 0x300f00fu;
    x = (x | (x << 4)) & 0x30c30c3u;
    x = (x | (x << 2)) & 0x9249249u;
    return x;
}
static inline uint32_t quant1024(float u)
{
    float v = u * 1024.0f;
    v = (v < 0.0f) ? 0.0f : v;      /* thrust::max(v, 0) */
    v = (1023.0f < v) ? 1023.0f : v; /* thrust::min(v, 1023) */
    if (v != v) return 0u;
    return (uint32_t)v;
}

/* Mesh AABB over all vertices (src/utils/mesh.cpp:91-98). */
ORACLE_API void oracle_mesh_aabb(const float *xyz, uint32_t nV, float *out6)
{
    box_t b;
    box_default(&b);
    for (uint32_t v = 0; v < nV; ++v)
        for (int k = 0; k < 3; ++k) {
            float p = xyz[3 * (size_t)v + k];
            b.mx[k] = glm_max(p, b.mx[k]);
            b.mn[k] = glm_min(p, b.mn[k]);
        }
    memcpy(out6, b.mn, 3 * sizeof(float));
    memcpy(out6 + 3, b.mx, 3 * sizeof(float));
}

/* calculate_aabb_and_morton_kernel (src/cuda/oibvh.cu:42-70) for one face */
static inline void face_box(const float *xyz, const uint32_t *f, box_t *b)
{
    const float *v0 = xyz + 3 * (size_t)f[0], *v1 = xyz + 3 * (size_t)f[1], *v2 = xyz + 3 * (size_t)f[2];
    for (int k = 0; k < 3; ++k) {
        b->mn[k] = glm_min(glm_min(v0[k], v1[k]), v2[k]);
        b->mx[k] = glm_max(glm_max(v0[k], v1[k]), v2[k]);
    }
}

ORACLE_API void oracle_morton_codes(const float *xyz, uint32_t nV, const uint32_t *tri, uint32_t nT, uint32_t *codes)
{
    float mb[6];
    oracle_mesh_aabb(xyz, nV, mb);
    for (uint32_t i = 0; i < nT; ++i) {
        box_t b;
        face_box(xyz, tri + 3 * (size_t)i, &b);
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            float c = (b.mn[k] + b.mx[k]) * 0.5f;
            float off = c - mb[k];
            float len = mb[3 + k] - mb[k];
            q[k] = quant1024(off / len);
        }
        codes[i] = (stretch3(q[0]) << 2) | (stretch3(q[1]) << 1) | stretch3(q[2]);
    }
}

static int cmp_key_idx(const void *a, const void *b)
{
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* Build (src/cuda/oibvhTree.cu:237-388): Morton codes, stable sort of the
 * faces by code (ties keep the original order, :294-297), then every level
 * of the implicit tree bottom-up (src/cuda/oibvh.cu:156-219). Outputs the
 * level-ordered real-node array (root first, 6 floats per node: min, max),
 * the sorted faces, and perm[sorted] = original face index. */
ORACLE_API int oracle_oibvh_build(const float *xyz, uint32_t nV, const uint32_t *tri, uint32_t nT, float *aabbs,
                                  uint32_t *sorted_tri, uint32_t *perm)
{
    if (nT == 0) return -1;
    uint32_t *codes = (uint32_t *)malloc((size_t)nT * sizeof(uint32_t));
    uint64_t *ki = (uint64_t *)malloc((size_t)nT * sizeof(uint64_t));
    if (!codes || !ki) { free(codes); free(ki); return -1; }
    oracle_morton_codes(xyz, nV, tri, nT, codes);
    for (uint32_t i = 0; i < nT; ++i) ki[i] = ((uint64_t)codes[i] << 32) | i;
    qsort(ki, nT, sizeof(uint64_t), cmp_key_idx);
    for (uint32_t i = 0; i < nT; ++i) {
        uint32_t o = (uint32_t)(ki[i] & 0xffffffffu);
        perm[i] = o;
        memcpy(sorted_tri + 3 * (size_t)i, tri + 3 * (size_t)o, 3 * sizeof(uint32_t));
    }
    free(codes);
    free(ki);
    return oracle_oibvh_refit(xyz, sorted_tri, nT, aabbs);
}

/* Refit (src/cuda/oibvhTree.cu:193-235): leaf boxes of the sorted faces,
 * then each level l node j = merge(child 2j, child 2j+1 when real). Level l
 * holds ceil(n_{l+1}/2) real nodes, which is 2^l - (vl >> (L-l)) of
 * include/cuda/oibvh.cuh:81-85. */
ORACLE_API int oracle_oibvh_refit(const float *xyz, const uint32_t *sorted_tri, uint32_t nT, float *aabbs)
{
    if (nT == 0) return -1;
    const uint32_t size = oracle_oibvh_size(nT);
    uint32_t L = ilog2_u32(next_pow2_u32(nT));
    uint32_t *lvl_off = (uint32_t *)malloc((size_t)(L + 2) * sizeof(uint32_t));
    uint32_t *lvl_cnt = (uint32_t *)malloc((size_t)(L + 2) * sizeof(uint32_t));
    if (!lvl_off || !lvl_cnt) { free(lvl_off); free(lvl_cnt); return -1; }
    lvl_cnt[L] = nT;
    for (int l = (int)L - 1; l >= 0; --l) lvl_cnt[l] = (lvl_cnt[l + 1] + 1) / 2;
    lvl_off[0] = 0;
    for (uint32_t l = 1; l <= L; ++l) lvl_off[l] = lvl_off[l - 1] + lvl_cnt[l - 1];
    if (lvl_off[L] + nT != size) { free(lvl_off); free(lvl_cnt); return -2; }
    for (uint32_t i = 0; i < nT; ++i) {
        box_t b;
        face_box(xyz, sorted_tri + 3 * (size_t)i, &b);
        float *o = aabbs + 6 * (size_t)(lvl_off[L] + i);
        memcpy(o, b.mn, 3 * sizeof(float));
        memcpy(o + 3, b.mx, 3 * sizeof(float));
    }
    for (int l = (int)L - 1; l >= 0; --l) {
        for (uint32_t j = 0; j < lvl_cnt[l]; ++j) {
            const float *lc = aabbs + 6 * (size_t)(lvl_off[l + 1] + 2 * j);
            float *o = aabbs + 6 * (size_t)(lvl_off[l] + j);
            if (2 * j + 1 < lvl_cnt[l + 1]) {
                const float *rc = lc + 6;
                /* merge_aabb (src/cuda/oibvh.cu:72-78): glm::min(left, right), glm::max(left, right) */
                for (int k = 0; k < 3; ++k) {
                    o[k] = glm_min(lc[k], rc[k]);
                    o[3 + k] = glm_max(lc[3 + k], rc[3 + k]);
                }
            } else {
                memcpy(o, lc, 6 * sizeof(float));
            }
        }
    }
    free(lvl_off);
    free(lvl_cnt);
    return 0;
}
