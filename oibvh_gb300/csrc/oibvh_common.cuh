// Shared device/host definitions of the oibvh GB300 collision library.
//
// Tree layout (the reference's, include/cuda/oibvh.cuh:56-182): T primitives
// sorted by Morton code are the leaves of a complete binary tree of height
// L = log2(nextpow2(T)); the vl = 2^L - T rightmost leaves are "virtual" and
// every node whose subtree holds only virtual leaves is dropped. The remaining
// ("real") nodes are stored level by level, root first, left-justified. Level
// l holds real(l) = 2^l - (vl >> (L-l)) = ceil(real(l+1)/2) nodes, node j of
// level l merges children 2j and 2j+1 (the latter only when 2j+1 < real(l+1)).
//
// In HBM only the internal nodes (levels 0..L-1, the first size-T real nodes)
// are stored, 32 bytes each: float4 (min.xyz, 0) then float4 (max.xyz, 0), so
// a node is one aligned 32-byte sector and loads as two float4. A leaf's box
// is rebuilt from its 16-byte face record (v0, v1, v2, original index) and
// the three vertices when it is needed.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace oibvh {

constexpr uint32_t kMaxLeafLevel = 23;   // T <= 2^23 triangles per mesh
constexpr uint32_t kMaxPairsPerPass = 1u << 14;  // pair id field of a BVTT node

// BVTT node / candidate encoding: [pair:14][d:2][a:24][b:24], a and b are
// implicit indices (candidates: leaf indices in Morton order, d = 0). d is how
// the traversal expands the node pair: kDescendBoth = both sides' children,
// kDescendA = a's children against b, kDescendB = a against b's children.
enum : uint32_t { kDescendBoth = 0, kDescendA = 1, kDescendB = 2 };
__host__ __device__ __forceinline__ uint64_t bvtt_pack(uint32_t pair, uint32_t a, uint32_t b, uint32_t d = 0)
{
    return ((uint64_t)pair << 50) | ((uint64_t)d << 48) | ((uint64_t)a << 24) | (uint64_t)b;
}
__host__ __device__ __forceinline__ uint32_t bvtt_pair(uint64_t v) { return (uint32_t)(v >> 50); }
__host__ __device__ __forceinline__ uint32_t bvtt_desc(uint64_t v) { return (uint32_t)(v >> 48) & 3u; }
__host__ __device__ __forceinline__ uint32_t bvtt_a(uint64_t v) { return (uint32_t)(v >> 24) & 0xffffffu; }
__host__ __device__ __forceinline__ uint32_t bvtt_b(uint64_t v) { return (uint32_t)v & 0xffffffu; }

// next_power_of_two / ilog2 (include/cuda/utils.cuh:66-86)
__host__ __device__ __forceinline__ uint32_t next_pow2(uint32_t x)
{
    x--;
    x |= x >> 1;
    x |= x >> 2;
    x |= x >> 4;
    x |= x >> 8;
    x |= x >> 16;
    return x + 1;
}

__host__ __device__ __forceinline__ uint32_t ilog2(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return 31u - (uint32_t)__clz(x);
#else
    return 31u - (uint32_t)__builtin_clz(x);
#endif
}

__host__ __device__ __forceinline__ uint32_t popc(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__popc(x);
#else
    return (uint32_t)__builtin_popcount(x);
#endif
}

// Static shape of one tree (everything derives from T).
struct TreeShape {
    uint32_t L;    // leaf level
    uint32_t vl;   // virtual leaves
    uint32_t nT;   // real leaves
    uint32_t size; // real nodes, oibvh_get_size (include/cuda/oibvh.cuh:56-59)

    __host__ __device__ static TreeShape of(uint32_t nT)
    {
        TreeShape s;
        s.nT = nT;
        const uint32_t p = next_pow2(nT);
        s.L = ilog2(p);
        s.vl = p - nT;
        s.size = 2u * nT + popc(s.vl) - 1u;
        return s;
    }
    // real(l): include/cuda/oibvh.cuh:81-85
    __host__ __device__ __forceinline__ uint32_t level_count(uint32_t l) const
    {
        return (1u << l) - (vl >> (L - l));
    }
    // number of virtual nodes above level l (levels 0..l-1): oibvh.cuh:94-99
    __host__ __device__ __forceinline__ uint32_t virtual_above(uint32_t l) const
    {
        if (l == 0) return 0;
        const uint32_t vc = vl >> (L - (l - 1));
        return (vc << 1) - popc(vc);
    }
    // offset of level l in the real-node array
    __host__ __device__ __forceinline__ uint32_t level_offset(uint32_t l) const
    {
        return (1u << l) - 1u - virtual_above(l);
    }
    // implicit index -> real index (include/cuda/oibvh.cuh:108-113)
    __host__ __device__ __forceinline__ uint32_t real_index(uint32_t implicit) const
    {
        return implicit - virtual_above(ilog2(implicit + 1u));
    }
};

// Device view of one tree. 32-byte aligned: its first 32 bytes (the three
// arrays, the leaf level and the virtual-leaf count: all that a traversal
// step needs) are read as one 256-bit load (TreeRef).
struct alignas(32) TreeView {
    float4* box;        // 2*(size-nT) float4: level-ordered real internal nodes
    const uint4* face;  // Morton-sorted faces: (v0, v1, v2, original face index)
    const float4* pos;  // vertex positions, (x, y, z, unused) per vertex
    TreeShape shape;
    uint32_t nV;
    uint32_t pad0;
};
static_assert(offsetof(TreeView, shape) == 24 && offsetof(TreeShape, vl) == 4, "TreeRef is TreeView's first 32 bytes");

// The first 32 bytes of a TreeView, in registers.
struct TreeRef {
    float4* box;
    const uint4* face;
    const float4* pos;
    uint32_t L, vl;
    // index arithmetic only needs L and vl
    __device__ __forceinline__ TreeShape shape() const
    {
        TreeShape s;
        s.L = L;
        s.vl = vl;
        s.nT = 0;
        s.size = 0;
        return s;
    }
};

// One mesh pair of a detection pass. The two tree views are copied in, so a
// traversal step reads its pair's record and then the boxes (one dependent
// load fewer than going through the TreeView table).
struct PairView {
    uint32_t a, b;            // tree ids (index into the TreeView table)
    uint32_t front_off;       // first initial-front node of this pair
    uint32_t front_cnt_a;     // real nodes of A at the entry level
    uint32_t front_cnt_b;     // real nodes of B at the entry level
    uint32_t entry_a, entry_b;
    uint32_t pad0;
    TreeView ta, tb;          // copies of views a and b
};

// Status bits a kernel can raise (the host turns them into status codes).
enum DeviceFlag : uint32_t {
    kFlagFrontOverflow = 1u << 0,
    kFlagCandOverflow = 1u << 1,
    kFlagHitOverflow = 1u << 2,
    kFlagBadInput = 1u << 3,
    kFlagTimeout = 1u << 4,
};

// glm::min / glm::max semantics (third/glm/detail/func_common.inl:17-29).
__host__ __device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__host__ __device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }

// An axis-aligned box in registers: min xyz, max xyz.
struct Box {
    float nx, ny, nz, xx, xy, xz;
};

// merge_aabb (src/cuda/oibvh.cu:72-78): glm::min(left, right), glm::max(left, right)
__device__ __forceinline__ Box merge(const Box& l, const Box& r)
{
    return Box{gmin(l.nx, r.nx), gmin(l.ny, r.ny), gmin(l.nz, r.nz),
               gmax(l.xx, r.xx), gmax(l.xy, r.xy), gmax(l.xz, r.xz)};
}

// Box of one face (v0, v1, v2, .): glm::min(glm::min(v0, v1), v2) and the
// max likewise, as calculate_aabb_kernel (src/cuda/oibvh.cu:24-40); one
// 16-byte load per vertex.
__device__ __forceinline__ Box leaf_box(const float4* __restrict__ pos, uint4 f)
{
    const float4 a = __ldg(pos + f.x), b = __ldg(pos + f.y), c = __ldg(pos + f.z);
    return Box{gmin(gmin(a.x, b.x), c.x), gmin(gmin(a.y, b.y), c.y), gmin(gmin(a.z, b.z), c.z),
               gmax(gmax(a.x, b.x), c.x), gmax(gmax(a.y, b.y), c.y), gmax(gmax(a.z, b.z), c.z)};
}

// Internal nodes are 32 bytes, (min.xyz, 0, max.xyz, 0), and 32-byte
// aligned (node arrays start at cudaMalloc or 256-byte arena boundaries), so
// one node moves as ONE 256-bit access (the .v8 forms of ld/st, sm_100 and
// later) instead of two 128-bit ones: half the load/store instructions and
// L1 requests per node.
// Read-only path: for nodes written by an earlier kernel.
__device__ __forceinline__ Box load_node_nc(const float4* p)
{
    float a, b, c, e, f, g;
    [[maybe_unused]] float d, h;  // the two padding words
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a), "=f"(b), "=f"(c), "=f"(d), "=f"(e), "=f"(f), "=f"(g), "=f"(h)
        : "l"(p));
    return Box{a, b, c, e, f, g};
}
// L2 path (no L1): for nodes written by other CTAs of the same kernel.
__device__ __forceinline__ Box load_node_cg(const float4* p)
{
    float a, b, c, e, f, g;
    [[maybe_unused]] float d, h;
    asm volatile("ld.global.cg.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(a), "=f"(b), "=f"(c), "=f"(d), "=f"(e), "=f"(f), "=f"(g), "=f"(h)
                 : "l"(p)
                 : "memory");
    return Box{a, b, c, e, f, g};
}
__device__ __forceinline__ void store_node_v8(float4* p, const Box& v)
{
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(v.nx), "f"(v.ny),
                 "f"(v.nz), "f"(0.0f), "f"(v.xx), "f"(v.xy), "f"(v.xz), "f"(0.0f)
                 : "memory");
}

// Two consecutive 16-byte face records as one 256-bit read-only load
// (face arrays start at cudaMalloc boundaries; p must be 32-byte aligned).
__device__ __forceinline__ void load_face_pair(const uint4* p, uint4& f0, uint4& f1)
{
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(f0.x), "=r"(f0.y), "=r"(f0.z), "=r"(f0.w), "=r"(f1.x), "=r"(f1.y), "=r"(f1.z), "=r"(f1.w)
        : "l"(p));
}

// Box of a node given by implicit index and level: internal nodes are read
// from the tree (one 32-byte load), leaves are rebuilt from their face.
__device__ __forceinline__ Box node_box(const TreeView& T, uint32_t implicit, uint32_t level)
{
    if (level == T.shape.L) return leaf_box(T.pos, __ldg(T.face + implicit - ((1u << level) - 1u)));
    return load_node_nc(T.box + 2 * (size_t)T.shape.real_index(implicit));
}
__device__ __forceinline__ Box node_box(const TreeRef& T, uint32_t implicit, uint32_t level)
{
    if (level == T.L) return leaf_box(T.pos, __ldg(T.face + implicit - ((1u << level) - 1u)));
    return load_node_nc(T.box + 2 * (size_t)T.shape().real_index(implicit));
}

// Boxes of `first` and, when `two`, its right neighbour on the same level.
// Leaves: sibling leaves 2j and 2j+1 have adjacent 16-byte face records, read
// as one 32-byte load (face arrays hold one record past the last face, so the
// load stays inside the array when the sibling is virtual); an odd leaf index
// only occurs for a leaf that stays put, read on its own.
__device__ __forceinline__ void node_boxes(const TreeRef& T, uint32_t first, uint32_t level, bool two, Box& b0,
                                           Box& b1)
{
    if (level == T.L) {
        const uint32_t i = first - ((1u << level) - 1u);
        uint4 f0, f1;
        if ((i & 1u) == 0) {
            load_face_pair(T.face + i, f0, f1);
        } else {
            f0 = __ldg(T.face + i);
            f1 = two ? __ldg(T.face + i + 1) : f0;
        }
        b0 = leaf_box(T.pos, f0);
        if (two) b1 = leaf_box(T.pos, f1);
    } else {
        const float4* p = T.box + 2 * (size_t)T.shape().real_index(first);
        b0 = load_node_nc(p);
        if (two) b1 = load_node_nc(p + 2);  // same level: the next real node
    }
}

// A tree view's first 32 bytes as one 256-bit read-only load (the views are
// written by the host before the kernels that read them run).
__device__ __forceinline__ TreeRef load_tree_ref(const TreeView& T)
{
    uint32_t r[8];
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "l"(&T));
    TreeRef t;
    t.box = (float4*)(((uint64_t)r[1] << 32) | r[0]);
    t.face = (const uint4*)(((uint64_t)r[3] << 32) | r[2]);
    t.pos = (const float4*)(((uint64_t)r[5] << 32) | r[4]);
    t.L = r[6];
    t.vl = r[7];
    return t;
}

// How to expand an overlapping node pair next: both sides while their boxes
// are of similar size (squared diagonals within `ratio`), else only the
// larger box's side; a leaf never descends. The pair set does not depend on
// it. Descending only the larger of two very different boxes keeps the pairs'
// boxes matched (trees of different depths, meshes of different scales) and
// tests fewer pairs; descending both keeps the number of expansion steps of
// equal trees at one per level. The ratio is a tuning parameter (default 16).
constexpr float kDescendRatio = 16.0f;
__device__ __forceinline__ float box_size2(const Box& b)
{
    const float x = b.xx - b.nx, y = b.xy - b.ny, z = b.xz - b.nz;
    return x * x + y * y + z * z;
}
__device__ __forceinline__ uint32_t descend_side(const Box& a, bool a_leaf, const Box& b, bool b_leaf, float ratio)
{
    if (a_leaf) return kDescendB;
    if (b_leaf) return kDescendA;
    const float sa = box_size2(a), sb = box_size2(b);
    if (sa > ratio * sb) return kDescendA;
    if (sb > ratio * sa) return kDescendB;
    return kDescendBoth;
}

// aabb_box_t::overlap (include/utils/utils.h:39-44; src/cuda/collide.cu:12-17)
__device__ __forceinline__ bool overlap(const Box& a, const Box& b)
{
    return (a.nx <= b.xx && a.xx >= b.nx) && (a.ny <= b.xy && a.xy >= b.ny) && (a.nz <= b.xz && a.xz >= b.nz);
}

} // namespace oibvh
