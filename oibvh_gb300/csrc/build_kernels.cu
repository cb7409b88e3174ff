// Build-time kernels: mesh bounds, leaf boxes + Morton codes, the stable
// LSD radix sort of the codes, and the gather of Morton-ordered faces; the
// same stages for any number of trees in one launch each (scene builds);
// and the rigid transform of every tree's vertices in one launch.
//
// Reference: src/cuda/oibvh.cu:6-70 (strech_by_3, morton3D,
// calculate_aabb_and_morton_kernel) and src/cuda/oibvhTree.cu:253-299
// (mesh bounds from Mesh::m_aabb, two thrust::stable_sort_by_key calls).
// Here one stable sort of (code, face index) replaces the two payload sorts
// and the permutation is kept, so faces are gathered once into a 16-byte
// record (v0, v1, v2, original index). Keys are the reference's 30 bits, or
// 63 bits (21 per axis) as an option, sorted as two stable 32-bit passes.
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh {

// ---------------------------------------------------------------------------
// Mesh bounds (src/utils/mesh.cpp:91-98): exact min/max over every vertex,
// accumulated as order-preserving unsigned keys with atomicMin/atomicMax.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t float_to_ordered(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(uint32_t k)
{
    const uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(b);
}

__global__ void k_bounds_init(uint32_t* keys)
{
    if (threadIdx.x < 3) {
        keys[threadIdx.x] = 0xffffffffu;  // min accumulators
        keys[3 + threadIdx.x] = 0u;       // max accumulators
    }
}

// Positions as given (x, y, z) to the device layout (x, y, z, 0): one
// 16-byte vector load per vertex everywhere else.
// Positions in the tree's vertex order: tree vertex v is the caller's vertex
// vperm[v] (vperm == nullptr: the caller's order).
__global__ void __launch_bounds__(256) k_xyz_to_pos4(const float* __restrict__ xyz, const uint32_t* __restrict__ vperm,
                                                     uint32_t nV, float4* __restrict__ pos)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const size_t u = vperm ? __ldg(vperm + v) : v;
    pos[v] = make_float4(__ldg(xyz + 3 * u), __ldg(xyz + 3 * u + 1), __ldg(xyz + 3 * u + 2), 0.0f);
}
__global__ void __launch_bounds__(256) k_gather_pos4(const float4* __restrict__ src, const uint32_t* __restrict__ vperm,
                                                     uint32_t nV, float4* __restrict__ pos)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    pos[v] = __ldg(src + (vperm ? __ldg(vperm + v) : v));
}

// ---------------------------------------------------------------------------
// Vertex order: after the faces are sorted, a tree renumbers its vertices in
// the order the sorted faces first use them, so that the refit's and the
// traversal's vertex gathers for consecutive leaves fall on nearby positions
// (the caller's order is arbitrary). Unreferenced vertices go last, in their
// previous order. Results do not depend on it: faces keep their order and
// original indices, and a face's three corners keep theirs.
// ---------------------------------------------------------------------------
constexpr uint32_t kUnused = (1u << 25) - 1u;  // above every 3 f + slot (f < 2^23): 25-bit sort keys

__global__ void __launch_bounds__(256) k_first_use_init(uint32_t* __restrict__ first, uint32_t* __restrict__ idx,
                                                        uint32_t nV)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    first[v] = kUnused;
    idx[v] = v;
}
__global__ void __launch_bounds__(256) k_first_use(const uint4* __restrict__ face, uint32_t nT,
                                                   uint32_t* __restrict__ first)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nT) return;
    const uint4 r = __ldg(face + f);
    atomicMin(first + r.x, 3u * f);
    atomicMin(first + r.y, 3u * f + 1u);
    atomicMin(first + r.z, 3u * f + 2u);
}
// order[j] = the current index of new vertex j: inv[order[j]] = j, the new
// positions and the new caller-order map.
__global__ void __launch_bounds__(256) k_apply_order(const uint32_t* __restrict__ order, uint32_t nV,
                                                     uint32_t* __restrict__ inv, const float4* __restrict__ pos,
                                                     float4* __restrict__ pos_new, const uint32_t* __restrict__ vperm,
                                                     uint32_t* __restrict__ vperm_new)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nV) return;
    const uint32_t o = __ldg(order + j);
    inv[o] = j;
    pos_new[j] = __ldg(pos + o);
    vperm_new[j] = vperm ? __ldg(vperm + o) : o;
}
__global__ void __launch_bounds__(256) k_renumber_faces(uint4* __restrict__ face, uint32_t* __restrict__ tri,
                                                        uint32_t nT, const uint32_t* __restrict__ inv)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nT) return;
    uint4 r = face[f];
    r.x = __ldg(inv + r.x);
    r.y = __ldg(inv + r.y);
    r.z = __ldg(inv + r.z);
    face[f] = r;
    tri[3 * (size_t)f] = __ldg(inv + tri[3 * (size_t)f]);
    tri[3 * (size_t)f + 1] = __ldg(inv + tri[3 * (size_t)f + 1]);
    tri[3 * (size_t)f + 2] = __ldg(inv + tri[3 * (size_t)f + 2]);
}

__global__ void __launch_bounds__(256) k_mesh_bounds(const float4* __restrict__ pos, uint32_t nV, uint32_t* keys)
{
    uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
    uint32_t mx[3] = {0u, 0u, 0u};
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
        const float4 p = __ldg(pos + v);
        const float c[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t o = float_to_ordered(c[k]);
            mn[k] = min(mn[k], o);
            mx[k] = max(mx[k], o);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int s = 16; s > 0; s >>= 1) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], s));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], s));
        }
    }
    __shared__ uint32_t smn[3][8], smx[3][8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 3; ++k) {
            smn[k][w] = mn[k];
            smx[k][w] = mx[k];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        uint32_t a = 0xffffffffu, b = 0u;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            a = min(a, smn[k][i]);
            b = max(b, smx[k][i]);
        }
        atomicMin(keys + k, a);
        atomicMax(keys + 3 + k, b);
    }
}

// ---------------------------------------------------------------------------
// Leaf boxes + Morton codes (src/cuda/oibvh.cu:6-22,42-70). The float ops are
// the reference's, each rounded on its own (the *0.5f and *1024.0f scalings
// are exact, the one division is IEEE round-to-nearest).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t stretch3(uint32_t x)
{
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x30000ffu;
    x = (x | (x << 8)) & 0x300f00fu;
    x = (x | (x << 4)) & 0x30c30c3u;
    x = (x | (x << 2)) & 0x9249249u;
    return x;
}

// 21 bits -> every third bit of 63 (the wide key: 21 bits per axis)
__device__ __forceinline__ uint64_t stretch3_21(uint32_t v)
{
    uint64_t x = v & 0x1fffffu;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// The wide key's quantisation: as quant1024 with 2^21 cells per axis (the
// scaling by 2^21 is exact, the clamp bound 2^21 - 1 is a float).
__device__ __forceinline__ uint32_t quant2m(float u)
{
    float v = __fmul_rn(u, 2097152.0f);
    v = (v < 0.0f) ? 0.0f : v;
    v = (2097151.0f < v) ? 2097151.0f : v;
    return __float2uint_rz(v);  // NaN -> 0
}

// The key of a leaf from its three cell coordinates: 30 bits (the
// reference's morton3D, x << 2 | y << 1 | z) in `lo`, or 63 bits (same
// interleave, 21 bits per axis) split into `lo` (bits 0..31) and `hi`.
__device__ __forceinline__ void morton_key(const float u[3], bool wide, uint32_t& lo, uint32_t& hi);

__device__ __forceinline__ uint32_t quant1024(float u)
{
    float v = __fmul_rn(u, 1024.0f);
    v = (v < 0.0f) ? 0.0f : v;        // thrust::max(v, 0.0f)
    v = (1023.0f < v) ? 1023.0f : v;  // thrust::min(v, 1023.0f)
    return __float2uint_rz(v);        // NaN -> 0
}

__device__ __forceinline__ void morton_key(const float u[3], bool wide, uint32_t& lo, uint32_t& hi)
{
    if (!wide) {
        lo = (stretch3(quant1024(u[0])) << 2) | (stretch3(quant1024(u[1])) << 1) | stretch3(quant1024(u[2]));
        hi = 0;
        return;
    }
    const uint64_t k = (stretch3_21(quant2m(u[0])) << 2) | (stretch3_21(quant2m(u[1])) << 1) | stretch3_21(quant2m(u[2]));
    lo = (uint32_t)k;
    hi = (uint32_t)(k >> 32);
}

__global__ void __launch_bounds__(256) k_leaf_morton(const uint32_t* __restrict__ tri, const float4* __restrict__ pos,
                                                     uint32_t nT, const uint32_t* __restrict__ bound_keys,
                                                     uint32_t* __restrict__ codes, uint32_t* __restrict__ idx,
                                                     uint32_t* __restrict__ codes_hi)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nT) return;
    float bmin[3], bmax[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        bmin[k] = ordered_to_float(bound_keys[k]);
        bmax[k] = ordered_to_float(bound_keys[3 + k]);
    }
    const uint32_t f0 = __ldg(tri + 3 * (size_t)i), f1 = __ldg(tri + 3 * (size_t)i + 1),
                   f2 = __ldg(tri + 3 * (size_t)i + 2);
    const float4 p0 = __ldg(pos + f0), p1 = __ldg(pos + f1), p2 = __ldg(pos + f2);
    const float va[3] = {p0.x, p0.y, p0.z}, vb[3] = {p1.x, p1.y, p1.z}, vc[3] = {p2.x, p2.y, p2.z};
    float u[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = va[k], b = vb[k], c = vc[k];
        const float mn = gmin(gmin(a, b), c), mx = gmax(gmax(a, b), c);
        const float centroid = __fmul_rn(__fadd_rn(mn, mx), 0.5f);
        const float off = __fsub_rn(centroid, bmin[k]);
        const float len = __fsub_rn(bmax[k], bmin[k]);
        u[k] = __fdiv_rn(off, len);
    }
    uint32_t lo, hi;
    morton_key(u, codes_hi != nullptr, lo, hi);
    codes[i] = lo;
    if (codes_hi) codes_hi[i] = hi;
    idx[i] = i;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits. A tile is 2048 consecutive items
// (8 warps x 8 rounds x 32 lanes); ranks inside a tile come from
// __match_any_sync peer groups in item order, so equal digits keep their
// input order and the sort is stable, as thrust::stable_sort_by_key is.
// ---------------------------------------------------------------------------
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 8;
constexpr int kRsTile = kRsThreads * kRsRounds;

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                        uint32_t* __restrict__ hist, uint32_t n_tiles)
{
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kRsTile;
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
        const uint32_t i = base + r * kRsThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(__ldg(keys + i) >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * n_tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (256 threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total, uint32_t* sh /*[8]*/)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, s);
        if (lane >= s) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    uint32_t wpre = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < kRsThreads / 32; ++i) {
        const uint32_t t = sh[i];
        if (i < w) wpre += t;
        tot += t;
    }
    __syncthreads();
    *total = tot;
    return wpre + x - v;
}

// One CTA per digit: exclusive scan of hist[d][0..n_tiles) in place, digit total out.
__global__ void __launch_bounds__(kRsThreads) k_rs_scan_digit(uint32_t* __restrict__ hist, uint32_t n_tiles,
                                                              uint32_t* __restrict__ totals)
{
    __shared__ uint32_t sh[8];
    uint32_t* row = hist + (size_t)blockIdx.x * n_tiles;
    uint32_t carry = 0;
    for (uint32_t s = 0; s < n_tiles; s += kRsThreads) {
        const uint32_t i = s + threadIdx.x;
        const uint32_t v = (i < n_tiles) ? row[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, &tot, sh);
        if (i < n_tiles) row[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, const uint32_t* __restrict__ hist,
                                                           uint32_t n_tiles, const uint32_t* __restrict__ totals)
{
    __shared__ uint32_t warp_cnt[kRsThreads / 32][256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t sh[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (kRsThreads / 32) * 256; i += kRsThreads) (&warp_cnt[0][0])[i] = 0;
    {
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(totals[threadIdx.x], &tot, sh);
        base[threadIdx.x] = ex + hist[(size_t)threadIdx.x * n_tiles + blockIdx.x];
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t key[kRsRounds], val[kRsRounds], rank[kRsRounds];
    const uint32_t tile0 = blockIdx.x * kRsTile + w * (kRsRounds * 32);
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
        const uint32_t i = tile0 + r * 32 + lane;
        const bool valid = i < n;
        key[r] = valid ? kin[i] : 0u;
        val[r] = valid ? vin[i] : 0u;
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        rank[r] = 0;
        if (valid) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const uint32_t peers = __match_any_sync(vmask, d);
            const uint32_t b = warp_cnt[w][d];
            rank[r] = b + __popc(peers & lt);
            __syncwarp(vmask);
            if (lane == __ffs(peers) - 1) warp_cnt[w][d] = b + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    {
        const int d = threadIdx.x;
        uint32_t s = 0;
#pragma unroll
        for (int i = 0; i < kRsThreads / 32; ++i) {
            const uint32_t t = warp_cnt[i][d];
            warp_cnt[i][d] = s;
            s += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
        const uint32_t i = tile0 + r * 32 + lane;
        if (i < n) {
            const uint32_t d = (key[r] >> shift) & 255u;
            const uint32_t dst = base[d] + warp_cnt[w][d] + rank[r];
            kout[dst] = key[r];
            vout[dst] = val[r];
        }
    }
}

// Morton-ordered face records: (v0, v1, v2, original face index).
__global__ void __launch_bounds__(256) k_gather_faces(const uint32_t* __restrict__ tri, const uint32_t* __restrict__ perm,
                                                      uint32_t nT, uint4* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nT) return;
    const uint32_t o = perm[i];
    out[i] = make_uint4(__ldg(tri + 3 * (size_t)o), __ldg(tri + 3 * (size_t)o + 1), __ldg(tri + 3 * (size_t)o + 2), o);
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
size_t radix_sort_scratch_bytes(uint32_t n)
{
    const uint32_t n_tiles = (n + kRsTile - 1) / kRsTile;
    return (size_t)256 * n_tiles * sizeof(uint32_t) + 256 * sizeof(uint32_t) + 2 * (size_t)n * sizeof(uint32_t);
}

cudaError_t launch_xyz_to_pos4(const float* xyz, const uint32_t* vperm, uint32_t nV, float4* pos, cudaStream_t s)
{
    note_launches(1);
    k_xyz_to_pos4<<<(nV + 255) / 256, 256, 0, s>>>(xyz, vperm, nV, pos);
    return cudaGetLastError();
}

cudaError_t launch_gather_pos4(const float4* src, const uint32_t* vperm, uint32_t nV, float4* pos, cudaStream_t s)
{
    note_launches(1);
    k_gather_pos4<<<(nV + 255) / 256, 256, 0, s>>>(src, vperm, nV, pos);
    return cudaGetLastError();
}

size_t reorder_scratch_bytes(uint32_t nV)
{
    const size_t arr = ((size_t)nV * 4 + 255) / 256 * 256;
    return 4 * arr + ((size_t)nV * 16 + 255) / 256 * 256 + radix_sort_scratch_bytes(nV);
}

cudaError_t launch_reorder_vertices(uint4* face, uint32_t* tri, uint32_t nT, uint32_t nV, float4* pos,
                                    uint32_t* vperm, bool has_vperm, void* scratch, cudaStream_t s)
{
    const size_t arr = ((size_t)nV * 4 + 255) / 256 * 256;
    uint8_t* base = (uint8_t*)scratch;
    uint32_t* first = (uint32_t*)base;
    uint32_t* order = (uint32_t*)(base + arr);
    uint32_t* inv = (uint32_t*)(base + 2 * arr);
    uint32_t* vperm_new = (uint32_t*)(base + 3 * arr);
    float4* pos_new = (float4*)(base + 4 * arr);
    void* sort_scratch = base + 4 * arr + ((size_t)nV * 16 + 255) / 256 * 256;
    const uint32_t vb = (nV + 255) / 256, fb = (nT + 255) / 256;
    note_launches(3);
    k_first_use_init<<<vb, 256, 0, s>>>(first, order, nV);
    k_first_use<<<fb, 256, 0, s>>>(face, nT, first);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = launch_radix_sort(first, order, nV, 25, sort_scratch, s);  // stable: unused vertices keep their order
    if (e != cudaSuccess) return e;
    k_apply_order<<<vb, 256, 0, s>>>(order, nV, inv, pos, pos_new, has_vperm ? vperm : nullptr, vperm_new);
    k_renumber_faces<<<fb, 256, 0, s>>>(face, tri, nT, inv);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(pos, pos_new, (size_t)nV * sizeof(float4), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(vperm, vperm_new, (size_t)nV * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
}

cudaError_t launch_mesh_bounds(const float4* xyz, uint32_t nV, uint32_t* bound_keys, int num_sms, cudaStream_t s)
{
    note_launches(1);
    k_bounds_init<<<1, 32, 0, s>>>(bound_keys);
    uint32_t blocks = (nV + 255) / 256;
    const uint32_t cap = (uint32_t)num_sms * 8u;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    note_launches(1);
    k_mesh_bounds<<<blocks, 256, 0, s>>>(xyz, nV, bound_keys);
    return cudaGetLastError();
}

cudaError_t launch_leaf_morton(const uint32_t* tri, const float4* xyz, uint32_t nT, const uint32_t* bound_keys,
                               uint32_t* codes, uint32_t* idx, uint32_t* codes_hi, cudaStream_t s)
{
    note_launches(1);
    k_leaf_morton<<<(nT + 255) / 256, 256, 0, s>>>(tri, xyz, nT, bound_keys, codes, idx, codes_hi);
    return cudaGetLastError();
}

cudaError_t launch_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int key_bits, void* scratch,
                              cudaStream_t s)
{
    if (n <= 1) return cudaSuccess;
    const uint32_t n_tiles = (n + kRsTile - 1) / kRsTile;
    uint32_t* hist = (uint32_t*)scratch;
    uint32_t* totals = hist + (size_t)256 * n_tiles;
    uint32_t* k2 = totals + 256;
    uint32_t* v2 = k2 + n;
    uint32_t *ki = keys, *vi = vals, *ko = k2, *vo = v2;
    int passes = 0;
    for (int shift = 0; shift < key_bits; shift += 8) {
        note_launches(1);
        k_rs_hist<<<n_tiles, kRsThreads, 0, s>>>(ki, n, shift, hist, n_tiles);
        note_launches(1);
        k_rs_scan_digit<<<256, kRsThreads, 0, s>>>(hist, n_tiles, totals);
        note_launches(1);
        k_rs_scatter<<<n_tiles, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, shift, hist, n_tiles, totals);
        uint32_t* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
        ++passes;
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, ki, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, vi, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    }
    return cudaGetLastError();
}

cudaError_t launch_gather_faces(const uint32_t* tri, const uint32_t* perm, uint32_t nT, uint4* out, cudaStream_t s)
{
    note_launches(1);
    k_gather_faces<<<(nT + 255) / 256, 256, 0, s>>>(tri, perm, nT, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Multi-tree build: every stage is one launch for all trees of a scene. A CTA
// finds its tree with a binary search over the jobs' first-CTA numbers.
// Faces of all trees are numbered globally (tree t owns [face_off, +nT)); one
// stable sort by Morton code followed by one stable sort by tree id gives,
// per tree, the order of the single-tree build: (code, original index).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_job(const BuildJob* jobs, uint32_t n, uint32_t block, bool faces,
                                             const uint32_t* __restrict__ table)
{
    if (table) return __ldg(table + block);  // host-built block -> job map: one load
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        const uint32_t b = faces ? jobs[mid].fblock_begin : jobs[mid].vblock_begin;
        if (b <= block) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_bounds_init_multi(const BuildJob* __restrict__ jobs, uint32_t n_jobs)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_jobs) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        jobs[j].bound_keys[k] = 0xffffffffu;
        jobs[j].bound_keys[3 + k] = 0u;
    }
}

__global__ void __launch_bounds__(256) k_mesh_bounds_multi(const BuildJob* __restrict__ jobs, uint32_t n_jobs,
                                                           const uint32_t* __restrict__ vjob)
{
    const uint32_t j = find_job(jobs, n_jobs, blockIdx.x, false, vjob);
    const BuildJob job = jobs[j];
    const uint32_t v = (blockIdx.x - job.vblock_begin) * blockDim.x + threadIdx.x;
    uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
    uint32_t mx[3] = {0u, 0u, 0u};
    if (v < job.nV) {
        const float4 p = __ldg(job.pos + v);
        const float c[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) mn[k] = mx[k] = float_to_ordered(c[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int s = 16; s > 0; s >>= 1) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], s));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], s));
        }
    }
    if ((threadIdx.x & 31) == 0 && (v - (threadIdx.x & 31)) < job.nV) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(job.bound_keys + k, mn[k]);
            atomicMax(job.bound_keys + 3 + k, mx[k]);
        }
    }
}

__global__ void __launch_bounds__(256) k_leaf_morton_multi(const BuildJob* __restrict__ jobs, uint32_t n_jobs,
                                                           const uint32_t* __restrict__ fjob,
                                                           uint32_t* __restrict__ codes, uint32_t* __restrict__ idx,
                                                           uint32_t* __restrict__ tree_of, uint32_t* __restrict__ codes_hi)
{
    const uint32_t j = find_job(jobs, n_jobs, blockIdx.x, true, fjob);
    const BuildJob job = jobs[j];
    const uint32_t i = (blockIdx.x - job.fblock_begin) * blockDim.x + threadIdx.x;
    if (i >= job.nT) return;
    float bmin[3], bmax[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        bmin[k] = ordered_to_float(job.bound_keys[k]);
        bmax[k] = ordered_to_float(job.bound_keys[3 + k]);
    }
    const uint32_t f0 = __ldg(job.tri + 3 * (size_t)i), f1 = __ldg(job.tri + 3 * (size_t)i + 1),
                   f2 = __ldg(job.tri + 3 * (size_t)i + 2);
    const float4 p0 = __ldg(job.pos + f0), p1 = __ldg(job.pos + f1), p2 = __ldg(job.pos + f2);
    const float va[3] = {p0.x, p0.y, p0.z}, vb[3] = {p1.x, p1.y, p1.z}, vc[3] = {p2.x, p2.y, p2.z};
    float u[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float mn = gmin(gmin(va[k], vb[k]), vc[k]), mx = gmax(gmax(va[k], vb[k]), vc[k]);
        const float centroid = __fmul_rn(__fadd_rn(mn, mx), 0.5f);
        u[k] = __fdiv_rn(__fsub_rn(centroid, bmin[k]), __fsub_rn(bmax[k], bmin[k]));
    }
    const uint32_t g = job.face_off + i;
    uint32_t lo, hi;
    morton_key(u, codes_hi != nullptr, lo, hi);
    codes[g] = lo;
    if (codes_hi) codes_hi[g] = hi;
    idx[g] = g;
    tree_of[g] = j;
}

__global__ void __launch_bounds__(256) k_gather_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx,
                                                    uint32_t n, uint32_t* __restrict__ dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __ldg(src + __ldg(idx + i));
}

// Sorted position i (grouped by tree, trees in job order) -> that tree's face records.
__global__ void __launch_bounds__(256) k_gather_faces_multi(const BuildJob* __restrict__ jobs, uint32_t n_jobs,
                                                            const uint32_t* __restrict__ idx,
                                                            const uint32_t* __restrict__ tree_of, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t g = __ldg(idx + i);
    const BuildJob& job = jobs[__ldg(tree_of + g)];
    const uint32_t o = g - job.face_off;
    job.face_out[i - job.face_off] =
        make_uint4(__ldg(job.tri + 3 * (size_t)o), __ldg(job.tri + 3 * (size_t)o + 1), __ldg(job.tri + 3 * (size_t)o + 2), o);
}

// ---------------------------------------------------------------------------
// Multi-tree vertex renumbering: the order of launch_reorder_vertices (used
// vertices in the order of their first use by the sorted faces, then unused
// ones in their previous order) for every tree at once, without a sort. A
// vertex's new index is the number of first uses before its own: each
// 256-face block counts the corners that are a first use, one scan over the
// block counts gives every block its offset, and the tree's own offset is
// that of its first block (blocks never straddle trees). Unused vertices are
// ranked the same way over 256-vertex blocks, after the tree's used ones.
// Global vertex index g = vert_off + v; six launches for any number of trees.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoUse = 0xffffffffu;

struct RenumberScratch {
    uint32_t* first;     // n_verts: first-use slot (3 f + corner) of each vertex
    uint32_t* inv;       // n_verts: new index of each vertex
    float4* pos_new;     // n_verts
    uint32_t* vperm_new; // n_verts
    uint32_t* fscan;     // f_blocks + 1: first uses per face block, then their exclusive scan
    uint32_t* vscan;     // v_blocks + 1: unused vertices per vertex block, then the scan
};

__host__ __device__ inline size_t rn_align(size_t b) { return (b + 255) / 256 * 256; }

__host__ __device__ inline RenumberScratch rn_scratch(void* base, uint32_t n_verts, uint32_t v_blocks,
                                                      uint32_t f_blocks)
{
    uint8_t* p = (uint8_t*)base;
    RenumberScratch r;
    const size_t a4 = rn_align((size_t)n_verts * 4);
    r.first = (uint32_t*)p;
    r.inv = (uint32_t*)(p + a4);
    r.vperm_new = (uint32_t*)(p + 2 * a4);
    r.pos_new = (float4*)(p + 3 * a4);
    r.fscan = (uint32_t*)(p + 3 * a4 + rn_align((size_t)n_verts * 16));
    r.vscan = r.fscan + rn_align((size_t)(f_blocks + 1) * 4) / 4;
    return r;
}

__global__ void __launch_bounds__(256) k_rn_init(const BuildJob* __restrict__ jobs, const uint32_t* __restrict__ vjob,
                                                 uint32_t* __restrict__ first)
{
    const BuildJob& job = jobs[__ldg(vjob + blockIdx.x)];
    const uint32_t v = (blockIdx.x - job.vblock_begin) * 256u + threadIdx.x;
    if (v < job.nV) first[job.vert_off + v] = kNoUse;
}

__global__ void __launch_bounds__(256) k_rn_first_use(const BuildJob* __restrict__ jobs,
                                                      const uint32_t* __restrict__ fjob, uint32_t* __restrict__ first)
{
    const BuildJob& job = jobs[__ldg(fjob + blockIdx.x)];
    const uint32_t f = (blockIdx.x - job.fblock_begin) * 256u + threadIdx.x;
    if (f >= job.nT) return;
    const uint4 r = job.face_out[f];
    uint32_t* fj = first + job.vert_off;
    atomicMin(fj + r.x, 3u * f);
    atomicMin(fj + r.y, 3u * f + 1u);
    atomicMin(fj + r.z, 3u * f + 2u);
}

// This thread's count (first-use corners of its face, or 1 for an unused
// vertex) for the block kinds below: CTAs [0, f_blocks) are face blocks,
// the rest vertex blocks.
struct RnItem {
    const BuildJob* job;
    bool face_block;
    uint32_t i;      // face or vertex of the job
    uint32_t cnt;
    uint32_t mask;   // face blocks: which corners are first uses
    uint4 r;         // face blocks: the face record
};
__device__ __forceinline__ RnItem rn_item(const BuildJob* jobs, const uint32_t* vjob, const uint32_t* fjob,
                                          uint32_t f_blocks, const uint32_t* first)
{
    RnItem it{};
    it.face_block = blockIdx.x < f_blocks;
    if (it.face_block) {
        it.job = jobs + __ldg(fjob + blockIdx.x);
        it.i = (blockIdx.x - it.job->fblock_begin) * 256u + threadIdx.x;
        if (it.i < it.job->nT) {
            it.r = it.job->face_out[it.i];
            const uint32_t* fj = first + it.job->vert_off;
            it.mask = (__ldg(fj + it.r.x) == 3u * it.i ? 1u : 0u) | (__ldg(fj + it.r.y) == 3u * it.i + 1u ? 2u : 0u) |
                      (__ldg(fj + it.r.z) == 3u * it.i + 2u ? 4u : 0u);
            it.cnt = __popc(it.mask);
        }
    } else {
        const uint32_t b = blockIdx.x - f_blocks;
        it.job = jobs + __ldg(vjob + b);
        it.i = (b - it.job->vblock_begin) * 256u + threadIdx.x;
        if (it.i < it.job->nV) it.cnt = __ldg(first + it.job->vert_off + it.i) == kNoUse ? 1u : 0u;
    }
    return it;
}

__global__ void __launch_bounds__(256) k_rn_count(const BuildJob* __restrict__ jobs, const uint32_t* __restrict__ vjob,
                                                  const uint32_t* __restrict__ fjob, uint32_t f_blocks,
                                                  RenumberScratch sc)
{
    __shared__ uint32_t sh[8];
    const RnItem it = rn_item(jobs, vjob, fjob, f_blocks, sc.first);
    uint32_t tot;
    block_exclusive_scan(it.cnt, &tot, sh);
    if (threadIdx.x == 0) {
        if (it.face_block) sc.fscan[blockIdx.x] = tot;
        else sc.vscan[blockIdx.x - f_blocks] = tot;
    }
}

// CTA 0 scans fscan[0..f_blocks), CTA 1 vscan[0..v_blocks), in place
// (exclusive; the total goes to entry n), 4 entries per thread per step.
__global__ void __launch_bounds__(256) k_rn_scan(RenumberScratch sc, uint32_t f_blocks, uint32_t v_blocks)
{
    __shared__ uint32_t sh[8];
    uint32_t* a = blockIdx.x == 0 ? sc.fscan : sc.vscan;
    const uint32_t n = blockIdx.x == 0 ? f_blocks : v_blocks;
    uint32_t carry = 0;
    for (uint32_t s = 0; s < n; s += 4 * 256) {
        const uint32_t i0 = s + 4 * threadIdx.x;
        uint32_t v[4], sum = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = i0 + k < n ? a[i0 + k] : 0u;
            sum += v[k];
        }
        uint32_t tot;
        uint32_t ex = carry + block_exclusive_scan(sum, &tot, sh);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i0 + k < n) a[i0 + k] = ex;
            ex += v[k];
        }
        carry += tot;
    }
    if (threadIdx.x == 0) a[n] = carry;
}

// New index of every vertex; positions and the caller-order map in the new
// order into the scratch.
__global__ void __launch_bounds__(256) k_rn_assign(const BuildJob* __restrict__ jobs, const uint32_t* __restrict__ vjob,
                                                   const uint32_t* __restrict__ fjob, uint32_t f_blocks,
                                                   RenumberScratch sc)
{
    __shared__ uint32_t sh[8];
    const RnItem it = rn_item(jobs, vjob, fjob, f_blocks, sc.first);
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(it.cnt, &tot, sh);
    if (it.cnt == 0) return;
    const BuildJob& job = *it.job;
    const uint32_t vo = job.vert_off;
    const uint32_t f_first = job.fblock_begin, f_end = job.fblock_begin + (job.nT + 255u) / 256u;
    auto place = [&](uint32_t v, uint32_t nv) {
        sc.inv[vo + v] = nv;
        sc.pos_new[vo + nv] = __ldg(job.pos_out + v);
        sc.vperm_new[vo + nv] = job.vperm ? __ldg(job.vperm + v) : v;
    };
    if (it.face_block) {
        uint32_t rank = sc.fscan[blockIdx.x] - sc.fscan[f_first] + ex;
        if (it.mask & 1u) place(it.r.x, rank++);
        if (it.mask & 2u) place(it.r.y, rank++);
        if (it.mask & 4u) place(it.r.z, rank);
    } else {
        const uint32_t used = sc.fscan[f_end] - sc.fscan[f_first];
        const uint32_t b = blockIdx.x - f_blocks;
        place(it.i, used + sc.vscan[b] - sc.vscan[job.vblock_begin] + ex);
    }
}

// Faces and `tri` to the new numbering; positions and the map copied back
// into each tree's own buffers.
__global__ void __launch_bounds__(256) k_rn_apply(const BuildJob* __restrict__ jobs, const uint32_t* __restrict__ vjob,
                                                  const uint32_t* __restrict__ fjob, uint32_t f_blocks,
                                                  RenumberScratch sc)
{
    if (blockIdx.x < f_blocks) {
        const BuildJob& job = jobs[__ldg(fjob + blockIdx.x)];
        const uint32_t f = (blockIdx.x - job.fblock_begin) * 256u + threadIdx.x;
        if (f >= job.nT) return;
        const uint32_t* inv = sc.inv + job.vert_off;
        uint4 r = job.face_out[f];
        r.x = __ldg(inv + r.x);
        r.y = __ldg(inv + r.y);
        r.z = __ldg(inv + r.z);
        job.face_out[f] = r;
        uint32_t* t = job.tri_rw + 3 * (size_t)f;
        t[0] = __ldg(inv + t[0]);
        t[1] = __ldg(inv + t[1]);
        t[2] = __ldg(inv + t[2]);
    } else {
        const uint32_t b = blockIdx.x - f_blocks;
        const BuildJob& job = jobs[__ldg(vjob + b)];
        const uint32_t v = (b - job.vblock_begin) * 256u + threadIdx.x;
        if (v >= job.nV) return;
        job.pos_out[v] = sc.pos_new[job.vert_off + v];
        job.vperm_out[v] = sc.vperm_new[job.vert_off + v];
    }
}

size_t reorder_multi_scratch_bytes(uint32_t n_verts, uint32_t v_blocks, uint32_t f_blocks)
{
    return 3 * rn_align((size_t)n_verts * 4) + rn_align((size_t)n_verts * 16) + rn_align((size_t)(f_blocks + 1) * 4) +
           rn_align((size_t)(v_blocks + 1) * 4);
}

cudaError_t launch_reorder_vertices_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks,
                                          uint32_t f_blocks, const uint32_t* vjob, const uint32_t* fjob,
                                          uint32_t n_verts, void* scratch, cudaStream_t s)
{
    if (n_jobs == 0 || v_blocks == 0 || f_blocks == 0) return cudaSuccess;
    const RenumberScratch sc = rn_scratch(scratch, n_verts, v_blocks, f_blocks);
    note_launches(6);
    k_rn_init<<<v_blocks, 256, 0, s>>>(d_jobs, vjob, sc.first);
    k_rn_first_use<<<f_blocks, 256, 0, s>>>(d_jobs, fjob, sc.first);
    k_rn_count<<<f_blocks + v_blocks, 256, 0, s>>>(d_jobs, vjob, fjob, f_blocks, sc);
    k_rn_scan<<<2, 256, 0, s>>>(sc, f_blocks, v_blocks);
    k_rn_assign<<<f_blocks + v_blocks, 256, 0, s>>>(d_jobs, vjob, fjob, f_blocks, sc);
    k_rn_apply<<<f_blocks + v_blocks, 256, 0, s>>>(d_jobs, vjob, fjob, f_blocks, sc);
    return cudaGetLastError();
}

// Rigid transforms of every tree: pos = M * rest, M a row-major 3x4 matrix per
// tree, each product and sum rounded on its own: x' = ((m0 x + m1 y) + m2 z) + m3.
// Four 256-vertex blocks per CTA (vertex v of block k at thread v): the four
// loads are issued before any arithmetic, for more bytes in flight.
constexpr uint32_t kTransformUnroll = 4;

__global__ void __launch_bounds__(256, 8) k_transform_multi(const BuildJob* __restrict__ jobs, uint32_t n_jobs,
                                                         const uint32_t* __restrict__ vjob,
                                                         const float4* __restrict__ rest,
                                                         const float* __restrict__ mats, uint32_t v_blocks,
                                                         bool rest_tree_order)
{
    float4 p[kTransformUnroll];
    uint32_t jj[kTransformUnroll], vv[kTransformUnroll];
#pragma unroll
    for (uint32_t k = 0; k < kTransformUnroll; ++k) {
        const uint32_t vb = blockIdx.x * kTransformUnroll + k;
        jj[k] = 0xffffffffu;
        if (vb >= v_blocks) continue;
        const uint32_t j = find_job(jobs, n_jobs, vb, false, vjob);
        const uint32_t v = (vb - jobs[j].vblock_begin) * 256u + threadIdx.x;
        if (v >= jobs[j].nV) continue;
        jj[k] = j;
        vv[k] = v;
        // packed rest positions of all jobs (the caller's vertex order: through vperm), or
        // (rest == nullptr) each job's own source (the tree's order)
        const uint32_t* vp = rest_tree_order ? nullptr : jobs[j].vperm;
        p[k] = rest ? __ldg(rest + jobs[j].vert_off + (vp ? __ldg(vp + v) : v)) : __ldg(jobs[j].pos + v);
    }
#pragma unroll
    for (uint32_t k = 0; k < kTransformUnroll; ++k) {
        if (jj[k] == 0xffffffffu) continue;
        const float* m = mats + 12 * (size_t)jj[k];
        float o[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            o[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(__ldg(m + 4 * r), p[k].x), __fmul_rn(__ldg(m + 4 * r + 1), p[k].y)),
                                       __fmul_rn(__ldg(m + 4 * r + 2), p[k].z)),
                             __ldg(m + 4 * r + 3));
        jobs[jj[k]].pos_out[vv[k]] = make_float4(o[0], o[1], o[2], 0.0f);
    }
}

cudaError_t launch_build_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks, uint32_t f_blocks,
                               const uint32_t* vjob, const uint32_t* fjob, uint32_t n_faces, uint32_t tree_bits,
                               bool wide, void* scratch, cudaStream_t s)
{
    // scratch: codes, idx, tree_of, keys2, codes_hi (5 x n_faces u32), then the sort scratch
    uint32_t* codes = (uint32_t*)scratch;
    uint32_t* idx = codes + n_faces;
    uint32_t* tree_of = idx + n_faces;
    uint32_t* keys2 = tree_of + n_faces;
    uint32_t* codes_hi = keys2 + n_faces;
    void* sort_scratch = codes_hi + n_faces;
    note_launches(4);
    k_bounds_init_multi<<<(n_jobs + 255) / 256, 256, 0, s>>>(d_jobs, n_jobs);
    k_mesh_bounds_multi<<<v_blocks, 256, 0, s>>>(d_jobs, n_jobs, vjob);
    k_leaf_morton_multi<<<f_blocks, 256, 0, s>>>(d_jobs, n_jobs, fjob, codes, idx, tree_of, wide ? codes_hi : nullptr);
    // stable LSD order: low key bits, [high key bits,] then the tree id
    cudaError_t e = launch_radix_sort(codes, idx, n_faces, wide ? 32 : 30, sort_scratch, s);
    if (e != cudaSuccess) return e;
    if (wide) {
        note_launches(1);
        k_gather_u32<<<(n_faces + 255) / 256, 256, 0, s>>>(codes_hi, idx, n_faces, keys2);
        e = launch_radix_sort(keys2, idx, n_faces, 31, sort_scratch, s);
        if (e != cudaSuccess) return e;
    }
    k_gather_u32<<<(n_faces + 255) / 256, 256, 0, s>>>(tree_of, idx, n_faces, keys2);
    if (tree_bits > 0) {
        e = launch_radix_sort(keys2, idx, n_faces, (int)tree_bits, sort_scratch, s);
        if (e != cudaSuccess) return e;
    }
    note_launches(1);
    k_gather_faces_multi<<<(n_faces + 255) / 256, 256, 0, s>>>(d_jobs, n_jobs, idx, tree_of, n_faces);
    return cudaGetLastError();
}

size_t build_multi_scratch_bytes(uint32_t n_faces)
{
    return 5 * (size_t)n_faces * sizeof(uint32_t) + radix_sort_scratch_bytes(n_faces);
}

cudaError_t launch_transform_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks, const uint32_t* vjob,
                                   const float4* rest, const float* mats, bool rest_tree_order, cudaStream_t s)
{
    note_launches(1);
    k_transform_multi<<<(v_blocks + kTransformUnroll - 1) / kTransformUnroll, 256, 0, s>>>(d_jobs, n_jobs, vjob, rest,
                                                                                            mats, v_blocks,
                                                                                            rest_tree_order);
    return cudaGetLastError();
}

// Packed rest positions (caller's vertex order per tree) into each tree's
// vertex order: out[vert_off + v] = rest[vert_off + vperm[v]].
__global__ void __launch_bounds__(256) k_gather_rest_multi(const BuildJob* __restrict__ jobs, uint32_t n_jobs,
                                                           const uint32_t* __restrict__ vjob,
                                                           const float4* __restrict__ rest, float4* __restrict__ out)
{
    const uint32_t j = find_job(jobs, n_jobs, blockIdx.x, false, vjob);
    const uint32_t v = (blockIdx.x - jobs[j].vblock_begin) * 256u + threadIdx.x;
    if (v >= jobs[j].nV) return;
    const uint32_t* vp = jobs[j].vperm;
    out[jobs[j].vert_off + v] = __ldg(rest + jobs[j].vert_off + (vp ? __ldg(vp + v) : v));
}

cudaError_t launch_gather_rest_multi(const BuildJob* d_jobs, uint32_t n_jobs, uint32_t v_blocks, const uint32_t* vjob,
                                     const float4* rest, float4* out, cudaStream_t s)
{
    if (v_blocks == 0) return cudaSuccess;
    note_launches(1);
    k_gather_rest_multi<<<v_blocks, 256, 0, s>>>(d_jobs, n_jobs, vjob, rest, out);
    return cudaGetLastError();
}


cudaError_t launch_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t n, uint32_t* out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    note_launches(1);
    k_gather_u32<<<(n + 255) / 256, 256, 0, s>>>(src, idx, n, out);
    return cudaGetLastError();
}

} // namespace oibvh
