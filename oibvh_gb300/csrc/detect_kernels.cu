// Broad phase (BVTT front expansion) and narrow phase (17-axis SAT).
//
// Reference: Scene::expandBvttNodes (src/cuda/scene.cu:192-223),
// traversal_kernel (src/cuda/collide.cu:76-246) driven by the host loop of
// Scene::detectCollisionOnGPU (src/cuda/scene.cu:270-311), and
// triangle_intersect_kernel (src/cuda/collide.cu:248-299) with
// triangleIntersection2 (third/gProximity/cuda_intersect_tritri.h:350-434).
//
// The broad phase is three kernels: k_init_front tests the cross product of
// the node pairs at a start level and lists the overlapping ones; k_top (one
// CTA) walks the narrow top levels until the front is wide; in k_walk every
// warp claims 32 items of that front at a time and walks them to the leaves
// through a private FIFO ring in shared memory (its capacity a tuning
// parameter); what outgrows it spills to the next round's list, so no grid-wide
// synchronisation is needed. The host enqueues the rounds and reads the
// counters back once. Appends (next front, spills, hits) are warp-aggregated:
// one atomic per warp, positions from ballot/shuffle prefix sums.
//
// Narrow phase: overlapping leaf pairs are buffered per warp in shared memory
// and, 32 at a time, tested inside the traversal (the kernels' <true>
// instantiation, the float test) or stored for a separate kernel (<false>,
// fewer registers): k_narrow (float test, split API) or, in precision mode,
// the FP64-filtered test's passes (k_prec_classify, k_prec_settle,
// k_prec_fp64_setup, k_prec_fp64).
//
// The float triangle test reproduces the reference's CPU arithmetic
// (src/utils/utils.cpp:71-169, glm scalar dot/cross): every product, sum and
// difference is rounded on its own (__fmul_rn/__fadd_rn/__fsub_rn, never
// contracted to FMA), so the GPU pair set is the CPU pair set bit for bit.
#include "oibvh_common.cuh"
#include "oibvh_launch.h"

namespace oibvh {

constexpr int kDetectThreads = 256;

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

// ---------------------------------------------------------------------------
// Precision mode: the same 17 tests with an FP64 filter.
//
// Each axis test compares two margins, d1 = mn1 - mx2 and d2 = mn2 - mx1
// (the axis separates when either is > 0). Every float quantity of the test
// carries a running forward error bound against its exact value over the
// same float inputs (u = 2^-24; c = fl(a - b): e_c = e_a + e_b + u|c|;
// c = fl(a b): e_c = |a| e_b + |b| e_a + e_a e_b + u|c| + 2^-149), so each projection
// P has a bound e_P and each margin the bound E = max e_P + max e_Q. The
// FP64 formula obeys the same recurrences with u = 2^-53, so its margin lies
// within 2^-29 E (plus second-order terms) of the exact one. A margin with
// |d| > 2E therefore has the same sign in float, exact and FP64 arithmetic.
//
// The test runs in two passes. Pass 1 evaluates all 17 axes in float: an
// axis whose margin is > 2E separates in every arithmetic and ends the
// test; an axis with both margins < -2E separates in none; the rest are
// undecided. Pass 2 evaluates only the undecided axes again in FP64, with
// the FP64 formula's own operations in its own order (no contraction),
// until one separates. The pair set then equals the all-FP64 pair set by
// construction, while the float answer (the reference arithmetic) is known
// for every candidate, so the disagreements between the two are counted.
//
// Shortcut: two triangles that share a vertex (equal coordinates) are never
// separated by this test in any arithmetic: the shared vertex gives the same
// projection in both triangles' sets, so mn1 <= s <= mx2 and mn2 <= s <= mx1
// on every axis. Relative extents outside [2^-20, 2^20] and non-finite
// inputs take the full FP64 test (the bounds could under- or overflow).
// ---------------------------------------------------------------------------
struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 to_d(const V3& v) { return D3{(double)v.x, (double)v.y, (double)v.z}; }
__device__ __forceinline__ D3 dsub(const D3& a, const D3& b)
{
    return D3{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}
__device__ __forceinline__ D3 dcross(const D3& x, const D3& y)
{
    return D3{__dsub_rn(__dmul_rn(x.y, y.z), __dmul_rn(y.y, x.z)), __dsub_rn(__dmul_rn(x.z, y.x), __dmul_rn(y.z, x.x)),
              __dsub_rn(__dmul_rn(x.x, y.y), __dmul_rn(y.x, x.y))};
}
__device__ __forceinline__ double ddot(const D3& a, const D3& b)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
// Relative vertices of the FP64 formula: p_i = P_i - P1, q_j = Q_j - P1.
struct D6 {
    D3 p2, p3, q1, q2, q3;
};
__device__ __forceinline__ D6 fp64_relative(const V3& P1, const V3& P2, const V3& P3, const V3& Q1, const V3& Q2,
                                            const V3& Q3)
{
    const D3 dP1 = to_d(P1);
    return D6{dsub(to_d(P2), dP1), dsub(to_d(P3), dP1), dsub(to_d(Q1), dP1), dsub(to_d(Q2), dP1), dsub(to_d(Q3), dP1)};
}

// A float vector with a componentwise bound on its error.
struct EV3 {
    V3 v, e;
};
constexpr float kU = 0x1p-24f;
constexpr float kEta = 0x1p-149f;  // a product that underflows is off by up to half the smallest subnormal
// (a sum or difference whose result is subnormal is exact)
__device__ __forceinline__ float err_sub(float c, float ea, float eb) { return ea + eb + kU * fabsf(c); }
__device__ __forceinline__ float err_mul(float a, float b, float c, float ea, float eb)
{
    return fabsf(a) * eb + fabsf(b) * ea + ea * eb + kU * fabsf(c) + kEta;
}
__device__ __forceinline__ EV3 esub(const EV3& a, const EV3& b)
{
    const V3 c = vsub(a.v, b.v);
    return EV3{c, V3{err_sub(c.x, a.e.x, b.e.x), err_sub(c.y, a.e.y, b.e.y), err_sub(c.z, a.e.z, b.e.z)}};
}
// glm::cross with bounds: c = fl(fl(a b) - fl(d g)) per component
__device__ __forceinline__ float ecross1(float a, float b, float d, float g, float ea, float eb, float ed, float eg,
                                         float& err)
{
    const float m1 = __fmul_rn(a, b), m2 = __fmul_rn(d, g), c = __fsub_rn(m1, m2);
    err = err_sub(c, err_mul(a, b, m1, ea, eb), err_mul(d, g, m2, ed, eg));
    return c;
}
__device__ __forceinline__ EV3 ecross(const EV3& x, const EV3& y)
{
    EV3 r;
    r.v.x = ecross1(x.v.y, y.v.z, y.v.y, x.v.z, x.e.y, y.e.z, y.e.y, x.e.z, r.e.x);
    r.v.y = ecross1(x.v.z, y.v.x, y.v.z, x.v.x, x.e.z, y.e.x, y.e.z, x.e.x, r.e.y);
    r.v.z = ecross1(x.v.x, y.v.y, y.v.x, x.v.y, x.e.x, y.e.y, y.e.x, x.e.y, r.e.z);
    return r;
}
// glm::dot with a bound: fl(fl(fl(ax px) + fl(ay py)) + fl(az pz))
__device__ __forceinline__ float edot(const EV3& a, const EV3& p, float& err)
{
    const float t0 = __fmul_rn(a.v.x, p.v.x), t1 = __fmul_rn(a.v.y, p.v.y), t2 = __fmul_rn(a.v.z, p.v.z);
    const float s = __fadd_rn(t0, t1), r = __fadd_rn(s, t2);
    const float e0 = err_mul(a.v.x, p.v.x, t0, a.e.x, p.e.x);
    const float e1 = err_mul(a.v.y, p.v.y, t1, a.e.y, p.e.y);
    const float e2 = err_mul(a.v.z, p.v.z, t2, a.e.z, p.e.z);
    err = err_sub(r, err_sub(s, e0, e1), e2);
    return r;
}
// One float axis test with bounds: 0 = separates in every arithmetic,
// 1 = separates in none, 2 = undecided; `sep32` is the plain float answer.
__device__ __forceinline__ uint32_t project6_bounded(const EV3& ax, const EV3& p1, const EV3& p2, const EV3& p3,
                                                     const EV3& q1, const EV3& q2, const EV3& q3, bool& sep32)
{
    float eP1, eP2, eP3, eQ1, eQ2, eQ3;
    const float P1 = edot(ax, p1, eP1), P2 = edot(ax, p2, eP2), P3 = edot(ax, p3, eP3);
    const float Q1 = edot(ax, q1, eQ1), Q2 = edot(ax, q2, eQ2), Q3 = edot(ax, q3, eQ3);
    const float mx1 = fmaxf(fmaxf(P1, P2), P3), mn1 = fminf(fminf(P1, P2), P3);
    const float mx2 = fmaxf(fmaxf(Q1, Q2), Q3), mn2 = fminf(fminf(Q1, Q2), Q3);
    sep32 = mn1 > mx2 || mn2 > mx1;
    // 2 E: covers the FP64 error (2^-29 E), second-order terms and the
    // rounding of the margins and of the bound itself
    const float tau = 2.0f * (fmaxf(fmaxf(eP1, eP2), eP3) + fmaxf(fmaxf(eQ1, eQ2), eQ3));
    const float d1 = __fsub_rn(mn1, mx2), d2 = __fsub_rn(mn2, mx1);
    if (d1 > tau || d2 > tau) return 0u;
    if (d1 < -tau && d2 < -tau) return 1u;
    return 2u;
}

__device__ __forceinline__ bool veq(const V3& a, const V3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

enum : uint32_t { kPass1Separated = 0, kPass1Hit = 1, kPass1Undecided = 2 };

// Pass 1 of the filtered test: every axis in float with error bounds.
// Returns kPass1Separated / kPass1Hit when the float and FP64 answers are
// known to agree, else kPass1Undecided with the axes to settle in FP64 in
// `mask` and the plain float answer in `hit32`.
__device__ __forceinline__ uint32_t tri_pass1(const V3& P1, const V3& P2, const V3& P3, const V3& Q1, const V3& Q2,
                                              const V3& Q3, uint32_t& mask, bool& hit32)
{
    const EV3 p1{V3{0.0f, 0.0f, 0.0f}, V3{0.0f, 0.0f, 0.0f}};
    const V3 p2v = vsub(P2, P1), p3v = vsub(P3, P1);
    const V3 q1v = vsub(Q1, P1), q2v = vsub(Q2, P1), q3v = vsub(Q3, P1);
    float A = fmaxf(fmaxf(fmaxf(fabsf(p2v.x), fabsf(p2v.y)), fmaxf(fabsf(p2v.z), fabsf(p3v.x))),
                    fmaxf(fmaxf(fabsf(p3v.y), fabsf(p3v.z)), fmaxf(fabsf(q1v.x), fabsf(q1v.y))));
    A = fmaxf(A, fmaxf(fmaxf(fabsf(q1v.z), fabsf(q2v.x)), fmaxf(fabsf(q2v.y), fabsf(q2v.z))));
    A = fmaxf(A, fmaxf(fmaxf(fabsf(q3v.x), fabsf(q3v.y)), fabsf(q3v.z)));
    if (!(A >= 0x1p-20f && A <= 0x1p20f)) {
        // the bounds could under- or overflow: every axis in FP64
        hit32 = tri_intersect_exact(P1, P2, P3, Q1, Q2, Q3);
        mask = (1u << 17) - 1u;
        return kPass1Undecided;
    }
    if (veq(P1, Q1) || veq(P1, Q2) || veq(P1, Q3) || veq(P2, Q1) || veq(P2, Q2) || veq(P2, Q3) || veq(P3, Q1) ||
        veq(P3, Q2) || veq(P3, Q3))
        return kPass1Hit;  // a shared vertex: never separated
    // relative vertices: one rounding each
    const EV3 p2{p2v, V3{kU * fabsf(p2v.x), kU * fabsf(p2v.y), kU * fabsf(p2v.z)}};
    const EV3 p3{p3v, V3{kU * fabsf(p3v.x), kU * fabsf(p3v.y), kU * fabsf(p3v.z)}};
    const EV3 q1{q1v, V3{kU * fabsf(q1v.x), kU * fabsf(q1v.y), kU * fabsf(q1v.z)}};
    const EV3 q2{q2v, V3{kU * fabsf(q2v.x), kU * fabsf(q2v.y), kU * fabsf(q2v.z)}};
    const EV3 q3{q3v, V3{kU * fabsf(q3v.x), kU * fabsf(q3v.y), kU * fabsf(q3v.z)}};
    const EV3 e1 = esub(p2, p1), e2 = esub(p3, p2), e3 = esub(p1, p3);
    const EV3 f1 = esub(q2, q1), f2 = esub(q3, q2), f3 = esub(q1, q3);
    const EV3 n1 = ecross(e1, e2), m1 = ecross(f1, f2);
    bool sep32 = false;
    uint32_t undecided = 0;
#define OIBVH_AXIS(K, AX)                                                        \
    {                                                                            \
        bool s32;                                                                \
        const uint32_t c = project6_bounded((AX), p1, p2, p3, q1, q2, q3, s32);  \
        if (c == 0u) return kPass1Separated;                                     \
        sep32 |= s32;                                                            \
        if (c == 2u) undecided |= 1u << (K);                                     \
    }
    OIBVH_AXIS(0, n1)
    OIBVH_AXIS(1, m1)
    OIBVH_AXIS(2, ecross(e1, f1))
    OIBVH_AXIS(3, ecross(e1, f2))
    OIBVH_AXIS(4, ecross(e1, f3))
    OIBVH_AXIS(5, ecross(e2, f1))
    OIBVH_AXIS(6, ecross(e2, f2))
    OIBVH_AXIS(7, ecross(e2, f3))
    OIBVH_AXIS(8, ecross(e3, f1))
    OIBVH_AXIS(9, ecross(e3, f2))
    OIBVH_AXIS(10, ecross(e3, f3))
    OIBVH_AXIS(11, ecross(e1, n1))
    OIBVH_AXIS(12, ecross(e2, n1))
    OIBVH_AXIS(13, ecross(e3, n1))
    OIBVH_AXIS(14, ecross(f1, m1))
    OIBVH_AXIS(15, ecross(f2, m1))
    OIBVH_AXIS(16, ecross(f3, m1))
#undef OIBVH_AXIS
    if (undecided == 0) return kPass1Hit;  // no axis separates, in any arithmetic
    mask = undecided;
    hit32 = !sep32;
    return kPass1Undecided;
}

__device__ __forceinline__ V3 load_vertex(const float4* __restrict__ pos, uint32_t v)
{
    const float4 p = __ldg(pos + v);
    return V3{p.x, p.y, p.z};
}

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

// Children of implicit node `ia` (level la) `e` levels down, clamped at the
// leaf level: the first child and the count of real ones
// (src/cuda/collide.cu:165-176). A leaf is its own only child.
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

// ---------------------------------------------------------------------------
// Per-warp candidate buffer: leaf pairs whose boxes overlap are queued in
// shared memory and tested 32 at a time, one per lane, so the 17-axis test
// runs at full SIMT width however sparse the candidates are.
// ---------------------------------------------------------------------------
constexpr int kCandBuf = 160;  // <= 31 left over + up to 4 per lane added by one expansion step
constexpr uint32_t kTopThreads = 1024;  // the single CTA of the top levels
constexpr uint32_t kTopCap = 8192;      // its front capacity (two buffers: 128 KB)
constexpr uint32_t kHandoff = 2048;     // front width at which the walkers take over
constexpr uint32_t kWalkCap = 128;      // default per-warp ring capacity of the walkers (node pairs)
constexpr uint32_t kWalkCapMax = 512;
// Ring entries per warp for a requested capacity (0: the default): at least
// 64, so that a top-up of 32 list items always fits beside up to 31 queued.
__host__ __device__ __forceinline__ uint32_t walk_ring(uint32_t cap)
{
    cap = cap ? cap : kWalkCap;
    return cap < 64u ? 64u : cap;
}

struct WarpCands {
    uint64_t* buf;       // kCandBuf entries
    uint32_t n;          // warp-uniform
    uint32_t found = 0;  // candidates found by this warp (added to the counter once, at the end)
};

__device__ __forceinline__ void flush_found(const DetectArgs& a, const WarpCands& wc, uint32_t lane)
{
    if (lane == 0 && wc.found) atomicAdd(a.counts + kCountCands, wc.found);
}

__device__ __forceinline__ void test_candidates(const DetectArgs& a, const uint64_t* buf, uint32_t count,
                                                uint32_t lane)
{
    bool hit = false;
    uint4 rec = make_uint4(0, 0, 0, 0);
    if (lane < count) {
        const uint64_t c = buf[lane];
        const PairView& pv = a.pairs[bvtt_pair(c)];
        const TreeRef TA = load_tree_ref(pv.ta);
        const TreeRef TB = load_tree_ref(pv.tb);
        const uint4 fa = __ldg(TA.face + bvtt_a(c));
        const uint4 fb = __ldg(TB.face + bvtt_b(c));
        hit = tri_intersect_exact(load_vertex(TA.pos, fa.x), load_vertex(TA.pos, fa.y), load_vertex(TA.pos, fa.z),
                                  load_vertex(TB.pos, fb.x), load_vertex(TB.pos, fb.y), load_vertex(TB.pos, fb.z));
        rec = make_uint4(pv.a, pv.b, fa.w, fb.w);
    }
    const uint32_t pos = warp_append(a.counts + kCountHits, hit, lane);
    if (hit) {
        if (pos < a.hit_cap) a.hits[pos] = rec;
        else atomicOr(a.counts + kCountFlags, (uint32_t)kFlagHitOverflow);
    }
}

// Queue (or, in broad-only mode, store) one candidate per lane where `pred`.
// Broad phase only: `count` buffered candidates (one per lane) to the global
// candidate queue with one atomic for the warp.
__device__ __forceinline__ void store_candidates(const DetectArgs& a, const uint64_t* buf, uint32_t count,
                                                 uint32_t lane)
{
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(a.counts + kCountCandSlots, count);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (lane < count) {
        if (base + lane < a.cand_cap) a.cand[base + lane] = buf[lane];
        else atomicOr(a.counts + kCountFlags, (uint32_t)kFlagCandOverflow);
    }
}

// The warp's buffered candidates: tested (fused narrow phase) or stored.
// kFused: the narrow phase is compiled into the traversal kernel (tested
// here); otherwise the candidates are stored, and the kernel carries no
// triangle-test code (fewer registers, more warps per SM).
template <bool kFused>
__device__ __forceinline__ void flush_candidates(const DetectArgs& a, const uint64_t* buf, uint32_t count,
                                                 uint32_t lane)
{
    if constexpr (kFused) test_candidates(a, buf, count, lane);
    else store_candidates(a, buf, count, lane);
}

// Queue one candidate per lane where `pred` in the warp's buffer (at most 4
// per lane between two drains).
template <bool kFused>
__device__ __forceinline__ void push_candidate(const DetectArgs& a, WarpCands& wc, bool pred, uint64_t cval,
                                               uint32_t lane)
{
    const uint32_t mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return;
    wc.found += __popc(mask);
    if (pred) wc.buf[wc.n + __popc(mask & ((1u << lane) - 1u))] = cval;
    wc.n += __popc(mask);
    __syncwarp();
}

// Every 32 queued candidates are tested (fused narrow phase) or stored (broad
// phase only) at once; called once per step, where little else is live.
template <bool kFused>
__device__ __forceinline__ void drain_candidates(const DetectArgs& a, WarpCands& wc, uint32_t lane)
{
    while (wc.n >= 32) {
        flush_candidates<kFused>(a, wc.buf + wc.n - 32, 32, lane);
        wc.n -= 32;
        __syncwarp();
    }
}

// One BVTT pair per lane, one level down on the sides its key names (both,
// or the larger box's; a leaf never descends): the up to 2 + 2 boxes (a side
// that stays contributes its own node) are loaded first (independent loads),
// the up to 4 child pairs are tested and overlapping leaf pairs become
// candidates. Returns the overlapping internal child pairs (bit 2x + y: child
// pair (fa + x, fb + y)) with how each of them expands next (bits 2k, 2k + 1
// of dm); `tested` gets the warp's number of child pairs tested (lane 0 only).
struct Expansion {
    uint32_t pair, fa, fb, m, dm;
};
template <bool kFused>
__device__ __forceinline__ Expansion expand_test(const DetectArgs& a, WarpCands& wc, bool valid, uint64_t node,
                                                 uint32_t lane, uint32_t& tested)
{
    uint32_t pair = 0, fa = 0, fb = 0, na = 0, nb = 0, leaf_a = 0, leaf_b = 0;
    bool leaves = false, a_leaf = false, b_leaf = false;
    Box A0{}, A1{}, B0{}, B1{};
    if (valid) {
        pair = bvtt_pair(node);
        const uint32_t ia = bvtt_a(node), ib = bvtt_b(node);
        const PairView& pv = a.pairs[pair];
        const TreeRef TA = load_tree_ref(pv.ta);
        const TreeRef TB = load_tree_ref(pv.tb);
        const uint32_t la = ilog2(ia + 1u), lb = ilog2(ib + 1u);
        // the sides to descend: the key's, never a leaf (a leaf side stays and
        // the other one descends), so every expansion goes one level down
        const uint32_t d = bvtt_desc(node);
        const bool down_a = la != TA.L && (d != kDescendB || lb == TB.L);
        const bool down_b = lb != TB.L && (d != kDescendA || la == TA.L);
        if (down_a) expand_side(TA.shape(), ia, la, 1, fa, na);
        else fa = ia, na = 1;
        if (down_b) expand_side(TB.shape(), ib, lb, 1, fb, nb);
        else fb = ib, nb = 1;
        const uint32_t lca = ilog2(fa + 1u), lcb = ilog2(fb + 1u);
        a_leaf = lca == TA.L;
        b_leaf = lcb == TB.L;
        leaves = a_leaf && b_leaf;
        leaf_a = fa - ((1u << lca) - 1u);  // Morton-order leaf index when lca is the leaf level
        leaf_b = fb - ((1u << lcb) - 1u);
        node_boxes(TA, fa, lca, na > 1, A0, A1);
        node_boxes(TB, fb, lcb, nb > 1, B0, B1);
    }
    // bit (2x + y): child pair (fa + x, fb + y) overlaps
    uint32_t m = 0, dm = 0;
    if (valid) {
        m |= overlap(A0, B0) ? 1u : 0u;
        if (nb > 1) m |= overlap(A0, B1) ? 2u : 0u;
        if (na > 1) m |= overlap(A1, B0) ? 4u : 0u;
        if (na > 1 && nb > 1) m |= overlap(A1, B1) ? 8u : 0u;
        if (!leaves) {
            const float r = a.descend_ratio;
            dm |= descend_side(A0, a_leaf, B0, b_leaf, r);
            if (nb > 1) dm |= descend_side(A0, a_leaf, B1, b_leaf, r) << 2;
            if (na > 1) dm |= descend_side(A1, a_leaf, B0, b_leaf, r) << 4;
            if (na > 1 && nb > 1) dm |= descend_side(A1, a_leaf, B1, b_leaf, r) << 6;
        }
    }
    const uint32_t t = __reduce_add_sync(0xffffffffu, na * nb);
    tested = lane == 0 ? t : 0u;
    // candidates, one bit per round (at most 4 rounds); every lane joins each round
    uint32_t cm = leaves ? m : 0u;
    while (__any_sync(0xffffffffu, cm != 0)) {
        const bool pred = cm != 0;
        uint64_t c = 0;
        if (pred) {
            const uint32_t k = __ffs(cm) - 1;
            cm &= cm - 1;
            c = bvtt_pack(pair, leaf_a + (k >> 1), leaf_b + (k & 1));
        }
        push_candidate<kFused>(a, wc, pred, c, lane);
    }
    return Expansion{pair, fa, fb, leaves ? 0u : m, dm};
}

// The key of child pair k (bit 2x + y) of an expansion.
__device__ __forceinline__ uint64_t child_key(const Expansion& e, uint32_t k)
{
    return bvtt_pack(e.pair, e.fa + (k >> 1), e.fb + (k & 1), (e.dm >> (2 * k)) & 3u);
}

// Exclusive prefix over the warp of each lane's child count; `total` = the
// warp's sum.
__device__ __forceinline__ uint32_t child_prefix(uint32_t cnt, uint32_t lane, uint32_t& total)
{
    uint32_t incl = cnt;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, s);
        if ((int)lane >= s) incl += y;
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - cnt;
}

// Children of position `pos` onward go to `slot(pos)` while pos < fit, the
// rest to the spill list from sbase.
template <typename Slot>
__device__ __forceinline__ void write_children(const DetectArgs& a, const Expansion& e, uint32_t pos, uint32_t fit,
                                               uint64_t* __restrict__ spill, uint32_t sbase, Slot slot)
{
    bool overflow = false;
    uint32_t mm = e.m;
    while (mm) {
        const uint32_t k = __ffs(mm) - 1;
        mm &= mm - 1;
        const uint64_t child = child_key(e, k);
        if (pos < fit) *slot(pos) = child;
        else {
            const uint32_t sp = sbase + (pos - fit);
            if (sp < a.work_cap) spill[sp] = child;
            else overflow = true;
        }
        ++pos;
    }
    if (overflow) atomicOr(a.counts + kCountFlags, (uint32_t)kFlagFrontOverflow);
}

// expand_test, then the overlapping internal pairs go to the CTA's next
// front in shared memory (one shared atomic per warp); what does not fit
// goes to the spill list of the next round. Returns the number of child
// pairs tested (lane 0 only, else 0).
template <bool kFused>
__device__ __forceinline__ uint32_t expand_pair(const DetectArgs& a, WarpCands& wc, bool valid, uint64_t node,
                                                uint64_t* next, uint32_t* next_cnt, uint32_t next_cap,
                                                uint64_t* __restrict__ spill, uint32_t* spill_cnt, uint32_t lane)
{
    uint32_t tested;
    const Expansion e = expand_test<kFused>(a, wc, valid, node, lane, tested);
    uint32_t total;
    const uint32_t ex = child_prefix((uint32_t)__popc(e.m), lane, total);
    if (total == 0) return tested;
    uint32_t wbase = 0, sbase = 0;
    if (lane == 31) {
        wbase = atomicAdd(next_cnt, total);
        const uint32_t fit = wbase >= next_cap ? 0u : min(total, next_cap - wbase);
        if (total > fit) sbase = atomicAdd(spill_cnt, total - fit);
    }
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    sbase = __shfl_sync(0xffffffffu, sbase, 31);
    // warp-relative positions: [0, fit) in the front from wbase, the rest spill
    const uint32_t fit = wbase >= next_cap ? 0u : min(total, next_cap - wbase);
    write_children(a, e, ex, fit, spill, sbase, [&](uint32_t p) { return next + wbase + p; });
    return tested;
}

// Initial work list: every start-level node pair of every mesh pair (the
// reference's Scene::expandBvttNodes cross product, src/cuda/scene.cu:192-223)
// is tested here; overlapping internal pairs go to work list 0, overlapping
// leaf pairs straight to the candidates.
template <bool kFused>
__global__ void __launch_bounds__(kDetectThreads) k_init_front(DetectArgs a, uint32_t total0)
{
    __shared__ uint64_t s_cand[kDetectThreads / 32][kCandBuf];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    WarpCands wc{s_cand[wib], 0};
    for (uint32_t base = warp * 32; base < total0; base += n_warps * 32) {
        const uint32_t i = base + lane;
        bool ov = false, leafpair = false;
        uint64_t node = 0, cval = 0;
        if (i < total0) {
            uint32_t lo = 0, hi = a.n_pairs - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (a.pairs[mid].front_off <= i) lo = mid;
                else hi = mid - 1;
            }
            const PairView& pv = a.pairs[lo];
            const uint32_t k = i - pv.front_off;
            const uint32_t x = k / pv.front_cnt_b, y = k - x * pv.front_cnt_b;
            const uint32_t ia = (1u << pv.entry_a) - 1u + x, ib = (1u << pv.entry_b) - 1u + y;
            const TreeRef TA = load_tree_ref(pv.ta);
            const TreeRef TB = load_tree_ref(pv.tb);
            const Box ba = node_box(TA, ia, pv.entry_a), bb = node_box(TB, ib, pv.entry_b);
            ov = overlap(ba, bb);
            leafpair = ov && pv.entry_a == TA.L && pv.entry_b == TB.L;
            node = bvtt_pack(lo, ia, ib, descend_side(ba, pv.entry_a == TA.L, bb, pv.entry_b == TB.L, a.descend_ratio));
            cval = bvtt_pack(lo, x, y);
        }
        push_candidate<kFused>(a, wc, leafpair, cval, lane);
        drain_candidates<kFused>(a, wc, lane);
        const bool push = ov && !leafpair;
        const uint32_t pos = warp_append(a.counts + kCountWork0, push, lane);
        if (push) {
            if (pos < a.work_cap) a.work[0][pos] = node;
            else atomicOr(a.counts + kCountFlags, (uint32_t)kFlagFrontOverflow);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.counts + kCountTested, total0);
    flush_found(a, wc, lane);
    if (wc.n > 0) flush_candidates<kFused>(a, wc.buf, wc.n, lane);
}

// The narrow top of the traversal: ONE CTA of kTopThreads walks the start
// list level by level with its front in shared memory (__syncthreads between
// levels) until the front holds more than kHandoff pairs; that front becomes
// the next work list. The first levels hold a few hundred pairs at most, so
// one CTA covers them with one round of loads per level and no grid-wide
// synchronisation.
template <bool kFused>
__global__ void __launch_bounds__(kTopThreads) k_top(DetectArgs a)
{
    extern __shared__ uint64_t s_dyn[];  // two front buffers of kTopCap
    __shared__ uint64_t s_cand[kTopThreads / 32][kCandBuf];
    __shared__ uint32_t s_cnt[2];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    constexpr uint32_t kWarps = kTopThreads / 32;
    WarpCands wc{s_cand[wib], 0};
    uint64_t* out = a.work[1];
    uint32_t* out_cnt = a.counts + kCountWork0 + 1;
    const uint32_t n0 = min(a.counts[kCountWork0], a.work_cap);
    uint32_t tested = 0;
    // the start list fits the front buffer, or goes straight to the walkers
    const uint32_t handoff = a.handoff ? min(a.handoff, kTopCap) : kHandoff;
    if (n0 > handoff) {
        for (uint32_t i = threadIdx.x; i < n0; i += kTopThreads) out[i] = __ldcg(a.work[0] + i);
        if (threadIdx.x == 0) *out_cnt = n0;
        return;
    }
    for (uint32_t i = threadIdx.x; i < n0; i += kTopThreads) s_dyn[i] = __ldcg(a.work[0] + i);
    uint32_t cur = 0, c = n0;
    __syncthreads();
    while (c > 0) {
        uint64_t* fc = cur ? s_dyn + kTopCap : s_dyn;
        uint64_t* fn = cur ? s_dyn : s_dyn + kTopCap;
        if (c > handoff) {
            // wide enough: hand the front to the walkers, after the children the
            // last level spilled to the list (a handoff above kTopCap / 4 lets a
            // level outgrow the buffer); the count is stable: every spill
            // happened before the last __syncthreads
            const uint32_t base = *(volatile uint32_t*)out_cnt;
            const uint32_t room = base < a.work_cap ? min(c, a.work_cap - base) : 0u;
            for (uint32_t i = threadIdx.x; i < room; i += kTopThreads) out[base + i] = fc[i];
            __syncthreads();  // every thread has read the count before it moves
            if (threadIdx.x == 0) {
                *out_cnt = base + c;
                if (room < c) atomicOr(a.counts + kCountFlags, (uint32_t)kFlagFrontOverflow);
            }
            break;
        }
        if (threadIdx.x == 0) s_cnt[cur ^ 1] = 0;
        __syncthreads();
        for (uint32_t base = wib * 32; base < c; base += kWarps * 32) {
            const uint32_t i = base + lane;
            const bool valid = i < c;
            const uint64_t node = valid ? fc[i] : 0ull;
            // what outgrows the buffer goes to the walkers' list directly
            tested += expand_pair<kFused>(a, wc, valid, node, fn, &s_cnt[cur ^ 1], kTopCap, out, out_cnt, lane);
            drain_candidates<kFused>(a, wc, lane);
        }
        __syncthreads();
        c = min(s_cnt[cur ^ 1], kTopCap);
        cur ^= 1;
    }
    if (lane == 0 && tested) atomicAdd(a.counts + kCountTested, tested);
    flush_found(a, wc, lane);
    if (wc.n > 0) flush_candidates<kFused>(a, wc.buf, wc.n, lane);
}

// The wide bottom of the traversal, round `round` (>= 1): every warp claims
// up to 32 consecutive work-list items at a time (one atomic on the round's
// claim counter; a list with fewer than claim_min items per warp, a tuning
// parameter, is dealt out statically instead, one interleaved share per
// warp) and walks them to the leaves through a private FIFO ring of node
// pairs in shared memory: each step pops up to 32 pairs (one per lane),
// expands them and appends the overlapping children at the tail, with no
// barrier between tree levels, so lanes stay busy as long as a warp's worth
// of pairs is queued (a level-by-level front leaves the last chunk of every
// level part empty). The ring is topped up with the next claim whenever it
// holds fewer than 32 pairs, so warps whose items expand less take more of
// the list. Warps never wait for each other; children that do not fit in the
// ring spill to the next round's list (consecutively per warp, so a claim of
// consecutive items keeps one subtree's spill together).
// kDense: compiled for 4 CTAs per SM (64 registers; the fused form spills a
// few bytes), used when the grid asks for 4; otherwise the register budget of
// 3 CTAs per SM (no spills).
template <bool kFused, bool kDense>
__global__ void __launch_bounds__(kDetectThreads, kDense ? 4 : 3) k_walk(DetectArgs a, uint32_t round)
{
    extern __shared__ uint64_t s_front[];  // [warp][walk_ring(cap)]: one ring per warp
    __shared__ uint64_t s_cand[kDetectThreads / 32][kCandBuf];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WarpCands wc{s_cand[wib], 0};
    const uint64_t* __restrict__ src = (round & 1) ? a.work[1] : a.work[0];
    uint64_t* __restrict__ spill = (round & 1) ? a.work[0] : a.work[1];
    uint32_t* spill_cnt = a.counts + kCountWork0 + round + 1;
    const uint32_t n_src = min(*(volatile uint32_t*)(a.counts + kCountWork0 + round), a.work_cap);
    uint32_t* claim = a.counts + kCountClaim0 + round;
    const uint32_t R = walk_ring(a.walk_cap);  // ring entries (>= 64)
    uint64_t* ring = s_front + (size_t)wib * R;
    // A list of at least claim_min items per warp is claimed `chunk`
    // consecutive items at a time (its items per warp, 1..32); a shorter one
    // is dealt out statically, items w, w + W, w + 2W, ... to warp w (W warps),
    // so that every warp gets work.
    const uint32_t W = (gridDim.x * blockDim.x) >> 5;
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const bool claiming = n_src >= max(1u, a.claim_min) * W;
    const uint32_t chunk = min(32u, max(1u, n_src / W));
    const uint32_t n_mine = claiming ? 0u : (n_src > w ? (n_src - w + W - 1) / W : 0u);
    uint32_t next_item = 0;
    bool drained = !claiming;     // warp-uniform: no unclaimed item left (claiming lists)
    uint32_t head = 0, live = 0;  // warp-uniform: ring[head .. head + live) mod R is queued
    uint32_t tested = 0;
    auto slot = [&](uint32_t off) {  // ring index of the entry `off` after head (off < R)
        const uint32_t i = head + off;
        return i >= R ? i - R : i;
    };
    for (;;) {
        if (live < 32 && !drained) {
            // the next `chunk` items of the list, claimed with one atomic per
            // warp: warps whose items expand less come back sooner and take
            // more, and neighbouring items (often one subtree's spill) stay together
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(claim, chunk);
            base = __shfl_sync(0xffffffffu, base, 0);
            const uint32_t take = base < n_src ? min(chunk, n_src - base) : 0u;  // live + take <= 63 < R
            drained = base + chunk >= n_src;
            if (lane < take) ring[slot(live + lane)] = __ldcg(src + base + lane);
            live += take;
            __syncwarp();
        } else if (live < 32 && next_item < n_mine) {
            const uint32_t take = min(32u, n_mine - next_item);  // live + take <= 63 < R
            if (lane < take) ring[slot(live + lane)] = __ldcg(src + w + (size_t)(next_item + lane) * W);
            next_item += take;
            live += take;
            __syncwarp();
        }
        if (live == 0) break;
        const uint32_t n = min(32u, live);
        const bool valid = lane < n;
        const uint64_t node = valid ? ring[slot(lane)] : 0ull;
        __syncwarp();  // every lane has read its entry before the slots are reused
        head = slot(n);
        live -= n;
        uint32_t t;
        const Expansion e = expand_test<kFused>(a, wc, valid, node, lane, t);
        tested += t;
        uint32_t total;
        const uint32_t ex = child_prefix((uint32_t)__popc(e.m), lane, total);
        if (total > 0) {
            const uint32_t fit = min(total, R - live);
            uint32_t sbase = 0;
            if (total > fit) {
                if (lane == 31) sbase = atomicAdd(spill_cnt, total - fit);
                sbase = __shfl_sync(0xffffffffu, sbase, 31);
            }
            write_children(a, e, ex, fit, spill, sbase, [&](uint32_t p) { return ring + slot(live + p); });
            live += fit;
            __syncwarp();  // appended entries are visible to the lanes that pop them
        }
        // the step's candidates are tested (or stored) after its children are
        // queued, where little else is live
        drain_candidates<kFused>(a, wc, lane);
    }
    if (lane == 0 && tested) atomicAdd(a.counts + kCountTested, tested);
    flush_found(a, wc, lane);
    if (wc.n > 0) flush_candidates<kFused>(a, wc.buf, wc.n, lane);
}

// Narrow phase over stored candidates (the split broad/narrow API):
// triangle_intersect_kernel (src/cuda/collide.cu:248-299).
__global__ void __launch_bounds__(kDetectThreads) k_narrow(DetectArgs a)
{
    const uint32_t n = min(a.counts[kCountCandSlots], a.cand_cap);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t base = warp * 32; base < n; base += n_warps * 32) {
        const uint32_t cnt = min(32u, n - base);
        test_candidates(a, a.cand + base, cnt, lane);
    }
}

// Precision mode's narrow phase over stored candidates: one candidate's
// triangles, and a hit appended with one atomic per warp.
__device__ __forceinline__ void load_tris(const DetectArgs& a, uint64_t c, V3& P1, V3& P2, V3& P3, V3& Q1, V3& Q2,
                                          V3& Q3, uint4& rec)
{
    const PairView& pv = a.pairs[bvtt_pair(c)];
    const TreeRef TA = load_tree_ref(pv.ta);
    const TreeRef TB = load_tree_ref(pv.tb);
    const uint4 fa = __ldg(TA.face + bvtt_a(c));
    const uint4 fb = __ldg(TB.face + bvtt_b(c));
    P1 = load_vertex(TA.pos, fa.x);
    P2 = load_vertex(TA.pos, fa.y);
    P3 = load_vertex(TA.pos, fa.z);
    Q1 = load_vertex(TB.pos, fb.x);
    Q2 = load_vertex(TB.pos, fb.y);
    Q3 = load_vertex(TB.pos, fb.z);
    rec = make_uint4(pv.a, pv.b, fa.w, fb.w);
}

__device__ __forceinline__ void append_hit(const DetectArgs& a, bool hit, const uint4& rec, uint32_t lane)
{
    const uint32_t pos = warp_append(a.counts + kCountHits, hit, lane);
    if (hit) {
        if (pos < a.hit_cap) a.hits[pos] = rec;
        else atomicOr(a.counts + kCountFlags, (uint32_t)kFlagHitOverflow);
    }
}

// One candidate's relative vertices and face normals (with error bounds),
// from which axis_of forms any of the 17 axes with selects only.
struct LaneTri {
    V3 p2, p3, q1, q2, q3;  // relative vertices (p1 = 0); their bound is u|x|
    EV3 n1, m1;             // face normals with error bounds
};

__device__ __forceinline__ EV3 ev_rel(const V3& v)
{
    return EV3{v, V3{kU * fabsf(v.x), kU * fabsf(v.y), kU * fabsf(v.z)}};
}
__device__ __forceinline__ V3 vsel(bool c, const V3& a, const V3& b)
{
    return V3{c ? a.x : b.x, c ? a.y : b.y, c ? a.z : b.z};
}
__device__ __forceinline__ EV3 esel(bool c, const EV3& a, const EV3& b) { return EV3{vsel(c, a.v, b.v), vsel(c, a.e, b.e)}; }

// Axis `k` (0..16, the reference numbering) of the lane's candidate, built
// with selects only (no divergence between lanes on different axes).
__device__ __forceinline__ EV3 axis_of(uint32_t k, const LaneTri& t)
{
    const EV3 zero{V3{0.0f, 0.0f, 0.0f}, V3{0.0f, 0.0f, 0.0f}};
    const EV3 p2 = ev_rel(t.p2), p3 = ev_rel(t.p3), q1 = ev_rel(t.q1), q2 = ev_rel(t.q2), q3 = ev_rel(t.q3);
    // edges as the reference forms them: e1 = p2 - p1, e2 = p3 - p2, e3 = p1 - p3,
    // f1 = q2 - q1, f2 = q3 - q2, f3 = q1 - q3
    const uint32_t ei = k < 11 ? (k - 2) / 3 : k - 11;  // edge of A (axes 2..13)
    const uint32_t fj = k < 11 ? (k - 2) % 3 : k - 14;  // edge of B (axes 2..10, 14..16)
    const EV3 E = esub(esel(ei == 0, p2, esel(ei == 1, p3, zero)), esel(ei == 0, zero, esel(ei == 1, p2, p3)));
    const EV3 F = esub(esel(fj == 0, q2, esel(fj == 1, q3, q1)), esel(fj == 0, q1, esel(fj == 1, q2, q3)));
    const bool ef = k >= 2 && k < 11, en = k >= 11 && k < 14;
    const EV3 X = esel(ef || en, E, F);
    const EV3 Y = esel(ef, F, esel(en, t.n1, t.m1));
    return esel(k == 0, t.n1, esel(k == 1, t.m1, ecross(X, Y)));
}

// ---------------------------------------------------------------------------
// Precision narrow phase in passes, grouping candidates by how much of the
// filtered test they need, so that the lanes of a warp run the same code:
//  1. k_prec_classify, one candidate per thread: the plain float SAT (the
//     reference's arithmetic), which also names the first separating axis. A
//     float-separated candidate needs only that axis bounded: a margin above
//     its error bound separates in every arithmetic (no hit, float and FP64
//     agree); otherwise it goes to the recheck list. Shared vertices are hits
//     at once, and so is a float hit whose every axis overlaps beyond a
//     static bound on the float and FP64 errors; other float hits go to the
//     float-hit list, whose members need all 17 bounded axes.
//  2. k_prec_settle over the float-hit list then the recheck list, one per
//     lane: pass 1 of the filtered test (all 17 axes bounded, straight-line
//     for float hits: no lane leaves early); what it leaves undecided goes to
//     the FP64 list with the mask of its undecided axes.
//  3. k_prec_df evaluates those axes in double-float arithmetic with a bound
//     on its own and FP64's errors, deciding each axis as FP64 would where
//     the bound allows; the axes it leaves open go on.
//  4. k_prec_fp64_setup forms each remaining entry's FP64 vertices and
//     normals with every lane busy; k_prec_fp64 then evaluates the open axes
//     in FP64, one axis per lane per iteration, lanes refilled from the list
//     as their candidates are decided.
// The pair set is the all-FP64 one by construction.
// ---------------------------------------------------------------------------

// project6 of the float test, which also clears `robust` unless both of the
// axis' margins are below -B (used only when no axis separates).
__device__ __forceinline__ bool project6_robust(const V3& ax, const V3& p1, const V3& p2, const V3& p3, const V3& q1,
                                                const V3& q2, const V3& q3, float B, bool& robust)
{
    const float P1 = vdot(ax, p1), P2 = vdot(ax, p2), P3 = vdot(ax, p3);
    const float Q1 = vdot(ax, q1), Q2 = vdot(ax, q2), Q3 = vdot(ax, q3);
    const float mx1 = fmaxf(fmaxf(P1, P2), P3), mn1 = fminf(fminf(P1, P2), P3);
    const float mx2 = fmaxf(fmaxf(Q1, Q2), Q3), mn2 = fminf(fminf(Q1, Q2), Q3);
    if (mn1 > mx2) return false;
    if (mn2 > mx1) return false;
    robust = robust && __fsub_rn(mn1, mx2) < -B && __fsub_rn(mn2, mx1) < -B;
    return true;
}

// The first of the 17 axes (reference order) that separates the triangles
// in float, 17 when none does (then they intersect in float). When none
// does, `robust` tells whether every axis overlaps by more than a bound on
// the float and FP64 errors: then the triangles intersect in FP64 as well.
//
// The bound follows from the largest relative coordinate A (|p_i|, |q_j| <=
// A; relative extents in [2^-20, 2^20], else never robust) by propagating
// the rounding of each operation (u = 2^-24): edges |e| <= 2A (error 4uA),
// edge x edge and the normals |c| <= 8A^2 (48uA^2), edge x normal 32A^3
// (320uA^3); a projection onto a degree-2 axis errs by at most 232uA^3, a
// margin by 512uA^3 = 2^-15 A^3; onto a degree-3 axis 1312uA^4, a margin by
// 2816uA^4 < 2^-12 A^4. FP64 errs by 2^-29 of that. B = twice (2^-14 A^3)
// and four times (2^-10 A^4) these, covering second-order terms, underflow
// (2^-149 per product, far below 2^-90) and the rounding of B itself.
__device__ __forceinline__ uint32_t tri_first_separating_axis(const V3& P1, const V3& P2, const V3& P3, const V3& Q1,
                                                              const V3& Q2, const V3& Q3, bool& robust)
{
    const V3 p1{0.0f, 0.0f, 0.0f};
    const V3 p2 = vsub(P2, P1), p3 = vsub(P3, P1);
    const V3 q1 = vsub(Q1, P1), q2 = vsub(Q2, P1), q3 = vsub(Q3, P1);
    float A = fmaxf(fmaxf(fmaxf(fabsf(p2.x), fabsf(p2.y)), fmaxf(fabsf(p2.z), fabsf(p3.x))),
                    fmaxf(fmaxf(fabsf(p3.y), fabsf(p3.z)), fmaxf(fabsf(q1.x), fabsf(q1.y))));
    A = fmaxf(A, fmaxf(fmaxf(fabsf(q1.z), fabsf(q2.x)), fmaxf(fabsf(q2.y), fabsf(q2.z))));
    A = fmaxf(A, fmaxf(fmaxf(fabsf(q3.x), fabsf(q3.y)), fabsf(q3.z)));
    robust = A >= 0x1p-20f && A <= 0x1p20f;
    const float A3 = A * A * A;
    const float B3 = 0x1p-14f * A3, B4 = 0x1p-10f * A3 * A;
    const V3 e1 = vsub(p2, p1), e2 = vsub(p3, p2), e3 = vsub(p1, p3);
    const V3 f1 = vsub(q2, q1), f2 = vsub(q3, q2), f3 = vsub(q1, q3);
    const V3 n1 = vcross(e1, e2);
    if (!project6_robust(n1, p1, p2, p3, q1, q2, q3, B3, robust)) return 0;
    const V3 m1 = vcross(f1, f2);
    if (!project6_robust(m1, p1, p2, p3, q1, q2, q3, B3, robust)) return 1;
    const V3 E[3] = {e1, e2, e3}, F[3] = {f1, f2, f3};
#pragma unroll
    for (uint32_t i = 0; i < 3; ++i)
#pragma unroll
        for (uint32_t j = 0; j < 3; ++j)
            if (!project6_robust(vcross(E[i], F[j]), p1, p2, p3, q1, q2, q3, B3, robust)) return 2 + 3 * i + j;
#pragma unroll
    for (uint32_t i = 0; i < 3; ++i)
        if (!project6_robust(vcross(E[i], n1), p1, p2, p3, q1, q2, q3, B4, robust)) return 11 + i;
#pragma unroll
    for (uint32_t j = 0; j < 3; ++j)
        if (!project6_robust(vcross(F[j], m1), p1, p2, p3, q1, q2, q3, B4, robust)) return 14 + j;
    return 17;
}

// Axis k with error bounds (kPass1Separated: its margin separates in every
// arithmetic; otherwise undecided). Relative extents outside [2^-20, 2^20]
// are never decided here (the bounds could under- or overflow).
__device__ __forceinline__ uint32_t bounded_axis_separates(uint32_t k, const V3& P1, const V3& P2, const V3& P3,
                                                           const V3& Q1, const V3& Q2, const V3& Q3)
{
    const V3 p2v = vsub(P2, P1), p3v = vsub(P3, P1);
    const V3 q1v = vsub(Q1, P1), q2v = vsub(Q2, P1), q3v = vsub(Q3, P1);
    float A = fmaxf(fmaxf(fmaxf(fabsf(p2v.x), fabsf(p2v.y)), fmaxf(fabsf(p2v.z), fabsf(p3v.x))),
                    fmaxf(fmaxf(fabsf(p3v.y), fabsf(p3v.z)), fmaxf(fabsf(q1v.x), fabsf(q1v.y))));
    A = fmaxf(A, fmaxf(fmaxf(fabsf(q1v.z), fabsf(q2v.x)), fmaxf(fabsf(q2v.y), fabsf(q2v.z))));
    A = fmaxf(A, fmaxf(fmaxf(fabsf(q3v.x), fabsf(q3v.y)), fabsf(q3v.z)));
    if (!(A >= 0x1p-20f && A <= 0x1p20f)) return kPass1Undecided;
    const EV3 zero{V3{0.0f, 0.0f, 0.0f}, V3{0.0f, 0.0f, 0.0f}};
    const EV3 p2 = ev_rel(p2v), p3 = ev_rel(p3v), q1 = ev_rel(q1v), q2 = ev_rel(q2v), q3 = ev_rel(q3v);
    LaneTri t;
    t.p2 = p2v;
    t.p3 = p3v;
    t.q1 = q1v;
    t.q2 = q2v;
    t.q3 = q3v;
    t.n1 = (k == 0 || (k >= 11 && k < 14)) ? ecross(esub(p2, zero), esub(p3, p2)) : zero;
    t.m1 = (k == 1 || k >= 14) ? ecross(esub(q2, q1), esub(q3, q2)) : zero;
    bool s32;
    return project6_bounded(axis_of(k, t), zero, p2, p3, q1, q2, q3, s32) == 0u ? kPass1Separated : kPass1Undecided;
}

__global__ void __launch_bounds__(kDetectThreads) k_prec_classify(DetectArgs a)
{
    const uint32_t n = min(a.counts[kCountCandSlots], a.cand_cap);
    const uint32_t lane = threadIdx.x & 31;
    uint32_t* hit_list = a.prec_lists;
    uint32_t* recheck = a.prec_lists + a.cand_cap;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool hit = false, to_hits = false, to_recheck = false;
        uint4 rec = make_uint4(0, 0, 0, 0);
        if (i < n) {
            V3 P1, P2, P3, Q1, Q2, Q3;
            load_tris(a, a.cand[i], P1, P2, P3, Q1, Q2, Q3, rec);
            if (veq(P1, Q1) || veq(P1, Q2) || veq(P1, Q3) || veq(P2, Q1) || veq(P2, Q2) || veq(P2, Q3) ||
                veq(P3, Q1) || veq(P3, Q2) || veq(P3, Q3)) {
                hit = true;  // a shared vertex: never separated, in any arithmetic
            } else {
                bool robust;
                const uint32_t k = tri_first_separating_axis(P1, P2, P3, Q1, Q2, Q3, robust);
                if (k == 17) {
                    if (robust) hit = true;  // every axis overlaps beyond the error bounds
                    else to_hits = true;
                } else {
                    to_recheck = bounded_axis_separates(k, P1, P2, P3, Q1, Q2, Q3) != kPass1Separated;
                }
            }
        }
        append_hit(a, hit, rec, lane);
        const uint32_t ph = warp_append(a.counts + kCountPrecHits, to_hits, lane);
        if (to_hits) hit_list[ph] = i;
        const uint32_t pr = warp_append(a.counts + kCountPrecRecheck, to_recheck, lane);
        if (to_recheck) recheck[pr] = i;
    }
}

__global__ void __launch_bounds__(kDetectThreads) k_prec_settle(DetectArgs a)
{
    const uint32_t n_hits = min(a.counts[kCountPrecHits], a.cand_cap);
    const uint32_t n = n_hits + min(a.counts[kCountPrecRecheck], a.cand_cap);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    uint2* fp64_list = (uint2*)(a.prec_lists + 2 * (size_t)a.cand_cap);
    for (uint32_t base = warp * 32; base < n; base += n_warps * 32) {
        const uint32_t j = base + lane;
        bool hit = false, queue = false;
        uint4 rec = make_uint4(0, 0, 0, 0);
        uint32_t i = 0, mask = 0;
        if (j < n) {
            i = j < n_hits ? a.prec_lists[j] : a.prec_lists[a.cand_cap + (j - n_hits)];
            V3 P1, P2, P3, Q1, Q2, Q3;
            load_tris(a, a.cand[i], P1, P2, P3, Q1, Q2, Q3, rec);
            bool hit32 = false;
            const uint32_t r = tri_pass1(P1, P2, P3, Q1, Q2, Q3, mask, hit32);
            if (r == kPass1Hit) hit = true;
            else if (r == kPass1Undecided) {
                queue = true;
                mask |= hit32 ? 0x80000000u : 0u;
            }
        }
        append_hit(a, hit, rec, lane);
        const uint32_t q = warp_append(a.counts + kCountPrecFp64, queue, lane);
        if (queue) fp64_list[q] = make_uint2(i, mask);
    }
}

// FP64 axis evaluation with every lane on the same instructions whatever its
// axis: the face normals n1 = e1 x e2 and m1 = f1 x f2 are formed once per
// candidate (FP64Tri), and per axis the cross product's two factors are
// picked by selects (integer work) before ONE FP64 cross product and the
// projections, so lanes on different kinds of axes do not issue their FP64
// instructions apart (each FP64 warp instruction takes the SM's FP64 pipe for
// many cycles). The operations and their order are the FP64 formula's
// (axis_overlaps_fp64); the projection of p1 = 0 is 0 in any order.
struct FP64Tri {
    D6 r;
    D3 n1, m1;
};
__device__ __forceinline__ FP64Tri fp64_tri(const V3& P1, const V3& P2, const V3& P3, const V3& Q1, const V3& Q2,
                                            const V3& Q3)
{
    FP64Tri t;
    t.r = fp64_relative(P1, P2, P3, Q1, Q2, Q3);
    t.n1 = dcross(t.r.p2, dsub(t.r.p3, t.r.p2));  // e1 = p2 - p1 = p2 exactly (p1 = +0)
    t.m1 = dcross(dsub(t.r.q2, t.r.q1), dsub(t.r.q3, t.r.q2));
    return t;
}
// A finite double as an unsigned key with the same order (-0 and +0 equal).
__device__ __forceinline__ uint64_t ordered_key(double d)
{
    uint64_t b = (uint64_t)__double_as_longlong(d);
    if (b == 0x8000000000000000ull) b = 0;
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ D3 dsel(bool c, const D3& a, const D3& b)
{
    return D3{c ? a.x : b.x, c ? a.y : b.y, c ? a.z : b.z};
}
// `edges`: some lane of the warp is on an edge axis (k >= 2); when none is,
// the warp skips the edge cross product (the plane axes are n1 and m1).
__device__ __forceinline__ bool axis_overlaps_fp64_uniform(uint32_t k, const FP64Tri& t, bool edges)
{
    const D3 z{0.0, 0.0, 0.0};
    const D6& r = t.r;
    D3 c = z;
    if (edges) {
        // e_i = (p2 - p1, p3 - p2, p1 - p3), f_j = (q2 - q1, q3 - q2, q1 - q3)
        const uint32_t i = k < 11 ? (k - 2) / 3 : k - 11;
        const uint32_t j = k < 11 ? (k - 2) % 3 : k - 14;
        const D3 E = dsub(dsel(i == 0, r.p2, dsel(i == 1, r.p3, z)), dsel(i == 0, z, dsel(i == 1, r.p2, r.p3)));
        const D3 F = dsub(dsel(j == 0, r.q2, dsel(j == 1, r.q3, r.q1)), dsel(j == 0, r.q1, dsel(j == 1, r.q2, r.q3)));
        const D3 X = dsel(k >= 14, F, E);
        const D3 Y = dsel(k < 11, F, dsel(k < 14, t.n1, t.m1));
        c = dcross(X, Y);
    }
    const D3 ax = dsel(k == 0, t.n1, dsel(k == 1, t.m1, c));
    // the comparisons on integer keys: the projections are finite, and after
    // -0 is made +0 the key order is the double order
    const uint64_t P1 = ordered_key(0.0), P2 = ordered_key(ddot(ax, r.p2)), P3 = ordered_key(ddot(ax, r.p3));
    const uint64_t Q1 = ordered_key(ddot(ax, r.q1)), Q2 = ordered_key(ddot(ax, r.q2)), Q3 = ordered_key(ddot(ax, r.q3));
    const uint64_t mx1 = max(max(P1, P2), P3), mn1 = min(min(P1, P2), P3);
    const uint64_t mx2 = max(max(Q1, Q2), Q3), mn2 = min(min(Q1, Q2), Q3);
    return !(mn1 > mx2) && !(mn2 > mx1);
}

// Idle lanes that trigger a refill: with the setups formed ahead a refill is
// loads only, so the lanes are refilled early (4 measured best of 4 / 8 / 12
// / 16 on the sheets; 16 was best while the refills formed the setups).
#ifndef OIBVH_FP64_REFILL
#define OIBVH_FP64_REFILL 4
#endif
constexpr uint32_t kFp64Refill = OIBVH_FP64_REFILL;

// ---------------------------------------------------------------------------
// Double-float pass: the FP64 list's undecided axes evaluated with pairs of
// floats on the FP32 pipe (the FP64 pipe of this part runs at 1/64 of its
// rate), with a bound W on |double-float value - exact| + |FP64 value -
// exact| for every quantity. The FP64 value of each projection then lies
// within W of the double-float one, so the FP64 comparisons of an axis are
// known whenever the intervals [v - W, v + W] of the two triangles' sets do
// not straddle: the axis separates in FP64, or overlaps in FP64, exactly as
// the FP64 pass would find. What stays undecided (nearly or exactly coplanar
// triangles, whose FP64 projections are rounding noise) goes on to FP64.
//
// Arithmetic (Joldes, Muller, Popescu, "Tight and rigorous error bounds for
// basic building blocks of double-word arithmetic", ACM TOMS 2017): exact
// TwoSum and Fast2Sum, the FMA-based exact product, AccurateDWPlusDW
// (relative error <= 3u^2/(1-4u)) and DWTimesDW3 (<= 4u^2), u = 2^-24. The
// relative coordinates are exact (TwoSum of two floats); the FP64 formula
// rounds them once (2^-53). Each operation then adds at most U|c| to W with
// U = 2^-44 (> 5u^2 + 2^-53, double-float and FP64 rounding together), and
// a product the propagated |a| W_b + |b| W_a + W_a W_b; 2^-140 per step covers
// underflowing low parts. The decision doubles W.
// ---------------------------------------------------------------------------
struct DF {
    float h, l;
};
struct DFB {  // a double-float value and its bound
    DF v;
    float w;
};
constexpr float kDfU = 0x1p-44f, kDfEta = 0x1p-140f;
__device__ __forceinline__ DF two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float ap = __fsub_rn(s, b), bp = __fsub_rn(s, ap);
    return DF{s, __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp))};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b)  // |a| >= |b| (or a's exponent at least b's)
{
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(const DF& x, const DF& y)  // AccurateDWPlusDW
{
    const DF s = two_sum(x.h, y.h), t = two_sum(x.l, y.l);
    const DF v = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(v.h, __fadd_rn(t.l, v.l));
}
__device__ __forceinline__ DF df_neg(const DF& x) { return DF{-x.h, -x.l}; }
__device__ __forceinline__ DF df_mul(const DF& x, const DF& y)  // DWTimesDW3
{
    const float ch = __fmul_rn(x.h, y.h), cl1 = __fmaf_rn(x.h, y.h, -ch);
    const float tl1 = __fmaf_rn(x.h, y.l, __fmul_rn(x.l, y.l));
    const float cl2 = __fmaf_rn(x.l, y.h, tl1);
    return fast_two_sum(ch, __fadd_rn(cl1, cl2));
}
__device__ __forceinline__ float df_abs(const DF& x) { return __fadd_ru(fabsf(x.h), fabsf(x.l)); }
// The propagated part is scaled by 1 + 2^-20, which covers the FP64
// rounding of the propagated error itself (2^-53 of it, second order).
constexpr float kDfGrow = 1.0f + 0x1p-20f;
__device__ __forceinline__ float dfb_w_sum(const DFB& a, const DFB& b, const DF& c)
{
    return __fadd_ru(__fmaf_ru(kDfU, df_abs(c), __fmul_ru(kDfGrow, __fadd_ru(a.w, b.w))), kDfEta);
}
__device__ __forceinline__ DFB dfb_sub(const DFB& a, const DFB& b)
{
    const DF c = df_add(a.v, df_neg(b.v));
    return DFB{c, dfb_w_sum(a, b, c)};
}
__device__ __forceinline__ DFB dfb_add(const DFB& a, const DFB& b)
{
    const DF c = df_add(a.v, b.v);
    return DFB{c, dfb_w_sum(a, b, c)};
}
// |ab - exact| + |FP64 ab - exact| <= |a| W_b + |b| W_a + 2 W_a W_b, plus the
// two roundings of the product
__device__ __forceinline__ DFB dfb_mul(const DFB& a, const DFB& b)
{
    const DF c = df_mul(a.v, b.v);
    float w = __fmaf_ru(df_abs(a.v), b.w, __fmul_ru(df_abs(b.v), a.w));
    w = __fmaf_ru(__fmul_ru(2.0f, a.w), b.w, w);
    w = __fadd_ru(__fmaf_ru(kDfU, df_abs(c), __fmul_ru(kDfGrow, w)), kDfEta);
    return DFB{c, w};
}
struct DFB3 {
    DFB x, y, z;
};
__device__ __forceinline__ DFB3 dfb3_sub(const DFB3& a, const DFB3& b)
{
    return DFB3{dfb_sub(a.x, b.x), dfb_sub(a.y, b.y), dfb_sub(a.z, b.z)};
}
// the FP64 formula's cross product: (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
__device__ __forceinline__ DFB3 dfb3_cross(const DFB3& x, const DFB3& y)
{
    return DFB3{dfb_sub(dfb_mul(x.y, y.z), dfb_mul(y.y, x.z)), dfb_sub(dfb_mul(x.z, y.x), dfb_mul(y.z, x.x)),
                dfb_sub(dfb_mul(x.x, y.y), dfb_mul(y.x, x.y))};
}
// (a.x*b.x + a.y*b.y) + a.z*b.z
__device__ __forceinline__ DFB dfb3_dot(const DFB3& a, const DFB3& b)
{
    return dfb_add(dfb_add(dfb_mul(a.x, b.x), dfb_mul(a.y, b.y)), dfb_mul(a.z, b.z));
}
// A relative coordinate P - P1: exact as a double-float; FP64 rounds it once.
__device__ __forceinline__ DFB dfb_rel(float a, float b)
{
    const DF d = two_sum(a, -b);
    return DFB{d, __fmul_ru(0x1p-53f, df_abs(d))};
}
__device__ __forceinline__ DFB3 dfb3_rel(const V3& p, const V3& o)
{
    return DFB3{dfb_rel(p.x, o.x), dfb_rel(p.y, o.y), dfb_rel(p.z, o.z)};
}
struct DFTri {
    DFB3 p2, p3, q1, q2, q3, n1, m1;
};
__device__ __forceinline__ DFB3 dfb3_sel(bool c, const DFB3& a, const DFB3& b)
{
    auto s = [c](const DFB& x, const DFB& y) {
        return DFB{DF{c ? x.v.h : y.v.h, c ? x.v.l : y.v.l}, c ? x.w : y.w};
    };
    return DFB3{s(a.x, b.x), s(a.y, b.y), s(a.z, b.z)};
}
// Axis k (0: n1, 1: m1, 2 + 3i + j: e_i x f_j, 11 + i: e_i x n1, 14 + j: f_j x
// m1), e_i = (p2 - 0, p3 - p2, 0 - p3), f_j = (q2 - q1, q3 - q2, q1 - q3) as
// the FP64 formula forms them (p2 - 0 and 0 - p3 are exact; their bounds
// grow by one rounding's share, which only widens the intervals). The two
// factors of the cross product are picked by selects, so the lanes of a warp
// run one cross product whatever their axes; `edges` (warp-uniform) is false
// when no lane of the warp is on a cross-product axis.
__device__ __forceinline__ DFB3 dfb_axis(uint32_t k, const DFTri& t, bool edges)
{
    if (!edges) return dfb3_sel(k == 0, t.n1, t.m1);
    const DFB z{DF{0.0f, 0.0f}, 0.0f};
    const DFB3 Z{z, z, z};
    const uint32_t i = k < 11 ? (k - 2) / 3 : k - 11;  // edge of A (axes 2..13)
    const uint32_t j = k < 11 ? (k - 2) % 3 : k - 14;  // edge of B (axes 2..10, 14..16)
    const DFB3 E = dfb3_sub(dfb3_sel(i == 0, t.p2, dfb3_sel(i == 1, t.p3, Z)),
                            dfb3_sel(i == 0, Z, dfb3_sel(i == 1, t.p2, t.p3)));
    const DFB3 F = dfb3_sub(dfb3_sel(j == 0, t.q2, dfb3_sel(j == 1, t.q3, t.q1)),
                            dfb3_sel(j == 0, t.q1, dfb3_sel(j == 1, t.q2, t.q3)));
    const bool ef = k >= 2 && k < 11, en = k >= 11 && k < 14;
    const DFB3 c = dfb3_cross(dfb3_sel(ef || en, E, F), dfb3_sel(ef, F, dfb3_sel(en, t.n1, t.m1)));
    return dfb3_sel(k == 0, t.n1, dfb3_sel(k == 1, t.m1, c));
}
// Axis k of FP64 known from double-floats: 0 = separates, 1 = overlaps, 2 = undecided.
__device__ __forceinline__ uint32_t dfb_axis_fp64(uint32_t k, const DFTri& t, bool edges)
{
    const DFB3 ax = dfb_axis(k, t, edges);
    const DFB P[3] = {DFB{DF{0.0f, 0.0f}, 0.0f}, dfb3_dot(ax, t.p2), dfb3_dot(ax, t.p3)};
    const DFB Q[3] = {dfb3_dot(ax, t.q1), dfb3_dot(ax, t.q2), dfb3_dot(ax, t.q3)};
    // intervals that hold the FP64 values: value as hi + lo (the sum's rounding
    // is inside the doubled bound)
    float pl = 3.4e38f, ph = -3.4e38f, ql = 3.4e38f, qh = -3.4e38f;  // min of lows, max of highs, ...
    float plh = -3.4e38f, phl = 3.4e38f, qlh = -3.4e38f, qhl = 3.4e38f;  // max of lows, min of highs
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float v = __fadd_rn(P[i].v.h, P[i].v.l), w = __fmul_ru(2.0f, __fadd_ru(P[i].w, __fmul_ru(0x1p-23f, fabsf(v))));
        const float lo = __fsub_rd(v, w), hi = __fadd_ru(v, w);
        pl = fminf(pl, lo); ph = fmaxf(ph, hi); plh = fmaxf(plh, lo); phl = fminf(phl, hi);
        const float u = __fadd_rn(Q[i].v.h, Q[i].v.l), x = __fmul_ru(2.0f, __fadd_ru(Q[i].w, __fmul_ru(0x1p-23f, fabsf(u))));
        const float ulo = __fsub_rd(u, x), uhi = __fadd_ru(u, x);
        ql = fminf(ql, ulo); qh = fmaxf(qh, uhi); qlh = fmaxf(qlh, ulo); qhl = fminf(qhl, uhi);
    }
    // FP64 mn1 lies in [pl, phl], mx1 in [plh, ph], mn2 in [ql, qhl], mx2 in [qlh, qh]
    if (pl > qh || ql > ph) return 0u;             // mn1 > mx2 or mn2 > mx1 for sure
    if (phl < qlh && qhl < plh) return 1u;         // mn1 < mx2 and mn2 < mx1 for sure
    return 2u;
}

// Idle lanes that trigger a refill of the double-float pass (a refill forms
// the new candidates' double-float vertices and normals with only the idle
// lanes active, so refilling early costs setups, late costs idle steps).
#ifndef OIBVH_DF_REFILL
#define OIBVH_DF_REFILL 12
#endif
constexpr uint32_t kDfRefill = OIBVH_DF_REFILL;

// The FP64 list through the double-float pass: each lane holds a candidate
// and evaluates one of its undecided axes per step, all lanes of a warp on
// the same instructions (dfb_axis picks the axis with selects), until an
// axis separates for sure or the mask is done; the axes still open (and the
// float answer) go to the list the FP64 passes take. A lane whose candidate
// is decided is refilled from the warp's share of the list once enough lanes
// are idle: the masks differ in length (most candidates end at their first
// axis, coplanar ones run all of theirs), so a lane per candidate for the
// whole walk would idle most lanes. The warp's share is chunks of 32
// consecutive entries, grid-strided.
__global__ void __launch_bounds__(kDetectThreads) k_prec_df(DetectArgs a)
{
    const uint32_t n = min(a.counts[kCountPrecFp64], a.cand_cap);
    const uint2* list = (const uint2*)(a.prec_lists + 2 * (size_t)a.cand_cap);
    uint2* left = (uint2*)a.prec_lists;  // the float-hit and recheck lists' room, free after the bounded pass
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t W = (gridDim.x * blockDim.x) >> 5;
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // the t-th entry of this warp's share (increasing in t)
    auto entry = [&](uint32_t t) { return (w + (t >> 5) * W) * 32u + (t & 31u); };
    uint32_t t_next = 0, dis = 0;
    bool more = entry(0) < n;
    bool live = false;
    uint2 item = make_uint2(0, 0);
    uint4 rec = make_uint4(0, 0, 0, 0);
    uint32_t mask = 0, open = 0;
    bool separated = false;
    DFTri t;
    const DFB z{DF{0.0f, 0.0f}, 0.0f};
    t.p2 = t.p3 = t.q1 = t.q2 = t.q3 = t.n1 = t.m1 = DFB3{z, z, z};
    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !live);
        if (more && (__popc(idle) >= kDfRefill || idle == 0xffffffffu)) {
            if (!live) {
                const uint32_t j = entry(t_next + __popc(idle & ((1u << lane) - 1u)));
                if (j < n) {
                    item = list[j];
                    V3 P1, P2, P3, Q1, Q2, Q3;
                    load_tris(a, a.cand[item.x], P1, P2, P3, Q1, Q2, Q3, rec);
                    live = true;
                    mask = item.y & 0x1ffffu;
                    open = 0;
                    separated = false;
                    const float A =
                        fmaxf(fmaxf(fmaxf(fabsf(__fsub_rn(P2.x, P1.x)), fabsf(__fsub_rn(P2.y, P1.y))),
                                    fmaxf(fabsf(__fsub_rn(P2.z, P1.z)), fabsf(__fsub_rn(P3.x, P1.x)))),
                              fmaxf(fmaxf(fabsf(__fsub_rn(P3.y, P1.y)), fabsf(__fsub_rn(P3.z, P1.z))),
                                    fmaxf(fabsf(__fsub_rn(Q1.x, P1.x)), fabsf(__fsub_rn(Q1.y, P1.y)))));
                    const float A2 =
                        fmaxf(fmaxf(fmaxf(fabsf(__fsub_rn(Q1.z, P1.z)), fabsf(__fsub_rn(Q2.x, P1.x))),
                                    fmaxf(fabsf(__fsub_rn(Q2.y, P1.y)), fabsf(__fsub_rn(Q2.z, P1.z)))),
                              fmaxf(fmaxf(fabsf(__fsub_rn(Q3.x, P1.x)), fabsf(__fsub_rn(Q3.y, P1.y))),
                                    fabsf(__fsub_rn(Q3.z, P1.z))));
                    const float Am = fmaxf(A, A2);
                    if (!(Am >= 0x1p-20f && Am <= 0x1p20f)) {
                        open = mask;  // the bounds could under- or overflow: all to FP64
                        mask = 0;
                    } else {
                        t.p2 = dfb3_rel(P2, P1);
                        t.p3 = dfb3_rel(P3, P1);
                        t.q1 = dfb3_rel(Q1, P1);
                        t.q2 = dfb3_rel(Q2, P1);
                        t.q3 = dfb3_rel(Q3, P1);
                        t.n1 = dfb3_cross(t.p2, dfb3_sub(t.p3, t.p2));
                        t.m1 = dfb3_cross(dfb3_sub(t.q2, t.q1), dfb3_sub(t.q3, t.q2));
                    }
                }
            }
            t_next += __popc(idle);
            more = entry(t_next) < n;
        }
        if (!__any_sync(0xffffffffu, live)) {
            if (!more) break;
            continue;
        }
        const bool busy = live && mask != 0u;
        if (__any_sync(0xffffffffu, busy)) {
            const uint32_t k = busy ? __ffs(mask) - 1 : 0u;
            const bool edges = __any_sync(0xffffffffu, busy && k >= 2);
            const uint32_t r = dfb_axis_fp64(k, t, edges);
            if (busy) {
                mask &= mask - 1;
                if (r == 0u) {
                    separated = true;
                    mask = 0;
                } else if (r == 2u) {
                    open |= 1u << k;
                }
            }
        }
        // decided lanes: the hit, or the entry with its open axes for FP64
        const bool done = live && mask == 0u;
        const bool hit = done && !separated && open == 0u;  // every axis overlaps in FP64
        const bool keep = done && !separated && open != 0u;
        if (done && !keep) dis += (hit != ((item.y >> 31) != 0u)) ? 1u : 0u;
        append_hit(a, hit, rec, lane);
        const uint32_t q = warp_append(a.counts + kCountPrecLeft, keep, lane);
        if (keep) left[q] = make_uint2(item.x, open | (item.y & 0x80000000u));
        if (done) live = false;
    }
    const uint32_t nd = __reduce_add_sync(0xffffffffu, dis);
    if (lane == 0 && nd) atomicAdd(a.counts + kCountDisagree, nd);
}

// FP64 setups (fp64_tri and the hit record) of the FP64 list's first
// fp64_tri_cap entries, one entry per lane: formed here with every lane of a
// warp busy, where k_prec_fp64 would form them in its refills with only the
// refilling lanes. Structure of arrays: row r of entry i at r * cap + i.
__device__ __forceinline__ void fp64_tri_store(double* base, uint32_t cap, uint32_t i, const FP64Tri& t, const uint4& rec)
{
    const double v[21] = {t.r.p2.x, t.r.p2.y, t.r.p2.z, t.r.p3.x, t.r.p3.y, t.r.p3.z, t.r.q1.x,
                          t.r.q1.y, t.r.q1.z, t.r.q2.x, t.r.q2.y, t.r.q2.z, t.r.q3.x, t.r.q3.y,
                          t.r.q3.z, t.n1.x, t.n1.y, t.n1.z, t.m1.x, t.m1.y, t.m1.z};
#pragma unroll
    for (uint32_t r = 0; r < 21; ++r) base[(size_t)r * cap + i] = v[r];
    uint64_t* w = (uint64_t*)base;
    w[(size_t)21 * cap + i] = ((uint64_t)rec.y << 32) | rec.x;
    w[(size_t)22 * cap + i] = ((uint64_t)rec.w << 32) | rec.z;
}
__device__ __forceinline__ void fp64_tri_load(const double* base, uint32_t cap, uint32_t i, FP64Tri& t, uint4& rec)
{
    double v[21];
#pragma unroll
    for (uint32_t r = 0; r < 21; ++r) v[r] = __ldcg(base + (size_t)r * cap + i);
    t.r.p2 = D3{v[0], v[1], v[2]};
    t.r.p3 = D3{v[3], v[4], v[5]};
    t.r.q1 = D3{v[6], v[7], v[8]};
    t.r.q2 = D3{v[9], v[10], v[11]};
    t.r.q3 = D3{v[12], v[13], v[14]};
    t.n1 = D3{v[15], v[16], v[17]};
    t.m1 = D3{v[18], v[19], v[20]};
    const uint64_t* w = (const uint64_t*)base;
    const uint64_t r0 = __ldcg(w + (size_t)21 * cap + i), r1 = __ldcg(w + (size_t)22 * cap + i);
    rec = make_uint4((uint32_t)r0, (uint32_t)(r0 >> 32), (uint32_t)r1, (uint32_t)(r1 >> 32));
}
__global__ void __launch_bounds__(kDetectThreads) k_prec_fp64_setup(DetectArgs a)
{
    const uint32_t n = min(min(a.counts[kCountPrecLeft], a.cand_cap), a.fp64_tri_cap);
    const uint2* list = (const uint2*)a.prec_lists;  // what the double-float pass left open
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        V3 P1, P2, P3, Q1, Q2, Q3;
        uint4 rec;
        load_tris(a, a.cand[list[i].x], P1, P2, P3, Q1, Q2, Q3, rec);
        fp64_tri_store(a.fp64_tri, a.fp64_tri_cap, i, fp64_tri(P1, P2, P3, Q1, Q2, Q3), rec);
    }
}

// The FP64 list in lockstep: every lane holds one undecided candidate and
// evaluates ONE of its undecided axes (in order) per iteration, so the FP64
// pipe sees full warps however many axes each candidate needs; a lane whose
// candidate is decided (an axis separates: no hit; none left: hit) takes the
// next one from the warp's range, once kFp64Refill lanes are idle (a refill
// costs the setup's loads, or, past the setup buffer, the chain candidate ->
// faces -> vertices and the setup's FP64 work).
__global__ void __launch_bounds__(kDetectThreads) k_prec_fp64(DetectArgs a)
{
    const uint32_t n = min(a.counts[kCountPrecLeft], a.cand_cap);
    const uint2* list = (const uint2*)a.prec_lists;  // what the double-float pass left open
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t per = (n + n_warps - 1) / n_warps;
    const uint32_t lo = min(n, warp * per), hi = min(n, lo + per);
    uint32_t next = lo;  // warp-uniform
    bool busy = false;
    uint32_t mask = 0, evaluated = 0, dis = 0, cands = 0;
    FP64Tri t{};
    uint4 rec = make_uint4(0, 0, 0, 0);
    for (;;) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !busy);
        const bool refill = __popc(idle) >= kFp64Refill || idle == 0xffffffffu;
        const uint32_t take = refill ? min((uint32_t)__popc(idle), hi - next) : 0u;
        const uint32_t rank = __popc(idle & ((1u << lane) - 1u));
        if (!busy && rank < take) {
            const uint32_t i = next + rank;
            const uint2 item = list[i];
            if (i < a.fp64_tri_cap) {  // formed by k_prec_fp64_setup
                fp64_tri_load(a.fp64_tri, a.fp64_tri_cap, i, t, rec);
            } else {
                V3 P1, P2, P3, Q1, Q2, Q3;
                load_tris(a, a.cand[item.x], P1, P2, P3, Q1, Q2, Q3, rec);
                t = fp64_tri(P1, P2, P3, Q1, Q2, Q3);
            }
            mask = item.y;
            busy = true;
            ++cands;
        }
        next += take;
        bool hit = false;
        const uint32_t k = busy ? __ffs(mask & 0x1ffffu) - 1 : 0u;
        const bool edges = __any_sync(0xffffffffu, busy && k >= 2);
        if (busy) {
            mask &= mask - 1;  // the lowest set bit is the axis just taken
            ++evaluated;
            const bool overlaps = axis_overlaps_fp64_uniform(k, t, edges);
            if (!overlaps || (mask & 0x1ffffu) == 0) {
                busy = false;
                hit = overlaps;
                dis += hit != ((mask >> 31) != 0u) ? 1u : 0u;
            }
        }
        append_hit(a, hit, rec, lane);
        if (!__any_sync(0xffffffffu, busy) && next >= hi) break;
    }
    const uint32_t axes = __reduce_add_sync(0xffffffffu, evaluated);
    const uint32_t nc = __reduce_add_sync(0xffffffffu, cands);
    const uint32_t nd = __reduce_add_sync(0xffffffffu, dis);
    if (lane == 0) {
        if (axes) atomicAdd(a.counts + kCountFp64Axes, axes);
        if (nc) atomicAdd(a.counts + kCountFp64Cands, nc);
        if (nd) atomicAdd(a.counts + kCountDisagree, nd);
    }
}

// The traversal kernels' fused narrow phase is the float test only; precision
// mode runs the broad phase alone and then its narrow-phase passes.
static inline bool fused_precision(const DetectArgs& a) { return a.precision && a.fuse_narrow; }

cudaError_t launch_init_front(const DetectArgs& a, uint32_t total0, cudaStream_t s)
{
    if (fused_precision(a)) return cudaErrorInvalidValue;
    uint32_t blocks = (total0 + kDetectThreads - 1) / kDetectThreads;
    if (blocks > (uint32_t)a.grid) blocks = (uint32_t)a.grid;
    if (blocks == 0) blocks = 1;
    note_launches(1);
    if (a.fuse_narrow) k_init_front<true><<<blocks, kDetectThreads, 0, s>>>(a, total0);
    else k_init_front<false><<<blocks, kDetectThreads, 0, s>>>(a, total0);
    return cudaGetLastError();
}

cudaError_t launch_top(const DetectArgs& a, cudaStream_t s)
{
    if (fused_precision(a)) return cudaErrorInvalidValue;
    const int smem = (int)(2 * kTopCap * sizeof(uint64_t));
    static bool configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_top<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_top<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    note_launches(1);
    if (a.fuse_narrow) k_top<true><<<1, kTopThreads, smem, s>>>(a);
    else k_top<false><<<1, kTopThreads, smem, s>>>(a);
    return cudaGetLastError();
}

static size_t walk_smem(uint32_t cap) { return (size_t)(kDetectThreads / 32) * walk_ring(cap) * 8; }  // one ring per warp

static int walk_sm_count()
{
    static int sms[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 1;
    if (!sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    return sms[dev] > 0 ? sms[dev] : 1;
}

static cudaError_t walk_configure()
{
    static bool configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && configured[dev]) return cudaSuccess;
    const int smem = (int)walk_smem(kWalkCapMax);
    cudaError_t e = cudaFuncSetAttribute(k_walk<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_walk<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_walk<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_walk<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess && dev >= 0 && dev < 64) configured[dev] = true;
    return e;
}

cudaError_t launch_walk(const DetectArgs& a, uint32_t round, cudaStream_t s)
{
    if (fused_precision(a)) return cudaErrorInvalidValue;
    if (a.walk_cap > kWalkCapMax || (a.walk_cap % 32) != 0) return cudaErrorInvalidValue;
    cudaError_t e = walk_configure();
    if (e != cudaSuccess) return e;
    note_launches(1);
    const size_t smem = walk_smem(a.walk_cap);
    const bool dense = a.grid > 3u * (uint32_t)walk_sm_count();  // 4 walker CTAs per SM asked for
    if (a.fuse_narrow) {
        if (dense) k_walk<true, true><<<a.grid, kDetectThreads, smem, s>>>(a, round);
        else k_walk<true, false><<<a.grid, kDetectThreads, smem, s>>>(a, round);
    } else {
        if (dense) k_walk<false, true><<<a.grid, kDetectThreads, smem, s>>>(a, round);
        else k_walk<false, false><<<a.grid, kDetectThreads, smem, s>>>(a, round);
    }
    return cudaGetLastError();
}

int walk_blocks_per_sm(uint32_t walk_cap, bool fused)
{
    if (walk_configure() != cudaSuccess) return 1;
    int n = 0;
    const cudaError_t e =
        fused ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_walk<true, true>, kDetectThreads, walk_smem(walk_cap))
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_walk<false, true>, kDetectThreads, walk_smem(walk_cap));
    if (e != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

uint32_t narrow_kernels(const DetectArgs& a) { return a.precision ? (a.fp64_tri_cap ? 5u : 4u) : 1u; }

cudaError_t launch_narrow(const DetectArgs& a, cudaStream_t s)
{
    if (a.precision) {
        if (a.prec_lists == nullptr || (a.fp64_tri_cap && a.fp64_tri == nullptr)) return cudaErrorInvalidValue;
        note_launches(narrow_kernels(a));
        k_prec_classify<<<a.grid, kDetectThreads, 0, s>>>(a);
        k_prec_settle<<<a.grid, kDetectThreads, 0, s>>>(a);
        k_prec_df<<<a.grid, kDetectThreads, 0, s>>>(a);
        if (a.fp64_tri_cap) k_prec_fp64_setup<<<a.grid, kDetectThreads, 0, s>>>(a);
        k_prec_fp64<<<a.grid, kDetectThreads, 0, s>>>(a);
        return cudaGetLastError();
    }
    note_launches(1);
    k_narrow<<<a.grid, kDetectThreads, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace oibvh
