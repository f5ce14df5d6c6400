// Shared device math and data layout of the GB300 SNCH-LBVH.
//
// Every translation unit that includes this header is compiled with
// -fmad=false: each + - * / below is exactly one IEEE-754 binary32 operation
// in the reference's left-to-right expression order, so the build and the
// queries reproduce the reference's arithmetic (tyanyuy3125/snch-lbvh,
// include/snch_lbvh/core/{aabb,cone,utility}.cuh and scene.cuh) bit for bit,
// except where CUDA's acosf/asinf/atan2f/sinf/cosf are called (cone code).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define SNCH_DEV __device__ __forceinline__

namespace snch
{

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr float kEps = 1.1920928955078125e-07f;  // epsilon<float>() utility.cuh:186
constexpr float kPi = 3.14159274101257324219f;   // static_cast<float>(M_PI)
constexpr float kPi2 = 1.57079637050628662109f;  // static_cast<float>(M_PI_2)
constexpr int kStackDepth = 64;                   // query.cuh:250, 338 (64-entry stacks)

// bits of the per-scene device status word
enum : uint32_t
{
    kStatusStackOverflow = 1u,     // a traversal needed more than kStackDepth entries
    kStatusLookbackTimeout = 2u,   // a decoupled look-back wait gave up
    kStatusHashFull = 4u,          // the edge hash table had no free slot
    kStatusRefitTimeout = 8u,      // reserved
    kStatusTreeDepth = 16u,        // a wide-record pass met a tree deeper than its bound
    kStatusCopyTimeout = 32u,      // a bulk copy into shared memory did not complete in time
    kStatusWorkTimeout = 64u,      // a persistent search stopped taking work (results incomplete)
};

struct f3
{
    float x, y, z;
};
struct Box  // aabb<float,3> aabb.cuh:11-16 (upper first)
{
    f3 upper, lower;
};
struct Cone  // cone<float,3> cone.cuh:10-16
{
    f3 axis;
    float half_angle, radius;
};

// ---------------------------------------------------------------- HBM layout
// Reference-layout records (bvh.cuh:27-33): nodes, aabbs and cones indexed by
// node id; internal nodes 0..N-2, the leaf of sorted position j is N-1+j.
struct NodeRec
{
    uint32_t parent, left, right, object;
};

// Traversal layout. One 64-byte record per internal node holds both child
// boxes and both child node ids, so expanding a node is one 64-B line
// (four 16-B vector loads) instead of the reference's four scattered records.
//   a = (L.upper.xyz, L.lower.x)  b = (L.lower.yz, R.upper.xy)
//   c = (R.upper.z, R.lower.xyz)  d = (bits L, bits R, 0, 0)
// d = (bits L, bits R, leaf info of L, leaf info of R); a leaf child's info is
// its DFS rank | owned-edge count << 30 (written by the rank pass), so the
// silhouette traversal reaches a leaf's edges without reading its LeafRec.
struct alignas(64) InnerRec
{
    float4 a, b, c, d;
};
constexpr uint32_t kLeafRankMask = (1u << 30) - 1u;
// Child cones of an internal node (silhouette traversal), 48 B:
//   a = (L.axis.xyz, L.half)  b = (L.radius, R.axis.xyz)  c = (R.half, R.radius, 0, 0)
struct alignas(16) InnerConeRec
{
    float4 a, b, c;
};
// Leaf triangle in sorted order, vertices gathered: 48 B
//   v0 = (pa.xyz, bits original index)  v1 = (pb.xyz, bits owned-edge count)  v2 = (pc.xyz, 0)
struct alignas(16) LeafRec
{
    float4 v0, v1, v2;
};
// Owned silhouette edge of a sorted leaf (slot 3*j+k), 64 B, with the two
// face normals precomputed exactly as silhouette_edge::normal(f) computes them:
//   a = (pa.xyz, bits has_face flags)  b = (pb.xyz, bits edge id)  c = (n0.xyz, 0)  d = (n1.xyz, 0)
struct alignas(64) EdgeRec
{
    float4 a, b, c, d;
};

// Wide traversal records (4- or 8-way nodes collapsed from the binary tree).
// The binary internal nodes whose depth below the (mesh) root is a multiple
// of k (k = 2 for W = 4, k = 3 for W = 8) become wide nodes. A record holds
// the k binary levels below its node as a slot tree: level l (1..k) has 2^l
// positions, flat index f = 2^l - 2 + j, parent ((f + 2) >> 1) - 2, so a
// search applies at every collapsed level exactly the tests the binary search
// applies there (which makes the set of leaves it reaches the binary one).
// A leaf met above the last level is forwarded to the leftmost position below
// it through "pass" positions (the leaf's box with an empty sibling, so the
// sibling test passes, and a cone of half-angle pi, so the cone test passes);
// positions under nothing are empty (empty box, cone half-angle -1).
// The last level's W positions are the children. Floats, structure of arrays
// over P = 2 W positions (F = 2 W - 2 used):
//   [0, 6 P)            lower.x, lower.y, lower.z, upper.x, upper.y, upper.z
//   [6 P, 6 P + W)      child: wide node index, kWideLeaf | sorted leaf position, or kInvalid
//   [6 P + W, 6 P + 2 W) leaf info of a leaf child: DFS rank | owned-edge count << 30
//   [6 P + 2 W, 11 P + 2 W) cone axis.x, axis.y, axis.z, half_angle, radius
// = 384 B (W = 4) / 768 B (W = 8); the nearest search reads the first
// 224 / 448 B of a record, the silhouette search all of it.
constexpr uint32_t kWideLeaf = 0x80000000u;
template <int W>
struct WideLayout
{
    static_assert(W == 4 || W == 8, "wide nodes are 4- or 8-way");
    static constexpr int P = 2 * W;                 // slot-tree positions (padded)
    static constexpr int F = 2 * W - 2;             // positions used
    static constexpr int S0 = W - 2;                // position of the first child slot
    static constexpr int kLevels = W == 4 ? 2 : 3;  // binary levels per record
    static constexpr int kChild = 6 * P;            // float offsets
    static constexpr int kInfo = 6 * P + W;
    static constexpr int kCone = 6 * P + 2 * W;
    static constexpr int kRecF4 = (11 * P + 2 * W) / 4;  // record size in float4
    static constexpr int kStack = W == 4 ? 96 : 128;     // traversal stack entries
};

// Everything a query kernel reads, passed by value.
struct TreeView
{
    uint32_t num_tris = 0;  // N
    const NodeRec *nodes = nullptr;
    const Box *aabbs = nullptr;  // aabbs[0] is the root box
    const InnerRec *inner = nullptr;
    const InnerConeRec *inner_cones = nullptr;
    const LeafRec *leaves = nullptr;
    const EdgeRec *edges = nullptr;
    uint32_t *status = nullptr;
    int near_first = 1;               // 1: near-first nearest/silhouette traversal, 0: the reference's stack order
    const uint32_t *order = nullptr;  // optional: thread i answers query order[i] (Morton-sorted batches)
    const uint32_t *order_count = nullptr;  // optional: device count of valid entries of order
    int persistent = 0;  // persistent lane-refill kernels (same results): bit 0 nearest, bit 1 silhouette, bit 2 ray
    // batched queries over a batched scene: the mesh of each query (input position)
    // selects the subtree it searches; results are reported per mesh
    const uint32_t *query_mesh = nullptr;
    const uint32_t *mesh_root = nullptr;       // subtree root per mesh (leaf id for one triangle)
    const uint32_t *mesh_tri_start = nullptr;  // first (global) triangle per mesh
    const int32_t *mesh_edge_start = nullptr;  // first (global) silhouette edge id per mesh
    uint32_t num_meshes = 0;
    // node width of the near-first nearest / silhouette searches: 2 (binary
    // records above) or 4 / 8 (wide records); same results at every width
    int width_near = 2, width_sil = 2;
    // threads per block of the binary near-first nearest / silhouette searches (64, 128, 256)
    int block_near = 128, block_sil = 128;
    // warp packets (a warp's 32 queries walk one shared traversal): 0 never,
    // 1 always, 2 when the batch is Morton-ordered (order_coherent)
    int packet_near = 0, packet_sil = 0;
    int64_t packet_persistent_min = int64_t(1) << 19;  // packet batches this large run persistent (rays: 4x)
    int order_coherent = 0;  // order[] is the batch's Morton order (neighbours share warps)
    // the internal nodes of the top tree levels in heap order (slot 0 the root,
    // the children of slot i at 2i+1 / 2i+2), staged in shared memory by the
    // persistent packet searches; top_slots = 2^levels - 1, 0 = off
    const InnerRec *top_inner = nullptr;
    const InnerConeRec *top_cones = nullptr;
    uint32_t top_slots = 0;
    // 1: results are written at their batch position i (coalesced) instead of at
    // query order[i]; the launcher then scatters them to query order (unseeded,
    // fully ordered batches of the kernels that support it)
    int order_bits = 24;  // Morton bits of a plain scene's query-order key (sorted in ceil(bits / 8) passes)
    int out_batch_order = 0;
    int out_batch_order_enabled = 0;  // SNCH_OPT_OUTPUT_SCATTER
    const float4 *wide4 = nullptr, *wide8 = nullptr;        // wide records
    const uint32_t *wide4_of = nullptr, *wide8_of = nullptr;  // wide index of each binary wide-root node
};

// Where a query's search starts: the whole tree (node 0), or for a batched
// query its mesh's subtree; kInvalid = nothing to search (no triangles, or an
// unknown mesh). Offsets turn batch-wide triangle / edge ids into per-mesh ids.
struct QueryRoot
{
    uint32_t node;
    uint32_t tri_off;
    int32_t edge_off;
};
SNCH_DEV QueryRoot query_root(const TreeView &t, int64_t q)
{
    QueryRoot r{t.num_tris ? 0u : 0xFFFFFFFFu, 0u, 0};
    if (t.query_mesh)
    {
        const uint32_t m = __ldg(t.query_mesh + q);
        r.node = m < t.num_meshes ? __ldg(t.mesh_root + m) : 0xFFFFFFFFu;
        if (r.node != 0xFFFFFFFFu)
        {
            r.tri_off = __ldg(t.mesh_tri_start + m);
            r.edge_off = __ldg(t.mesh_edge_start + m);
        }
    }
    return r;
}

// Seeded search: per-query initial radius, and where queries that find
// nothing inside it are marked for the unbounded fallback pass.
struct SeedArgs
{
    const float *radius = nullptr;   // nullptr: unbounded
    uint32_t *fail_flag = nullptr;   // per query index: 1 = empty seeded result (finite radius)
    // Tail cap (near-first kernels): a query still searching after `cap` node
    // expansions stops, writes the distance of the best candidate it has (an
    // upper bound of its answer; +inf if none) to defer_radius[q] and is listed
    // in defer_list; a second, seeded pass over the list finishes it with the
    // same result. The warps of the first pass no longer wait for their slowest
    // lane, and the second pass runs the long searches densely, tightly bounded.
    uint32_t cap = 0;                // 0: no cap
    uint32_t *defer_list = nullptr;
    uint32_t *defer_count = nullptr;
    float *defer_radius = nullptr;
};

// index of the query answered by global thread i
SNCH_DEV int64_t query_index(const TreeView &t, int64_t i) { return t.order ? (int64_t)__ldg(t.order + i) : i; }
// where the result of the query at batch position i (query index q) is written
SNCH_DEV int64_t out_pos(const TreeView &t, int64_t i, int64_t q) { return t.out_batch_order ? i : q; }
// number of queries of this launch (the fallback pass reads it from the device)
SNCH_DEV int64_t query_count(const TreeView &t, int64_t n) { return t.order_count ? (int64_t)*t.order_count : n; }

// warp-aggregated append of q to list (order of the list is irrelevant)
SNCH_DEV void append_failed(uint32_t *list, uint32_t *count, uint32_t q, bool failed)
{
    const uint32_t active = __activemask();
    const uint32_t mask = __ballot_sync(active, failed);
    if (!failed)
        return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(count, (uint32_t)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    list[base + __popc(mask & ((1u << lane) - 1u))] = q;
}

// ---------------------------------------------------------------- vector math
SNCH_DEV f3 mk(float x, float y, float z)
{
    f3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
SNCH_DEV f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
// dot / length / squared_length / normalize / cross: utility.cuh:238, 382-389, 400-407, 427-431, 449-455
SNCH_DEV float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SNCH_DEV float len3(f3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
SNCH_DEV float sqlen3(f3 a) { return (a.x * a.x + a.y * a.y + a.z * a.z); }
SNCH_DEV f3 normalize3(f3 v)
{
    float n = len3(v);
    return mk(v.x / n, v.y / n, v.z / n);
}
SNCH_DEV f3 cross3(f3 u, f3 v) { return mk(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x); }
SNCH_DEV f3 cabs3(f3 a) { return mk(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
// std::min / std::max with their argument order (matters for NaN)
SNCH_DEV float smin(float a, float b) { return (b < a) ? b : a; }
SNCH_DEV float smax(float a, float b) { return (a < b) ? b : a; }

SNCH_DEV f3 load_vert(const float *__restrict__ v, int32_t i)
{
    const float *p = v + 3 * (int64_t)i;
    return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

// centroid aabb.cuh:271-279; the reference's "* 0.5" (double) rounds exactly like "* 0.5f"
SNCH_DEV f3 centroid(const Box &b)
{
    return mk((b.upper.x + b.lower.x) * 0.5f, (b.upper.y + b.lower.y) * 0.5f, (b.upper.z + b.lower.z) * 0.5f);
}

// merge(aabb,aabb) aabb.cuh:113-124
SNCH_DEV Box merge_box(const Box &l, const Box &r)
{
    Box m;
    m.upper = mk(fmaxf(l.upper.x, r.upper.x), fmaxf(l.upper.y, r.upper.y), fmaxf(l.upper.z, r.upper.z));
    m.lower = mk(fminf(l.lower.x, r.lower.x), fminf(l.lower.y, r.lower.y), fminf(l.lower.z, r.lower.z));
    return m;
}

// mindist aabb.cuh:144-150 (squared)
// Scalar on purpose: the sm_100-family paired forms (mul.rn.f32x2, add.rn.f32x2)
// would halve the issue slots of these sums, but the compiler was seen to fuse
// a paired product and the paired sum that consumes it into one fused
// multiply-add despite the explicit rounding modifiers (a GPU probe: 1.6M of
// 4.2M paired sums of products differed from the scalar ones), which would
// change the reference's roundings.
SNCH_DEV float mindist(const Box &b, f3 p)
{
    const float dx = fminf(b.upper.x, fmaxf(b.lower.x, p.x)) - p.x;
    const float dy = fminf(b.upper.y, fmaxf(b.lower.y, p.y)) - p.y;
    const float dz = fminf(b.upper.z, fmaxf(b.lower.z, p.z)) - p.z;
    return dx * dx + dy * dy + dz * dz;
}

// minmaxdist aabb.cuh:182-209 (squared)
SNCH_DEV float minmaxdist(const Box &b, f3 p)
{
    float rmx = (b.lower.x - p.x) * (b.lower.x - p.x), rmy = (b.lower.y - p.y) * (b.lower.y - p.y),
          rmz = (b.lower.z - p.z) * (b.lower.z - p.z);
    float rMx = (b.upper.x - p.x) * (b.upper.x - p.x), rMy = (b.upper.y - p.y) * (b.upper.y - p.y),
          rMz = (b.upper.z - p.z) * (b.upper.z - p.z);
    float t;
    if ((b.upper.x + b.lower.x) * 0.5f < p.x) { t = rmx; rmx = rMx; rMx = t; }
    if ((b.upper.y + b.lower.y) * 0.5f < p.y) { t = rmy; rmy = rMy; rMy = t; }
    if ((b.upper.z + b.lower.z) * 0.5f < p.z) { t = rmz; rmz = rMz; rMz = t; }
    const float dx = rmx + rMy + rMz;
    const float dy = rMx + rmy + rMz;
    const float dz = rMx + rMy + rmz;
    return fminf(dx, fminf(dy, dz));
}

// -------------------------------------------------------------- record packing
SNCH_DEV void unpack_inner(const InnerRec &r, Box &l, Box &rb, uint32_t &L, uint32_t &R)
{
    l.upper = mk(r.a.x, r.a.y, r.a.z);
    l.lower = mk(r.a.w, r.b.x, r.b.y);
    rb.upper = mk(r.b.z, r.b.w, r.c.x);
    rb.lower = mk(r.c.y, r.c.z, r.c.w);
    L = __float_as_uint(r.d.x);
    R = __float_as_uint(r.d.y);
}
SNCH_DEV void unpack_leaf_info(const InnerRec &r, uint32_t &Linfo, uint32_t &Rinfo)
{
    Linfo = __float_as_uint(r.d.z);
    Rinfo = __float_as_uint(r.d.w);
}
SNCH_DEV InnerRec pack_inner(const Box &l, const Box &r, uint32_t L, uint32_t R)
{
    InnerRec o;
    o.a = make_float4(l.upper.x, l.upper.y, l.upper.z, l.lower.x);
    o.b = make_float4(l.lower.y, l.lower.z, r.upper.x, r.upper.y);
    o.c = make_float4(r.upper.z, r.lower.x, r.lower.y, r.lower.z);
    o.d = make_float4(__uint_as_float(L), __uint_as_float(R), 0.0f, 0.0f);
    return o;
}
SNCH_DEV InnerRec load_inner(const InnerRec *p)
{
    const float4 *q = reinterpret_cast<const float4 *>(p);
    InnerRec r;
    r.a = __ldg(q);
    r.b = __ldg(q + 1);
    r.c = __ldg(q + 2);
    r.d = __ldg(q + 3);
    return r;
}
SNCH_DEV void unpack_cones(const InnerConeRec &r, Cone &l, Cone &rc)
{
    l.axis = mk(r.a.x, r.a.y, r.a.z);
    l.half_angle = r.a.w;
    l.radius = r.b.x;
    rc.axis = mk(r.b.y, r.b.z, r.b.w);
    rc.half_angle = r.c.x;
    rc.radius = r.c.y;
}
SNCH_DEV InnerConeRec pack_cones(const Cone &l, const Cone &r)
{
    InnerConeRec o;
    o.a = make_float4(l.axis.x, l.axis.y, l.axis.z, l.half_angle);
    o.b = make_float4(l.radius, r.axis.x, r.axis.y, r.axis.z);
    o.c = make_float4(r.half_angle, r.radius, 0.0f, 0.0f);
    return o;
}
SNCH_DEV void load_leaf(const LeafRec *p, f3 &pa, f3 &pb, f3 &pc, uint32_t &orig, uint32_t &n_owned)
{
    const float4 *q = reinterpret_cast<const float4 *>(p);
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    pa = mk(a.x, a.y, a.z);
    pb = mk(b.x, b.y, b.z);
    pc = mk(c.x, c.y, c.z);
    orig = __float_as_uint(a.w);
    n_owned = __float_as_uint(b.w);
}

// relaxed device-scope loads/stores for cross-block flags (no stale L1 lines)
SNCH_DEV uint32_t ld_relaxed(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
SNCH_DEV void st_relaxed(uint32_t *p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
SNCH_DEV uint32_t ld_acquire(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
SNCH_DEV void st_release(uint32_t *p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// float <-> order-preserving uint32 (atomicMin/atomicMax on floats)
SNCH_DEV uint32_t float_to_ordered(float f)
{
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
SNCH_DEV float ordered_to_float(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

}  // namespace snch
