/*
 * snch_device.cuh -- header-only device face of the GB300 SNCH-LBVH.
 *
 * For per-thread callers: kernels that call the reference's
 *   lbvh::query_device(bvh, lbvh::nearest(p), lbvh::scene<3>::distance_calculator())
 *   lbvh::query_device(bvh, lbvh::nearest_silhouette(p, flip), ...silhouette_distance_calculator())
 *   lbvh::query_device(bvh, lbvh::ray_intersect(lbvh::ray<float, 3>(o, d), tmax), ...intersect_test())
 *   lbvh::sample_object_in_sphere(bvh, lbvh::sphere_intersect(sph), intersect_sphere,
 *                                 measurement_getter, green_weight, u)
 *   lbvh::sample_on_object(bvh, idx, sample_on_object, u, v)
 * (tyanyuy3125/snch-lbvh core/query.cuh:82-169, 239-318, 326-423; core/sample.cuh:10-22, 26-91)
 * from inside their own kernels, under arbitrary divergence, with no shared
 * memory and no warp-collective requirement. The same call forms live here in
 * namespace snch and run this library's near-first traversal over its 64-byte
 * records (snch_traversal_view, from snch_get_traversal_view()):
 *
 *   snch::query_device(view, snch::nearest(p))                 -> thrust::pair<unsigned, float>
 *   snch::query_device(view, snch::nearest_silhouette(p, flip)) -> float
 *   snch::query_device(view, snch::nearest_silhouette_edge(p, flip)) -> thrust::pair<float, int>
 *   snch::query_device(view, snch::ray_intersect(snch::ray(o, d), tmax))
 *                                                 -> thrust::tuple<bool, float, float2, unsigned>
 *   snch::query_device(view, snch::ray_intersect<true>(snch::ray(o, d), tmax)) -> bool
 *   snch::sample_object_in_sphere(view, snch::sphere_intersect(snch::sphere(c, r)), u)
 *                                                 -> thrust::pair<int, float>
 *   snch::sample_on_object(view, idx, u, v)       -> float3
 *
 * The reference's functor arguments (distance_calculator, intersect_test, ...)
 * are accepted and ignored: the scene is always scene<3> triangles, and the
 * functors' arithmetic is built in. The snch::scene3 tag types below let the
 * existing call sites compile with `lbvh::` replaced by `snch::` and
 * `lbvh::scene<3>::` by `snch::scene3::`.
 *
 * Results are those of the library's own batch kernels (and so the
 * reference's): indices, distances, hit parameters and pdfs bit for bit. Every
 * sum and product below is an explicit round-to-nearest intrinsic
 * (__fmul_rn, __fadd_rn, ...), which the compiler never contracts into an FMA,
 * so this holds whatever -fmad setting the including kernel is compiled with.
 * Do not compile it with --use_fast_math or -ftz=true (flushed denormals change
 * the arithmetic of near-degenerate triangles).
 *
 * Per call: one traversal by the calling thread; a 64-entry stack in local
 * memory (512 B). A traversal that would need more entries stops, returns the
 * reference's "not found" value (index 0xFFFFFFFF / NaN distance) and sets
 * SNCH_DEVICE_STACK_OVERFLOW in view.status (if not NULL). Plain scenes only
 * (a batched scene's view is rejected by snch_get_traversal_view).
 */
#ifndef SNCH_DEVICE_CUH
#define SNCH_DEVICE_CUH

#include <cstdint>
#include <cuda_runtime.h>
#include <thrust/pair.h>
#include <thrust/tuple.h>

#include "snch_gb300.h"

namespace snch
{

// ------------------------------------------------------------------ queries
struct nearest_query  // query_nearest, predicator.cuh:139-171
{
    float3 target;
};
struct nearest_silhouette_query  // query_nearest_silhouette, predicator.cuh:174-207
{
    float3 target;
    bool flip_normal_orientation;
};
struct nearest_silhouette_edge_query  // the same, also returning the edge id
{
    float3 target;
    bool flip_normal_orientation;
};
struct ray  // ray<float,3>, aabb.cuh:298-313
{
    float3 origin, direction;
    __host__ __device__ ray(float3 o, float3 d) : origin(o), direction(d) {}
};
template <bool TestOnly>
struct ray_intersect_query  // query_ray_intersect<TestOnly>, predicator.cuh:43-78
{
    ray r;
    float max_dist;
};
struct sphere  // sphere<float,3>
{
    float3 center;
    float radius;
    __host__ __device__ sphere(float3 c, float r) : center(c), radius(r) {}
};
struct sphere_intersect_query  // query_sphere_intersect, predicator.cuh:82-113
{
    sphere s;
};

__host__ __device__ inline nearest_query nearest(float3 p) { return {p}; }
__host__ __device__ inline nearest_silhouette_query nearest_silhouette(float3 p, bool flip = false)
{
    return {p, flip};
}
__host__ __device__ inline nearest_silhouette_edge_query nearest_silhouette_edge(float3 p, bool flip = false)
{
    return {p, flip};
}
template <bool TestOnly = false>
__host__ __device__ inline ray_intersect_query<TestOnly> ray_intersect(const ray &r, float max_dist)
{
    return {r, max_dist};
}
__host__ __device__ inline sphere_intersect_query sphere_intersect(const sphere &s) { return {s}; }

// the reference's scene<3> functor names, as tags
struct scene3
{
    struct distance_calculator {};
    struct silhouette_distance_calculator {};
    struct intersect_test {};
    struct intersect_sphere {};
    struct measurement_getter {};
    struct green_weight {};
    struct sample_on_object {};
};

namespace detail
{
enum : uint32_t
{
    kNone = 0xFFFFFFFFu  // an enumerator: usable by reference in device code
};
constexpr float kEps = 1.1920928955078125e-07f;  // epsilon<float>()
constexpr float kPi2 = 1.57079637050628662109f;  // static_cast<float>(M_PI_2)
constexpr int kStack = 64;
constexpr uint32_t kRankMask = (1u << 30) - 1u;

struct v3
{
    float x, y, z;
};
struct box
{
    v3 upper, lower;
};
struct cone
{
    v3 axis;
    float half_angle, radius;
};

// one IEEE operation each, never contracted
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }

__device__ __forceinline__ v3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return mk(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
__device__ __forceinline__ float dot(v3 a, v3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ float length(v3 a) { return sqrt_(dot(a, a)); }
__device__ __forceinline__ v3 cross(v3 u, v3 v)
{
    return mk(sub(mul(u.y, v.z), mul(u.z, v.y)), sub(mul(u.z, v.x), mul(u.x, v.z)), sub(mul(u.x, v.y), mul(u.y, v.x)));
}
__device__ __forceinline__ v3 cabs(v3 a) { return mk(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }  // std::min
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }  // std::max
// a + b * s per axis, as the reference writes it (a + (b * s))
__device__ __forceinline__ v3 madd(v3 a, v3 b, float s) { return mk(add(a.x, mul(b.x, s)), add(a.y, mul(b.y, s)), add(a.z, mul(b.z, s))); }

__device__ __forceinline__ v3 centroid(const box &b)
{
    return mk(mul(add(b.upper.x, b.lower.x), 0.5f), mul(add(b.upper.y, b.lower.y), 0.5f),
              mul(add(b.upper.z, b.lower.z), 0.5f));
}
// mindist aabb.cuh:144-150 (squared)
__device__ __forceinline__ float mindist(const box &b, v3 p)
{
    const float dx = sub(fminf(b.upper.x, fmaxf(b.lower.x, p.x)), p.x);
    const float dy = sub(fminf(b.upper.y, fmaxf(b.lower.y, p.y)), p.y);
    const float dz = sub(fminf(b.upper.z, fmaxf(b.lower.z, p.z)), p.z);
    return add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz));
}

// ---- records (layout of snch_traversal_view, see snch_gb300.h)
struct inner
{
    box l, r;
    uint32_t L, R, Linfo, Rinfo;
};
__device__ __forceinline__ inner load_inner(const snch_traversal_view &t, uint32_t node)
{
    const float4 *q = static_cast<const float4 *>(t.inner) + 4 * (size_t)node;
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
    inner r;
    r.l.upper = mk(a.x, a.y, a.z);
    r.l.lower = mk(a.w, b.x, b.y);
    r.r.upper = mk(b.z, b.w, c.x);
    r.r.lower = mk(c.y, c.z, c.w);
    r.L = __float_as_uint(d.x);
    r.R = __float_as_uint(d.y);
    r.Linfo = __float_as_uint(d.z);
    r.Rinfo = __float_as_uint(d.w);
    return r;
}
__device__ __forceinline__ void load_cones(const snch_traversal_view &t, uint32_t node, cone &l, cone &r)
{
    const float4 *q = static_cast<const float4 *>(t.inner_cones) + 3 * (size_t)node;
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    l.axis = mk(a.x, a.y, a.z);
    l.half_angle = a.w;
    l.radius = b.x;
    r.axis = mk(b.y, b.z, b.w);
    r.half_angle = c.x;
    r.radius = c.y;
}
struct leaf
{
    v3 a, b, c;
    uint32_t orig, rank;
};
__device__ __forceinline__ leaf load_leaf(const snch_traversal_view &t, uint32_t pos)
{
    const float4 *q = static_cast<const float4 *>(t.leaves) + 3 * (size_t)pos;
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    return {mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), __float_as_uint(a.w), __float_as_uint(c.w)};
}
__device__ __forceinline__ box root_box(const snch_traversal_view &t)
{
    const float *q = t.root_box;
    return {mk(__ldg(q), __ldg(q + 1), __ldg(q + 2)), mk(__ldg(q + 3), __ldg(q + 4), __ldg(q + 5))};
}
__device__ __forceinline__ void overflow(const snch_traversal_view &t)
{
    if (t.status)
        atomicOr(t.status, SNCH_DEVICE_STACK_OVERFLOW);
}

// ---- nearest
// find_closest_point_triangle scene.cuh:34-110 (Ericson's Voronoi regions), distance
__device__ inline float triangle_distance(v3 pa, v3 pb, v3 pc, v3 x)
{
    const v3 ab = vsub(pb, pa), ac = vsub(pc, pa), ax = vsub(x, pa);
    const float d1 = dot(ab, ax), d2 = dot(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f)
        return length(vsub(x, pa));
    const v3 bx = vsub(x, pb);
    const float d3 = dot(ab, bx), d4 = dot(ac, bx);
    if (d3 >= 0.0f && d4 <= d3)
        return length(vsub(x, pb));
    const v3 cx = vsub(x, pc);
    const float d5 = dot(ab, cx), d6 = dot(ac, cx);
    if (d6 >= 0.0f && d5 <= d6)
        return length(vsub(x, pc));
    const float vc = sub(mul(d1, d4), mul(d3, d2));
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f)
        return length(vsub(x, madd(pa, ab, div(d1, sub(d1, d3)))));
    const float vb = sub(mul(d5, d2), mul(d1, d6));
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f)
        return length(vsub(x, madd(pa, ac, div(d2, sub(d2, d6)))));
    const float va = sub(mul(d3, d6), mul(d5, d4));
    if (va <= 0.0f && sub(d4, d3) >= 0.0f && sub(d5, d6) >= 0.0f)
    {
        const float w = div(sub(d4, d3), add(sub(d4, d3), sub(d5, d6)));
        return length(vsub(x, madd(pb, vsub(pc, pb), w)));
    }
    const float denom = div(1.0f, add(add(va, vb), vc));
    const float v = mul(vb, denom), w = mul(vc, denom);
    return length(vsub(x, mk(add(add(pa.x, mul(ab.x, v)), mul(ac.x, w)), add(add(pa.y, mul(ab.y, v)), mul(ac.y, w)),
                             add(add(pa.z, mul(ab.z, v)), mul(ac.z, w)))));
}
// among equal squared distances the reference keeps the leaf it visits last
// (query.cuh:286, 304); LeafRec carries each leaf's depth-first rank
__device__ __forceinline__ void nearest_leaf(const snch_traversal_view &t, uint32_t pos, v3 p, float &best,
                                             uint32_t &best_rank, uint32_t &nearest)
{
    const leaf f = load_leaf(t, pos);
    float d = triangle_distance(f.a, f.b, f.c, p);
    d = mul(d, d);
    if (d < best || (d == best && (nearest == kNone || f.rank > best_rank)))
    {
        best = d;
        best_rank = f.rank;
        nearest = f.orig;
    }
}

// ---- silhouette
__device__ inline float project_to_plane(v3 n, v3 e)  // cone.cuh:34-42, 58-66
{
    const float sign = copysignf(1.0f, n.z);
    const float a = div(-1.0f, add(sign, n.z));
    const float b = mul(mul(n.x, n.y), a);
    const v3 b1 = mk(add(1.0f, mul(mul(mul(sign, n.x), n.x), a)), mul(sign, b), -mul(sign, n.x));
    const v3 b2 = mk(b, add(sign, mul(mul(n.y, n.y), a)), -n.y);
    const float r1 = dot(e, cabs(b1)), r2 = dot(e, cabs(b2));
    return sqrt_(add(mul(r1, r1), mul(r2, r2)));
}
__device__ __forceinline__ bool inrange(float v, float lo, float hi) { return v >= lo && v <= hi; }
// overlap(cone<float,3>, ...) cone.cuh:168-212
__device__ inline bool cone_overlap(const cone &bc, v3 o, const box &b, float dist_to_box)
{
    if (bc.half_angle >= kPi2 || dist_to_box < kEps)
        return true;
    const v3 c = centroid(b);
    v3 v = vsub(c, o);
    const float l = length(v);
    v = mk(div(v.x, l), div(v.y, l), div(v.z, l));
    const float dax = acosf(smax(-1.0f, smin(1.0f, dot(bc.axis, v))));
    if (inrange(kPi2, sub(dax, bc.half_angle), add(dax, bc.half_angle)))
        return true;
    if (l > bc.radius)
    {
        const float hs = add(bc.half_angle, asinf(div(bc.radius, l)));
        return hs >= kPi2 ? true : inrange(kPi2, sub(dax, hs), add(dax, hs));
    }
    const v3 e = vsub(b.upper, c);
    const float s = sub(l, dot(e, cabs(v)));
    if (s <= 0.0f)
        return true;
    const float hs = add(bc.half_angle, atan2f(project_to_plane(v, e), s));
    return hs >= kPi2 ? true : inrange(kPi2, sub(dax, hs), add(dax, hs));
}
// A decision-identical filter in front of cone_overlap: arccos from Abramowitz &
// Stegun 4.4.45 (|error| <= 6.8e-5), trusted only with a margin of kConeTol
// that bounds both evaluations' errors; otherwise cone_overlap decides.
constexpr float kConeTol = 4.0e-4f;
constexpr float kIllCond = 0.999f;
__device__ __forceinline__ float acos_as(float x)
{
    return mul(sqrt_(sub(1.0f, x)),
               add(1.5707288f, mul(x, add(-0.2121144f, mul(x, add(0.0742610f, mul(x, -0.0187293f)))))));
}
__device__ inline int cone_overlap_fast(const cone &bc, v3 o, const box &b, float dist_to_box)
{
    if (bc.half_angle >= kPi2 || dist_to_box < kEps)
        return 1;
    const v3 v = vsub(centroid(b), o);
    const float l = length(v);
    if (!(l > 0.0f))
        return -1;
    const float ax = mul(fabsf(dot(bc.axis, v)), __frcp_rn(l));
    if (!(ax <= kIllCond))
        return -1;
    const float dev = sub(kPi2, acos_as(ax));
    const float ha = bc.half_angle;
    if (dev <= sub(ha, kConeTol))
        return 1;
    if (!(l > bc.radius))
        return -1;
    const float y = __fdividef(bc.radius, l);
    if (!(y <= kIllCond))
        return -1;
    const float hs = add(ha, sub(kPi2, acos_as(fmaxf(y, 0.0f))));
    if (hs >= add(kPi2, kConeTol) || dev <= sub(hs, kConeTol))
        return 1;
    if (hs <= sub(kPi2, kConeTol) && dev >= add(hs, kConeTol))
        return 0;
    return -1;
}
__device__ __forceinline__ bool cone_test(const cone &c, v3 o, const box &b, float md)
{
    const int f = cone_overlap_fast(c, o, b, md);
    return f >= 0 ? f == 1 : cone_overlap(c, o, b, md);
}
// find_closest_point_line_segment scene.cuh:230-255
__device__ inline float segment_distance(v3 pa, v3 pb, v3 x, v3 &pt)
{
    const v3 u = vsub(pb, pa), v = vsub(x, pa);
    const float c1 = dot(u, v);
    if (c1 <= 0.0f)
    {
        pt = pa;
        return length(vsub(x, pt));
    }
    const float c2 = dot(u, u);
    if (c2 <= c1)
    {
        pt = pb;
        return length(vsub(x, pt));
    }
    pt = madd(pa, u, div(c1, c2));
    return length(vsub(x, pt));
}
// is_silhouette_edge scene.cuh:143-174
__device__ inline bool is_silhouette_edge(v3 pa, v3 pb, v3 n0, v3 n1, v3 view_dir, float d, bool flip)
{
    const float precision = 1e-3f;
    const float sign = flip ? 1.0f : -1.0f;
    if (d <= precision)
    {
        v3 ed = vsub(pb, pa);
        const float n = length(ed);
        ed = mk(div(ed.x, n), div(ed.y, n), div(ed.z, n));
        const float sda = atan2f(dot(ed, cross(n0, n1)), dot(n0, n1));
        return mul(sign, sda) > precision;
    }
    const float dot0 = dot(view_dir, n0), dot1 = dot(view_dir, n1);
    if (fabsf(dot0) <= precision)
        return mul(sign, dot1) > precision;
    if (fabsf(dot1) <= precision)
        return mul(sign, dot0) > precision;
    return mul(dot0, dot1) < 0.0f;
}
// silhouette_distance_calculator scene.cuh:978-1003 over the leaf's owned edges;
// ties: the last in the reference's visit order wins, at distance 0 the first
// (scene.cuh:791-794); key = depth-first rank * 4 + slot
__device__ inline void silhouette_leaf(const snch_traversal_view &t, uint32_t pos, uint32_t info, v3 o, bool flip,
                                       float &best, uint32_t &best_key, int32_t &best_edge)
{
    const uint32_t n_owned = info >> 30, rank = info & kRankMask;
    for (uint32_t k = 0; k < n_owned; ++k)
    {
        const float4 *e = static_cast<const float4 *>(t.edges) + 4 * (3 * (size_t)pos + k);
        const float4 ea = __ldg(e), eb = __ldg(e + 1);
        const v3 pa = mk(ea.x, ea.y, ea.z), pb = mk(eb.x, eb.y, eb.z);
        v3 cp;
        const float d = segment_distance(pa, pb, o, cp);
        if (d > best)
            continue;
        const uint32_t flags = __float_as_uint(ea.w);
        bool is_sil = (flags & 1u) == 0u || (flags & 2u) == 0u;
        if (!is_sil)
        {
            const float4 ec = __ldg(e + 2), ed = __ldg(e + 3);
            is_sil = is_silhouette_edge(pa, pb, mk(ec.x, ec.y, ec.z), mk(ed.x, ed.y, ed.z), vsub(o, cp), d, flip);
        }
        if (!is_sil)
            continue;
        const uint32_t key = rank * 4u + k;
        if (d < best || best_edge < 0 || (d > 0.0f ? key > best_key : key < best_key))
        {
            best = d;
            best_key = key;
            best_edge = __float_as_int(eb.w);
        }
    }
}
__device__ inline thrust::pair<float, int> silhouette_search(const snch_traversal_view &t, v3 p, bool flip)
{
    float best = INFINITY;
    uint32_t best_key = 0;
    int32_t best_edge = -1;
    const uint32_t ni = t.num_triangles - 1;
    if (t.num_triangles == 0)
        return {best, best_edge};
    if (t.num_triangles == 1)
    {
        // a one-triangle tree: its only leaf, with its own rank and edge count
        const float4 *q = static_cast<const float4 *>(t.leaves);
        const uint32_t info = __float_as_uint(__ldg(&q[2].w)) | (__float_as_uint(__ldg(&q[1].w)) << 30);
        silhouette_leaf(t, 0, info, p, flip, best, best_key, best_edge);
        return {best, best_edge};
    }
    uint32_t sn[kStack];
    float sd[kStack];
    int sp = 0;
    uint32_t node = 0;
    bool live = !(mindist(root_box(t), p) > mul(best, best));
    while (live)
    {
        const inner r = load_inner(t, node);
        cone lc, rc;
        load_cones(t, node, lc, rc);
        const float Lmd = mindist(r.l, p), Rmd = mindist(r.r, p);
        const float b2 = mul(best, best);
        const bool hitL = Lmd <= b2 && lc.half_angle >= 0.0f && cone_test(lc, p, r.l, Lmd);
        const bool hitR = Rmd <= b2 && rc.half_angle >= 0.0f && cone_test(rc, p, r.r, Rmd);
        if (hitL && r.L >= ni)
            silhouette_leaf(t, r.L - ni, r.Linfo, p, flip, best, best_key, best_edge);
        if (hitR && r.R >= ni)
            silhouette_leaf(t, r.R - ni, r.Rinfo, p, flip, best, best_key, best_edge);
        const float b2n = mul(best, best);
        const bool pL = hitL && r.L < ni && Lmd <= b2n, pR = hitR && r.R < ni && Rmd <= b2n;
        if (pL && pR)
        {
            if (sp > kStack - 2)
            {
                overflow(t);
                return {NAN, -1};
            }
            const bool l_first = Lmd <= Rmd;
            sn[sp] = l_first ? r.R : r.L;
            sd[sp] = l_first ? Rmd : Lmd;
            ++sp;
            node = l_first ? r.L : r.R;
            continue;
        }
        if (pL || pR)
        {
            node = pL ? r.L : r.R;
            continue;
        }
        live = false;
        while (sp > 0)
        {
            --sp;
            if (!(sd[sp] > mul(best, best)))
            {
                node = sn[sp];
                live = true;
                break;
            }
        }
    }
    return {best, best_edge};
}

// ---- ray
__device__ __forceinline__ bool ray_box(v3 o, v3 inv, const box &b, float max_dist, float &dist)  // aabb.cuh:398-431
{
    float t1 = mul(sub(b.lower.x, o.x), inv.x), t2 = mul(sub(b.upper.x, o.x), inv.x);
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = mul(sub(b.lower.y, o.y), inv.y);
    t2 = mul(sub(b.upper.y, o.y), inv.y);
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = mul(sub(b.lower.z, o.z), inv.z);
    t2 = mul(sub(b.upper.z, o.z), inv.z);
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    if (tmax >= tmin && tmax >= 0.0f && tmin <= max_dist)
    {
        dist = tmin >= 0.0f ? tmin : 0.0f;
        return true;
    }
    return false;
}
// intersect_test scene.cuh:1005-1052 (Moller-Trumbore, __frcp_rn as there)
__device__ inline bool ray_triangle(v3 o, v3 dir, v3 v0, v3 v1, v3 v2, float &t, float &uo, float &vo)
{
    const v3 e1 = vsub(v1, v0), e2 = vsub(v2, v0);
    const v3 h = cross(dir, e2);
    const float det = dot(e1, h);
    if (fabsf(det) < kEps)
        return false;
    const float inv_det = __frcp_rn(det);
    const v3 s = vsub(o, v0);
    const float u = mul(dot(s, h), inv_det);
    if (u < 0.0f || u > 1.0f)
        return false;
    const v3 qv = cross(s, e1);
    const float v = mul(dot(dir, qv), inv_det);
    if (v < 0.0f || add(u, v) > 1.0f)
        return false;
    const float tt = mul(dot(e2, qv), inv_det);
    if (tt >= 0.0f)
    {
        t = tt;
        uo = u;
        vo = v;
        return true;
    }
    return false;
}
template <bool kAny>
__device__ inline thrust::tuple<bool, float, float2, unsigned> ray_search(const snch_traversal_view &t, v3 o, v3 dir,
                                                                         float max_dist)
{
    const v3 inv = mk(div(1.0f, dir.x), div(1.0f, dir.y), div(1.0f, dir.z));
    float min_dist = INFINITY, bu = 0.0f, bv = 0.0f;
    bool found = false;
    uint32_t nearest = kNone;
    const uint32_t ni = t.num_triangles - 1;
    if (t.num_triangles > 0)
    {
        // the closer hit child is processed next without a trip through the stack
        // (the reference pushes it last and pops it at once): the reference's order
        uint32_t sn[kStack];
        float sd[kStack];
        int sp = 0;
        uint32_t node = 0;
        float nd = INFINITY;
        for (;;)
        {
            bool next = !(nd > min_dist);
            if (next && node >= ni)
            {
                const leaf f = load_leaf(t, node - ni);
                float tt, uu, vv;
                if (ray_triangle(o, dir, f.a, f.b, f.c, tt, uu, vv) && tt < max_dist && tt < min_dist)
                {
                    min_dist = tt;
                    found = true;
                    bu = uu;
                    bv = vv;
                    nearest = f.orig;
                    if (kAny)
                        break;
                }
                next = false;
            }
            else if (next)
            {
                if (sp > kStack - 2)
                {
                    overflow(t);
                    return thrust::make_tuple(false, NAN, make_float2(0.0f, 0.0f), kNone);
                }
                const inner r = load_inner(t, node);
                float Ld = 0.0f, Rd = 0.0f;
                const bool Lh = ray_box(o, inv, r.l, max_dist, Ld);
                const bool Rh = ray_box(o, inv, r.r, max_dist, Rd);
                if (Lh && Rh)
                {
                    uint32_t closer = r.L, other = r.R;
                    if (Rd < Ld)
                    {
                        const float tmp = Ld;
                        Ld = Rd;
                        Rd = tmp;
                        closer = r.R;
                        other = r.L;
                    }
                    sn[sp] = other;
                    sd[sp] = Rd;
                    ++sp;
                    node = closer;
                    nd = Ld;
                    continue;
                }
                if (Lh || Rh)
                {
                    node = Lh ? r.L : r.R;
                    nd = Lh ? Ld : Rd;
                    continue;
                }
                next = false;
            }
            if (sp == 0)
                break;
            --sp;
            node = sn[sp];
            nd = sd[sp];
        }
    }
    return thrust::make_tuple(found, min_dist, make_float2(bu, bv), nearest);
}

// ---- sphere sampling
__device__ __forceinline__ bool sphere_box(v3 c, float r, const box &b)  // aabb.cuh:433-449
{
    const float dx = sub(smax(b.lower.x, smin(c.x, b.upper.x)), c.x);
    const float dy = sub(smax(b.lower.y, smin(c.y, b.upper.y)), c.y);
    float d2 = add(mul(dx, dx), mul(dy, dy));
    const float dz = sub(smax(b.lower.z, smin(c.z, b.upper.z)), c.z);
    d2 = add(d2, mul(dz, dz));
    return d2 <= mul(r, r);
}
__device__ inline bool sphere_triangle(v3 c, float radius, v3 p1, v3 p2, v3 p3)  // scene.cuh:1054-1117
{
    const v3 e1 = vsub(p2, p1), e2 = vsub(p3, p1);
    v3 nn = cross(e1, e2);
    const float nl = length(nn);
    nn = mk(div(nn.x, nl), div(nn.y, nl), div(nn.z, nl));
    const float d = dot(nn, p1);
    const float dp = sub(dot(nn, c), d);
    const v3 proj = mk(sub(c.x, mul(dp, nn.x)), sub(c.y, mul(dp, nn.y)), sub(c.z, mul(dp, nn.z)));
    const v3 v0 = vsub(p3, p1), v1 = vsub(p2, p1), v2 = vsub(proj, p1);
    const float d00 = dot(v0, v0), d01 = dot(v0, v1), d02 = dot(v0, v2), d11 = dot(v1, v1), d12 = dot(v1, v2);
    const float inv = div(1.0f, sub(mul(d00, d11), mul(d01, d01)));
    const float u = mul(sub(mul(d11, d02), mul(d01, d12)), inv);
    const float v = mul(sub(mul(d00, d12), mul(d01, d02)), inv);
    if (u >= 0 && v >= 0 && add(u, v) <= 1)
        return fabsf(dp) <= radius;
    v3 cp = proj;
    if (u < 0)
        cp = p1;
    else if (v < 0)
        cp = p3;
    else if (add(u, v) > 1)
        cp = p2;
    const v3 dd = vsub(cp, c);
    return dot(dd, dd) <= mul(radius, radius);
}
__device__ __forceinline__ float green_weight(v3 x, v3 y)  // scene.cuh:1119-1126
{
    const float r = fmaxf(length(vsub(x, y)), 1e-4f);
    return div(1.0f, mul(3.14159265358979323846f * 4.0f, r));
}
}  // namespace detail

// ------------------------------------------------------------------ entry points
// nearest primitive: (original triangle index, distance); (0xFFFFFFFF, +inf) if none
template <typename Calc = scene3::distance_calculator>
__device__ inline thrust::pair<unsigned, float> query_device(const snch_traversal_view &t, const nearest_query &q,
                                                             Calc = Calc())
{
    using namespace detail;
    const v3 p = mk(q.target.x, q.target.y, q.target.z);
    uint32_t nearest = kNone, best_rank = 0;
    float best = INFINITY;
    const uint32_t ni = t.num_triangles - 1;
    if (t.num_triangles == 1)
        nearest_leaf(t, 0, p, best, best_rank, nearest);
    else if (t.num_triangles > 1)
    {
        // near-first: the nearer passing child next, the farther one on the stack
        uint32_t sn[kStack];
        float sd[kStack];
        int sp = 0;
        uint32_t node = 0;
        bool live = !(mindist(root_box(t), p) > best);
        while (live)
        {
            const inner r = load_inner(t, node);
            const float Lmd = mindist(r.l, p), Rmd = mindist(r.r, p);
            if (r.L >= ni && Lmd <= best)
                nearest_leaf(t, r.L - ni, p, best, best_rank, nearest);
            if (r.R >= ni && Rmd <= best)
                nearest_leaf(t, r.R - ni, p, best, best_rank, nearest);
            const bool pL = r.L < ni && Lmd <= best, pR = r.R < ni && Rmd <= best;
            if (pL && pR)
            {
                if (sp > kStack - 2)
                {
                    overflow(t);
                    return {kNone, NAN};
                }
                const bool l_first = Lmd <= Rmd;
                sn[sp] = l_first ? r.R : r.L;
                sd[sp] = l_first ? Rmd : Lmd;
                ++sp;
                node = l_first ? r.L : r.R;
                continue;
            }
            if (pL || pR)
            {
                node = pL ? r.L : r.R;
                continue;
            }
            live = false;
            while (sp > 0)
            {
                --sp;
                if (!(sd[sp] > best))
                {
                    node = sn[sp];
                    live = true;
                    break;
                }
            }
        }
    }
    return {nearest, detail::sqrt_(best)};
}

// nearest silhouette distance (+inf if none), as the reference returns it
template <typename Calc = scene3::silhouette_distance_calculator>
__device__ inline float query_device(const snch_traversal_view &t, const nearest_silhouette_query &q, Calc = Calc())
{
    return detail::silhouette_search(t, detail::mk(q.target.x, q.target.y, q.target.z), q.flip_normal_orientation)
        .first;
}

// the same with the silhouette edge id (-1 if none)
__device__ inline thrust::pair<float, int> query_device(const snch_traversal_view &t,
                                                        const nearest_silhouette_edge_query &q)
{
    return detail::silhouette_search(t, detail::mk(q.target.x, q.target.y, q.target.z), q.flip_normal_orientation);
}

// closest hit with t < max_dist: (hit, t, (u, v), original triangle index)
template <typename Test = scene3::intersect_test>
__device__ inline thrust::tuple<bool, float, float2, unsigned> query_device(const snch_traversal_view &t,
                                                                           const ray_intersect_query<false> &q,
                                                                           Test = Test())
{
    using namespace detail;
    return ray_search<false>(t, mk(q.r.origin.x, q.r.origin.y, q.r.origin.z),
                             mk(q.r.direction.x, q.r.direction.y, q.r.direction.z), q.max_dist);
}
// occlusion (TestOnly = true, query.cuh:117-121): stops at the first accepted hit
template <typename Test = scene3::intersect_test>
__device__ inline bool query_device(const snch_traversal_view &t, const ray_intersect_query<true> &q, Test = Test())
{
    using namespace detail;
    return thrust::get<0>(ray_search<true>(t, mk(q.r.origin.x, q.r.origin.y, q.r.origin.z),
                                           mk(q.r.direction.x, q.r.direction.y, q.r.direction.z), q.max_dist));
}

// SampleTriangleInSphere: one stochastic descent weighted by the Green's function
// of the ball; (original triangle index, pdf), (-1, 0) if no triangle is hit
__device__ inline thrust::pair<int, float> sample_object_in_sphere(const snch_traversal_view &t,
                                                                   const sphere_intersect_query &q, float u)
{
    using namespace detail;
    const v3 c = mk(q.s.center.x, q.s.center.y, q.s.center.z);
    const float rad = q.s.radius;
    int oi = -1;
    float opdf = 0.0f;
    const uint32_t ni = t.num_triangles - 1;
    if (t.num_triangles == 0)
        return {oi, opdf};
    uint32_t node = 0;
    float npdf = 1.0f;
    for (int level = 0; level < 2 * kStack; ++level)
    {
        if (node >= ni)
        {
            const leaf f = load_leaf(t, node - ni);
            if (sphere_triangle(c, rad, f.a, f.b, f.c))
            {
                oi = (int)f.orig;
                // measurement_getter scene.cuh:855-868: the triangle's area
                opdf = div(npdf, div(length(cross(vsub(f.c, f.a), vsub(f.b, f.a))), 2.0f));
            }
            break;
        }
        const inner r = load_inner(t, node);
        const float Lw = sphere_box(c, rad, r.l) ? green_weight(c, centroid(r.l)) : 0.0f;
        const float Rw = sphere_box(c, rad, r.r) ? green_weight(c, centroid(r.r)) : 0.0f;
        const float tw = add(Lw, Rw);
        if (!(tw > 0))
            break;
        const float Lp = div(Lw, tw);
        if (u < Lp)
        {
            u = div(u, Lp);
            node = r.L;
            npdf = mul(Lp, npdf);
        }
        else
        {
            const float Rp = sub(1.0f, Lp);
            u = div(sub(u, Lp), Rp);
            node = r.R;
            npdf = mul(Rp, npdf);
        }
    }
    return {oi, opdf};
}
template <typename Isect, typename Measure, typename Green>
__device__ inline thrust::pair<int, float> sample_object_in_sphere(const snch_traversal_view &t,
                                                                   const sphere_intersect_query &q, Isect, Measure,
                                                                   Green, float u)
{
    return sample_object_in_sphere(t, q, u);
}

// sample_on_object sample.cuh:10-22 with sample_triangle scene.cuh:14-27: a
// point on triangle idx (original index); NaN for an index out of range
__device__ inline float3 sample_on_object(const snch_traversal_view &t, int idx, float u, float v)
{
    using namespace detail;
    if (idx < 0 || (uint32_t)idx >= t.num_triangles)
        return make_float3(NAN, NAN, NAN);
    const int32_t *tr = t.triangles + 3 * (size_t)idx;
    const float *V = t.vertices;
    const int32_t i0 = __ldg(tr), i1 = __ldg(tr + 1), i2 = __ldg(tr + 2);
    const v3 pa = mk(__ldg(V + 3 * (size_t)i0), __ldg(V + 3 * (size_t)i0 + 1), __ldg(V + 3 * (size_t)i0 + 2));
    const v3 pb = mk(__ldg(V + 3 * (size_t)i1), __ldg(V + 3 * (size_t)i1 + 1), __ldg(V + 3 * (size_t)i1 + 2));
    const v3 pc = mk(__ldg(V + 3 * (size_t)i2), __ldg(V + 3 * (size_t)i2 + 1), __ldg(V + 3 * (size_t)i2 + 2));
    if (add(u, v) > 1.0f)
    {
        u = sub(1.0f, u);
        v = sub(1.0f, v);
    }
    const float w = sub(sub(1.0f, u), v);
    return make_float3(add(add(mul(w, pa.x), mul(u, pb.x)), mul(v, pc.x)),
                       add(add(mul(w, pa.y), mul(u, pb.y)), mul(v, pc.y)),
                       add(add(mul(w, pa.z), mul(u, pb.z)), mul(v, pc.z)));
}
template <typename Sampler>
__device__ inline float3 sample_on_object(const snch_traversal_view &t, int idx, Sampler, float u, float v)
{
    return sample_on_object(t, idx, u, v);
}

}  // namespace snch

#endif /* SNCH_DEVICE_CUH */
