// 2D scenes: the reference's scene<2> (include/snch_lbvh/scene.cuh:287-703) on
// the GPU -- line segments with silhouette VERTICES, the LBVH over 2D boxes and
// normal cones (bvh.cuh with aabb<float,2>, cone<float,2>), and the nearest /
// silhouette / ray / circle-sample queries (query.cuh, sample.cuh over the 2D
// functors), behind the snch_scene2_* C ABI.
//
// Compiled with -fmad=false: every + - * / is one binary32 operation in the
// reference's expression order, so topology, Morton codes, tree and boxes are
// bit-identical to the reference's and the queries replay its traversal order
// (its stack discipline and tie rules); acosf / asinf / atan2f / logf / sinf /
// cosf are CUDA's.
#include <algorithm>
#include <string>

#include "internal.h"

namespace snch
{
namespace
{

constexpr float kBvhOffset = 1e-3f;  // bvh_offset scene.cuh:12

struct B2  // aabb<float,2>, upper first
{
    float2 upper, lower;
};
struct C2  // cone<float,2>
{
    float2 axis;
    float half_angle, radius;
};

SNCH_DEV float2 f2(float x, float y) { return make_float2(x, y); }
SNCH_DEV float2 sub2(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
SNCH_DEV float dot2(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
SNCH_DEV float len2(float2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
SNCH_DEV float2 norm2(float2 v)
{
    const float n = len2(v);
    return f2(v.x / n, v.y / n);
}
SNCH_DEV float2 vload2(const float *__restrict__ v, int32_t i) { return f2(__ldg(v + 2 * i), __ldg(v + 2 * i + 1)); }
SNCH_DEV float2 centroid2(const B2 &b)
{
    return f2((b.upper.x + b.lower.x) * 0.5f, (b.upper.y + b.lower.y) * 0.5f);
}
SNCH_DEV B2 load_b2(const float4 *p)
{
    const float4 v = __ldcg(p);
    B2 b;
    b.upper = f2(v.x, v.y);
    b.lower = f2(v.z, v.w);
    return b;
}
SNCH_DEV C2 load_c2(const float4 *p)
{
    const float4 v = __ldcg(p);
    C2 c;
    c.axis = f2(v.x, v.y);
    c.half_angle = v.z;
    c.radius = v.w;
    return c;
}
SNCH_DEV float4 pack_b2(const B2 &b) { return make_float4(b.upper.x, b.upper.y, b.lower.x, b.lower.y); }
SNCH_DEV float4 pack_c2(const C2 &c) { return make_float4(c.axis.x, c.axis.y, c.half_angle, c.radius); }

// ------------------------------------------------------------------ topology
// compute_silhouettes scene.cuh:642-664: silhouette vertex v = {prev, v, next, -1}
// where later segments overwrite earlier ones (the last segment starting at v
// gives next, the last ending at v gives prev); build_bvh scene.cuh:666-683: a
// segment owns the endpoints no earlier segment touched, in (x, y) order.
__global__ void topo2_init_kernel(int64_t nv, int32_t *last_start, int32_t *last_end, int32_t *first_ref)
{
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v < nv)
    {
        last_start[v] = -1;
        last_end[v] = -1;
        first_ref[v] = 0x7FFFFFFF;
    }
}
__global__ void topo2_scan_kernel(const int32_t *__restrict__ segs, int64_t n, int32_t *last_start, int32_t *last_end,
                                  int32_t *first_ref)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int32_t a = segs[2 * i], b = segs[2 * i + 1];
    atomicMax(last_start + a, (int32_t)i);
    atomicMax(last_end + b, (int32_t)i);
    atomicMin(first_ref + a, (int32_t)i);
    atomicMin(first_ref + b, (int32_t)i);
}
__global__ void topo2_vertex_kernel(const int32_t *__restrict__ segs, int64_t nv, const int32_t *last_start,
                                    const int32_t *last_end, int4 *sv)
{
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    const int32_t s0 = last_start[v], s1 = last_end[v];
    int4 r = make_int4(-1, -1, -1, -1);
    // the later of the two writers of index 1 writes v either way
    if (s0 >= 0 || s1 >= 0)
        r.y = (int32_t)v;
    if (s0 >= 0)
        r.z = segs[2 * s0 + 1];
    if (s1 >= 0)
        r.x = segs[2 * s1];
    sv[v] = r;
}
__global__ void topo2_owned_kernel(const int32_t *__restrict__ segs, int64_t n, const int32_t *first_ref,
                                   int2 *seg_owned)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int32_t a = segs[2 * i], b = segs[2 * i + 1];
    int32_t own[2] = {-1, -1}, k = 0;
    if (first_ref[a] == (int32_t)i)
        own[k++] = a;
    if (b != a && first_ref[b] == (int32_t)i)
        own[k++] = b;
    seg_owned[i] = make_int2(own[0], own[1]);
}

// silhouette_vertex scene.cuh:291-384
SNCH_DEV bool sv_has_face(const int4 &sv, int f) { return f == 0 ? sv.z != -1 : sv.x != -1; }
SNCH_DEV float2 sv_face_normal(const float *verts, const int4 &sv, int f, bool do_normalize)
{
    const float2 pa = f == 0 ? vload2(verts, sv.y) : vload2(verts, sv.x);
    const float2 pb = f == 0 ? vload2(verts, sv.z) : vload2(verts, sv.y);
    const float2 s = sub2(pb, pa);
    const float2 nn = f2(s.y, -s.x);
    return do_normalize ? norm2(nn) : nn;
}
SNCH_DEV float2 sv_normal(const float *verts, const int4 &sv)
{
    float2 nn = f2(0.0f, 0.0f);
    if (sv_has_face(sv, 0))
    {
        const float2 a = sv_face_normal(verts, sv, 0, false);
        nn = f2(nn.x + a.x, nn.y + a.y);
    }
    if (sv_has_face(sv, 1))
    {
        const float2 a = sv_face_normal(verts, sv, 1, false);
        nn = f2(nn.x + a.x, nn.y + a.y);
    }
    return norm2(nn);
}

// ------------------------------------------------------------------ build
struct Build2
{
    uint32_t n;
    const float *verts;
    const int32_t *segs;
    const int4 *sv;
    const int2 *seg_owned;
    uint32_t *scene_box;  // ordered uints: upper.xy (max), lower.xy (min)
    float4 *leaf_box, *leaf_cone;  // original order
    uint32_t *keys, *vals;
    NodeRec *nodes;
    float4 *aabbs, *cones;  // 2N-1 each
    uint32_t *flags;
};

// aabb_getter scene.cuh:420-432
SNCH_DEV B2 seg_box(float2 p0, float2 p1)
{
    B2 b;
    b.upper = f2(fmaxf(p0.x, p1.x) + kBvhOffset, fmaxf(p0.y, p1.y) + kBvhOffset);
    b.lower = f2(fminf(p0.x, p1.x) - kBvhOffset, fminf(p0.y, p1.y) - kBvhOffset);
    return b;
}
// cone_getter scene.cuh:434-494
SNCH_DEV C2 seg_cone(const Build2 &a, const B2 &bb, int2 owned)
{
    const float2 bc = centroid2(bb);
    C2 r;
    r.axis = f2(0.0f, 0.0f);
    r.half_angle = kPi;
    r.radius = 0.0f;
    bool any = false, all_two = true;
    const int32_t ow[2] = {owned.x, owned.y};
    for (int i = 0; i < 2; ++i)
    {
        if (ow[i] == -1)
            continue;
        const int4 sv = a.sv[ow[i]];
        const float2 nn = sv_normal(a.verts, sv);
        r.axis.x += nn.x;
        r.axis.y += nn.y;
        const float2 c = vload2(a.verts, sv.y);
        r.radius = smax(r.radius, len2(f2(c.x - bc.x, c.y - bc.y)));
        all_two = all_two && sv_has_face(sv, 0) && sv_has_face(sv, 1);
        any = true;
    }
    if (!any)
        r.half_angle = -kPi;
    else if (!all_two)
        r.half_angle = kPi;
    else
    {
        const float an = len2(r.axis);
        if (an > kEps)
        {
            r.axis.x /= an;
            r.axis.y /= an;
            r.half_angle = 0.0f;
            for (int i = 0; i < 2; ++i)
            {
                if (ow[i] == -1)
                    continue;
                const int4 sv = a.sv[ow[i]];
                float2 fn[2];
                fn[0] = sv_has_face(sv, 0) ? sv_face_normal(a.verts, sv, 0, true) : f2(0.0f, 0.0f);
                fn[1] = sv_has_face(sv, 1) ? sv_face_normal(a.verts, sv, 1, true) : f2(0.0f, 0.0f);
                for (int j = 0; j < 2; ++j)
                    r.half_angle = smax(r.half_angle, acosf(smax(-1.0f, smin(1.0f, dot2(r.axis, fn[j])))));
            }
        }
    }
    return r;
}

__global__ void init2_kernel(uint32_t *scene_box)
{
    if (threadIdx.x < 2)
        scene_box[threadIdx.x] = float_to_ordered(-INFINITY);
    else if (threadIdx.x < 4)
        scene_box[threadIdx.x] = float_to_ordered(INFINITY);
}
// leaf boxes and cones in original order, and the scene box (bvh.cuh:423-432)
__global__ void __launch_bounds__(256) leaf2_kernel(Build2 a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const float2 p0 = vload2(a.verts, a.segs[2 * i]), p1 = vload2(a.verts, a.segs[2 * i + 1]);
    const B2 b = seg_box(p0, p1);
    a.leaf_box[i] = pack_b2(b);
    a.leaf_cone[i] = pack_c2(seg_cone(a, b, a.seg_owned[i]));
    atomicMax(a.scene_box + 0, float_to_ordered(b.upper.x));
    atomicMax(a.scene_box + 1, float_to_ordered(b.upper.y));
    atomicMin(a.scene_box + 2, float_to_ordered(b.lower.x));
    atomicMin(a.scene_box + 3, float_to_ordered(b.lower.y));
}
// expand_bits morton_code.cuh:19-38; morton_code(float2) 83-91: the 3D spreading, x * 2 + y
SNCH_DEV uint32_t spread3(uint32_t v)
{
    v = (v | (v << 16)) & 0x070000FFu;
    v = (v | (v << 8)) & 0x0700F00Fu;
    v = (v | (v << 4)) & 0x430C30C3u;
    v = (v | (v << 2)) & 0x49249249u;
    return v;
}
// default_morton_code_calculator<Real,2> bvh.cuh:257-279
__global__ void __launch_bounds__(256) morton2_kernel(Build2 a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n)
        return;
    const float4 lb = a.leaf_box[i];
    const float ux = ordered_to_float(a.scene_box[0]), uy = ordered_to_float(a.scene_box[1]);
    const float lx = ordered_to_float(a.scene_box[2]), ly = ordered_to_float(a.scene_box[3]);
    float px = (lb.x + lb.z) * 0.5f, py = (lb.y + lb.w) * 0.5f;
    px -= lx;
    py -= ly;
    px /= (ux - lx);
    py /= (uy - ly);
    const float res = 1024.0f;
    px = fminf(fmaxf(px * res, 0.0f), res - 1.0f);
    py = fminf(fmaxf(py * res, 0.0f), res - 1.0f);
    a.keys[i] = spread3((uint32_t)px) * 2 + spread3((uint32_t)py);
    a.vals[i] = i;
}

// rotate(float2) cone.cuh:266-275
SNCH_DEV float2 rotate2(float2 u, float2 v, float theta)
{
    const float det = u.x * v.y - u.y * v.x;
    theta *= copysignf(1.0f, det);
    const float ct = cosf(theta), st = sinf(theta);
    return f2(ct * u.x - st * u.y, st * u.x + ct * u.y);
}
// merge(cone<float,2>) cone.cuh:320-371; pi where the reference leaves the half
// angle unassigned (o_theta >= pi, lines 347-351), zeros for the axis / radius
// of a merge of two invalid cones (unset there)
SNCH_DEV C2 cone_merge2(const C2 &a, const C2 &b, float2 oa, float2 ob, float2 on)
{
    C2 r;
    r.axis = f2(0.0f, 0.0f);
    r.half_angle = 0.0f;
    r.radius = 0.0f;
    const bool va = a.half_angle >= 0.0f, vb = b.half_angle >= 0.0f;
    if (va && vb)
    {
        float2 axis_a = a.axis, axis_b = b.axis;
        float ha = a.half_angle, hb = b.half_angle;
        const float2 da = sub2(on, oa), db = sub2(on, ob);
        r.radius = sqrtf(smax(a.radius * a.radius + (da.x * da.x + da.y * da.y),
                              b.radius * b.radius + (db.x * db.x + db.y * db.y)));
        if (hb > ha)
        {
            const float2 t = axis_a;
            axis_a = axis_b;
            axis_b = t;
            const float h = ha;
            ha = hb;
            hb = h;
        }
        const float theta = acosf(smax(-1.0f, smin(1.0f, dot2(axis_a, axis_b))));
        if (smin(theta + hb, kPi) <= ha)
        {
            r.axis = axis_a;
            r.half_angle = ha;
            return r;
        }
        const float o_theta = (ha + theta + hb) / 2.0f;
        if (o_theta >= kPi)
        {
            r.axis = axis_a;
            r.half_angle = kPi;
            return r;
        }
        r.axis = rotate2(axis_a, axis_b, o_theta - ha);
        r.half_angle = o_theta;
    }
    else if (va)
        r = a;
    else if (vb)
        r = b;
    else
        r.half_angle = -kPi;
    return r;
}

// bottom-up AABB + cone refit with arrival counters (bvh.cuh:517-604, one pass)
__global__ void __launch_bounds__(128) refit2_kernel(Build2 a)
{
    const uint32_t n = a.n, ni = n - 1;
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const uint32_t orig = a.vals[j];
    if (orig >= n)
        return;
    const uint32_t leaf = ni + j;
    a.aabbs[leaf] = a.leaf_box[orig];
    a.cones[leaf] = a.leaf_cone[orig];
    if (n == 1)
        return;
    uint32_t cur = leaf;
    for (int level = 0; level < 96; ++level)
    {
        const uint32_t p = a.nodes[cur].parent;
        if (p >= ni)
            return;
        __threadfence();
        if (atomicAdd(a.flags + p, 1u) == 0u)
            return;
        __threadfence();
        const uint32_t L = a.nodes[p].left, R = a.nodes[p].right;
        const B2 lb = load_b2(a.aabbs + L), rb = load_b2(a.aabbs + R);
        const C2 lc = load_c2(a.cones + L), rc = load_c2(a.cones + R);
        B2 m;
        m.upper = f2(fmaxf(lb.upper.x, rb.upper.x), fmaxf(lb.upper.y, rb.upper.y));
        m.lower = f2(fminf(lb.lower.x, rb.lower.x), fminf(lb.lower.y, rb.lower.y));
        a.aabbs[p] = pack_b2(m);
        a.cones[p] = pack_c2(cone_merge2(lc, rc, centroid2(lb), centroid2(rb), centroid2(m)));
        cur = p;
    }
}

// ------------------------------------------------------------------ queries
struct Tree2
{
    uint32_t n;
    const float *verts;
    const int32_t *segs;
    const int4 *sv;
    const int2 *seg_owned;
    const NodeRec *nodes;
    const float4 *aabbs, *cones;
    uint32_t *status;
};
SNCH_DEV B2 node_box2(const Tree2 &t, uint32_t i)
{
    const float4 v = __ldg(t.aabbs + i);
    B2 b;
    b.upper = f2(v.x, v.y);
    b.lower = f2(v.z, v.w);
    return b;
}
SNCH_DEV C2 node_cone2(const Tree2 &t, uint32_t i)
{
    const float4 v = __ldg(t.cones + i);
    C2 c;
    c.axis = f2(v.x, v.y);
    c.half_angle = v.z;
    c.radius = v.w;
    return c;
}
// mindist / minmaxdist aabb.cuh:130-135, 161-180
SNCH_DEV float mindist2(const B2 &b, float2 p)
{
    const float dx = fminf(b.upper.x, fmaxf(b.lower.x, p.x)) - p.x;
    const float dy = fminf(b.upper.y, fmaxf(b.lower.y, p.y)) - p.y;
    return dx * dx + dy * dy;
}
SNCH_DEV float minmaxdist2(const B2 &b, float2 p)
{
    float rmx = (b.lower.x - p.x) * (b.lower.x - p.x), rmy = (b.lower.y - p.y) * (b.lower.y - p.y);
    float rMx = (b.upper.x - p.x) * (b.upper.x - p.x), rMy = (b.upper.y - p.y) * (b.upper.y - p.y);
    float t;
    if ((b.upper.x + b.lower.x) * 0.5f < p.x)
    {
        t = rmx;
        rmx = rMx;
        rMx = t;
    }
    if ((b.upper.y + b.lower.y) * 0.5f < p.y)
    {
        t = rmy;
        rmy = rMy;
        rMy = t;
    }
    return fminf(rmx + rMy, rMx + rmy);
}
// find_closest_point_line_segment(float2) scene.cuh:176-199
SNCH_DEV float closest_point_segment2(float2 pa, float2 pb, float2 x)
{
    const float2 u = sub2(pb, pa), v = sub2(x, pa);
    const float c1 = dot2(u, v);
    if (c1 <= 0.0f)
        return len2(sub2(x, pa));
    const float c2 = dot2(u, u);
    if (c2 <= c1)
        return len2(sub2(x, pb));
    const float t = c1 / c2;
    const float2 pt = f2(pa.x + u.x * t, pa.y + u.y * t);
    return len2(f2(x.x - pt.x, x.y - pt.y));
}
SNCH_DEV float seg_distance(const Tree2 &t, uint32_t obj, float2 p)
{
    return closest_point_segment2(vload2(t.verts, t.segs[2 * obj]), vload2(t.verts, t.segs[2 * obj + 1]), p);
}
SNCH_DEV float2 load_pt2(const float *p, int64_t q) { return f2(__ldg(p + 2 * q), __ldg(p + 2 * q + 1)); }

// query_device(nearest) query.cuh:239-318 over segments, the reference's order;
// a one-segment tree (where the reference reads past its node array) evaluates its leaf
__global__ void __launch_bounds__(128) nearest2_kernel(Tree2 t, const float *__restrict__ pts, int64_t n,
                                                       uint32_t *__restrict__ out_idx, float *__restrict__ out_dist)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const float2 p = load_pt2(pts, q);
    uint32_t nearest = kInvalid;
    float best = INFINITY;
    if (t.n == 1)
    {
        const float d = seg_distance(t, t.nodes[0].object, p);
        best = d * d;
        nearest = t.nodes[0].object;
    }
    else if (t.n > 1)
    {
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        sn[sp] = 0;
        sd[sp++] = mindist2(node_box2(t, 0), p);
        do
        {
            --sp;
            const uint32_t node = sn[sp];
            if (sd[sp] > best)
                continue;
            const uint32_t ch[2] = {t.nodes[node].left, t.nodes[node].right};
            const B2 lb = node_box2(t, ch[0]), rb = node_box2(t, ch[1]);
            const float md[2] = {mindist2(lb, p), mindist2(rb, p)};
            const bool ok[2] = {md[0] <= minmaxdist2(rb, p), md[1] <= minmaxdist2(lb, p)};
            for (int k = 0; k < 2; ++k)
            {
                if (!ok[k])
                    continue;
                const uint32_t obj = t.nodes[ch[k]].object;
                if (obj != kInvalid)
                {
                    float d = seg_distance(t, obj, p);
                    d *= d;
                    if (d <= best)
                    {
                        best = d;
                        nearest = obj;
                    }
                }
                else
                {
                    if (sp >= kStackDepth)
                    {
                        atomicOr(t.status, kStatusStackOverflow);
                        out_idx[q] = kInvalid;
                        out_dist[q] = NAN;
                        return;
                    }
                    sn[sp] = ch[k];
                    sd[sp++] = md[k];
                }
            }
        } while (sp > 0);
    }
    out_idx[q] = nearest;
    out_dist[q] = sqrtf(best);
}

// is_silhouette_vertex scene.cuh:112-141
SNCH_DEV bool is_silhouette_vertex(float2 n0, float2 n1, float2 view_dir, float d, bool flip)
{
    const float precision = 1e-3f;
    const float sign = flip ? 1.0f : -1.0f;
    if (d <= precision)
        return sign * (n0.x * n1.y - n0.y * n1.x) > precision;
    const float2 vu = f2(view_dir.x / d, view_dir.y / d);
    const float dot0 = dot2(vu, n0), dot1 = dot2(vu, n1);
    if (fabsf(dot0) <= precision)
        return sign * dot1 > precision;
    if (fabsf(dot1) <= precision)
        return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}
// silhouette_distance_calculator scene.cuh:512-532 with
// find_closest_silhouette_point scene.cuh:354-381 per owned vertex
SNCH_DEV bool leaf_silhouette2(const Tree2 &t, uint32_t obj, float2 o, float max_r2, float &dist, bool flip,
                               int32_t &vid)
{
    const int2 own = t.seg_owned[obj];
    const int32_t ow[2] = {own.x, own.y};
    float mr2 = max_r2;
    bool ret = false;
    for (int i = 0; i < 2; ++i)
    {
        if (ow[i] == -1 || 0.0f >= mr2)
            continue;
        const int4 sv = t.sv[ow[i]];
        const float2 pv = vload2(t.verts, sv.y);
        const float2 vd = f2(o.x - pv.x, o.y - pv.y);
        const float d = len2(vd);
        if (d * d > mr2)
            continue;
        bool is_sil = !sv_has_face(sv, 0) || !sv_has_face(sv, 1);
        if (!is_sil)
            is_sil = is_silhouette_vertex(sv_face_normal(t.verts, sv, 0, true), sv_face_normal(t.verts, sv, 1, true),
                                          vd, d, flip);
        if (is_sil && d * d <= mr2)
        {
            dist = d;
            ret = true;
            mr2 = d * d;
            vid = ow[i];
        }
    }
    return ret;
}
// overlap(cone<float,2>) cone.cuh:78-120 with project_to_plane(float2) 44-49
SNCH_DEV bool cone_overlap2(const C2 &bc, float2 o, const B2 &b, float dist_to_box)
{
    if (bc.half_angle >= kPi2 || dist_to_box < kEps)
        return true;
    const float2 c = centroid2(b);
    float2 v = f2(c.x - o.x, c.y - o.y);
    const float l = len2(v);
    v.x /= l;
    v.y /= l;
    const float dax = acosf(smax(-1.0f, smin(1.0f, dot2(bc.axis, v))));
    if (kPi2 >= dax - bc.half_angle && kPi2 <= dax + bc.half_angle)
        return true;
    if (l > bc.radius)
    {
        const float hs = bc.half_angle + asinf(bc.radius / l);
        return hs >= kPi2 ? true : (kPi2 >= dax - hs && kPi2 <= dax + hs);
    }
    const float2 e = f2(b.upper.x - c.x, b.upper.y - c.y);
    float d = dot2(e, f2(fabsf(v.x), fabsf(v.y)));
    const float s = l - d;
    if (s <= 0.0f)
        return true;
    d = fabsf(dot2(e, f2(fabsf(-v.y), fabsf(v.x))));
    const float hs = bc.half_angle + atan2f(d, s);
    return hs >= kPi2 ? true : (kPi2 >= dax - hs && kPi2 <= dax + hs);
}
// query_device(nearest_silhouette) query.cuh:326-423 over segments, the
// reference's order; also the silhouette vertex (mesh vertex id) of the answer
__global__ void __launch_bounds__(128) silhouette2_kernel(Tree2 t, const float *__restrict__ pts,
                                                          const uint8_t *__restrict__ flips, int64_t n,
                                                          float *__restrict__ out_dist, int32_t *__restrict__ out_vid)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const float2 p = load_pt2(pts, q);
    const bool flip = flips ? __ldg(flips + q) != 0 : false;
    float best = INFINITY;
    int32_t bv = -1;
    if (t.n == 1)
    {
        float d = INFINITY;
        int32_t v = -1;
        if (leaf_silhouette2(t, t.nodes[0].object, p, best * best, d, flip, v) && d <= best)
        {
            best = d;
            bv = v;
        }
    }
    else if (t.n > 1)
    {
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        sn[sp] = 0;
        sd[sp++] = mindist2(node_box2(t, 0), p);
        do
        {
            --sp;
            const uint32_t node = sn[sp];
            if (sd[sp] > best * best)
                continue;
            const uint32_t ch[2] = {t.nodes[node].left, t.nodes[node].right};
            for (int k = 0; k < 2; ++k)
            {
                const B2 b = node_box2(t, ch[k]);
                const C2 c = node_cone2(t, ch[k]);
                const float md = mindist2(b, p);
                if (!(c.half_angle >= 0.0f && cone_overlap2(c, p, b, md)))
                    continue;
                const uint32_t obj = t.nodes[ch[k]].object;
                if (obj != kInvalid)
                {
                    float d = INFINITY;
                    int32_t v = -1;
                    if (leaf_silhouette2(t, obj, p, best * best, d, flip, v) && d <= best)
                    {
                        best = d;
                        bv = v;
                    }
                }
                else
                {
                    if (sp >= kStackDepth)
                    {
                        atomicOr(t.status, kStatusStackOverflow);
                        out_dist[q] = NAN;
                        if (out_vid)
                            out_vid[q] = -1;
                        return;
                    }
                    sn[sp] = ch[k];
                    sd[sp++] = md;
                }
            }
        } while (sp > 0);
    }
    out_dist[q] = best;
    if (out_vid)
        out_vid[q] = bv;
}

// intersects_d(ray<float,2>) aabb.cuh:366-390
SNCH_DEV bool ray_box2(float2 o, float2 inv, const B2 &b, float max_dist, float &dist)
{
    float t1 = (b.lower.x - o.x) * inv.x, t2 = (b.upper.x - o.x) * inv.x;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b.lower.y - o.y) * inv.y;
    t2 = (b.upper.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    if (tmax >= tmin && tmax >= 0.0f && tmin <= max_dist)
    {
        dist = tmin >= 0.0f ? tmin : 0.0f;
        return true;
    }
    return false;
}
// scene<2>::intersect_test scene.cuh:555-583
SNCH_DEV bool ray_segment(float2 o, float2 dir, float2 p0, float2 p1, float &t, float &s)
{
    const float2 sd = sub2(p1, p0);
    const float D = dir.x * (-sd.y) + dir.y * sd.x;
    if (fabsf(D) < kEps)
        return false;
    const float inv = __frcp_rn(D);
    const float tt = ((p0.x - o.x) * (-sd.y) - (p0.y - o.y) * (-sd.x)) * inv;
    const float ss = (dir.x * (p0.y - o.y) - dir.y * (p0.x - o.x)) * inv;
    if (ss >= -1e-3f && ss <= 1.0f + 1e-3f && tt >= 0.0f)
    {
        t = tt;
        s = ss;
        return true;
    }
    return false;
}
// query_device(ray_intersect) query.cuh:82-169 over segments, the reference's order;
// kAny: TestOnly = true (query.cuh:117-121), stop at the first accepted hit and
// write only the hit flag
template <bool kAny = false>
__global__ void __launch_bounds__(128) ray2_kernel(Tree2 t, const float *__restrict__ origins,
                                                   const float *__restrict__ dirs, const float *__restrict__ tmaxs,
                                                   int64_t n, uint8_t *__restrict__ out_hit, float *__restrict__ out_t,
                                                   float *__restrict__ out_s, uint32_t *__restrict__ out_idx)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const float2 o = load_pt2(origins, q), dir = load_pt2(dirs, q);
    const float2 inv = f2(1.0f / dir.x, 1.0f / dir.y);
    const float max_dist = __ldg(tmaxs + q);
    float min_dist = INFINITY, bs = 0.0f;
    bool found = false;
    uint32_t nearest = kInvalid;
    if (t.n > 0)
    {
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        sn[sp] = 0;
        sd[sp++] = INFINITY;
        do
        {
            --sp;
            const uint32_t node = sn[sp];
            if (sd[sp] > min_dist)
                continue;
            const uint32_t obj = t.nodes[node].object;
            if (obj != kInvalid)
            {
                float tt, ss;
                if (ray_segment(o, dir, vload2(t.verts, t.segs[2 * obj]), vload2(t.verts, t.segs[2 * obj + 1]), tt,
                                ss) &&
                    tt < max_dist && tt < min_dist)
                {
                    min_dist = tt;
                    found = true;
                    bs = ss;
                    nearest = obj;
                    if (kAny)
                        break;
                }
                continue;
            }
            const uint32_t L = t.nodes[node].left, R = t.nodes[node].right;
            float Ld = 0.0f, Rd = 0.0f;
            const bool Lh = ray_box2(o, inv, node_box2(t, L), max_dist, Ld);
            const bool Rh = ray_box2(o, inv, node_box2(t, R), max_dist, Rd);
            if (sp > kStackDepth - 2)
            {
                atomicOr(t.status, kStatusStackOverflow);
                found = false;
                nearest = kInvalid;
                min_dist = NAN;
                break;
            }
            if (Lh && Rh)
            {
                uint32_t closer = L, other = R;
                if (Rd < Ld)
                {
                    const float tmp = Ld;
                    Ld = Rd;
                    Rd = tmp;
                    closer = R;
                    other = L;
                }
                sn[sp] = other;
                sd[sp++] = Rd;
                sn[sp] = closer;
                sd[sp++] = Ld;
            }
            else if (Lh)
            {
                sn[sp] = L;
                sd[sp++] = Ld;
            }
            else if (Rh)
            {
                sn[sp] = R;
                sd[sp++] = Rd;
            }
        } while (sp > 0);
    }
    out_hit[q] = found ? 1 : 0;
    if (kAny)
        return;
    out_t[q] = min_dist;
    out_s[q] = bs;
    out_idx[q] = nearest;
}

// intersect_sphere(sphere<float,2>, aabb) aabb.cuh:433-449
SNCH_DEV bool circle_box(float2 c, float r, const B2 &b)
{
    const float cx = smax(b.lower.x, smin(c.x, b.upper.x)), cy = smax(b.lower.y, smin(c.y, b.upper.y));
    const float dx = cx - c.x, dy = cy - c.y;
    return dx * dx + dy * dy <= (r * r);
}
// scene<2>::intersect_sphere scene.cuh:585-608
SNCH_DEV bool circle_segment(float2 c, float radius, float2 p1, float2 p2)
{
    const float2 d = sub2(p2, p1);
    const float len_sq = d.x * d.x + d.y * d.y;
    float t = ((c.x - p1.x) * d.x + (c.y - p1.y) * d.y) / len_sq;
    t = smax(0.0f, smin(1.0f, t));
    const float dx = (p1.x + t * d.x) - c.x, dy = (p1.y + t * d.y) - c.y;
    return dx * dx + dy * dy <= (radius * radius);
}
// scene<2>::green_weight scene.cuh:610-617
SNCH_DEV float green_weight2(float2 x, float2 y)
{
    const float r = smax(len2(f2(x.x - y.x, x.y - y.y)), 1e-2f);
    return fabsf(logf(r) / (3.14159265358979323846f * 2.0f));
}
// sample_object_in_sphere sample.cuh:23-91 over segments (measurement_getter:
// segment length); pdf 0 where the reference leaves it unset
__global__ void __launch_bounds__(128) sample2_kernel(Tree2 t, const float *__restrict__ centers,
                                                      const float *__restrict__ radii, const float *__restrict__ us,
                                                      int64_t n, int32_t *__restrict__ out_idx,
                                                      float *__restrict__ out_pdf)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const float2 ctr = load_pt2(centers, q);
    const float rad = __ldg(radii + q);
    float u = __ldg(us + q);
    int32_t oi = -1;
    float opdf = 0.0f;
    if (t.n > 0)
    {
        uint32_t node = 0;
        float npdf = 1.0f;
        for (int level = 0; level < 128; ++level)
        {
            const uint32_t obj = t.nodes[node].object;
            if (obj != kInvalid)
            {
                const float2 p0 = vload2(t.verts, t.segs[2 * obj]), p1 = vload2(t.verts, t.segs[2 * obj + 1]);
                if (circle_segment(ctr, rad, p0, p1))
                {
                    oi = (int32_t)obj;
                    opdf = npdf;
                    opdf /= len2(f2(p0.x - p1.x, p0.y - p1.y));
                }
                break;
            }
            const uint32_t L = t.nodes[node].left, R = t.nodes[node].right;
            const B2 lb = node_box2(t, L), rb = node_box2(t, R);
            const float Lw = circle_box(ctr, rad, lb) ? green_weight2(ctr, centroid2(lb)) : 0.0f;
            const float Rw = circle_box(ctr, rad, rb) ? green_weight2(ctr, centroid2(rb)) : 0.0f;
            const float tw = Lw + Rw;
            if (!(tw > 0.0f))
                break;
            const float Lp = Lw / tw;
            if (u < Lp)
            {
                u /= Lp;
                node = L;
                npdf = Lp * npdf;
            }
            else
            {
                const float Rp = 1.0f - Lp;
                u = (u - Lp) / Rp;
                node = R;
                npdf = Rp * npdf;
            }
        }
    }
    out_idx[q] = oi;
    out_pdf[q] = opdf;
}
// sample_on_object scene.cuh:619-623 -> sample_line scene.cuh:29-32
__global__ void sample_point2_kernel(const float *verts, const int32_t *segs, uint32_t ns, const int32_t *idx,
                                     const float *u, int64_t n, float *out)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const int32_t i = idx[q];
    if (i < 0 || (uint32_t)i >= ns)
    {
        out[2 * q] = NAN;
        out[2 * q + 1] = NAN;
        return;
    }
    const float2 pa = vload2(verts, segs[2 * i]), pb = vload2(verts, segs[2 * i + 1]);
    const float uu = u[q];
    out[2 * q] = pa.x + uu * (pb.x - pa.x);
    out[2 * q + 1] = pa.y + uu * (pb.y - pa.y);
}

inline unsigned blocks(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace
}  // namespace snch

using namespace snch;

struct snch_scene2_s
{
    uint32_t nv = 0, n = 0;
    float *verts = nullptr;
    int32_t *segs = nullptr;
    int4 *sv = nullptr;
    int2 *seg_owned = nullptr;
    int32_t *topo = nullptr;  // 3 x nv: last segment starting / ending at, first touching each vertex
    float4 *leaf_box = nullptr, *leaf_cone = nullptr, *aabbs = nullptr, *cones = nullptr;
    uint32_t *keys = nullptr, *vals = nullptr, *keys_tmp = nullptr, *vals_tmp = nullptr, *flags = nullptr,
             *sizes = nullptr, *small = nullptr;
    NodeRec *nodes = nullptr;
    void *scratch = nullptr;
    bool built = false;
    Tree2 tree() const
    {
        return Tree2{n, verts, segs, sv, seg_owned, nodes, aabbs, cones, small + 8};
    }
};

namespace
{
#define SNCH2_CUDA(expr)                                                                                 \
    do                                                                                                   \
    {                                                                                                    \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return report_error(e_ == cudaErrorMemoryAllocation ? SNCH_ERR_OUT_OF_MEMORY : SNCH_ERR_CUDA, \
                                std::string(#expr) + ": " + cudaGetErrorString(e_));                     \
    } while (0)

inline cudaStream_t S2(snch_stream_t s) { return static_cast<cudaStream_t>(s); }

void free2(snch_scene2_s *s)
{
    void *ptrs[] = {s->verts, s->segs, s->sv, s->seg_owned, s->topo, s->leaf_box, s->leaf_cone, s->aabbs,
                    s->cones, s->keys, s->vals, s->keys_tmp, s->vals_tmp, s->flags, s->sizes, s->small,
                    s->nodes, s->scratch};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    delete s;
}
template <typename T>
cudaError_t dalloc2(T **p, size_t count)
{
    return cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * (count ? count : 1));
}
int check2(snch_scene2_t s, int64_t n, std::initializer_list<const void *> ptrs)
{
    if (!s)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (!s->built)
        return report_error(SNCH_ERR_NOT_BUILT, "BVH is not built yet.");
    if (n < 0)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "negative query count");
    if (n > 0)
        for (const void *p : ptrs)
            if (!p)
                return report_error(SNCH_ERR_INVALID_ARGUMENT, "NULL query buffer");
    return SNCH_OK;
}
}  // namespace

extern "C" {

int snch_scene2_create(const float *verts_xy, int64_t nv, const int32_t *segs, int64_t ns, snch_scene2_t *out)
{
    if (!out)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "out_scene is NULL");
    *out = nullptr;
    if (nv < 0 || ns < 0 || (nv > 0 && !verts_xy) || (ns > 0 && !segs))
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "bad vertex or segment buffer");
    if (ns >= (int64_t(1) << 30) || nv >= (int64_t(1) << 31))
        return report_error(SNCH_ERR_TOO_LARGE, "at most 2^30 - 1 segments and 2^31 - 1 vertices are supported");
    for (int64_t i = 0; i < 2 * ns; ++i)
        if (segs[i] < 0 || segs[i] >= nv)
            return report_error(SNCH_ERR_INVALID_ARGUMENT,
                                "segment vertex index out of range at segment " + std::to_string(i / 2));
    snch_scene2_s *s = new snch_scene2_s();
    s->nv = (uint32_t)nv;
    s->n = (uint32_t)ns;
    const size_t n = s->n, nn = n ? 2 * n - 1 : 1;
    cudaError_t e = cudaSuccess;
    auto A = [&](cudaError_t x) {
        if (e == cudaSuccess)
            e = x;
    };
    A(dalloc2(&s->verts, 2 * (size_t)nv));
    A(dalloc2(&s->segs, 2 * n));
    A(dalloc2(&s->sv, (size_t)nv));
    A(dalloc2(&s->seg_owned, n));
    A(dalloc2(&s->topo, 3 * (size_t)nv));
    A(dalloc2(&s->leaf_box, n));
    A(dalloc2(&s->leaf_cone, n));
    A(dalloc2(&s->aabbs, nn));
    A(dalloc2(&s->cones, nn));
    A(dalloc2(&s->keys, n));
    A(dalloc2(&s->vals, n));
    A(dalloc2(&s->keys_tmp, n));
    A(dalloc2(&s->vals_tmp, n));
    A(dalloc2(&s->flags, n));
    A(dalloc2(&s->sizes, n));
    A(dalloc2(&s->small, 1056));
    A(dalloc2(&s->nodes, nn));
    if (e == cudaSuccess)
        e = cudaMalloc(&s->scratch, std::max<size_t>(sort_scratch_bytes((uint32_t)std::max<size_t>(n, 1), 30), 256));
    if (e == cudaSuccess)
        e = cudaMemset(s->small, 0, 1056 * 4);
    if (e == cudaSuccess && nv)
        e = cudaMemcpy(s->verts, verts_xy, 8 * (size_t)nv, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n)
        e = cudaMemcpy(s->segs, segs, 8 * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
    {
        free2(s);
        return report_error(e == cudaErrorMemoryAllocation ? SNCH_ERR_OUT_OF_MEMORY : SNCH_ERR_CUDA,
                            std::string("2D scene: ") + cudaGetErrorString(e));
    }
    *out = s;
    return SNCH_OK;
}

int snch_scene2_destroy(snch_scene2_t s)
{
    if (!s)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    free2(s);
    return SNCH_OK;
}

int snch_scene2_build(snch_scene2_t s, snch_stream_t stream)
{
    if (!s)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    cudaStream_t st = S2(stream);
    const uint32_t n = s->n, nv = s->nv;
    int32_t *last_start = s->topo, *last_end = s->topo + nv, *first_ref = s->topo + 2 * (size_t)nv;
    if (nv)
    {
        topo2_init_kernel<<<blocks(nv, 256), 256, 0, st>>>(nv, last_start, last_end, first_ref);
        note_launch();
    }
    if (n)
    {
        topo2_scan_kernel<<<blocks(n, 256), 256, 0, st>>>(s->segs, n, last_start, last_end, first_ref);
        topo2_owned_kernel<<<blocks(n, 256), 256, 0, st>>>(s->segs, n, first_ref, s->seg_owned);
        note_launch(2);
    }
    if (nv)
    {
        topo2_vertex_kernel<<<blocks(nv, 256), 256, 0, st>>>(s->segs, nv, last_start, last_end, s->sv);
        note_launch();
    }
    SNCH2_CUDA(cudaGetLastError());
    if (n)
    {
        Build2 a{n, s->verts, s->segs, s->sv, s->seg_owned, s->small, s->leaf_box, s->leaf_cone, s->keys, s->vals,
                 s->nodes, s->aabbs, s->cones, s->flags};
        init2_kernel<<<1, 32, 0, st>>>(s->small);
        leaf2_kernel<<<blocks(n, 256), 256, 0, st>>>(a);
        morton2_kernel<<<blocks(n, 256), 256, 0, st>>>(a);
        note_launch(3);
        SNCH2_CUDA(cudaGetLastError());
        SNCH2_CUDA(radix_sort_pairs(s->keys, s->vals, s->keys_tmp, s->vals_tmp, n, 30, nullptr, s->scratch,
                                    s->small + 8, st));
        BuildArgs k{};
        k.num_tris = n;
        k.keys = s->keys;
        k.vals = s->vals;
        k.nodes = s->nodes;
        k.sizes = s->sizes;
        SNCH2_CUDA(launch_karras(k, st));
        if (n > 1)
            SNCH2_CUDA(cudaMemsetAsync(s->flags, 0, 4 * (size_t)(n - 1), st));
        refit2_kernel<<<blocks(n, 128), 128, 0, st>>>(a);
        note_launch();
        SNCH2_CUDA(cudaGetLastError());
    }
    s->built = true;
    return SNCH_OK;
}

int snch_scene2_get_device_status(snch_scene2_t s, uint32_t *out_bits, int reset, snch_stream_t stream)
{
    if (!s || !out_bits)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "scene and out_bits are required");
    SNCH2_CUDA(cudaMemcpyAsync(out_bits, s->small + 8, 4, cudaMemcpyDeviceToHost, S2(stream)));
    SNCH2_CUDA(cudaStreamSynchronize(S2(stream)));
    if (reset)
        SNCH2_CUDA(cudaMemsetAsync(s->small + 8, 0, 4, S2(stream)));
    return SNCH_OK;
}

int snch_scene2_export(snch_scene2_t s, int32_t *sv, int32_t *seg_owned, uint32_t *sorted_morton,
                       uint32_t *sorted_idx, uint32_t *nodes, float *aabbs, float *cones, snch_stream_t stream)
{
    int rc = check2(s, 0, {});
    if (rc != SNCH_OK)
        return rc;
    cudaStream_t st = S2(stream);
    const size_t n = s->n, nn = n ? 2 * n - 1 : 0;
    const auto cp = [&](void *dst, const void *src, size_t bytes) {
        return dst && bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st) : cudaSuccess;
    };
    SNCH2_CUDA(cp(sv, s->sv, 16 * (size_t)s->nv));
    SNCH2_CUDA(cp(seg_owned, s->seg_owned, 8 * n));
    SNCH2_CUDA(cp(sorted_morton, s->keys, 4 * n));
    SNCH2_CUDA(cp(sorted_idx, s->vals, 4 * n));
    SNCH2_CUDA(cp(nodes, s->nodes, 16 * nn));
    SNCH2_CUDA(cp(aabbs, s->aabbs, 16 * nn));
    SNCH2_CUDA(cp(cones, s->cones, 16 * nn));
    return SNCH_OK;
}

int snch_scene2_query_nearest(snch_scene2_t s, const float *pts, int64_t n, uint32_t *idx, float *dist,
                              snch_stream_t stream)
{
    int rc = check2(s, n, {pts, idx, dist});
    if (rc != SNCH_OK || n == 0)
        return rc;
    nearest2_kernel<<<blocks(n, 128), 128, 0, S2(stream)>>>(s->tree(), pts, n, idx, dist);
    note_launch();
    SNCH2_CUDA(cudaGetLastError());
    return SNCH_OK;
}

int snch_scene2_query_silhouette(snch_scene2_t s, const float *pts, const uint8_t *flip, int64_t n, float *dist,
                                 int32_t *vertex, snch_stream_t stream)
{
    int rc = check2(s, n, {pts, dist});
    if (rc != SNCH_OK || n == 0)
        return rc;
    silhouette2_kernel<<<blocks(n, 128), 128, 0, S2(stream)>>>(s->tree(), pts, flip, n, dist, vertex);
    note_launch();
    SNCH2_CUDA(cudaGetLastError());
    return SNCH_OK;
}

int snch_scene2_query_ray(snch_scene2_t s, const float *origins, const float *dirs, const float *tmax, int64_t n,
                          uint8_t *hit, float *t, float *seg_param, uint32_t *idx, snch_stream_t stream)
{
    int rc = check2(s, n, {origins, dirs, tmax, hit, t, seg_param, idx});
    if (rc != SNCH_OK || n == 0)
        return rc;
    ray2_kernel<<<blocks(n, 128), 128, 0, S2(stream)>>>(s->tree(), origins, dirs, tmax, n, hit, t, seg_param, idx);
    note_launch();
    SNCH2_CUDA(cudaGetLastError());
    return SNCH_OK;
}

int snch_scene2_query_ray_test(snch_scene2_t s, const float *origins, const float *dirs, const float *tmax,
                               int64_t n, uint8_t *hit, snch_stream_t stream)
{
    int rc = check2(s, n, {origins, dirs, tmax, hit});
    if (rc != SNCH_OK || n == 0)
        return rc;
    ray2_kernel<true><<<blocks(n, 128), 128, 0, S2(stream)>>>(s->tree(), origins, dirs, tmax, n, hit, nullptr,
                                                               nullptr, nullptr);
    note_launch();
    SNCH2_CUDA(cudaGetLastError());
    return SNCH_OK;
}

int snch_scene2_sample_in_circle(snch_scene2_t s, const float *centers, const float *radii, const float *u, int64_t n,
                                 int32_t *idx, float *pdf, snch_stream_t stream)
{
    int rc = check2(s, n, {centers, radii, u, idx, pdf});
    if (rc != SNCH_OK || n == 0)
        return rc;
    sample2_kernel<<<blocks(n, 128), 128, 0, S2(stream)>>>(s->tree(), centers, radii, u, n, idx, pdf);
    note_launch();
    SNCH2_CUDA(cudaGetLastError());
    return SNCH_OK;
}

int snch_scene2_sample_on_object(snch_scene2_t s, const int32_t *idx, const float *u, int64_t n, float *pts,
                                 snch_stream_t stream)
{
    int rc = check2(s, n, {idx, u, pts});
    if (rc != SNCH_OK || n == 0)
        return rc;
    sample_point2_kernel<<<blocks(n, 256), 256, 0, S2(stream)>>>(s->verts, s->segs, s->n, idx, u, n, pts);
    note_launch();
    SNCH2_CUDA(cudaGetLastError());
    return SNCH_OK;
}

}  // extern "C"
