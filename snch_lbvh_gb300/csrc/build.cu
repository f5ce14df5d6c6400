// LBVH construction kernels (replaces bvh::construct, include/snch_lbvh/core/bvh.cuh:380-613).
//
//   leaf_bounds_kernel  leaf AABB per triangle (scene.cuh:870-885), its centroid,
//                       block-reduced scene AABB (bvh.cuh:428-432) via ordered atomics
//   morton_kernel       30-bit codes (bvh.cuh:292-302, morton_code.cuh:19-70) and the
//                       digit histograms of all four radix passes in the same read
//   [radix_sort_pairs]  stable onesweep sort of (code, triangle index), scan_sort.cu
//   karras_kernel       internal nodes (bvh.cuh:109-229) with the reference's node
//                       numbering; ties of equal codes broken by the sorted object
//                       index exactly as the 64-bit (code << 32 | idx) keys do
//   refit_kernel        one bottom-up pass per leaf with atomic arrival counters that
//                       merges AABBs (bvh.cuh:520-554) AND normal cones (bvh.cuh:559-604,
//                       cone.cuh:427-480) and packs the 64-B traversal records
#include <algorithm>

#include "internal.h"

namespace snch
{


// aabb(p) aabb.cuh:21-50 + expand_to_include aabb.cuh:94-101 (scene.cuh:870-885)
SNCH_DEV Box tri_box(f3 pa, f3 pb, f3 pc)
{
    Box b;
    b.upper = mk(pa.x + kEps, pa.y + kEps, pa.z + kEps);
    b.lower = mk(pa.x - kEps, pa.y - kEps, pa.z - kEps);
    const f3 q[2] = {pb, pc};
#pragma unroll
    for (int k = 0; k < 2; ++k)
    {
        const f3 pl = mk(q[k].x - kEps, q[k].y - kEps, q[k].z - kEps);
        const f3 pu = mk(q[k].x + kEps, q[k].y + kEps, q[k].z + kEps);
        b.lower = mk(fminf(b.lower.x, pl.x), fminf(b.lower.y, pl.y), fminf(b.lower.z, pl.z));
        b.upper = mk(fmaxf(b.upper.x, pu.x), fmaxf(b.upper.y, pu.y), fmaxf(b.upper.z, pu.z));
    }
    return b;
}

// expand_bits morton_code.cuh:19-38, morton_code(float3, 1024) morton_code.cuh:61-70
SNCH_DEV uint32_t expand_bits(uint32_t v)
{
    v = (v | (v << 16)) & 0x070000FFu;
    v = (v | (v << 8)) & 0x0700F00Fu;
    v = (v | (v << 4)) & 0x430C30C3u;
    v = (v | (v << 2)) & 0x49249249u;
    return v;
}
SNCH_DEV uint32_t morton3(f3 p)
{
    const float res = 1024.0f;
    p.x = fminf(fmaxf(p.x * res, 0.0f), res - 1.0f);
    p.y = fminf(fmaxf(p.y * res, 0.0f), res - 1.0f);
    p.z = fminf(fmaxf(p.z * res, 0.0f), res - 1.0f);
    return expand_bits((uint32_t)p.x) * 4 + expand_bits((uint32_t)p.y) * 2 + expand_bits((uint32_t)p.z);
}

__global__ void init_build_kernel(uint32_t *scene_box, uint32_t *hist)
{
    const int t = threadIdx.x;
    if (t < 3)
        scene_box[t] = float_to_ordered(-INFINITY);
    else if (t < 6)
        scene_box[t] = float_to_ordered(INFINITY);
    for (int i = t; i < 4 * 256; i += blockDim.x)
        hist[i] = 0;
}

__global__ void __launch_bounds__(256) leaf_bounds_kernel(BuildArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    Box b;
    b.upper = mk(-INFINITY, -INFINITY, -INFINITY);
    b.lower = mk(INFINITY, INFINITY, INFINITY);
    if (i < a.num_tris)
    {
        const int32_t *t = a.tris + 3 * (uint64_t)i;
        b = tri_box(load_vert(a.verts, __ldg(t)), load_vert(a.verts, __ldg(t + 1)), load_vert(a.verts, __ldg(t + 2)));
        const f3 c = centroid(b);
        a.centroids[i] = make_float4(c.x, c.y, c.z, 0.0f);
    }
    float v[6] = {b.upper.x, b.upper.y, b.upper.z, b.lower.x, b.lower.y, b.lower.z};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
#pragma unroll
        for (int c = 0; c < 6; ++c)
        {
            const float w = __shfl_xor_sync(0xffffffffu, v[c], o);
            v[c] = c < 3 ? fmaxf(v[c], w) : fminf(v[c], w);
        }
    }
    __shared__ float s[8][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // batched scenes: a block whose triangles all belong to one mesh reduces into
    // that mesh's box; a block straddling meshes adds each triangle on its own
    uint32_t *box = a.scene_box;
    if (a.num_meshes)
    {
        const uint32_t first = blockIdx.x * blockDim.x;
        const uint32_t last = min(first + blockDim.x, a.num_tris) - 1;
        const uint32_t m0 = __ldg(a.tri_mesh + first), m1 = __ldg(a.tri_mesh + last);
        if (m0 != m1)
        {
            if (i < a.num_tris)
            {
                uint32_t *mb = a.mesh_box + 6 * (uint64_t)__ldg(a.tri_mesh + i);
                const float w[6] = {b.upper.x, b.upper.y, b.upper.z, b.lower.x, b.lower.y, b.lower.z};
                for (int c = 0; c < 6; ++c)
                    if (c < 3)
                        atomicMax(mb + c, float_to_ordered(w[c]));
                    else
                        atomicMin(mb + c, float_to_ordered(w[c]));
            }
            return;
        }
        box = a.mesh_box + 6 * (uint64_t)m0;
    }
    if (lane == 0)
        for (int c = 0; c < 6; ++c)
            s[warp][c] = v[c];
    __syncthreads();
    if (threadIdx.x < 6)
    {
        const int c = threadIdx.x;
        float r = s[0][c];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            r = c < 3 ? fmaxf(r, s[w][c]) : fminf(r, s[w][c]);
        if (c < 3)
            atomicMax(box + c, float_to_ordered(r));
        else
            atomicMin(box + c, float_to_ordered(r));
    }
}

// batched scenes: empty per-mesh boxes, no mesh roots yet, no first edge yet
__global__ void init_mesh_kernel(uint32_t *mesh_box, uint32_t *mesh_root, int32_t *mesh_edge_start,
                                 uint32_t num_meshes)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= num_meshes)
        return;
    for (int c = 0; c < 3; ++c)
    {
        mesh_box[6 * (uint64_t)m + c] = float_to_ordered(-INFINITY);
        mesh_box[6 * (uint64_t)m + 3 + c] = float_to_ordered(INFINITY);
    }
    mesh_root[m] = kInvalid;
    mesh_edge_start[m] = 0x7FFFFFFF;
}

// first silhouette edge id of each mesh: edge ids are handed out in triangle
// order, so a mesh's edges are the ids from its smallest one on
__global__ void mesh_edges_kernel(const int32_t *__restrict__ tri_edges, const uint32_t *__restrict__ tri_mesh,
                                  uint32_t n, int32_t *mesh_edge_start)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int32_t e = 0x7FFFFFFF;
    for (int k = 0; k < 3; ++k)
    {
        const int32_t x = __ldg(tri_edges + 3 * (uint64_t)i + k);
        if (x >= 0 && x < e)
            e = x;
    }
    if (e != 0x7FFFFFFF)
        atomicMin(mesh_edge_start + __ldg(tri_mesh + i), e);
}

// batched scene set-up: mesh of every triangle (binary search of the mesh
// starts), and the triangles' per-mesh vertex indices made batch-wide; counts
// indices outside their own mesh's vertex range
__global__ void mesh_setup_kernel(const uint32_t *__restrict__ tri_start, const int64_t *__restrict__ vert_start,
                                  uint32_t num_meshes, uint32_t n, uint32_t *__restrict__ tri_mesh,
                                  int32_t *__restrict__ tris, uint32_t *bad)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t lo = 0, hi = num_meshes;  // last m with tri_start[m] <= i
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(tri_start + mid) <= i)
            lo = mid;
        else
            hi = mid;
    }
    while (lo + 1 < num_meshes && __ldg(tri_start + lo + 1) <= i)  // empty meshes share a start
        ++lo;
    tri_mesh[i] = lo;
    const int64_t v0 = vert_start[lo], nv = vert_start[lo + 1] - v0;
    uint32_t b = 0;
    for (int k = 0; k < 3; ++k)
    {
        const int32_t v = tris[3 * (uint64_t)i + k];
        b += (v < 0 || v >= nv) ? 1u : 0u;
        tris[3 * (uint64_t)i + k] = (int32_t)(v0 + v);
    }
    if (b)
        atomicAdd(bad, b);
}

// default_morton_code_calculator<Real,3> bvh.cuh:281-304
__global__ void __launch_bounds__(256) morton_kernel(BuildArgs a)
{
    __shared__ uint32_t s_hist[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
        (&s_hist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.num_tris)
    {
        const uint32_t *box = a.num_meshes ? a.mesh_box + 6 * (uint64_t)__ldg(a.tri_mesh + i) : a.scene_box;
        const f3 upper = mk(ordered_to_float(box[0]), ordered_to_float(box[1]), ordered_to_float(box[2]));
        const f3 lower = mk(ordered_to_float(box[3]), ordered_to_float(box[4]), ordered_to_float(box[5]));
        const float4 c = a.centroids[i];
        f3 p = mk(c.x, c.y, c.z);
        p.x -= lower.x;
        p.y -= lower.y;
        p.z -= lower.z;
        p.x /= (upper.x - lower.x);
        p.y /= (upper.y - lower.y);
        p.z /= (upper.z - lower.z);
        const uint32_t code = morton3(p);
        a.keys[i] = code;
        a.vals[i] = i;
#pragma unroll
        for (int d = 0; d < 4; ++d)
            atomicAdd(&s_hist[d][(code >> (8 * d)) & 255u], 1u);
    }
    __syncthreads();
    for (int i2 = threadIdx.x; i2 < 4 * 256; i2 += blockDim.x)
    {
        const uint32_t c = (&s_hist[0][0])[i2];
        if (c)
            atomicAdd(a.hist + i2, c);
    }
}

// common_upper_bits on the 64-bit key (code << 32 | sorted object index):
// equal to the reference's 32-bit path whenever the codes are unique
// (bvh.cuh:505-515, morton_code.cuh:144-167)
// Batched scenes compare (mesh id : 16 bits, code, index within the mesh): keys
// of different meshes share fewer than 16 leading bits, keys of one mesh 16 +
// their single-mesh value, so inside a mesh every comparison the build makes
// comes out as in a build of that mesh alone, and a mesh boundary acts like
// the end of the array.
struct KeyView
{
    const uint32_t *k;      // codes, sorted
    const uint32_t *s;      // original triangle index of each sorted position
    const uint32_t *m;      // mesh of each sorted position (nullptr: one mesh)
    const uint32_t *start;  // first triangle of each mesh
};
SNCH_DEV int delta(const KeyView &v, uint32_t a, uint32_t b)
{
    const uint32_t x = __ldg(v.k + a) ^ __ldg(v.k + b);
    if (!v.m)
        return x ? __clz(x) : 32 + __clz(__ldg(v.s + a) ^ __ldg(v.s + b));
    const uint32_t ma = __ldg(v.m + a), mb = __ldg(v.m + b);
    if (ma != mb)
        return __clz(ma ^ mb) - 16;
    const uint32_t st = __ldg(v.start + ma);
    return 16 + (x ? __clz(x) : 32 + __clz((__ldg(v.s + a) - st) ^ (__ldg(v.s + b) - st)));
}

// determine_range bvh.cuh:109-167 (unsigned index arithmetic as in the reference)
SNCH_DEV void determine_range(const KeyView &kv, uint32_t n, uint32_t idx, uint32_t &lo, uint32_t &hi)
{
    if (idx == 0)
    {
        lo = 0;
        hi = n - 1;
        return;
    }
    const int L_delta = delta(kv, idx, idx - 1);
    const int R_delta = delta(kv, idx, idx + 1);
    const int d = (R_delta > L_delta) ? 1 : -1;
    const int delta_min = L_delta < R_delta ? L_delta : R_delta;
    int l_max = 2;
    int dl = -1;
    int i_tmp = (int)(idx + (uint32_t)(d * l_max));
    if (0 <= i_tmp && (uint32_t)i_tmp < n)
        dl = delta(kv, idx, (uint32_t)i_tmp);
    while (dl > delta_min)
    {
        l_max <<= 1;
        i_tmp = (int)(idx + (uint32_t)(d * l_max));
        dl = -1;
        if (0 <= i_tmp && (uint32_t)i_tmp < n)
            dl = delta(kv, idx, (uint32_t)i_tmp);
    }
    int l = 0;
    int t = l_max >> 1;
    while (t > 0)
    {
        i_tmp = (int)(idx + (uint32_t)((l + t) * d));
        dl = -1;
        if (0 <= i_tmp && (uint32_t)i_tmp < n)
            dl = delta(kv, idx, (uint32_t)i_tmp);
        if (dl > delta_min)
            l += t;
        t >>= 1;
    }
    uint32_t jdx = idx + (uint32_t)(l * d);
    if (d < 0)
    {
        const uint32_t tmp = idx;
        idx = jdx;
        jdx = tmp;
    }
    lo = idx;
    hi = jdx;
}

// find_split bvh.cuh:169-199
SNCH_DEV uint32_t find_split(const KeyView &kv, uint32_t first, uint32_t last)
{
    if (first == last)
        return first;
    const int delta_node = delta(kv, first, last);
    int split = (int)first;
    int stride = (int)(last - first);
    do
    {
        stride = (stride + 1) >> 1;
        const int middle = split + stride;
        if ((uint32_t)middle < last)
        {
            if (delta(kv, first, (uint32_t)middle) > delta_node)
                split = middle;
        }
    } while (stride > 1);
    return (uint32_t)split;
}

// construct_internal_nodes bvh.cuh:200-229 + leaf records bvh.cuh:489-499
__global__ void __launch_bounds__(256) karras_kernel(BuildArgs a)
{
    const uint32_t n = a.num_tris, ni = n - 1;
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n)
        return;
    NodeRec *nodes = a.nodes;
    // leaf of sorted position idx
    nodes[ni + idx].left = kInvalid;
    nodes[ni + idx].right = kInvalid;
    nodes[ni + idx].object = a.vals[idx];
    if (idx == 0)
        nodes[0].parent = kInvalid;
    if (a.num_meshes)
    {
        // a one-triangle mesh: its root is its leaf
        const uint32_t m = __ldg(a.sorted_mesh + idx);
        if ((idx == 0 || __ldg(a.sorted_mesh + idx - 1) != m) && (idx == n - 1 || __ldg(a.sorted_mesh + idx + 1) != m))
            a.mesh_root[m] = ni + idx;
    }
    if (idx >= ni)
        return;
    uint32_t lo, hi;
    const KeyView kv{a.keys, a.vals, a.num_meshes ? a.sorted_mesh : nullptr, a.mesh_tri_start};
    determine_range(kv, n, idx, lo, hi);
    const uint32_t gamma = find_split(kv, lo, hi);
    if (a.num_meshes)
    {
        // the internal node covering exactly one mesh is that mesh's root
        const uint32_t m = __ldg(a.sorted_mesh + lo);
        if (__ldg(a.sorted_mesh + hi) == m && (lo == 0 || __ldg(a.sorted_mesh + lo - 1) != m) &&
            (hi == n - 1 || __ldg(a.sorted_mesh + hi + 1) != m))
            a.mesh_root[m] = idx;
    }
    uint32_t left = gamma, right = gamma + 1;
    if ((lo < hi ? lo : hi) == gamma)
        left += ni;
    if ((lo > hi ? lo : hi) == gamma + 1)
        right += ni;
    nodes[idx].left = left;
    nodes[idx].right = right;
    nodes[idx].object = kInvalid;
    a.sizes[idx] = hi - lo + 1;
    nodes[left].parent = idx;
    nodes[right].parent = idx;
}

// silhouette_edge::normal(f, normalize) scene.cuh:745-771
SNCH_DEV f3 edge_face_normal(const float *verts, const int4 &se, int f, bool do_normalize)
{
    int32_t vi, vj, vk;
    if (f == 0)
    {
        vi = se.w;
        vj = se.y;
        vk = se.z;
    }
    else
    {
        vi = se.x;
        vj = se.z;
        vk = se.y;
    }
    const f3 pa = load_vert(verts, vj), pb = load_vert(verts, vk), pc = load_vert(verts, vi);
    const f3 n = cross3(sub(pb, pa), sub(pc, pa));
    return do_normalize ? normalize3(n) : n;
}

// cone_getter scene.cuh:887-961 for one triangle; also emits the traversal
// records of its owned edges (slots 3*pos .. 3*pos+2) and returns their count
SNCH_DEV Cone leaf_cone(const BuildArgs &a, uint32_t orig, const Box &b, uint32_t pos, uint32_t &n_owned)
{
    const f3 c = centroid(b);
    Cone r;
    r.axis = mk(0.0f, 0.0f, 0.0f);
    r.half_angle = kPi;
    r.radius = 0.0f;
    bool any = false, all_two = true;
    int4 se[3];
    n_owned = 0;
    for (int i = 0; i < 3; ++i)
    {
        const int32_t s = __ldg(a.tri_owned + 3 * (uint64_t)orig + i);
        if (s < 0 || (uint32_t)s >= 3 * a.num_tris)
            continue;
        const int4 e = __ldg(reinterpret_cast<const int4 *>(a.edge_verts) + s);
        const bool h0 = e.w != -1, h1 = e.x != -1;  // has_face(0), has_face(1) scene.cuh:741-744
        // silhouette_edge::normal() scene.cuh:772-786
        f3 nsum = mk(0.0f, 0.0f, 0.0f);
        if (h0)
        {
            const f3 n0 = edge_face_normal(a.verts, e, 0, false);
            nsum = mk(nsum.x + n0.x, nsum.y + n0.y, nsum.z + n0.z);
        }
        if (h1)
        {
            const f3 n1 = edge_face_normal(a.verts, e, 1, false);
            nsum = mk(nsum.x + n1.x, nsum.y + n1.y, nsum.z + n1.z);
        }
        const f3 sn = normalize3(nsum);
        r.axis.x += sn.x;
        r.axis.y += sn.y;
        r.axis.z += sn.z;
        const f3 pa = load_vert(a.verts, e.y), pb = load_vert(a.verts, e.z);
        const f3 sc = mk((pa.x + pb.x) / 2, (pa.y + pb.y) / 2, (pa.z + pb.z) / 2);  // centroid() 734-740
        r.radius = smax(r.radius, len3(mk(sc.x - c.x, sc.y - c.y, sc.z - c.z)));
        all_two = all_two && h0 && h1;
        any = true;
        // traversal record of this owned edge
        const f3 fn0 = h0 ? edge_face_normal(a.verts, e, 0, true) : mk(0.0f, 0.0f, 0.0f);
        const f3 fn1 = h1 ? edge_face_normal(a.verts, e, 1, true) : mk(0.0f, 0.0f, 0.0f);
        EdgeRec er;
        er.a = make_float4(pa.x, pa.y, pa.z, __uint_as_float((h0 ? 1u : 0u) | (h1 ? 2u : 0u)));
        er.b = make_float4(pb.x, pb.y, pb.z, __int_as_float(s));
        er.c = make_float4(fn0.x, fn0.y, fn0.z, 0.0f);
        er.d = make_float4(fn1.x, fn1.y, fn1.z, 0.0f);
        a.edges[3 * (uint64_t)pos + n_owned] = er;
        se[n_owned] = e;
        ++n_owned;
    }
    if (!any)
        r.half_angle = -kPi;
    else if (!all_two)
        r.half_angle = kPi;
    else
    {
        const float axis_norm = len3(r.axis);
        if (axis_norm > kEps)
        {
            r.axis.x /= axis_norm;
            r.axis.y /= axis_norm;
            r.axis.z /= axis_norm;
            r.half_angle = 0.0f;
            for (uint32_t i = 0; i < n_owned; ++i)
            {
                const bool h0 = se[i].w != -1, h1 = se[i].x != -1;
                const f3 fn[2] = {h0 ? edge_face_normal(a.verts, se[i], 0, true) : mk(0.0f, 0.0f, 0.0f),
                                  h1 ? edge_face_normal(a.verts, se[i], 1, true) : mk(0.0f, 0.0f, 0.0f)};
                for (int j = 0; j < 2; ++j)
                {
                    const float angle = acosf(smax(-1.0f, smin(1.0f, dot3(r.axis, fn[j]))));
                    r.half_angle = smax(r.half_angle, angle);
                }
            }
        }
    }
    return r;
}

// rotate(float3) cone.cuh:288-302
SNCH_DEV f3 rotate3(f3 u, f3 v, float theta)
{
    const float ct = cosf(theta), st = sinf(theta);
    const f3 w = normalize3(cross3(u, v));
    const f3 o = mk((1.0f - ct) * w.x, (1.0f - ct) * w.y, (1.0f - ct) * w.z);
    const float r00 = ct + o.x * w.x, r01 = o.y * w.x - st * w.z, r02 = o.z * w.x + st * w.y;
    const float r10 = o.x * w.y + st * w.z, r11 = ct + o.y * w.y, r12 = o.z * w.y - st * w.x;
    const float r20 = o.x * w.z - st * w.y, r21 = o.y * w.z + st * w.x, r22 = ct + o.z * w.z;
    return mk(r00 * u.x + r01 * u.y + r02 * u.z, r10 * u.x + r11 * u.y + r12 * u.z, r20 * u.x + r21 * u.y + r22 * u.z);
}

// merge(cone, cone, origins) cone.cuh:427-480; where the reference leaves
// half_angle unassigned (o_theta >= pi, 454-458) the conservative pi is stored,
// and a merge of two invalid cones gets a zero axis and radius.
SNCH_DEV Cone cone_merge(const Cone &a, const Cone &b, f3 oa, f3 ob, f3 on)
{
    Cone r;
    r.axis = mk(0.0f, 0.0f, 0.0f);
    r.half_angle = 0.0f;
    r.radius = 0.0f;
    const bool va = a.half_angle >= 0.0f, vb = b.half_angle >= 0.0f;
    if (va && vb)
    {
        f3 axis_a = a.axis, axis_b = b.axis;
        float ha = a.half_angle, hb = b.half_angle;
        const f3 da = sub(on, oa), db = sub(on, ob);
        r.radius = sqrtf(smax(a.radius * a.radius + sqlen3(da), b.radius * b.radius + sqlen3(db)));
        if (hb > ha)
        {
            const f3 t = axis_a;
            axis_a = axis_b;
            axis_b = t;
            const float h = ha;
            ha = hb;
            hb = h;
        }
        const float theta = acosf(smax(-1.0f, smin(1.0f, dot3(axis_a, axis_b))));
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
        const float r_theta = o_theta - ha;
        r.axis = rotate3(axis_a, axis_b, r_theta);
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

SNCH_DEV Box ldcg_box(const Box *p)
{
    const float *q = reinterpret_cast<const float *>(p);
    Box b;
    b.upper = mk(__ldcg(q), __ldcg(q + 1), __ldcg(q + 2));
    b.lower = mk(__ldcg(q + 3), __ldcg(q + 4), __ldcg(q + 5));
    return b;
}
SNCH_DEV Cone ldcg_cone(const Cone *p)
{
    const float *q = reinterpret_cast<const float *>(p);
    Cone c;
    c.axis = mk(__ldcg(q), __ldcg(q + 1), __ldcg(q + 2));
    c.half_angle = __ldcg(q + 3);
    c.radius = __ldcg(q + 4);
    return c;
}

// One thread per sorted leaf: leaf box + cone + traversal records, then the
// walk towards the root. The first thread to reach a node stops; the second
// (whose sibling's results are published by the sibling's fence + atomic)
// merges both children.
__global__ void __launch_bounds__(128) refit_kernel(BuildArgs a)
{
    const uint32_t n = a.num_tris, ni = n - 1;
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const uint32_t orig = __ldg(a.vals + j);
    if (orig >= n)  // only after a failed sort (status bit set)
        return;
    const int32_t *t = a.tris + 3 * (uint64_t)orig;
    const f3 pa = load_vert(a.verts, __ldg(t)), pb = load_vert(a.verts, __ldg(t + 1)),
             pc = load_vert(a.verts, __ldg(t + 2));
    const Box b = tri_box(pa, pb, pc);
    uint32_t n_owned;
    const Cone c = leaf_cone(a, orig, b, j, n_owned);
    const uint32_t leaf = ni + j;
    a.aabbs[leaf] = b;
    a.cones[leaf] = c;
    LeafRec lr;
    lr.v0 = make_float4(pa.x, pa.y, pa.z, __uint_as_float(orig));
    lr.v1 = make_float4(pb.x, pb.y, pb.z, __uint_as_float(n_owned));
    lr.v2 = make_float4(pc.x, pc.y, pc.z, 0.0f);
    a.leaves[j] = lr;
    if (n == 1)
        return;
    uint32_t cur = leaf;
    // a Karras tree over 64-bit keys is at most 65 levels deep
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
        const Box lb = ldcg_box(a.aabbs + L), rb = ldcg_box(a.aabbs + R);
        const Cone lc = ldcg_cone(a.cones + L), rc = ldcg_cone(a.cones + R);
        const Box m = merge_box(lb, rb);
        a.aabbs[p] = m;
        a.cones[p] = cone_merge(lc, rc, centroid(lb), centroid(rb), centroid(m));
        a.inner[p] = pack_inner(lb, rb, L, R);
        a.inner_cones[p] = pack_cones(lc, rc);
        cur = p;
    }
}

// Position of every leaf in the reference's full depth-first visit order
// (query.cuh:256-316): expanding node n emits its leaf children (left, then
// right), then visits the right subtree, then the left one. A leaf's position
// is the sum, over the path to the root, of the offset of each node within its
// parent's emission sequence. The near-first traversals use it to resolve exact
// distance ties the way the reference's visit order does. Stored in LeafRec.v2.w.
__global__ void __launch_bounds__(256) rank_kernel(BuildArgs a)
{
    const uint32_t n = a.num_tris, ni = n - 1;
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    uint32_t node = ni + j, r = 0;
    for (int level = 0; level < 96 && n > 1; ++level)
    {
        const uint32_t p = a.nodes[node].parent;
        if (p >= ni)
            break;
        const uint32_t L = a.nodes[p].left, R = a.nodes[p].right;
        const uint32_t lleaf = L >= ni ? 1u : 0u, rleaf = R >= ni ? 1u : 0u;
        if (node == L)
            r += lleaf ? 0u : lleaf + rleaf + (rleaf ? 0u : a.sizes[R]);
        else
            r += rleaf ? lleaf : lleaf + rleaf;
        node = p;
    }
    a.leaves[j].v2.w = __uint_as_float(r);
    // the leaf's rank and owned-edge count in its parent's traversal record
    const uint32_t p = n > 1 ? a.nodes[ni + j].parent : kInvalid;
    if (p < ni)
    {
        const uint32_t info = (r & kLeafRankMask) | (__float_as_uint(a.leaves[j].v1.w) << 30);
        float *d = reinterpret_cast<float *>(&a.inner[p].d);
        d[a.nodes[p].left == ni + j ? 2 : 3] = __uint_as_float(info);
    }
}

// Objects in the reference's device layout (scene.cuh:708-722 silhouette_edge,
// 826-840 triangle) so that snch_get_bvh_view() is a drop-in bvh_device view.
__global__ void ref_objects_kernel(const float *verts, const int32_t *tris, const int32_t *tri_owned,
                                   const int32_t *edge_verts, uint32_t num_tris, snch_triangle *objs,
                                   snch_silhouette_edge *edges)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_tris)
        return;
    snch_triangle o;
    for (int k = 0; k < 3; ++k)
    {
        o.vertex_indices[k] = tris[3 * (uint64_t)i + k];
        o.silhouette_indices[k] = tri_owned[3 * (uint64_t)i + k];
    }
    o.vertices = verts;
    o.silhouettes = edges;
    objs[i] = o;
    // every edge is owned by exactly one triangle: that triangle writes it
    for (int k = 0; k < 3; ++k)
    {
        const int32_t e = o.silhouette_indices[k];
        if (e < 0 || (uint32_t)e >= 3 * num_tris)
            continue;
        snch_silhouette_edge se;
        const int4 ev = reinterpret_cast<const int4 *>(edge_verts)[e];
        se.indices[0] = ev.x;
        se.indices[1] = ev.y;
        se.indices[2] = ev.z;
        se.indices[3] = ev.w;
        se.vertices = verts;
        se.pad_ = 0;
        edges[e] = se;
    }
}

// counts vertex indices outside [0, num_verts)
__global__ void validate_kernel(const int32_t *tris, int64_t n, int64_t num_verts, uint32_t *bad)
{
    uint32_t c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int32_t v = tris[i];
        c += (v < 0 || v >= num_verts) ? 1u : 0u;
    }
    if (c)
        atomicAdd(bad, c);
}

// ------------------------------------------------------------------ wide records
// Mesh roots of a batched scene: a wide node's depth is counted from its mesh's
// root, and the nodes that join meshes (above every mesh root) are never searched.
__global__ void wide_mark_kernel(const uint32_t *__restrict__ mesh_root, uint32_t num_meshes, uint32_t ni,
                                 uint8_t *__restrict__ stop)
{
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < num_meshes)
    {
        const uint32_t r = mesh_root[m];
        if (r < ni)
            stop[r] = 1;
    }
}

// flags[i] = 1 when binary internal node i roots a wide record: its depth below
// the tree root (or its mesh root, stop != nullptr) is a multiple of k
__global__ void __launch_bounds__(256) wide_flag_kernel(const NodeRec *__restrict__ nodes, uint32_t ni, int k,
                                                        const uint8_t *__restrict__ stop, uint32_t *__restrict__ flags,
                                                        uint32_t *status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni)
        return;
    uint32_t node = i, d = 0;
    bool found = false, joins_meshes = false;
    for (int level = 0; level < 256; ++level)
    {
        if (stop && stop[node])
        {
            found = true;
            break;
        }
        const uint32_t p = nodes[node].parent;
        if (p >= ni)
        {
            found = true;
            joins_meshes = stop != nullptr;
            break;
        }
        node = p;
        ++d;
    }
    if (!found)
        atomicOr(status, kStatusTreeDepth);
    flags[i] = (found && !joins_meshes && d % (uint32_t)k == 0u) ? 1u : 0u;
}

// One wide record per flagged node: the slot tree of its binary descendants
// kLevels down (node / pass / empty positions, see WideLayout).
template <int W>
__global__ void __launch_bounds__(128) wide_fill_kernel(const NodeRec *__restrict__ nodes, const Box *__restrict__ aabbs,
                                                        const Cone *__restrict__ cones,
                                                        const LeafRec *__restrict__ leaves, uint32_t ni,
                                                        const uint32_t *__restrict__ flags,
                                                        const uint32_t *__restrict__ wide_of, float4 *__restrict__ out,
                                                        uint32_t capacity, uint32_t *status)
{
    using Lay = WideLayout<W>;
    constexpr int P = Lay::P, F = Lay::F;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni || !flags[i])
        return;
    if (wide_of[i] >= capacity)
    {
        atomicOr(status, kStatusTreeDepth);
        return;
    }
    enum : uint8_t
    {
        kEmpty = 0,
        kNode = 1,
        kPass = 2
    };
    uint32_t at[F];
    uint8_t kind[F];
    at[0] = nodes[i].left;
    at[1] = nodes[i].right;
    kind[0] = kind[1] = kNode;
#pragma unroll
    for (int f = 2; f < F; ++f)
    {
        const int pf = ((f + 2) >> 1) - 2;
        const bool left = (f & 1) == 0;
        at[f] = kInvalid;
        kind[f] = kEmpty;
        if (kind[pf] == kNode && at[pf] < ni)
        {
            at[f] = left ? nodes[at[pf]].left : nodes[at[pf]].right;
            kind[f] = kNode;
        }
        else if (kind[pf] != kEmpty && left)  // a leaf above: forwarded to the leftmost position
        {
            at[f] = at[pf];
            kind[f] = kPass;
        }
    }
    float *rec = reinterpret_cast<float *>(out + (size_t)wide_of[i] * Lay::kRecF4);
    uint32_t *u = reinterpret_cast<uint32_t *>(rec);
    float *cn = rec + Lay::kCone;
#pragma unroll
    for (int f = 0; f < P; ++f)
    {
        Box b;
        Cone c;
        const uint8_t k = f < F ? kind[f] : (uint8_t)kEmpty;
        if (k == kNode)
        {
            b = aabbs[at[f]];
            c = cones[at[f]];
        }
        else
        {
            // a pass position carries its leaf's box (its sibling is empty, so
            // the sibling test passes; the distance tests stay those of the leaf)
            // and a cone that passes every test
            b.lower = mk(INFINITY, INFINITY, INFINITY);
            b.upper = mk(-INFINITY, -INFINITY, -INFINITY);
            if (k == kPass)
                b = aabbs[at[f]];
            c.axis = mk(0.0f, 0.0f, 0.0f);
            c.half_angle = k == kPass ? kPi : -1.0f;
            c.radius = 0.0f;
        }
        rec[0 * P + f] = b.lower.x;
        rec[1 * P + f] = b.lower.y;
        rec[2 * P + f] = b.lower.z;
        rec[3 * P + f] = b.upper.x;
        rec[4 * P + f] = b.upper.y;
        rec[5 * P + f] = b.upper.z;
        cn[0 * P + f] = c.axis.x;
        cn[1 * P + f] = c.axis.y;
        cn[2 * P + f] = c.axis.z;
        cn[3 * P + f] = c.half_angle;
        cn[4 * P + f] = c.radius;
    }
#pragma unroll
    for (int sl = 0; sl < W; ++sl)
    {
        const int f = Lay::S0 + sl;
        uint32_t child = kInvalid, info = 0;
        if (kind[f] != kEmpty)
        {
            const uint32_t g = at[f];
            if (g < ni)
            {
                if (!flags[g])
                    atomicOr(status, kStatusTreeDepth);
                child = wide_of[g];
            }
            else
            {
                const uint32_t pos = g - ni;
                child = kWideLeaf | pos;
                const uint32_t rank = __float_as_uint(leaves[pos].v2.w);
                info = (rank & kLeafRankMask) | (__float_as_uint(leaves[pos].v1.w) << 30);
            }
        }
        u[Lay::kChild + sl] = child;
        u[Lay::kInfo + sl] = info;
    }
}

size_t wide_scratch_bytes(uint32_t num_tris)
{
    const uint32_t ni = num_tris > 1 ? num_tris - 1 : 1;
    return 256 + ((ni + 255) & ~255u) + scan_flags_scratch_bytes(ni) + 256;
}

cudaError_t launch_wide_count(const WideArgs &a, cudaStream_t st)
{
    const uint32_t ni = a.num_tris - 1;
    char *sc = static_cast<char *>(a.scratch);
    uint8_t *stop = nullptr;
    cudaError_t e = cudaSuccess;
    if (a.num_meshes)
    {
        stop = reinterpret_cast<uint8_t *>(sc + 256);
        if ((e = cudaMemsetAsync(stop, 0, ni, st)) != cudaSuccess)
            return e;
        wide_mark_kernel<<<(a.num_meshes + 255) / 256, 256, 0, st>>>(a.mesh_root, a.num_meshes, ni, stop);
        note_launch();
    }
    wide_flag_kernel<<<(ni + 255) / 256, 256, 0, st>>>(a.nodes, ni, a.width == 4 ? 2 : 3, stop, a.flags, a.status);
    note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    void *scan_scratch = sc + 256 + ((ni + 255) & ~255u);
    return scan_flags(a.flags, a.wide_of, ni, a.count, scan_scratch, a.status, st);
}

cudaError_t launch_wide_fill(const WideArgs &a, cudaStream_t st)
{
    const uint32_t ni = a.num_tris - 1;
    if (a.width == 4)
        wide_fill_kernel<4><<<(ni + 127) / 128, 128, 0, st>>>(a.nodes, a.aabbs, a.cones, a.leaves, ni, a.flags,
                                                              a.wide_of, a.out, a.capacity, a.status);
    else
        wide_fill_kernel<8><<<(ni + 127) / 128, 128, 0, st>>>(a.nodes, a.aabbs, a.cones, a.leaves, ni, a.flags,
                                                              a.wide_of, a.out, a.capacity, a.status);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ launchers
// Karras internal nodes alone, over a.keys / a.vals (sorted), into a.nodes and
// a.sizes: the 2D build shares it (the construction does not depend on the
// dimension)
cudaError_t launch_karras(const BuildArgs &a, cudaStream_t st)
{
    karras_kernel<<<(a.num_tris + 255) / 256, 256, 0, st>>>(a);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_build_front(const BuildArgs &a, cudaStream_t st)
{
    const uint32_t n = a.num_tris;
    init_build_kernel<<<1, 256, 0, st>>>(a.scene_box, a.hist);
    note_launch();
    if (a.num_meshes)
    {
        init_mesh_kernel<<<(a.num_meshes + 255) / 256, 256, 0, st>>>(a.mesh_box, a.mesh_root, a.mesh_edge_start,
                                                                     a.num_meshes);
        note_launch();
        mesh_edges_kernel<<<(n + 255) / 256, 256, 0, st>>>(a.tri_edges, a.tri_mesh, n, a.mesh_edge_start);
        note_launch();
    }
    const uint32_t g = (n + 255) / 256;
    leaf_bounds_kernel<<<g, 256, 0, st>>>(a);
    note_launch();
    morton_kernel<<<g, 256, 0, st>>>(a);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_build_back(const BuildArgs &a, cudaStream_t st)
{
    const uint32_t n = a.num_tris;
    karras_kernel<<<(n + 255) / 256, 256, 0, st>>>(a);
    note_launch();
    if (n > 1)
    {
        cudaError_t e = cudaMemsetAsync(a.flags, 0, 4 * (size_t)(n - 1), st);
        if (e != cudaSuccess)
            return e;
    }
    refit_kernel<<<(n + 127) / 128, 128, 0, st>>>(a);
    note_launch();
    rank_kernel<<<(n + 255) / 256, 256, 0, st>>>(a);
    note_launch();
    return cudaGetLastError();
}

// batched scenes, after the Morton sort: mesh id of each sorted position and
// the identity permutation, then (after the stable sort by mesh id) the codes
// and triangle indices gathered into (mesh, code, index) order
__global__ void mesh_keys_kernel(const uint32_t *__restrict__ vals, const uint32_t *__restrict__ tri_mesh, uint32_t n,
                                 uint32_t *__restrict__ mkey, uint32_t *__restrict__ perm)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const uint32_t v = vals[i];
        mkey[i] = v < n ? __ldg(tri_mesh + v) : 0u;
        perm[i] = i;
    }
}
__global__ void gather_pairs_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                                    const uint32_t *__restrict__ perm, uint32_t n, uint32_t *__restrict__ keys_out,
                                    uint32_t *__restrict__ vals_out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const uint32_t p = perm[i];
        keys_out[i] = p < n ? keys[p] : 0u;
        vals_out[i] = p < n ? vals[p] : kInvalid;
    }
}

cudaError_t launch_mesh_setup(const uint32_t *tri_start, const int64_t *vert_start, uint32_t num_meshes, uint32_t n,
                              uint32_t *tri_mesh, int32_t *tris, uint32_t *bad, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(bad, 0, 4, st);
    if (e != cudaSuccess || n == 0)
        return e;
    mesh_setup_kernel<<<(n + 255) / 256, 256, 0, st>>>(tri_start, vert_start, num_meshes, n, tri_mesh, tris, bad);
    note_launch();
    return cudaGetLastError();
}

int mesh_key_bits(uint32_t num_meshes)
{
    int b = 1;
    while (b < 16 && (1u << b) < num_meshes)
        ++b;
    return b;
}

size_t mesh_pass_scratch_bytes(uint32_t n, uint32_t num_meshes)
{
    return sort_scratch_bytes(n, mesh_key_bits(num_meshes));
}

// keys/vals hold the Morton-sorted (code, triangle); keys_tmp/vals_tmp are n words each
cudaError_t launch_mesh_pass(const BuildArgs &a, void *scratch, cudaStream_t st)
{
    const uint32_t n = a.num_tris;
    if (!a.num_meshes || n == 0)
        return cudaSuccess;
    mesh_keys_kernel<<<(n + 255) / 256, 256, 0, st>>>(a.vals, a.tri_mesh, n, a.sorted_mesh, a.perm);
    note_launch();
    cudaError_t e = radix_sort_pairs(a.sorted_mesh, a.perm, a.mkey_tmp, a.perm_tmp, n, mesh_key_bits(a.num_meshes),
                                     nullptr, scratch, a.status, st);
    if (e != cudaSuccess)
        return e;
    // gathered into the scratch pair, then back
    gather_pairs_kernel<<<(n + 255) / 256, 256, 0, st>>>(a.keys, a.vals, a.perm, n, a.mkey_tmp, a.perm_tmp);
    note_launch();
    if ((e = cudaMemcpyAsync(a.keys, a.mkey_tmp, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(a.vals, a.perm_tmp, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return e;
    return cudaGetLastError();
}

}  // namespace snch

namespace snch
{
cudaError_t launch_ref_objects(const float *verts, const int32_t *tris, const int32_t *tri_owned,
                               const int32_t *edge_verts, uint32_t num_tris, snch_triangle *objs,
                               snch_silhouette_edge *edges, cudaStream_t st)
{
    if (num_tris)
    {
        ref_objects_kernel<<<(num_tris + 255) / 256, 256, 0, st>>>(verts, tris, tri_owned, edge_verts, num_tris, objs,
                                                                  edges);
        note_launch();
    }
    return cudaGetLastError();
}

cudaError_t launch_validate(const int32_t *tris, int64_t n, int64_t num_verts, uint32_t *bad, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(bad, 0, 4, st);
    if (e != cudaSuccess || n == 0)
        return e;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
    validate_kernel<<<(unsigned)blocks, 256, 0, st>>>(tris, n, num_verts, bad);
    note_launch();
    return cudaGetLastError();
}
}  // namespace snch
