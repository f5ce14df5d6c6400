// Per-query traversal kernels over the 64-B node layout.
//
// Each kernel keeps the reference's visit order (stack discipline, child order,
// pruning tests and tie rules) so that it returns the reference's results bit
// for bit, while reading one 64-byte record per expanded node:
//   nearest_kernel     query_device(nearest)            query.cuh:239-318
//   silhouette_kernel  query_device(nearest_silhouette) query.cuh:326-423
//   ray_kernel         query_device(ray_intersect)      query.cuh:82-169
//   sample_kernel      sample_object_in_sphere          sample.cuh:26-91
//   sample_point_kernel sample_on_object                sample.cuh:10-22
// A one-triangle tree (where the reference reads past its node array,
// bvh.cuh:388-390) evaluates its only leaf directly. A traversal that would
// need more than 64 stack entries (undefined in the reference) stops, writes
// NaN / 0xFFFFFFFF and sets kStatusStackOverflow.
#include "internal.h"

namespace snch
{

// find_closest_point_triangle scene.cuh:34-110: the squared length whose square root
// is the distance (the argument of len3's sqrtf, summed in the same order)
SNCH_DEV float closest_point_triangle_sq(f3 pa, f3 pb, f3 pc, f3 x)
{
    const f3 ab = sub(pb, pa), ac = sub(pc, pa), ax = sub(x, pa);
    const float d1 = dot3(ab, ax), d2 = dot3(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f)
        return sqlen3(sub(x, pa));
    const f3 bx = sub(x, pb);
    const float d3 = dot3(ab, bx), d4 = dot3(ac, bx);
    if (d3 >= 0.0f && d4 <= d3)
        return sqlen3(sub(x, pb));
    const f3 cx = sub(x, pc);
    const float d5 = dot3(ab, cx), d6 = dot3(ac, cx);
    if (d6 >= 0.0f && d5 <= d6)
        return sqlen3(sub(x, pc));
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f)
    {
        const float v = d1 / (d1 - d3);
        return sqlen3(sub(x, mk(pa.x + ab.x * v, pa.y + ab.y * v, pa.z + ab.z * v)));
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f)
    {
        const float w = d2 / (d2 - d6);
        return sqlen3(sub(x, mk(pa.x + ac.x * w, pa.y + ac.y * w, pa.z + ac.z * w)));
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
    {
        const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return sqlen3(sub(x, mk(pb.x + (pc.x - pb.x) * w, pb.y + (pc.y - pb.y) * w, pb.z + (pc.z - pb.z) * w)));
    }
    const float denom = 1.0f / (va + vb + vc);
    const float v = vb * denom, w = vc * denom;
    return sqlen3(sub(x, mk(pa.x + ab.x * v + ac.x * w, pa.y + ab.y * v + ac.y * w, pa.z + ab.z * v + ac.z * w)));
}

SNCH_DEV float closest_point_triangle(f3 pa, f3 pb, f3 pc, f3 x) { return sqrtf(closest_point_triangle_sq(pa, pb, pc, x)); }

// A candidate whose squared length s exceeds beyond(b) cannot pass a test
// "sqrtf(s) <= b" (silhouette: b a distance) nor "sqrtf(s)^2 <= b" (nearest: b a
// squared distance): b (1 + 2^-19), rounded twice, exceeds b (1 + 2^-20), and
// both rounded forms of s then exceed b. So the IEEE square root is taken only
// for candidates the exact test could accept; the answers do not change.
SNCH_DEV float beyond_sq(float best_sq) { return best_sq * 1.0000019073486328125f; }

SNCH_DEV Box load_root_box(const Box *p)
{
    const float *q = reinterpret_cast<const float *>(p);
    Box b;
    b.upper = mk(__ldg(q), __ldg(q + 1), __ldg(q + 2));
    b.lower = mk(__ldg(q + 3), __ldg(q + 4), __ldg(q + 5));
    return b;
}

// Query inputs are read once and results written once: with streaming hints
// (ld.global.cs / st.global.cs) their lines leave L2 first, and the tree
// records the traversals re-read stay cached longer.
#ifndef SNCH_STREAM_HINTS
#define SNCH_STREAM_HINTS 1
#endif
constexpr bool kStreamHints = SNCH_STREAM_HINTS != 0;
template <typename T>
SNCH_DEV T ld_in(const T *p)
{
    return kStreamHints ? __ldcs(p) : __ldg(p);
}
template <typename T>
SNCH_DEV void st_out(T *p, T v)
{
    if (kStreamHints)
        __stcs(p, v);
    else
        *p = v;
}
SNCH_DEV f3 load_point(const float *__restrict__ p, int64_t q)
{
    if (kStreamHints)
        return mk(__ldcs(p + 3 * q), __ldcs(p + 3 * q + 1), __ldcs(p + 3 * q + 2));
    return mk(__ldg(p + 3 * q), __ldg(p + 3 * q + 1), __ldg(p + 3 * q + 2));
}

// ------------------------------------------------------------------ nearest
SNCH_DEV float leaf_distance2(const TreeView &t, uint32_t pos, f3 p, uint32_t &orig)
{
    f3 pa, pb, pc;
    uint32_t n_owned;
    load_leaf(t.leaves + pos, pa, pb, pc, orig, n_owned);
    float d = closest_point_triangle(pa, pb, pc, p);
    d *= d;
    return d;
}

// seed.radius: the search starts with best = r^2 (query.cuh:255 with a bound);
// nodes holding a primitive at the final distance d* <= r are never pruned and
// the traversal order does not depend on best, so the same leaf wins; when
// nothing lies within r the query is listed for the unbounded fallback pass.
__global__ void __launch_bounds__(128) nearest_kernel(TreeView t, const float *__restrict__ pts, int64_t n,
                                                      uint32_t *__restrict__ out_idx, float *__restrict__ out_dist,
                                                      SeedArgs seed)
{
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 p = load_point(pts, q);
    uint32_t nearest = kInvalid;
    float best = INFINITY;
    if (seed.radius)
    {
        const float r = __ldg(seed.radius + q);
        best = r * r;
    }
    const uint32_t ni = t.num_tris - 1;
    if (t.num_tris == 1)
    {
        uint32_t orig;
        const float d = leaf_distance2(t, 0, p, orig);
        if (!seed.radius || d <= best)
        {
            best = d;
            nearest = orig;
        }
    }
    else if (t.num_tris > 1)
    {
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        sn[0] = 0;
        sd[0] = mindist(load_root_box(t.aabbs), p);
        sp = 1;
        do
        {
            --sp;
            const uint32_t node = sn[sp];
            if (sd[sp] > best)
                continue;
            if (sp > kStackDepth - 2)
            {
                atomicOr(t.status, kStatusStackOverflow);
                nearest = kInvalid;
                best = NAN;
                break;
            }
            Box lb, rb;
            uint32_t L, R;
            unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
            const float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
            const float Lmm = minmaxdist(lb, p), Rmm = minmaxdist(rb, p);
            if (Lmd <= Rmm)
            {
                if (L >= ni)
                {
                    uint32_t orig;
                    const float d = leaf_distance2(t, L - ni, p, orig);
                    if (d <= best)
                    {
                        best = d;
                        nearest = orig;
                    }
                }
                else
                {
                    sn[sp] = L;
                    sd[sp] = Lmd;
                    ++sp;
                }
            }
            if (Rmd <= Lmm)
            {
                if (R >= ni)
                {
                    uint32_t orig;
                    const float d = leaf_distance2(t, R - ni, p, orig);
                    if (d <= best)
                    {
                        best = d;
                        nearest = orig;
                    }
                }
                else
                {
                    sn[sp] = R;
                    sd[sp] = Rmd;
                    ++sp;
                }
            }
        } while (sp > 0);
    }
    if (seed.radius && nearest == kInvalid)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    out_idx[q] = nearest;
    out_dist[q] = sqrtf(best);
    if (seed.fail_flag)
        seed.fail_flag[q] = nearest == kInvalid ? 1u : 0u;
}

// ------------------------------------------------------------------ silhouette
// compute_orthonormal_basis(float3) cone.cuh:34-42 + project_to_plane cone.cuh:58-66
SNCH_DEV float project_to_plane(f3 n, f3 e)
{
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float b = n.x * n.y * a;
    const f3 b1 = mk(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    const f3 b2 = mk(b, sign + n.y * n.y * a, -n.y);
    const float r1 = dot3(e, cabs3(b1));
    const float r2 = dot3(e, cabs3(b2));
    return sqrtf(r1 * r1 + r2 * r2);
}
SNCH_DEV bool inrange(float v, float lo, float hi) { return v >= lo && v <= hi; }

// overlap(cone<float,3>, ...) cone.cuh:168-212
SNCH_DEV bool cone_overlap(const Cone &bc, f3 o, const Box &b, float dist_to_box)
{
    if (bc.half_angle >= kPi2 || dist_to_box < kEps)
        return true;
    const f3 c = centroid(b);
    f3 v = mk(c.x - o.x, c.y - o.y, c.z - o.z);
    const float l = len3(v);
    v.x /= l;
    v.y /= l;
    v.z /= l;
    const float dax = acosf(smax(-1.0f, smin(1.0f, dot3(bc.axis, v))));
    if (inrange(kPi2, dax - bc.half_angle, dax + bc.half_angle))
        return true;
    if (l > bc.radius)
    {
        const float vch = asinf(bc.radius / l);
        const float hs = bc.half_angle + vch;
        const float mn = dax - hs, mx = dax + hs;
        return hs >= kPi2 ? true : inrange(kPi2, mn, mx);
    }
    const f3 e = mk(b.upper.x - c.x, b.upper.y - c.y, b.upper.z - c.z);
    float d = dot3(e, cabs3(v));
    const float s = l - d;
    if (s <= 0.0f)
        return true;
    d = project_to_plane(v, e);
    const float vch = atan2f(d, s);
    const float hs = bc.half_angle + vch;
    const float mn = dax - hs, mx = dax + hs;
    return hs >= kPi2 ? true : inrange(kPi2, mn, mx);
}

// ---- fast, decision-identical form of cone_overlap
// cone_overlap's answer (for a query outside the box) is "the angle between the
// cone axis and the direction to the box centroid is within hs = half_angle +
// vch of 90 degrees", with vch = asin(radius / l) when the query is outside the
// cone's bounding sphere (l > radius), or "hs >= 90 degrees". In angle space:
// dev = |pi/2 - dax| = asin(|x|), x = axis . v / l; the test is dev <= hs. The
// reference evaluates it with acosf/asinf/atan2f and IEEE divisions; here dev
// and vch come from Abramowitz & Stegun 4.4.45 (arccos x = sqrt(1 - x) (a0 + a1 x
// + a2 x^2 + a3 x^3), |error| <= 6.8e-5 on [0, 1], also in float32), and the
// answer is taken only when the margin |dev - hs| exceeds kConeTol, which bounds
// the error of both evaluations: 2 x 6.8e-5 for the polynomials, and the
// propagated rounding of x (a few 1e-7 absolute, amplified by 1/sqrt(1 - x^2)
// <= 22.4 for |x| <= 0.999, the same for radius / l), plus the reference's own
// acosf/asinf error of a few ulps. Otherwise (ill-conditioned |x| or radius / l
// above 0.999, a query inside the bounding sphere, a margin below kConeTol) the
// exact cone_overlap decides. A decided answer therefore equals the one the
// reference's float arithmetic gives.
constexpr float kConeTol = 4.0e-4f;
constexpr float kIllCond = 0.999f;

// Hardware approximations (MUFU) and fused multiply-adds: the filter only needs
// its angles to within its margin kConeTol = 4e-4 rad, and these add a few 1e-7
// relative (amplified at most 22.4x through arccos below kIllCond), against the
// multi-instruction IEEE sqrtf / __frcp_rn sequences the exact path needs.
SNCH_DEV float sqrt_approx(float x)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
SNCH_DEV float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
SNCH_DEV float acos_as(float x)  // 0 <= x <= 1
{
    const float a0 = 1.5707288f, a1 = -0.2121144f, a2 = 0.0742610f, a3 = -0.0187293f;
    return sqrt_approx(1.0f - x) * __fmaf_rn(x, __fmaf_rn(x, __fmaf_rn(x, a3, a2), a1), a0);
}

// 1: overlap, 0: no overlap, -1: undecided (take cone_overlap)
SNCH_DEV int cone_overlap_fast(const Cone &bc, f3 o, const Box &b, float dist_to_box)
{
    if (bc.half_angle >= kPi2 || dist_to_box < kEps)
        return 1;  // the same first test as cone_overlap
    // (computing centroid - o as one fused multiply-add per axis, the same value,
    // measured 2 % slower: 34.44 against 33.70 ms per 16M silhouette queries)
    const f3 c = centroid(b);
    const f3 v = mk(c.x - o.x, c.y - o.y, c.z - o.z);
    // approximate l: the asin branch below is taken only when radius / l <= kIllCond,
    // i.e. l exceeds the radius by 0.1 %, so the exact l > radius holds there too.
    // One reciprocal square root gives l, axis . v / l and radius / l (relative
    // error a few 1e-7, like the square root and two divisions it replaces, which
    // measured 1.4 % slower on the silhouette packets: 34.22 against 33.75 ms per
    // 16M queries).
    const float l2 = __fmaf_rn(v.x, v.x, __fmaf_rn(v.y, v.y, v.z * v.z));
    const float rl = rsqrt_approx(l2);
    const float l = l2 * rl;  // l2 = 0: 0 * inf = NaN, which fails the next test
    if (!(l > 0.0f))
        return -1;
    const float ax = fabsf(__fmaf_rn(bc.axis.x, v.x, __fmaf_rn(bc.axis.y, v.y, bc.axis.z * v.z))) * rl;
    if (!(ax <= kIllCond))
        return -1;
    const float dev = kPi2 - acos_as(ax);
    const float ha = bc.half_angle;
    if (dev <= ha - kConeTol)
        return 1;
    if (!(l > bc.radius))
        return -1;
    const float y = bc.radius * rl;
    if (!(y <= kIllCond))
        return -1;
    const float hs = ha + (kPi2 - acos_as(fmaxf(y, 0.0f)));
    if (hs >= kPi2 + kConeTol || dev <= hs - kConeTol)
        return 1;
    if (hs <= kPi2 - kConeTol && dev >= hs + kConeTol)
        return 0;
    return -1;
}

SNCH_DEV bool cone_test(const Cone &bc, f3 o, const Box &b, float dist_to_box)
{
    const int f = cone_overlap_fast(bc, o, b, dist_to_box);
    return f >= 0 ? f == 1 : cone_overlap(bc, o, b, dist_to_box);
}

// Self-check: counts where the fast form decides and agrees / disagrees with
// cone_overlap, and where it leaves the decision to cone_overlap, on random
// boxes, cones and points, half of them placed within 1e-3 rad of the decision
// boundary. counts[0] agree, counts[1] disagree, counts[2] undecided.
SNCH_DEV uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
SNCH_DEV float unit_rand(uint64_t &st)
{
    st += 0x9E3779B97F4A7C15ull;
    return (float)(mix64(st) >> 40) * (1.0f / 16777216.0f);
}

__global__ void cone_filter_check_kernel(int64_t n, uint64_t seed, unsigned long long *counts)
{
    __shared__ unsigned long long s_c[3];
    if (threadIdx.x < 3)
        s_c[threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n)
    {
        uint64_t st = mix64(seed ^ (0x632BE59BD9B4E019ull * (uint64_t)(i + 1)));
        Box b;
        const f3 c = mk(2.f * unit_rand(st) - 1.f, 2.f * unit_rand(st) - 1.f, 2.f * unit_rand(st) - 1.f);
        const f3 h = mk(exp2f(-12.f + 11.f * unit_rand(st)), exp2f(-12.f + 11.f * unit_rand(st)),
                        exp2f(-12.f + 11.f * unit_rand(st)));
        b.lower = mk(c.x - h.x, c.y - h.y, c.z - h.z);
        b.upper = mk(c.x + h.x, c.y + h.y, c.z + h.z);
        Cone k;
        const float z = 2.f * unit_rand(st) - 1.f, ph = 6.2831853f * unit_rand(st), rr = sqrtf(fmaxf(0.f, 1.f - z * z));
        k.axis = mk(rr * cosf(ph), rr * sinf(ph), z);
        k.half_angle = unit_rand(st) < 0.5f ? 0.3f * unit_rand(st) : kPi2 * unit_rand(st);
        k.radius = len3(h) * (0.5f + unit_rand(st));
        const float l = k.radius * exp2f(-1.f + 6.f * unit_rand(st));
        // direction at a chosen angle to the axis: random, or near the decision boundary
        float theta;
        if (unit_rand(st) < 0.5f)
            theta = 3.14159265f * unit_rand(st);
        else
        {
            const float vch = l > k.radius ? asinf(k.radius / l) : 0.f;
            const float hs = k.half_angle + vch;
            const float side = unit_rand(st) < 0.5f ? -1.f : 1.f;
            theta = kPi2 + side * hs + 1e-3f * (2.f * unit_rand(st) - 1.f);
        }
        // perpendicular to the axis
        f3 pp = fabsf(k.axis.x) < 0.9f ? mk(0.f, -k.axis.z, k.axis.y) : mk(-k.axis.z, 0.f, k.axis.x);
        const float pl = len3(pp);
        pp = mk(pp.x / pl, pp.y / pl, pp.z / pl);
        const f3 dir = mk(cosf(theta) * k.axis.x + sinf(theta) * pp.x, cosf(theta) * k.axis.y + sinf(theta) * pp.y,
                          cosf(theta) * k.axis.z + sinf(theta) * pp.z);
        const f3 o = mk(c.x - l * dir.x, c.y - l * dir.y, c.z - l * dir.z);
        const float md = mindist(b, o);
        const int f = cone_overlap_fast(k, o, b, md);
        const int slot = f < 0 ? 2 : ((f == 1) == cone_overlap(k, o, b, md) ? 0 : 1);
        atomicAdd(&s_c[slot], 1ull);
    }
    __syncthreads();
    if (threadIdx.x < 3 && s_c[threadIdx.x])
        atomicAdd(counts + threadIdx.x, s_c[threadIdx.x]);
}

// find_closest_point_line_segment(float3) scene.cuh:230-255: the closest point pt
// and the squared length whose square root is the distance
SNCH_DEV float closest_point_segment_sq(f3 pa, f3 pb, f3 x, f3 &pt)
{
    const f3 u = sub(pb, pa), v = sub(x, pa);
    const float c1 = dot3(u, v);
    if (c1 <= 0.0f)
    {
        pt = pa;
        return sqlen3(sub(x, pt));
    }
    const float c2 = dot3(u, u);
    if (c2 <= c1)
    {
        pt = pb;
        return sqlen3(sub(x, pt));
    }
    const float tt = c1 / c2;
    pt = mk(pa.x + u.x * tt, pa.y + u.y * tt, pa.z + u.z * tt);
    return sqlen3(sub(x, pt));
}

SNCH_DEV float closest_point_segment(f3 pa, f3 pb, f3 x, f3 &pt) { return sqrtf(closest_point_segment_sq(pa, pb, x, pt)); }

// is_silhouette_edge scene.cuh:143-174 (view_dir left unnormalised, as there)
SNCH_DEV bool is_silhouette_edge(f3 pa, f3 pb, f3 n0, f3 n1, f3 view_dir, float d, bool flip)
{
    const float precision = 1e-3f;
    const float sign = flip ? 1.0f : -1.0f;
    if (d <= precision)
    {
        const f3 ed = normalize3(sub(pb, pa));
        const float sda = atan2f(dot3(ed, cross3(n0, n1)), dot3(n0, n1));
        return sign * sda > precision;
    }
    const float dot0 = dot3(view_dir, n0), dot1 = dot3(view_dir, n1);
    if (fabsf(dot0) <= precision)
        return sign * dot1 > precision;
    if (fabsf(dot1) <= precision)
        return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}

// silhouette_distance_calculator scene.cuh:978-1003 with
// find_closest_silhouette_point scene.cuh:788-824 per owned edge (min radius 0)
SNCH_DEV bool leaf_silhouette(const TreeView &t, uint32_t pos, f3 o, float max_r2, float &dist, bool flip,
                              int32_t &edge_id)
{
    const uint32_t n_owned = __float_as_uint(__ldg(&t.leaves[pos].v1.w));
    float mr2 = max_r2;
    bool ret = false;
    for (uint32_t k = 0; k < n_owned; ++k)
    {
        if (0.0f >= mr2)
            continue;
        const float4 *e = reinterpret_cast<const float4 *>(t.edges + 3 * (uint64_t)pos + k);
        const float4 ea = __ldg(e), eb = __ldg(e + 1);
        const f3 pa = mk(ea.x, ea.y, ea.z), pb = mk(eb.x, eb.y, eb.z);
        f3 cp;
        const float d = closest_point_segment(pa, pb, o, cp);
        if (d * d > mr2)
            continue;
        const uint32_t flags = __float_as_uint(ea.w);
        bool is_sil = (flags & 1u) == 0u || (flags & 2u) == 0u;
        if (!is_sil)
        {
            const float4 ec = __ldg(e + 2), ed = __ldg(e + 3);
            is_sil = is_silhouette_edge(pa, pb, mk(ec.x, ec.y, ec.z), mk(ed.x, ed.y, ed.z),
                                        mk(o.x - cp.x, o.y - cp.y, o.z - cp.z), d, flip);
        }
        if (is_sil && d * d <= mr2)
        {
            dist = d;
            ret = true;
            mr2 = dist * dist;
            edge_id = __float_as_int(eb.w);
        }
    }
    return ret;
}

// seed.radius: the search starts with best = r (same argument as nearest_kernel:
// the cone tests do not depend on best and the visit order is fixed)
__global__ void __launch_bounds__(128) silhouette_kernel(TreeView t, const float *__restrict__ pts,
                                                         const uint8_t *__restrict__ flips, int64_t n,
                                                         float *__restrict__ out_dist, int32_t *__restrict__ out_edge,
                                                         SeedArgs seed)
{
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 p = load_point(pts, q);
    const bool flip = flips ? ld_in(flips + q) != 0 : false;
    float best = seed.radius ? __ldg(seed.radius + q) : INFINITY;
    int32_t best_edge = -1;
    const uint32_t ni = t.num_tris - 1;
    if (t.num_tris == 1)
    {
        float dist = INFINITY;
        int32_t eid = -1;
        if (leaf_silhouette(t, 0, p, best * best, dist, flip, eid) && dist <= best)
        {
            best = dist;
            best_edge = eid;
        }
    }
    else if (t.num_tris > 1)
    {
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        sn[0] = 0;
        sd[0] = mindist(load_root_box(t.aabbs), p);
        sp = 1;
        do
        {
            --sp;
            const uint32_t node = sn[sp];
            if (sd[sp] > best * best)
                continue;
            if (sp > kStackDepth - 2)
            {
                atomicOr(t.status, kStatusStackOverflow);
                best = NAN;
                best_edge = -1;
                break;
            }
            Box lb, rb;
            uint32_t L, R;
            unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
            const float4 *cr = reinterpret_cast<const float4 *>(t.inner_cones + node);
            InnerConeRec icr;
            icr.a = __ldg(cr);
            icr.b = __ldg(cr + 1);
            icr.c = __ldg(cr + 2);
            Cone lc, rc;
            unpack_cones(icr, lc, rc);
            const float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
            const bool hitL = lc.half_angle >= 0.0f && cone_overlap(lc, p, lb, Lmd);
            const bool hitR = rc.half_angle >= 0.0f && cone_overlap(rc, p, rb, Rmd);
            if (hitL)
            {
                if (L >= ni)
                {
                    float dist = INFINITY;
                    int32_t eid = -1;
                    if (leaf_silhouette(t, L - ni, p, best * best, dist, flip, eid) && dist <= best)
                    {
                        best = dist;
                        best_edge = eid;
                    }
                }
                else
                {
                    sn[sp] = L;
                    sd[sp] = Lmd;
                    ++sp;
                }
            }
            if (hitR)
            {
                if (R >= ni)
                {
                    float dist = INFINITY;
                    int32_t eid = -1;
                    if (leaf_silhouette(t, R - ni, p, best * best, dist, flip, eid) && dist <= best)
                    {
                        best = dist;
                        best_edge = eid;
                    }
                }
                else
                {
                    sn[sp] = R;
                    sd[sp] = Rmd;
                    ++sp;
                }
            }
        } while (sp > 0);
    }
    if (seed.radius && best_edge < 0)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    out_dist[q] = best;
    if (out_edge)
        out_edge[q] = best_edge;
    if (seed.fail_flag)
        seed.fail_flag[q] = best_edge < 0 ? 1u : 0u;
}

// ------------------------------------------------------------------ near-first forms
// Same results as nearest_kernel / silhouette_kernel, fewer visits. The
// reference's answer is a minimum over the leaves its traversal evaluates;
// the child tests that decide which leaves can be reached (minmaxdist for the
// nearest query, the normal-cone test for the silhouette query) depend only on
// the node and the query point, and pruning by the running best never removes
// a leaf that attains the final minimum. So any visit order reaches the same
// minimum; only exact ties depend on the order, and those are resolved with
// the leaf's position in the reference's depth-first order (LeafRec.v2.w):
//   nearest:    among equal squared distances the reference keeps the leaf it
//               visits last (query.cuh:286, 304: "<=");
//   silhouette: among equal distances it keeps the last (edge slot order inside
//               a leaf, scene.cuh:989-999), except at distance 0, after which
//               no edge is accepted any more (scene.cuh:791-794) -- the first wins.
// Children are pushed far-then-near so the nearer subtree is searched first.

SNCH_DEV void leaf_nearest_fast(const TreeView &t, uint32_t pos, f3 p, float &best, uint32_t &best_rank,
                                uint32_t &nearest)
{
    const float4 *q = reinterpret_cast<const float4 *>(t.leaves + pos);
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    const float sq = closest_point_triangle_sq(mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), p);
    if (sq > beyond_sq(best))
        return;  // d > best: not a candidate
    float d = sqrtf(sq);
    d *= d;
    const uint32_t rank = __float_as_uint(c.w);
    if (d < best || (d == best && (nearest == kInvalid || rank > best_rank)))
    {
        best = d;
        best_rank = rank;
        nearest = __float_as_uint(a.w);
    }
}

// Child records the traversal may expand next can be requested into L1 before
// the leaf work of this node runs, to overlap their latency with it. Measured
// 2 % slower on the 2M-triangle scene (the prefetched lines of the farther
// child evict lines still in use), so off.
constexpr bool kPrefetchChildren = false;
SNCH_DEV void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
// The same request by the packet searches (both internal children's records,
// one warp-uniform prefetch each at the start of a step) measured 15 % slower
// for silhouettes (40.9 vs 35.6 ms per 16M queries) and 11 % for nearest, so
// they do not prefetch either.

// (128, 10): at most 48 registers, ten blocks per SM (silhouette: (128, 9), 56
// registers, nine blocks). The traversals wait on dependent L2 loads; the extra
// resident warps hide more of that latency (measured on the 2M-triangle scene:
// silhouette -12 %, nearest -2 % against 60 registers / eight blocks).
// Block size kBlock (64, 128 or 256; TreeView::block_near / block_sil): the same threads per SM
// (1280 nearest, 1152 silhouette) in smaller or larger blocks. A block's slot
// on the SM is freed only when its slowest query is done, so smaller blocks
// lose less to the long tail of per-query work.
template <bool kStats, int kBlock = 128>
__global__ void __launch_bounds__(kBlock, 1280 / kBlock) nearest_fast_kernel(TreeView t, const float *__restrict__ pts, int64_t n,
                                                           uint32_t *__restrict__ out_idx, float *__restrict__ out_dist,
                                                           uint32_t *__restrict__ stats, SeedArgs seed)
{
    uint32_t n_int = 0, n_leaf = 0;
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 p = load_point(pts, q);
    uint32_t nearest = kInvalid, best_rank = 0;
    float best = INFINITY, r0 = INFINITY;
    if (seed.radius)
    {
        r0 = __ldg(seed.radius + q);
        best = r0 * r0;
    }
    bool deferred = false;
    uint32_t budget = seed.cap ? seed.cap : 0xFFFFFFFFu;
    const uint32_t ni = t.num_tris - 1;
    const QueryRoot qr = query_root(t, q);
    if (qr.node == kInvalid)
    {
    }
    else if (qr.node >= ni)  // a one-triangle tree or mesh
        leaf_nearest_fast(t, qr.node - ni, p, best, best_rank, nearest);
    else
    {
        // The nearer passing child is expanded next without a trip through the
        // stack (it would be popped at once, and its bound re-check cannot fail);
        // only the farther one is pushed. Same expansions in the same order.
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        uint32_t node = qr.node;
        bool live = !(mindist(load_root_box(t.aabbs + qr.node), p) > best);
        while (live)
        {
            if (!kStats && budget-- == 0)
            {
                deferred = true;
                break;
            }
            Box lb, rb;
            uint32_t L, R;
            unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
            if (kStats)
                ++n_int;
            // no minmaxdist sibling test (query.cuh:279, 297) here: it only removes
            // subtrees whose every triangle is strictly farther than one in the
            // sibling, which a near-first search never needs (same expansions, same
            // answers and tie winners, measured 12 % faster without it)
            const float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
            constexpr bool aL = true, aR = true;
            if (kPrefetchChildren)
            {
                if (aL && L < ni && Lmd <= best)
                    prefetch_l1(t.inner + L);
                if (aR && R < ni && Rmd <= best)
                    prefetch_l1(t.inner + R);
            }
            if (aL && L >= ni && Lmd <= best)
            {
                leaf_nearest_fast(t, L - ni, p, best, best_rank, nearest);
                if (kStats)
                    ++n_leaf;
            }
            if (aR && R >= ni && Rmd <= best)
            {
                leaf_nearest_fast(t, R - ni, p, best, best_rank, nearest);
                if (kStats)
                    ++n_leaf;
            }
            const bool pL = aL && L < ni && Lmd <= best, pR = aR && R < ni && Rmd <= best;
            if (pL && pR)
            {
                if (sp > kStackDepth - 2)
                {
                    atomicOr(t.status, kStatusStackOverflow);
                    nearest = kInvalid;
                    best = NAN;
                    break;
                }
                const bool l_first = Lmd <= Rmd;
                sn[sp] = l_first ? R : L;
                sd[sp] = l_first ? Rmd : Lmd;
                ++sp;
                node = l_first ? L : R;
                continue;
            }
            if (pL || pR)
            {
                node = pL ? L : R;
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
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = 0;
    }
    if (deferred)
    {
        // the bound handed to the second pass: a float whose square is >= best
        seed.defer_radius[q] = best < INFINITY ? nextafterf(sqrtf(best), INFINITY) : INFINITY;
        append_failed(seed.defer_list, seed.defer_count, (uint32_t)q, true);
        return;
    }
    const bool failed = seed.radius && nearest == kInvalid && r0 < INFINITY;
    if (seed.radius && nearest == kInvalid)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    st_out(out_idx + out_pos(t, qi, q), nearest == kInvalid ? kInvalid : nearest - qr.tri_off);
    st_out(out_dist + out_pos(t, qi, q), sqrtf(best));
    if (seed.fail_flag)
        seed.fail_flag[q] = failed ? 1u : 0u;
}

// one leaf of the silhouette query; key = rank * 4 + slot orders candidates
// like the reference's visit order
SNCH_DEV void leaf_silhouette_fast(const TreeView &t, uint32_t pos, f3 o, bool flip, float &best, uint32_t &best_key,
                                   int32_t &best_edge, uint32_t &n_edge)
{
    const float4 *lr = reinterpret_cast<const float4 *>(t.leaves + pos);
    const uint32_t n_owned = __float_as_uint(__ldg(&lr[1].w));
    const uint32_t rank = __float_as_uint(__ldg(&lr[2].w));
    n_edge += n_owned;
    for (uint32_t k = 0; k < n_owned; ++k)
    {
        const float4 *e = reinterpret_cast<const float4 *>(t.edges + 3 * (uint64_t)pos + k);
        const float4 ea = __ldg(e), eb = __ldg(e + 1);
        const f3 pa = mk(ea.x, ea.y, ea.z), pb = mk(eb.x, eb.y, eb.z);
        f3 cp;
        const float sq = closest_point_segment_sq(pa, pb, o, cp);
        if (sq > beyond_sq(best * best))
            continue;  // d > best
        const float d = sqrtf(sq);
        if (d > best)
            continue;
        const uint32_t flags = __float_as_uint(ea.w);
        bool is_sil = (flags & 1u) == 0u || (flags & 2u) == 0u;
        if (!is_sil)
        {
            const float4 ec = __ldg(e + 2), ed = __ldg(e + 3);
            is_sil = is_silhouette_edge(pa, pb, mk(ec.x, ec.y, ec.z), mk(ed.x, ed.y, ed.z),
                                        mk(o.x - cp.x, o.y - cp.y, o.z - cp.z), d, flip);
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

// owned edge k of the leaf at sorted position pos (rank: the leaf's rank) as a
// silhouette candidate
SNCH_DEV void edge_candidate(const TreeView &t, uint32_t pos, uint32_t k, uint32_t rank, f3 o, bool flip, float &best,
                             uint32_t &best_key, int32_t &best_edge)
{
    const float4 *e = reinterpret_cast<const float4 *>(t.edges + 3 * (uint64_t)pos + k);
    const float4 ea = __ldg(e), eb = __ldg(e + 1);
    const f3 pa = mk(ea.x, ea.y, ea.z), pb = mk(eb.x, eb.y, eb.z);
    f3 cp;
    const float sq = closest_point_segment_sq(pa, pb, o, cp);
    if (sq > beyond_sq(best * best))
        return;  // d > best
    const float d = sqrtf(sq);
    if (d > best)
        return;
    const uint32_t flags = __float_as_uint(ea.w);
    bool is_sil = (flags & 1u) == 0u || (flags & 2u) == 0u;
    if (!is_sil)
    {
        const float4 ec = __ldg(e + 2), ed = __ldg(e + 3);
        is_sil = is_silhouette_edge(pa, pb, mk(ec.x, ec.y, ec.z), mk(ed.x, ed.y, ed.z),
                                    mk(o.x - cp.x, o.y - cp.y, o.z - cp.z), d, flip);
    }
    if (!is_sil)
        return;
    const uint32_t key = rank * 4u + k;
    if (d < best || best_edge < 0 || (d > 0.0f ? key > best_key : key < best_key))
    {
        best = d;
        best_key = key;
        best_edge = __float_as_int(eb.w);
    }
}

// the same for a leaf reached through its parent: rank and owned-edge count
// come from the parent's record (InnerRec.d), not from the LeafRec
SNCH_DEV void leaf_silhouette_info(const TreeView &t, uint32_t pos, uint32_t info, f3 o, bool flip, float &best,
                                   uint32_t &best_key, int32_t &best_edge, uint32_t &n_edge)
{
    const uint32_t n_owned = info >> 30;
    const uint32_t rank = info & kLeafRankMask;
    n_edge += n_owned;
    for (uint32_t k = 0; k < n_owned; ++k)
        edge_candidate(t, pos, k, rank, o, flip, best, best_key, best_edge);
}

template <bool kStats, int kBlock = 128>
__global__ void __launch_bounds__(kBlock, 1152 / kBlock) silhouette_fast_kernel(TreeView t, const float *__restrict__ pts,
                                                              const uint8_t *__restrict__ flips, int64_t n,
                                                              float *__restrict__ out_dist,
                                                              int32_t *__restrict__ out_edge,
                                                              uint32_t *__restrict__ stats, SeedArgs seed)
{
    uint32_t n_int = 0, n_leaf = 0, n_edge = 0;
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 p = load_point(pts, q);
    const bool flip = flips ? ld_in(flips + q) != 0 : false;
    const float r0 = seed.radius ? __ldg(seed.radius + q) : INFINITY;
    float best = r0;
    uint32_t best_key = 0;
    int32_t best_edge = -1;
    bool deferred = false;
    uint32_t budget = seed.cap ? seed.cap : 0xFFFFFFFFu;
    const uint32_t ni = t.num_tris - 1;
    const QueryRoot qr = query_root(t, q);
    if (qr.node == kInvalid)
    {
    }
    else if (qr.node >= ni)  // a one-triangle tree or mesh
        leaf_silhouette_fast(t, qr.node - ni, p, flip, best, best_key, best_edge, n_edge);
    else
    {
        // nearer passing child next, farther one on the stack (as nearest_fast_kernel)
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        uint32_t node = qr.node;
        bool live = !(mindist(load_root_box(t.aabbs + qr.node), p) > best * best);
        while (live)
        {
            if (!kStats && budget-- == 0)
            {
                deferred = true;
                break;
            }
            Box lb, rb;
            uint32_t L, R, Linfo, Rinfo;
            const InnerRec rec = load_inner(t.inner + node);
            unpack_inner(rec, lb, rb, L, R);
            unpack_leaf_info(rec, Linfo, Rinfo);
            const float4 *cr = reinterpret_cast<const float4 *>(t.inner_cones + node);
            InnerConeRec icr;
            icr.a = __ldg(cr);
            icr.b = __ldg(cr + 1);
            icr.c = __ldg(cr + 2);
            Cone lc, rc;
            unpack_cones(icr, lc, rc);
            const float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
            const float b2 = best * best;
            const bool hitL = Lmd <= b2 && lc.half_angle >= 0.0f && cone_test(lc, p, lb, Lmd);
            const bool hitR = Rmd <= b2 && rc.half_angle >= 0.0f && cone_test(rc, p, rb, Rmd);
            if (kStats)
                ++n_int;
            if (kPrefetchChildren)
            {
                if (hitL && L < ni)
                {
                    prefetch_l1(t.inner + L);
                    prefetch_l1(t.inner_cones + L);
                }
                if (hitR && R < ni)
                {
                    prefetch_l1(t.inner + R);
                    prefetch_l1(t.inner_cones + R);
                }
            }
            if (hitL && L >= ni)
            {
                leaf_silhouette_info(t, L - ni, Linfo, p, flip, best, best_key, best_edge, n_edge);
                if (kStats)
                    ++n_leaf;
            }
            if (hitR && R >= ni)
            {
                leaf_silhouette_info(t, R - ni, Rinfo, p, flip, best, best_key, best_edge, n_edge);
                if (kStats)
                    ++n_leaf;
            }
            const float b2n = best * best;
            const bool pL = hitL && L < ni && Lmd <= b2n, pR = hitR && R < ni && Rmd <= b2n;
            if (pL && pR)
            {
                if (sp > kStackDepth - 2)
                {
                    atomicOr(t.status, kStatusStackOverflow);
                    best = NAN;
                    best_edge = -1;
                    break;
                }
                const bool l_first = Lmd <= Rmd;
                sn[sp] = l_first ? R : L;
                sd[sp] = l_first ? Rmd : Lmd;
                ++sp;
                node = l_first ? L : R;
                continue;
            }
            if (pL || pR)
            {
                node = pL ? L : R;
                continue;
            }
            live = false;
            while (sp > 0)
            {
                --sp;
                if (!(sd[sp] > best * best))
                {
                    node = sn[sp];
                    live = true;
                    break;
                }
            }
        }
    }
    if (deferred)
    {
        seed.defer_radius[q] = best;  // best candidate so far, or the seed radius
        append_failed(seed.defer_list, seed.defer_count, (uint32_t)q, true);
        return;
    }
    const bool failed = seed.radius && best_edge < 0 && r0 < INFINITY;
    if (seed.radius && best_edge < 0)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    st_out(out_dist + out_pos(t, qi, q), best);
    if (out_edge)
        st_out(out_edge + out_pos(t, qi, q), best_edge < 0 ? best_edge : best_edge - qr.edge_off);
    if (seed.fail_flag)
        seed.fail_flag[q] = failed ? 1u : 0u;
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = n_edge;
    }
}

// ------------------------------------------------------------------ wide nodes
// Near-first searches over 4- or 8-way records (WideLayout): one expansion
// reads a record of k = 2 or 3 binary levels as consecutive 16-B loads. At
// every collapsed level the search applies the test the binary search applies
// there -- nearest: a child is kept iff its mindist <= its sibling's
// minmaxdist (query.cuh:279, 297); silhouette: iff its cone is valid, its
// mindist <= best^2 and the cone test passes (query.cuh:356-381) -- so it
// reaches the leaves the binary search reaches, and the answer (the minimum
// over them, exact ties broken by the leaf's rank in the reference's order)
// is the binary search's. Pruning by the running best (mindist > best, strict)
// is applied where it is cheap; it never removes a leaf that attains the
// minimum, so where it is applied does not change the answer.

// resident blocks per SM of the wide kernels (measured on the 2M-triangle
// scene: 10 beats 8 and 12 for both widths)
#ifndef SNCH_WIDE_MIN_BLOCKS
#define SNCH_WIDE_MIN_BLOCKS 10
#endif

// ascending compare-exchange on (key, value) pairs held in registers
SNCH_DEV void cas_pair(float &ka, uint32_t &va, float &kb, uint32_t &vb)
{
    if (kb < ka)
    {
        const float tk = ka;
        ka = kb;
        kb = tk;
        const uint32_t tv = va;
        va = vb;
        vb = tv;
    }
}
// sorting networks: 5 comparators for 4 keys, Batcher's 19 for 8
template <int W>
SNCH_DEV void sort_children(float (&k)[W], uint32_t (&v)[W])
{
    if constexpr (W == 4)
    {
        cas_pair(k[0], v[0], k[1], v[1]);
        cas_pair(k[2], v[2], k[3], v[3]);
        cas_pair(k[0], v[0], k[2], v[2]);
        cas_pair(k[1], v[1], k[3], v[3]);
        cas_pair(k[1], v[1], k[2], v[2]);
    }
    else
    {
        constexpr int net[19][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3}, {4, 6}, {5, 7}, {1, 2}, {5, 6},
                                    {0, 4}, {1, 5}, {2, 6}, {3, 7}, {2, 4}, {3, 5}, {1, 2}, {3, 4}, {5, 6}};
#pragma unroll
        for (int c = 0; c < 19; ++c)
            cas_pair(k[net[c][0]], v[net[c][0]], k[net[c][1]], v[net[c][1]]);
    }
}

// box / cone of slot-tree position f (scalar loads; the record's lines are in L1)
template <int W>
SNCH_DEV Box wide_box(const float4 *__restrict__ rec, int f)
{
    constexpr int P = WideLayout<W>::P;
    const float *x = reinterpret_cast<const float *>(rec) + f;
    Box b;
    b.lower = mk(__ldg(x), __ldg(x + P), __ldg(x + 2 * P));
    b.upper = mk(__ldg(x + 3 * P), __ldg(x + 4 * P), __ldg(x + 5 * P));
    return b;
}
template <int W>
SNCH_DEV Cone wide_cone(const float4 *__restrict__ rec, int f)
{
    constexpr int P = WideLayout<W>::P;
    const float *x = reinterpret_cast<const float *>(rec) + WideLayout<W>::kCone + f;
    Cone c;
    c.axis = mk(__ldg(x), __ldg(x + P), __ldg(x + 2 * P));
    c.half_angle = __ldg(x + 3 * P);
    c.radius = __ldg(x + 4 * P);
    return c;
}

template <int W>
SNCH_DEV void wide_child_ids(const float4 *__restrict__ rec, uint32_t (&ch)[W], uint32_t (&info)[W])
{
    using Lay = WideLayout<W>;
    const uint4 *c4 = reinterpret_cast<const uint4 *>(reinterpret_cast<const float *>(rec) + Lay::kChild);
    const uint4 *i4 = reinterpret_cast<const uint4 *>(reinterpret_cast<const float *>(rec) + Lay::kInfo);
#pragma unroll
    for (int q4 = 0; q4 < W / 4; ++q4)
    {
        const uint4 c = __ldg(c4 + q4), i = __ldg(i4 + q4);
        ch[4 * q4 + 0] = c.x;
        ch[4 * q4 + 1] = c.y;
        ch[4 * q4 + 2] = c.z;
        ch[4 * q4 + 3] = c.w;
        info[4 * q4 + 0] = i.x;
        info[4 * q4 + 1] = i.y;
        info[4 * q4 + 2] = i.z;
        info[4 * q4 + 3] = i.w;
    }
}

// Nearest: the sibling tests of every slot-tree position, four positions per
// group of 16-B loads (siblings never straddle a group). Returns the accepted
// positions as a bit mask and the children's squared mindist in md.
template <int W>
SNCH_DEV uint32_t wide_nearest_tests(const float4 *__restrict__ rec, f3 p, float (&md)[W])
{
    using Lay = WideLayout<W>;
    constexpr int Q = Lay::P / 4;
    uint32_t acc = 0;
#pragma unroll
    for (int g = 0; g < Q; ++g)
    {
        if (4 * g >= Lay::F)
            break;
        const float4 lx = __ldg(rec + 0 * Q + g), ly = __ldg(rec + 1 * Q + g), lz = __ldg(rec + 2 * Q + g);
        const float4 hx = __ldg(rec + 3 * Q + g), hy = __ldg(rec + 4 * Q + g), hz = __ldg(rec + 5 * Q + g);
        const float lxa[4] = {lx.x, lx.y, lx.z, lx.w}, lya[4] = {ly.x, ly.y, ly.z, ly.w},
                    lza[4] = {lz.x, lz.y, lz.z, lz.w};
        const float hxa[4] = {hx.x, hx.y, hx.z, hx.w}, hya[4] = {hy.x, hy.y, hy.z, hy.w},
                    hza[4] = {hz.x, hz.y, hz.z, hz.w};
        float gmd[4], gmm[4];
#pragma unroll
        for (int c = 0; c < 4; ++c)
        {
            Box b;
            b.lower = mk(lxa[c], lya[c], lza[c]);
            b.upper = mk(hxa[c], hya[c], hza[c]);
            gmd[c] = mindist(b, p);
            gmm[c] = minmaxdist(b, p);
        }
#pragma unroll
        for (int c = 0; c < 4; c += 2)
        {
            const int f = 4 * g + c;
            if (f >= Lay::F)
                break;
            const bool pok = f < 2 || ((acc >> (((f + 2) >> 1) - 2)) & 1u);
            acc |= (uint32_t)(pok && gmd[c] <= gmm[c + 1]) << f;
            acc |= (uint32_t)(pok && gmd[c + 1] <= gmm[c]) << (f + 1);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
        {
            const int f = 4 * g + c;
            if (f >= Lay::S0 && f < Lay::S0 + W)
                md[f - Lay::S0] = gmd[c];
        }
    }
    return acc >> Lay::S0;
}

// After the leaves of a record: continue with the nearest accepted internal
// child, push the others (farthest deepest). key[i] = mindist of an accepted
// internal child, val[i] = its wide index, kInvalid for the rest. Returns false
// when the stack is full.
template <int W, int S>
SNCH_DEV bool wide_descend(float (&key)[W], uint32_t (&val)[W], uint32_t (&sn)[S], float (&sd)[S], int &sp,
                           uint32_t &next)
{
    sort_children<W>(key, val);
    next = kInvalid;
#pragma unroll
    for (int i = 0; i < W; ++i)
        if (next == kInvalid && val[i] != kInvalid)
            next = val[i];
#pragma unroll
    for (int i = W - 1; i >= 0; --i)
    {
        if (val[i] != kInvalid && val[i] != next)
        {
            if (sp >= S)
                return false;
            sn[sp] = val[i];
            sd[sp] = key[i];
            ++sp;
        }
    }
    return true;
}

template <int W, bool kStats>
__global__ void __launch_bounds__(128, SNCH_WIDE_MIN_BLOCKS)
    nearest_wide_kernel(TreeView t, const float *__restrict__ pts, int64_t n, uint32_t *__restrict__ out_idx,
                        float *__restrict__ out_dist, uint32_t *__restrict__ stats, SeedArgs seed)
{
    using Lay = WideLayout<W>;
    uint32_t n_int = 0, n_leaf = 0;
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 p = load_point(pts, q);
    uint32_t nearest = kInvalid, best_rank = 0;
    float best = INFINITY, r0 = INFINITY;
    if (seed.radius)
    {
        r0 = __ldg(seed.radius + q);
        best = r0 * r0;
    }
    const uint32_t ni = t.num_tris - 1;
    const float4 *__restrict__ recs = W == 4 ? t.wide4 : t.wide8;
    const QueryRoot qr = query_root(t, q);
    if (qr.node == kInvalid)
    {
    }
    else if (qr.node >= ni)  // a one-triangle tree or mesh
        leaf_nearest_fast(t, qr.node - ni, p, best, best_rank, nearest);
    else
    {
        uint32_t sn[Lay::kStack];
        float sd[Lay::kStack];
        int sp = 0;
        uint32_t node = __ldg((W == 4 ? t.wide4_of : t.wide8_of) + qr.node);
        bool live = !(mindist(load_root_box(t.aabbs + qr.node), p) > best);
        while (live)
        {
            const float4 *rec = recs + (size_t)node * Lay::kRecF4;
            float md[W];
            const uint32_t acc = wide_nearest_tests<W>(rec, p, md);
            uint32_t ch[W], info[W];
            wide_child_ids<W>(rec, ch, info);
            if (kStats)
                ++n_int;
#pragma unroll
            for (int i = 0; i < W; ++i)
            {
                if (((acc >> i) & 1u) && ch[i] != kInvalid && (ch[i] & kWideLeaf) && md[i] <= best)
                {
                    leaf_nearest_fast(t, ch[i] & ~kWideLeaf, p, best, best_rank, nearest);
                    if (kStats)
                        ++n_leaf;
                }
            }
            float key[W];
            uint32_t val[W];
#pragma unroll
            for (int i = 0; i < W; ++i)
            {
                const bool ok = ((acc >> i) & 1u) && ch[i] != kInvalid && !(ch[i] & kWideLeaf) && md[i] <= best;
                key[i] = ok ? md[i] : INFINITY;
                val[i] = ok ? ch[i] : kInvalid;
            }
            uint32_t next;
            if (!wide_descend<W, Lay::kStack>(key, val, sn, sd, sp, next))
            {
                atomicOr(t.status, kStatusStackOverflow);
                nearest = kInvalid;
                best = NAN;
                break;
            }
            if (next != kInvalid)
            {
                node = next;
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
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = 0;
    }
    const bool failed = seed.radius && nearest == kInvalid && r0 < INFINITY;
    if (seed.radius && nearest == kInvalid)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    st_out(out_idx + out_pos(t, qi, q), nearest == kInvalid ? kInvalid : nearest - qr.tri_off);
    st_out(out_dist + out_pos(t, qi, q), sqrtf(best));
    if (seed.fail_flag)
        seed.fail_flag[q] = failed ? 1u : 0u;
}

template <int W, bool kStats>
__global__ void __launch_bounds__(128, SNCH_WIDE_MIN_BLOCKS)
    silhouette_wide_kernel(TreeView t, const float *__restrict__ pts, const uint8_t *__restrict__ flips, int64_t n,
                           float *__restrict__ out_dist, int32_t *__restrict__ out_edge, uint32_t *__restrict__ stats,
                           SeedArgs seed)
{
    using Lay = WideLayout<W>;
    uint32_t n_int = 0, n_leaf = 0, n_edge = 0;
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 p = load_point(pts, q);
    const bool flip = flips ? ld_in(flips + q) != 0 : false;
    const float r0 = seed.radius ? __ldg(seed.radius + q) : INFINITY;
    float best = r0;
    uint32_t best_key = 0;
    int32_t best_edge = -1;
    const uint32_t ni = t.num_tris - 1;
    const float4 *__restrict__ recs = W == 4 ? t.wide4 : t.wide8;
    const QueryRoot qr = query_root(t, q);
    if (qr.node == kInvalid)
    {
    }
    else if (qr.node >= ni)  // a one-triangle tree or mesh
        leaf_silhouette_fast(t, qr.node - ni, p, flip, best, best_key, best_edge, n_edge);
    else
    {
        uint32_t sn[Lay::kStack];
        float sd[Lay::kStack];
        int sp = 0;
        uint32_t node = __ldg((W == 4 ? t.wide4_of : t.wide8_of) + qr.node);
        bool live = !(mindist(load_root_box(t.aabbs + qr.node), p) > best * best);
        while (live)
        {
            const float4 *rec = recs + (size_t)node * Lay::kRecF4;
            const float b2 = best * best;
            // slot-tree positions in level order (a rolled loop: one inlined cone
            // test); a position is tested only if its parent position passed;
            // empty positions fail through their invalid cone, pass positions pass
            uint32_t acc = 0;
#pragma unroll 1
            for (int f = 0; f < Lay::F; ++f)
            {
                if (f >= 2 && !((acc >> (((f + 2) >> 1) - 2)) & 1u))
                    continue;
                const Box b = wide_box<W>(rec, f);
                const float m = mindist(b, p);
                if (m <= b2)
                {
                    const Cone cn = wide_cone<W>(rec, f);
                    if (cn.half_angle >= 0.0f && cone_test(cn, p, b, m))
                        acc |= 1u << f;
                }
            }
            const uint32_t hits = acc >> Lay::S0;
            uint32_t ch[W], info[W];
            wide_child_ids<W>(rec, ch, info);
            if (kStats)
                ++n_int;
#pragma unroll
            for (int i = 0; i < W; ++i)
            {
                if (((hits >> i) & 1u) && (ch[i] & kWideLeaf))
                {
                    leaf_silhouette_info(t, ch[i] & ~kWideLeaf, info[i], p, flip, best, best_key, best_edge, n_edge);
                    if (kStats)
                        ++n_leaf;
                }
            }
            const float b2n = best * best;
            float key[W];
            uint32_t val[W];
#pragma unroll
            for (int i = 0; i < W; ++i)
            {
                key[i] = INFINITY;
                val[i] = kInvalid;
                if (((hits >> i) & 1u) && !(ch[i] & kWideLeaf))
                {
                    const float m = mindist(wide_box<W>(rec, Lay::S0 + i), p);
                    if (m <= b2n)
                    {
                        key[i] = m;
                        val[i] = ch[i];
                    }
                }
            }
            uint32_t next;
            if (!wide_descend<W, Lay::kStack>(key, val, sn, sd, sp, next))
            {
                atomicOr(t.status, kStatusStackOverflow);
                best = NAN;
                best_edge = -1;
                break;
            }
            if (next != kInvalid)
            {
                node = next;
                continue;
            }
            live = false;
            while (sp > 0)
            {
                --sp;
                if (!(sd[sp] > best * best))
                {
                    node = sn[sp];
                    live = true;
                    break;
                }
            }
        }
    }
    const bool failed = seed.radius && best_edge < 0 && r0 < INFINITY;
    if (seed.radius && best_edge < 0)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    st_out(out_dist + out_pos(t, qi, q), best);
    if (out_edge)
        st_out(out_edge + out_pos(t, qi, q), best_edge < 0 ? best_edge : best_edge - qr.edge_off);
    if (seed.fail_flag)
        seed.fail_flag[q] = failed ? 1u : 0u;
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = n_edge;
    }
}

// ------------------------------------------------------------------ warp packets
// Packet forms of the near-first nearest / silhouette searches (SNCH_OPT_PACKET):
// the 32 queries of a warp -- neighbours, when the batch is Morton-ordered --
// walk ONE traversal together. The warp keeps one stack of (node, lane mask)
// entries in shared memory; at a node every lane whose bit is set applies its
// own tests to the two children (the record is one broadcast load), the
// ballots of the lanes that keep each child become the children's masks, and a
// leaf is evaluated by the lanes that keep it. A lane therefore reaches the
// leaves its own per-lane search reaches, with the same tests (cone tests,
// pruning by its own best), and its answer -- the minimum over them, ties
// broken by leaf rank -- is the per-lane answer. The
// warp visits the union of its lanes' nodes, in the order most of them prefer,
// with every control decision uniform across the warp.

constexpr int kPacketWarps = 4;  // 128-thread blocks

// ---- packet pools per SM
// The persistent packet searches hand out packets (32 consecutive queries of the
// batch) through a pool per SM: a pool holds a chunk of kPoolChunk consecutive
// packets taken from the batch-wide counter, and the warps of that SM take its
// packets one at a time, refilling it from the counter when it is used up. At
// any moment the SMs work on neighbouring chunks of the Morton-ordered batch (a
// window as narrow as with one counter), and the warps of one SM on neighbouring
// packets, so they also share the tree records in that SM's L1. 16M-query
// batches of the 2M-triangle scene: nearest 12.04 -> 11.42 ms, silhouette 35.63
// -> 34.61 ms (chunks of 16 / 64 / 128 packets: 11.51 / 11.46 / 11.47 and 34.82 /
// 34.60 / 34.96 ms). Which SM a warp runs on only decides which pool it uses,
// never which packets exist: every packet of the batch is taken exactly once.
// Pool word: (first packet of the chunk + 1) << 24 | packets taken; 0 = empty,
// kPoolDone << 24 = the batch is handed out.
#ifndef SNCH_PACKET_POOLS
#define SNCH_PACKET_POOLS 1
#endif
constexpr bool kPacketPools = SNCH_PACKET_POOLS != 0;  // 0: every packet straight from the counter
constexpr uint32_t kPoolSlots = 1024;                  // pools (SM id modulo kPoolSlots)
#ifndef SNCH_POOL_CHUNK
#define SNCH_POOL_CHUNK 32
#endif
constexpr uint64_t kPoolChunk = SNCH_POOL_CHUNK;  // packets per refill
constexpr unsigned long long kPoolDone = (1ull << 40) - 1ull;
constexpr uint32_t kPoolSpins = 1u << 16;
// work[0]: the batch-wide packet counter, work[1 + s]: pool s (zeroed before
// the launch). Returns a packet index (>= total_packets: the unused end of the
// last chunk, take again; at most kPoolChunk of those before the pool is done)
// or ~0 when every packet has been handed out.
__device__ __noinline__ unsigned long long take_packet(unsigned long long *work, unsigned long long total_packets)
{
    if (!kPacketPools)
    {
        const unsigned long long p = atomicAdd(work, 1ull);
        return p < total_packets ? p : ~0ull;
    }
    uint32_t smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    unsigned long long *pool = work + 1 + (smid & (kPoolSlots - 1u));
    for (uint32_t spin = 0; spin < kPoolSpins; ++spin)
    {
        const unsigned long long old = atomicAdd(pool, 1ull);
        const unsigned long long first = old >> 24, taken = old & 0xFFFFFFull;
        if (first == kPoolDone)
            return ~0ull;
        if (first != 0 && taken < kPoolChunk)
            return first - 1 + taken;
        // the first taker of an empty pool, or the one just past the end of its
        // chunk, refills it; the others take again after the refill
        if ((first == 0 && taken == 0) || (first != 0 && taken == kPoolChunk))
        {
            const unsigned long long next = atomicAdd(work, kPoolChunk);
            atomicExch(pool, next < total_packets ? (next + 1) << 24 : kPoolDone << 24);
        }
    }
    // a pool that stayed busy this long: one packet from the counter (the pool's
    // remaining packets go to the other warps of the SM)
    const unsigned long long p = atomicAdd(work, 1ull);
    return p < total_packets ? p : ~0ull;
}

// per-lane start of a packet: lanes of a batched query set may search
// different meshes; the warp runs one packet per distinct root
struct PacketLane
{
    bool valid;
    int64_t q;
    f3 p;
    QueryRoot qr;
};

// one warp's packet: the 32 queries qi .. qi + 31 (lane order) of the batch
// Top levels (kTop): the node's heap slot travels with it (slot of a child:
// 2 s + 1 / 2 s + 2), and a node whose slot is below top_slots is read from the
// shared-memory copy s_top instead of global memory; kNoSlot below the top.
constexpr uint32_t kNoSlot = 0xFFu;
SNCH_DEV uint32_t child_slot(uint32_t slot, uint32_t k, uint32_t top_slots)
{
    const uint32_t c = 2u * slot + 1u + k;
    return slot < top_slots && c < top_slots ? c : kNoSlot;
}

template <bool kStats, bool kTop = false>
SNCH_DEV void nearest_packet_chunk(const TreeView &t, const float *__restrict__ pts, int64_t n,
                                   uint32_t *__restrict__ out_idx, float *__restrict__ out_dist,
                                   uint32_t *__restrict__ stats, const SeedArgs &seed, int64_t qi, uint32_t *st_node,
                                   uint32_t *st_mask, uint8_t *st_slot = nullptr, const InnerRec *s_top = nullptr,
                                   uint32_t top_slots = 0)
{
    const int lane = threadIdx.x & 31;
    const bool valid = qi < query_count(t, n);
    if (__ballot_sync(0xffffffffu, valid) == 0u)
        return;
    const int64_t q = valid ? query_index(t, qi) : 0;
    const f3 p = valid ? load_point(pts, q) : mk(0.0f, 0.0f, 0.0f);
    uint32_t nearest = kInvalid, best_rank = 0, n_int = 0, n_leaf = 0;
    float best = INFINITY, r0 = INFINITY;
    if (valid && seed.radius)
    {
        r0 = __ldg(seed.radius + q);
        best = r0 * r0;
    }
    const uint32_t ni = t.num_tris - 1;
    QueryRoot qr = valid ? query_root(t, q) : QueryRoot{kInvalid, 0u, 0};
    if (valid && qr.node != kInvalid && qr.node >= ni)  // a one-triangle tree or mesh
        leaf_nearest_fast(t, qr.node - ni, p, best, best_rank, nearest);
    bool overflow = false;
    uint32_t pending = __ballot_sync(0xffffffffu, valid && qr.node != kInvalid && qr.node < ni);
    while (pending)
    {
        const int leader = __ffs(pending) - 1;
        const uint32_t root = __shfl_sync(0xffffffffu, qr.node, leader);
        const uint32_t mine = __ballot_sync(0xffffffffu, ((pending >> lane) & 1u) && qr.node == root);
        pending &= ~mine;
        bool in = (mine >> lane) & 1u;
        if (in)
            in = !(mindist(load_root_box(t.aabbs + root), p) > best);
        uint32_t mask = __ballot_sync(0xffffffffu, in);
        uint32_t node = root;
        uint32_t slot = kTop && root == 0u && !t.query_mesh ? 0u : kNoSlot;
        int sp = 0;
        while (true)
        {
            if (mask == 0u)
            {
                if (sp == 0)
                    break;
                --sp;
                node = st_node[sp];
                mask = st_mask[sp];
                if (kTop)
                    slot = st_slot[sp];
                continue;
            }
            const bool act = (mask >> lane) & 1u;
            Box lb, rb;
            uint32_t L, R;
            unpack_inner(kTop && slot < top_slots ? s_top[slot] : load_inner(t.inner + node), lb, rb, L, R);
            float Lmd = INFINITY, Rmd = INFINITY;
            bool aL = false, aR = false;
            if (act)
            {
                if (kStats)
                    ++n_int;
                Lmd = mindist(lb, p);
                Rmd = mindist(rb, p);
                aL = aR = true;  // no minmaxdist sibling test: as nearest_fast_kernel
                // two branches: one loop over both leaves (as the silhouette packets
                // run them) measured 12 % slower here (16M queries, 13.43 vs 12.02 ms)
                if (aL && L >= ni && Lmd <= best)
                {
                    leaf_nearest_fast(t, L - ni, p, best, best_rank, nearest);
                    if (kStats)
                        ++n_leaf;
                }
                if (aR && R >= ni && Rmd <= best)
                {
                    leaf_nearest_fast(t, R - ni, p, best, best_rank, nearest);
                    if (kStats)
                        ++n_leaf;
                }
            }
            const uint32_t pL = __ballot_sync(0xffffffffu, aL && L < ni && Lmd <= best);
            const uint32_t pR = __ballot_sync(0xffffffffu, aR && R < ni && Rmd <= best);
            const uint32_t votes = __ballot_sync(0xffffffffu, act && Lmd <= Rmd) & (pL | pR);
            if (pL && pR)
            {
                if (sp >= kStackDepth)
                {
                    overflow = true;
                    break;
                }
                const bool l_first = 2 * __popc(votes) >= __popc(pL | pR);
                __syncwarp();  // every lane has read the slot it may reuse
                if (lane == 0)
                {
                    st_node[sp] = l_first ? R : L;
                    st_mask[sp] = l_first ? pR : pL;
                    if (kTop)
                        st_slot[sp] = (uint8_t)child_slot(slot, l_first ? 1u : 0u, top_slots);
                }
                __syncwarp();
                ++sp;
                node = l_first ? L : R;
                mask = l_first ? pL : pR;
                if (kTop)
                    slot = child_slot(slot, l_first ? 0u : 1u, top_slots);
            }
            else if (pL | pR)
            {
                node = pL ? L : R;
                mask = pL ? pL : pR;
                if (kTop)
                    slot = child_slot(slot, pL ? 0u : 1u, top_slots);
            }
            else
                mask = 0u;
        }
        if (overflow)
            break;
    }
    if (overflow)
    {
        if (lane == 0)
            atomicOr(t.status, kStatusStackOverflow);
        nearest = kInvalid;
        best = NAN;
    }
    if (!valid)
        return;
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = 0;
    }
    const bool failed = seed.radius && nearest == kInvalid && r0 < INFINITY;
    if (seed.radius && nearest == kInvalid)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    st_out(out_idx + out_pos(t, qi, q), nearest == kInvalid ? kInvalid : nearest - qr.tri_off);
    st_out(out_dist + out_pos(t, qi, q), sqrtf(best));
    if (seed.fail_flag)
        seed.fail_flag[q] = failed ? 1u : 0u;}

template <bool kStats>
__global__ void __launch_bounds__(128, 10) nearest_packet_kernel(TreeView t, const float *__restrict__ pts, int64_t n,
                                                             uint32_t *__restrict__ out_idx,
                                                             float *__restrict__ out_dist,
                                                             uint32_t *__restrict__ stats, SeedArgs seed)
{
    __shared__ uint32_t st_node[kPacketWarps][kStackDepth];
    __shared__ uint32_t st_mask[kPacketWarps][kStackDepth];
    const int w = threadIdx.x >> 5;
    nearest_packet_chunk<kStats>(t, pts, n, out_idx, out_dist, stats, seed,
                                 blockIdx.x * (int64_t)blockDim.x + threadIdx.x, st_node[w], st_mask[w]);
}

// ---- top tree levels staged in shared memory (TMA bulk copies)
// The block's first thread copies the heap-ordered top-level records (and, for
// silhouettes, their cones) from global memory with cp.async.bulk, completing on
// an mbarrier that every thread waits on with a bounded poll. If the copy does
// not complete in time the block sets kStatusCopyTimeout, waits once more
// (bounded) for it, and searches from global memory (same answers).
constexpr uint32_t kCopyPolls = 1u << 22;
SNCH_DEV uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
SNCH_DEV void bulk_copy_to_smem(void *dst, const void *src, uint32_t bytes, uint64_t *mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(mbar))
                 : "memory");
}
SNCH_DEV bool mbar_wait_parity(uint64_t *mbar, uint32_t parity, uint32_t polls)
{
    for (uint32_t i = 0; i < polls; ++i)
    {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(mbar)), "r"(parity)
            : "memory");
        if (done)
            return true;
    }
    return false;
}
// returns the number of top slots this block may read from shared memory (0 on a timeout)
SNCH_DEV uint32_t stage_top_levels(const TreeView &t, InnerRec *s_top, InnerConeRec *s_topc, uint64_t *mbar)
{
    if (threadIdx.x == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const uint32_t bi = t.top_slots * (uint32_t)sizeof(InnerRec);
    const uint32_t bc = s_topc ? t.top_slots * (uint32_t)sizeof(InnerConeRec) : 0u;
    if (threadIdx.x == 0)
    {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bi + bc)
                     : "memory");
        bulk_copy_to_smem(s_top, t.top_inner, bi, mbar);
        if (bc)
            bulk_copy_to_smem(s_topc, t.top_cones, bc, mbar);
    }
    const bool ok = __syncthreads_and(mbar_wait_parity(mbar, 0, kCopyPolls));
    if (ok)
        return t.top_slots;
    if (threadIdx.x == 0)
        atomicOr(t.status, kStatusCopyTimeout);
    __syncthreads_and(mbar_wait_parity(mbar, 0, kCopyPolls));  // the copy must not outlive the block
    return 0;
}
inline size_t top_smem_bytes(uint32_t slots, bool cones)
{
    return (size_t)slots * (sizeof(InnerRec) + (cones ? sizeof(InnerConeRec) : 0));
}

// the same packets, persistent: each warp takes its next packet (32 queries
// of the batch) from its SM's pool (take_packet) when its packet is done, so no
// warp slot waits for the slowest packet of its block. kTop: the top tree levels are read
// from a shared-memory copy (dynamic shared memory, top_smem_bytes).
// blocks per SM the persistent nearest packet kernel is compiled for (at least
// 7: the compiler then takes 63 registers, so 8 blocks fit; measured on
// 16M-query batches of the 2M-triangle scene with the per-SM packet pools:
// 10.83 ms, against 11.05 compiled for 8 blocks (64 registers), 11.27 for 9 /
// 56 and 11.82 for 10 / 48, where its loop state spills)
#ifndef SNCH_NEAR_PACKET_MIN_BLOCKS
#define SNCH_NEAR_PACKET_MIN_BLOCKS 7
#endif
template <bool kTop>
__global__ void __launch_bounds__(128, SNCH_NEAR_PACKET_MIN_BLOCKS)
    nearest_packet_persistent_kernel(TreeView t, const float *__restrict__ pts, int64_t n, uint32_t *__restrict__ out_idx,
                                     float *__restrict__ out_dist, SeedArgs seed, unsigned long long *counter)
{
    __shared__ uint32_t st_node[kPacketWarps][kStackDepth];
    __shared__ uint32_t st_mask[kPacketWarps][kStackDepth];
    __shared__ uint8_t st_slot[kPacketWarps][kStackDepth];
    __shared__ uint64_t mbar;
    extern __shared__ __align__(128) unsigned char s_dyn[];
    InnerRec *s_top = reinterpret_cast<InnerRec *>(s_dyn);
    const uint32_t top_slots = kTop ? stage_top_levels(t, s_top, nullptr, &mbar) : 0u;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned long long total = (unsigned long long)query_count(t, n);
    uint32_t empty_takes = 0;
    for (;;)
    {
        unsigned long long packet = 0;
        if (lane == 0)
            packet = take_packet(counter, (total + 31ull) / 32ull);
        packet = __shfl_sync(0xffffffffu, packet, 0);
        if (packet == ~0ull)
            break;
        if (packet >= (total + 31ull) / 32ull)
        {
            if (++empty_takes > kPoolSpins)  // cannot happen: see take_packet
            {
                if (lane == 0)
                    atomicOr(t.status, kStatusWorkTimeout);
                break;
            }
            continue;
        }
        empty_takes = 0;
        const unsigned long long base = packet * 32ull;
        nearest_packet_chunk<false, kTop>(t, pts, n, out_idx, out_dist, nullptr, seed, (int64_t)base + lane,
                                          st_node[w], st_mask[w], st_slot[w], s_top, top_slots);
        __syncwarp();
    }
}

// one warp's packet: the 32 queries qi .. qi + 31 (lane order) of the batch
template <bool kStats, bool kTop = false>
SNCH_DEV void silhouette_packet_chunk(const TreeView &t, const float *__restrict__ pts, const uint8_t *__restrict__ flips,
                                      int64_t n, float *__restrict__ out_dist, int32_t *__restrict__ out_edge,
                                      uint32_t *__restrict__ stats, const SeedArgs &seed, int64_t qi,
                                      uint32_t *st_node, uint32_t *st_mask, uint8_t *st_slot = nullptr,
                                      const InnerRec *s_top = nullptr, const InnerConeRec *s_topc = nullptr,
                                      uint32_t top_slots = 0)
{
    const int lane = threadIdx.x & 31;
    const bool valid = qi < query_count(t, n);
    if (__ballot_sync(0xffffffffu, valid) == 0u)
        return;
    const int64_t q = valid ? query_index(t, qi) : 0;
    const f3 p = valid ? load_point(pts, q) : mk(0.0f, 0.0f, 0.0f);
    const bool flip = valid && flips ? ld_in(flips + q) != 0 : false;
    const float r0 = valid && seed.radius ? __ldg(seed.radius + q) : INFINITY;
    float best = r0;
    uint32_t best_key = 0, n_int = 0, n_leaf = 0, n_edge = 0;
    int32_t best_edge = -1;
    const uint32_t ni = t.num_tris - 1;
    QueryRoot qr = valid ? query_root(t, q) : QueryRoot{kInvalid, 0u, 0};
    if (valid && qr.node != kInvalid && qr.node >= ni)  // a one-triangle tree or mesh
        leaf_silhouette_fast(t, qr.node - ni, p, flip, best, best_key, best_edge, n_edge);
    bool overflow = false;
    uint32_t pending = __ballot_sync(0xffffffffu, valid && qr.node != kInvalid && qr.node < ni);
    while (pending)
    {
        const int leader = __ffs(pending) - 1;
        const uint32_t root = __shfl_sync(0xffffffffu, qr.node, leader);
        const uint32_t mine = __ballot_sync(0xffffffffu, ((pending >> lane) & 1u) && qr.node == root);
        pending &= ~mine;
        bool in = (mine >> lane) & 1u;
        if (in)
            in = !(mindist(load_root_box(t.aabbs + root), p) > best * best);
        uint32_t mask = __ballot_sync(0xffffffffu, in);
        uint32_t node = root;
        uint32_t slot = kTop && root == 0u && !t.query_mesh ? 0u : kNoSlot;
        int sp = 0;
        while (true)
        {
            if (mask == 0u)
            {
                if (sp == 0)
                    break;
                --sp;
                node = st_node[sp];
                mask = st_mask[sp];
                if (kTop)
                    slot = st_slot[sp];
                continue;
            }
            const bool act = (mask >> lane) & 1u;
            const bool in_top = kTop && slot < top_slots;
            Box lb, rb;
            uint32_t L, R, Linfo, Rinfo;
            const InnerRec rec = in_top ? s_top[slot] : load_inner(t.inner + node);
            unpack_inner(rec, lb, rb, L, R);
            unpack_leaf_info(rec, Linfo, Rinfo);
            float Lmd = INFINITY, Rmd = INFINITY;
            bool hitL = false, hitR = false;
            if (act)
            {
                if (kStats)
                    ++n_int;
                InnerConeRec icr;
                if (in_top)
                    icr = s_topc[slot];
                else
                {
                    const float4 *cr = reinterpret_cast<const float4 *>(t.inner_cones + node);
                    icr.a = __ldg(cr);
                    icr.b = __ldg(cr + 1);
                    icr.c = __ldg(cr + 2);
                }
                Cone lc, rc;
                unpack_cones(icr, lc, rc);
                Lmd = mindist(lb, p);
                Rmd = mindist(rb, p);
                const float b2 = best * best;
                hitL = Lmd <= b2 && lc.half_angle >= 0.0f && cone_test(lc, p, lb, Lmd);
                hitR = Rmd <= b2 && rc.half_angle >= 0.0f && cone_test(rc, p, rb, Rmd);
                // the leaf work of both children as one loop of edge_candidate calls
                // (the left leaf's edges, then the right leaf's, per lane: the order of
                // two leaf_silhouette_info calls), so a lane with only the right leaf
                // to test runs in the same iterations as a lane with only the left one
                // (16M queries of the 2M-triangle scene: 35.61 against 35.78 ms)
                const uint32_t nL = hitL && L >= ni ? Linfo >> 30 : 0u;
                const uint32_t nR = hitR && R >= ni ? Rinfo >> 30 : 0u;
                if (kStats)
                {
                    n_leaf += (hitL && L >= ni ? 1u : 0u) + (hitR && R >= ni ? 1u : 0u);
                    n_edge += nL + nR;
                }
                for (uint32_t k = 0; k < nL + nR; ++k)
                {
                    const bool right = k >= nL;
                    edge_candidate(t, right ? R - ni : L - ni, right ? k - nL : k,
                                   (right ? Rinfo : Linfo) & kLeafRankMask, p, flip, best, best_key, best_edge);
                }
            }
            const float b2n = best * best;
            const uint32_t pL = __ballot_sync(0xffffffffu, hitL && L < ni && Lmd <= b2n);
            const uint32_t pR = __ballot_sync(0xffffffffu, hitR && R < ni && Rmd <= b2n);
            const uint32_t votes = __ballot_sync(0xffffffffu, act && Lmd <= Rmd) & (pL | pR);
            if (pL && pR)
            {
                if (sp >= kStackDepth)
                {
                    overflow = true;
                    break;
                }
                const bool l_first = 2 * __popc(votes) >= __popc(pL | pR);
                __syncwarp();  // every lane has read the slot it may reuse
                if (lane == 0)
                {
                    st_node[sp] = l_first ? R : L;
                    st_mask[sp] = l_first ? pR : pL;
                    if (kTop)
                        st_slot[sp] = (uint8_t)child_slot(slot, l_first ? 1u : 0u, top_slots);
                }
                __syncwarp();
                ++sp;
                node = l_first ? L : R;
                mask = l_first ? pL : pR;
                if (kTop)
                    slot = child_slot(slot, l_first ? 0u : 1u, top_slots);
            }
            else if (pL | pR)
            {
                node = pL ? L : R;
                mask = pL ? pL : pR;
                if (kTop)
                    slot = child_slot(slot, pL ? 0u : 1u, top_slots);
            }
            else
                mask = 0u;
        }
        if (overflow)
            break;
    }
    if (overflow)
    {
        if (lane == 0)
            atomicOr(t.status, kStatusStackOverflow);
        best = NAN;
        best_edge = -1;
    }
    if (!valid)
        return;
    const bool failed = seed.radius && best_edge < 0 && r0 < INFINITY;
    if (seed.radius && best_edge < 0)
        best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
    st_out(out_dist + out_pos(t, qi, q), best);
    if (out_edge)
        st_out(out_edge + out_pos(t, qi, q), best_edge < 0 ? best_edge : best_edge - qr.edge_off);
    if (seed.fail_flag)
        seed.fail_flag[q] = failed ? 1u : 0u;
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = n_edge;
    }}

// blocks per SM the silhouette packet kernels are compiled for (8: 64 registers;
// measured on 16M-query batches of the 2M-triangle scene: 35.82 ms, against 36.03
// at 9 blocks / 56 registers and 41.2 at 10 blocks / 48 registers)
#ifndef SNCH_SIL_PACKET_MIN_BLOCKS
#define SNCH_SIL_PACKET_MIN_BLOCKS 8
#endif
template <bool kStats>
__global__ void __launch_bounds__(128, SNCH_SIL_PACKET_MIN_BLOCKS)
    silhouette_packet_kernel(TreeView t, const float *__restrict__ pts, const uint8_t *__restrict__ flips, int64_t n,
                             float *__restrict__ out_dist, int32_t *__restrict__ out_edge,
                             uint32_t *__restrict__ stats, SeedArgs seed)
{
    __shared__ uint32_t st_node[kPacketWarps][kStackDepth];
    __shared__ uint32_t st_mask[kPacketWarps][kStackDepth];
    const int w = threadIdx.x >> 5;
    silhouette_packet_chunk<kStats>(t, pts, flips, n, out_dist, out_edge, stats, seed,
                                    blockIdx.x * (int64_t)blockDim.x + threadIdx.x, st_node[w], st_mask[w]);
}

// the same packets, persistent (see nearest_packet_persistent_kernel)
template <bool kTop>
__global__ void __launch_bounds__(128, SNCH_SIL_PACKET_MIN_BLOCKS)
    silhouette_packet_persistent_kernel(TreeView t, const float *__restrict__ pts, const uint8_t *__restrict__ flips,
                                        int64_t n, float *__restrict__ out_dist, int32_t *__restrict__ out_edge,
                                        SeedArgs seed, unsigned long long *counter)
{
    __shared__ uint32_t st_node[kPacketWarps][kStackDepth];
    __shared__ uint32_t st_mask[kPacketWarps][kStackDepth];
    __shared__ uint8_t st_slot[kPacketWarps][kStackDepth];
    __shared__ uint64_t mbar;
    extern __shared__ __align__(128) unsigned char s_dyn[];
    InnerRec *s_top = reinterpret_cast<InnerRec *>(s_dyn);
    InnerConeRec *s_topc = reinterpret_cast<InnerConeRec *>(s_dyn + (kTop ? t.top_slots : 0u) * sizeof(InnerRec));
    const uint32_t top_slots = kTop ? stage_top_levels(t, s_top, s_topc, &mbar) : 0u;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned long long total = (unsigned long long)query_count(t, n);
    uint32_t empty_takes = 0;
    for (;;)
    {
        unsigned long long packet = 0;
        if (lane == 0)
            packet = take_packet(counter, (total + 31ull) / 32ull);
        packet = __shfl_sync(0xffffffffu, packet, 0);
        if (packet == ~0ull)
            break;
        if (packet >= (total + 31ull) / 32ull)
        {
            if (++empty_takes > kPoolSpins)  // cannot happen: see take_packet
            {
                if (lane == 0)
                    atomicOr(t.status, kStatusWorkTimeout);
                break;
            }
            continue;
        }
        empty_takes = 0;
        const unsigned long long base = packet * 32ull;
        silhouette_packet_chunk<false, kTop>(t, pts, flips, n, out_dist, out_edge, nullptr, seed, (int64_t)base + lane,
                                             st_node[w], st_mask[w], st_slot[w], s_top, s_topc, top_slots);
        __syncwarp();
    }
}

// ------------------------------------------------------------------ persistent forms
// The per-query traversals above run one query per thread; a warp then runs
// until its slowest query is done, and the per-query work of the nearest and
// silhouette searches has a long tail (a point far from every silhouette edge
// expands hundreds of nodes), so most lanes idle. The persistent forms below
// run the SAME per-query traversal (same visits, same results) but refill a
// lane with the next query of the batch as soon as its own query finishes:
// each warp takes chunks of 32 consecutive queries (spatially coherent when
// the batch is Morton-ordered) from a global counter, and lanes take queries
// from the warp's chunk in lane order.

struct WarpQueue
{
    unsigned long long next = 0, end = 0;
    bool exhausted = false;
};

// lanes with `need` set receive a query index (qi >= 0) while the batch lasts;
// called by all 32 lanes of the warp
SNCH_DEV int64_t take_query(WarpQueue &wq, unsigned long long total, unsigned long long *counter, bool need)
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int64_t qi = -1;
    unsigned mask = __ballot_sync(full, need);
    while (mask && !wq.exhausted)
    {
        if (wq.next >= wq.end)
        {
            unsigned long long base = 0;
            if (lane == 0)
                base = atomicAdd(counter, 32ull);
            base = __shfl_sync(full, base, 0);
            if (base >= total)
            {
                wq.exhausted = true;
                break;
            }
            wq.next = base;
            wq.end = base + 32ull < total ? base + 32ull : total;
        }
        const unsigned avail = (unsigned)(wq.end - wq.next);
        const unsigned r = __popc(mask & lt);
        const bool mine = ((mask >> lane) & 1u) && r < avail;
        if (mine)
            qi = (int64_t)(wq.next + r);
        const unsigned taken = __ballot_sync(full, mine);
        wq.next += __popc(taken);
        mask &= ~taken;
    }
    return qi;
}

struct SilState
{
    int64_t q;
    f3 p;
    bool flip;
    float best;
    uint32_t best_key;
    int32_t best_edge;
    int32_t edge_off;  // batched scenes: first edge id of the query's mesh
    int sp;
};

// Starts the search of query q at its (mesh's) root. Returns false when the
// answer is already known -- no tree, or a one-triangle tree or mesh, whose
// single leaf is evaluated here -- and true when nodes are left to expand.
SNCH_DEV bool start_silhouette(const TreeView &t, SilState &s, uint32_t *sn, float *sd, const SeedArgs &seed)
{
    const uint32_t ni = t.num_tris - 1;
    s.best = seed.radius ? __ldg(seed.radius + s.q) : INFINITY;
    s.best_key = 0;
    s.best_edge = -1;
    s.sp = 0;
    const QueryRoot qr = query_root(t, s.q);
    s.edge_off = qr.edge_off;
    if (qr.node == kInvalid)
        return false;
    if (qr.node >= ni)
    {
        uint32_t dummy = 0;
        leaf_silhouette_fast(t, qr.node - ni, s.p, s.flip, s.best, s.best_key, s.best_edge, dummy);
        return false;
    }
    sn[0] = qr.node;
    sd[0] = mindist(load_root_box(t.aabbs + qr.node), s.p);
    s.sp = 1;
    return true;
}

template <bool kSeed>
__global__ void __launch_bounds__(128) silhouette_persistent_kernel(TreeView t, const float *__restrict__ pts,
                                                                    const uint8_t *__restrict__ flips, int64_t n,
                                                                    float *__restrict__ out_dist,
                                                                    int32_t *__restrict__ out_edge, SeedArgs seed,
                                                                    unsigned long long *counter)
{
    const unsigned long long total = (unsigned long long)query_count(t, n);
    const uint32_t ni = t.num_tris - 1;
    uint32_t sn[kStackDepth];
    float sd[kStackDepth];
    SilState s;
    s.q = -1;
    s.sp = 0;
    bool active = false;
    WarpQueue wq;
    uint32_t dummy = 0;
    for (;;)
    {
        const int64_t qi = take_query(wq, total, counter, !active);
        bool done = false;
        if (qi >= 0)
        {
            s.q = query_index(t, qi);
            s.p = load_point(pts, s.q);
            s.flip = flips ? __ldg(flips + s.q) != 0 : false;
            active = true;
            done = !start_silhouette(t, s, sn, sd, seed);
        }
        if (!__any_sync(0xFFFFFFFFu, active))
        {
            if (wq.exhausted)
                break;
            continue;
        }
        if (!active)
            continue;
        if (!done)
        {
            --s.sp;
            const uint32_t node = sn[s.sp];
            if (!(sd[s.sp] > s.best * s.best))
            {
                if (s.sp > kStackDepth - 2)
                {
                    atomicOr(t.status, kStatusStackOverflow);
                    s.best = NAN;
                    s.best_edge = -1;
                    done = true;
                }
                else
                {
                    Box lb, rb;
                    uint32_t L, R;
                    unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
                    const float4 *cr = reinterpret_cast<const float4 *>(t.inner_cones + node);
                    InnerConeRec icr;
                    icr.a = __ldg(cr);
                    icr.b = __ldg(cr + 1);
                    icr.c = __ldg(cr + 2);
                    Cone lc, rc;
                    unpack_cones(icr, lc, rc);
                    const f3 p = s.p;
                    const float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
                    const float b2 = s.best * s.best;
                    const bool hitL = Lmd <= b2 && lc.half_angle >= 0.0f && cone_test(lc, p, lb, Lmd);
                    const bool hitR = Rmd <= b2 && rc.half_angle >= 0.0f && cone_test(rc, p, rb, Rmd);
                    if (hitL && L >= ni)
                        leaf_silhouette_fast(t, L - ni, p, s.flip, s.best, s.best_key, s.best_edge, dummy);
                    if (hitR && R >= ni)
                        leaf_silhouette_fast(t, R - ni, p, s.flip, s.best, s.best_key, s.best_edge, dummy);
                    const float b2n = s.best * s.best;
                    const bool pL = hitL && L < ni && Lmd <= b2n, pR = hitR && R < ni && Rmd <= b2n;
                    if (pL && pR)
                    {
                        const bool l_first = Lmd <= Rmd;
                        sn[s.sp] = l_first ? R : L;
                        sd[s.sp] = l_first ? Rmd : Lmd;
                        sn[s.sp + 1] = l_first ? L : R;
                        sd[s.sp + 1] = l_first ? Lmd : Rmd;
                        s.sp += 2;
                    }
                    else if (pL || pR)
                    {
                        sn[s.sp] = pL ? L : R;
                        sd[s.sp] = pL ? Lmd : Rmd;
                        ++s.sp;
                    }
                }
            }
        }
        if (done || s.sp == 0)
        {
            if (kSeed && s.best_edge < 0)
                s.best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
            out_dist[s.q] = s.best;
            if (out_edge)
                out_edge[s.q] = s.best_edge < 0 ? s.best_edge : s.best_edge - s.edge_off;
            if (kSeed && seed.fail_flag)
                seed.fail_flag[s.q] = s.best_edge < 0 ? 1u : 0u;
            active = false;
        }
    }
}

template <bool kSeed>
__global__ void __launch_bounds__(128) nearest_persistent_kernel(TreeView t, const float *__restrict__ pts, int64_t n,
                                                                 uint32_t *__restrict__ out_idx,
                                                                 float *__restrict__ out_dist, SeedArgs seed,
                                                                 unsigned long long *counter)
{
    const unsigned long long total = (unsigned long long)query_count(t, n);
    const uint32_t ni = t.num_tris - 1;
    uint32_t sn[kStackDepth];
    float sd[kStackDepth];
    int64_t q = -1;
    f3 p = mk(0.f, 0.f, 0.f);
    uint32_t nearest = kInvalid, best_rank = 0, tri_off = 0;
    float best = INFINITY;
    int sp = 0;
    bool active = false;
    WarpQueue wq;
    for (;;)
    {
        const int64_t qi = take_query(wq, total, counter, !active);
        bool done = false;
        if (qi >= 0)
        {
            q = query_index(t, qi);
            p = load_point(pts, q);
            nearest = kInvalid;
            best_rank = 0;
            best = INFINITY;
            if (kSeed)
            {
                const float r = __ldg(seed.radius + q);
                best = r * r;
            }
            active = true;
            // start at the query's (mesh's) root; no tree, or a one-triangle
            // tree or mesh, is answered here
            const QueryRoot qr = query_root(t, q);
            tri_off = qr.tri_off;
            sp = 0;
            if (qr.node == kInvalid)
                done = true;
            else if (qr.node >= ni)
            {
                leaf_nearest_fast(t, qr.node - ni, p, best, best_rank, nearest);
                done = true;
            }
            else
            {
                sn[0] = qr.node;
                sd[0] = mindist(load_root_box(t.aabbs + qr.node), p);
                sp = 1;
            }
        }
        if (!__any_sync(0xFFFFFFFFu, active))
        {
            if (wq.exhausted)
                break;
            continue;
        }
        if (!active)
            continue;
        if (!done)
        {
            --sp;
            const uint32_t node = sn[sp];
            if (!(sd[sp] > best))
            {
                if (sp > kStackDepth - 2)
                {
                    atomicOr(t.status, kStatusStackOverflow);
                    nearest = kInvalid;
                    best = NAN;
                    done = true;
                }
                else
                {
                    // near-first without the minmaxdist sibling test, as
                    // nearest_fast_kernel: the same leaves decide the answer
                    Box lb, rb;
                    uint32_t L, R;
                    unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
                    const float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
                    if (L >= ni && Lmd <= best)
                        leaf_nearest_fast(t, L - ni, p, best, best_rank, nearest);
                    if (R >= ni && Rmd <= best)
                        leaf_nearest_fast(t, R - ni, p, best, best_rank, nearest);
                    const bool pL = L < ni && Lmd <= best, pR = R < ni && Rmd <= best;
                    if (pL && pR)
                    {
                        const bool l_first = Lmd <= Rmd;
                        sn[sp] = l_first ? R : L;
                        sd[sp] = l_first ? Rmd : Lmd;
                        sn[sp + 1] = l_first ? L : R;
                        sd[sp + 1] = l_first ? Lmd : Rmd;
                        sp += 2;
                    }
                    else if (pL || pR)
                    {
                        sn[sp] = pL ? L : R;
                        sd[sp] = pL ? Lmd : Rmd;
                        ++sp;
                    }
                }
            }
        }
        if (done || sp == 0)
        {
            if (kSeed && nearest == kInvalid)
                best = INFINITY;  // nothing within the seed radius: the fallback pass answers it
            out_idx[q] = nearest == kInvalid ? kInvalid : nearest - tri_off;
            out_dist[q] = sqrtf(best);
            if (kSeed && seed.fail_flag)
                seed.fail_flag[q] = nearest == kInvalid ? 1u : 0u;
            active = false;
        }
    }
}

// ------------------------------------------------------------------ ray
// intersects_d(ray<float,3>) aabb.cuh:397-431
SNCH_DEV bool ray_box(f3 o, f3 inv, const Box &b, float max_dist, float &dist)
{
    float t1 = (b.lower.x - o.x) * inv.x, t2 = (b.upper.x - o.x) * inv.x;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b.lower.y - o.y) * inv.y;
    t2 = (b.upper.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = (b.lower.z - o.z) * inv.z;
    t2 = (b.upper.z - o.z) * inv.z;
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
SNCH_DEV bool ray_triangle(f3 o, f3 dir, f3 v0, f3 v1, f3 v2, float &t, float &uo, float &vo)
{
    const f3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const f3 h = mk(dir.y * e2.z - dir.z * e2.y, dir.z * e2.x - dir.x * e2.z, dir.x * e2.y - dir.y * e2.x);
    const float det = e1.x * h.x + e1.y * h.y + e1.z * h.z;
    if (fabsf(det) < kEps)
        return false;
    const float inv_det = __frcp_rn(det);
    const f3 s = sub(o, v0);
    const float u = (s.x * h.x + s.y * h.y + s.z * h.z) * inv_det;
    if (u < 0.0f || u > 1.0f)
        return false;
    const f3 qv = mk(s.y * e1.z - s.z * e1.y, s.z * e1.x - s.x * e1.z, s.x * e1.y - s.y * e1.x);
    const float v = (dir.x * qv.x + dir.y * qv.y + dir.z * qv.z) * inv_det;
    if (v < 0.0f || u + v > 1.0f)
        return false;
    const float tt = (e2.x * qv.x + e2.y * qv.y + e2.z * qv.z) * inv_det;
    if (tt >= 0.0f)
    {
        t = tt;
        uo = u;
        vo = v;
        return true;
    }
    return false;
}

// kAny: query_ray_intersect<TestOnly = true> (query.cuh:117-121): stop at the
// first accepted hit of the same traversal and report only whether there is one
// (always the hit flag of the closest-hit search: both take the same path up to
// that hit); t, uv and idx are not written.
// minimum blocks per SM the ray kernel is compiled for (0: the compiler's choice, 48
// registers and ten blocks)
#ifndef SNCH_RAY_MIN_BLOCKS
#define SNCH_RAY_MIN_BLOCKS 0
#endif
// ray batches of at least 4 x SNCH_OPT_PACKET_PERSISTENT_MIN rays use ray_pool_kernel
// (sphere draws, whose single descent is short, measured 3 % slower that way and
// keep one thread per draw)
#ifndef SNCH_RAY_POOLS
#define SNCH_RAY_POOLS 1
#endif
constexpr bool kRayPools = SNCH_RAY_POOLS != 0;
// one ray of the batch (batch position qi)
template <bool kStats, bool kAny>
SNCH_DEV void ray_query(const TreeView &t, const float *__restrict__ origins, const float *__restrict__ dirs,
                        const float *__restrict__ tmaxs, int64_t n, uint8_t *__restrict__ out_hit,
                        float *__restrict__ out_t, float *__restrict__ out_uv, uint32_t *__restrict__ out_idx,
                        uint32_t *__restrict__ stats, int64_t qi)
{
    uint32_t n_int = 0, n_leaf = 0;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 o = load_point(origins, q), dir = load_point(dirs, q);
    const f3 inv = mk(1 / dir.x, 1 / dir.y, 1 / dir.z);  // ray ctor aabb.cuh:305-312
    const float max_dist = ld_in(tmaxs + q);
    float min_dist = INFINITY, bu = 0.0f, bv = 0.0f;
    bool found = false;
    uint32_t nearest = kInvalid;
    const uint32_t ni = t.num_tris - 1;
    if (t.num_tris > 0)
    {
        // The closer hit child is processed next without a trip through the
        // stack (the reference pushes it last and pops it at once, with the
        // same bound check), so the visit order is the reference's.
        uint32_t sn[kStackDepth];
        float sd[kStackDepth];
        int sp = 0;
        uint32_t node = 0;
        float nd = INFINITY;
        for (;;)
        {
            bool next = !(nd > min_dist);
            if (next && node >= ni)
            {
                f3 pa, pb, pc;
                uint32_t orig, n_owned;
                load_leaf(t.leaves + (node - ni), pa, pb, pc, orig, n_owned);
                if (kStats)
                    ++n_leaf;
                float tt, uu, vv;
                if (ray_triangle(o, dir, pa, pb, pc, tt, uu, vv) && tt < max_dist && tt < min_dist)
                {
                    min_dist = tt;
                    found = true;
                    bu = uu;
                    bv = vv;
                    nearest = orig;
                    if (kAny)
                        break;
                }
                next = false;
            }
            else if (next)
            {
                if (sp > kStackDepth - 2)
                {
                    atomicOr(t.status, kStatusStackOverflow);
                    found = false;
                    nearest = kInvalid;
                    min_dist = NAN;
                    break;
                }
                Box lb, rb;
                uint32_t L, R;
                unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
                if (kStats)
                    ++n_int;
                float Ld = 0.0f, Rd = 0.0f;
                const bool Lh = ray_box(o, inv, lb, max_dist, Ld);
                const bool Rh = ray_box(o, inv, rb, max_dist, Rd);
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
                    sd[sp] = Rd;
                    ++sp;
                    node = closer;
                    nd = Ld;
                    continue;
                }
                if (Lh || Rh)
                {
                    node = Lh ? L : R;
                    nd = Lh ? Ld : Rd;
                    continue;
                }
                next = false;
            }
            // pop
            if (sp == 0)
                break;
            --sp;
            node = sn[sp];
            nd = sd[sp];
        }
    }
    st_out(out_hit + out_pos(t, qi, q), (uint8_t)(found ? 1 : 0));
    if (kAny)
        return;
    st_out(out_t + out_pos(t, qi, q), min_dist);
    st_out(out_uv + 2 * out_pos(t, qi, q), bu);
    st_out(out_uv + 2 * out_pos(t, qi, q) + 1, bv);
    st_out(out_idx + out_pos(t, qi, q), nearest);
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = 0;
    }
}
template <bool kStats, bool kAny = false>
__global__ void __launch_bounds__(128, SNCH_RAY_MIN_BLOCKS) ray_kernel(TreeView t, const float *__restrict__ origins,
                                                  const float *__restrict__ dirs, const float *__restrict__ tmaxs,
                                                  int64_t n, uint8_t *__restrict__ out_hit, float *__restrict__ out_t,
                                                  float *__restrict__ out_uv, uint32_t *__restrict__ out_idx,
                                                  uint32_t *__restrict__ stats)
{
    ray_query<kStats, kAny>(t, origins, dirs, tmaxs, n, out_hit, out_t, out_uv, out_idx, stats,
                            blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}
// The same rays, one per thread, handed out 32 at a time through the per-SM
// pools of the packet searches (take_packet): a warp takes the next 32 rays of
// its SM's chunk when its last ray ends, so the warps of an SM trace rays from
// neighbouring origins (the batch is Morton-ordered by origin) and share the
// tree records in its L1, and no warp waits for the slowest ray of its block.
template <bool kAny>
__global__ void __launch_bounds__(128, SNCH_RAY_MIN_BLOCKS)
    ray_pool_kernel(TreeView t, const float *__restrict__ origins, const float *__restrict__ dirs,
                    const float *__restrict__ tmaxs, int64_t n, uint8_t *__restrict__ out_hit,
                    float *__restrict__ out_t, float *__restrict__ out_uv, uint32_t *__restrict__ out_idx,
                    unsigned long long *work)
{
    const int lane = threadIdx.x & 31;
    const unsigned long long total = (unsigned long long)query_count(t, n), packets = (total + 31ull) / 32ull;
    uint32_t empty_takes = 0;
    for (;;)
    {
        unsigned long long packet = 0;
        if (lane == 0)
            packet = take_packet(work, packets);
        packet = __shfl_sync(0xffffffffu, packet, 0);
        if (packet == ~0ull)
            break;
        if (packet >= packets)
        {
            if (++empty_takes > kPoolSpins)  // cannot happen: see take_packet
            {
                if (lane == 0)
                    atomicOr(t.status, kStatusWorkTimeout);
                break;
            }
            continue;
        }
        empty_takes = 0;
        ray_query<false, kAny>(t, origins, dirs, tmaxs, n, out_hit, out_t, out_uv, out_idx, nullptr,
                               (int64_t)(packet * 32ull) + lane);
        __syncwarp();
    }
}

// The same ray traversal, persistent (lane refill): a lane takes the next ray
// of the batch when its own is done (warp-chunked counter, take_query). Rays
// with tmax log-uniform over three decades differ in cost by orders of
// magnitude, so a one-ray-per-thread warp waits for its longest ray; here the
// finished lanes start new rays instead. Each iteration is one step of the
// reference's near-first order (same visits, same answers).
template <bool kAny>
__global__ void __launch_bounds__(128) ray_persistent_kernel(TreeView t, const float *__restrict__ origins,
                                                             const float *__restrict__ dirs,
                                                             const float *__restrict__ tmaxs, int64_t n,
                                                             uint8_t *__restrict__ out_hit, float *__restrict__ out_t,
                                                             float *__restrict__ out_uv,
                                                             uint32_t *__restrict__ out_idx,
                                                             unsigned long long *counter)
{
    const unsigned long long total = (unsigned long long)query_count(t, n);
    const uint32_t ni = t.num_tris - 1;
    uint32_t sn[kStackDepth];
    float sd[kStackDepth];
    int sp = 0;
    int64_t q = -1;
    f3 o = mk(0.f, 0.f, 0.f), dir = o, inv = o;
    float max_dist = 0.f, min_dist = INFINITY, bu = 0.f, bv = 0.f, nd = INFINITY;
    bool found = false, active = false;
    uint32_t nearest = kInvalid, node = 0;
    WarpQueue wq;
    for (;;)
    {
        const int64_t qi = take_query(wq, total, counter, !active);
        bool done = false;
        if (qi >= 0)
        {
            q = query_index(t, qi);
            o = load_point(origins, q);
            dir = load_point(dirs, q);
            inv = mk(1 / dir.x, 1 / dir.y, 1 / dir.z);  // ray ctor aabb.cuh:305-312
            max_dist = ld_in(tmaxs + q);
            min_dist = INFINITY;
            bu = bv = 0.f;
            found = false;
            nearest = kInvalid;
            node = 0;
            nd = INFINITY;
            sp = 0;
            active = true;
            done = t.num_tris == 0;
        }
        if (!__any_sync(0xFFFFFFFFu, active))
        {
            if (wq.exhausted)
                break;
            continue;
        }
        if (!active)
            continue;
        if (!done)
        {
            bool next = !(nd > min_dist);
            if (next && node >= ni)
            {
                f3 pa, pb, pc;
                uint32_t orig, n_owned;
                load_leaf(t.leaves + (node - ni), pa, pb, pc, orig, n_owned);
                float tt, uu, vv;
                if (ray_triangle(o, dir, pa, pb, pc, tt, uu, vv) && tt < max_dist && tt < min_dist)
                {
                    min_dist = tt;
                    found = true;
                    bu = uu;
                    bv = vv;
                    nearest = orig;
                    if (kAny)
                        done = true;
                }
                next = false;
            }
            else if (next)
            {
                if (sp > kStackDepth - 2)
                {
                    atomicOr(t.status, kStatusStackOverflow);
                    found = false;
                    nearest = kInvalid;
                    min_dist = NAN;
                    done = true;
                }
                else
                {
                    Box lb, rb;
                    uint32_t L, R;
                    unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
                    float Ld = 0.0f, Rd = 0.0f;
                    const bool Lh = ray_box(o, inv, lb, max_dist, Ld);
                    const bool Rh = ray_box(o, inv, rb, max_dist, Rd);
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
                        sd[sp] = Rd;
                        ++sp;
                        node = closer;
                        nd = Ld;
                    }
                    else if (Lh || Rh)
                    {
                        node = Lh ? L : R;
                        nd = Lh ? Ld : Rd;
                    }
                    else
                        next = false;
                }
            }
            if (!done && !next)
            {
                // pop (the reference's stack order)
                if (sp == 0)
                    done = true;
                else
                {
                    --sp;
                    node = sn[sp];
                    nd = sd[sp];
                }
            }
        }
        if (done)
        {
            out_hit[q] = found ? 1 : 0;
            if (!kAny)
            {
                out_t[q] = min_dist;
                out_uv[2 * q] = bu;
                out_uv[2 * q + 1] = bv;
                out_idx[q] = nearest;
            }
            active = false;
        }
    }
}

// ------------------------------------------------------------------ top levels
// Heap slot i (children 2i+1, 2i+2) of the top levels: the internal node reached
// from the root by the bits of i + 1 below its leading one (0 = left); a slot
// under a leaf is left zero (the searches never read it).
__global__ void top_levels_kernel(const InnerRec *__restrict__ inner, const InnerConeRec *__restrict__ cones,
                                  uint32_t num_tris, uint32_t slots, InnerRec *__restrict__ top,
                                  InnerConeRec *__restrict__ topc)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots)
        return;
    const uint32_t ni = num_tris - 1, h = i + 1;
    uint32_t node = 0;
    bool ok = num_tris > 1;
    for (int b = 30 - __clz(h); b >= 0 && ok; --b)
    {
        const float4 d = __ldg(reinterpret_cast<const float4 *>(inner + node) + 3);
        node = ((h >> b) & 1u) ? __float_as_uint(d.y) : __float_as_uint(d.x);
        ok = node < ni;
    }
    InnerRec r{};
    InnerConeRec c{};
    if (ok)
    {
        r = inner[node];
        c = cones[node];
    }
    top[i] = r;
    topc[i] = c;
}
cudaError_t launch_top_levels(const InnerRec *inner, const InnerConeRec *cones, uint32_t num_tris, uint32_t slots,
                              InnerRec *top, InnerConeRec *topc, cudaStream_t st)
{
    if (slots == 0 || num_tris < 2)
        return cudaSuccess;
    top_levels_kernel<<<1, 256, 0, st>>>(inner, cones, num_tris, slots, top, topc);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ sampling
// intersect_sphere(sphere, aabb) aabb.cuh:433-449
SNCH_DEV bool sphere_box(f3 c, float r, const Box &b)
{
    const float cx = smax(b.lower.x, smin(c.x, b.upper.x));
    const float cy = smax(b.lower.y, smin(c.y, b.upper.y));
    const float dx = cx - c.x, dy = cy - c.y;
    float d2 = dx * dx + dy * dy;
    const float cz = smax(b.lower.z, smin(c.z, b.upper.z));
    const float dz = cz - c.z;
    d2 += dz * dz;
    return d2 <= (r * r);
}

// scene<3>::intersect_sphere scene.cuh:1054-1117
SNCH_DEV bool sphere_triangle(f3 c, float radius, f3 p1, f3 p2, f3 p3)
{
    const f3 e1 = sub(p2, p1), e2 = sub(p3, p1);
    f3 nn = mk(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
    const float nl = sqrtf(nn.x * nn.x + nn.y * nn.y + nn.z * nn.z);
    nn = mk(nn.x / nl, nn.y / nl, nn.z / nl);
    const float d = nn.x * p1.x + nn.y * p1.y + nn.z * p1.z;
    const float dp = nn.x * c.x + nn.y * c.y + nn.z * c.z - d;
    const f3 proj = mk(c.x - dp * nn.x, c.y - dp * nn.y, c.z - dp * nn.z);
    const f3 v0 = sub(p3, p1), v1 = sub(p2, p1), v2 = sub(proj, p1);
    const float d00 = v0.x * v0.x + v0.y * v0.y + v0.z * v0.z;
    const float d01 = v0.x * v1.x + v0.y * v1.y + v0.z * v1.z;
    const float d02 = v0.x * v2.x + v0.y * v2.y + v0.z * v2.z;
    const float d11 = v1.x * v1.x + v1.y * v1.y + v1.z * v1.z;
    const float d12 = v1.x * v2.x + v1.y * v2.y + v1.z * v2.z;
    const float inv = 1.0f / (d00 * d11 - d01 * d01);
    const float u = (d11 * d02 - d01 * d12) * inv;
    const float v = (d00 * d12 - d01 * d02) * inv;
    if (u >= 0 && v >= 0 && u + v <= 1)
        return fabsf(dp) <= radius;
    f3 cp = proj;
    if (u < 0)
        cp = p1;
    else if (v < 0)
        cp = p3;
    else if (u + v > 1)
        cp = p2;
    const float dx = cp.x - c.x, dy = cp.y - c.y, dz = cp.z - c.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    return d2 <= (radius * radius);
}

// green_weight scene.cuh:1119-1126
SNCH_DEV float green_weight(f3 x, f3 y)
{
    const float r = fmaxf(len3(mk(x.x - y.x, x.y - y.y, x.z - y.z)), 1e-4f);
    const float four_pi = 3.14159265358979323846f * 4.0f;
    return 1.0f / (four_pi * r);
}

template <bool kStats>
__global__ void __launch_bounds__(128) sample_kernel(TreeView t, const float *__restrict__ centers,
                                                     const float *__restrict__ radii, const float *__restrict__ us,
                                                     int64_t n, int32_t *__restrict__ out_idx,
                                                     float *__restrict__ out_pdf, uint32_t *__restrict__ stats)
{
    uint32_t n_int = 0, n_leaf = 0;
    const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (qi >= query_count(t, n))
        return;
    const int64_t q = query_index(t, qi);
    const f3 c = load_point(centers, q);
    const float rad = ld_in(radii + q);
    float u = ld_in(us + q);
    int32_t oi = -1;
    float opdf = 0.0f;
    const uint32_t ni = t.num_tris - 1;
    if (t.num_tris > 0)
    {
        uint32_t node = 0;
        float npdf = 1.0f;
        // the reference's stack never holds more than one entry (sample.cuh:41-90);
        // a descent is at most one step per tree level
        for (int level = 0; level < 2 * kStackDepth; ++level)
        {
            if (node >= ni)
            {
                f3 pa, pb, pc;
                uint32_t orig, n_owned;
                load_leaf(t.leaves + (node - ni), pa, pb, pc, orig, n_owned);
                if (kStats)
                    ++n_leaf;
                if (sphere_triangle(c, rad, pa, pb, pc))
                {
                    oi = (int32_t)orig;
                    opdf = npdf;
                    opdf /= len3(cross3(sub(pc, pa), sub(pb, pa))) / 2;  // measurement_getter scene.cuh:855-868
                }
                break;
            }
            Box lb, rb;
            uint32_t L, R;
            unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
            if (kStats)
                ++n_int;
            const float Lw = sphere_box(c, rad, lb) ? green_weight(c, centroid(lb)) : 0;
            const float Rw = sphere_box(c, rad, rb) ? green_weight(c, centroid(rb)) : 0;
            const float tw = Lw + Rw;
            if (!(tw > 0))
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
    st_out(out_idx + out_pos(t, qi, q), oi);
    st_out(out_pdf + out_pos(t, qi, q), opdf);
    if (kStats)
    {
        stats[3 * q] = n_int;
        stats[3 * q + 1] = n_leaf;
        stats[3 * q + 2] = 0;
    }
}

// sample_triangle scene.cuh:14-27 on the triangle of ORIGINAL index idx
// an index outside [0, num_tris) (a draw that found no triangle) gives a NaN point
__global__ void sample_point_kernel(const float *__restrict__ verts, const int32_t *__restrict__ tris,
                                    uint32_t num_tris, const int32_t *__restrict__ idx,
                                    const float *__restrict__ us, const float *__restrict__ vs, int64_t n,
                                    float *__restrict__ out)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    const int32_t k = __ldg(idx + q);
    if (k < 0 || (uint32_t)k >= num_tris)
    {
        out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = NAN;
        return;
    }
    const int32_t *tr = tris + 3 * (int64_t)k;
    const f3 pa = load_vert(verts, __ldg(tr)), pb = load_vert(verts, __ldg(tr + 1)), pc = load_vert(verts, __ldg(tr + 2));
    float u = ld_in(us + q), v = __ldg(vs + q);
    if (u + v > 1.0f)
    {
        u = 1.0f - u;
        v = 1.0f - v;
    }
    const float w = 1.0f - u - v;
    out[3 * q] = w * pa.x + u * pb.x + v * pc.x;
    out[3 * q + 1] = w * pa.y + u * pb.y + v * pc.y;
    out[3 * q + 2] = w * pa.z + u * pb.z + v * pc.z;
}

// ------------------------------------------------------------------ query ordering
// 30-bit Morton code of each query point inside the root box (same encoding
// as the leaves, morton_code.cuh:61-70); sorting a batch by it makes the 32
// queries of a warp spatial neighbours. Results do not depend on the order.
// Morton code of the query point in the tree's root box; for batched queries
// (mesh of each query given) in its mesh's root box, below the mesh id:
// key = mesh << (32 - mesh_bits) | the code's top (32 - mesh_bits) bits
// With lengths (rays: tmax), a plain scene's key is the ray's length bucket --
// floor(log2(tmax / the root box's largest side)), 16 buckets from 2^-15 up --
// above the top order_bits - 4 bits of the origin's code, so that a warp's rays have similar
// lengths (a ray's work grows with its length) and, within a bucket, neighbouring
// origins.
__global__ void query_keys_kernel(const float *__restrict__ pts, int64_t n, const Box *__restrict__ root,
                                  uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, TreeView t,
                                  int mesh_bits, const float *__restrict__ len)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t m = 0, node = 0;
    if (t.query_mesh)
    {
        m = __ldg(t.query_mesh + i);
        node = m < t.num_meshes ? __ldg(t.mesh_root + m) : kInvalid;
        if (node == kInvalid)
        {
            keys[i] = 0xFFFFFFFFu;
            vals[i] = (uint32_t)i;
            return;
        }
    }
    const Box b = load_root_box(root + node);
    f3 p = load_point(pts, i);
    p.x = (p.x - b.lower.x) / (b.upper.x - b.lower.x);
    p.y = (p.y - b.lower.y) / (b.upper.y - b.lower.y);
    p.z = (p.z - b.lower.z) / (b.upper.z - b.lower.z);
    const float res = 1024.0f;
    const uint32_t x = (uint32_t)fminf(fmaxf(p.x * res, 0.0f), res - 1.0f);
    const uint32_t y = (uint32_t)fminf(fmaxf(p.y * res, 0.0f), res - 1.0f);
    const uint32_t z = (uint32_t)fminf(fmaxf(p.z * res, 0.0f), res - 1.0f);
    auto expand = [](uint32_t v) {
        v = (v | (v << 16)) & 0x070000FFu;
        v = (v | (v << 8)) & 0x0700F00Fu;
        v = (v | (v << 4)) & 0x430C30C3u;
        v = (v | (v << 2)) & 0x49249249u;
        return v;
    };
    const uint32_t code = expand(x) * 4 + expand(y) * 2 + expand(z);
    if (len && !t.query_mesh)
    {
        const float side = fmaxf(b.upper.x - b.lower.x, fmaxf(b.upper.y - b.lower.y, b.upper.z - b.lower.z));
        const float r = __ldg(len + i) / side;
        const int lb = r > 0.0f ? (isinf(r) ? 0 : ilogbf(r)) : -15;
        const uint32_t bucket = (uint32_t)min(max(lb + 15, 0), 15);
        keys[i] = (bucket << (t.order_bits - 4)) | (code >> (34 - t.order_bits));
        vals[i] = (uint32_t)i;
        return;
    }
    // plain scenes: the top order_bits of the 30-bit code (the sort takes that many bits)
    keys[i] = t.query_mesh ? (m << (32 - mesh_bits)) | (code >> (mesh_bits - 2)) : code >> (30 - t.order_bits);
    vals[i] = (uint32_t)i;
}

// ------------------------------------------------------------------ enumeration queries
// query_device(overlaps(box)) query.cuh:177-231 and query_device(line_intersect(line),
// element_test) query.cuh:15-77 over the scene's triangles. The reference's stack
// discipline is kept (push L then R, pop the top; leaf children reported when their
// parent is expanded, L before R), so the results come out in its order; the
// first max_out go to the query's row, the total is counted (the reference's
// return value). The line's element test is intersect_test's arithmetic
// (scene.cuh:1005-1052) for a line: any t, returned with the triangle.

// intersects(aabb, aabb) aabb.cuh:66-81 (query box first, as query.cuh:199)
SNCH_DEV bool box_overlap(const Box &a, const Box &b)
{
    if (a.upper.x < b.lower.x || b.upper.x < a.lower.x)
        return false;
    if (a.upper.y < b.lower.y || b.upper.y < a.lower.y)
        return false;
    if (a.upper.z < b.lower.z || b.upper.z < a.lower.z)
        return false;
    return true;
}
// intersects(line<float,3>, aabb) aabb.cuh:329-348
SNCH_DEV bool line_box(f3 o, f3 inv, const Box &b)
{
    float t1 = (b.lower.x - o.x) * inv.x, t2 = (b.upper.x - o.x) * inv.x;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b.lower.y - o.y) * inv.y;
    t2 = (b.upper.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = (b.lower.z - o.z) * inv.z;
    t2 = (b.upper.z - o.z) * inv.z;
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
    return tmax >= tmin;
}
SNCH_DEV bool line_triangle(f3 o, f3 dir, f3 v0, f3 v1, f3 v2, float &t)
{
    const f3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    const f3 h = mk(dir.y * e2.z - dir.z * e2.y, dir.z * e2.x - dir.x * e2.z, dir.x * e2.y - dir.y * e2.x);
    const float det = e1.x * h.x + e1.y * h.y + e1.z * h.z;
    if (fabsf(det) < kEps)
        return false;
    const float inv_det = __frcp_rn(det);
    const f3 sv = sub(o, v0);
    const float u = (sv.x * h.x + sv.y * h.y + sv.z * h.z) * inv_det;
    if (u < 0.0f || u > 1.0f)
        return false;
    const f3 qv = mk(sv.y * e1.z - sv.z * e1.y, sv.z * e1.x - sv.x * e1.z, sv.x * e1.y - sv.y * e1.x);
    const float v = (dir.x * qv.x + dir.y * qv.y + dir.z * qv.z) * inv_det;
    if (v < 0.0f || u + v > 1.0f)
        return false;
    t = (e2.x * qv.x + e2.y * qv.y + e2.z * qv.z) * inv_det;
    return true;
}

template <bool kLine>
__global__ void __launch_bounds__(128) enumerate_kernel(TreeView t, const float *__restrict__ q0,
                                                        const float *__restrict__ q1, int64_t n, uint32_t max_out,
                                                        uint32_t *__restrict__ out_idx, float *__restrict__ out_t,
                                                        uint32_t *__restrict__ out_count)
{
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n)
        return;
    Box qb;
    f3 o = mk(0.0f, 0.0f, 0.0f), dir = o, inv = o;
    if (kLine)
    {
        o = load_point(q0, q);
        dir = load_point(q1, q);
        inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);  // line ctor aabb.cuh:288-295
    }
    else
    {
        const float *x = q0 + 6 * q;
        qb.lower = mk(__ldg(x), __ldg(x + 1), __ldg(x + 2));
        qb.upper = mk(__ldg(x + 3), __ldg(x + 4), __ldg(x + 5));
    }
    uint32_t found = 0;
    const uint64_t row = (uint64_t)q * max_out;
    auto visit = [&](const Box &b) { return kLine ? line_box(o, inv, b) : box_overlap(qb, b); };
    auto emit = [&](uint32_t pos) {
        const float4 *lr = reinterpret_cast<const float4 *>(t.leaves + pos);
        const float4 a = __ldg(lr);
        float tt = 0.0f;
        if (kLine)
        {
            const float4 b = __ldg(lr + 1), c = __ldg(lr + 2);
            if (!line_triangle(o, dir, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), tt))
                return;
        }
        if (found < max_out)
        {
            out_idx[row + found] = __float_as_uint(a.w);
            if (kLine)
                out_t[row + found] = tt;
        }
        ++found;
    };
    const uint32_t N = t.num_tris, ni = N - 1;
    if (N == 1)
    {
        if (visit(load_root_box(t.aabbs)))
            emit(0);
    }
    else if (N > 1)
    {
        uint32_t stack[kStackDepth];
        int sp = 0;
        stack[sp++] = 0;
        do
        {
            const uint32_t node = stack[--sp];
            Box lb, rb;
            uint32_t L, R;
            unpack_inner(load_inner(t.inner + node), lb, rb, L, R);
            bool full = false;
            if (visit(lb))
            {
                if (L >= ni)
                    emit(L - ni);
                else if (sp < kStackDepth)
                    stack[sp++] = L;
                else
                    full = true;
            }
            if (visit(rb))
            {
                if (R >= ni)
                    emit(R - ni);
                else if (sp < kStackDepth)
                    stack[sp++] = R;
                else
                    full = true;
            }
            if (full)
            {
                atomicOr(t.status, kStatusStackOverflow);
                break;
            }
        } while (sp > 0);
    }
    out_count[q] = found;
}

// ------------------------------------------------------------------ launchers
namespace
{
inline unsigned grid_for(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }
// the packet searches serve near-first, binary-record, uncapped launches
inline bool packet_ok(const TreeView &t, int packet, int width, const SeedArgs &seed)
{
    const bool on = packet == 1 || (packet == 2 && t.order_coherent);
    return on && width == 2 && t.near_first && !seed.cap && t.num_tris > 1;
}
// Automatic packets for nearest searches need a dense batch: a warp's 32
// neighbours must share most of their traversal. Measured crossover, with the
// persistent packets drawing from per-SM pools: about 1 query per triangle
// (2M-triangle scene: per lane x1.56 faster at 0.26 and x1.23 at 0.5 queries per
// triangle; at 1 / 2 / 3 packets take 2.80 / 4.15 / 5.45 ms against 2.87 / 4.99 /
// 7.07 per lane; before the pools the crossover was near 3). Silhouette packets
// won at every measured density (0.26 queries per triangle up).
constexpr uint64_t kPacketNearestMinQueriesPerTri = 1;
inline bool packet_dense(const TreeView &t, int packet, int64_t n)
{
    return packet == 1 || (uint64_t)n >= kPacketNearestMinQueriesPerTri * t.num_tris;
}
// the wide searches serve near-first, one-thread-per-query, uncapped launches
// over a tree whose wide records of that width exist
inline bool wide_ok(const TreeView &t, int width, bool persistent, const SeedArgs &seed)
{
    if (!t.near_first || persistent || seed.cap || t.num_tris < 2)
        return false;
    return (width == 4 && t.wide4 && t.wide4_of) || (width == 8 && t.wide8 && t.wide8_of);
}
// persistent launch: as many 128-thread blocks as the GPU holds at once (fewer for
// small batches), and a zeroed 64-bit work counter of its own (stream-ordered
// allocation, so concurrent calls on other streams do not share it)
template <typename... KArgs, typename... Args>
cudaError_t launch_persistent_smem(void (*kernel)(KArgs...), size_t smem, int64_t n, cudaStream_t st, Args... args)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, smem);
    if (e != cudaSuccess)
        return e;
    const int64_t need = (n + 127) / 128;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * std::max(per_sm, 1)));
    unsigned long long *counter = nullptr;
    // the work counter and, for the packet searches, the per-SM packet pools
    constexpr size_t work_bytes = (1 + kPoolSlots) * sizeof(unsigned long long);
    if ((e = scratch_alloc_raw(reinterpret_cast<void **>(&counter), work_bytes, st)) != cudaSuccess)
        return e;
    e = cudaMemsetAsync(counter, 0, work_bytes, st);
    if (e == cudaSuccess)
    {
        kernel<<<grid, 128, smem, st>>>(args..., counter);
        note_launch();
        e = cudaGetLastError();
    }
    const cudaError_t f = cudaFreeAsync(counter, st);
    return e != cudaSuccess ? e : f;
}
template <typename... KArgs, typename... Args>
cudaError_t launch_persistent(void (*kernel)(KArgs...), int64_t n, cudaStream_t st, Args... args)
{
    return launch_persistent_smem(kernel, 0, n, st, args...);
}
// Results of an unseeded, fully Morton-ordered batch are written at their batch
// position into a stream-ordered temporary (warp-contiguous, coalesced stores)
// and moved to query order by one scatter pass per batch. Written at query
// order[i] directly, neighbouring lanes store to unrelated 4-byte slots: each
// store dirties a 32-byte sector that L2 evicts long before the other seven
// slots arrive (the search streams the tree through L2), so DRAM sees about 8x
// the output bytes (16M nearest queries: 1.07 GB written for 128 MB of results).
// The scatter pass touches only the output arrays, which stay in L2 while
// their sectors fill.
inline bool batch_order_ok(const TreeView &t, const SeedArgs &seed, const uint32_t *stats)
{
    return t.order && !t.order_count && t.out_batch_order_enabled && !stats && !seed.radius && !seed.fail_flag &&
           !seed.cap;
}

// out[order[i]] = tmp[i] for two 4-byte result arrays (streaming loads keep L2
// for the scattered stores)
__global__ void scatter2_kernel(const uint32_t *__restrict__ order, int64_t n, const uint32_t *__restrict__ a,
                                uint32_t *__restrict__ A, const uint32_t *__restrict__ b, uint32_t *__restrict__ B)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t q = __ldcs(order + i);
    A[q] = __ldcs(a + i);
    if (B)
        B[q] = __ldcs(b + i);
}
// the ray's four result arrays; uv as one 8-byte store when the caller's array allows it
__global__ void scatter_ray_kernel(const uint32_t *__restrict__ order, int64_t n, const uint8_t *__restrict__ th,
                                   const float *__restrict__ tt, const float2 *__restrict__ tuv,
                                   const uint32_t *__restrict__ ti, uint8_t *__restrict__ hit, float *__restrict__ t,
                                   float *__restrict__ uv, uint32_t *__restrict__ idx, int uv_aligned)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t q = __ldcs(order + i);
    hit[q] = __ldcs(th + i);
    t[q] = __ldcs(tt + i);
    const float2 w = __ldcs(tuv + i);
    if (uv_aligned)
        reinterpret_cast<float2 *>(uv)[q] = w;
    else
    {
        uv[2 * (int64_t)q] = w.x;
        uv[2 * (int64_t)q + 1] = w.y;
    }
    idx[q] = __ldcs(ti + i);
}

// stream-ordered temporary for one batch's results in batch order
struct BatchOut
{
    char *base = nullptr;
    cudaStream_t st = nullptr;
    cudaError_t alloc(int64_t n, size_t bytes_per_query, cudaStream_t s)
    {
        st = s;
        return scratch_alloc_raw(reinterpret_cast<void **>(&base), bytes_per_query * (size_t)n + 1024, s);
    }
    // the k-th array of `elem` bytes per query, 256-byte aligned after the previous ones
    template <typename T>
    T *at(size_t offset_bytes) const
    {
        return reinterpret_cast<T *>(base + offset_bytes);
    }
    ~BatchOut()
    {
        if (base)
            cudaFreeAsync(base, st);
    }
};
inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
}  // namespace

cudaError_t launch_nearest(const TreeView &t0, const float *pts, int64_t n, uint32_t *idx_out, float *dist_out,
                           cudaStream_t st, uint32_t *stats, const SeedArgs &seed)
{
    if (n <= 0)
        return cudaSuccess;
    TreeView t = t0;
    const bool persistent = (t.persistent & 1) != 0;
    const bool packets = packet_ok(t, t.packet_near, t.width_near, seed) && packet_dense(t, t.packet_near, n);
    const bool wide = !packets && wide_ok(t, t.width_near, persistent, seed);
    const bool lane_persistent = !packets && !wide && !stats && t.near_first && t.num_tris > 1 && persistent;
    // the kernels below that write at out_pos() (all but the lane-refill and reference-order ones)
    const bool supports = packets || wide || (t.near_first && !lane_persistent);
    BatchOut tmp;
    uint32_t *idx = idx_out;
    float *dist = dist_out;
    if (supports && batch_order_ok(t, seed, stats))
    {
        cudaError_t e = tmp.alloc(n, 8, st);
        if (e != cudaSuccess)
            return e;
        idx = tmp.at<uint32_t>(0);
        dist = tmp.at<float>(align256(4 * (size_t)n));
        t.out_batch_order = 1;
    }
    cudaError_t e = cudaSuccess;
    bool launched = false;
    if (packets)
    {
        // persistent packets for large batches: the same packets and answers, 2-7 %
        // faster there (no warp slot waits for the slowest packet of its block);
        // 6 % slower on 1M-query batches. The counters' pass keeps the grid form.
        if (stats)
            nearest_packet_kernel<true><<<grid_for(n, 128), 128, 0, st>>>(t, pts, n, idx, dist, stats, seed);
        else if (n >= t.packet_persistent_min)
        {
            e = t.top_slots && !t.query_mesh
                    ? launch_persistent_smem(nearest_packet_persistent_kernel<true>, top_smem_bytes(t.top_slots, false),
                                             n, st, t, pts, n, idx, dist, seed)
                    : launch_persistent(nearest_packet_persistent_kernel<false>, n, st, t, pts, n, idx, dist, seed);
            launched = true;
        }
        else
            nearest_packet_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, pts, n, idx, dist, nullptr, seed);
    }
    else if (wide)
    {
        const unsigned g = grid_for(n, 128);
        if (t.width_near == 4)
            stats ? nearest_wide_kernel<4, true><<<g, 128, 0, st>>>(t, pts, n, idx, dist, stats, seed)
                  : nearest_wide_kernel<4, false><<<g, 128, 0, st>>>(t, pts, n, idx, dist, nullptr, seed);
        else
            stats ? nearest_wide_kernel<8, true><<<g, 128, 0, st>>>(t, pts, n, idx, dist, stats, seed)
                  : nearest_wide_kernel<8, false><<<g, 128, 0, st>>>(t, pts, n, idx, dist, nullptr, seed);
    }
    else if (stats)
        nearest_fast_kernel<true><<<grid_for(n, 128), 128, 0, st>>>(t, pts, n, idx, dist, stats, seed);
    else if (lane_persistent)
    {
        e = seed.radius ? launch_persistent(nearest_persistent_kernel<true>, n, st, t, pts, n, idx, dist, seed)
                        : launch_persistent(nearest_persistent_kernel<false>, n, st, t, pts, n, idx, dist, seed);
        launched = true;
    }
    else if (t.near_first && t.block_near == 64)
        nearest_fast_kernel<false, 64><<<grid_for(n, 64), 64, 0, st>>>(t, pts, n, idx, dist, nullptr, seed);
    else if (t.near_first && t.block_near == 256)
        nearest_fast_kernel<false, 256><<<grid_for(n, 256), 256, 0, st>>>(t, pts, n, idx, dist, nullptr, seed);
    else if (t.near_first)
        nearest_fast_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, pts, n, idx, dist, nullptr, seed);
    else
        nearest_kernel<<<grid_for(n, 128), 128, 0, st>>>(t, pts, n, idx, dist, seed);
    if (!launched)
    {
        note_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && t.out_batch_order)
    {
        scatter2_kernel<<<grid_for(n, 256), 256, 0, st>>>(t.order, n, idx, idx_out,
                                                         reinterpret_cast<const uint32_t *>(dist),
                                                         reinterpret_cast<uint32_t *>(dist_out));
        note_launch();
        e = cudaGetLastError();
    }
    return e;
}
cudaError_t launch_silhouette(const TreeView &t0, const float *pts, const uint8_t *flip, int64_t n, float *dist_out,
                              int32_t *edge_out, cudaStream_t st, uint32_t *stats, const SeedArgs &seed)
{
    if (n <= 0)
        return cudaSuccess;
    TreeView t = t0;
    const bool persistent = (t.persistent & 2) != 0;
    const bool packets = packet_ok(t, t.packet_sil, t.width_sil, seed);
    const bool wide = !packets && wide_ok(t, t.width_sil, persistent, seed);
    const bool lane_persistent = !packets && !wide && !stats && t.near_first && t.num_tris > 1 && persistent;
    const bool supports = packets || wide || (t.near_first && !lane_persistent);
    BatchOut tmp;
    float *dist = dist_out;
    int32_t *edge = edge_out;
    if (supports && batch_order_ok(t, seed, stats))
    {
        cudaError_t e = tmp.alloc(n, 8, st);
        if (e != cudaSuccess)
            return e;
        dist = tmp.at<float>(0);
        edge = edge_out ? tmp.at<int32_t>(align256(4 * (size_t)n)) : nullptr;
        t.out_batch_order = 1;
    }
    cudaError_t e = cudaSuccess;
    bool launched = false;
    if (packets)
    {
        if (stats)
            silhouette_packet_kernel<true>
                <<<grid_for(n, 128), 128, 0, st>>>(t, pts, flip, n, dist, edge, stats, seed);
        else if (n >= t.packet_persistent_min)
        {
            e = t.top_slots && !t.query_mesh
                    ? launch_persistent_smem(silhouette_packet_persistent_kernel<true>,
                                             top_smem_bytes(t.top_slots, true), n, st, t, pts, flip, n, dist, edge,
                                             seed)
                    : launch_persistent(silhouette_packet_persistent_kernel<false>, n, st, t, pts, flip, n, dist, edge,
                                        seed);
            launched = true;
        }
        else
            silhouette_packet_kernel<false>
                <<<grid_for(n, 128), 128, 0, st>>>(t, pts, flip, n, dist, edge, nullptr, seed);
    }
    else if (wide)
    {
        const unsigned g = grid_for(n, 128);
        if (t.width_sil == 4)
            stats ? silhouette_wide_kernel<4, true><<<g, 128, 0, st>>>(t, pts, flip, n, dist, edge, stats, seed)
                  : silhouette_wide_kernel<4, false><<<g, 128, 0, st>>>(t, pts, flip, n, dist, edge, nullptr, seed);
        else
            stats ? silhouette_wide_kernel<8, true><<<g, 128, 0, st>>>(t, pts, flip, n, dist, edge, stats, seed)
                  : silhouette_wide_kernel<8, false><<<g, 128, 0, st>>>(t, pts, flip, n, dist, edge, nullptr, seed);
    }
    else if (stats)
        silhouette_fast_kernel<true><<<grid_for(n, 128), 128, 0, st>>>(t, pts, flip, n, dist, edge, stats, seed);
    else if (lane_persistent)
    {
        e = seed.radius
                ? launch_persistent(silhouette_persistent_kernel<true>, n, st, t, pts, flip, n, dist, edge, seed)
                : launch_persistent(silhouette_persistent_kernel<false>, n, st, t, pts, flip, n, dist, edge, seed);
        launched = true;
    }
    else if (t.near_first && t.block_sil == 64)
        silhouette_fast_kernel<false, 64><<<grid_for(n, 64), 64, 0, st>>>(t, pts, flip, n, dist, edge, nullptr, seed);
    else if (t.near_first && t.block_sil == 256)
        silhouette_fast_kernel<false, 256>
            <<<grid_for(n, 256), 256, 0, st>>>(t, pts, flip, n, dist, edge, nullptr, seed);
    else if (t.near_first)
        silhouette_fast_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, pts, flip, n, dist, edge, nullptr, seed);
    else
        silhouette_kernel<<<grid_for(n, 128), 128, 0, st>>>(t, pts, flip, n, dist, edge, seed);
    if (!launched)
    {
        note_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && t.out_batch_order)
    {
        scatter2_kernel<<<grid_for(n, 256), 256, 0, st>>>(t.order, n, reinterpret_cast<const uint32_t *>(dist),
                                                         reinterpret_cast<uint32_t *>(dist_out),
                                                         reinterpret_cast<const uint32_t *>(edge),
                                                         reinterpret_cast<uint32_t *>(edge_out));
        note_launch();
        e = cudaGetLastError();
    }
    return e;
}
cudaError_t launch_cone_filter_check(int64_t n, uint64_t seed, unsigned long long *counts, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    cone_filter_check_kernel<<<grid_for(n, 256), 256, 0, st>>>(n, seed, counts);
    note_launch();
    return cudaGetLastError();
}
cudaError_t launch_ray(const TreeView &t0, const float *o, const float *d, const float *tmax, int64_t n,
                       uint8_t *hit_out, float *t_out, float *uv_out, uint32_t *idx_out, cudaStream_t st,
                       uint32_t *stats)
{
    if (n <= 0)
        return cudaSuccess;
    TreeView t = t0;
    if (stats)
        ray_kernel<true><<<grid_for(n, 128), 128, 0, st>>>(t, o, d, tmax, n, hit_out, t_out, uv_out, idx_out, stats);
    else if (t.persistent & 4)
        return launch_persistent(ray_persistent_kernel<false>, n, st, t, o, d, tmax, n, hit_out, t_out, uv_out,
                                 idx_out);
    else if (batch_order_ok(t, SeedArgs(), nullptr))
    {
        BatchOut tmp;
        const size_t a_t = align256((size_t)n), a_uv = a_t + align256(4 * (size_t)n),
                     a_idx = a_uv + align256(8 * (size_t)n);
        cudaError_t e = tmp.alloc(n, 17, st);
        if (e != cudaSuccess)
            return e;
        t.out_batch_order = 1;
        ray_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, o, d, tmax, n, tmp.at<uint8_t>(0), tmp.at<float>(a_t),
                                                            tmp.at<float>(a_uv), tmp.at<uint32_t>(a_idx), nullptr);
        note_launch();
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        scatter_ray_kernel<<<grid_for(n, 256), 256, 0, st>>>(
            t.order, n, tmp.at<uint8_t>(0), tmp.at<float>(a_t), tmp.at<float2>(a_uv), tmp.at<uint32_t>(a_idx),
            hit_out, t_out, uv_out, idx_out, (reinterpret_cast<uintptr_t>(uv_out) & 7) == 0);
    }
    else if (kRayPools && n / 4 >= t.packet_persistent_min)
        return launch_persistent(ray_pool_kernel<false>, n, st, t, o, d, tmax, n, hit_out, t_out, uv_out, idx_out);
    else
        ray_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, o, d, tmax, n, hit_out, t_out, uv_out, idx_out,
                                                            nullptr);
    note_launch();
    return cudaGetLastError();
}
cudaError_t launch_ray_test(const TreeView &t, const float *o, const float *d, const float *tmax, int64_t n,
                            uint8_t *hit, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    if (t.persistent & 4)
        return launch_persistent(ray_persistent_kernel<true>, n, st, t, o, d, tmax, n, hit, (float *)nullptr,
                                 (float *)nullptr, (uint32_t *)nullptr);
    if (kRayPools && n / 4 >= t.packet_persistent_min)
        return launch_persistent(ray_pool_kernel<true>, n, st, t, o, d, tmax, n, hit, (float *)nullptr,
                                 (float *)nullptr, (uint32_t *)nullptr);
    ray_kernel<false, true><<<grid_for(n, 128), 128, 0, st>>>(t, o, d, tmax, n, hit, nullptr, nullptr, nullptr,
                                                               nullptr);
    note_launch();
    return cudaGetLastError();
}
cudaError_t launch_sample(const TreeView &t0, const float *c, const float *r, const float *u, int64_t n,
                          int32_t *idx_out, float *pdf_out, cudaStream_t st, uint32_t *stats)
{
    if (n <= 0)
        return cudaSuccess;
    TreeView t = t0;
    if (stats)
        sample_kernel<true><<<grid_for(n, 128), 128, 0, st>>>(t, c, r, u, n, idx_out, pdf_out, stats);
    else if (batch_order_ok(t, SeedArgs(), nullptr))
    {
        BatchOut tmp;
        cudaError_t e = tmp.alloc(n, 8, st);
        if (e != cudaSuccess)
            return e;
        t.out_batch_order = 1;
        int32_t *ti = tmp.at<int32_t>(0);
        float *tp = tmp.at<float>(align256(4 * (size_t)n));
        sample_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, c, r, u, n, ti, tp, nullptr);
        note_launch();
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        scatter2_kernel<<<grid_for(n, 256), 256, 0, st>>>(t.order, n, reinterpret_cast<const uint32_t *>(ti),
                                                         reinterpret_cast<uint32_t *>(idx_out),
                                                         reinterpret_cast<const uint32_t *>(tp),
                                                         reinterpret_cast<uint32_t *>(pdf_out));
    }
    else
        sample_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, c, r, u, n, idx_out, pdf_out, nullptr);
    note_launch();
    return cudaGetLastError();
}
cudaError_t launch_enumerate(const TreeView &t, bool line, const float *q0, const float *q1, int64_t n,
                             uint32_t max_out, uint32_t *idx, float *tt, uint32_t *count, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    if (line)
        enumerate_kernel<true><<<grid_for(n, 128), 128, 0, st>>>(t, q0, q1, n, max_out, idx, tt, count);
    else
        enumerate_kernel<false><<<grid_for(n, 128), 128, 0, st>>>(t, q0, q1, n, max_out, idx, tt, count);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_query_order(const TreeView &t, const float *pts, int64_t n, void *scratch, uint32_t **order,
                               cudaStream_t st, const float *len)
{
    uint32_t *keys = static_cast<uint32_t *>(scratch);
    uint32_t *vals = keys + n, *keys_tmp = vals + n, *vals_tmp = keys_tmp + n;
    void *sort_scratch = vals_tmp + n;
    // batched: mesh ids take the top mesh_bits (>= 2) bits of the key
    int mesh_bits = 2;
    while (mesh_bits < 16 && (1u << mesh_bits) < t.num_meshes)
        ++mesh_bits;
    query_keys_kernel<<<grid_for(n, 256), 256, 0, st>>>(pts, n, t.aabbs, keys, vals, t, mesh_bits, len);
    note_launch();
    cudaError_t e = cudaGetLastError();
    // the batch order only needs to be read: take it from whichever buffer the
    // last pass wrote instead of copying it back (an odd number of passes, as
    // the default 24-bit keys take, ends in the temporaries; the copy cost
    // 0.16 ms per step of four 16M-query batches)
    SortResult res{keys, vals};
    if (e == cudaSuccess)
        e = radix_sort_pairs(keys, vals, keys_tmp, vals_tmp, (uint32_t)n, t.query_mesh ? 32 : t.order_bits, nullptr,
                             sort_scratch, t.status, st, &res);
    *order = res.vals;
    return e;
}
size_t query_order_scratch_bytes(int64_t n) { return 16 * (size_t)n + sort_scratch_bytes((uint32_t)n, 32) + 256; }

// ---- the fallback list of a seeded batch, in the batch's own order
// g[i] = fail_flag of the i-th query in batch order; list = those queries, in order
__global__ void gather_fail_flags_kernel(const uint32_t *__restrict__ order, const uint32_t *__restrict__ flag,
                                         uint32_t n, uint32_t *__restrict__ g)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        g[i] = flag[order ? order[i] : i];
}
__global__ void compact_failed_kernel(const uint32_t *__restrict__ order, const uint32_t *__restrict__ g,
                                      const uint32_t *__restrict__ pos, uint32_t n, uint32_t *__restrict__ list)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && g[i])
        list[pos[i]] = order ? order[i] : i;
}
size_t failed_list_scratch_bytes(int64_t n) { return 8 * (size_t)n + scan_flags_scratch_bytes((uint64_t)n) + 256; }
cudaError_t launch_failed_list(const uint32_t *order, const uint32_t *fail_flag, int64_t n, uint32_t *list,
                               uint32_t *count, void *scratch, uint32_t *status, cudaStream_t st)
{
    if (n <= 0)
        return cudaMemsetAsync(count, 0, 4, st);
    uint32_t *g = static_cast<uint32_t *>(scratch), *pos = g + n;
    void *scan_scratch = pos + n;
    const unsigned grid = (unsigned)((n + 255) / 256);
    gather_fail_flags_kernel<<<grid, 256, 0, st>>>(order, fail_flag, (uint32_t)n, g);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = scan_flags(g, pos, (uint32_t)n, count, scan_scratch, status, st);
    if (e != cudaSuccess)
        return e;
    compact_failed_kernel<<<grid, 256, 0, st>>>(order, g, pos, (uint32_t)n, list);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_sample_point(const float *verts, const int32_t *tris, uint32_t num_tris, const int32_t *idx,
                                const float *u, const float *v, int64_t n, float *out, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    sample_point_kernel<<<grid_for(n, 256), 256, 0, st>>>(verts, tris, num_tris, idx, u, v, n, out);
    note_launch();
    return cudaGetLastError();
}

}  // namespace snch
