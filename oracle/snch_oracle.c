/*
 * CPU oracle for the SNCH-LBVH hot path -- TEST INFRASTRUCTURE ONLY (see snch_oracle.h).
 *
 * Every function restates the reference (tyanyuy3125/snch-lbvh) in plain C and
 * cites the file:line it follows. Compile with -ffp-contract=off: each
 * arithmetic operator is then exactly one binary32 operation, in the
 * reference's left-to-right expression order.
 */
#include "snch_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EPS FLT_EPSILON          /* epsilon<float>(), utility.cuh:186 */
#define ORC_PI ((float)3.14159265358979323846)      /* static_cast<float>(M_PI)   */
#define ORC_PI_2 ((float)1.57079632679489661923)    /* static_cast<float>(M_PI_2) */
#define ORC_INVALID 0xFFFFFFFFu
#define ORC_STACK 256

typedef struct { float x, y, z; } f3;
typedef struct { f3 upper, lower; } box3;                /* aabb.cuh:12-16, upper first */
typedef struct { f3 axis; float half_angle, radius; } cone3; /* cone.cuh:11-16 */
typedef struct { double x, y, z; } d3;

/* std::min / std::max of the reference, argument order included (NaN behaviour) */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }

static inline f3 mk(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
/* dot / length / normalize / cross, utility.cuh:238, 382-389, 427-431, 449-455 */
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float len3(f3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline float sqlen3(f3 a) { return (a.x * a.x + a.y * a.y + a.z * a.z); }
static inline f3 normalize3(f3 v) { float n = len3(v); return mk(v.x / n, v.y / n, v.z / n); }
static inline f3 cross3(f3 u, f3 v) {
    return mk(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
static inline f3 cabs3(f3 a) { return mk(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
static inline f3 vload(const float *v, int32_t i) { return mk(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }

/* ------------------------------------------------------------------ threads */
typedef void (*orc_body)(void *ctx, int64_t begin, int64_t end);
typedef struct { orc_body body; void *ctx; int64_t n, chunk; int64_t next; } orc_pool;

static void *orc_worker(void *arg) {
    orc_pool *p = (orc_pool *)arg;
    for (;;) {
        int64_t b = __atomic_fetch_add(&p->next, p->chunk, __ATOMIC_RELAXED);
        if (b >= p->n) break;
        int64_t e = b + p->chunk < p->n ? b + p->chunk : p->n;
        p->body(p->ctx, b, e);
    }
    return NULL;
}

static void orc_parallel(int64_t n, int nthreads, orc_body body, void *ctx) {
    if (n <= 0) return;
    if (nthreads <= 1 || n < 64) { body(ctx, 0, n); return; }
    if (nthreads > 256) nthreads = 256;
    orc_pool p = {body, ctx, n, 64, 0};
    pthread_t th[256];
    int started = 0;
    for (int i = 0; i < nthreads - 1; ++i)
        if (pthread_create(&th[started], NULL, orc_worker, &p) == 0) ++started;
    orc_worker(&p);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
}

/* ----------------------------------------------------------- topology */
typedef struct { uint64_t key; int64_t occ; } occ_t;
static int occ_cmp(const void *a, const void *b) {
    const occ_t *x = (const occ_t *)a, *y = (const occ_t *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->occ < y->occ ? -1 : (x->occ > y->occ);
}
static int i64_cmp(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return x < y ? -1 : (x > y);
}

/* assign_edge_indices scene.cuh:1135-1166 (edge ids in first-seen order over
 * (triangle, j) with edge j = (v_j, v_{j+1})), compute_silhouettes
 * scene.cuh:1167-1204 (4-vertex edge records, later occurrences overwrite),
 * build_bvh ownership scene.cuh:1207-1225 (first triangle that meets an edge owns it). */
int64_t orc_topology(const int32_t *tris, int64_t nt, int32_t *tri_edges, int32_t *tri_owned,
                     int32_t *edge_verts) {
    int64_t m = 3 * nt;
    occ_t *occ = (occ_t *)malloc(sizeof(occ_t) * (m ? m : 1));
    for (int64_t i = 0; i < nt; ++i)
        for (int j = 0; j < 3; ++j) {
            int32_t I = tris[3 * i + j], J = tris[3 * i + (j + 1) % 3];
            if (I > J) { int32_t t = I; I = J; J = t; }
            occ[3 * i + j].key = ((uint64_t)(uint32_t)I << 32) | (uint32_t)J;
            occ[3 * i + j].occ = 3 * i + j;
        }
    qsort(occ, (size_t)m, sizeof(occ_t), occ_cmp);
    /* group heads = first occurrence of every distinct edge */
    int64_t ngroups = 0;
    int64_t *heads = (int64_t *)malloc(sizeof(int64_t) * (m ? m : 1));
    for (int64_t k = 0; k < m; ++k)
        if (k == 0 || occ[k].key != occ[k - 1].key) heads[ngroups++] = occ[k].occ;
    int64_t *sorted_heads = (int64_t *)malloc(sizeof(int64_t) * (ngroups ? ngroups : 1));
    memcpy(sorted_heads, heads, sizeof(int64_t) * ngroups);
    qsort(sorted_heads, (size_t)ngroups, sizeof(int64_t), i64_cmp);
    /* first-seen rank of a head occurrence -> binary search in sorted_heads */
    int64_t g = -1;
    for (int64_t k = 0; k < m; ++k) {
        if (k == 0 || occ[k].key != occ[k - 1].key) {
            ++g;
            int64_t lo = 0, hi = ngroups - 1, h = heads[g];
            while (lo < hi) { int64_t mid = (lo + hi) / 2; if (sorted_heads[mid] < h) lo = mid + 1; else hi = mid; }
            heads[g] = lo; /* reuse: group -> edge id */
        }
        tri_edges[occ[k].occ] = (int32_t)heads[g];
    }
    free(occ); free(heads); free(sorted_heads);

    for (int64_t e = 0; e < 4 * ngroups; ++e) edge_verts[e] = -1;
    for (int64_t i = 0; i < nt; ++i) {
        const int32_t *vi = tris + 3 * i;
        for (int j = 0; j < 3; ++j) {
            int I = j - 1 < 0 ? 2 : j - 1, J = j, K = j + 1 > 2 ? 0 : j + 1;
            int32_t e = tri_edges[3 * i + j];
            int orientation = 1;
            if (vi[J] > vi[K]) { int t = J; J = K; K = t; orientation = -1; }
            int32_t *se = edge_verts + 4 * (int64_t)e;
            se[orientation == 1 ? 0 : 3] = vi[I];
            se[1] = vi[J];
            se[2] = vi[K];
        }
    }
    uint8_t *seen = (uint8_t *)calloc((size_t)(ngroups ? ngroups : 1), 1);
    for (int64_t i = 0; i < nt; ++i) {
        int p = 0;
        tri_owned[3 * i] = tri_owned[3 * i + 1] = tri_owned[3 * i + 2] = -1;
        for (int j = 0; j < 3; ++j) {
            int32_t e = tri_edges[3 * i + j];
            if (!seen[e]) { seen[e] = 1; tri_owned[3 * i + p++] = e; }
        }
    }
    free(seen);
    return ngroups;
}

/* ----------------------------------------------------------- leaf functors */
/* aabb(p) aabb.cuh:21-50; expand_to_include aabb.cuh:94-101; aabb_getter scene.cuh:870-885 */
static box3 tri_box(const float *verts, const int32_t *t) {
    f3 pa = vload(verts, t[0]), pb = vload(verts, t[1]), pc = vload(verts, t[2]);
    box3 b;
    b.upper = mk(pa.x + ORC_EPS, pa.y + ORC_EPS, pa.z + ORC_EPS);
    b.lower = mk(pa.x - ORC_EPS, pa.y - ORC_EPS, pa.z - ORC_EPS);
    f3 q[2] = {pb, pc};
    for (int k = 0; k < 2; ++k) {
        f3 pl = mk(q[k].x - ORC_EPS, q[k].y - ORC_EPS, q[k].z - ORC_EPS);
        f3 pu = mk(q[k].x + ORC_EPS, q[k].y + ORC_EPS, q[k].z + ORC_EPS);
        b.lower = mk(fminf(b.lower.x, pl.x), fminf(b.lower.y, pl.y), fminf(b.lower.z, pl.z));
        b.upper = mk(fmaxf(b.upper.x, pu.x), fmaxf(b.upper.y, pu.y), fmaxf(b.upper.z, pu.z));
    }
    return b;
}

/* centroid aabb.cuh:271-279: (upper + lower) * 0.5 (double literal, exact halving) */
static inline f3 centroid(box3 b) {
    return mk((float)((double)(b.upper.x + b.lower.x) * 0.5), (float)((double)(b.upper.y + b.lower.y) * 0.5),
              (float)((double)(b.upper.z + b.lower.z) * 0.5));
}

/* silhouette_edge::has_face scene.cuh:741-744 */
static inline int has_face(const int32_t *se, int f) { return f == 0 ? se[3] != -1 : se[0] != -1; }

/* silhouette_edge::normal(f, normalize) scene.cuh:745-771 */
static f3 edge_face_normal(const float *verts, const int32_t *se, int f, int do_normalize) {
    int i, j, k;
    if (f == 0) { i = 3; j = 1; k = 2; } else { i = 0; j = 2; k = 1; }
    f3 pa = vload(verts, se[j]), pb = vload(verts, se[k]), pc = vload(verts, se[i]);
    f3 v1 = sub(pb, pa), v2 = sub(pc, pa);
    f3 n = cross3(v1, v2);
    return do_normalize ? normalize3(n) : n;
}

/* silhouette_edge::normal() scene.cuh:772-786 */
static f3 edge_normal(const float *verts, const int32_t *se) {
    f3 n = mk(0.0f, 0.0f, 0.0f);
    if (has_face(se, 0)) { f3 n0 = edge_face_normal(verts, se, 0, 0); n = mk(n.x + n0.x, n.y + n0.y, n.z + n0.z); }
    if (has_face(se, 1)) { f3 n1 = edge_face_normal(verts, se, 1, 0); n = mk(n.x + n1.x, n.y + n1.y, n.z + n1.z); }
    return normalize3(n);
}

/* cone_getter scene.cuh:887-961 */
static cone3 tri_cone(const float *verts, const int32_t *t, const int32_t *owned, const int32_t *edge_verts) {
    box3 b = tri_box(verts, t);
    f3 c = centroid(b);
    cone3 r;
    r.axis = mk(0.0f, 0.0f, 0.0f);
    r.half_angle = ORC_PI;
    r.radius = 0.0f;
    int any = 0, all_two = 1;
    for (int i = 0; i < 3; ++i) {
        int32_t s = owned[i];
        if (s == -1) continue;
        const int32_t *se = edge_verts + 4 * (int64_t)s;
        f3 sn = edge_normal(verts, se);
        r.axis.x += sn.x; r.axis.y += sn.y; r.axis.z += sn.z;
        f3 pa = vload(verts, se[1]), pb = vload(verts, se[2]);
        f3 sc = mk((pa.x + pb.x) / 2, (pa.y + pb.y) / 2, (pa.z + pb.z) / 2); /* centroid() 734-740 */
        r.radius = smax(r.radius, len3(mk(sc.x - c.x, sc.y - c.y, sc.z - c.z)));
        all_two = all_two && has_face(se, 0) && has_face(se, 1);
        any = 1;
    }
    if (!any) {
        r.half_angle = -ORC_PI;
    } else if (!all_two) {
        r.half_angle = ORC_PI;
    } else {
        float axis_norm = len3(r.axis);
        if (axis_norm > ORC_EPS) {
            r.axis.x /= axis_norm; r.axis.y /= axis_norm; r.axis.z /= axis_norm;
            r.half_angle = 0.0f;
            for (int i = 0; i < 3; ++i) {
                int32_t s = owned[i];
                if (s == -1) continue;
                const int32_t *se = edge_verts + 4 * (int64_t)s;
                f3 fn[2];
                fn[0] = has_face(se, 0) ? edge_face_normal(verts, se, 0, 1) : mk(0.0f, 0.0f, 0.0f);
                fn[1] = has_face(se, 1) ? edge_face_normal(verts, se, 1, 1) : mk(0.0f, 0.0f, 0.0f);
                for (int j = 0; j < 2; ++j) {
                    float angle = acosf(smax(-1.0f, smin(1.0f, dot3(r.axis, fn[j]))));
                    r.half_angle = smax(r.half_angle, angle);
                }
            }
        }
    }
    return r;
}

void orc_leaf_aabbs(const float *verts, const int32_t *tris, int64_t nt, float *out) {
    for (int64_t i = 0; i < nt; ++i) {
        box3 b = tri_box(verts, tris + 3 * i);
        memcpy(out + 6 * i, &b, sizeof(b));
    }
}

void orc_leaf_cones(const float *verts, const int32_t *tris, int64_t nt, const int32_t *tri_owned,
                    const int32_t *edge_verts, float *out) {
    for (int64_t i = 0; i < nt; ++i) {
        cone3 c = tri_cone(verts, tris + 3 * i, tri_owned + 3 * i, edge_verts);
        memcpy(out + 5 * i, &c, sizeof(c));
    }
}

/* ----------------------------------------------------------- build */
/* expand_bits morton_code.cuh:19-38 */
static uint32_t expand_bits(uint32_t v) {
    v = (v | (v << 16)) & 0x070000FFu;
    v = (v | (v << 8)) & 0x0700F00Fu;
    v = (v | (v << 4)) & 0x430C30C3u;
    v = (v | (v << 2)) & 0x49249249u;
    return v;
}
/* morton_code(float3, 1024) morton_code.cuh:61-70 */
static uint32_t morton3(f3 p) {
    const float res = 1024.0f;
    p.x = fminf(fmaxf(p.x * res, 0.0f), res - 1.0f);
    p.y = fminf(fmaxf(p.y * res, 0.0f), res - 1.0f);
    p.z = fminf(fmaxf(p.z * res, 0.0f), res - 1.0f);
    uint32_t xx = expand_bits((uint32_t)p.x), yy = expand_bits((uint32_t)p.y), zz = expand_bits((uint32_t)p.z);
    return xx * 4 + yy * 2 + zz;
}

static inline int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }
static inline int clz64(uint64_t v) { return v ? __builtin_clzll(v) : 64; }

/* common_upper_bits morton_code.cuh:144-167, on the 32-bit codes when they
 * are unique and on (code << 32 | sorted index) otherwise (bvh.cuh:459-476) */
typedef struct { const uint64_t *keys; int wide; } keyset;
static inline int cub(const keyset *k, uint64_t a, uint64_t b) {
    return k->wide ? clz64(a ^ b) : clz32((uint32_t)(a ^ b));
}

/* determine_range bvh.cuh:109-167 (the reference's unsigned index arithmetic kept) */
static void determine_range(const keyset *ks, unsigned num_leaves, unsigned idx, unsigned *lo, unsigned *hi) {
    if (idx == 0) { *lo = 0; *hi = num_leaves - 1; return; }
    const uint64_t *c = ks->keys;
    uint64_t self = c[idx];
    int L_delta = cub(ks, self, c[idx - 1]);
    int R_delta = cub(ks, self, c[idx + 1]);
    int d = (R_delta > L_delta) ? 1 : -1;
    int delta_min = L_delta < R_delta ? L_delta : R_delta;
    int l_max = 2;
    int delta = -1;
    int i_tmp = (int)(idx + (unsigned)(d * l_max));
    if (0 <= i_tmp && (unsigned)i_tmp < num_leaves) delta = cub(ks, self, c[i_tmp]);
    while (delta > delta_min) {
        l_max <<= 1;
        i_tmp = (int)(idx + (unsigned)(d * l_max));
        delta = -1;
        if (0 <= i_tmp && (unsigned)i_tmp < num_leaves) delta = cub(ks, self, c[i_tmp]);
    }
    int l = 0;
    int t = l_max >> 1;
    while (t > 0) {
        i_tmp = (int)(idx + (unsigned)((l + t) * d));
        delta = -1;
        if (0 <= i_tmp && (unsigned)i_tmp < num_leaves) delta = cub(ks, self, c[i_tmp]);
        if (delta > delta_min) l += t;
        t >>= 1;
    }
    unsigned jdx = idx + (unsigned)(l * d);
    if (d < 0) { unsigned s = idx; idx = jdx; jdx = s; }
    *lo = idx; *hi = jdx;
}

/* find_split bvh.cuh:169-199 */
static unsigned find_split(const keyset *ks, unsigned first, unsigned last) {
    const uint64_t *c = ks->keys;
    uint64_t fc = c[first], lc = c[last];
    if (fc == lc) return (first + last) >> 1;
    int delta_node = cub(ks, fc, lc);
    int split = (int)first;
    int stride = (int)(last - first);
    do {
        stride = (stride + 1) >> 1;
        int middle = split + stride;
        if ((unsigned)middle < last) {
            int delta = cub(ks, fc, c[middle]);
            if (delta > delta_node) split = middle;
        }
    } while (stride > 1);
    return (unsigned)split;
}

/* rotate(float3) cone.cuh:288-302 */
static f3 rotate3(f3 u, f3 v, float theta) {
    float ct = cosf(theta), st = sinf(theta);
    f3 w = normalize3(cross3(u, v));
    f3 o = mk((1.0f - ct) * w.x, (1.0f - ct) * w.y, (1.0f - ct) * w.z);
    float R[3][3] = {{ct + o.x * w.x, o.y * w.x - st * w.z, o.z * w.x + st * w.y},
                     {o.x * w.y + st * w.z, ct + o.y * w.y, o.z * w.y - st * w.x},
                     {o.x * w.z - st * w.y, o.y * w.z + st * w.x, ct + o.z * w.z}};
    return mk(R[0][0] * u.x + R[0][1] * u.y + R[0][2] * u.z, R[1][0] * u.x + R[1][1] * u.y + R[1][2] * u.z,
              R[2][0] * u.x + R[2][1] * u.y + R[2][2] * u.z);
}

/* merge(cone, cone, ...) cone.cuh:427-480. Where the reference leaves
 * half_angle unassigned (o_theta >= pi, lines 454-458) this stores pi. */
static cone3 cone_merge(cone3 a, cone3 b, f3 oa, f3 ob, f3 on, int *d1) {
    cone3 r;
    r.axis = mk(0.0f, 0.0f, 0.0f); r.half_angle = 0.0f; r.radius = 0.0f;
    int va = a.half_angle >= 0.0f, vb = b.half_angle >= 0.0f; /* is_valid cone.cuh:18-22 */
    if (va && vb) {
        f3 axis_a = a.axis, axis_b = b.axis;
        float ha = a.half_angle, hb = b.half_angle;
        f3 da = sub(on, oa), db = sub(on, ob);
        r.radius = sqrtf(smax(a.radius * a.radius + sqlen3(da), b.radius * b.radius + sqlen3(db)));
        if (hb > ha) { f3 t = axis_a; axis_a = axis_b; axis_b = t; float h = ha; ha = hb; hb = h; }
        float theta = acosf(smax(-1.0f, smin(1.0f, dot3(axis_a, axis_b))));
        if (smin(theta + hb, ORC_PI) <= ha) { r.axis = axis_a; r.half_angle = ha; return r; }
        float o_theta = (ha + theta + hb) / 2.0f;
        if (o_theta >= ORC_PI) { r.axis = axis_a; r.half_angle = ORC_PI; *d1 = 1; return r; }
        float r_theta = o_theta - ha;
        r.axis = rotate3(axis_a, axis_b, r_theta);
        r.half_angle = o_theta;
    } else if (va) {
        r = a;
    } else if (vb) {
        r = b;
    } else {
        r.half_angle = -ORC_PI;
    }
    return r;
}

typedef struct { uint64_t key; } sortkey;
static int u64_cmp(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return x < y ? -1 : (x > y);
}

int orc_build(const float *verts, const int32_t *tris, int64_t nt, const int32_t *tri_owned,
              const int32_t *edge_verts, uint32_t *morton, uint32_t *sorted_idx, uint32_t *nodes,
              float *aabbs, float *cones, uint8_t *d1_flags) {
    if (nt <= 0) return 1;
    const unsigned N = (unsigned)nt, NI = N - 1, NN = 2 * N - 1;
    box3 *bx = (box3 *)aabbs;
    cone3 *cn = (cone3 *)cones;
    box3 *leaf_box = (box3 *)malloc(sizeof(box3) * N);
    cone3 *leaf_cone = (cone3 *)malloc(sizeof(cone3) * N);
    for (unsigned i = 0; i < N; ++i) {
        leaf_box[i] = tri_box(verts, tris + 3 * (int64_t)i);
        leaf_cone[i] = tri_cone(verts, tris + 3 * (int64_t)i, tri_owned + 3 * (int64_t)i, edge_verts);
    }
    /* scene AABB: thrust::reduce with merge, bvh.cuh:428-432; merge aabb.cuh:113-124 */
    box3 whole;
    whole.upper = mk(-INFINITY, -INFINITY, -INFINITY);
    whole.lower = mk(INFINITY, INFINITY, INFINITY);
    for (unsigned i = 0; i < N; ++i) {
        whole.upper = mk(fmaxf(whole.upper.x, leaf_box[i].upper.x), fmaxf(whole.upper.y, leaf_box[i].upper.y),
                         fmaxf(whole.upper.z, leaf_box[i].upper.z));
        whole.lower = mk(fminf(whole.lower.x, leaf_box[i].lower.x), fminf(whole.lower.y, leaf_box[i].lower.y),
                         fminf(whole.lower.z, leaf_box[i].lower.z));
    }
    /* default_morton_code_calculator<Real,3> bvh.cuh:281-304 */
    for (unsigned i = 0; i < N; ++i) {
        f3 p = centroid(leaf_box[i]);
        p.x -= whole.lower.x; p.y -= whole.lower.y; p.z -= whole.lower.z;
        p.x /= (whole.upper.x - whole.lower.x);
        p.y /= (whole.upper.y - whole.lower.y);
        p.z /= (whole.upper.z - whole.lower.z);
        morton[i] = morton3(p);
    }
    /* stable_sort_by_key bvh.cuh:444-454 == sort by (code, original index) */
    uint64_t *ck = (uint64_t *)malloc(sizeof(uint64_t) * N);
    for (unsigned i = 0; i < N; ++i) ck[i] = ((uint64_t)morton[i] << 32) | i;
    qsort(ck, N, sizeof(uint64_t), u64_cmp);
    int unique = 1;
    for (unsigned i = 0; i < N; ++i) {
        sorted_idx[i] = (uint32_t)(ck[i] & 0xFFFFFFFFu);
        if (i > 0 && (ck[i] >> 32) == (ck[i - 1] >> 32)) unique = 0;
    }
    /* node codes: 32-bit when unique, else (m << 32) | idx (bvh.cuh:459-476) */
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * N);
    for (unsigned i = 0; i < N; ++i) keys[i] = unique ? (ck[i] >> 32) : ck[i];
    keyset ks = {keys, !unique};

    /* nodes: defaults bvh.cuh:481-499; boxes/cones defaults bvh.cuh:395-420 */
    for (unsigned i = 0; i < NN; ++i) {
        nodes[4 * i] = nodes[4 * i + 1] = nodes[4 * i + 2] = nodes[4 * i + 3] = ORC_INVALID;
        bx[i].upper = mk(-INFINITY, -INFINITY, -INFINITY);
        bx[i].lower = mk(INFINITY, INFINITY, INFINITY);
        cn[i].axis = mk(0.0f, 0.0f, 0.0f); cn[i].half_angle = ORC_PI; cn[i].radius = 0.0f;
        if (d1_flags) d1_flags[i] = 0;
    }
    for (unsigned j = 0; j < N; ++j) {
        nodes[4 * (NI + j) + 3] = sorted_idx[j];
        bx[NI + j] = leaf_box[sorted_idx[j]];
        cn[NI + j] = leaf_cone[sorted_idx[j]];
    }
    /* construct_internal_nodes bvh.cuh:200-229 */
    for (unsigned idx = 0; idx < NI; ++idx) {
        unsigned lo, hi;
        determine_range(&ks, N, idx, &lo, &hi);
        int gamma = (int)find_split(&ks, lo, hi);
        uint32_t left = (uint32_t)gamma, right = (uint32_t)gamma + 1;
        if ((lo < hi ? lo : hi) == (unsigned)gamma) left += NI;
        if ((lo > hi ? lo : hi) == (unsigned)gamma + 1) right += NI;
        nodes[4 * idx + 1] = left;
        nodes[4 * idx + 2] = right;
        nodes[4 * idx + 3] = ORC_INVALID;
        nodes[4 * left] = idx;
        nodes[4 * right] = idx;
    }
    /* bottom-up refits bvh.cuh:517-604: every internal node after its two
     * children (explicit post-order); the result does not depend on the order. */
    if (NI > 0) {
        uint32_t *stk = (uint32_t *)malloc(sizeof(uint32_t) * 2 * NN);
        uint8_t *expanded = (uint8_t *)calloc(NN, 1);
        int64_t sp = 0;
        stk[sp++] = 0;
        while (sp > 0) {
            uint32_t p = stk[sp - 1];
            uint32_t L = nodes[4 * p + 1], R = nodes[4 * p + 2];
            if (!expanded[p]) {
                expanded[p] = 1;
                if (R < NI) stk[sp++] = R;
                if (L < NI) stk[sp++] = L;
                continue;
            }
            --sp;
            box3 lb = bx[L], rb = bx[R], m;
            m.upper = mk(fmaxf(lb.upper.x, rb.upper.x), fmaxf(lb.upper.y, rb.upper.y), fmaxf(lb.upper.z, rb.upper.z));
            m.lower = mk(fminf(lb.lower.x, rb.lower.x), fminf(lb.lower.y, rb.lower.y), fminf(lb.lower.z, rb.lower.z));
            bx[p] = m;
            int d1 = 0;
            cn[p] = cone_merge(cn[L], cn[R], centroid(lb), centroid(rb), centroid(m), &d1);
            if (d1_flags) d1_flags[p] = (uint8_t)d1;
        }
        free(stk); free(expanded);
    }
    free(keys); free(ck); free(leaf_box); free(leaf_cone);
    return unique;
}

int orc_max_depth(const uint32_t *nodes, int64_t nt) {
    if (nt <= 1) return 0;
    const uint32_t NI = (uint32_t)(nt - 1);
    int best = 0;
    for (int64_t j = 0; j < nt; ++j) {
        int d = 0;
        uint32_t n = NI + (uint32_t)j;
        while (nodes[4 * n] != ORC_INVALID) { n = nodes[4 * n]; ++d; }
        if (d > best) best = d;
    }
    return best;
}

void orc_leaf_ranks(const uint32_t *nodes, int64_t nt, uint32_t *ranks) {
    if (nt <= 0) return;
    if (nt == 1) { ranks[0] = 0; return; }
    const uint32_t NI = (uint32_t)(nt - 1);
    uint32_t *stk = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)nt);
    int64_t sp = 0;
    uint32_t r = 0;
    stk[sp++] = 0;
    while (sp > 0) {
        uint32_t n = stk[--sp];
        uint32_t L = nodes[4 * n + 1], R = nodes[4 * n + 2];
        if (L >= NI) ranks[L - NI] = r++;
        if (R >= NI) ranks[R - NI] = r++;
        if (L < NI) stk[sp++] = L;
        if (R < NI) stk[sp++] = R;
    }
    free(stk);
}

/* ----------------------------------------------------------- query math */
/* mindist aabb.cuh:144-150 */
static inline float mindist(box3 b, f3 p) {
    float dx = fminf(b.upper.x, fmaxf(b.lower.x, p.x)) - p.x;
    float dy = fminf(b.upper.y, fmaxf(b.lower.y, p.y)) - p.y;
    float dz = fminf(b.upper.z, fmaxf(b.lower.z, p.z)) - p.z;
    return dx * dx + dy * dy + dz * dz;
}
/* minmaxdist aabb.cuh:182-209 */
static inline float minmaxdist(box3 b, f3 p) {
    f3 rm = mk((b.lower.x - p.x) * (b.lower.x - p.x), (b.lower.y - p.y) * (b.lower.y - p.y),
               (b.lower.z - p.z) * (b.lower.z - p.z));
    f3 rM = mk((b.upper.x - p.x) * (b.upper.x - p.x), (b.upper.y - p.y) * (b.upper.y - p.y),
               (b.upper.z - p.z) * (b.upper.z - p.z));
    float t;
    if ((b.upper.x + b.lower.x) * 0.5f < p.x) { t = rm.x; rm.x = rM.x; rM.x = t; }
    if ((b.upper.y + b.lower.y) * 0.5f < p.y) { t = rm.y; rm.y = rM.y; rM.y = t; }
    if ((b.upper.z + b.lower.z) * 0.5f < p.z) { t = rm.z; rm.z = rM.z; rM.z = t; }
    float dx = rm.x + rM.y + rM.z;
    float dy = rM.x + rm.y + rM.z;
    float dz = rM.x + rM.y + rm.z;
    return fminf(dx, fminf(dy, dz));
}

/* find_closest_point_triangle scene.cuh:34-110 (returns the distance) */
static float closest_point_triangle(f3 pa, f3 pb, f3 pc, f3 x) {
    f3 ab = sub(pb, pa), ac = sub(pc, pa), ax = sub(x, pa);
    float d1 = dot3(ab, ax), d2 = dot3(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f) return len3(sub(x, pa));
    f3 bx = sub(x, pb);
    float d3 = dot3(ab, bx), d4 = dot3(ac, bx);
    if (d3 >= 0.0f && d4 <= d3) return len3(sub(x, pb));
    f3 cx = sub(x, pc);
    float d5 = dot3(ab, cx), d6 = dot3(ac, cx);
    if (d6 >= 0.0f && d5 <= d6) return len3(sub(x, pc));
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = d1 / (d1 - d3);
        f3 pt = mk(pa.x + ab.x * v, pa.y + ab.y * v, pa.z + ab.z * v);
        return len3(sub(x, pt));
    }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        float w = d2 / (d2 - d6);
        f3 pt = mk(pa.x + ac.x * w, pa.y + ac.y * w, pa.z + ac.z * w);
        return len3(sub(x, pt));
    }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        f3 pt = mk(pb.x + (pc.x - pb.x) * w, pb.y + (pc.y - pb.y) * w, pb.z + (pc.z - pb.z) * w);
        return len3(sub(x, pt));
    }
    float denom = 1.0f / (va + vb + vc);
    float v = vb * denom, w = vc * denom;
    f3 pt = mk(pa.x + ab.x * v + ac.x * w, pa.y + ab.y * v + ac.y * w, pa.z + ab.z * v + ac.z * w);
    return len3(sub(x, pt));
}

static inline box3 node_box(const orc_scene *s, uint32_t n) {
    box3 b;
    memcpy(&b, s->aabbs + 6 * (int64_t)n, sizeof(b));
    return b;
}
static inline cone3 node_cone(const orc_scene *s, uint32_t n) {
    cone3 c;
    memcpy(&c, s->cones + 5 * (int64_t)n, sizeof(c));
    return c;
}
static inline float tri_distance(const orc_scene *s, uint32_t obj, f3 p) {
    const int32_t *t = s->tris + 3 * (int64_t)obj;
    return closest_point_triangle(vload(s->verts, t[0]), vload(s->verts, t[1]), vload(s->verts, t[2]), p);
}

/* query_device(nearest) query.cuh:239-318. A one-leaf tree (N = 1), where the
 * reference reads past its node array, evaluates that leaf directly. */
typedef struct { const orc_scene *s; const float *pts; uint32_t *idx; float *dist; uint32_t *stats; } near_ctx;
static void near_body(void *vc, int64_t b, int64_t e) {
    near_ctx *c = (near_ctx *)vc;
    const orc_scene *s = c->s;
    typedef struct { uint32_t n; float d; } ent;
    ent stk[ORC_STACK];
    for (int64_t q = b; q < e; ++q) {
        f3 p = mk(c->pts[3 * q], c->pts[3 * q + 1], c->pts[3 * q + 2]);
        uint32_t nearest = ORC_INVALID, n_int = 0, n_leaf = 0;
        float best = INFINITY;
        if (s->num_tris == 1) {
            float d = tri_distance(s, s->nodes[3], p);
            d *= d;
            best = d; nearest = s->nodes[3]; n_leaf = 1;
        } else if (s->num_tris > 1) {
            int sp = 0;
            stk[sp].n = 0; stk[sp].d = mindist(node_box(s, 0), p); ++sp;
            do {
                ent nd = stk[--sp];
                if (nd.d > best) continue;
                ++n_int;
                uint32_t L = s->nodes[4 * nd.n + 1], R = s->nodes[4 * nd.n + 2];
                box3 lb = node_box(s, L), rb = node_box(s, R);
                float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
                float Lmmd = minmaxdist(lb, p), Rmmd = minmaxdist(rb, p);
                if (Lmd <= Rmmd) {
                    uint32_t obj = s->nodes[4 * L + 3];
                    if (obj != ORC_INVALID) {
                        float d = tri_distance(s, obj, p); ++n_leaf;
                        d *= d;
                        if (d <= best) { best = d; nearest = obj; }
                    } else { stk[sp].n = L; stk[sp].d = Lmd; ++sp; }
                }
                if (Rmd <= Lmmd) {
                    uint32_t obj = s->nodes[4 * R + 3];
                    if (obj != ORC_INVALID) {
                        float d = tri_distance(s, obj, p); ++n_leaf;
                        d *= d;
                        if (d <= best) { best = d; nearest = obj; }
                    } else { stk[sp].n = R; stk[sp].d = Rmd; ++sp; }
                }
                if (sp >= ORC_STACK - 2) { nearest = ORC_INVALID; best = NAN; break; }
            } while (sp > 0);
        }
        c->idx[q] = nearest;
        c->dist[q] = sqrtf(best);
        if (c->stats) { c->stats[3 * q] = n_int; c->stats[3 * q + 1] = n_leaf; c->stats[3 * q + 2] = 0; }
    }
}
void orc_query_nearest(const orc_scene *s, const float *pts, int64_t n, uint32_t *idx, float *dist,
                       uint32_t *stats, int nthreads) {
    near_ctx c = {s, pts, idx, dist, stats};
    orc_parallel(n, nthreads, near_body, &c);
}

/* compute_orthonormal_basis(float3) cone.cuh:34-42 and project_to_plane 58-66 */
static float project_to_plane(f3 n, f3 e) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    f3 b1 = mk(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f3 b2 = mk(b, sign + n.y * n.y * a, -n.y);
    float r1 = dot3(e, cabs3(b1));
    float r2 = dot3(e, cabs3(b2));
    return sqrtf(r1 * r1 + r2 * r2);
}
static inline int inrange(float v, float lo, float hi) { return v >= lo && v <= hi; } /* utility.cuh:241 */

/* overlap(cone<float,3>, ...) cone.cuh:168-212 */
static int cone_overlap(cone3 bc, f3 o, box3 b, float dist_to_box) {
    if (bc.half_angle >= ORC_PI_2 || dist_to_box < ORC_EPS) return 1;
    f3 c = centroid(b);
    f3 v = mk(c.x - o.x, c.y - o.y, c.z - o.z);
    float l = len3(v);
    v.x /= l; v.y /= l; v.z /= l;
    float dax = acosf(smax(-1.0f, smin(1.0f, dot3(bc.axis, v))));
    if (inrange(ORC_PI_2, dax - bc.half_angle, dax + bc.half_angle)) return 1;
    if (l > bc.radius) {
        float vch = asinf(bc.radius / l);
        float hs = bc.half_angle + vch;
        float mn = dax - hs, mx = dax + hs;
        return hs >= ORC_PI_2 ? 1 : inrange(ORC_PI_2, mn, mx);
    }
    f3 e = mk(b.upper.x - c.x, b.upper.y - c.y, b.upper.z - c.z);
    float d = dot3(e, cabs3(v));
    float sdist = l - d;
    if (sdist <= 0.0f) return 1;
    d = project_to_plane(v, e);
    float vch = atan2f(d, sdist);
    float hs = bc.half_angle + vch;
    float mn = dax - hs, mx = dax + hs;
    return hs >= ORC_PI_2 ? 1 : inrange(ORC_PI_2, mn, mx);
}

/* find_closest_point_line_segment(float3) scene.cuh:230-255 */
static float closest_point_segment(f3 pa, f3 pb, f3 x, f3 *pt) {
    f3 u = sub(pb, pa), v = sub(x, pa);
    float c1 = dot3(u, v);
    if (c1 <= 0.0f) { *pt = pa; return len3(sub(x, *pt)); }
    float c2 = dot3(u, u);
    if (c2 <= c1) { *pt = pb; return len3(sub(x, *pt)); }
    float t = c1 / c2;
    *pt = mk(pa.x + u.x * t, pa.y + u.y * t, pa.z + u.z * t);
    return len3(sub(x, *pt));
}

/* is_silhouette_edge scene.cuh:143-174 (view_dir is not normalised there) */
static int is_silhouette_edge(f3 pa, f3 pb, f3 n0, f3 n1, f3 view_dir, float d, int flip) {
    const float precision = 1e-3f;
    float sign = flip ? 1.0f : -1.0f;
    if (d <= precision) {
        f3 ed = normalize3(sub(pb, pa));
        float sda = atan2f(dot3(ed, cross3(n0, n1)), dot3(n0, n1));
        return sign * sda > precision;
    }
    float dot0 = dot3(view_dir, n0), dot1 = dot3(view_dir, n1);
    if (fabsf(dot0) <= precision) return sign * dot1 > precision;
    if (fabsf(dot1) <= precision) return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}

/* silhouette_edge::find_closest_silhouette_point scene.cuh:788-824 */
static int closest_silhouette_point(const orc_scene *s, const int32_t *se, f3 o, float max_r2, float *dist,
                                    int flip, float min_r2) {
    if (min_r2 >= max_r2) return 0;
    f3 pa = vload(s->verts, se[1]), pb = vload(s->verts, se[2]);
    f3 cp;
    float d = closest_point_segment(pa, pb, o, &cp);
    if (d * d > max_r2) return 0;
    int is_sil = !has_face(se, 0) || !has_face(se, 1);
    if (!is_sil) {
        f3 n0 = edge_face_normal(s->verts, se, 0, 1), n1 = edge_face_normal(s->verts, se, 1, 1);
        f3 vd = mk(o.x - cp.x, o.y - cp.y, o.z - cp.z);
        is_sil = is_silhouette_edge(pa, pb, n0, n1, vd, d, flip);
    }
    if (is_sil && d * d <= max_r2) { *dist = d; return 1; }
    return 0;
}

/* silhouette_distance_calculator scene.cuh:978-1003; *edge receives the id of
 * the edge that produced the returned distance */
static int leaf_silhouette(const orc_scene *s, uint32_t obj, f3 o, float max_r2, float *dist, int flip,
                           int32_t *edge, uint32_t *n_edges) {
    const int32_t *own = s->tri_owned + 3 * (int64_t)obj;
    float mr2 = max_r2;
    int ret = 0;
    for (int i = 0; i < 3; ++i) {
        int32_t si = own[i];
        if (si == -1) continue;
        ++*n_edges;
        if (closest_silhouette_point(s, s->edge_verts + 4 * (int64_t)si, o, mr2, dist, flip, 0.0f)) {
            ret = 1;
            mr2 = *dist * *dist;
            *edge = si;
        }
    }
    return ret;
}

/* query_device(nearest_silhouette) query.cuh:326-423; a one-leaf tree
 * evaluates its leaf directly */
typedef struct { const orc_scene *s; const float *pts; const uint8_t *flip; float *dist; int32_t *edge; uint32_t *stats; } sil_ctx;
static void sil_body(void *vc, int64_t b, int64_t e) {
    sil_ctx *c = (sil_ctx *)vc;
    const orc_scene *s = c->s;
    typedef struct { uint32_t n; float d; } ent;
    ent stk[ORC_STACK];
    for (int64_t q = b; q < e; ++q) {
        f3 p = mk(c->pts[3 * q], c->pts[3 * q + 1], c->pts[3 * q + 2]);
        int flip = c->flip ? c->flip[q] != 0 : 0;
        float best = INFINITY;
        int32_t best_edge = -1;
        uint32_t n_int = 0, n_leaf = 0, n_edge = 0;
        if (s->num_tris == 1) {
            float dist = INFINITY; int32_t eid = -1;
            if (leaf_silhouette(s, s->nodes[3], p, best * best, &dist, flip, &eid, &n_edge) && dist <= best) {
                best = dist; best_edge = eid;
            }
            n_leaf = 1;
        } else if (s->num_tris > 1) {
            int sp = 0;
            stk[sp].n = 0; stk[sp].d = mindist(node_box(s, 0), p); ++sp;
            do {
                ent nd = stk[--sp];
                if (nd.d > best * best) continue;
                ++n_int;
                uint32_t L = s->nodes[4 * nd.n + 1], R = s->nodes[4 * nd.n + 2];
                box3 lb = node_box(s, L), rb = node_box(s, R);
                cone3 lc = node_cone(s, L), rc = node_cone(s, R);
                float Lmd = mindist(lb, p), Rmd = mindist(rb, p);
                int hitL = lc.half_angle >= 0.0f && cone_overlap(lc, p, lb, Lmd);
                int hitR = rc.half_angle >= 0.0f && cone_overlap(rc, p, rb, Rmd);
                uint32_t ch[2] = {L, R};
                int hit[2] = {hitL, hitR};
                float md[2] = {Lmd, Rmd};
                for (int k = 0; k < 2; ++k) {
                    if (!hit[k]) continue;
                    uint32_t obj = s->nodes[4 * ch[k] + 3];
                    if (obj != ORC_INVALID) {
                        float dist = INFINITY; int32_t eid = -1;
                        ++n_leaf;
                        int found = leaf_silhouette(s, obj, p, best * best, &dist, flip, &eid, &n_edge);
                        if (found && dist <= best) { best = dist; best_edge = eid; }
                    } else { stk[sp].n = ch[k]; stk[sp].d = md[k]; ++sp; }
                }
                if (sp >= ORC_STACK - 2) { best = NAN; best_edge = -1; break; }
            } while (sp > 0);
        }
        c->dist[q] = best;
        if (c->edge) c->edge[q] = best_edge;
        if (c->stats) { c->stats[3 * q] = n_int; c->stats[3 * q + 1] = n_leaf; c->stats[3 * q + 2] = n_edge; }
    }
}
void orc_query_silhouette(const orc_scene *s, const float *pts, const uint8_t *flip, int64_t n, float *dist,
                          int32_t *edge, uint32_t *stats, int nthreads) {
    sil_ctx c = {s, pts, flip, dist, edge, stats};
    orc_parallel(n, nthreads, sil_body, &c);
}

/* intersects_d(ray<float,3>) aabb.cuh:397-431 */
static int ray_box(f3 o, f3 inv, box3 b, float max_dist, float *dist) {
    float t1 = (b.lower.x - o.x) * inv.x, t2 = (b.upper.x - o.x) * inv.x;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b.lower.y - o.y) * inv.y; t2 = (b.upper.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(t1, t2)); tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = (b.lower.z - o.z) * inv.z; t2 = (b.upper.z - o.z) * inv.z;
    tmin = fmaxf(tmin, fminf(t1, t2)); tmax = fminf(tmax, fmaxf(t1, t2));
    if (tmax >= tmin && tmax >= 0.0f && tmin <= max_dist) {
        *dist = tmin >= 0.0f ? tmin : 0.0f;
        return 1;
    }
    return 0;
}

/* intersect_test scene.cuh:1005-1052 (Moller-Trumbore; __frcp_rn == 1/x correctly rounded) */
static int ray_triangle(f3 o, f3 dir, f3 v0, f3 v1, f3 v2, float *t, float *u_out, float *v_out) {
    f3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    f3 h = mk(dir.y * e2.z - dir.z * e2.y, dir.z * e2.x - dir.x * e2.z, dir.x * e2.y - dir.y * e2.x);
    float det = e1.x * h.x + e1.y * h.y + e1.z * h.z;
    if (fabsf(det) < ORC_EPS) return 0;
    float inv_det = 1.0f / det;
    f3 s = sub(o, v0);
    float u = (s.x * h.x + s.y * h.y + s.z * h.z) * inv_det;
    if (u < 0.0f || u > 1.0f) return 0;
    f3 q = mk(s.y * e1.z - s.z * e1.y, s.z * e1.x - s.x * e1.z, s.x * e1.y - s.y * e1.x);
    float v = (dir.x * q.x + dir.y * q.y + dir.z * q.z) * inv_det;
    if (v < 0.0f || u + v > 1.0f) return 0;
    float tt = (e2.x * q.x + e2.y * q.y + e2.z * q.z) * inv_det;
    if (tt >= 0.0f) { *t = tt; *u_out = u; *v_out = v; return 1; }
    return 0;
}

/* query_device(ray_intersect) query.cuh:79-169; ray ctor aabb.cuh:298-313 */
typedef struct { const orc_scene *s; const float *o, *d, *tmax; uint8_t *hit; float *t, *uv; uint32_t *idx, *stats; } ray_ctx;
static void ray_body(void *vc, int64_t b, int64_t e) {
    ray_ctx *c = (ray_ctx *)vc;
    const orc_scene *s = c->s;
    typedef struct { uint32_t n; float d; } ent;
    ent stk[ORC_STACK];
    for (int64_t q = b; q < e; ++q) {
        f3 o = mk(c->o[3 * q], c->o[3 * q + 1], c->o[3 * q + 2]);
        f3 dir = mk(c->d[3 * q], c->d[3 * q + 1], c->d[3 * q + 2]);
        f3 inv = mk(1 / dir.x, 1 / dir.y, 1 / dir.z);
        float max_dist = c->tmax[q];
        float min_dist = INFINITY, bu = 0.0f, bv = 0.0f;
        int found = 0;
        uint32_t nearest = ORC_INVALID, n_int = 0, n_leaf = 0;
        if (s->num_tris > 0) {
            int sp = 0;
            stk[sp].n = 0; stk[sp].d = INFINITY; ++sp;
            do {
                ent nd = stk[--sp];
                if (nd.d > min_dist) continue;
                uint32_t obj = s->nodes[4 * nd.n + 3];
                if (obj != ORC_INVALID) {
                    const int32_t *t = s->tris + 3 * (int64_t)obj;
                    float tt, uu, vv;
                    ++n_leaf;
                    if (ray_triangle(o, dir, vload(s->verts, t[0]), vload(s->verts, t[1]), vload(s->verts, t[2]), &tt, &uu, &vv)
                        && tt < max_dist && tt < min_dist) {
                        min_dist = tt; found = 1; bu = uu; bv = vv; nearest = obj;
                    }
                } else {
                    ++n_int;
                    uint32_t L = s->nodes[4 * nd.n + 1], R = s->nodes[4 * nd.n + 2];
                    float Ld = 0.0f, Rd = 0.0f;
                    int Lh = ray_box(o, inv, node_box(s, L), max_dist, &Ld);
                    int Rh = ray_box(o, inv, node_box(s, R), max_dist, &Rd);
                    if (Lh && Rh) {
                        uint32_t closer = L, other = R;
                        if (Rd < Ld) { float t = Ld; Ld = Rd; Rd = t; closer = R; other = L; }
                        stk[sp].n = other; stk[sp].d = Rd; ++sp;
                        stk[sp].n = closer; stk[sp].d = Ld; ++sp;
                    } else if (Lh) { stk[sp].n = L; stk[sp].d = Ld; ++sp; }
                    else if (Rh) { stk[sp].n = R; stk[sp].d = Rd; ++sp; }
                }
                if (sp >= ORC_STACK - 2) { found = 0; nearest = ORC_INVALID; min_dist = NAN; break; }
            } while (sp > 0);
        }
        c->hit[q] = (uint8_t)found;
        c->t[q] = min_dist;
        c->uv[2 * q] = bu; c->uv[2 * q + 1] = bv;
        c->idx[q] = nearest;
        if (c->stats) { c->stats[3 * q] = n_int; c->stats[3 * q + 1] = n_leaf; c->stats[3 * q + 2] = 0; }
    }
}
void orc_query_ray(const orc_scene *s, const float *origins, const float *dirs, const float *tmax, int64_t n,
                   uint8_t *hit, float *t, float *uv, uint32_t *idx, uint32_t *stats, int nthreads) {
    ray_ctx c = {s, origins, dirs, tmax, hit, t, uv, idx, stats};
    orc_parallel(n, nthreads, ray_body, &c);
}

/* intersect_sphere(sphere, aabb) aabb.cuh:433-449 */
static int sphere_box(f3 c, float r, box3 b) {
    float cx = smax(b.lower.x, smin(c.x, b.upper.x));
    float cy = smax(b.lower.y, smin(c.y, b.upper.y));
    float dx = cx - c.x, dy = cy - c.y;
    float d2 = dx * dx + dy * dy;
    float cz = smax(b.lower.z, smin(c.z, b.upper.z));
    float dz = cz - c.z;
    d2 += dz * dz;
    return d2 <= (r * r);
}

/* scene<3>::intersect_sphere scene.cuh:1054-1117 */
static int sphere_triangle(f3 c, float radius, f3 p1, f3 p2, f3 p3) {
    f3 e1 = sub(p2, p1), e2 = sub(p3, p1);
    f3 n = mk(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x);
    float nl = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    n = mk(n.x / nl, n.y / nl, n.z / nl);
    float d = n.x * p1.x + n.y * p1.y + n.z * p1.z;
    float dp = n.x * c.x + n.y * c.y + n.z * c.z - d;
    f3 proj = mk(c.x - dp * n.x, c.y - dp * n.y, c.z - dp * n.z);
    f3 v0 = sub(p3, p1), v1 = sub(p2, p1), v2 = sub(proj, p1);
    float d00 = v0.x * v0.x + v0.y * v0.y + v0.z * v0.z;
    float d01 = v0.x * v1.x + v0.y * v1.y + v0.z * v1.z;
    float d02 = v0.x * v2.x + v0.y * v2.y + v0.z * v2.z;
    float d11 = v1.x * v1.x + v1.y * v1.y + v1.z * v1.z;
    float d12 = v1.x * v2.x + v1.y * v2.y + v1.z * v2.z;
    float inv = 1.0f / (d00 * d11 - d01 * d01);
    float u = (d11 * d02 - d01 * d12) * inv;
    float v = (d00 * d12 - d01 * d02) * inv;
    if (u >= 0 && v >= 0 && u + v <= 1) return fabsf(dp) <= radius;
    f3 cp = proj;
    if (u < 0) cp = p1;
    else if (v < 0) cp = p3;
    else if (u + v > 1) cp = p2;
    float dx = cp.x - c.x, dy = cp.y - c.y, dz = cp.z - c.z;
    float d2 = dx * dx + dy * dy + dz * dz;
    return d2 <= (radius * radius);
}

/* green_weight scene.cuh:1119-1126: 1 / (M_PIf * 4 * max(|x - y|, 1e-4)) */
static inline float green_weight(f3 x, f3 y) {
    float r = smax(len3(mk(x.x - y.x, x.y - y.y, x.z - y.z)), 1e-4f);
    const float four_pi = 3.14159265358979323846f * 4.0f;
    return 1.0f / (four_pi * r);
}

/* measurement_getter scene.cuh:855-868 */
static inline float tri_area(const orc_scene *s, uint32_t obj) {
    const int32_t *t = s->tris + 3 * (int64_t)obj;
    f3 pa = vload(s->verts, t[0]), pb = vload(s->verts, t[1]), pc = vload(s->verts, t[2]);
    return len3(cross3(sub(pc, pa), sub(pb, pa))) / 2;
}

/* sample_object_in_sphere sample.cuh:23-91; pdf is 0 where the reference leaves it unset */
typedef struct { const orc_scene *s; const float *c, *r, *u; int32_t *idx; float *pdf; uint32_t *stats; } smp_ctx;
static void smp_body(void *vc, int64_t b, int64_t e) {
    smp_ctx *c = (smp_ctx *)vc;
    const orc_scene *s = c->s;
    for (int64_t q = b; q < e; ++q) {
        f3 ctr = mk(c->c[3 * q], c->c[3 * q + 1], c->c[3 * q + 2]);
        float rad = c->r[q];
        float u = c->u[q];
        int32_t oi = -1;
        float opdf = 0.0f;
        uint32_t n_int = 0, n_leaf = 0;
        if (s->num_tris > 0) {
            uint32_t node = 0;
            float npdf = 1.0f;
            int have = 1;
            while (have) {
                have = 0;
                uint32_t obj = s->nodes[4 * node + 3];
                if (obj != ORC_INVALID) {
                    const int32_t *t = s->tris + 3 * (int64_t)obj;
                    ++n_leaf;
                    if (sphere_triangle(ctr, rad, vload(s->verts, t[0]), vload(s->verts, t[1]), vload(s->verts, t[2]))) {
                        oi = (int32_t)obj;
                        opdf = npdf;
                        opdf /= tri_area(s, obj);
                    }
                } else {
                    ++n_int;
                    uint32_t L = s->nodes[4 * node + 1], R = s->nodes[4 * node + 2];
                    box3 lb = node_box(s, L), rb = node_box(s, R);
                    float Lw = sphere_box(ctr, rad, lb) ? green_weight(ctr, centroid(lb)) : 0;
                    float Rw = sphere_box(ctr, rad, rb) ? green_weight(ctr, centroid(rb)) : 0;
                    float tw = Lw + Rw;
                    if (tw > 0) {
                        float Lp = Lw / tw;
                        if (u < Lp) { u /= Lp; node = L; npdf = Lp * npdf; }
                        else { float Rp = 1.0f - Lp; u = (u - Lp) / Rp; node = R; npdf = Rp * npdf; }
                        have = 1;
                    }
                }
            }
        }
        c->idx[q] = oi;
        c->pdf[q] = opdf;
        if (c->stats) { c->stats[3 * q] = n_int; c->stats[3 * q + 1] = n_leaf; c->stats[3 * q + 2] = 0; }
    }
}
void orc_sample_in_sphere(const orc_scene *s, const float *centers, const float *radii, const float *u, int64_t n,
                          int32_t *idx, float *pdf, uint32_t *stats, int nthreads) {
    smp_ctx c = {s, centers, radii, u, idx, pdf, stats};
    orc_parallel(n, nthreads, smp_body, &c);
}

/* sample_triangle scene.cuh:14-27 */
void orc_sample_on_object(const orc_scene *s, const int32_t *idx, const float *u, const float *v, int64_t n, float *pts) {
    for (int64_t q = 0; q < n; ++q) {
        const int32_t *t = s->tris + 3 * (int64_t)idx[q];
        f3 pa = vload(s->verts, t[0]), pb = vload(s->verts, t[1]), pc = vload(s->verts, t[2]);
        float uu = u[q], vv = v[q];
        if (uu + vv > 1.0f) { uu = 1.0f - uu; vv = 1.0f - vv; }
        float w = 1.0f - uu - vv;
        pts[3 * q] = w * pa.x + uu * pb.x + vv * pc.x;
        pts[3 * q + 1] = w * pa.y + uu * pb.y + vv * pc.y;
        pts[3 * q + 2] = w * pa.z + uu * pb.z + vv * pc.z;
    }
}

/* ----------------------------------------------------------- FP64 brute force */
static inline d3 dk(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static inline d3 dsub(d3 a, d3 b) { return dk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double dlen(d3 a) { return sqrt(ddot(a, a)); }
static inline d3 dcross(d3 u, d3 v) { return dk(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x); }
static inline d3 dnorm(d3 v) { double n = dlen(v); return dk(v.x / n, v.y / n, v.z / n); }
static inline d3 dload(const float *v, int32_t i) { return dk(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }

static double closest_point_triangle_d(d3 pa, d3 pb, d3 pc, d3 x) {
    d3 ab = dsub(pb, pa), ac = dsub(pc, pa), ax = dsub(x, pa);
    double d1 = ddot(ab, ax), d2 = ddot(ac, ax);
    if (d1 <= 0 && d2 <= 0) return dlen(dsub(x, pa));
    d3 bx = dsub(x, pb);
    double d3v = ddot(ab, bx), d4 = ddot(ac, bx);
    if (d3v >= 0 && d4 <= d3v) return dlen(dsub(x, pb));
    d3 cx = dsub(x, pc);
    double d5 = ddot(ab, cx), d6 = ddot(ac, cx);
    if (d6 >= 0 && d5 <= d6) return dlen(dsub(x, pc));
    double vc = d1 * d4 - d3v * d2;
    if (vc <= 0 && d1 >= 0 && d3v <= 0) {
        double v = d1 / (d1 - d3v);
        return dlen(dsub(x, dk(pa.x + ab.x * v, pa.y + ab.y * v, pa.z + ab.z * v)));
    }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
        double w = d2 / (d2 - d6);
        return dlen(dsub(x, dk(pa.x + ac.x * w, pa.y + ac.y * w, pa.z + ac.z * w)));
    }
    double va = d3v * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3v) >= 0 && (d5 - d6) >= 0) {
        double w = (d4 - d3v) / ((d4 - d3v) + (d5 - d6));
        return dlen(dsub(x, dk(pb.x + (pc.x - pb.x) * w, pb.y + (pc.y - pb.y) * w, pb.z + (pc.z - pb.z) * w)));
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom, w = vc * denom;
    return dlen(dsub(x, dk(pa.x + ab.x * v + ac.x * w, pa.y + ab.y * v + ac.y * w, pa.z + ab.z * v + ac.z * w)));
}

typedef struct { const float *verts; const int32_t *prim; int64_t np; const float *pts; const uint8_t *flip;
                 const float *dirs, *tmax; uint32_t *idx; double *dist; uint8_t *hit; } brute_ctx;
static void brute_near_body(void *vc, int64_t b, int64_t e) {
    brute_ctx *c = (brute_ctx *)vc;
    for (int64_t q = b; q < e; ++q) {
        d3 x = dk(c->pts[3 * q], c->pts[3 * q + 1], c->pts[3 * q + 2]);
        double best = INFINITY; uint32_t bi = ORC_INVALID;
        for (int64_t i = 0; i < c->np; ++i) {
            const int32_t *t = c->prim + 3 * i;
            double d = closest_point_triangle_d(dload(c->verts, t[0]), dload(c->verts, t[1]), dload(c->verts, t[2]), x);
            if (d < best) { best = d; bi = (uint32_t)i; }
        }
        c->idx[q] = bi; c->dist[q] = best;
    }
}
void orc_brute_nearest_f64(const float *verts, const int32_t *tris, int64_t nt, const float *pts, int64_t n,
                           uint32_t *idx, double *dist, int nthreads) {
    brute_ctx c = {verts, tris, nt, pts, NULL, NULL, NULL, idx, dist, NULL};
    orc_parallel(n, nthreads, brute_near_body, &c);
}

static d3 edge_face_normal_d(const float *verts, const int32_t *se, int f) {
    int i, j, k;
    if (f == 0) { i = 3; j = 1; k = 2; } else { i = 0; j = 2; k = 1; }
    d3 pa = dload(verts, se[j]), pb = dload(verts, se[k]), pc = dload(verts, se[i]);
    return dnorm(dcross(dsub(pb, pa), dsub(pc, pa)));
}
static void brute_sil_body(void *vc, int64_t b, int64_t e) {
    brute_ctx *c = (brute_ctx *)vc;
    const double precision = 1e-3;
    for (int64_t q = b; q < e; ++q) {
        d3 x = dk(c->pts[3 * q], c->pts[3 * q + 1], c->pts[3 * q + 2]);
        double sign = (c->flip && c->flip[q]) ? 1.0 : -1.0;
        double best = INFINITY;
        for (int64_t i = 0; i < c->np; ++i) {
            const int32_t *se = c->prim + 4 * i;
            d3 pa = dload(c->verts, se[1]), pb = dload(c->verts, se[2]);
            d3 u = dsub(pb, pa), v = dsub(x, pa), cp;
            double c1 = ddot(u, v), c2 = ddot(u, u);
            if (c1 <= 0) cp = pa;
            else if (c2 <= c1) cp = pb;
            else { double t = c1 / c2; cp = dk(pa.x + u.x * t, pa.y + u.y * t, pa.z + u.z * t); }
            double d = dlen(dsub(x, cp));
            if (d >= best) continue;
            int is_sil = se[3] == -1 || se[0] == -1;
            if (!is_sil) {
                d3 n0 = edge_face_normal_d(c->verts, se, 0), n1 = edge_face_normal_d(c->verts, se, 1);
                if (d <= precision) {
                    d3 ed = dnorm(dsub(pb, pa));
                    is_sil = sign * atan2(ddot(ed, dcross(n0, n1)), ddot(n0, n1)) > precision;
                } else {
                    d3 vd = dsub(x, cp);
                    double dot0 = ddot(vd, n0), dot1 = ddot(vd, n1);
                    if (fabs(dot0) <= precision) is_sil = sign * dot1 > precision;
                    else if (fabs(dot1) <= precision) is_sil = sign * dot0 > precision;
                    else is_sil = dot0 * dot1 < 0;
                }
            }
            if (is_sil) best = d;
        }
        c->dist[q] = best;
    }
}
void orc_brute_silhouette_f64(const float *verts, const int32_t *edge_verts, int64_t ne, const float *pts,
                              const uint8_t *flip, int64_t n, double *dist, int nthreads) {
    brute_ctx c = {verts, edge_verts, ne, pts, flip, NULL, NULL, NULL, dist, NULL};
    orc_parallel(n, nthreads, brute_sil_body, &c);
}

static void brute_ray_body(void *vc, int64_t b, int64_t e) {
    brute_ctx *c = (brute_ctx *)vc;
    for (int64_t q = b; q < e; ++q) {
        d3 o = dk(c->pts[3 * q], c->pts[3 * q + 1], c->pts[3 * q + 2]);
        d3 dir = dk(c->dirs[3 * q], c->dirs[3 * q + 1], c->dirs[3 * q + 2]);
        double tmax = c->tmax[q], best = INFINITY;
        uint32_t bi = ORC_INVALID;
        for (int64_t i = 0; i < c->np; ++i) {
            const int32_t *t = c->prim + 3 * i;
            d3 v0 = dload(c->verts, t[0]), v1 = dload(c->verts, t[1]), v2 = dload(c->verts, t[2]);
            d3 e1 = dsub(v1, v0), e2 = dsub(v2, v0), h = dcross(dir, e2);
            double det = ddot(e1, h);
            if (fabs(det) < (double)ORC_EPS) continue;
            double inv = 1.0 / det;
            d3 s = dsub(o, v0);
            double u = ddot(s, h) * inv;
            if (u < 0 || u > 1) continue;
            d3 qv = dcross(s, e1);
            double v = ddot(dir, qv) * inv;
            if (v < 0 || u + v > 1) continue;
            double tt = ddot(e2, qv) * inv;
            if (tt >= 0 && tt < tmax && tt < best) { best = tt; bi = (uint32_t)i; }
        }
        c->hit[q] = bi != ORC_INVALID; c->dist[q] = best; c->idx[q] = bi;
    }
}
void orc_brute_ray_f64(const float *verts, const int32_t *tris, int64_t nt, const float *origins, const float *dirs,
                       const float *tmax, int64_t n, uint8_t *hit, double *t, uint32_t *idx, int nthreads) {
    brute_ctx c = {verts, tris, nt, origins, NULL, dirs, tmax, idx, t, hit};
    orc_parallel(n, nthreads, brute_ray_body, &c);
}


/* ---------------------------------------------------------------- enumeration queries
 * query_device(overlaps(box)) query.cuh:177-231 and query_device(line_intersect(line),
 * element_test) query.cuh:15-77: the traversal pushes L then R and pops the top, leaf
 * children are reported when their parent is expanded (L before R); results beyond
 * max_out are counted, not written. counts[q] = the total. A one-leaf tree (where the
 * reference reads past its node array) tests its only leaf. */

/* intersects(aabb, aabb) aabb.cuh:66-81 */
static inline int box_overlap(box3 a, box3 b) {
    if (a.upper.x < b.lower.x || b.upper.x < a.lower.x) return 0;
    if (a.upper.y < b.lower.y || b.upper.y < a.lower.y) return 0;
    if (a.upper.z < b.lower.z || b.upper.z < a.lower.z) return 0;
    return 1;
}
/* intersects(line<float,3>, aabb) aabb.cuh:329-348 (fmin / fmax drop NaN) */
static inline int line_box(f3 o, f3 inv, box3 b) {
    float t1 = (b.lower.x - o.x) * inv.x, t2 = (b.upper.x - o.x) * inv.x;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b.lower.y - o.y) * inv.y; t2 = (b.upper.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(t1, t2)); tmax = fminf(tmax, fmaxf(t1, t2));
    t1 = (b.lower.z - o.z) * inv.z; t2 = (b.upper.z - o.z) * inv.z;
    tmin = fmaxf(tmin, fminf(t1, t2)); tmax = fminf(tmax, fmaxf(t1, t2));
    return tmax >= tmin;
}
/* the line's element test: scene<3>::intersect_test's Moller-Trumbore arithmetic
 * (scene.cuh:1005-1052) for a line (any t) */
static int line_triangle(f3 o, f3 dir, f3 v0, f3 v1, f3 v2, float *t) {
    f3 e1 = sub(v1, v0), e2 = sub(v2, v0);
    f3 h = mk(dir.y * e2.z - dir.z * e2.y, dir.z * e2.x - dir.x * e2.z, dir.x * e2.y - dir.y * e2.x);
    float det = e1.x * h.x + e1.y * h.y + e1.z * h.z;
    if (fabsf(det) < ORC_EPS) return 0;
    float inv_det = 1.0f / det;
    f3 sv = sub(o, v0);
    float u = (sv.x * h.x + sv.y * h.y + sv.z * h.z) * inv_det;
    if (u < 0.0f || u > 1.0f) return 0;
    f3 qv = mk(sv.y * e1.z - sv.z * e1.y, sv.z * e1.x - sv.x * e1.z, sv.x * e1.y - sv.y * e1.x);
    float v = (dir.x * qv.x + dir.y * qv.y + dir.z * qv.z) * inv_det;
    if (v < 0.0f || u + v > 1.0f) return 0;
    *t = (e2.x * qv.x + e2.y * qv.y + e2.z * qv.z) * inv_det;
    return 1;
}

typedef struct {
    const orc_scene *s; const float *q0; const float *q1; int64_t max_out;
    uint32_t *idx; float *t; uint32_t *count; int line;
} enum_ctx;
static void enum_leaf(enum_ctx *c, uint32_t obj, f3 o, f3 dir, int64_t q, uint32_t *found) {
    float t = 0.0f;
    if (c->line) {
        const int32_t *tr = c->s->tris + 3 * (int64_t)obj;
        if (!line_triangle(o, dir, vload(c->s->verts, tr[0]), vload(c->s->verts, tr[1]), vload(c->s->verts, tr[2]), &t))
            return;
    }
    if (*found < c->max_out) {
        c->idx[q * c->max_out + *found] = obj;
        if (c->line) c->t[q * c->max_out + *found] = t;
    }
    ++*found;
}
static void enum_body(void *vc, int64_t b, int64_t e) {
    enum_ctx *c = (enum_ctx *)vc;
    const orc_scene *s = c->s;
    const uint32_t N = (uint32_t)s->num_tris;
    uint32_t stk[ORC_STACK];
    for (int64_t q = b; q < e; ++q) {
        box3 qb = {{0, 0, 0}, {0, 0, 0}};
        f3 o = mk(0, 0, 0), dir = mk(0, 0, 0), inv = mk(0, 0, 0);
        if (c->line) {
            o = vload(c->q0, (int32_t)q); dir = vload(c->q1, (int32_t)q);
            inv = mk(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
        } else {
            const float *x = c->q0 + 6 * q;
            qb.lower = mk(x[0], x[1], x[2]); qb.upper = mk(x[3], x[4], x[5]);
        }
        uint32_t found = 0;
        if (N == 1) {
            box3 lb = node_box(s, 0);
            if (c->line ? line_box(o, inv, lb) : box_overlap(qb, lb)) enum_leaf(c, s->nodes[3], o, dir, q, &found);
        } else if (N > 1) {
            int sp = 0;
            stk[sp++] = 0;
            do {
                uint32_t node = stk[--sp];
                uint32_t ch[2] = {s->nodes[4 * (int64_t)node + 1], s->nodes[4 * (int64_t)node + 2]};
                for (int k = 0; k < 2; ++k) {
                    box3 cb = node_box(s, ch[k]);
                    if (!(c->line ? line_box(o, inv, cb) : box_overlap(qb, cb))) continue;
                    uint32_t obj = s->nodes[4 * (int64_t)ch[k] + 3];
                    if (obj != 0xFFFFFFFFu) enum_leaf(c, obj, o, dir, q, &found);
                    else if (sp < ORC_STACK) stk[sp++] = ch[k];
                }
            } while (sp > 0);
        }
        c->count[q] = found;
    }
}
void orc_query_overlap(const orc_scene *s, const float *boxes, int64_t n, int64_t max_out, uint32_t *idx,
                       uint32_t *count, int nthreads) {
    enum_ctx c = {s, boxes, NULL, max_out, idx, NULL, count, 0};
    orc_parallel(n, nthreads, enum_body, &c);
}
void orc_query_line(const orc_scene *s, const float *origins, const float *dirs, int64_t n, int64_t max_out,
                    uint32_t *idx, float *t, uint32_t *count, int nthreads) {
    enum_ctx c = {s, origins, dirs, max_out, idx, t, count, 1};
    orc_parallel(n, nthreads, enum_body, &c);
}

/* ================================================================ 2D scenes
 * scene<2> (scene.cuh:287-703): line segments with silhouette VERTICES, the
 * same LBVH build in 2D (bvh.cuh with aabb<float,2>, cone<float,2>) and the
 * same four query templates (query.cuh, sample.cuh) over the 2D functors. */
typedef struct { float x, y; } f2;
typedef struct { f2 upper, lower; } box2;                    /* aabb<float,2>, upper first */
typedef struct { f2 axis; float half_angle, radius; } cone2; /* cone<float,2> */
#define ORC_BVH_OFFSET 1e-3f                                  /* bvh_offset scene.cuh:12 */

static inline f2 mk2(float x, float y) { f2 r = {x, y}; return r; }
static inline f2 sub2(f2 a, f2 b) { return mk2(a.x - b.x, a.y - b.y); }
static inline float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
static inline float len2(f2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
static inline f2 norm2(f2 v) { float n = len2(v); return mk2(v.x / n, v.y / n); }
static inline f2 vload2(const float *v, int32_t i) { return mk2(v[2 * i], v[2 * i + 1]); }
static inline f2 centroid2(box2 b) { return mk2((b.upper.x + b.lower.x) * 0.5f, (b.upper.y + b.lower.y) * 0.5f); }

/* compute_silhouettes scene.cuh:642-664: one silhouette vertex per mesh vertex,
 * {prev, self, next, -1}, later segments overwriting earlier ones; build_bvh
 * scene.cuh:666-683: a segment owns the endpoints no earlier segment touched,
 * in (x, y) order. sv: V x 4, seg_owned: N x 2 (-1 padded). */
void orc2_topology(const int32_t *segs, int64_t n, int64_t nv, int32_t *sv, int32_t *seg_owned) {
    for (int64_t v = 0; v < 4 * nv; ++v) sv[v] = -1;
    for (int64_t i = 0; i < n; ++i) {
        int32_t a = segs[2 * i], b = segs[2 * i + 1];
        sv[4 * a + 1] = a; sv[4 * a + 2] = b;
        sv[4 * b + 0] = a; sv[4 * b + 1] = b;
    }
    uint8_t *seen = (uint8_t *)calloc((size_t)(nv > 0 ? nv : 1), 1);
    for (int64_t i = 0; i < n; ++i) {
        int32_t own[2] = {-1, -1};
        int k = 0;
        for (int j = 0; j < 2; ++j) {
            int32_t v = segs[2 * i + j];
            if (!seen[v]) { seen[v] = 1; own[k++] = v; }
        }
        seg_owned[2 * i] = own[0];
        seg_owned[2 * i + 1] = own[1];
    }
    free(seen);
}

/* silhouette_vertex scene.cuh:291-384 */
static inline int sv_has_face(const int32_t *sv, int f) { return f == 0 ? sv[2] != -1 : sv[0] != -1; }
static f2 sv_face_normal(const float *verts, const int32_t *sv, int f, int do_normalize) {
    int i = f == 0 ? 1 : 0;
    f2 pa = vload2(verts, sv[i]), pb = vload2(verts, sv[i + 1]);
    f2 s = sub2(pb, pa);
    f2 nn = mk2(s.y, -s.x);
    return do_normalize ? norm2(nn) : nn;
}
static f2 sv_normal(const float *verts, const int32_t *sv) {
    f2 nn = mk2(0.0f, 0.0f);
    if (sv_has_face(sv, 0)) { f2 a = sv_face_normal(verts, sv, 0, 0); nn = mk2(nn.x + a.x, nn.y + a.y); }
    if (sv_has_face(sv, 1)) { f2 a = sv_face_normal(verts, sv, 1, 0); nn = mk2(nn.x + a.x, nn.y + a.y); }
    return norm2(nn);
}

/* aabb_getter scene.cuh:420-432 */
static box2 seg_box(const float *verts, const int32_t *s) {
    f2 p0 = vload2(verts, s[0]), p1 = vload2(verts, s[1]);
    box2 b;
    b.upper = mk2(fmaxf(p0.x, p1.x) + ORC_BVH_OFFSET, fmaxf(p0.y, p1.y) + ORC_BVH_OFFSET);
    b.lower = mk2(fminf(p0.x, p1.x) - ORC_BVH_OFFSET, fminf(p0.y, p1.y) - ORC_BVH_OFFSET);
    return b;
}
/* cone_getter scene.cuh:434-494 */
static cone2 seg_cone(const float *verts, const int32_t *s, const int32_t *owned, const int32_t *svs) {
    box2 bb = seg_box(verts, s);
    f2 bc = centroid2(bb);
    cone2 r;
    r.axis = mk2(0.0f, 0.0f); r.half_angle = ORC_PI; r.radius = 0.0f;
    int any = 0, all_two = 1;
    for (int i = 0; i < 2; ++i) {
        int32_t si = owned[i];
        if (si == -1) continue;
        const int32_t *sv = svs + 4 * (int64_t)si;
        f2 nn = sv_normal(verts, sv);
        r.axis.x += nn.x; r.axis.y += nn.y;
        f2 c = vload2(verts, sv[1]);
        r.radius = smax(r.radius, len2(mk2(c.x - bc.x, c.y - bc.y)));
        all_two = all_two && sv_has_face(sv, 0) && sv_has_face(sv, 1);
        any = 1;
    }
    if (!any) r.half_angle = -ORC_PI;
    else if (!all_two) r.half_angle = ORC_PI;
    else {
        float an = len2(r.axis);
        if (an > ORC_EPS) {
            r.axis.x /= an; r.axis.y /= an;
            r.half_angle = 0.0f;
            for (int i = 0; i < 2; ++i) {
                int32_t si = owned[i];
                if (si == -1) continue;
                const int32_t *sv = svs + 4 * (int64_t)si;
                f2 fn[2];
                fn[0] = sv_has_face(sv, 0) ? sv_face_normal(verts, sv, 0, 1) : mk2(0.0f, 0.0f);
                fn[1] = sv_has_face(sv, 1) ? sv_face_normal(verts, sv, 1, 1) : mk2(0.0f, 0.0f);
                for (int j = 0; j < 2; ++j) {
                    float ang = acosf(smax(-1.0f, smin(1.0f, dot2(r.axis, fn[j]))));
                    r.half_angle = smax(r.half_angle, ang);
                }
            }
        }
    }
    return r;
}
void orc2_leaf_boxes(const float *verts, const int32_t *segs, int64_t n, float *out) {
    for (int64_t i = 0; i < n; ++i) { box2 b = seg_box(verts, segs + 2 * i); memcpy(out + 4 * i, &b, sizeof b); }
}

/* morton_code(float2) morton_code.cuh:83-91 (the 3D bit spreading, x * 2 + y) */
static uint32_t morton2(f2 p) {
    const float res = 1024.0f;
    p.x = fminf(fmaxf(p.x * res, 0.0f), res - 1.0f);
    p.y = fminf(fmaxf(p.y * res, 0.0f), res - 1.0f);
    return expand_bits((uint32_t)p.x) * 2 + expand_bits((uint32_t)p.y);
}

/* rotate(float2) cone.cuh:266-275 */
static f2 rotate2(f2 u, f2 v, float theta) {
    float det = u.x * v.y - u.y * v.x;
    theta *= copysignf(1.0f, det);
    float ct = cosf(theta), st = sinf(theta);
    return mk2(ct * u.x - st * u.y, st * u.x + ct * u.y);
}
/* merge(cone<float,2>) cone.cuh:320-371; pi where the reference leaves the
 * half angle unassigned (o_theta >= pi, lines 347-351) */
static cone2 cone_merge2(cone2 a, cone2 b, f2 oa, f2 ob, f2 on, int *d1) {
    cone2 r;
    r.axis = mk2(0.0f, 0.0f); r.half_angle = 0.0f; r.radius = 0.0f;
    int va = a.half_angle >= 0.0f, vb = b.half_angle >= 0.0f;
    if (va && vb) {
        f2 axis_a = a.axis, axis_b = b.axis;
        float ha = a.half_angle, hb = b.half_angle;
        f2 da = sub2(on, oa), db = sub2(on, ob);
        r.radius = sqrtf(smax(a.radius * a.radius + (da.x * da.x + da.y * da.y),
                              b.radius * b.radius + (db.x * db.x + db.y * db.y)));
        if (hb > ha) { f2 t = axis_a; axis_a = axis_b; axis_b = t; float h = ha; ha = hb; hb = h; }
        float theta = acosf(smax(-1.0f, smin(1.0f, dot2(axis_a, axis_b))));
        if (smin(theta + hb, ORC_PI) <= ha) { r.axis = axis_a; r.half_angle = ha; return r; }
        float o_theta = (ha + theta + hb) / 2.0f;
        if (o_theta >= ORC_PI) { r.axis = axis_a; r.half_angle = ORC_PI; *d1 = 1; return r; }
        float r_theta = o_theta - ha;
        r.axis = rotate2(axis_a, axis_b, r_theta);
        r.half_angle = o_theta;
    } else if (va) {
        r = a;
    } else if (vb) {
        r = b;
    } else {
        r.half_angle = -ORC_PI;
    }
    return r;
}

int orc2_build(const float *verts, const int32_t *segs, int64_t nseg, const int32_t *seg_owned, const int32_t *svs,
               uint32_t *morton, uint32_t *sorted_idx, uint32_t *nodes, float *aabbs, float *cones,
               uint8_t *d1_flags) {
    if (nseg <= 0) return 1;
    const unsigned N = (unsigned)nseg, NI = N - 1, NN = 2 * N - 1;
    box2 *bx = (box2 *)aabbs;
    cone2 *cn = (cone2 *)cones;
    box2 *lb_ = (box2 *)malloc(sizeof(box2) * N);
    cone2 *lc_ = (cone2 *)malloc(sizeof(cone2) * N);
    box2 whole;
    whole.upper = mk2(-INFINITY, -INFINITY);
    whole.lower = mk2(INFINITY, INFINITY);
    for (unsigned i = 0; i < N; ++i) {
        lb_[i] = seg_box(verts, segs + 2 * (int64_t)i);
        lc_[i] = seg_cone(verts, segs + 2 * (int64_t)i, seg_owned + 2 * (int64_t)i, svs);
        whole.upper = mk2(fmaxf(whole.upper.x, lb_[i].upper.x), fmaxf(whole.upper.y, lb_[i].upper.y));
        whole.lower = mk2(fminf(whole.lower.x, lb_[i].lower.x), fminf(whole.lower.y, lb_[i].lower.y));
    }
    /* default_morton_code_calculator<Real,2> bvh.cuh:257-279 */
    for (unsigned i = 0; i < N; ++i) {
        f2 p = centroid2(lb_[i]);
        p.x -= whole.lower.x; p.y -= whole.lower.y;
        p.x /= (whole.upper.x - whole.lower.x);
        p.y /= (whole.upper.y - whole.lower.y);
        morton[i] = morton2(p);
    }
    uint64_t *ck = (uint64_t *)malloc(sizeof(uint64_t) * N);
    for (unsigned i = 0; i < N; ++i) ck[i] = ((uint64_t)morton[i] << 32) | i;
    qsort(ck, N, sizeof(uint64_t), u64_cmp);
    int unique = 1;
    for (unsigned i = 0; i < N; ++i) {
        sorted_idx[i] = (uint32_t)(ck[i] & 0xFFFFFFFFu);
        if (i > 0 && (ck[i] >> 32) == (ck[i - 1] >> 32)) unique = 0;
    }
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * N);
    for (unsigned i = 0; i < N; ++i) keys[i] = unique ? (ck[i] >> 32) : ck[i];
    keyset ks = {keys, !unique};
    for (unsigned i = 0; i < NN; ++i) {
        nodes[4 * i] = nodes[4 * i + 1] = nodes[4 * i + 2] = nodes[4 * i + 3] = ORC_INVALID;
        bx[i].upper = mk2(-INFINITY, -INFINITY);
        bx[i].lower = mk2(INFINITY, INFINITY);
        cn[i].axis = mk2(0.0f, 0.0f); cn[i].half_angle = ORC_PI; cn[i].radius = 0.0f;
        if (d1_flags) d1_flags[i] = 0;
    }
    for (unsigned j = 0; j < N; ++j) {
        nodes[4 * (NI + j) + 3] = sorted_idx[j];
        bx[NI + j] = lb_[sorted_idx[j]];
        cn[NI + j] = lc_[sorted_idx[j]];
    }
    for (unsigned idx = 0; idx < NI; ++idx) {
        unsigned lo, hi;
        determine_range(&ks, N, idx, &lo, &hi);
        int gamma = (int)find_split(&ks, lo, hi);
        uint32_t left = (uint32_t)gamma, right = (uint32_t)gamma + 1;
        if ((lo < hi ? lo : hi) == (unsigned)gamma) left += NI;
        if ((lo > hi ? lo : hi) == (unsigned)gamma + 1) right += NI;
        nodes[4 * idx + 1] = left;
        nodes[4 * idx + 2] = right;
        nodes[4 * idx + 3] = ORC_INVALID;
        nodes[4 * left] = idx;
        nodes[4 * right] = idx;
    }
    if (NI > 0) {
        uint32_t *stk = (uint32_t *)malloc(sizeof(uint32_t) * 2 * NN);
        uint8_t *expanded = (uint8_t *)calloc(NN, 1);
        int64_t sp = 0;
        stk[sp++] = 0;
        while (sp > 0) {
            uint32_t p = stk[sp - 1];
            uint32_t L = nodes[4 * p + 1], R = nodes[4 * p + 2];
            if (!expanded[p]) {
                expanded[p] = 1;
                if (R < NI) stk[sp++] = R;
                if (L < NI) stk[sp++] = L;
                continue;
            }
            --sp;
            box2 lb = bx[L], rb = bx[R], m;
            m.upper = mk2(fmaxf(lb.upper.x, rb.upper.x), fmaxf(lb.upper.y, rb.upper.y));
            m.lower = mk2(fminf(lb.lower.x, rb.lower.x), fminf(lb.lower.y, rb.lower.y));
            bx[p] = m;
            int d1 = 0;
            cn[p] = cone_merge2(cn[L], cn[R], centroid2(lb), centroid2(rb), centroid2(m), &d1);
            if (d1_flags) d1_flags[p] = (uint8_t)d1;
        }
        free(stk); free(expanded);
    }
    free(keys); free(ck); free(lb_); free(lc_);
    return unique;
}

/* ---------------- 2D query math */
static inline float mindist2(box2 b, f2 p) {  /* aabb.cuh:130-135 */
    const float dx = fminf(b.upper.x, fmaxf(b.lower.x, p.x)) - p.x;
    const float dy = fminf(b.upper.y, fmaxf(b.lower.y, p.y)) - p.y;
    return dx * dx + dy * dy;
}
static inline float minmaxdist2(box2 b, f2 p) {  /* aabb.cuh:161-180 */
    float rmx = (b.lower.x - p.x) * (b.lower.x - p.x), rmy = (b.lower.y - p.y) * (b.lower.y - p.y);
    float rMx = (b.upper.x - p.x) * (b.upper.x - p.x), rMy = (b.upper.y - p.y) * (b.upper.y - p.y);
    float t;
    if ((b.upper.x + b.lower.x) * 0.5f < p.x) { t = rmx; rmx = rMx; rMx = t; }
    if ((b.upper.y + b.lower.y) * 0.5f < p.y) { t = rmy; rmy = rMy; rMy = t; }
    const float dx = rmx + rMy, dy = rMx + rmy;
    return fminf(dx, dy);
}
/* find_closest_point_line_segment(float2) scene.cuh:176-199 */
static float closest_point_segment2(f2 pa, f2 pb, f2 x) {
    f2 u = sub2(pb, pa), v = sub2(x, pa);
    float c1 = dot2(u, v);
    if (c1 <= 0.0f) return len2(sub2(x, pa));
    float c2 = dot2(u, u);
    if (c2 <= c1) return len2(sub2(x, pb));
    float t = c1 / c2;
    f2 pt = mk2(pa.x + u.x * t, pa.y + u.y * t);
    return len2(mk2(x.x - pt.x, x.y - pt.y));
}
/* is_silhouette_vertex scene.cuh:112-141 */
static int is_silhouette_vertex(f2 n0, f2 n1, f2 view_dir, float d, int flip) {
    const float precision = 1e-3f;
    float sign = flip ? 1.0f : -1.0f;
    if (d <= precision) {
        float det = n0.x * n1.y - n0.y * n1.x;
        return sign * det > precision;
    }
    f2 vu = mk2(view_dir.x / d, view_dir.y / d);
    float dot0 = dot2(vu, n0), dot1 = dot2(vu, n1);
    if (fabsf(dot0) <= precision) return sign * dot1 > precision;
    if (fabsf(dot1) <= precision) return sign * dot0 > precision;
    return dot0 * dot1 < 0.0f;
}
/* overlap(cone<float,2>) cone.cuh:78-120 with project_to_plane(float2) 44-49 */
static int cone_overlap2(cone2 bc, f2 o, box2 b, float dist_to_box) {
    if (bc.half_angle >= ORC_PI_2 || dist_to_box < ORC_EPS) return 1;
    f2 c = centroid2(b);
    f2 v = mk2(c.x - o.x, c.y - o.y);
    float l = len2(v);
    v.x /= l; v.y /= l;
    float dax = acosf(smax(-1.0f, smin(1.0f, dot2(bc.axis, v))));
    if (inrange(ORC_PI_2, dax - bc.half_angle, dax + bc.half_angle)) return 1;
    if (l > bc.radius) {
        float vch = asinf(bc.radius / l);
        float hs = bc.half_angle + vch;
        return hs >= ORC_PI_2 ? 1 : inrange(ORC_PI_2, dax - hs, dax + hs);
    }
    f2 e = mk2(b.upper.x - c.x, b.upper.y - c.y);
    float d = dot2(e, mk2(fabsf(v.x), fabsf(v.y)));
    float s = l - d;
    if (s <= 0.0f) return 1;
    f2 bb = mk2(-v.y, v.x);
    d = fabsf(dot2(e, mk2(fabsf(bb.x), fabsf(bb.y))));
    float vch = atan2f(d, s);
    float hs = bc.half_angle + vch;
    return hs >= ORC_PI_2 ? 1 : inrange(ORC_PI_2, dax - hs, dax + hs);
}

typedef struct {
    int64_t num_segs, num_verts;
    const float *verts;        /* V x 2 */
    const int32_t *segs;       /* N x 2 */
    const int32_t *seg_owned;  /* N x 2 owned silhouette vertices, -1 padded */
    const int32_t *sv;         /* V x 4 {prev, self, next, -1} */
    const uint32_t *nodes;     /* (2N-1) x 4 */
    const float *aabbs;        /* (2N-1) x {upper.xy, lower.xy} */
    const float *cones;        /* (2N-1) x {axis.xy, half_angle, radius} */
} orc2_scene;

static inline box2 node_box2(const orc2_scene *s, uint32_t n) { box2 b; memcpy(&b, s->aabbs + 4 * (int64_t)n, sizeof b); return b; }
static inline cone2 node_cone2(const orc2_scene *s, uint32_t n) { cone2 c; memcpy(&c, s->cones + 4 * (int64_t)n, sizeof c); return c; }
static inline float seg_distance(const orc2_scene *s, uint32_t obj, f2 p) {
    const int32_t *g = s->segs + 2 * (int64_t)obj;
    return closest_point_segment2(vload2(s->verts, g[0]), vload2(s->verts, g[1]), p);
}

/* query_device(nearest) query.cuh:239-318 over segments */
void orc2_query_nearest(const orc2_scene *s, const float *pts, int64_t n, uint32_t *idx, float *dist) {
    typedef struct { uint32_t n; float d; } ent;
    ent stk[ORC_STACK];
    for (int64_t q = 0; q < n; ++q) {
        f2 p = mk2(pts[2 * q], pts[2 * q + 1]);
        uint32_t nearest = ORC_INVALID;
        float best = INFINITY;
        if (s->num_segs == 1) {
            float d = seg_distance(s, s->nodes[3], p);
            best = d * d; nearest = s->nodes[3];
        } else if (s->num_segs > 1) {
            int sp = 0;
            stk[sp].n = 0; stk[sp].d = mindist2(node_box2(s, 0), p); ++sp;
            do {
                ent nd = stk[--sp];
                if (nd.d > best) continue;
                uint32_t L = s->nodes[4 * nd.n + 1], R = s->nodes[4 * nd.n + 2];
                box2 lb = node_box2(s, L), rb = node_box2(s, R);
                float Lmd = mindist2(lb, p), Rmd = mindist2(rb, p);
                float Lmm = minmaxdist2(lb, p), Rmm = minmaxdist2(rb, p);
                uint32_t ch[2] = {L, R};
                int ok[2] = {Lmd <= Rmm, Rmd <= Lmm};
                float md[2] = {Lmd, Rmd};
                for (int k = 0; k < 2; ++k) {
                    if (!ok[k]) continue;
                    uint32_t obj = s->nodes[4 * ch[k] + 3];
                    if (obj != ORC_INVALID) {
                        float d = seg_distance(s, obj, p);
                        d *= d;
                        if (d <= best) { best = d; nearest = obj; }
                    } else { stk[sp].n = ch[k]; stk[sp].d = md[k]; ++sp; }
                }
                if (sp >= ORC_STACK - 2) { nearest = ORC_INVALID; best = NAN; break; }
            } while (sp > 0);
        }
        idx[q] = nearest;
        dist[q] = sqrtf(best);
    }
}

/* silhouette_vertex::find_closest_silhouette_point scene.cuh:354-381 */
static int sv_closest(const orc2_scene *s, int32_t si, f2 o, float max_r2, float *dist, int flip) {
    if (0.0f >= max_r2) return 0;
    const int32_t *sv = s->sv + 4 * (int64_t)si;
    f2 p = vload2(s->verts, sv[1]);
    f2 vd = mk2(o.x - p.x, o.y - p.y);
    float d = len2(vd);
    if (d * d > max_r2) return 0;
    int is_sil = !sv_has_face(sv, 0) || !sv_has_face(sv, 1);
    if (!is_sil)
        is_sil = is_silhouette_vertex(sv_face_normal(s->verts, sv, 0, 1), sv_face_normal(s->verts, sv, 1, 1), vd, d, flip);
    if (is_sil && d * d <= max_r2) { *dist = d; return 1; }
    return 0;
}
/* silhouette_distance_calculator scene.cuh:512-532 */
static int leaf_silhouette2(const orc2_scene *s, uint32_t obj, f2 o, float max_r2, float *dist, int flip, int32_t *vid) {
    const int32_t *own = s->seg_owned + 2 * (int64_t)obj;
    float mr2 = max_r2;
    int ret = 0;
    for (int i = 0; i < 2; ++i) {
        if (own[i] == -1) continue;
        if (sv_closest(s, own[i], o, mr2, dist, flip)) { ret = 1; mr2 = *dist * *dist; *vid = own[i]; }
    }
    return ret;
}
/* query_device(nearest_silhouette) query.cuh:326-423 over segments; vid: the
 * silhouette vertex (mesh vertex id) that gave the distance */
void orc2_query_silhouette(const orc2_scene *s, const float *pts, const uint8_t *flip, int64_t n, float *dist,
                           int32_t *vid) {
    typedef struct { uint32_t n; float d; } ent;
    ent stk[ORC_STACK];
    for (int64_t q = 0; q < n; ++q) {
        f2 p = mk2(pts[2 * q], pts[2 * q + 1]);
        int fl = flip ? flip[q] != 0 : 0;
        float best = INFINITY;
        int32_t bv = -1;
        if (s->num_segs == 1) {
            float d = INFINITY; int32_t v = -1;
            if (leaf_silhouette2(s, s->nodes[3], p, best * best, &d, fl, &v) && d <= best) { best = d; bv = v; }
        } else if (s->num_segs > 1) {
            int sp = 0;
            stk[sp].n = 0; stk[sp].d = mindist2(node_box2(s, 0), p); ++sp;
            do {
                ent nd = stk[--sp];
                if (nd.d > best * best) continue;
                uint32_t L = s->nodes[4 * nd.n + 1], R = s->nodes[4 * nd.n + 2];
                box2 lb = node_box2(s, L), rb = node_box2(s, R);
                cone2 lc = node_cone2(s, L), rc = node_cone2(s, R);
                float Lmd = mindist2(lb, p), Rmd = mindist2(rb, p);
                int hit[2] = {lc.half_angle >= 0.0f && cone_overlap2(lc, p, lb, Lmd),
                              rc.half_angle >= 0.0f && cone_overlap2(rc, p, rb, Rmd)};
                uint32_t ch[2] = {L, R};
                float md[2] = {Lmd, Rmd};
                for (int k = 0; k < 2; ++k) {
                    if (!hit[k]) continue;
                    uint32_t obj = s->nodes[4 * ch[k] + 3];
                    if (obj != ORC_INVALID) {
                        float d = INFINITY; int32_t v = -1;
                        if (leaf_silhouette2(s, obj, p, best * best, &d, fl, &v) && d <= best) { best = d; bv = v; }
                    } else { stk[sp].n = ch[k]; stk[sp].d = md[k]; ++sp; }
                }
                if (sp >= ORC_STACK - 2) { best = NAN; bv = -1; break; }
            } while (sp > 0);
        }
        dist[q] = best;
        if (vid) vid[q] = bv;
    }
}

/* intersects_d(ray<float,2>) aabb.cuh:366-390 */
static int ray_box2(f2 o, f2 inv, box2 b, float max_dist, float *dist) {
    float t1 = (b.lower.x - o.x) * inv.x, t2 = (b.upper.x - o.x) * inv.x;
    float tmin = fminf(t1, t2), tmax = fmaxf(t1, t2);
    t1 = (b.lower.y - o.y) * inv.y; t2 = (b.upper.y - o.y) * inv.y;
    tmin = fmaxf(tmin, fminf(t1, t2)); tmax = fminf(tmax, fmaxf(t1, t2));
    if (tmax >= tmin && tmax >= 0.0f && tmin <= max_dist) { *dist = tmin >= 0.0f ? tmin : 0.0f; return 1; }
    return 0;
}
/* scene<2>::intersect_test scene.cuh:555-583: (hit, t, segment parameter s) */
static int ray_segment(f2 o, f2 dir, f2 p0, f2 p1, float *t, float *sp) {
    f2 sd = sub2(p1, p0);
    float D = dir.x * (-sd.y) + dir.y * sd.x;
    if (fabsf(D) < ORC_EPS) return 0;
    float invD = 1.0f / D;
    float tt = ((p0.x - o.x) * (-sd.y) - (p0.y - o.y) * (-sd.x)) * invD;
    float ss = (dir.x * (p0.y - o.y) - dir.y * (p0.x - o.x)) * invD;
    if (ss >= -1e-3f && ss <= 1.0f + 1e-3f && tt >= 0.0f) { *t = tt; *sp = ss; return 1; }
    return 0;
}
/* query_device(ray_intersect) query.cuh:82-169 over segments */
void orc2_query_ray(const orc2_scene *s, const float *origins, const float *dirs, const float *tmax, int64_t n,
                    uint8_t *hit, float *t, float *sparam, uint32_t *idx) {
    typedef struct { uint32_t n; float d; } ent;
    ent stk[ORC_STACK];
    for (int64_t q = 0; q < n; ++q) {
        f2 o = mk2(origins[2 * q], origins[2 * q + 1]);
        f2 dir = mk2(dirs[2 * q], dirs[2 * q + 1]);
        f2 inv = mk2(1 / dir.x, 1 / dir.y);
        float max_dist = tmax[q], min_dist = INFINITY, bs = 0.0f;
        int found = 0;
        uint32_t nearest = ORC_INVALID;
        if (s->num_segs > 0) {
            int sp = 0;
            stk[sp].n = 0; stk[sp].d = INFINITY; ++sp;
            do {
                ent nd = stk[--sp];
                if (nd.d > min_dist) continue;
                uint32_t obj = s->nodes[4 * nd.n + 3];
                if (obj != ORC_INVALID) {
                    const int32_t *g = s->segs + 2 * (int64_t)obj;
                    float tt, ss;
                    if (ray_segment(o, dir, vload2(s->verts, g[0]), vload2(s->verts, g[1]), &tt, &ss) &&
                        tt < max_dist && tt < min_dist) {
                        min_dist = tt; found = 1; bs = ss; nearest = obj;
                    }
                } else {
                    uint32_t L = s->nodes[4 * nd.n + 1], R = s->nodes[4 * nd.n + 2];
                    float Ld = 0.0f, Rd = 0.0f;
                    int Lh = ray_box2(o, inv, node_box2(s, L), max_dist, &Ld);
                    int Rh = ray_box2(o, inv, node_box2(s, R), max_dist, &Rd);
                    if (Lh && Rh) {
                        uint32_t closer = L, other = R;
                        if (Rd < Ld) { float tmp = Ld; Ld = Rd; Rd = tmp; closer = R; other = L; }
                        stk[sp].n = other; stk[sp].d = Rd; ++sp;
                        stk[sp].n = closer; stk[sp].d = Ld; ++sp;
                    } else if (Lh) { stk[sp].n = L; stk[sp].d = Ld; ++sp; }
                    else if (Rh) { stk[sp].n = R; stk[sp].d = Rd; ++sp; }
                }
                if (sp >= ORC_STACK - 2) { found = 0; nearest = ORC_INVALID; min_dist = NAN; break; }
            } while (sp > 0);
        }
        hit[q] = (uint8_t)found;
        t[q] = min_dist;
        sparam[q] = bs;
        idx[q] = nearest;
    }
}

/* intersect_sphere(sphere<float,2>, aabb) aabb.cuh:433-449 */
static int circle_box(f2 c, float r, box2 b) {
    float cx = smax(b.lower.x, smin(c.x, b.upper.x));
    float cy = smax(b.lower.y, smin(c.y, b.upper.y));
    float dx = cx - c.x, dy = cy - c.y;
    return dx * dx + dy * dy <= (r * r);
}
/* scene<2>::intersect_sphere scene.cuh:585-608 */
static int circle_segment(f2 c, float radius, f2 p1, f2 p2) {
    f2 d = sub2(p2, p1);
    float len_sq = d.x * d.x + d.y * d.y;
    float t = ((c.x - p1.x) * d.x + (c.y - p1.y) * d.y) / len_sq;
    t = smax(0.0f, smin(1.0f, t));
    f2 cp = mk2(p1.x + t * d.x, p1.y + t * d.y);
    float dx = cp.x - c.x, dy = cp.y - c.y;
    return dx * dx + dy * dy <= (radius * radius);
}
/* scene<2>::green_weight scene.cuh:610-617: |log(max(|x - y|, 1e-2)) / (2 pi)| */
static inline float green_weight2(f2 x, f2 y) {
    float r = smax(len2(mk2(x.x - y.x, x.y - y.y)), 1e-2f);
    return fabsf(logf(r) / (3.14159265358979323846f * 2.0f));
}
/* sample_object_in_sphere sample.cuh:23-91 over segments (measurement = length) */
void orc2_sample_in_circle(const orc2_scene *s, const float *centers, const float *radii, const float *u_in,
                           int64_t n, int32_t *idx, float *pdf) {
    for (int64_t q = 0; q < n; ++q) {
        f2 ctr = mk2(centers[2 * q], centers[2 * q + 1]);
        float rad = radii[q], u = u_in[q];
        int32_t oi = -1;
        float opdf = 0.0f;
        if (s->num_segs > 0) {
            uint32_t node = 0;
            float npdf = 1.0f;
            int have = 1;
            while (have) {
                have = 0;
                uint32_t obj = s->nodes[4 * node + 3];
                if (obj != ORC_INVALID) {
                    const int32_t *g = s->segs + 2 * (int64_t)obj;
                    f2 p0 = vload2(s->verts, g[0]), p1 = vload2(s->verts, g[1]);
                    if (circle_segment(ctr, rad, p0, p1)) {
                        oi = (int32_t)obj;
                        opdf = npdf;
                        opdf /= len2(mk2(p0.x - p1.x, p0.y - p1.y));
                    }
                } else {
                    uint32_t L = s->nodes[4 * node + 1], R = s->nodes[4 * node + 2];
                    box2 lb = node_box2(s, L), rb = node_box2(s, R);
                    float Lw = circle_box(ctr, rad, lb) ? green_weight2(ctr, centroid2(lb)) : 0;
                    float Rw = circle_box(ctr, rad, rb) ? green_weight2(ctr, centroid2(rb)) : 0;
                    float tw = Lw + Rw;
                    if (tw > 0) {
                        float Lp = Lw / tw;
                        if (u < Lp) { u /= Lp; node = L; npdf = Lp * npdf; }
                        else { float Rp = 1.0f - Lp; u = (u - Lp) / Rp; node = R; npdf = Rp * npdf; }
                        have = 1;
                    }
                }
            }
        }
        idx[q] = oi;
        pdf[q] = opdf;
    }
}
