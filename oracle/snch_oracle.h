/*
 * CPU oracle for the SNCH-LBVH hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP32 restatement of tyanyuy3125/snch-lbvh's LBVH build
 * (include/snch_lbvh/core/bvh.cuh), its 3D scene functors
 * (include/snch_lbvh/scene.cuh) and its per-thread device queries
 * (include/snch_lbvh/core/query.cuh, core/sample.cuh), plus FP64 brute-force
 * references. Only the test-suite, the smoke check and bench.py's CPU-baseline
 * leg load this library; the product path never does.
 *
 * Arithmetic contract: compiled with -ffp-contract=off so every + - * / sqrt is
 * one IEEE-754 binary32 operation in the reference's expression order; the
 * transcendental calls (acosf, asinf, atan2f, sinf, cosf) are libm's.
 * Pinned against the reference's own code (compiled from its headers by
 * oracle/Makefile into oracle/_ref/ref_harness) through tests/golden/.
 */
#ifndef SNCH_ORACLE_H
#define SNCH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flat tree in the reference's layout (bvh.cuh:27-33, aabb.cuh:12-16, cone.cuh:11-16):
 * internal nodes 0..N-2, leaf for sorted position j at N-1+j, root 0.
 *   nodes : (2N-1) x {parent, left, right, object}       (uint32)
 *   aabbs : (2N-1) x {upper.xyz, lower.xyz}              (float, upper first)
 *   cones : (2N-1) x {axis.xyz, half_angle, radius}      (float)
 */
typedef struct {
    int64_t num_tris;          /* N                                              */
    int64_t num_verts;
    int64_t num_edges;         /* E, silhouette edges                            */
    const float *verts;        /* num_verts x 3                                  */
    const int32_t *tris;       /* N x 3 vertex ids                               */
    const int32_t *tri_owned;  /* N x 3 owned edge ids, -1 padded (scene.cuh:1205-1225) */
    const int32_t *edge_verts; /* E x 4 {opp0, min, max, opp1}, -1 = no face    */
    const uint32_t *nodes;
    const float *aabbs;
    const float *cones;
} orc_scene;

/* silhouette topology, scene.cuh:1135-1203 and 1205-1225.
 * tri_edges: N x 3 edge ids, tri_owned: N x 3, edge_verts: capacity 3N x 4.
 * Returns E. */
int64_t orc_topology(const int32_t *tris, int64_t nt, int32_t *tri_edges, int32_t *tri_owned,
                     int32_t *edge_verts);

/* leaf AABB of every triangle (scene.cuh:870-885), N x 6 */
void orc_leaf_aabbs(const float *verts, const int32_t *tris, int64_t nt, float *aabbs_out);

/* leaf cone of every triangle (scene.cuh:887-961), N x 5 */
void orc_leaf_cones(const float *verts, const int32_t *tris, int64_t nt, const int32_t *tri_owned,
                    const int32_t *edge_verts, float *cones_out);

/* full construction, bvh.cuh:380-613.
 * morton: N codes in ORIGINAL triangle order (bvh.cuh:436-439)
 * sorted_idx: N original indices in sorted order (bvh.cuh:445-454)
 * d1_flags: per node, 1 where the reference's cone merge leaves half_angle
 *           undefined (cone.cuh:454-458); this oracle stores pi there.
 * returns 1 if the 30-bit codes were unique, 0 if the 64-bit fallback ran. */
int orc_build(const float *verts, const int32_t *tris, int64_t nt, const int32_t *tri_owned,
              const int32_t *edge_verts, uint32_t *morton, uint32_t *sorted_idx, uint32_t *nodes,
              float *aabbs, float *cones, uint8_t *d1_flags);

/* Per-query statistics (optional, may be NULL): stats[q*3+0] internal nodes
 * expanded, [1] leaves evaluated, [2] silhouette edges evaluated. */

/* query_device(nearest), query.cuh:239-318 -> (index, distance) */
void orc_query_nearest(const orc_scene *s, const float *pts, int64_t n, uint32_t *idx, float *dist,
                       uint32_t *stats, int nthreads);

/* query_device(nearest_silhouette), query.cuh:326-423 -> distance (+ the
 * owning edge id of the last accepted update; the reference tracks none) */
void orc_query_silhouette(const orc_scene *s, const float *pts, const uint8_t *flip, int64_t n,
                          float *dist, int32_t *edge, uint32_t *stats, int nthreads);

/* query_device(ray_intersect<false>), query.cuh:82-169 -> (found, t, uv, index) */
void orc_query_ray(const orc_scene *s, const float *origins, const float *dirs, const float *tmax,
                   int64_t n, uint8_t *hit, float *t, float *uv, uint32_t *idx, uint32_t *stats,
                   int nthreads);

/* sample_object_in_sphere, sample.cuh:26-91 -> (index or -1, pdf; 0 when -1) */
void orc_sample_in_sphere(const orc_scene *s, const float *centers, const float *radii,
                          const float *u, int64_t n, int32_t *idx, float *pdf, uint32_t *stats,
                          int nthreads);

/* sample_on_object + scene<3>::sample_on_object, sample.cuh:10-22, scene.cuh:14-27, 1231-1240 */
void orc_sample_on_object(const orc_scene *s, const int32_t *idx, const float *u, const float *v,
                          int64_t n, float *pts);

/* FP64 brute force over all primitives (same formulas in double). */
void orc_brute_nearest_f64(const float *verts, const int32_t *tris, int64_t nt, const float *pts,
                           int64_t n, uint32_t *idx, double *dist, int nthreads);
void orc_brute_silhouette_f64(const float *verts, const int32_t *edge_verts, int64_t ne,
                              const float *pts, const uint8_t *flip, int64_t n, double *dist,
                              int nthreads);
void orc_brute_ray_f64(const float *verts, const int32_t *tris, int64_t nt, const float *origins,
                       const float *dirs, const float *tmax, int64_t n, uint8_t *hit, double *t,
                       uint32_t *idx, int nthreads);

/* query_device(overlaps(box)) query.cuh:177-231 / query_device(line_intersect(line))
 * query.cuh:15-77 (element test: intersect_test's arithmetic for a line, any t):
 * boxes n x {lower.xyz, upper.xyz}; the first max_out results per query in the
 * reference's order at idx[q * max_out ...] (and t), the total in count[q]. */
void orc_query_overlap(const orc_scene *s, const float *boxes, int64_t n, int64_t max_out, uint32_t *idx,
                       uint32_t *count, int nthreads);
void orc_query_line(const orc_scene *s, const float *origins, const float *dirs, int64_t n, int64_t max_out,
                    uint32_t *idx, float *t, uint32_t *count, int nthreads);
int orc_max_depth(const uint32_t *nodes, int64_t nt);

/* Position of every sorted leaf in the reference's full depth-first order
 * (query.cuh:256-316: leaf children evaluated left then right when a node is
 * expanded; the right child is pushed last and so expanded first). */
void orc_leaf_ranks(const uint32_t *nodes, int64_t nt, uint32_t *ranks);

#ifdef __cplusplus
}
#endif
#endif
