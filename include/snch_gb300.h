/*
 * snch_gb300.h -- C ABI of the GB300-native SNCH-LBVH (libsnch_gb300.so).
 *
 * Drop-in boundary for the LBVH build + query path of tyanyuy3125/snch-lbvh,
 * whose interface is header-only C++ (include/snch_lbvh/scene.cuh,
 * core/bvh.cuh, core/query.cuh, core/sample.cuh). Every entry point below
 * names the reference call it replaces. Conventions:
 *   - plain pointers and sizes; no C++ or CUDA types in the signatures
 *     (a stream is a cudaStream_t passed as void*, NULL = legacy default stream);
 *   - "device" buffers live in GPU memory and are owned by the caller; the
 *     scene owns its tree; "host" buffers are CPU memory (pinned for speed);
 *   - every call returns an snch_status; snch_last_error() describes the
 *     last failure of the calling thread; no exception crosses the boundary;
 *   - query calls are asynchronous on the given stream, exactly like the
 *     reference's per-thread device calls inside a user kernel;
 *   - results are those of the reference's own code on the same inputs
 *     (indices bit-exact, distances bit-exact except where CUDA's
 *     transcendental functions enter the normal-cone tests).
 */
#ifndef SNCH_GB300_H
#define SNCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct snch_scene_s *snch_scene_t;
typedef void *snch_stream_t; /* cudaStream_t */

typedef enum
{
    SNCH_OK = 0,
    SNCH_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, index out of range */
    SNCH_ERR_CUDA = 2,             /* a CUDA runtime call failed (see snch_last_error) */
    SNCH_ERR_NOT_BUILT = 3,        /* query before build: "BVH is not built yet." (scene.cuh:1250) */
    SNCH_ERR_OUT_OF_MEMORY = 4,
    SNCH_ERR_DEVICE_STATUS = 5,    /* a kernel reported a failure, see snch_get_device_status */
    SNCH_ERR_TOO_LARGE = 6         /* more than 2^30 triangles, or a no-allocation limit exceeded */
} snch_status;

/* bits of the device status word (snch_get_device_status) */
#define SNCH_DEVICE_STACK_OVERFLOW 1u   /* a traversal needed more stack entries than it holds */
#define SNCH_DEVICE_LOOKBACK_TIMEOUT 2u /* a bounded cross-block wait gave up (results invalid) */
#define SNCH_DEVICE_HASH_FULL 4u        /* the edge hash table overflowed (results invalid)    */
#define SNCH_DEVICE_TREE_DEPTH 16u      /* a wide-record pass met a tree deeper than its bound  */
#define SNCH_DEVICE_COPY_TIMEOUT 32u    /* a bulk copy into shared memory did not complete in time */
#define SNCH_DEVICE_WORK_TIMEOUT 64u    /* a persistent search stopped taking work (results invalid) */

/* Reference-layout records, byte-compatible with the reference's device view
 * (bvh.cuh:27-33 node, aabb.cuh:12-16 aabb<float,3>, cone.cuh:11-16 cone<float,3>,
 * scene.cuh:708-722 silhouette_edge, scene.cuh:826-840 triangle,
 * bvh.cuh:36-72 basic_device_bvh). */
typedef struct { uint32_t parent_idx, left_idx, right_idx, object_idx; } snch_node;
typedef struct { float upper[3], lower[3]; } snch_aabb;
typedef struct { float axis[3], half_angle, radius; } snch_cone;
typedef struct { int32_t indices[4]; const float *vertices; uint64_t pad_; } snch_silhouette_edge; /* 32 B */
typedef struct
{
    int32_t vertex_indices[3];
    int32_t silhouette_indices[3];
    const float *vertices;                    /* float3 array */
    const snch_silhouette_edge *silhouettes;  /* 40 B */
} snch_triangle;
typedef struct
{
    uint32_t num_nodes;   /* 2N-1 */
    uint32_t num_objects; /* N    */
    const snch_node *nodes;
    const snch_aabb *aabbs;
    const snch_cone *cones;
    const snch_triangle *objects;
} snch_bvh_view;

/* ------------------------------------------------------------------ scene */

/* lbvh::scene<3>(vertices_first, vertices_last, indices_first, indices_last)
 * scene.cuh:1128-1133: host float3 vertices and int3 faces, copied to the GPU. */
int snch_scene_create(const float *vertices_xyz, int64_t num_vertices, const int32_t *triangles,
                      int64_t num_triangles, snch_scene_t *out_scene);

/* Same from device buffers (no host round trip). */
int snch_scene_create_device(const float *vertices_xyz, int64_t num_vertices, const int32_t *triangles,
                             int64_t num_triangles, snch_scene_t *out_scene, snch_stream_t stream);

/* scene<3>::compute_silhouettes() scene.cuh:1167-1204 (with assign_edge_indices 1135-1166),
 * computed on the GPU: edge ids in first-seen order and the 4-vertex edge records. */
int snch_compute_silhouettes(snch_scene_t scene, snch_stream_t stream);

/* scene<3>::build_bvh() scene.cuh:1205-1229 -> bvh::construct() bvh.cuh:380-613:
 * edge ownership, leaf boxes and cones, Morton codes, stable radix sort, Karras
 * internal nodes, bottom-up AABB + normal-cone refit. Runs compute_silhouettes
 * first if it has not been called. Asynchronous on `stream`. */
int snch_build_bvh(snch_scene_t scene, snch_stream_t stream);

/* scene<3>::get_bvh_device_ptr() scene.cuh:1242-1252: the tree in the
 * reference's device layout (device pointers owned by the scene). */
int snch_get_bvh_view(snch_scene_t scene, snch_bvh_view *out_view);

/* The built tree in this library's traversal layout, for the header-only
 * device functions of snch_device.cuh (snch::query_device and friends, called
 * per thread from a caller's own kernels). No reference counterpart: it plays
 * the role of the reference's device view (bvh_device, bvh.cuh:36-72) for the
 * device-side query_device of query.cuh:82-423 and sample.cuh:10-91. Device
 * pointers owned by the scene, valid until it is rebuilt or destroyed. Records
 * (32-bit floats; "bits" = a uint32 stored in a float slot):
 *   inner[N-1], 64 B: (Lup.xyz, Llo.x) (Llo.yz, Rup.xy) (Rup.z, Rlo.xyz)
 *                     (bits L, bits R, bits Linfo, bits Rinfo); children are
 *                     node ids (internal < N-1 <= leaf N-1+j for sorted leaf j);
 *                     a leaf child's info = depth-first rank | owned edges << 30
 *   inner_cones[N-1], 48 B: (L.axis, L.half) (L.radius, R.axis) (R.half, R.radius, 0, 0)
 *   leaves[N], 48 B:  (a.xyz, bits original index) (b.xyz, bits owned edges) (c.xyz, bits rank)
 *   edges[3N], 64 B:  owned silhouette edge k of sorted leaf j at 3j+k:
 *                     (p0.xyz, bits face flags) (p1.xyz, bits edge id) (n0.xyz, 0) (n1.xyz, 0)
 *   root_box:         6 floats, upper xyz then lower xyz
 *   vertices / triangles: the scene's own arrays (sample_on_object)
 *   status:           the scene's device status word (stack overflow bit)
 * Plain scenes only (a batched scene returns SNCH_ERR_INVALID_ARGUMENT). */
typedef struct
{
    uint32_t num_triangles;
    uint32_t reserved;
    const float *root_box;
    const void *inner;
    const void *inner_cones;
    const void *leaves;
    const void *edges;
    const float *vertices;
    const int32_t *triangles;
    uint32_t *status;
} snch_traversal_view;
int snch_get_traversal_view(snch_scene_t scene, snch_traversal_view *out_view);

/* scene_loader<3>(filename) scene_loader.cuh:86-152, a host-side reader: "v x y z"
 * vertices and "f a b c" triangles (1-based in the file, 0-based out; the first
 * three indices of a longer face; every other line ignored), into caller HOST
 * buffers of vert_capacity vertices (3 floats each) and tri_capacity triangles;
 * *num_verts / *num_tris receive the counts in the file whatever the capacities,
 * so a call with capacities 0 sizes the buffers. A face token "7/1/3" or "7//3"
 * gives vertex 7 (the reference's loader cannot read such files). Missing
 * numbers read as 0. Error "Could not open .obj file." as the reference's. */
int snch_obj_read(const char *path, float *verts, int64_t vert_capacity, int32_t *tris, int64_t tri_capacity,
                  int64_t *num_verts, int64_t *num_tris);

/* A built plain scene to / from a flat binary file (no reference counterpart;
 * the reference rebuilds every time): the mesh, the silhouette topology and
 * every tree array, so that snch_scene_load gives a built scene with the same
 * tree and the same query results without rebuilding. Host-endian, for this
 * library's version; save synchronises `stream`, load is synchronous. */
int snch_scene_save(snch_scene_t scene, const char *path, snch_stream_t stream);
int snch_scene_load(const char *path, snch_scene_t *out_scene, snch_stream_t stream);

/* ~scene<3>: frees every device buffer of the scene (the reference's scene owns
 * its device vectors and a unique_ptr to its bvh, scene.cuh:1254-1268). */
int snch_scene_destroy(snch_scene_t scene);

/* Sizes: vertices_h.size(), indices_h.size() and silhouettes_h.size() of the
 * reference's scene (scene.cuh:1255-1264); synchronises the scene's build
 * stream for num_edges. */
int snch_scene_info(snch_scene_t scene, int64_t *num_vertices, int64_t *num_triangles, int64_t *num_edges);
/* The scene's DEVICE vertex buffer (3 floats per vertex, the scene's own copy;
 * no reference counterpart): a caller that moves the vertices writes them here
 * (stream-ordered before the next snch_build_bvh) instead of re-creating the
 * scene. The triangles, and so the silhouette topology, stay as created. */
int snch_scene_vertices(snch_scene_t scene, float **out_device_xyz);

/* Device status word of the scene (OR of SNCH_DEVICE_* bits set by its
 * kernels since the last reset); synchronises the given stream. No reference
 * counterpart: the reference's device code has asserts only, while these
 * kernels finish every bounded wait and report here instead. */
int snch_get_device_status(snch_scene_t scene, uint32_t *out_bits, int reset, snch_stream_t stream);

/* Thread-local description of the last failure: the message the reference
 * throws as an exception ("BVH is not built yet.", scene.cuh:1250; Thrust's
 * system_error on a CUDA failure), returned here since no exception crosses
 * the C ABI. */
const char *snch_last_error(void);

/* Copies of the build products into caller DEVICE buffers (parity checks; the
 * reference's bvh keeps them as its device vectors, bvh.cuh:624-633, and its
 * sort inputs, bvh.cuh:436-454): morton codes sorted (N), sorted original
 * indices (N), nodes ((2N-1)*4), aabbs ((2N-1)*6), cones ((2N-1)*5); any
 * pointer may be NULL. */
int snch_export_tree(snch_scene_t scene, uint32_t *sorted_morton, uint32_t *sorted_indices, uint32_t *nodes,
                     float *aabbs, float *cones, snch_stream_t stream);
/* The silhouette topology (compute_silhouettes, scene.cuh:1135-1229: each
 * triangle's edge ids, its owned edges, each edge's 4 vertex ids) into caller
 * DEVICE buffers: tri_edges (N*3), tri_owned (N*3), edge_verts (E*4). */
int snch_export_topology(snch_scene_t scene, int32_t *tri_edges, int32_t *tri_owned, int32_t *edge_verts,
                         snch_stream_t stream);

/* Traversal order of the nearest-primitive and nearest-silhouette queries.
 * NEAR_FIRST (default) searches the nearer child first; REFERENCE_ORDER replays
 * the reference's stack order (query.cuh:256-316, 344-421). Both return the
 * same indices and distances: exact ties are resolved with each leaf's
 * position in the reference's depth-first order. */
#define SNCH_TRAVERSAL_NEAR_FIRST 0
#define SNCH_TRAVERSAL_REFERENCE_ORDER 1
int snch_set_traversal(snch_scene_t scene, int mode);

/* Scene options (snch_set_option; no reference counterpart: the reference has
 * one fixed search per query type, which the defaults reproduce result for
 * result, and every option below changes only how fast an answer comes):
 *   SNCH_OPT_TRAVERSAL        SNCH_TRAVERSAL_NEAR_FIRST (default) / _REFERENCE_ORDER
 *   SNCH_OPT_QUERY_ORDER      1 (default): nearest, silhouette and ray batches are
 *                             answered in the Morton order of their query points
 *                             (results still land at their input positions and do not
 *                             change); 0: input order. Sphere draws always run in input
 *                             order: their single descent gains less from the order
 *                             than the sort costs (4M draws: 0.77 ms against 0.93).
 *   SNCH_OPT_ORDER_MIN_BATCH  smallest batch that is reordered (default 65536) */
#define SNCH_OPT_TRAVERSAL 1
#define SNCH_OPT_QUERY_ORDER 2
#define SNCH_OPT_ORDER_MIN_BATCH 3
/*   SNCH_OPT_PERSISTENT       1: near-first nearest/silhouette batches (plain or batched
 *                             scenes) searched one query per lane run as persistent
 *                             work-stealing kernels: a warp takes 32 queries at a time
 *                             from a batch-wide counter and a lane takes the next query
 *                             when its own is done; 0 (default): one thread per query.
 *                             Same results; on the 2M-triangle scene with Morton-ordered
 *                             batches the refilled lanes lose their warp's coherence and
 *                             run slower. (Warp packets of batches of at least
 *                             SNCH_OPT_PACKET_PERSISTENT_MIN queries always run
 *                             persistent: a warp takes the next 32 queries when its
 *                             packet is done.)
 *   SNCH_OPT_PERSISTENT_NEAREST / _SILHOUETTE  the same for one query type. */
#define SNCH_OPT_PERSISTENT 4
#define SNCH_OPT_PERSISTENT_NEAREST 16
#define SNCH_OPT_PERSISTENT_SILHOUETTE 17
/*   SNCH_OPT_PERSISTENT_RAY   1: ray batches (closest hit and occlusion) run as persistent
 *                             lane-refill kernels, a lane taking the next ray when its own
 *                             is done; 0 (default): one thread per ray. Same results;
 *                             measured 1.4-1.8x slower on Morton-ordered batches of the
 *                             2M-triangle scene (refilled lanes lose their warp's coherence). */
#define SNCH_OPT_PERSISTENT_RAY 18
/*   SNCH_OPT_TAIL_CAP         near-first nearest/silhouette searches still running after
 *                             this many node expansions (0 = no cap, the default) are
 *                             finished by a second pass seeded with the best distance
 *                             they had reached. Same results; on the 2M-triangle scene
 *                             every cap from 48 to 256 ran 3-27 % slower than none. */
#define SNCH_OPT_TAIL_CAP 5
/*   SNCH_OPT_NODE_WIDTH       2 (default), 4 or 8: the near-first nearest and
 *                             silhouette searches read binary nodes, or 4- / 8-way
 *                             nodes collapsed from the same tree. Same results at
 *                             every width. Setting 4 or 8 allocates that width's
 *                             records (3N/4 + 1 records of 256 / 512 B) and, on a
 *                             built scene, fills them on the legacy default stream
 *                             (synchronous); every later snch_build_bvh fills them
 *                             on its own stream with no host synchronisation.
 *   SNCH_OPT_NODE_WIDTH_NEAREST / _SILHOUETTE  the same for one query type. */
#define SNCH_OPT_NODE_WIDTH 6
#define SNCH_OPT_NODE_WIDTH_NEAREST 7
#define SNCH_OPT_NODE_WIDTH_SILHOUETTE 8
/*   SNCH_OPT_BLOCK            64, 128 (default) or 256 threads per block of the binary
 *                             near-first nearest and silhouette searches (the same
 *                             threads per SM in smaller or larger blocks; a block's
 *                             slot is freed only when its slowest query is done).
 *   SNCH_OPT_BLOCK_NEAREST / _SILHOUETTE  the same for one query type. */
#define SNCH_OPT_BLOCK 9
#define SNCH_OPT_BLOCK_NEAREST 10
#define SNCH_OPT_BLOCK_SILHOUETTE 11
/*   SNCH_OPT_PACKET           warp packets for the binary near-first nearest and
 *                             silhouette searches: a warp's 32 queries walk one shared
 *                             traversal, each lane applying its own tests and keeping its
 *                             own answer. 2 (default): for Morton-ordered batches (nearest
 *                             batches also need at least 1 query per triangle); 1:
 *                             always; 0: never (each lane walks its own). Same distances;
 *                             the silhouette edge id / nearest index equals the per-lane
 *                             one except on an exact distance tie that falls on a
 *                             rounding boundary of a box test, where the reference's own
 *                             choice depends on its visit order.
 *   SNCH_OPT_PACKET_NEAREST / _SILHOUETTE  the same for one query type. */
#define SNCH_OPT_PACKET 12
#define SNCH_OPT_PACKET_NEAREST 13
#define SNCH_OPT_PACKET_SILHOUETTE 14
/*   SNCH_OPT_PACKET_PERSISTENT_MIN  smallest warp-packet batch (nearest and silhouette)
 *                             that runs persistent: each warp takes the next 32 queries
 *                             of the batch when its packet ends, from a pool per SM
 *                             refilled with 32 consecutive packets at a time (same
 *                             packets, same answers); ray batches of at least 4 times
 *                             this run the same way, 32 rays (one per lane) per take.
 *                             Default 2^19 (measured: silhouette packets faster from
 *                             524,288 queries, rays from about 2M); >= 1. */
#define SNCH_OPT_PACKET_PERSISTENT_MIN 19
/*   SNCH_OPT_OUTPUT_SCATTER   1: the results of a Morton-ordered, unseeded batch are
 *                             written in batch order to a temporary and then moved to
 *                             input order by one scatter pass, so that each warp's stores
 *                             fill whole sectors (written at input positions directly,
 *                             neighbouring lanes store 4 bytes each to unrelated sectors
 *                             and DRAM sees 5-9x the output bytes). 0 (default): results
 *                             written at input positions by the search kernels, which are
 *                             bound by instruction issue and latency, not by DRAM: the
 *                             extra pass costs more time than the writes it saves. Same
 *                             results either way. */
#define SNCH_OPT_OUTPUT_SCATTER 20
/*   SNCH_OPT_TOP_LEVELS       0 (default) to 7: the persistent warp-packet searches
 *                             (nearest and silhouette batches of at least
 *                             SNCH_OPT_PACKET_PERSISTENT_MIN queries, plain scenes) copy
 *                             the records of the top levels of the tree (2^levels - 1
 *                             nodes, 112 bytes each) into each block's shared memory
 *                             once, with a bulk copy, and read those nodes from there.
 *                             Same results. */
#define SNCH_OPT_TOP_LEVELS 21
/*   SNCH_OPT_RAY_ORDER        0 (default): ray batches are answered in the Morton order of
 *                             their origins; 1: by length bucket first (floor(log2(tmax /
 *                             the scene box's largest side)), 16 buckets), then by origin,
 *                             so that the rays of a warp have similar lengths (measured 1.6 %
 *                             slower on 16M rays with tmax log-uniform over three decades:
 *                             the lost spatial coherence costs more). Same results. */
#define SNCH_OPT_RAY_ORDER 22
/*   SNCH_OPT_ORDER_BITS       bits of a query's Morton code (plain scenes) that order a
 *                             batch: 12 to 30, default 24 (a 256^3 grid, sorted in three
 *                             radix passes; measured on 16M-query batches of the
 *                             2M-triangle scene: 0.4 % faster per step than 30 bits in four
 *                             passes, 16 bits 52 % slower). Queries of one cell keep their
 *                             input order; only the speed changes. */
#define SNCH_OPT_ORDER_BITS 23
/*   SNCH_OPT_HOST_CHUNK       queries per chunk of the *_host forms (at most 29 bytes in
 *                             and 17 out per query on each of two streams): chunk i's
 *                             input copy, search and output copy run on stream i % 2, so
 *                             copies overlap searches; a larger chunk gives each
 *                             Morton-ordered search a denser batch. 0 (default): 2^24
 *                             for nearest / silhouette, 2^22 for ray / sphere sample. */
#define SNCH_OPT_HOST_CHUNK 15
int snch_set_option(snch_scene_t scene, int option, int64_t value);
/* current value of an option (SNCH_OPT_NODE_WIDTH / _BLOCK / _PACKET read the
 * nearest search's) */
int snch_get_option(snch_scene_t scene, int option, int64_t *value);

/* Position of each sorted leaf in the reference's depth-first visit order,
 * copied to a HOST buffer of N entries (synchronous). */
int snch_export_leaf_ranks(snch_scene_t scene, uint32_t *ranks);

/* ------------------------------------------------------------------ queries
 * All buffers are DEVICE buffers of n entries (float3 = 3 packed floats). */

/* query_device(bvh, nearest(p), scene<3>::distance_calculator()) query.cuh:239-318
 * -> (object index, distance); index 0xFFFFFFFF and +inf for an empty scene. */
int snch_query_nearest(snch_scene_t scene, const float *points_xyz, int64_t n, uint32_t *out_index,
                       float *out_distance, snch_stream_t stream);

/* query_device(bvh, nearest_silhouette(p, flip), silhouette_distance_calculator())
 * query.cuh:326-423 -> distance (+inf if none). flip may be NULL (all false).
 * out_edge (may be NULL) receives the silhouette edge id of the returned
 * distance, which the reference does not report (query.cuh:386), or -1. */
int snch_query_silhouette(snch_scene_t scene, const float *points_xyz, const uint8_t *flip, int64_t n,
                          float *out_distance, int32_t *out_edge, snch_stream_t stream);

/* query_device(bvh, overlaps(box), out, max) query.cuh:177-231: for each query
 * box (6 floats: lower xyz, upper xyz) the ORIGINAL indices of the triangles whose
 * leaf box (FLT_EPSILON-inflated, scene.cuh:870-885) overlaps it, in the
 * reference's visit order; the first max_per_query of them go to
 * out_index[q * max_per_query + k], out_count[q] = how many overlap in all (the
 * reference's return value; may exceed max_per_query). Plain scenes only. */
int snch_query_overlap(snch_scene_t scene, const float *boxes, int64_t n, uint32_t max_per_query,
                       uint32_t *out_index, uint32_t *out_count, snch_stream_t stream);
/* query_device(bvh, line_intersect(line), element_test, out, max) query.cuh:15-77
 * with the scene's triangles as elements: for each line (origin xyz, direction
 * xyz; infinite both ways, the slab test of aabb.cuh:329-348) the triangles it
 * crosses, each with the line parameter t of the crossing, in the reference's
 * visit order. The element test (the caller's functor in the reference, which
 * ships none for triangles) is intersect_test's arithmetic (scene.cuh:1005-1052)
 * for a line: any t. Layout as snch_query_overlap; out_t beside out_index. */
int snch_query_line(snch_scene_t scene, const float *origins, const float *dirs, int64_t n, uint32_t max_per_query,
                    uint32_t *out_index, float *out_t, uint32_t *out_count, snch_stream_t stream);

/* query_device(bvh, ray_intersect(ray(o, d), tmax), intersect_test()) query.cuh:82-169
 * -> (hit, t, uv (2 floats), object index); t = +inf, uv = 0, index 0xFFFFFFFF on a miss. */
int snch_query_ray(snch_scene_t scene, const float *origins_xyz, const float *dirs_xyz, const float *tmax,
                   int64_t n, uint8_t *out_hit, float *out_t, float *out_uv, uint32_t *out_index,
                   snch_stream_t stream);
/* the same with ray_intersect<TestOnly = true> (query.cuh:117-121): an occlusion
 * test that stops at the first hit it accepts -> out_hit only (equal to
 * snch_query_ray's hit flag) */
int snch_query_ray_test(snch_scene_t scene, const float *origins_xyz, const float *dirs_xyz, const float *tmax,
                        int64_t n, uint8_t *out_hit, snch_stream_t stream);

/* sample_object_in_sphere(bvh, sphere_intersect(sphere(c, r)), intersect_sphere(),
 * measurement_getter(), green_weight(), u) sample.cuh:26-91 -> (object index or -1,
 * pdf; 0 when -1, where the reference leaves it unset). */
int snch_sample_in_sphere(snch_scene_t scene, const float *centers_xyz, const float *radii, const float *u,
                          int64_t n, int32_t *out_index, float *out_pdf, snch_stream_t stream);

/* sample_on_object(bvh, idx, scene<3>::sample_on_object(), u, v) sample.cuh:10-22 ->
 * point on triangle idx (original index). */
int snch_sample_on_object(snch_scene_t scene, const int32_t *index, const float *u, const float *v, int64_t n,
                          float *out_points_xyz, snch_stream_t stream);

/* Nearest / silhouette queries with a per-query search radius (DEVICE float[n],
 * e.g. predicted by snch_mlp_predict_radius): the search starts as if a
 * primitive at that distance had been found, so only nodes within it are
 * visited; queries with nothing inside their radius are answered again without
 * a bound within the same call. Results equal snch_query_nearest /
 * snch_query_silhouette for any radii (tie winners included); the radius only
 * changes the work. num_fallback (DEVICE uint32, may be NULL) receives the
 * number of queries that needed the unbounded pass. No reference counterpart:
 * the reference always starts unbounded (query.cuh:255, 343). */
int snch_query_nearest_seeded(snch_scene_t scene, const float *points_xyz, const float *radius, int64_t n,
                              uint32_t *out_index, float *out_distance, uint32_t *num_fallback,
                              snch_stream_t stream);
int snch_query_silhouette_seeded(snch_scene_t scene, const float *points_xyz, const uint8_t *flip,
                                 const float *radius, int64_t n, float *out_distance, int32_t *out_edge,
                                 uint32_t *num_fallback, snch_stream_t stream);

/* ------------------------------------------------------------------ batched scenes
 * Many independent meshes in one scene: one topology pass, one LBVH build and
 * one query launch for all of them (no reference counterpart; a reference user
 * builds one lbvh::scene<3> per mesh). Vertices and triangles are concatenated
 * mesh after mesh; triangle vertex indices are PER MESH (0 = the mesh's first
 * vertex). mesh_vert_start / mesh_tri_start are HOST arrays of num_meshes + 1
 * entries (0 ... nv, 0 ... nt). device != 0: v and t are DEVICE buffers.
 * snch_compute_silhouettes / snch_build_bvh / snch_destroy work as for a scene;
 * each mesh's subtree is exactly the tree a scene of that mesh alone gets. */
int snch_batch_create(const float *v, int64_t nv, const int32_t *t, int64_t nt, const int64_t *mesh_vert_start,
                      const int64_t *mesh_tri_start, int32_t num_meshes, int device, snch_scene_t *out,
                      snch_stream_t stream);
/* number of meshes of a batched scene (0 for a plain scene) */
int snch_batch_num_meshes(snch_scene_t scene, int32_t *out);
/* per-query mesh (DEVICE int32); results as snch_query_nearest / _silhouette on a
 * scene of that mesh alone: triangle index and edge id within the mesh */
int snch_batch_query_nearest(snch_scene_t scene, const int32_t *mesh, const float *points, int64_t n,
                             int32_t *index, float *distance, snch_stream_t stream);
int snch_batch_query_silhouette(snch_scene_t scene, const int32_t *mesh, const float *points,
                                const uint8_t *flip_or_null, int64_t n, float *distance, int32_t *edge_or_null,
                                snch_stream_t stream);
/* the same seeded with a per-query radius (DEVICE float), as snch_query_*_seeded:
 * identical results whatever the radii; num_fallback (DEVICE uint32, may be NULL)
 * receives how many queries found nothing inside their radius */
int snch_batch_query_nearest_seeded(snch_scene_t scene, const int32_t *mesh, const float *points,
                                    const float *radius, int64_t n, int32_t *index, float *distance,
                                    uint32_t *num_fallback, snch_stream_t stream);
int snch_batch_query_silhouette_seeded(snch_scene_t scene, const int32_t *mesh, const float *points,
                                       const float *radius, const uint8_t *flip_or_null, int64_t n, float *distance,
                                       int32_t *edge_or_null, uint32_t *num_fallback, snch_stream_t stream);

/* Autotuner (no reference counterpart): times this scene's nearest and
 * silhouette searches in SNCH_AUTOTUNE_CONFIGS configurations -- (node width,
 * threads per block, SNCH_OPT_PACKET, SNCH_OPT_PERSISTENT) = (2, 128, 1, 0)
 * [warp packets: 32 queries per traversal], (2, 128, 0, 0), (4, 128, 0, 0),
 * (8, 128, 0, 0), (2, 64, 0, 0), (2, 256, 0, 0) [one query per traversal],
 * (2, 128, 0, 1) [persistent work-stealing lanes] -- on caller sample batches
 * (DEVICE buffers; for a batched scene near_mesh / sil_mesh give each query's
 * mesh, else NULL; a count of 0 skips that query type), keeps the fastest
 * configuration per query type (SNCH_OPT_NODE_WIDTH_*, SNCH_OPT_BLOCK_*,
 * SNCH_OPT_PACKET_*, SNCH_OPT_PERSISTENT_*) and releases the wide records no
 * type keeps. out_ms (HOST, may be NULL): 2 x SNCH_AUTOTUNE_CONFIGS floats,
 * milliseconds per batch in that order for nearest, then silhouette.
 * Synchronous. Distances are the same in every configuration (indices too, up
 * to the exact ties described under SNCH_OPT_PACKET); only their speed
 * differs. Stack depth is not a candidate: a search touches its stack only to
 * the depth it reaches. Give a sample with the query density of the real
 * batches (for a batched scene, all queries of some meshes rather than a few
 * of every mesh's): warp packets gain with density and lose on sparse batches. */
#define SNCH_AUTOTUNE_CONFIGS 7
int snch_autotune(snch_scene_t scene, const int32_t *near_mesh, const float *near_points, int64_t n_near,
                  const int32_t *sil_mesh, const float *sil_points, const uint8_t *sil_flip_or_null, int64_t n_sil,
                  float *out_ms, snch_stream_t stream);
/* node width and threads per block of the nearest (which = 0) or silhouette (1)
 * search; either output may be NULL */
int snch_get_search_config(snch_scene_t scene, int which, int32_t *out_width, int32_t *out_block);

/* CUDA-graph capture (no reference counterpart): one graph holds a rebuild of
 * the scene (rebuild != 0: silhouette topology + LBVH + wide records) and one
 * nearest and one silhouette batch (a count of 0 leaves that batch out; for a
 * batched scene near_mesh / sil_mesh give each query's mesh), so that a solver
 * step is one snch_graph_launch. The graph keeps the buffer ADDRESSES given
 * here: refill the same device buffers (vertex positions through
 * snch_scene_vertices, queries) between launches. The scene must have been
 * built once before the capture and must outlive the graph; its tree holds what
 * the last launch built. `stream` must be a created stream. A launch rewrites the
 * scene's tree: order it after every other call still using the scene (an event
 * or a synchronisation when they run on other streams), as for snch_build_bvh. */
typedef struct snch_graph_s *snch_graph_t;
int snch_graph_create(snch_scene_t scene, int rebuild, const int32_t *near_mesh, const float *near_points,
                      int64_t n_near, int32_t *near_index, float *near_distance, const int32_t *sil_mesh,
                      const float *sil_points, const uint8_t *sil_flip_or_null, int64_t n_sil, float *sil_distance,
                      int32_t *sil_edge_or_null, snch_graph_t *out_graph, snch_stream_t stream);
int snch_graph_launch(snch_graph_t graph, snch_stream_t stream);
int snch_graph_destroy(snch_graph_t graph);

/* ------------------------------------------------------------------ 2D scenes
 * lbvh::scene<2> (scene.cuh:287-703): line segments (int2 vertex ids into float2
 * vertices) with silhouette VERTICES. snch_scene2_build = compute_silhouettes()
 * + build_bvh() (scene.cuh:642-683) on the GPU: the same topology, Morton codes,
 * tree and boxes as the reference bit for bit. The queries replay the reference's
 * traversals over the 2D functors: query_device(nearest) (segment index,
 * distance), query_device(nearest_silhouette) (distance; also the silhouette
 * vertex id), query_device(ray_intersect) (hit, t, segment parameter s of
 * intersect_test scene.cuh:555-583, index) and sample_object_in_sphere with a
 * circle (index, pdf; pdf 0 where none is hit), sample_on_object (a point on the
 * segment). Vertices and segments are HOST buffers; everything else DEVICE
 * buffers (float2 = 2 packed floats). A one-segment tree evaluates its segment
 * (the reference reads past its node array there). */
typedef struct snch_scene2_s *snch_scene2_t;
int snch_scene2_create(const float *vertices_xy, int64_t num_vertices, const int32_t *segments,
                       int64_t num_segments, snch_scene2_t *out_scene);
int snch_scene2_destroy(snch_scene2_t scene);
int snch_scene2_build(snch_scene2_t scene, snch_stream_t stream);
int snch_scene2_get_device_status(snch_scene2_t scene, uint32_t *out_bits, int reset, snch_stream_t stream);
/* silhouette vertices (V x int4 {prev, self, next, -1}), owned vertices per segment
 * (N x int2), sorted Morton codes and segment indices (N), nodes ((2N-1) x 4),
 * aabbs ((2N-1) x {upper.xy, lower.xy}), cones ((2N-1) x {axis.xy, half, radius})
 * into caller DEVICE buffers; any may be NULL */
int snch_scene2_export(snch_scene2_t scene, int32_t *silhouette_vertices, int32_t *segment_owned,
                       uint32_t *sorted_morton, uint32_t *sorted_indices, uint32_t *nodes, float *aabbs,
                       float *cones, snch_stream_t stream);
int snch_scene2_query_nearest(snch_scene2_t scene, const float *points_xy, int64_t n, uint32_t *out_index,
                              float *out_distance, snch_stream_t stream);
int snch_scene2_query_silhouette(snch_scene2_t scene, const float *points_xy, const uint8_t *flip_or_null,
                                 int64_t n, float *out_distance, int32_t *out_vertex_or_null, snch_stream_t stream);
int snch_scene2_query_ray(snch_scene2_t scene, const float *origins_xy, const float *dirs_xy, const float *tmax,
                          int64_t n, uint8_t *out_hit, float *out_t, float *out_segment_param, uint32_t *out_index,
                          snch_stream_t stream);
int snch_scene2_query_ray_test(snch_scene2_t scene, const float *origins_xy, const float *dirs_xy, const float *tmax,
                               int64_t n, uint8_t *out_hit, snch_stream_t stream);
int snch_scene2_sample_in_circle(snch_scene2_t scene, const float *centers_xy, const float *radii, const float *u,
                                 int64_t n, int32_t *out_index, float *out_pdf, snch_stream_t stream);
int snch_scene2_sample_on_object(snch_scene2_t scene, const int32_t *index, const float *u, int64_t n,
                                 float *out_points_xy, snch_stream_t stream);

typedef struct snch_mlp_s *snch_mlp_t;

/* ------------------------------------------------------------------ walk-on-stars driver
 * Wavefront walk-on-stars (Sawhney et al. 2023) on a Dirichlet scene (its nearest
 * query gives the distance to the Dirichlet boundary) and a Neumann scene
 * (silhouette distance, rays, SampleTriangleInSphere), for the test problem
 * u(x) = x_0: g = x_0 on Dirichlet faces, h = outward normal . e_0 on Neumann
 * faces. Each step issues, for every live walker, one nearest, one silhouette,
 * one ray and one sphere-sample query (the library's own batched calls);
 * finished walkers are compacted away. With an MLP the nearest and silhouette
 * queries are seeded with its radii (output 0: Dirichlet distance, output 1:
 * Neumann silhouette distance); the walks are the same either way. The
 * reference has no walk driver (its consumer, elaina, is an external project). */
#define SNCH_WOST_MAX_STEPS 128
typedef struct
{
    int64_t walkers;
    int32_t max_steps; /* 1 .. SNCH_WOST_MAX_STEPS */
    float epsilon;     /* Dirichlet shell: a walk ends at distance < epsilon */
    float center[3];   /* walkers start uniform in this ball (inside the domain) */
    float radius;
    uint64_t seed;
    float margin, floor_; /* learned radius = exp(prediction) * margin + floor_ */
} snch_wost_params;
typedef struct
{
    int32_t steps;                          /* steps run */
    int64_t terminated;                     /* walks that reached the Dirichlet shell */
    int64_t live[SNCH_WOST_MAX_STEPS];      /* walkers at the start of each step */
    int64_t queries[SNCH_WOST_MAX_STEPS];   /* queries of each step, all four types */
    float step_ms[SNCH_WOST_MAX_STEPS];     /* device time of each step */
    float query_ms[SNCH_WOST_MAX_STEPS];    /* of which in the query batches and the radius model */
    uint32_t fallback[SNCH_WOST_MAX_STEPS]; /* seeded queries that needed the unbounded pass */
} snch_wost_stats;
/* estimates: DEVICE float[walkers] (by walker); start_points: DEVICE float[3 walkers] or NULL;
 * stats: HOST. Synchronous. */
int snch_wost_trace(snch_scene_t dirichlet, snch_scene_t neumann, snch_mlp_t mlp_or_null,
                    const snch_wost_params *params, float *estimates, float *start_points, snch_wost_stats *stats,
                    snch_stream_t stream);

/* ------------------------------------------------------------------ learned search radius
 * A small MLP (32-frequency Fourier features of the point -> 4 x 64 ReLU ->
 * 2 outputs) predicts log(nearest distance) and log(silhouette distance);
 * its layers run on the 5th-generation tensor cores (tcgen05, BF16 x BF16 ->
 * FP32 in tensor memory). radius = exp(prediction) * margin + floor feeds
 * snch_query_*_seeded, whose fallback keeps results exact whatever the
 * prediction. No reference counterpart. */
int64_t snch_mlp_num_params(void);
/* points are normalised by the box [lo, hi]; seed fixes the initial weights */
int snch_mlp_create(const float *box_lo, const float *box_hi, uint64_t seed, snch_mlp_t *out);
int snch_mlp_destroy(snch_mlp_t mlp);
/* fp32 parameter block (W1 64x192, b1, W2, b2, W3, b3, W4, b4, W5 2x64, b5) to / from HOST memory */
int snch_mlp_get_params(snch_mlp_t mlp, float *host_params, int64_t count);
int snch_mlp_set_params(snch_mlp_t mlp, const float *host_params, int64_t count);
/* pinball-loss gradient (quantile tau) of n samples without an update: DEVICE points (n x 3),
 * DEVICE targets (n x 2 log distances, NaN = no target); HOST gradient and loss (synchronous) */
int snch_mlp_gradient(snch_mlp_t mlp, const float *points, const float *targets, int64_t n, float tau,
                      float *host_grad, float *host_loss, snch_stream_t stream);
/* Adam over `epochs` passes of n samples in batches; *host_loss = mean loss of the last epoch (synchronous) */
int snch_mlp_train(snch_mlp_t mlp, const float *points, const float *targets, int64_t n, int epochs, int64_t batch,
                   float lr, float tau, float *host_loss, snch_stream_t stream);
/* fused tensor-core inference: DEVICE radius_near / radius_sil (either may be NULL) */
int snch_mlp_predict_radius(snch_mlp_t mlp, const float *points, int64_t n, float margin, float floor,
                            float *radius_near, float *radius_sil, snch_stream_t stream);
/* Self-check of the silhouette traversal's fast normal-cone test against the
 * exact one (no reference counterpart): n random box / cone / point cases, half
 * of them within 1e-3 rad of the decision boundary; adds to DEVICE
 * device_counts[3] = {decided and equal, decided and different, left to the
 * exact test}. device_counts[1] must stay 0. */
int snch_selfcheck_cone_filter(int64_t n, uint64_t seed, uint64_t *device_counts, snch_stream_t stream);

/* building block: C[M x N] (+)= A[M x K] * B[N x K]^T, bf16 row-major A and B, fp32 C, on
 * tcgen05 with TMA operand loads; M % 128 == 0, K % 64 == 0, N in {64, 128, 192, 256}; all
 * DEVICE buffers, 16-byte aligned (SNCH_ERR_CUDA otherwise) */
int snch_gemm_bf16(const void *A, const void *B, float *C, int64_t M, int64_t N, int64_t K, int accumulate,
                   uint32_t *device_status, snch_stream_t stream);

/* Host-buffer forms of the four queries: copy in, run, copy out in pipelined
 * chunks on the scene's own streams; return when results are in host memory.
 * The searches start after the work queued on the legacy default stream
 * before the call (stream 0, where a NULL snch_stream_t builds; the input
 * copies overlap it); a build queued on any other stream must be complete
 * before the call.
 * This is the call shape of the reference's benchmark loop (benchmark.cu:395-409). */
int snch_query_nearest_host(snch_scene_t scene, const float *points_xyz, int64_t n, uint32_t *out_index,
                            float *out_distance);
int snch_query_silhouette_host(snch_scene_t scene, const float *points_xyz, const uint8_t *flip, int64_t n,
                               float *out_distance, int32_t *out_edge);
int snch_query_ray_host(snch_scene_t scene, const float *origins_xyz, const float *dirs_xyz, const float *tmax,
                        int64_t n, uint8_t *out_hit, float *out_t, float *out_uv, uint32_t *out_index);
int snch_sample_in_sphere_host(snch_scene_t scene, const float *centers_xyz, const float *radii, const float *u,
                               int64_t n, int32_t *out_index, float *out_pdf);

/* Work counters of the traversal these calls run: for each of n queries, 3
 * words {internal nodes expanded, leaves evaluated, silhouette edges
 * evaluated} into the DEVICE buffer `visits` (results are discarded). kind:
 * 0 nearest (in0 = points), 1 silhouette (in0 = points, flip), 2 ray
 * (in0, in1, in2 = origins, dirs, tmax), 3 sphere sample (centers, radii, u).
 * Used to count algorithmic bytes; no reference counterpart. */
int snch_query_visits(snch_scene_t scene, int kind, const float *in0, const float *in1, const float *in2,
                      const uint8_t *flip, int64_t n, uint32_t *visits, snch_stream_t stream);
/* The same counters for the first pass of a seeded nearest (kind 0) or
 * silhouette (kind 1) search (snch_query_*_seeded): the search starts with the
 * DEVICE radii `radius` as its bound; queries that find nothing inside their
 * radius would then be answered by an unbounded pass, which is not counted
 * here. Shows what a learned radius saves; no reference counterpart. */
int snch_query_visits_seeded(snch_scene_t scene, int kind, const float *points, const uint8_t *flip,
                             const float *radius, int64_t n, uint32_t *visits, snch_stream_t stream);

/* ------------------------------------------------------------------ building blocks */

/* Stable radix sort of (key, value) uint32 pairs on the low key_bits bits, in
 * place on DEVICE buffers (the sort behind bvh.cuh:452-454). keys_tmp/vals_tmp
 * are n-entry DEVICE buffers; scratch is snch_sort_scratch_bytes(n, key_bits)
 * bytes of DEVICE memory. Asynchronous. */
size_t snch_sort_scratch_bytes(int64_t n, int key_bits);
int snch_sort_pairs(uint32_t *keys, uint32_t *values, uint32_t *keys_tmp, uint32_t *values_tmp, int64_t n,
                    int key_bits, void *scratch, uint32_t *device_status, snch_stream_t stream);

/* Number of kernels this library has launched in this process (all scenes). */
uint64_t snch_kernel_launch_count(void);

/* Device memory held for reuse. A destroyed scene's arrays and its host-form
 * staging buffers stay allocated for the next scene of similar size (a scene
 * rebuilt from scratch every batch then pays no cudaMalloc / cudaFree), and
 * per-call scratch comes from a pool that keeps its pages mapped.
 * snch_cached_memory_bytes: bytes of released scene blocks held now (the
 * scratch pool is not counted). snch_release_cached_memory: waits for the
 * device, then returns both to the driver (like emptying a caching
 * allocator). A cudaMalloc that runs out of memory does the same and retries. */
int64_t snch_cached_memory_bytes(void);
int snch_release_cached_memory(void);

/* snch_sort_pairs for callers that cannot allocate GPU memory -- a real-time
 * solver loop that must never stall the device (cudaMalloc/cudaFree can
 * synchronise it), a host plug-in whose GPU memory belongs to the host
 * application's allocator. No counterpart in the reference (whose Thrust sort
 * allocates). Sorts (keys_in, values_in) by the low key_bits bits into
 * (keys_out, values_out) (in == out is allowed), stably, asynchronously on
 * `stream`, calling no allocating routine: all other working memory is one
 * fixed array of about 10 MB that every GPU loading this library holds until
 * exit. At most SNCH_SORT_NOALLOC_MAX_PAIRS pairs per call (larger n returns
 * SNCH_ERR_TOO_LARGE). Calls share that array: calls that overlap on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller. Each call outside a stream capture looks up the array's device
 * address in the current CUDA context (cudaGetSymbolAddress; a context of the
 * caller's own and a context re-created after cudaDeviceReset both work); a
 * call during a capture reuses the address its context last looked up, so make
 * the first call in each context before any stream capture. device_status
 * (may be NULL) is a caller DEVICE word that receives SNCH_DEVICE_* bits; with
 * NULL the bits go to a word inside the shared array that no caller can read,
 * so a sort that gave up on a look-back wait (its output then incomplete) goes
 * unnoticed: pass a status word wherever that matters. */
#define SNCH_SORT_NOALLOC_MAX_PAIRS 1048576
int snch_sort_pairs_noalloc(const uint32_t *keys_in, const uint32_t *values_in, uint32_t *keys_out,
                            uint32_t *values_out, int64_t n, int key_bits, uint32_t *device_status,
                            snch_stream_t stream);

/* Library version string. */
const char *snch_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SNCH_GB300_H */
