// Host-side launchers shared between the translation units of libsnch_gb300.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "../../include/snch_gb300.h"
#include "common.cuh"

namespace snch
{

// Number of kernels this library has launched (snch_kernel_launch_count).
void note_launch(unsigned count = 1);

// Records msg as the calling thread's snch_last_error() and returns code.
int report_error(int code, const std::string &msg);

// Device arrays of one LBVH construction (build.cu).
struct BuildArgs
{
    uint32_t num_tris;
    const float *verts;
    const int32_t *tris;
    const int32_t *tri_owned;
    const int32_t *edge_verts;
    float4 *centroids;
    uint32_t *scene_box;  // 6 ordered uints: upper.xyz (max), lower.xyz (min)
    uint32_t *keys;       // Morton codes, sorted in place
    uint32_t *vals;       // original triangle indices, sorted in place
    uint32_t *hist;       // 4 x 256 digit counts
    NodeRec *nodes;
    Box *aabbs;
    Cone *cones;
    uint32_t *flags;      // refit arrival counters, N-1
    uint32_t *sizes;      // leaves under each internal node, N-1
    InnerRec *inner;
    InnerConeRec *inner_cones;
    LeafRec *leaves;
    EdgeRec *edges;
    uint32_t *status;
    // batched scenes (num_meshes > 0): many independent meshes in one build. The
    // triangles are mesh-major; each mesh gets its own Morton box, the sort key
    // is (mesh, code, local index) and the Karras split prefers mesh boundaries,
    // so every mesh's subtree is exactly the tree a build of that mesh alone gives.
    uint32_t num_meshes;
    const uint32_t *tri_mesh;        // mesh of each (original) triangle
    const uint32_t *mesh_tri_start;  // num_meshes + 1
    uint32_t *mesh_box;              // 6 ordered uints per mesh
    uint32_t *sorted_mesh;           // mesh of each sorted position
    uint32_t *mesh_root;             // subtree root per mesh (a leaf id for one triangle, kInvalid for none)
    uint32_t *perm, *perm_tmp, *mkey_tmp;  // mesh-pass sort scratch
    const int32_t *tri_edges;        // edge id of each triangle side (topology)
    int32_t *mesh_edge_start;        // first silhouette edge id per mesh
};

// Wide (4- or 8-way) traversal records of a built tree (build.cu): a count
// pass (flags + exclusive scan -> wide_of, *count on the device), then a fill
// pass into `out` (capacity records of WideLayout<W>::kRecF4 float4; a record
// index at or beyond it is not written and sets kStatusTreeDepth).
struct WideArgs
{
    int width;  // 4 or 8
    uint32_t num_tris;  // >= 2
    const NodeRec *nodes;
    const Box *aabbs;
    const Cone *cones;
    const LeafRec *leaves;
    uint32_t num_meshes;  // batched scenes: depth counted from each mesh root
    const uint32_t *mesh_root;
    uint32_t *flags;    // N-1 words (the refit's arrival counters, free after a build)
    uint32_t *wide_of;  // N-1 words: wide index of each wide-root node
    uint32_t *count;    // device word: number of wide records
    void *scratch;      // wide_scratch_bytes(num_tris)
    float4 *out;
    uint32_t capacity;  // records of out
    uint32_t *status;
};
size_t wide_scratch_bytes(uint32_t num_tris);
cudaError_t launch_wide_count(const WideArgs &a, cudaStream_t st);
cudaError_t launch_wide_fill(const WideArgs &a, cudaStream_t st);

// ---- build.cu
cudaError_t launch_karras(const BuildArgs &a, cudaStream_t st);  // keys, vals, nodes, sizes, num_tris
cudaError_t launch_build_front(const BuildArgs &a, cudaStream_t st);
cudaError_t launch_build_back(const BuildArgs &a, cudaStream_t st);
// batched scenes: after the Morton sort, the stable pass by mesh id
cudaError_t launch_mesh_pass(const BuildArgs &a, void *scratch, cudaStream_t st);
size_t mesh_pass_scratch_bytes(uint32_t n, uint32_t num_meshes);
cudaError_t launch_mesh_setup(const uint32_t *tri_start, const int64_t *vert_start, uint32_t num_meshes, uint32_t n,
                              uint32_t *tri_mesh, int32_t *tris, uint32_t *bad, cudaStream_t st);
cudaError_t launch_ref_objects(const float *verts, const int32_t *tris, const int32_t *tri_owned,
                               const int32_t *edge_verts, uint32_t num_tris, snch_triangle *objs,
                               snch_silhouette_edge *edges, cudaStream_t st);
cudaError_t launch_validate(const int32_t *tris, int64_t n, int64_t num_verts, uint32_t *bad, cudaStream_t st);

// ---- wost.cu: wavefront walk-on-stars walker updates
struct WalkState  // structure of arrays, one entry per live walker
{
    float *x;        // 3 per walker: current point
    float *nb;       // 3 per walker: outward normal of the Neumann face it stands on
    uint8_t *on_b;   // 1: on the Neumann boundary
    float *total;    // accumulated Neumann source terms
    uint32_t *id;    // walker index (estimates are written at it)
};
struct WalkStep  // per-step batch inputs and results of the ray and sphere-sample queries
{
    float *dir, *radius, *u, *su, *sv;
    uint8_t *hit;
    float *t, *uv;
    uint32_t *hit_idx;
    int32_t *smp_idx;
    float *smp_pdf, *smp_pt;
};
cudaError_t launch_wost_init(const WalkState &s, int64_t n, const float center[3], float radius, uint64_t seed,
                             float *start, cudaStream_t st);
cudaError_t launch_wost_prepare(const WalkState &in, int64_t n, const float *d_dir, const float *d_sil,
                                const WalkState &out, const WalkStep &step_in, uint32_t step, uint32_t last_step,
                                float eps, uint64_t seed, float *estimates, uint32_t *counts, cudaStream_t st);
cudaError_t launch_wost_update(const WalkState &s, int64_t n, const WalkStep &step, const float *nverts,
                               const int32_t *ntris, cudaStream_t st);

// ---- queries.cu (stats != nullptr: per-query work counters, 3 words per query)
cudaError_t launch_nearest(const TreeView &t, const float *pts, int64_t n, uint32_t *idx, float *dist, cudaStream_t st,
                           uint32_t *stats = nullptr, const SeedArgs &seed = SeedArgs());
cudaError_t launch_silhouette(const TreeView &t, const float *pts, const uint8_t *flip, int64_t n, float *dist,
                              int32_t *edge, cudaStream_t st, uint32_t *stats = nullptr,
                              const SeedArgs &seed = SeedArgs());
cudaError_t launch_cone_filter_check(int64_t n, uint64_t seed, unsigned long long *counts, cudaStream_t st);
cudaError_t launch_ray(const TreeView &t, const float *o, const float *d, const float *tmax, int64_t n, uint8_t *hit,
                       float *tt, float *uv, uint32_t *idx, cudaStream_t st, uint32_t *stats = nullptr);
cudaError_t launch_ray_test(const TreeView &t, const float *o, const float *d, const float *tmax, int64_t n,
                            uint8_t *hit, cudaStream_t st);
cudaError_t launch_sample(const TreeView &t, const float *c, const float *r, const float *u, int64_t n, int32_t *idx,
                          float *pdf, cudaStream_t st, uint32_t *stats = nullptr);
// overlap (line = false: q0 = boxes, lower xyz + upper xyz) / line (q0 = origins,
// q1 = directions) enumeration: first max_out results per query, total count
cudaError_t launch_enumerate(const TreeView &t, bool line, const float *q0, const float *q1, int64_t n,
                             uint32_t max_out, uint32_t *idx, float *tt, uint32_t *count, cudaStream_t st);
// Morton-sorted order of a query batch (thread i answers query order[i]);
// Stream-ordered scratch from the library's memory pool on the current device
// (kept mapped between calls; cudaMallocAsync under stream capture). Free with
// cudaFreeAsync on the same stream.
cudaError_t scratch_alloc_raw(void **p, size_t bytes, cudaStream_t st);
// The queries of a seeded batch whose fail_flag is set, listed in batch order
// (order[i], or i without an order) with their count, all on the device.
size_t failed_list_scratch_bytes(int64_t n);
cudaError_t launch_failed_list(const uint32_t *order, const uint32_t *fail_flag, int64_t n, uint32_t *list,
                               uint32_t *count, void *scratch, uint32_t *status, cudaStream_t st);
// the top `slots` (2^levels - 1) heap slots of the tree's internal-node records
cudaError_t launch_top_levels(const InnerRec *inner, const InnerConeRec *cones, uint32_t num_tris, uint32_t slots,
                              InnerRec *top, InnerConeRec *topc, cudaStream_t st);
// scratch holds query_order_scratch_bytes(n) bytes and owns *order.
size_t query_order_scratch_bytes(int64_t n);
// len (optional, rays: tmax): order by length bucket, then by the origin's Morton code
cudaError_t launch_query_order(const TreeView &t, const float *pts, int64_t n, void *scratch, uint32_t **order,
                               cudaStream_t st, const float *len = nullptr);
cudaError_t launch_sample_point(const float *verts, const int32_t *tris, uint32_t num_tris, const int32_t *idx,
                                const float *u, const float *v, int64_t n, float *out, cudaStream_t st);

// ---- mlp.cu (learned search radius)
struct MlpWorkspace
{
    void *X;      // rows x 192 bf16 features
    void *H[4];   // rows x 64 bf16 activations
    void *dZ[4];  // rows x 64 bf16 pre-activation gradients
    void *T;      // 256 x rows bf16 (transposed activations, zero padded)
    void *T2;     // 64 x rows bf16 (transposed gradients)
    void *Wt;     // 64 x 64 bf16 (transposed weight)
    void *Wb;     // bf16 copies of W1..W4
    float *Z, *dH;  // rows x 64 fp32
    float *C;       // 256 x 64 fp32 (weight-gradient GEMM result)
};
size_t mlp_num_params();
cudaError_t set_mlp_scales(const float *scales);
// splits > 1: split K, C holds one M x N slice per split (the caller reduces them)
cudaError_t launch_gemm_bf16(const void *A, const void *B, float *C, int64_t M, int64_t N, int64_t K, int accumulate,
                             uint32_t *status, cudaStream_t st, int splits = 1);
// the same with H non-null: H = bf16(max(A B^T + bias, 0)) (N = 64) instead of C
cudaError_t launch_gemm_bf16_ex(const void *A, const void *B, float *C, const float *bias, void *H, int64_t M,
                                int64_t N, int64_t K, int accumulate, uint32_t *status, cudaStream_t st, int splits);
cudaError_t launch_mlp_radius(const float *params, const float *pts, int64_t n, const float center[3],
                              const float inv_half[3], float margin, float floor_, float *r_near, float *r_sil,
                              uint32_t *status, cudaStream_t st);
cudaError_t mlp_forward_backward(float *params, float *grad, const float *pts, const float *target, int64_t n,
                                 int64_t rows, const float center[3], const float inv_half[3], float tau,
                                 const MlpWorkspace &ws, float *loss, uint32_t *status, cudaStream_t st);
cudaError_t mlp_adam(float *params, const float *grad, float *m, float *v, float lr, int step, cudaStream_t st);

// ---- scan_sort.cu
// Exclusive scan of 0/1 flags (totals below 2^30), one pass, decoupled look-back.
size_t scan_flags_scratch_bytes(uint64_t n);
cudaError_t scan_flags(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, void *scratch,
                       uint32_t *status, cudaStream_t st);

// Stable LSD radix sort of (key, value) pairs on the low key_bits bits,
// onesweep style: one histogram pass then one scatter pass per 8-bit digit.
// Data ping-pongs between (keys, vals) and (keys_tmp, vals_tmp); the result
// is written back to (keys, vals), unless result is non-null: then *result
// receives the buffer pair that holds it ((keys, vals) or (keys_tmp,
// vals_tmp), after an odd number of passes) and nothing is copied back. If
// hist is non-null it already holds the per-pass digit counts (passes x 256)
// and the histogram pass is skipped.
constexpr int kSortTile = 4096;
size_t sort_scratch_bytes(uint32_t n, int key_bits);
struct SortResult
{
    uint32_t *keys, *vals;
};
cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_tmp, uint32_t *vals_tmp, uint32_t n,
                             int key_bits, const uint32_t *hist, void *scratch, uint32_t *status, cudaStream_t st,
                             SortResult *result = nullptr);
inline int sort_passes(int key_bits) { return (key_bits + 7) / 8; }

// ---- topology.cu (scene.cuh:1135-1225 on the device)
size_t topology_scratch_bytes(uint32_t num_tris);
// Outputs: tri_edges, tri_owned (int32 x 3N), edge_verts (int32 x 4 x capacity 3N), *num_edges (device).
cudaError_t compute_topology(const int32_t *tris, uint32_t num_tris, int32_t *tri_edges, int32_t *tri_owned,
                             int32_t *edge_verts, uint32_t *num_edges, void *scratch, uint32_t *status,
                             cudaStream_t st);

}  // namespace snch
