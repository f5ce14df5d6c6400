// C ABI of libsnch_gb300 (declared in include/snch_gb300.h): scene lifetime,
// build orchestration, query dispatch and the pipelined host-buffer forms.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <cmath>

#include <atomic>
#include <map>
#include <mutex>
#include <unordered_map>

#include "internal.h"

namespace snch
{
static std::atomic<unsigned long long> g_kernel_launches{0};
void note_launch(unsigned count) { g_kernel_launches.fetch_add(count, std::memory_order_relaxed); }
}  // namespace snch

using namespace snch;

namespace
{
thread_local std::string g_error;

int fail(int code, const std::string &msg)
{
    g_error = msg;
    return code;
}
}  // namespace

int snch::report_error(int code, const std::string &msg) { return fail(code, msg); }

namespace
{

#define SNCH_CUDA(expr)                                                                                    \
    do                                                                                                     \
    {                                                                                                      \
        cudaError_t e_ = (expr);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return fail(e_ == cudaErrorMemoryAllocation ? SNCH_ERR_OUT_OF_MEMORY : SNCH_ERR_CUDA,          \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));                               \
    } while (0)

inline cudaStream_t S(snch_stream_t s) { return static_cast<cudaStream_t>(s); }

// small device words: [0..5] scene box, [8..1031] histograms, [1040] status,
// [1041] num_edges, [1042] bad-index counter
constexpr size_t kSmallWords = 1056;
constexpr size_t kWStatus = 1040, kWNumEdges = 1041, kWBad = 1042, kWHist = 8;

// queries per pipelined host-form chunk when SNCH_OPT_HOST_CHUNK is 0 (auto):
// nearest / silhouette searches gain from a dense Morton-ordered batch, ray and
// sphere-sample batches from copies that overlap the next chunk's search
constexpr int64_t kHostChunkSearch = 1 << 24, kHostChunkRay = 1 << 22;

struct HostStage
{
    void *in[2] = {nullptr, nullptr};
    void *out[2] = {nullptr, nullptr};
    size_t in_bytes = 0, out_bytes = 0;
};
}  // namespace

struct snch_scene_s
{
    uint32_t num_verts = 0, num_tris = 0;
    int64_t num_edges_host = -1;
    float *verts = nullptr;
    int32_t *tris = nullptr, *tri_edges = nullptr, *tri_owned = nullptr, *edge_verts = nullptr;
    NodeRec *nodes = nullptr;
    Box *aabbs = nullptr;
    Cone *cones = nullptr;
    InnerRec *inner = nullptr;
    InnerConeRec *inner_cones = nullptr;
    LeafRec *leaves = nullptr;
    EdgeRec *edges = nullptr;
    uint32_t *keys = nullptr, *vals = nullptr, *keys_tmp = nullptr, *vals_tmp = nullptr, *flags = nullptr;
    uint32_t *sizes = nullptr;
    float4 *centroids = nullptr;
    uint32_t *small = nullptr;
    void *scratch = nullptr;
    snch_triangle *ref_objects = nullptr;
    snch_silhouette_edge *ref_edges = nullptr;
    bool topology_ready = false, built = false;
    int traversal = SNCH_TRAVERSAL_NEAR_FIRST;
    int query_order = 1;             // Morton-sort batches of at least order_min queries
    int64_t order_min = 65536;
    int64_t host_chunk = 0;  // queries per pipelined host-form chunk; 0: per query type
    int persistent_near = 0, persistent_sil = 0;  // lane-refill (work-stealing) searches
    int persistent_ray = 0;
    int64_t tail_cap = 0;            // near-first expansions before a query is deferred (0: off; measured slower)
    // batched scene (num_meshes > 0): independent meshes, one build, per-mesh queries
    uint32_t num_meshes = 0;
    uint32_t *tri_mesh = nullptr, *mesh_tri_start = nullptr, *mesh_box = nullptr, *sorted_mesh = nullptr,
             *mesh_root = nullptr, *perm = nullptr, *perm_tmp = nullptr, *mkey_tmp = nullptr;
    int32_t *mesh_edge_start = nullptr;
    cudaStream_t pipe[2] = {nullptr, nullptr};
    cudaEvent_t pipe_ready = nullptr;  // legacy-stream work before a host-form call
    HostStage stage;
    // Fallback fraction of the last seeded nearest [0] / silhouette [1] call,
    // read back without a synchronisation: the count is copied to pinned host
    // memory behind an event and taken at a later call once the event is done.
    float fallback_frac[2] = {0.0f, 0.0f};
    uint32_t *fallback_host = nullptr;  // pinned: [kind] = fallback count
    cudaEvent_t fallback_event[2] = {nullptr, nullptr};
    int64_t fallback_pending[2] = {0, 0};  // batch size whose count is in flight
    // node width of the near-first nearest / silhouette searches (2, 4 or 8)
    // and the wide records of the built tree: [0] 4-way, [1] 8-way
    int width_near = 2, width_sil = 2;
    int block_near = 128, block_sil = 128;  // threads per block of the binary searches
    int packet_near = 2, packet_sil = 2;    // warp packets: 0 never, 1 always, 2 Morton-ordered batches
    int64_t packet_persistent_min = int64_t(1) << 19;  // packet batches this large run persistent (rays: 4x)
    int output_scatter = 0;  // ordered batches: results in batch order, then one scatter pass (measured slower)
    int ray_order = 0;       // ray batches ordered by length bucket, then origin
    int order_bits = 24;     // Morton bits of the query-order key of plain scenes (3 sort passes; faster than 30)
    // top tree levels staged in shared memory by the persistent packet searches:
    // the first 2^levels - 1 of kTopSlots heap slots, gathered after every build
    int top_levels = 0;
    InnerRec *top_inner = nullptr;
    InnerConeRec *top_cones = nullptr;
    float4 *wide[2] = {nullptr, nullptr};
    uint32_t *wide_idx[2] = {nullptr, nullptr};  // wide index of each wide-root binary node
    size_t wide_cap[2] = {0, 0};  // records allocated
    bool wide_ready[2] = {false, false};

    TreeView view() const
    {
        TreeView t{};
        t.num_tris = num_tris;
        t.nodes = nodes;
        t.aabbs = aabbs;
        t.inner = inner;
        t.inner_cones = inner_cones;
        t.leaves = leaves;
        t.edges = edges;
        t.status = small + kWStatus;
        t.near_first = traversal == SNCH_TRAVERSAL_NEAR_FIRST ? 1 : 0;
        t.persistent = (persistent_near ? 1 : 0) | (persistent_sil ? 2 : 0) | (persistent_ray ? 4 : 0);
        t.width_near = width_near;
        t.width_sil = width_sil;
        t.block_near = block_near;
        t.block_sil = block_sil;
        t.packet_near = packet_near;
        t.packet_sil = packet_sil;
        t.packet_persistent_min = packet_persistent_min;
        t.out_batch_order_enabled = output_scatter;
        t.order_bits = order_bits;
        if (top_levels > 0 && num_meshes == 0)
        {
            t.top_inner = top_inner;
            t.top_cones = top_cones;
            t.top_slots = (1u << top_levels) - 1u;
        }
        if (wide_ready[0])
        {
            t.wide4 = wide[0];
            t.wide4_of = wide_idx[0];
        }
        if (wide_ready[1])
        {
            t.wide8 = wide[1];
            t.wide8_of = wide_idx[1];
        }
        return t;
    }
};

namespace
{
constexpr uint32_t kTopSlots = 127;  // seven levels: 8 KB of records + 6 KB of cones
// Scene arrays and host-form staging buffers come from a cache of released
// device blocks: a scene created and destroyed once per batch of work reuses
// the previous scene's blocks instead of paying cudaMalloc / cudaFree (and the
// device-wide synchronisation of cudaFree) each time. A block is released to
// the cache only when no queued device work uses it; a request takes the
// smallest cached block of at least its size and at most 1/8 larger. A failed
// cudaMalloc returns the cache to the driver and tries once more;
// snch_release_cached_memory() does the same on request.
struct BlockCache
{
    std::mutex mu;
    std::multimap<size_t, void *> free_blocks;        // size -> block
    std::unordered_map<void *, size_t> live;          // block -> size
    size_t cached_bytes = 0;
};
BlockCache &block_cache()
{
    static BlockCache *c = new BlockCache();  // never destroyed: scenes may outlive static destructors
    return *c;
}

void cache_trim_locked(BlockCache &c)
{
    for (auto &kv : c.free_blocks)
        cudaFree(kv.second);
    c.free_blocks.clear();
    c.cached_bytes = 0;
}

cudaError_t cache_alloc(void **p, size_t bytes)
{
    *p = nullptr;
    bytes = (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
    BlockCache &c = block_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    auto it = c.free_blocks.lower_bound(bytes);
    if (it != c.free_blocks.end() && it->first <= bytes + bytes / 8)
    {
        *p = it->second;
        c.live[it->second] = it->first;
        c.cached_bytes -= it->first;
        c.free_blocks.erase(it);
        return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation && !c.free_blocks.empty())
    {
        cudaGetLastError();
        cache_trim_locked(c);
        e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess)
    {
        *p = nullptr;
        return e;
    }
    c.live[*p] = bytes;
    return cudaSuccess;
}

// p must be idle: no queued device work may read or write it
void cache_release(void *p)
{
    if (!p)
        return;
    BlockCache &c = block_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    auto it = c.live.find(p);
    if (it == c.live.end())
    {
        cudaFree(p);  // not from the cache
        return;
    }
    c.free_blocks.emplace(it->second, p);
    c.cached_bytes += it->second;
    c.live.erase(it);
}

// Per-call scratch (query orders, deferred lists, workspaces) is stream-ordered
// and comes from this library's own memory pool on the current device, which
// keeps released memory mapped (release threshold: unlimited) so a call does
// not map fresh pages each time. Under stream capture the allocation is left
// to the graph (cudaMallocAsync). Released by snch_release_cached_memory().
constexpr int kMaxDevices = 64;
cudaMemPool_t g_pool[kMaxDevices] = {};
std::mutex g_pool_mu;

cudaMemPool_t scratch_pool()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return nullptr;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pool[dev])
    {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess)
        {
            cudaGetLastError();
            return nullptr;
        }
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pool[dev] = pool;
    }
    return g_pool[dev];
}

void trim_pools()
{
    std::lock_guard<std::mutex> lock(g_pool_mu);
    for (cudaMemPool_t pool : g_pool)
        if (pool)
            cudaMemPoolTrimTo(pool, 0);
}

}  // namespace

cudaError_t snch::scratch_alloc_raw(void **pp, size_t bytes, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return cudaMallocAsync(pp, bytes, st);
    cudaMemPool_t pool = scratch_pool();
    if (!pool)
        return cudaMallocAsync(pp, bytes, st);
    cudaError_t e = cudaMallocFromPoolAsync(pp, bytes, pool, st);
    if (e == cudaErrorMemoryAllocation)
    {
        cudaGetLastError();
        {
            BlockCache &c = block_cache();
            std::lock_guard<std::mutex> lock(c.mu);
            cache_trim_locked(c);
        }
        cudaStreamSynchronize(st);
        cudaMemPoolTrimTo(pool, 0);
        e = cudaMallocFromPoolAsync(pp, bytes, pool, st);
    }
    return e;
}


namespace
{
template <typename T>
cudaError_t scratch_alloc(T **p, size_t bytes, cudaStream_t st)
{
    void *q = nullptr;
    const cudaError_t e = scratch_alloc_raw(&q, bytes, st);
    *p = static_cast<T *>(q);
    return e;
}

template <typename T>
cudaError_t dalloc(T **p, size_t count)
{
    void *q = nullptr;
    const cudaError_t e = cache_alloc(&q, sizeof(T) * std::max<size_t>(count, 1));
    *p = static_cast<T *>(q);
    return e;
}

void free_scene(snch_scene_s *s)
{
    void *ptrs[] = {s->verts, s->tris, s->tri_edges, s->tri_owned, s->edge_verts, s->nodes, s->aabbs, s->cones,
                    s->inner, s->inner_cones, s->leaves, s->edges, s->keys, s->vals, s->keys_tmp, s->vals_tmp,
                    s->flags, s->sizes, s->centroids, s->small, s->scratch, s->ref_objects, s->ref_edges,
                    s->stage.in[0], s->stage.in[1], s->stage.out[0], s->stage.out[1],
                    s->tri_mesh, s->mesh_tri_start, s->mesh_box, s->sorted_mesh, s->mesh_root, s->perm,
                    s->perm_tmp, s->mkey_tmp, s->mesh_edge_start, s->wide[0], s->wide[1], s->wide_idx[0],
                    s->wide_idx[1], s->top_inner, s->top_cones};
    cudaDeviceSynchronize();  // the scene's queued work ends before its blocks are reused
    for (void *p : ptrs)
        cache_release(p);
    for (cudaStream_t st : s->pipe)
        if (st)
            cudaStreamDestroy(st);
    for (cudaEvent_t ev : s->fallback_event)
        if (ev)
            cudaEventDestroy(ev);
    if (s->pipe_ready)
        cudaEventDestroy(s->pipe_ready);
    if (s->fallback_host)
        cudaFreeHost(s->fallback_host);
    delete s;
}

int allocate(snch_scene_s *s)
{
    const size_t n = s->num_tris, nn = n ? 2 * n - 1 : 1, ni = n > 1 ? n - 1 : 1;
    SNCH_CUDA(dalloc(&s->verts, 3 * (size_t)s->num_verts));
    SNCH_CUDA(dalloc(&s->tris, 3 * n));
    SNCH_CUDA(dalloc(&s->tri_edges, 3 * n));
    SNCH_CUDA(dalloc(&s->tri_owned, 3 * n));
    SNCH_CUDA(dalloc(&s->edge_verts, 4 * 3 * n));
    SNCH_CUDA(dalloc(&s->nodes, nn));
    SNCH_CUDA(dalloc(&s->aabbs, nn));
    SNCH_CUDA(dalloc(&s->cones, nn));
    SNCH_CUDA(dalloc(&s->inner, ni));
    SNCH_CUDA(dalloc(&s->inner_cones, ni));
    SNCH_CUDA(dalloc(&s->leaves, n));
    SNCH_CUDA(dalloc(&s->edges, 3 * n));
    SNCH_CUDA(dalloc(&s->keys, n));
    SNCH_CUDA(dalloc(&s->vals, n));
    SNCH_CUDA(dalloc(&s->keys_tmp, n));
    SNCH_CUDA(dalloc(&s->vals_tmp, n));
    SNCH_CUDA(dalloc(&s->flags, ni));
    SNCH_CUDA(dalloc(&s->sizes, ni));
    SNCH_CUDA(dalloc(&s->centroids, n));
    SNCH_CUDA(dalloc(&s->small, kSmallWords));
    SNCH_CUDA(dalloc(&s->ref_objects, n));
    SNCH_CUDA(dalloc(&s->ref_edges, 3 * n));
    SNCH_CUDA(dalloc(&s->top_inner, kTopSlots));
    SNCH_CUDA(dalloc(&s->top_cones, kTopSlots));
    const size_t scratch = std::max(topology_scratch_bytes((uint32_t)n), sort_scratch_bytes((uint32_t)n, 30));
    SNCH_CUDA(cache_alloc(&s->scratch, scratch));
    SNCH_CUDA(cudaMemset(s->small, 0, kSmallWords * 4));
    return SNCH_OK;
}

int allocate_batch(snch_scene_s *s)
{
    const size_t n = s->num_tris, m = s->num_meshes;
    SNCH_CUDA(dalloc(&s->tri_mesh, n));
    SNCH_CUDA(dalloc(&s->mesh_tri_start, m + 1));
    SNCH_CUDA(dalloc(&s->mesh_box, 6 * m));
    SNCH_CUDA(dalloc(&s->sorted_mesh, n));
    SNCH_CUDA(dalloc(&s->mesh_root, m));
    SNCH_CUDA(dalloc(&s->perm, n));
    SNCH_CUDA(dalloc(&s->perm_tmp, n));
    SNCH_CUDA(dalloc(&s->mkey_tmp, n));
    SNCH_CUDA(dalloc(&s->mesh_edge_start, m));
    return SNCH_OK;
}

int create_common(const float *v, int64_t nv, const int32_t *t, int64_t nt, snch_scene_t *out, bool device,
                  cudaStream_t st)
{
    if (!out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "out_scene is NULL");
    *out = nullptr;
    if (nv < 0 || nt < 0)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "negative vertex or triangle count");
    if ((nv > 0 && !v) || (nt > 0 && !t))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL vertex or triangle buffer");
    if (nt >= (int64_t(1) << 30) || nv >= (int64_t(1) << 31))
        return fail(SNCH_ERR_TOO_LARGE, "at most 2^30 - 1 triangles and 2^31 - 1 vertices are supported");
    if (!device)
    {
        // one branch-free pass (an unsigned compare also catches negative
        // indices), then a search for the first bad index only on failure
        uint32_t any_bad = 0;
        const uint32_t unv = (uint32_t)nv;
        for (int64_t i = 0; i < 3 * nt; ++i)
            any_bad |= (uint32_t)((uint32_t)t[i] >= unv);
        if (any_bad)
            for (int64_t i = 0; i < 3 * nt; ++i)
                if (t[i] < 0 || t[i] >= nv)
                    return fail(SNCH_ERR_INVALID_ARGUMENT,
                                "triangle vertex index out of range at triangle " + std::to_string(i / 3));
    }
    snch_scene_s *s = new snch_scene_s();
    s->num_verts = (uint32_t)nv;
    s->num_tris = (uint32_t)nt;
    int rc = allocate(s);
    if (rc != SNCH_OK)
    {
        free_scene(s);
        return rc;
    }
    const cudaMemcpyKind kind = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaError_t e = cudaSuccess;
    if (nv)
        e = cudaMemcpyAsync(s->verts, v, 12 * (size_t)nv, kind, st);
    if (e == cudaSuccess && nt)
        e = cudaMemcpyAsync(s->tris, t, 12 * (size_t)nt, kind, st);
    if (e == cudaSuccess && device && nt)
    {
        e = launch_validate(s->tris, 3 * nt, nv, s->small + kWBad, st);
        uint32_t bad = 0;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&bad, s->small + kWBad, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && bad)
        {
            free_scene(s);
            return fail(SNCH_ERR_INVALID_ARGUMENT, std::to_string(bad) + " triangle vertex indices out of range");
        }
    }
    if (e == cudaSuccess && !device)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        free_scene(s);
        return fail(SNCH_ERR_CUDA, std::string("scene upload: ") + cudaGetErrorString(e));
    }
    *out = s;
    return SNCH_OK;
}

int topology(snch_scene_s *s, cudaStream_t st)
{
    SNCH_CUDA(compute_topology(s->tris, s->num_tris, s->tri_edges, s->tri_owned, s->edge_verts,
                               s->small + kWNumEdges, s->scratch, s->small + kWStatus, st));
    s->topology_ready = true;
    s->num_edges_host = -1;
    return SNCH_OK;
}

BuildArgs build_args(snch_scene_s *s)
{
    BuildArgs a{};
    a.num_tris = s->num_tris;
    a.verts = s->verts;
    a.tris = s->tris;
    a.tri_owned = s->tri_owned;
    a.edge_verts = s->edge_verts;
    a.centroids = s->centroids;
    a.scene_box = s->small;
    a.keys = s->keys;
    a.vals = s->vals;
    a.hist = s->small + kWHist;
    a.nodes = s->nodes;
    a.aabbs = s->aabbs;
    a.cones = s->cones;
    a.flags = s->flags;
    a.sizes = s->sizes;
    a.inner = s->inner;
    a.inner_cones = s->inner_cones;
    a.leaves = s->leaves;
    a.edges = s->edges;
    a.status = s->small + kWStatus;
    a.num_meshes = s->num_meshes;
    a.tri_mesh = s->tri_mesh;
    a.mesh_tri_start = s->mesh_tri_start;
    a.mesh_box = s->mesh_box;
    a.sorted_mesh = s->sorted_mesh;
    a.mesh_root = s->mesh_root;
    a.perm = s->perm;
    a.perm_tmp = s->perm_tmp;
    a.mkey_tmp = s->mkey_tmp;
    a.tri_edges = s->tri_edges;
    a.mesh_edge_start = s->mesh_edge_start;
    return a;
}

// Wide records of width W. A tree of n >= 2 leaves has fewer than 3n/4 wide
// nodes (a wide node has at least three children unless both its binary
// children are leaves; such nodes hold two leaves each, so with a of them and
// b others, 2a + 3b <= (a + b - 1) + n and a <= n/2), so the records are
// allocated once per scene at that bound, when a width first needs them, and
// every later build fills them without a host synchronisation.
size_t wide_capacity(uint32_t num_tris) { return (size_t)num_tris * 3 / 4 + 1; }

int alloc_wide(snch_scene_s *s, int W)
{
    const int k = W == 4 ? 0 : 1;
    if (s->wide[k] || s->num_tris < 2)
        return SNCH_OK;
    const size_t rec = sizeof(float4) * (W == 4 ? WideLayout<4>::kRecF4 : WideLayout<8>::kRecF4);
    SNCH_CUDA(dalloc(&s->wide_idx[k], s->num_tris - 1));
    SNCH_CUDA(cudaMalloc(reinterpret_cast<void **>(&s->wide[k]), wide_capacity(s->num_tris) * rec));
    s->wide_cap[k] = wide_capacity(s->num_tris);
    return SNCH_OK;
}

// Fills the wide records of width W for the built tree (stream-ordered).
int ensure_wide(snch_scene_s *s, int W, cudaStream_t st)
{
    const int k = W == 4 ? 0 : 1;
    if (s->wide_ready[k])
        return SNCH_OK;
    if (s->num_tris < 2)
    {
        s->wide_ready[k] = true;  // a one-triangle tree is searched as its leaf
        return SNCH_OK;
    }
    if (!s->wide[k])
        return fail(SNCH_ERR_INVALID_ARGUMENT, "wide records are allocated by snch_set_option (node width)");
    WideArgs a{};
    a.width = W;
    a.num_tris = s->num_tris;
    a.nodes = s->nodes;
    a.aabbs = s->aabbs;
    a.cones = s->cones;
    a.leaves = s->leaves;
    a.num_meshes = s->num_meshes;
    a.mesh_root = s->mesh_root;
    a.flags = s->flags;
    a.wide_of = s->wide_idx[k];
    a.capacity = (uint32_t)s->wide_cap[k];
    a.out = s->wide[k];
    a.status = s->small + kWStatus;
    char *scratch = nullptr;
    SNCH_CUDA(scratch_alloc(&scratch, wide_scratch_bytes(s->num_tris) + 256, st));
    a.count = reinterpret_cast<uint32_t *>(scratch);
    a.scratch = scratch + 256;
    cudaError_t e = launch_wide_count(a, st);
    if (e == cudaSuccess)
        e = launch_wide_fill(a, st);
    cudaFreeAsync(scratch, st);
    SNCH_CUDA(e);
    s->wide_ready[k] = true;
    return SNCH_OK;
}

int ensure_widths(snch_scene_s *s, cudaStream_t st)
{
    for (int W : {4, 8})
        if (s->width_near == W || s->width_sil == W)
        {
            int rc = ensure_wide(s, W, st);
            if (rc != SNCH_OK)
                return rc;
        }
    return SNCH_OK;
}

int check_built(snch_scene_t s)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (!s->built)
        return fail(SNCH_ERR_NOT_BUILT, "BVH is not built yet.");
    return SNCH_OK;
}

int check_n(int64_t n, std::initializer_list<const void *> ptrs)
{
    if (n < 0)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "negative query count");
    if (n > 0)
        for (const void *p : ptrs)
            if (!p)
                return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL query buffer");
    return SNCH_OK;
}

// Tree view for one batch: Morton-sorted query order when enabled (the
// ordering scratch is stream-ordered memory released after the launch).
struct BatchView
{
    TreeView t;
    void *scratch = nullptr;
    cudaStream_t st = nullptr;
    ~BatchView()
    {
        if (scratch)
            cudaFreeAsync(scratch, st);
    }
};
cudaError_t batch_view(const snch_scene_s *s, const float *keys_from, int64_t n, cudaStream_t st, BatchView &b,
                       const uint32_t *query_mesh = nullptr, const float *ray_len = nullptr, bool ordered = true)
{
    b.t = s->view();
    b.st = st;
    if (query_mesh)
    {
        // batched queries: per-mesh subtrees, near-first one-thread-per-query kernels
        b.t.query_mesh = query_mesh;
        b.t.mesh_root = s->mesh_root;
        b.t.mesh_tri_start = s->mesh_tri_start;
        b.t.mesh_edge_start = s->mesh_edge_start;
        b.t.num_meshes = s->num_meshes;
        b.t.near_first = 1;
    }
    if (!ordered || !s->query_order || n < s->order_min || n >= (int64_t(1) << 30) || s->num_tris < 2)
        return cudaSuccess;
    cudaError_t e = scratch_alloc(&b.scratch, query_order_scratch_bytes(n), st);
    if (e != cudaSuccess)
        return e;
    uint32_t *order = nullptr;
    e = launch_query_order(b.t, keys_from, n, b.scratch, &order, st, s->ray_order ? ray_len : nullptr);
    b.t.order = order;
    b.t.order_coherent = 1;
    return e;
}

// Fallback lists of at least this fraction of their batch run as warp packets
// (when the batch itself qualifies): measured on the 2M-triangle scene (3.3 %
// silhouette fallbacks: packets x1.08) and the 20,480-triangle sphere (5.5 %:
// x1.5), against a walk-on-stars trace (0.08 %: packets x0.86 overall).
constexpr float kPacketFallbackMinFrac = 0.01f;

// Takes the count of an earlier seeded call of this kind if it has arrived
// (never waits for it).
void refresh_fallback_frac(snch_scene_s *s, int kind)
{
    if (s->fallback_pending[kind] <= 0)
        return;
    if (cudaEventQuery(s->fallback_event[kind]) != cudaSuccess)
    {
        cudaGetLastError();  // cudaErrorNotReady is not an error
        return;
    }
    s->fallback_frac[kind] = (float)s->fallback_host[kind] / (float)s->fallback_pending[kind];
    s->fallback_pending[kind] = 0;
}

// Queues the copy of this call's fallback count to pinned host memory (not
// under stream capture, and not while an earlier copy is still in flight).
cudaError_t queue_fallback_count(snch_scene_s *s, int kind, const uint32_t *count, int64_t n, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess || cs != cudaStreamCaptureStatusNone || n <= 0 || s->fallback_pending[kind] > 0)
        return e;
    if (!s->fallback_host)
    {
        if ((e = cudaHostAlloc(reinterpret_cast<void **>(&s->fallback_host), 2 * sizeof(uint32_t),
                               cudaHostAllocDefault)) != cudaSuccess)
            return e;
        s->fallback_host[0] = s->fallback_host[1] = 0;
    }
    if (!s->fallback_event[kind] &&
        (e = cudaEventCreateWithFlags(&s->fallback_event[kind], cudaEventDisableTiming)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(s->fallback_host + kind, count, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return e;
    s->fallback_pending[kind] = n;
    return cudaEventRecord(s->fallback_event[kind], st);
}

// One nearest / silhouette batch in up to three passes:
//   1. the batch (Morton-ordered), seeded with `radius` if given, near-first
//      searches capped at tail_cap expansions (the long ones are deferred with
//      the best distance they had);
//   2. the deferred queries, seeded with that distance (same results);
//   3. with a user radius: the queries with nothing inside it, unbounded.
// Every pass reads its query list and count on the device: no host sync.
template <typename Launch>
int run_query(snch_scene_s *s, int kind, const float *pts, const float *radius, int64_t n, uint32_t *num_fallback,
              cudaStream_t st, Launch launch, const uint32_t *query_mesh = nullptr)
{
    const bool persistent = kind == 0 ? s->persistent_near : s->persistent_sil;
    const bool capped = s->tail_cap > 0 && s->traversal == SNCH_TRAVERSAL_NEAR_FIRST && !persistent;
    BatchView b;
    if (!capped && !radius)
    {
        SNCH_CUDA(batch_view(s, pts, n, st, b, query_mesh));
        SNCH_CUDA(launch(b.t, SeedArgs()));
        return SNCH_OK;
    }
    // scratch: [counts][fail_flag][fail_list][list-building scratch][defer_list][defer_radius]
    const size_t per = 4 * (size_t)n + 256;
    const size_t fl_bytes = radius ? 2 * per + failed_list_scratch_bytes(n) + 256 : 0;
    char *scratch = nullptr;
    SNCH_CUDA(scratch_alloc(&scratch, 256 + fl_bytes + (capped ? 2 * per : 0), st));
    uint32_t *defer_count = reinterpret_cast<uint32_t *>(scratch), *fail_count = defer_count + 1;
    char *next = scratch + 256;
    auto take = [&](size_t bytes) {
        char *q = next;
        next += (bytes + 255) & ~size_t(255);
        return q;
    };
    uint32_t *fail_flag = radius ? reinterpret_cast<uint32_t *>(take(per)) : nullptr;
    uint32_t *fail_list = radius ? reinterpret_cast<uint32_t *>(take(per)) : nullptr;
    void *list_scratch = radius ? take(failed_list_scratch_bytes(n)) : nullptr;
    uint32_t *defer_list = capped ? reinterpret_cast<uint32_t *>(take(per)) : nullptr;
    float *defer_radius = capped ? reinterpret_cast<float *>(take(per)) : nullptr;
    cudaError_t e = cudaMemsetAsync(scratch, 0, 256, st);
    if (e == cudaSuccess && radius)  // a deferred query's flag is written by the second pass
        e = cudaMemsetAsync(fail_flag, 0, 4 * (size_t)n, st);
    if (e == cudaSuccess)
        e = batch_view(s, pts, n, st, b, query_mesh);
    SeedArgs s1;
    s1.radius = radius;
    s1.fail_flag = fail_flag;
    if (capped)
    {
        s1.cap = (uint32_t)s->tail_cap;
        s1.defer_list = defer_list;
        s1.defer_count = defer_count;
        s1.defer_radius = defer_radius;
    }
    if (e == cudaSuccess)
        e = launch(b.t, s1);
    if (e == cudaSuccess && capped)
    {
        TreeView t2 = b.t;
        t2.order = defer_list;
        t2.order_count = defer_count;
        t2.order_coherent = 0;
        SeedArgs s2;
        s2.radius = defer_radius;
        s2.fail_flag = fail_flag;
        e = launch(t2, s2);
    }
    if (e == cudaSuccess && radius)
    {
        // The fallback pass runs the failed queries in the batch's own (Morton)
        // order. Failures that cluster (a few percent of a batch, e.g. points
        // far inside a closed mesh) keep neighbouring queries in a warp and run
        // as warp packets; sparse ones (a fraction of a percent spread over the
        // batch) run one search per lane, where packets lose. The fraction is
        // the previous seeded call's of this kind (the current one is known
        // only on the device).
        e = launch_failed_list(b.t.order, fail_flag, n, fail_list, fail_count, list_scratch, b.t.status, st);
        TreeView t3 = b.t;
        t3.order = fail_list;
        t3.order_count = fail_count;
        refresh_fallback_frac(s, kind);
        if (s->fallback_frac[kind] < kPacketFallbackMinFrac)
            t3.order_coherent = 0;
        if (e == cudaSuccess)
            e = launch(t3, SeedArgs());
        if (e == cudaSuccess)
            e = queue_fallback_count(s, kind, fail_count, n, st);
    }
    if (e == cudaSuccess && num_fallback)
        e = cudaMemcpyAsync(num_fallback, fail_count, 4, cudaMemcpyDeviceToDevice, st);
    cudaFreeAsync(scratch, st);
    SNCH_CUDA(e);
    return SNCH_OK;
}

// ---- learned search radius
struct MlpState
{
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
    uint32_t *status = nullptr;
    float center[3], inv_half[3];
    int step = 0;
};

uint64_t splitmix64(uint64_t &x)
{
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// He-uniform weights for the ReLU layers, a small head, zero biases, head bias log(0.05)
std::vector<float> mlp_init_params(uint64_t seed)
{
    const int in[5] = {192, 64, 64, 64, 64}, out[5] = {64, 64, 64, 64, 2};
    std::vector<float> p;
    uint64_t st = seed;
    for (int l = 0; l < 5; ++l)
    {
        const float bound = l < 4 ? std::sqrt(6.0f / in[l]) : 0.1f * std::sqrt(3.0f / in[l]);
        for (int i = 0; i < in[l] * out[l]; ++i)
        {
            const double u = (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0);
            p.push_back((float)((2.0 * u - 1.0) * bound));
        }
        for (int i = 0; i < out[l]; ++i)
            p.push_back(l < 4 ? 0.0f : std::log(0.05f));
    }
    return p;
}

size_t mlp_workspace_bytes(int64_t rows)
{
    const size_t r = (size_t)rows;
    return r * 192 * 2 + 8 * r * 64 * 2 + 256 * r * 2 + 64 * r * 2 + 64 * 64 * 2 + (64 * 192 + 3 * 4096) * 2 +
           2 * r * 64 * 4 + 64 * 256 * 64 * 4 + 16 * 256;
}

MlpWorkspace mlp_workspace(char *base, int64_t rows)
{
    MlpWorkspace w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = base + off;
        off += (bytes + 255) & ~size_t(255);
        return p;
    };
    const size_t r = (size_t)rows;
    w.X = take(r * 192 * 2);
    for (int l = 0; l < 4; ++l)
        w.H[l] = take(r * 64 * 2);
    for (int l = 0; l < 4; ++l)
        w.dZ[l] = take(r * 64 * 2);
    w.T = take(256 * r * 2);
    w.T2 = take(64 * r * 2);
    w.Wt = take(64 * 64 * 2);
    w.Wb = take((64 * 192 + 3 * 4096) * 2);
    w.Z = reinterpret_cast<float *>(take(r * 64 * 4));
    w.dH = reinterpret_cast<float *>(take(r * 64 * 4));
    w.C = reinterpret_cast<float *>(take(64 * 256 * 64 * 4));  // up to 64 split-K slices
    return w;
}

// ---- host-form pipeline: chunk i runs on pipe[i % 2]: H2D inputs, kernel, D2H outputs.
// The searches wait for an event recorded on the legacy default stream at the
// start of the call (so a build queued there with a NULL stream is complete);
// the input copies do not, so they overlap that build.
int ensure_stage(snch_scene_s *s, size_t in_bytes, size_t out_bytes)
{
    for (int k = 0; k < 2; ++k)
        if (!s->pipe[k])
            SNCH_CUDA(cudaStreamCreateWithFlags(&s->pipe[k], cudaStreamNonBlocking));
    if (!s->pipe_ready)
        SNCH_CUDA(cudaEventCreateWithFlags(&s->pipe_ready, cudaEventDisableTiming));
    if (in_bytes <= s->stage.in_bytes && out_bytes <= s->stage.out_bytes)
        return SNCH_OK;
    // a call that failed part-way may have left copies queued on the stage
    for (int k = 0; k < 2; ++k)
        SNCH_CUDA(cudaStreamSynchronize(s->pipe[k]));
    if (in_bytes > s->stage.in_bytes)
    {
        for (int k = 0; k < 2; ++k)
        {
            cache_release(s->stage.in[k]);
            s->stage.in[k] = nullptr;
        }
        s->stage.in_bytes = 0;
        for (int k = 0; k < 2; ++k)
            SNCH_CUDA(cache_alloc(&s->stage.in[k], in_bytes));
        s->stage.in_bytes = in_bytes;
    }
    if (out_bytes > s->stage.out_bytes)
    {
        for (int k = 0; k < 2; ++k)
        {
            cache_release(s->stage.out[k]);
            s->stage.out[k] = nullptr;
        }
        s->stage.out_bytes = 0;
        for (int k = 0; k < 2; ++k)
            SNCH_CUDA(cache_alloc(&s->stage.out[k], out_bytes));
        s->stage.out_bytes = out_bytes;
    }
    return SNCH_OK;
}

struct Field
{
    const void *host_in;
    void *host_out;
    size_t elem;  // bytes per query
};

// Runs `body(chunk_begin, count, dev_in[], dev_out[], stream)` over chunks.
template <typename Body>
int run_host_pipeline(snch_scene_s *s, int64_t n, int64_t auto_chunk, const Field *ins, int nin, const Field *outs,
                      int nout, Body body)
{
    if (n == 0)
        return SNCH_OK;
    size_t in_per = 0, out_per = 0;
    for (int i = 0; i < nin; ++i)
        in_per += ins[i].elem;
    for (int i = 0; i < nout; ++i)
        out_per += outs[i].elem;
    const int64_t chunk = std::min<int64_t>(n, s->host_chunk > 0 ? s->host_chunk : auto_chunk);
    int rc = ensure_stage(s, in_per * chunk + 256 * nin, out_per * chunk + 256 * nout);
    if (rc != SNCH_OK)
        return rc;
    SNCH_CUDA(cudaEventRecord(s->pipe_ready, cudaStreamLegacy));
    // Every chunk is queued before the first wait. The pipe streams do not
    // synchronise with the legacy default stream, so a call that fails part-way
    // still waits for the chunks it queued: they read the tree and the stage,
    // which a later NULL-stream build of this scene or the next call overwrites.
    const int queued = [&]() -> int {
        for (int64_t b = 0, c = 0; b < n; b += chunk, ++c)
        {
            const int64_t m = std::min<int64_t>(chunk, n - b);
            const int k = (int)(c & 1);
            cudaStream_t st = s->pipe[k];
            char *din = static_cast<char *>(s->stage.in[k]);
            char *dout = static_cast<char *>(s->stage.out[k]);
            void *dev_in[4], *dev_out[4];
            size_t off = 0;
            for (int i = 0; i < nin; ++i)
            {
                dev_in[i] = din + off;
                if (ins[i].host_in)
                    SNCH_CUDA(cudaMemcpyAsync(din + off, static_cast<const char *>(ins[i].host_in) + b * ins[i].elem,
                                              m * ins[i].elem, cudaMemcpyHostToDevice, st));
                else
                    dev_in[i] = nullptr;
                off += (ins[i].elem * chunk + 255) & ~size_t(255);
            }
            off = 0;
            for (int i = 0; i < nout; ++i)
            {
                dev_out[i] = outs[i].host_out ? dout + off : nullptr;
                off += (outs[i].elem * chunk + 255) & ~size_t(255);
            }
            SNCH_CUDA(cudaStreamWaitEvent(st, s->pipe_ready, 0));
            SNCH_CUDA(body(m, dev_in, dev_out, st));
            for (int i = 0; i < nout; ++i)
                if (outs[i].host_out)
                    SNCH_CUDA(cudaMemcpyAsync(static_cast<char *>(outs[i].host_out) + b * outs[i].elem, dev_out[i],
                                              m * outs[i].elem, cudaMemcpyDeviceToHost, st));
        }
        return SNCH_OK;
    }();
    const cudaError_t e0 = cudaStreamSynchronize(s->pipe[0]);
    const cudaError_t e1 = cudaStreamSynchronize(s->pipe[1]);
    if (queued != SNCH_OK)
        return queued;
    SNCH_CUDA(e0);
    SNCH_CUDA(e1);
    return SNCH_OK;
}

}  // namespace

extern "C" {

const char *snch_version(void) { return "snch_gb300 0.1 (sm_103a)"; }

const char *snch_last_error(void) { return g_error.c_str(); }

int64_t snch_cached_memory_bytes(void)
{
    BlockCache &c = block_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    return (int64_t)c.cached_bytes;
}

int snch_release_cached_memory(void)
{
    BlockCache &c = block_cache();
    {
        std::lock_guard<std::mutex> lock(c.mu);
        cache_trim_locked(c);
    }
    cudaDeviceSynchronize();
    trim_pools();
    return SNCH_OK;
}

uint64_t snch_kernel_launch_count(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

int snch_scene_create(const float *v, int64_t nv, const int32_t *t, int64_t nt, snch_scene_t *out)
{
    return create_common(v, nv, t, nt, out, false, nullptr);
}

int snch_scene_create_device(const float *v, int64_t nv, const int32_t *t, int64_t nt, snch_scene_t *out,
                             snch_stream_t stream)
{
    return create_common(v, nv, t, nt, out, true, S(stream));
}

int snch_scene_destroy(snch_scene_t s)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    free_scene(s);
    return SNCH_OK;
}

int snch_compute_silhouettes(snch_scene_t s, snch_stream_t stream)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    s->built = false;
    return topology(s, S(stream));
}

int snch_build_bvh(snch_scene_t s, snch_stream_t stream)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    cudaStream_t st = S(stream);
    if (!s->topology_ready)
    {
        int rc = topology(s, st);
        if (rc != SNCH_OK)
            return rc;
    }
    if (s->num_tris > 0)
    {
        BuildArgs a = build_args(s);
        SNCH_CUDA(launch_build_front(a, st));
        SNCH_CUDA(radix_sort_pairs(s->keys, s->vals, s->keys_tmp, s->vals_tmp, s->num_tris, 30, s->small + kWHist,
                                   s->scratch, s->small + kWStatus, st));
        SNCH_CUDA(launch_mesh_pass(a, s->scratch, st));  // batched scenes only
        SNCH_CUDA(launch_build_back(a, st));
        SNCH_CUDA(launch_ref_objects(s->verts, s->tris, s->tri_owned, s->edge_verts, s->num_tris, s->ref_objects,
                                     s->ref_edges, st));
        if (s->num_meshes == 0)
            SNCH_CUDA(launch_top_levels(s->inner, s->inner_cones, s->num_tris, kTopSlots, s->top_inner,
                                        s->top_cones, st));
    }
    s->wide_ready[0] = s->wide_ready[1] = false;
    s->built = true;
    return ensure_widths(s, st);
}

int snch_set_traversal(snch_scene_t s, int mode)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (mode != SNCH_TRAVERSAL_NEAR_FIRST && mode != SNCH_TRAVERSAL_REFERENCE_ORDER)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "unknown traversal mode " + std::to_string(mode));
    s->traversal = mode;
    return SNCH_OK;
}

int snch_set_option(snch_scene_t s, int option, int64_t value)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    switch (option)
    {
    case SNCH_OPT_TRAVERSAL:
        return snch_set_traversal(s, (int)value);
    case SNCH_OPT_QUERY_ORDER:
        if (value != 0 && value != 1)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_QUERY_ORDER takes 0 or 1");
        s->query_order = (int)value;
        return SNCH_OK;
    case SNCH_OPT_ORDER_MIN_BATCH:
        if (value < 0)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_ORDER_MIN_BATCH must be >= 0");
        s->order_min = value;
        return SNCH_OK;
    case SNCH_OPT_TOP_LEVELS:
        if (value < 0 || value > 7)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_TOP_LEVELS must be in [0, 7]");
        s->top_levels = (int)value;
        return SNCH_OK;
    case SNCH_OPT_ORDER_BITS:
        if (value < 12 || value > 30)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_ORDER_BITS must be in [12, 30]");
        s->order_bits = (int)value;
        return SNCH_OK;
    case SNCH_OPT_RAY_ORDER:
        if (value != 0 && value != 1)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_RAY_ORDER takes 0 or 1");
        s->ray_order = (int)value;
        return SNCH_OK;
    case SNCH_OPT_OUTPUT_SCATTER:
        if (value != 0 && value != 1)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_OUTPUT_SCATTER takes 0 or 1");
        s->output_scatter = (int)value;
        return SNCH_OK;
    case SNCH_OPT_PACKET_PERSISTENT_MIN:
        if (value < 1)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_PACKET_PERSISTENT_MIN must be >= 1");
        s->packet_persistent_min = value;
        return SNCH_OK;
    case SNCH_OPT_PERSISTENT_RAY:
        if (value != 0 && value != 1)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_PERSISTENT_RAY takes 0 or 1");
        s->persistent_ray = (int)value;
        return SNCH_OK;
    case SNCH_OPT_HOST_CHUNK:
        if (value != 0 && (value < 1024 || value >= (int64_t(1) << 30)))
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_HOST_CHUNK must be 0 or in [1024, 2^30)");
        s->host_chunk = value;
        return SNCH_OK;
    case SNCH_OPT_TAIL_CAP:
        if (value < 0 || value > (int64_t(1) << 30))
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_TAIL_CAP must be in [0, 2^30]");
        s->tail_cap = value;
        return SNCH_OK;
    case SNCH_OPT_PERSISTENT:
    case SNCH_OPT_PERSISTENT_NEAREST:
    case SNCH_OPT_PERSISTENT_SILHOUETTE:
        if (value != 0 && value != 1)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_PERSISTENT takes 0 or 1");
        if (option != SNCH_OPT_PERSISTENT_SILHOUETTE)
            s->persistent_near = (int)value;
        if (option != SNCH_OPT_PERSISTENT_NEAREST)
            s->persistent_sil = (int)value;
        return SNCH_OK;
    case SNCH_OPT_PACKET:
    case SNCH_OPT_PACKET_NEAREST:
    case SNCH_OPT_PACKET_SILHOUETTE:
        if (value < 0 || value > 2)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "SNCH_OPT_PACKET takes 0, 1 or 2");
        if (option != SNCH_OPT_PACKET_SILHOUETTE)
            s->packet_near = (int)value;
        if (option != SNCH_OPT_PACKET_NEAREST)
            s->packet_sil = (int)value;
        return SNCH_OK;
    case SNCH_OPT_BLOCK:
    case SNCH_OPT_BLOCK_NEAREST:
    case SNCH_OPT_BLOCK_SILHOUETTE:
        if (value != 64 && value != 128 && value != 256)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "block size must be 64, 128 or 256");
        if (option != SNCH_OPT_BLOCK_SILHOUETTE)
            s->block_near = (int)value;
        if (option != SNCH_OPT_BLOCK_NEAREST)
            s->block_sil = (int)value;
        return SNCH_OK;
    case SNCH_OPT_NODE_WIDTH:
    case SNCH_OPT_NODE_WIDTH_NEAREST:
    case SNCH_OPT_NODE_WIDTH_SILHOUETTE:
    {
        if (value != 2 && value != 4 && value != 8)
            return fail(SNCH_ERR_INVALID_ARGUMENT, "node width must be 2, 4 or 8");
        if (option != SNCH_OPT_NODE_WIDTH_SILHOUETTE)
            s->width_near = (int)value;
        if (option != SNCH_OPT_NODE_WIDTH_NEAREST)
            s->width_sil = (int)value;
        if (value > 2)
        {
            int rc = alloc_wide(s, (int)value);
            if (rc != SNCH_OK)
                return rc;
        }
        if (!s->built)
            return SNCH_OK;
        int rc = ensure_widths(s, nullptr);
        if (rc == SNCH_OK)
            SNCH_CUDA(cudaStreamSynchronize(nullptr));
        return rc;
    }
    default:
        return fail(SNCH_ERR_INVALID_ARGUMENT, "unknown option " + std::to_string(option));
    }
}

int snch_export_leaf_ranks(snch_scene_t s, uint32_t *ranks)
{
    int rc = check_built(s);
    if (rc != SNCH_OK)
        return rc;
    if (!ranks && s->num_tris)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "ranks is NULL");
    if (s->num_tris)
        SNCH_CUDA(cudaMemcpy2D(ranks, 4, reinterpret_cast<const char *>(s->leaves) + 44, sizeof(LeafRec), 4,
                               s->num_tris, cudaMemcpyDeviceToHost));
    return SNCH_OK;
}

int snch_get_bvh_view(snch_scene_t s, snch_bvh_view *out)
{
    int rc = check_built(s);
    if (rc != SNCH_OK)
        return rc;
    if (!out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "out_view is NULL");
    out->num_nodes = s->num_tris ? 2 * s->num_tris - 1 : 0;
    out->num_objects = s->num_tris;
    out->nodes = reinterpret_cast<const snch_node *>(s->nodes);
    out->aabbs = reinterpret_cast<const snch_aabb *>(s->aabbs);
    out->cones = reinterpret_cast<const snch_cone *>(s->cones);
    out->objects = s->ref_objects;
    return SNCH_OK;
}

int snch_get_traversal_view(snch_scene_t s, snch_traversal_view *out)
{
    int rc = check_built(s);
    if (rc != SNCH_OK)
        return rc;
    if (!out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "out_view is NULL");
    if (s->num_meshes > 0)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "snch_get_traversal_view serves plain scenes, not batched ones");
    *out = snch_traversal_view{};
    out->num_triangles = s->num_tris;
    out->root_box = reinterpret_cast<const float *>(s->aabbs);
    out->inner = s->inner;
    out->inner_cones = s->inner_cones;
    out->leaves = s->leaves;
    out->edges = s->edges;
    out->vertices = s->verts;
    out->triangles = s->tris;
    out->status = s->small + kWStatus;
    return SNCH_OK;
}

int snch_scene_info(snch_scene_t s, int64_t *nv, int64_t *nt, int64_t *ne)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (nv)
        *nv = s->num_verts;
    if (nt)
        *nt = s->num_tris;
    if (ne)
    {
        if (!s->topology_ready)
            *ne = -1;
        else
        {
            if (s->num_edges_host < 0)
            {
                uint32_t e = 0;
                SNCH_CUDA(cudaMemcpy(&e, s->small + kWNumEdges, 4, cudaMemcpyDeviceToHost));
                s->num_edges_host = e;
            }
            *ne = s->num_edges_host;
        }
    }
    return SNCH_OK;
}

int snch_get_device_status(snch_scene_t s, uint32_t *out, int reset, snch_stream_t stream)
{
    if (!s || !out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaStream_t st = S(stream);
    SNCH_CUDA(cudaMemcpyAsync(out, s->small + kWStatus, 4, cudaMemcpyDeviceToHost, st));
    if (reset)
        SNCH_CUDA(cudaMemsetAsync(s->small + kWStatus, 0, 4, st));
    SNCH_CUDA(cudaStreamSynchronize(st));
    return SNCH_OK;
}

int snch_export_tree(snch_scene_t s, uint32_t *morton, uint32_t *sidx, uint32_t *nodes, float *aabbs, float *cones,
                     snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc != SNCH_OK)
        return rc;
    cudaStream_t st = S(stream);
    const size_t n = s->num_tris, nn = n ? 2 * n - 1 : 0;
    if (morton && n)
        SNCH_CUDA(cudaMemcpyAsync(morton, s->keys, 4 * n, cudaMemcpyDeviceToDevice, st));
    if (sidx && n)
        SNCH_CUDA(cudaMemcpyAsync(sidx, s->vals, 4 * n, cudaMemcpyDeviceToDevice, st));
    if (nodes && nn)
        SNCH_CUDA(cudaMemcpyAsync(nodes, s->nodes, 16 * nn, cudaMemcpyDeviceToDevice, st));
    if (aabbs && nn)
        SNCH_CUDA(cudaMemcpyAsync(aabbs, s->aabbs, 24 * nn, cudaMemcpyDeviceToDevice, st));
    if (cones && nn)
        SNCH_CUDA(cudaMemcpyAsync(cones, s->cones, 20 * nn, cudaMemcpyDeviceToDevice, st));
    return SNCH_OK;
}

int snch_export_topology(snch_scene_t s, int32_t *tri_edges, int32_t *tri_owned, int32_t *edge_verts,
                         snch_stream_t stream)
{
    if (!s)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (!s->topology_ready)
        return fail(SNCH_ERR_NOT_BUILT, "silhouettes are not computed yet");
    int64_t ne = 0;
    int rc = snch_scene_info(s, nullptr, nullptr, &ne);
    if (rc != SNCH_OK)
        return rc;
    cudaStream_t st = S(stream);
    const size_t n = s->num_tris;
    if (tri_edges && n)
        SNCH_CUDA(cudaMemcpyAsync(tri_edges, s->tri_edges, 12 * n, cudaMemcpyDeviceToDevice, st));
    if (tri_owned && n)
        SNCH_CUDA(cudaMemcpyAsync(tri_owned, s->tri_owned, 12 * n, cudaMemcpyDeviceToDevice, st));
    if (edge_verts && ne)
        SNCH_CUDA(cudaMemcpyAsync(edge_verts, s->edge_verts, 16 * (size_t)ne, cudaMemcpyDeviceToDevice, st));
    return SNCH_OK;
}


int snch_query_nearest(snch_scene_t s, const float *pts, int64_t n, uint32_t *idx, float *dist, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, idx, dist});
    if (rc != SNCH_OK)
        return rc;
    if (n == 0)
        return SNCH_OK;
    return run_query(s, 0, pts, nullptr, n, nullptr, S(stream), [&](const TreeView &t, const SeedArgs &seed) {
        return launch_nearest(t, pts, n, idx, dist, S(stream), nullptr, seed);
    });
}

int snch_query_silhouette(snch_scene_t s, const float *pts, const uint8_t *flip, int64_t n, float *dist, int32_t *edge,
                          snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, dist});
    if (rc != SNCH_OK)
        return rc;
    if (n == 0)
        return SNCH_OK;
    return run_query(s, 1, pts, nullptr, n, nullptr, S(stream), [&](const TreeView &t, const SeedArgs &seed) {
        return launch_silhouette(t, pts, flip, n, dist, edge, S(stream), nullptr, seed);
    });
}

int snch_query_overlap(snch_scene_t s, const float *boxes, int64_t n, uint32_t max_per_query, uint32_t *out_index,
                       uint32_t *out_count, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {boxes, out_count});
    if (rc == SNCH_OK && max_per_query > 0 && n > 0 && !out_index)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "out_index is NULL");
    if (rc == SNCH_OK && s->num_meshes)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "enumeration queries take a plain scene");
    if (rc != SNCH_OK || n == 0)
        return rc;
    SNCH_CUDA(launch_enumerate(s->view(), false, boxes, nullptr, n, max_per_query, out_index, nullptr, out_count,
                               S(stream)));
    return SNCH_OK;
}

int snch_query_line(snch_scene_t s, const float *origins, const float *dirs, int64_t n, uint32_t max_per_query,
                    uint32_t *out_index, float *out_t, uint32_t *out_count, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {origins, dirs, out_count});
    if (rc == SNCH_OK && max_per_query > 0 && n > 0 && (!out_index || !out_t))
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "out_index / out_t is NULL");
    if (rc == SNCH_OK && s->num_meshes)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "enumeration queries take a plain scene");
    if (rc != SNCH_OK || n == 0)
        return rc;
    SNCH_CUDA(launch_enumerate(s->view(), true, origins, dirs, n, max_per_query, out_index, out_t, out_count,
                               S(stream)));
    return SNCH_OK;
}

int snch_query_ray(snch_scene_t s, const float *o, const float *d, const float *tmax, int64_t n, uint8_t *hit, float *t,
                   float *uv, uint32_t *idx, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {o, d, tmax, hit, t, uv, idx});
    if (rc != SNCH_OK)
        return rc;
    BatchView b;
    SNCH_CUDA(batch_view(s, o, n, S(stream), b, nullptr, tmax));
    SNCH_CUDA(launch_ray(b.t, o, d, tmax, n, hit, t, uv, idx, S(stream)));
    return SNCH_OK;
}

int snch_query_ray_test(snch_scene_t s, const float *o, const float *d, const float *tmax, int64_t n, uint8_t *hit,
                        snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {o, d, tmax, hit});
    if (rc != SNCH_OK)
        return rc;
    BatchView b;
    SNCH_CUDA(batch_view(s, o, n, S(stream), b, nullptr, tmax));
    SNCH_CUDA(launch_ray_test(b.t, o, d, tmax, n, hit, S(stream)));
    return SNCH_OK;
}

int snch_sample_in_sphere(snch_scene_t s, const float *c, const float *r, const float *u, int64_t n, int32_t *idx,
                          float *pdf, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {c, r, u, idx, pdf});
    if (rc != SNCH_OK)
        return rc;
    // sphere draws run in input order: a draw is one short descent, and the
    // Morton sort costs more than the coherence it gives (4M draws on the
    // 2M-triangle scene: 0.77 ms unordered, 0.93 ms sorted first)
    BatchView b;
    SNCH_CUDA(batch_view(s, c, n, S(stream), b, nullptr, nullptr, false));
    SNCH_CUDA(launch_sample(b.t, c, r, u, n, idx, pdf, S(stream)));
    return SNCH_OK;
}

int snch_sample_on_object(snch_scene_t s, const int32_t *idx, const float *u, const float *v, int64_t n, float *pts,
                          snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {idx, u, v, pts});
    if (rc != SNCH_OK)
        return rc;
    if (n > 0 && s->num_tris == 0)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "sample_on_object on an empty scene");
    SNCH_CUDA(launch_validate(idx, n, s->num_tris, s->small + kWBad, S(stream)));
    uint32_t bad = 0;
    SNCH_CUDA(cudaMemcpyAsync(&bad, s->small + kWBad, 4, cudaMemcpyDeviceToHost, S(stream)));
    SNCH_CUDA(cudaStreamSynchronize(S(stream)));
    if (bad)
        return fail(SNCH_ERR_INVALID_ARGUMENT, std::to_string(bad) + " object indices out of range");
    SNCH_CUDA(launch_sample_point(s->verts, s->tris, s->num_tris, idx, u, v, n, pts, S(stream)));
    return SNCH_OK;
}

int snch_query_nearest_host(snch_scene_t s, const float *pts, int64_t n, uint32_t *idx, float *dist)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, idx, dist});
    if (rc != SNCH_OK)
        return rc;
    const Field ins[] = {{pts, nullptr, 12}};
    const Field outs[] = {{nullptr, idx, 4}, {nullptr, dist, 4}};
    return run_host_pipeline(s, n, kHostChunkSearch, ins, 1, outs, 2,
                             [&](int64_t m, void **di, void **dout, cudaStream_t st) {
        BatchView b;
        cudaError_t e = batch_view(s, (const float *)di[0], m, st, b);
        return e != cudaSuccess ? e : launch_nearest(b.t, (const float *)di[0], m, (uint32_t *)dout[0],
                                                     (float *)dout[1], st);
    });
}

int snch_query_silhouette_host(snch_scene_t s, const float *pts, const uint8_t *flip, int64_t n, float *dist,
                               int32_t *edge)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, dist});
    if (rc != SNCH_OK)
        return rc;
    const Field ins[] = {{pts, nullptr, 12}, {flip, nullptr, 1}};
    const Field outs[] = {{nullptr, dist, 4}, {nullptr, edge, 4}};
    return run_host_pipeline(s, n, kHostChunkSearch, ins, 2, outs, 2,
                             [&](int64_t m, void **di, void **dout, cudaStream_t st) {
        BatchView b;
        cudaError_t e = batch_view(s, (const float *)di[0], m, st, b);
        return e != cudaSuccess ? e : launch_silhouette(b.t, (const float *)di[0], (const uint8_t *)di[1], m,
                                                        (float *)dout[0], (int32_t *)dout[1], st);
    });
}

int snch_query_ray_host(snch_scene_t s, const float *o, const float *d, const float *tmax, int64_t n, uint8_t *hit,
                        float *t, float *uv, uint32_t *idx)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {o, d, tmax, hit, t, uv, idx});
    if (rc != SNCH_OK)
        return rc;
    const Field ins[] = {{o, nullptr, 12}, {d, nullptr, 12}, {tmax, nullptr, 4}};
    const Field outs[] = {{nullptr, hit, 1}, {nullptr, t, 4}, {nullptr, uv, 8}, {nullptr, idx, 4}};
    return run_host_pipeline(s, n, kHostChunkRay, ins, 3, outs, 4,
                             [&](int64_t m, void **di, void **dout, cudaStream_t st) {
        BatchView b;
        cudaError_t e = batch_view(s, (const float *)di[0], m, st, b, nullptr, (const float *)di[2]);
        return e != cudaSuccess ? e
                                : launch_ray(b.t, (const float *)di[0], (const float *)di[1], (const float *)di[2], m,
                                             (uint8_t *)dout[0], (float *)dout[1], (float *)dout[2],
                                             (uint32_t *)dout[3], st);
    });
}

int snch_sample_in_sphere_host(snch_scene_t s, const float *c, const float *r, const float *u, int64_t n, int32_t *idx,
                               float *pdf)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {c, r, u, idx, pdf});
    if (rc != SNCH_OK)
        return rc;
    const Field ins[] = {{c, nullptr, 12}, {r, nullptr, 4}, {u, nullptr, 4}};
    const Field outs[] = {{nullptr, idx, 4}, {nullptr, pdf, 4}};
    return run_host_pipeline(s, n, kHostChunkRay, ins, 3, outs, 2,
                             [&](int64_t m, void **di, void **dout, cudaStream_t st) {
        BatchView b;
        cudaError_t e = batch_view(s, (const float *)di[0], m, st, b, nullptr, nullptr, false);
        return e != cudaSuccess ? e : launch_sample(b.t, (const float *)di[0], (const float *)di[1],
                                                    (const float *)di[2], m, (int32_t *)dout[0], (float *)dout[1], st);
    });
}

int snch_query_nearest_seeded(snch_scene_t s, const float *pts, const float *radius, int64_t n, uint32_t *idx,
                              float *dist, uint32_t *num_fallback, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, radius, idx, dist});
    if (rc != SNCH_OK || n == 0)
        return rc;
    return run_query(s, 0, pts, radius, n, num_fallback, S(stream), [&](const TreeView &t, const SeedArgs &seed) {
        return launch_nearest(t, pts, n, idx, dist, S(stream), nullptr, seed);
    });
}

int snch_query_silhouette_seeded(snch_scene_t s, const float *pts, const uint8_t *flip, const float *radius, int64_t n,
                                 float *dist, int32_t *edge, uint32_t *num_fallback, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, radius, dist});
    if (rc != SNCH_OK || n == 0)
        return rc;
    return run_query(s, 1, pts, radius, n, num_fallback, S(stream), [&](const TreeView &t, const SeedArgs &seed) {
        return launch_silhouette(t, pts, flip, n, dist, edge, S(stream), nullptr, seed);
    });
}

int snch_query_visits(snch_scene_t s, int kind, const float *in0, const float *in1, const float *in2,
                      const uint8_t *flip, int64_t n, uint32_t *visits, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {in0, visits});
    if (rc != SNCH_OK)
        return rc;
    if (n == 0)
        return SNCH_OK;
    if ((kind == 2 || kind == 3) && (!in1 || !in2))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL query buffer");
    cudaStream_t st = S(stream);
    // result buffers of the counted launch (discarded)
    char *scratch = nullptr;
    SNCH_CUDA(scratch_alloc(&scratch, 32 * (size_t)n + 256, st));
    // nearest / silhouette batches are counted in the order a query call runs them
    // (Morton-ordered above the ordering threshold, which selects the packet form)
    BatchView b;
    cudaError_t e = kind <= 1 ? batch_view(s, in0, n, st, b) : cudaSuccess;
    if (e != cudaSuccess)
    {
        cudaFreeAsync(scratch, st);
        SNCH_CUDA(e);
    }
    const TreeView t = kind <= 1 ? b.t : s->view();
    switch (kind)
    {
    case 0:
        e = launch_nearest(t, in0, n, (uint32_t *)scratch, (float *)(scratch + 8 * n), st, visits);
        break;
    case 1:
        e = launch_silhouette(t, in0, flip, n, (float *)scratch, (int32_t *)(scratch + 8 * n), st, visits);
        break;
    case 2:
        e = launch_ray(t, in0, in1, in2, n, (uint8_t *)scratch, (float *)(scratch + 4 * n),
                       (float *)(scratch + 8 * n), (uint32_t *)(scratch + 16 * n), st, visits);
        break;
    case 3:
        e = launch_sample(t, in0, in1, in2, n, (int32_t *)scratch, (float *)(scratch + 8 * n), st, visits);
        break;
    default:
        cudaFreeAsync(scratch, st);
        return fail(SNCH_ERR_INVALID_ARGUMENT, "kind must be 0..3");
    }
    cudaFreeAsync(scratch, st);
    SNCH_CUDA(e);
    return SNCH_OK;
}

int snch_query_visits_seeded(snch_scene_t s, int kind, const float *pts, const uint8_t *flip, const float *radius,
                             int64_t n, uint32_t *visits, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n, {pts, radius, visits});
    if (rc != SNCH_OK)
        return rc;
    if (kind != 0 && kind != 1)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "kind must be 0 (nearest) or 1 (silhouette)");
    if (n == 0)
        return SNCH_OK;
    cudaStream_t st = S(stream);
    char *scratch = nullptr;
    SNCH_CUDA(scratch_alloc(&scratch, 8 * (size_t)n + 256, st));
    BatchView b;
    cudaError_t e = batch_view(s, pts, n, st, b);
    SeedArgs seed;
    seed.radius = radius;
    if (e == cudaSuccess)
        e = kind == 0 ? launch_nearest(b.t, pts, n, (uint32_t *)scratch, (float *)(scratch + 4 * n), st, visits, seed)
                      : launch_silhouette(b.t, pts, flip, n, (float *)scratch, (int32_t *)(scratch + 4 * n), st,
                                          visits, seed);
    cudaFreeAsync(scratch, st);
    SNCH_CUDA(e);
    return SNCH_OK;
}

size_t snch_sort_scratch_bytes(int64_t n, int key_bits)
{
    if (n <= 0 || n >= (int64_t(1) << 30) || key_bits < 1 || key_bits > 32)
        return 0;
    return sort_scratch_bytes((uint32_t)n, key_bits);
}

int snch_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_tmp, uint32_t *vals_tmp, int64_t n, int key_bits,
                    void *scratch, uint32_t *device_status, snch_stream_t stream)
{
    if (n < 0 || key_bits < 1 || key_bits > 32)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "n < 0 or key_bits outside [1, 32]");
    if (n >= (int64_t(1) << 30))
        return fail(SNCH_ERR_TOO_LARGE, "at most 2^30 - 1 pairs");
    if (n > 1 && (!keys || !vals || !keys_tmp || !vals_tmp || !scratch || !device_status))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL buffer");
    SNCH_CUDA(radix_sort_pairs(keys, vals, keys_tmp, vals_tmp, (uint32_t)n, key_bits, nullptr, scratch, device_status,
                               S(stream)));
    return SNCH_OK;
}

// ------------------------------------------------------------------ learned search radius
struct snch_mlp_s
{
    MlpState st;
};

int64_t snch_mlp_num_params(void) { return (int64_t)mlp_num_params(); }

int snch_mlp_create(const float *lo, const float *hi, uint64_t seed, snch_mlp_t *out)
{
    if (!lo || !hi || !out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    float scales[32];
    for (int k = 0; k < 32; ++k)
        scales[k] = (float)std::exp2(0.25 * k);
    SNCH_CUDA(set_mlp_scales(scales));
    auto *m = new snch_mlp_s();
    for (int c = 0; c < 3; ++c)
    {
        if (!(hi[c] > lo[c]))
        {
            delete m;
            return fail(SNCH_ERR_INVALID_ARGUMENT, "empty box");
        }
        m->st.center[c] = 0.5f * (lo[c] + hi[c]);
        m->st.inv_half[c] = 2.0f / (hi[c] - lo[c]);
    }
    const size_t np = mlp_num_params();
    const std::vector<float> p = mlp_init_params(seed);
    cudaError_t e = cudaMalloc(&m->st.params, 4 * np);
    if (e == cudaSuccess)
        e = cudaMalloc(&m->st.grad, 4 * np);
    if (e == cudaSuccess)
        e = cudaMalloc(&m->st.m, 4 * np);
    if (e == cudaSuccess)
        e = cudaMalloc(&m->st.v, 4 * np);
    if (e == cudaSuccess)
        e = cudaMalloc(&m->st.loss, 256);
    if (e == cudaSuccess)
        e = cudaMalloc(&m->st.status, 256);
    if (e == cudaSuccess)
        e = cudaMemcpy(m->st.params, p.data(), 4 * np, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemset(m->st.m, 0, 4 * np);
    if (e == cudaSuccess)
        e = cudaMemset(m->st.v, 0, 4 * np);
    if (e == cudaSuccess)
        e = cudaMemset(m->st.status, 0, 4);
    if (e != cudaSuccess)
    {
        snch_mlp_destroy(m);
        return fail(SNCH_ERR_CUDA, std::string("snch_mlp_create: ") + cudaGetErrorString(e));
    }
    *out = m;
    return SNCH_OK;
}

int snch_mlp_destroy(snch_mlp_t m)
{
    if (!m)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "mlp is NULL");
    for (void *p : {(void *)m->st.params, (void *)m->st.grad, (void *)m->st.m, (void *)m->st.v, (void *)m->st.loss,
                    (void *)m->st.status})
        if (p)
            cudaFree(p);
    delete m;
    return SNCH_OK;
}

int snch_mlp_get_params(snch_mlp_t m, float *host, int64_t count)
{
    if (!m || !host || count != (int64_t)mlp_num_params())
        return fail(SNCH_ERR_INVALID_ARGUMENT, "need snch_mlp_num_params() floats");
    SNCH_CUDA(cudaMemcpy(host, m->st.params, 4 * (size_t)count, cudaMemcpyDeviceToHost));
    return SNCH_OK;
}

int snch_mlp_set_params(snch_mlp_t m, const float *host, int64_t count)
{
    if (!m || !host || count != (int64_t)mlp_num_params())
        return fail(SNCH_ERR_INVALID_ARGUMENT, "need snch_mlp_num_params() floats");
    SNCH_CUDA(cudaMemcpy(m->st.params, host, 4 * (size_t)count, cudaMemcpyHostToDevice));
    return SNCH_OK;
}

int snch_mlp_gradient(snch_mlp_t m, const float *pts, const float *targets, int64_t n, float tau, float *host_grad,
                      float *host_loss, snch_stream_t stream)
{
    if (!m || !pts || !targets || n <= 0 || n > (int64_t(1) << 24))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "bad arguments");
    cudaStream_t st = S(stream);
    const int64_t rows = (n + 127) / 128 * 128;
    char *ws = nullptr;
    SNCH_CUDA(scratch_alloc(&ws, mlp_workspace_bytes(rows), st));
    cudaError_t e = mlp_forward_backward(m->st.params, m->st.grad, pts, targets, n, rows, m->st.center,
                                         m->st.inv_half, tau, mlp_workspace(ws, rows), m->st.loss, m->st.status, st);
    if (e == cudaSuccess && host_grad)
        e = cudaMemcpyAsync(host_grad, m->st.grad, 4 * mlp_num_params(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && host_loss)
        e = cudaMemcpyAsync(host_loss, m->st.loss, 4, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(ws, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    SNCH_CUDA(e);
    return SNCH_OK;
}

int snch_mlp_train(snch_mlp_t m, const float *pts, const float *targets, int64_t n, int epochs, int64_t batch,
                   float lr, float tau, float *host_loss, snch_stream_t stream)
{
    if (!m || !pts || !targets || n <= 0 || epochs < 0 || batch < 128 || batch > (int64_t(1) << 20))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "bad arguments");
    cudaStream_t st = S(stream);
    const int64_t rows_max = (batch + 127) / 128 * 128;
    char *ws = nullptr;
    const int64_t steps = (n + batch - 1) / batch;
    float *losses = nullptr;
    SNCH_CUDA(scratch_alloc(&ws, mlp_workspace_bytes(rows_max), st));
    cudaError_t e = scratch_alloc(&losses, 4 * (size_t)steps, st);
    const MlpWorkspace w = mlp_workspace(ws, rows_max);
    for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep)
        for (int64_t s = 0; s < steps && e == cudaSuccess; ++s)
        {
            const int64_t b0 = s * batch, cnt = std::min<int64_t>(batch, n - b0), rows = (cnt + 127) / 128 * 128;
            e = mlp_forward_backward(m->st.params, m->st.grad, pts + 3 * b0, targets + 2 * b0, cnt, rows,
                                     m->st.center, m->st.inv_half, tau, w, m->st.loss, m->st.status, st);
            if (e == cudaSuccess)
                e = mlp_adam(m->st.params, m->st.grad, m->st.m, m->st.v, lr, ++m->st.step, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(losses + s, m->st.loss, 4, cudaMemcpyDeviceToDevice, st);
        }
    std::vector<float> h((size_t)steps, 0.0f);
    if (e == cudaSuccess && host_loss && epochs > 0)
        e = cudaMemcpyAsync(h.data(), losses, 4 * (size_t)steps, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(losses, st);
    cudaFreeAsync(ws, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    SNCH_CUDA(e);
    if (host_loss)
    {
        double acc = 0;
        for (float x : h)
            acc += x;
        *host_loss = steps ? (float)(acc / steps) : 0.0f;
    }
    return SNCH_OK;
}

int snch_mlp_predict_radius(snch_mlp_t m, const float *pts, int64_t n, float margin, float floor_, float *r_near,
                            float *r_sil, snch_stream_t stream)
{
    if (!m || n < 0 || (n > 0 && (!pts || (!r_near && !r_sil))))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "bad arguments");
    SNCH_CUDA(launch_mlp_radius(m->st.params, pts, n, m->st.center, m->st.inv_half, margin, floor_, r_near, r_sil,
                                m->st.status, S(stream)));
    return SNCH_OK;
}

// ------------------------------------------------------------------ batched scenes
int snch_batch_create(const float *v, int64_t nv, const int32_t *t, int64_t nt, const int64_t *mesh_vert_start,
                      const int64_t *mesh_tri_start, int32_t num_meshes, int device, snch_scene_t *out,
                      snch_stream_t stream)
{
    if (!out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "out_scene is NULL");
    *out = nullptr;
    if (num_meshes < 1 || num_meshes > 65536 || !mesh_vert_start || !mesh_tri_start)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "need 1..65536 meshes and their vertex / triangle starts");
    if (mesh_vert_start[0] != 0 || mesh_tri_start[0] != 0 || mesh_vert_start[num_meshes] != nv ||
        mesh_tri_start[num_meshes] != nt)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "mesh starts must run from 0 to the vertex / triangle counts");
    for (int32_t m = 0; m < num_meshes; ++m)
        if (mesh_vert_start[m + 1] < mesh_vert_start[m] || mesh_tri_start[m + 1] < mesh_tri_start[m])
            return fail(SNCH_ERR_INVALID_ARGUMENT, "mesh starts must not decrease (mesh " + std::to_string(m) + ")");
    cudaStream_t st = S(stream);
    if (nv < 0 || nt < 0 || (nv > 0 && !v) || (nt > 0 && !t))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "bad vertex or triangle buffer");
    if (nt >= (int64_t(1) << 30) || nv >= (int64_t(1) << 31))
        return fail(SNCH_ERR_TOO_LARGE, "at most 2^30 - 1 triangles and 2^31 - 1 vertices are supported");
    snch_scene_s *s = new snch_scene_s();
    s->num_verts = (uint32_t)nv;
    s->num_tris = (uint32_t)nt;
    s->num_meshes = (uint32_t)num_meshes;
    int rc = allocate(s);
    if (rc == SNCH_OK)
        rc = allocate_batch(s);
    if (rc != SNCH_OK)
    {
        free_scene(s);
        return rc;
    }
    std::vector<uint32_t> ts(num_meshes + 1);
    for (int32_t m = 0; m <= num_meshes; ++m)
        ts[m] = (uint32_t)mesh_tri_start[m];
    int64_t *vs_dev = nullptr;
    cudaError_t e = cudaSuccess;
    if (nv)
        e = cudaMemcpyAsync(s->verts, v, 12 * (size_t)nv, device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                            st);
    if (e == cudaSuccess)
        e = scratch_alloc(&vs_dev, 8 * (size_t)(num_meshes + 1), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(vs_dev, mesh_vert_start, 8 * (size_t)(num_meshes + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->mesh_tri_start, ts.data(), 4 * (size_t)(num_meshes + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nt)
        e = cudaMemcpyAsync(s->tris, t, 12 * (size_t)nt, device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                            st);
    if (e == cudaSuccess)
        e = launch_mesh_setup(s->mesh_tri_start, vs_dev, (uint32_t)num_meshes, (uint32_t)nt, s->tri_mesh, s->tris,
                              s->small + kWBad, st);
    uint32_t bad = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&bad, s->small + kWBad, 4, cudaMemcpyDeviceToHost, st);
    if (vs_dev)
        cudaFreeAsync(vs_dev, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        free_scene(s);
        return fail(SNCH_ERR_CUDA, std::string("batch upload: ") + cudaGetErrorString(e));
    }
    if (bad)
    {
        free_scene(s);
        return fail(SNCH_ERR_INVALID_ARGUMENT, std::to_string(bad) + " triangle vertex indices outside their mesh");
    }
    *out = s;
    return SNCH_OK;
}

int snch_batch_num_meshes(snch_scene_t s, int32_t *out)
{
    if (!s || !out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = (int32_t)s->num_meshes;
    return SNCH_OK;
}

int snch_batch_query_nearest(snch_scene_t s, const int32_t *mesh, const float *pts, int64_t n, int32_t *idx,
                             float *dist, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK && !s->num_meshes)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "not a batched scene");
    if (rc == SNCH_OK)
        rc = check_n(n, {mesh, pts, idx, dist});
    if (rc != SNCH_OK || n == 0)
        return rc;
    return run_query(
        s, 0, pts, nullptr, n, nullptr, S(stream),
        [&](const TreeView &t, const SeedArgs &seed) {
            return launch_nearest(t, pts, n, reinterpret_cast<uint32_t *>(idx), dist, S(stream), nullptr, seed);
        },
        reinterpret_cast<const uint32_t *>(mesh));
}

int snch_batch_query_silhouette(snch_scene_t s, const int32_t *mesh, const float *pts, const uint8_t *flip,
                                int64_t n, float *dist, int32_t *edge, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK && !s->num_meshes)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "not a batched scene");
    if (rc == SNCH_OK)
        rc = check_n(n, {mesh, pts, dist});
    if (rc != SNCH_OK || n == 0)
        return rc;
    return run_query(
        s, 1, pts, nullptr, n, nullptr, S(stream),
        [&](const TreeView &t, const SeedArgs &seed) {
            return launch_silhouette(t, pts, flip, n, dist, edge, S(stream), nullptr, seed);
        },
        reinterpret_cast<const uint32_t *>(mesh));
}

int snch_batch_query_nearest_seeded(snch_scene_t s, const int32_t *mesh, const float *pts, const float *radius,
                                    int64_t n, int32_t *idx, float *dist, uint32_t *num_fallback,
                                    snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK && !s->num_meshes)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "not a batched scene");
    if (rc == SNCH_OK)
        rc = check_n(n, {mesh, pts, radius, idx, dist});
    if (rc != SNCH_OK)
        return rc;
    if (n == 0)
    {
        if (num_fallback)
            SNCH_CUDA(cudaMemsetAsync(num_fallback, 0, 4, S(stream)));
        return SNCH_OK;
    }
    return run_query(
        s, 0, pts, radius, n, num_fallback, S(stream),
        [&](const TreeView &t, const SeedArgs &seed) {
            return launch_nearest(t, pts, n, reinterpret_cast<uint32_t *>(idx), dist, S(stream), nullptr, seed);
        },
        reinterpret_cast<const uint32_t *>(mesh));
}

int snch_batch_query_silhouette_seeded(snch_scene_t s, const int32_t *mesh, const float *pts, const float *radius,
                                       const uint8_t *flip, int64_t n, float *dist, int32_t *edge,
                                       uint32_t *num_fallback, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK && !s->num_meshes)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "not a batched scene");
    if (rc == SNCH_OK)
        rc = check_n(n, {mesh, pts, radius, dist});
    if (rc != SNCH_OK)
        return rc;
    if (n == 0)
    {
        if (num_fallback)
            SNCH_CUDA(cudaMemsetAsync(num_fallback, 0, 4, S(stream)));
        return SNCH_OK;
    }
    return run_query(
        s, 1, pts, radius, n, num_fallback, S(stream),
        [&](const TreeView &t, const SeedArgs &seed) {
            return launch_silhouette(t, pts, flip, n, dist, edge, S(stream), nullptr, seed);
        },
        reinterpret_cast<const uint32_t *>(mesh));
}

int snch_autotune(snch_scene_t s, const int32_t *near_mesh, const float *near_pts, int64_t n_near,
                  const int32_t *sil_mesh, const float *sil_pts, const uint8_t *sil_flip, int64_t n_sil, float *out_ms,
                  snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc == SNCH_OK)
        rc = check_n(n_near, {near_pts});
    if (rc == SNCH_OK)
        rc = check_n(n_sil, {sil_pts});
    if (rc == SNCH_OK && s->num_meshes && ((n_near && !near_mesh) || (n_sil && !sil_mesh)))
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, "a batched scene needs the mesh of every sample query");
    if (rc != SNCH_OK)
        return rc;
    cudaStream_t st = S(stream);
    // candidates (node width, threads per block, SNCH_OPT_PACKET, SNCH_OPT_PERSISTENT):
    // warp packets (1: whatever the sample's size), one search per lane, or
    // persistent work-stealing lanes; the block size applies to the per-lane
    // binary searches
    constexpr int kConfigs = SNCH_AUTOTUNE_CONFIGS;
    const int cw[kConfigs] = {2, 2, 4, 8, 2, 2, 2}, cb[kConfigs] = {128, 128, 128, 128, 64, 256, 128},
              cp[kConfigs] = {1, 0, 0, 0, 0, 0, 0}, cr[kConfigs] = {0, 0, 0, 0, 0, 0, 1};
    float ms[2][kConfigs] = {};
    char *out = nullptr;
    const int64_t nmax = std::max<int64_t>(1, std::max(n_near, n_sil));
    SNCH_CUDA(scratch_alloc(&out, 8 * (size_t)nmax, st));
    uint32_t *o_idx = reinterpret_cast<uint32_t *>(out);
    float *o_dist = reinterpret_cast<float *>(out + 4 * (size_t)nmax);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess)
        e = cudaEventCreate(&ev[1]);
    const int saved[8] = {s->width_near, s->width_sil,  s->block_near,      s->block_sil,
                          s->packet_near, s->packet_sil, s->persistent_near, s->persistent_sil};
    auto run = [&](int kind) -> int {
        if (kind == 0)
            return s->num_meshes
                       ? snch_batch_query_nearest(s, near_mesh, near_pts, n_near, reinterpret_cast<int32_t *>(o_idx),
                                                  o_dist, stream)
                       : snch_query_nearest(s, near_pts, n_near, o_idx, o_dist, stream);
        return s->num_meshes ? snch_batch_query_silhouette(s, sil_mesh, sil_pts, sil_flip, n_sil, o_dist,
                                                           reinterpret_cast<int32_t *>(o_idx), stream)
                             : snch_query_silhouette(s, sil_pts, sil_flip, n_sil, o_dist,
                                                     reinterpret_cast<int32_t *>(o_idx), stream);
    };
    for (int c = 0; c < kConfigs && e == cudaSuccess && rc == SNCH_OK; ++c)
    {
        const int w = cw[c];
        if (w > 2)
            rc = alloc_wide(s, w);
        s->width_near = s->width_sil = w;
        s->block_near = s->block_sil = cb[c];
        s->packet_near = s->packet_sil = cp[c];
        s->persistent_near = s->persistent_sil = cr[c];
        if (rc == SNCH_OK)
            rc = ensure_widths(s, st);
        for (int kind = 0; kind < 2 && rc == SNCH_OK && e == cudaSuccess; ++kind)
        {
            if ((kind == 0 ? n_near : n_sil) == 0)
                continue;
            rc = run(kind);  // warm-up
            if (rc == SNCH_OK)
                e = cudaEventRecord(ev[0], st);
            constexpr int kReps = 3;
            for (int r = 0; r < kReps && rc == SNCH_OK && e == cudaSuccess; ++r)
                rc = run(kind);
            if (rc == SNCH_OK && e == cudaSuccess)
                e = cudaEventRecord(ev[1], st);
            if (rc == SNCH_OK && e == cudaSuccess)
                e = cudaEventSynchronize(ev[1]);
            float t = 0.0f;
            if (rc == SNCH_OK && e == cudaSuccess)
                e = cudaEventElapsedTime(&t, ev[0], ev[1]);
            ms[kind][c] = t / kReps;
        }
    }
    for (cudaEvent_t x : ev)
        if (x)
            cudaEventDestroy(x);
    cudaFreeAsync(out, st);
    if (rc != SNCH_OK || e != cudaSuccess)
    {
        s->width_near = saved[0];
        s->width_sil = saved[1];
        s->block_near = saved[2];
        s->block_sil = saved[3];
        s->packet_near = saved[4];
        s->packet_sil = saved[5];
        s->persistent_near = saved[6];
        s->persistent_sil = saved[7];
        if (rc != SNCH_OK)
            return rc;
        SNCH_CUDA(e);
    }
    int best[2] = {-1, -1};
    for (int kind = 0; kind < 2; ++kind)
    {
        if ((kind == 0 ? n_near : n_sil) == 0)
            continue;
        best[kind] = 0;
        for (int c = 1; c < kConfigs; ++c)
            if (ms[kind][c] < ms[kind][best[kind]])
                best[kind] = c;
    }
    s->width_near = best[0] < 0 ? saved[0] : cw[best[0]];
    s->block_near = best[0] < 0 ? saved[2] : cb[best[0]];
    s->width_sil = best[1] < 0 ? saved[1] : cw[best[1]];
    s->block_sil = best[1] < 0 ? saved[3] : cb[best[1]];
    s->packet_near = best[0] < 0 ? saved[4] : cp[best[0]];
    s->packet_sil = best[1] < 0 ? saved[5] : cp[best[1]];
    s->persistent_near = best[0] < 0 ? saved[6] : cr[best[0]];
    s->persistent_sil = best[1] < 0 ? saved[7] : cr[best[1]];
    // records of a width no query type keeps are released
    SNCH_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 2; ++k)
    {
        const int w = k == 0 ? 4 : 8;
        if (s->width_near != w && s->width_sil != w && s->wide[k])
        {
            cache_release(s->wide[k]);
            cache_release(s->wide_idx[k]);
            s->wide[k] = nullptr;
            s->wide_idx[k] = nullptr;
            s->wide_cap[k] = 0;
            s->wide_ready[k] = false;
        }
    }
    if (out_ms)
        for (int kind = 0; kind < 2; ++kind)
            for (int c = 0; c < kConfigs; ++c)
                out_ms[kConfigs * kind + c] = ms[kind][c];
    return SNCH_OK;
}

struct snch_graph_s
{
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;  // kernels per launch of the graph
};

int snch_graph_create(snch_scene_t s, int rebuild, const int32_t *near_mesh, const float *near_pts, int64_t n_near,
                      int32_t *near_idx, float *near_dist, const int32_t *sil_mesh, const float *sil_pts,
                      const uint8_t *sil_flip, int64_t n_sil, float *sil_dist, int32_t *sil_edge, snch_graph_t *out,
                      snch_stream_t stream)
{
    if (!out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "out_graph is NULL");
    *out = nullptr;
    int rc = check_built(s);
    if (rc != SNCH_OK)
        return rc == SNCH_ERR_NOT_BUILT ? fail(rc, "build the scene once before capturing it") : rc;
    if (!stream)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "graph capture needs a created stream (not the legacy default stream)");
    if ((rc = check_n(n_near, {near_pts, near_idx, near_dist})) != SNCH_OK ||
        (rc = check_n(n_sil, {sil_pts, sil_dist})) != SNCH_OK)
        return rc;
    if (s->num_meshes && ((n_near && !near_mesh) || (n_sil && !sil_mesh)))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "a batched scene needs the mesh of every query");
    cudaStream_t st = S(stream);
    const uint64_t k0 = g_kernel_launches.load(std::memory_order_relaxed);
    SNCH_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    if (rebuild)
    {
        rc = snch_compute_silhouettes(s, stream);
        if (rc == SNCH_OK)
            rc = snch_build_bvh(s, stream);
    }
    if (rc == SNCH_OK && n_near)
        rc = s->num_meshes ? snch_batch_query_nearest(s, near_mesh, near_pts, n_near, near_idx, near_dist, stream)
                           : snch_query_nearest(s, near_pts, n_near, reinterpret_cast<uint32_t *>(near_idx), near_dist,
                                                stream);
    if (rc == SNCH_OK && n_sil)
        rc = s->num_meshes
                 ? snch_batch_query_silhouette(s, sil_mesh, sil_pts, sil_flip, n_sil, sil_dist, sil_edge, stream)
                 : snch_query_silhouette(s, sil_pts, sil_flip, n_sil, sil_dist, sil_edge, stream);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    const uint64_t kernels = g_kernel_launches.load(std::memory_order_relaxed) - k0;
    g_kernel_launches.fetch_sub(kernels, std::memory_order_relaxed);  // recorded, not launched
    if (rc != SNCH_OK || e != cudaSuccess)
    {
        if (graph)
            cudaGraphDestroy(graph);
        if (rc != SNCH_OK)
            return rc;
        SNCH_CUDA(e);
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    if (ei != cudaSuccess)
    {
        cudaGraphDestroy(graph);
        SNCH_CUDA(ei);
    }
    *out = new snch_graph_s{graph, exec, kernels};
    return SNCH_OK;
}

int snch_graph_launch(snch_graph_t g, snch_stream_t stream)
{
    if (!g)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "graph is NULL");
    SNCH_CUDA(cudaGraphLaunch(g->exec, S(stream)));
    note_launch((unsigned)g->kernels);
    return SNCH_OK;
}

int snch_graph_destroy(snch_graph_t g)
{
    if (!g)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "graph is NULL");
    if (g->exec)
        cudaGraphExecDestroy(g->exec);
    if (g->graph)
        cudaGraphDestroy(g->graph);
    delete g;
    return SNCH_OK;
}

// ---- flat binary file of a built scene: header, then the arrays below in order
namespace
{
constexpr char kFileMagic[8] = {'S', 'N', 'C', 'H', 'B', 'V', 'H', '1'};
struct FileHeader
{
    char magic[8];
    uint32_t version, num_verts, num_tris, reserved;
    int64_t num_edges;
};
struct FileArray
{
    void *dev;
    size_t bytes;
};
std::vector<FileArray> file_arrays(snch_scene_s *s, int64_t num_edges)
{
    const size_t n = s->num_tris, nn = n ? 2 * n - 1 : 0, ni = n > 1 ? n - 1 : 0;
    return {{s->verts, 12 * (size_t)s->num_verts}, {s->tris, 12 * n}, {s->tri_edges, 12 * n},
            {s->tri_owned, 12 * n}, {s->edge_verts, 16 * (size_t)num_edges}, {s->keys, 4 * n}, {s->vals, 4 * n},
            {s->nodes, sizeof(NodeRec) * nn}, {s->aabbs, sizeof(Box) * nn}, {s->cones, sizeof(Cone) * nn},
            {s->inner, sizeof(InnerRec) * ni}, {s->inner_cones, sizeof(InnerConeRec) * ni},
            {s->leaves, sizeof(LeafRec) * n}, {s->edges, sizeof(EdgeRec) * 3 * n}};
}
int64_t scene_num_edges(snch_scene_s *s)
{
    if (s->num_edges_host < 0)
    {
        uint32_t e = 0;
        if (cudaMemcpy(&e, s->small + kWNumEdges, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return -1;
        s->num_edges_host = e;
    }
    return s->num_edges_host;
}
}  // namespace

int snch_scene_save(snch_scene_t s, const char *path, snch_stream_t stream)
{
    int rc = check_built(s);
    if (rc != SNCH_OK)
        return rc;
    if (!path)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "path is NULL");
    if (s->num_meshes)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "only plain scenes are saved");
    SNCH_CUDA(cudaStreamSynchronize(S(stream)));
    const int64_t ne = scene_num_edges(s);
    if (ne < 0)
        return fail(SNCH_ERR_CUDA, "reading the edge count failed");
    FILE *fp = std::fopen(path, "wb");
    if (!fp)
        return fail(SNCH_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    FileHeader h{};
    std::memcpy(h.magic, kFileMagic, 8);
    h.version = 1;
    h.num_verts = s->num_verts;
    h.num_tris = s->num_tris;
    h.num_edges = ne;
    bool ok = std::fwrite(&h, sizeof h, 1, fp) == 1;
    std::vector<char> buf;
    for (const FileArray &a : file_arrays(s, ne))
    {
        if (!ok || a.bytes == 0)
            continue;
        buf.resize(a.bytes);
        ok = cudaMemcpy(buf.data(), a.dev, a.bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
             std::fwrite(buf.data(), 1, a.bytes, fp) == a.bytes;
    }
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok)
        return fail(SNCH_ERR_CUDA, std::string("writing ") + path + " failed");
    return SNCH_OK;
}

int snch_scene_load(const char *path, snch_scene_t *out, snch_stream_t stream)
{
    if (!out || !path)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "path and out_scene are required");
    *out = nullptr;
    FILE *fp = std::fopen(path, "rb");
    if (!fp)
        return fail(SNCH_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    FileHeader h{};
    if (std::fread(&h, sizeof h, 1, fp) != 1 || std::memcmp(h.magic, kFileMagic, 8) != 0 || h.version != 1 ||
        h.num_tris >= (1u << 30) || h.num_edges < 0 || h.num_edges > 3 * (int64_t)h.num_tris)
    {
        std::fclose(fp);
        return fail(SNCH_ERR_INVALID_ARGUMENT, std::string(path) + " is not a scene file of this library");
    }
    snch_scene_s *s = new snch_scene_s();
    s->num_verts = h.num_verts;
    s->num_tris = h.num_tris;
    int rc = allocate(s);
    std::vector<char> buf;
    cudaStream_t st = S(stream);
    for (const FileArray &a : rc == SNCH_OK ? file_arrays(s, h.num_edges) : std::vector<FileArray>())
    {
        if (rc != SNCH_OK || a.bytes == 0)
            continue;
        buf.resize(a.bytes);
        if (std::fread(buf.data(), 1, a.bytes, fp) != a.bytes)
            rc = fail(SNCH_ERR_INVALID_ARGUMENT, std::string(path) + " is truncated");
        else if (cudaMemcpy(a.dev, buf.data(), a.bytes, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = fail(SNCH_ERR_CUDA, "upload of the scene file failed");
    }
    char extra = 0;
    if (rc == SNCH_OK && std::fread(&extra, 1, 1, fp) != 0)
        rc = fail(SNCH_ERR_INVALID_ARGUMENT, std::string(path) + " has trailing bytes");
    std::fclose(fp);
    if (rc == SNCH_OK)
    {
        const uint32_t ne = (uint32_t)h.num_edges;
        cudaError_t e = cudaMemcpyAsync(s->small + kWNumEdges, &ne, 4, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = launch_ref_objects(s->verts, s->tris, s->tri_owned, s->edge_verts, s->num_tris, s->ref_objects,
                                   s->ref_edges, st);
        if (e == cudaSuccess)
            e = launch_top_levels(s->inner, s->inner_cones, s->num_tris, kTopSlots, s->top_inner, s->top_cones, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            rc = fail(SNCH_ERR_CUDA, std::string("scene load: ") + cudaGetErrorString(e));
    }
    if (rc != SNCH_OK)
    {
        free_scene(s);
        return rc;
    }
    s->num_edges_host = h.num_edges;
    s->topology_ready = true;
    s->built = true;
    *out = s;
    return SNCH_OK;
}

int snch_scene_vertices(snch_scene_t s, float **out)
{
    if (!s || !out)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene and out are required");
    *out = s->verts;
    return SNCH_OK;
}

int snch_get_option(snch_scene_t s, int option, int64_t *value)
{
    if (!s || !value)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene and value are required");
    switch (option)
    {
    case SNCH_OPT_TRAVERSAL: *value = s->traversal; break;
    case SNCH_OPT_QUERY_ORDER: *value = s->query_order; break;
    case SNCH_OPT_ORDER_MIN_BATCH: *value = s->order_min; break;
    case SNCH_OPT_PERSISTENT:
    case SNCH_OPT_PERSISTENT_NEAREST: *value = s->persistent_near; break;
    case SNCH_OPT_PERSISTENT_SILHOUETTE: *value = s->persistent_sil; break;
    case SNCH_OPT_TAIL_CAP: *value = s->tail_cap; break;
    case SNCH_OPT_NODE_WIDTH:
    case SNCH_OPT_NODE_WIDTH_NEAREST: *value = s->width_near; break;
    case SNCH_OPT_NODE_WIDTH_SILHOUETTE: *value = s->width_sil; break;
    case SNCH_OPT_BLOCK:
    case SNCH_OPT_BLOCK_NEAREST: *value = s->block_near; break;
    case SNCH_OPT_BLOCK_SILHOUETTE: *value = s->block_sil; break;
    case SNCH_OPT_PACKET:
    case SNCH_OPT_PACKET_NEAREST: *value = s->packet_near; break;
    case SNCH_OPT_PACKET_SILHOUETTE: *value = s->packet_sil; break;
    case SNCH_OPT_HOST_CHUNK: *value = s->host_chunk; break;
    case SNCH_OPT_PERSISTENT_RAY: *value = s->persistent_ray; break;
    case SNCH_OPT_PACKET_PERSISTENT_MIN: *value = s->packet_persistent_min; break;
    case SNCH_OPT_OUTPUT_SCATTER: *value = s->output_scatter; break;
    case SNCH_OPT_TOP_LEVELS: *value = s->top_levels; break;
    case SNCH_OPT_RAY_ORDER: *value = s->ray_order; break;
    case SNCH_OPT_ORDER_BITS: *value = s->order_bits; break;
    default: return fail(SNCH_ERR_INVALID_ARGUMENT, "unknown option " + std::to_string(option));
    }
    return SNCH_OK;
}

int snch_get_search_config(snch_scene_t s, int which, int32_t *out_width, int32_t *out_block)
{
    if (!s || (which != 0 && which != 1))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "scene and which (0 or 1) are required");
    if (out_width)
        *out_width = which == 0 ? s->width_near : s->width_sil;
    if (out_block)
        *out_block = which == 0 ? s->block_near : s->block_sil;
    return SNCH_OK;
}

int snch_selfcheck_cone_filter(int64_t n, uint64_t seed, uint64_t *device_counts, snch_stream_t stream)
{
    if (n < 0 || (n > 0 && !device_counts))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "bad arguments");
    SNCH_CUDA(launch_cone_filter_check(n, seed, reinterpret_cast<unsigned long long *>(device_counts), S(stream)));
    return SNCH_OK;
}

int snch_gemm_bf16(const void *A, const void *B, float *C, int64_t M, int64_t N, int64_t K, int accumulate,
                   uint32_t *device_status, snch_stream_t stream)
{
    if (!A || !B || !C || !device_status || M <= 0 || M % 128 || K <= 0 || K % 64 ||
        (N != 64 && N != 128 && N != 192 && N != 256) || M > (int64_t(1) << 31) || K > (int64_t(1) << 30))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "need M % 128 == 0, K % 64 == 0, N in {64, 128, 192, 256}");
    SNCH_CUDA(launch_gemm_bf16(A, B, C, M, N, K, accumulate, device_status, S(stream)));
    return SNCH_OK;
}


// ------------------------------------------------------------------ walk-on-stars driver
int snch_wost_trace(snch_scene_t dir, snch_scene_t neu, snch_mlp_t mlp, const snch_wost_params *p, float *estimates,
                    float *start_points, snch_wost_stats *stats, snch_stream_t stream)
{
    int rc = check_built(dir);
    if (rc == SNCH_OK)
        rc = check_built(neu);
    if (rc != SNCH_OK)
        return rc;
    if (!p || !estimates || !stats || p->walkers <= 0 || p->walkers >= (int64_t(1) << 31) || p->max_steps < 1 ||
        p->max_steps > SNCH_WOST_MAX_STEPS || !(p->epsilon > 0.f) || !(p->radius >= 0.f))
        return fail(SNCH_ERR_INVALID_ARGUMENT, "bad walk-on-stars parameters");
    if (dir->num_tris == 0)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "the Dirichlet scene is empty: walks would never end");
    if (dir->num_meshes || neu->num_meshes)
        return fail(SNCH_ERR_INVALID_ARGUMENT, "walk-on-stars takes plain scenes");
    std::memset(stats, 0, sizeof(*stats));
    cudaStream_t st = S(stream);
    const size_t n = (size_t)p->walkers;
    const bool has_neu = neu->num_tris > 0;
    // one block: two walker states, the step batches, query outputs, counters
    const size_t per = 2 * (12 + 12 + 1 + 4 + 4) + 4 + 4 + 4 + 4 + 4 + 4 + 12 + 4 + 4 + 4 + 4 + 1 + 4 + 8 + 4 + 4 + 4 +
                       12 + 4 + 4;
    char *blk = nullptr;
    SNCH_CUDA(scratch_alloc(&blk, per * n + 64 * 256, st));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *q = blk + off;
        off += (bytes + 255) & ~size_t(255);
        return q;
    };
    WalkState A, B;
    for (WalkState *w : {&A, &B})
    {
        w->x = reinterpret_cast<float *>(take(12 * n));
        w->nb = reinterpret_cast<float *>(take(12 * n));
        w->on_b = reinterpret_cast<uint8_t *>(take(n));
        w->total = reinterpret_cast<float *>(take(4 * n));
        w->id = reinterpret_cast<uint32_t *>(take(4 * n));
    }
    float *d_dir = reinterpret_cast<float *>(take(4 * n)), *d_sil = reinterpret_cast<float *>(take(4 * n));
    float *r_near = reinterpret_cast<float *>(take(4 * n)), *r_sil = reinterpret_cast<float *>(take(4 * n));
    uint32_t *near_idx = reinterpret_cast<uint32_t *>(take(4 * n));
    int32_t *sil_edge = reinterpret_cast<int32_t *>(take(4 * n));
    WalkStep ws{};
    ws.dir = reinterpret_cast<float *>(take(12 * n));
    ws.radius = reinterpret_cast<float *>(take(4 * n));
    ws.u = reinterpret_cast<float *>(take(4 * n));
    ws.su = reinterpret_cast<float *>(take(4 * n));
    ws.sv = reinterpret_cast<float *>(take(4 * n));
    ws.hit = reinterpret_cast<uint8_t *>(take(n));
    ws.t = reinterpret_cast<float *>(take(4 * n));
    ws.uv = reinterpret_cast<float *>(take(8 * n));
    ws.hit_idx = reinterpret_cast<uint32_t *>(take(4 * n));
    ws.smp_idx = reinterpret_cast<int32_t *>(take(4 * n));
    ws.smp_pdf = reinterpret_cast<float *>(take(4 * n));
    ws.smp_pt = reinterpret_cast<float *>(take(12 * n));
    uint32_t *counts = reinterpret_cast<uint32_t *>(take(256));  // live, terminated, fallback x2
    WalkStep run_step = ws;
    if (!has_neu)
    {
        run_step.hit = nullptr;
        run_step.smp_idx = nullptr;
    }
    cudaEvent_t ev[4];
    for (auto &e : ev)
        cudaEventCreate(&e);
    auto finish = [&](int code) {
        for (auto &e : ev)
            cudaEventDestroy(e);
        cudaFreeAsync(blk, st);
        cudaStreamSynchronize(st);
        return code;
    };
#define WOST_TRY(expr)                                                                                              \
    do                                                                                                              \
    {                                                                                                               \
        cudaError_t e_ = (expr);                                                                                    \
        if (e_ != cudaSuccess)                                                                                      \
            return finish(fail(SNCH_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)));                 \
    } while (0)
#define WOST_RC(expr)                                                                                               \
    do                                                                                                              \
    {                                                                                                               \
        const int r_ = (expr);                                                                                      \
        if (r_ != SNCH_OK)                                                                                          \
            return finish(r_);                                                                                      \
    } while (0)
    WOST_TRY(launch_wost_init(A, (int64_t)n, p->center, p->radius, p->seed, start_points, st));
    int64_t live = (int64_t)n;
    for (int step = 0; step < p->max_steps && live > 0; ++step)
    {
        stats->live[step] = live;
        WOST_TRY(cudaMemsetAsync(counts, 0, 16, st));
        WOST_TRY(cudaEventRecord(ev[0], st));
        // distances: to the Dirichlet boundary, to the Neumann silhouettes
        if (mlp)
        {
            WOST_TRY(launch_mlp_radius(mlp->st.params, A.x, live, mlp->st.center, mlp->st.inv_half, p->margin,
                                       p->floor_, r_near, has_neu ? r_sil : nullptr, mlp->st.status, st));
            WOST_RC(snch_query_nearest_seeded(dir, A.x, r_near, live, near_idx, d_dir, counts + 2, stream));
            if (has_neu)
                WOST_RC(snch_query_silhouette_seeded(neu, A.x, nullptr, r_sil, live, d_sil, sil_edge, counts + 3,
                                                     stream));
        }
        else
        {
            WOST_RC(snch_query_nearest(dir, A.x, live, near_idx, d_dir, stream));
            if (has_neu)
                WOST_RC(snch_query_silhouette(neu, A.x, nullptr, live, d_sil, sil_edge, stream));
        }
        WOST_TRY(cudaEventRecord(ev[1], st));
        WOST_TRY(launch_wost_prepare(A, live, d_dir, has_neu ? d_sil : nullptr, B, ws, (uint32_t)step,
                                     (uint32_t)(p->max_steps - 1), p->epsilon, p->seed, estimates, counts, st));
        uint32_t h[4] = {0, 0, 0, 0};
        WOST_TRY(cudaMemcpyAsync(h, counts, 16, cudaMemcpyDeviceToHost, st));
        WOST_TRY(cudaStreamSynchronize(st));
        const int64_t next = h[0];
        stats->terminated += h[1];
        stats->fallback[step] = h[2] + h[3];
        WOST_TRY(cudaEventRecord(ev[2], st));
        if (next > 0 && has_neu)
        {
            WOST_RC(snch_query_ray(neu, B.x, ws.dir, ws.radius, next, ws.hit, ws.t, ws.uv, ws.hit_idx, stream));
            WOST_RC(snch_sample_in_sphere(neu, B.x, ws.radius, ws.u, next, ws.smp_idx, ws.smp_pdf, stream));
            WOST_TRY(launch_sample_point(neu->verts, neu->tris, neu->num_tris, ws.smp_idx, ws.su, ws.sv, next,
                                         ws.smp_pt, st));
        }
        WOST_TRY(cudaEventRecord(ev[3], st));
        WOST_TRY(launch_wost_update(B, next, run_step, neu->verts, neu->tris, st));
        WOST_TRY(cudaStreamSynchronize(st));
        float a = 0.f, b = 0.f, c = 0.f;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[2], ev[3]);
        cudaEventElapsedTime(&c, ev[0], ev[3]);
        stats->query_ms[step] = a + b;
        stats->step_ms[step] = c;
        stats->queries[step] = live * (has_neu ? 2 : 1) + next * (has_neu ? 2 : 0);
        stats->steps = step + 1;
        std::swap(A, B);
        live = next;
    }
#undef WOST_TRY
#undef WOST_RC
    return finish(SNCH_OK);
}

}  // extern "C"
