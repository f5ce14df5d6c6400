// Silhouette topology on the device: the reference does this on the host with
// std::map / std::unordered_map (include/snch_lbvh/scene.cuh:1135-1225).
//
// Every (triangle i, corner j) is an edge occurrence k = 3i+j of the edge
// (v_j, v_{j+1}). The occurrences are inserted into an open-addressing hash
// table keyed by (min vertex, max vertex); per distinct edge the table keeps
//   * the first occurrence (atomicMin)            -> edge ids in first-seen
//     order (assign_edge_indices, 1135-1166) and ownership (build_bvh, 1207-1225:
//     the first triangle that meets an edge owns it);
//   * the last occurrence of each orientation (atomicMax) -> the 4-vertex
//     record {opp0, min, max, opp1} that compute_silhouettes (1167-1204)
//     leaves after its in-order overwrites.
// All of these are order-independent reductions, so the result is
// deterministic and identical to the reference's host loop.
#include "common.cuh"
#include "internal.h"

namespace snch
{
namespace
{

constexpr unsigned long long kEmpty = ~0ull;

inline uint32_t table_capacity(uint32_t num_tris)
{
    uint64_t need = 3ull * num_tris;
    uint64_t c = 64;
    while (c < need)
        c <<= 1;
    return (uint32_t)(2 * c);
}

struct Table
{
    unsigned long long *keys;
    uint32_t *first, *last_pos, *last_neg;
    uint32_t cap_mask;
};

__device__ __forceinline__ uint32_t hash64(unsigned long long k, uint32_t mask)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)k & mask;
}

__global__ void edge_insert_kernel(const int32_t *__restrict__ tris, uint32_t num_occ, Table t,
                                   uint32_t *__restrict__ slot_of, uint32_t *status)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= num_occ)
        return;
    const uint32_t i = k / 3, j = k - 3 * i;
    const int32_t vj = tris[3 * (uint64_t)i + j], vk = tris[3 * (uint64_t)i + (j + 1) % 3];
    // compute_silhouettes swaps (J, K) only when v_J > v_K (orientation -1)
    const bool neg = vj > vk;
    const uint32_t lo = (uint32_t)(neg ? vk : vj), hi = (uint32_t)(neg ? vj : vk);
    const unsigned long long key = ((unsigned long long)lo << 32) | hi;
    uint32_t h = hash64(key, t.cap_mask);
    for (uint32_t probe = 0; probe <= t.cap_mask; ++probe)
    {
        const unsigned long long prev = atomicCAS(t.keys + h, kEmpty, key);
        if (prev == kEmpty || prev == key)
        {
            atomicMin(t.first + h, k);
            atomicMax(neg ? t.last_neg + h : t.last_pos + h, k + 1);
            slot_of[k] = h;
            return;
        }
        h = (h + 1) & t.cap_mask;
    }
    atomicOr(status, kStatusHashFull);
    slot_of[k] = 0;
}

__global__ void edge_flag_kernel(const uint32_t *__restrict__ slot_of, uint32_t num_occ, Table t,
                                 uint32_t *__restrict__ is_first)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < num_occ)
        is_first[k] = (t.first[slot_of[k]] == k) ? 1u : 0u;
}

__device__ __forceinline__ int32_t opposite_vertex(const int32_t *tris, uint32_t k)
{
    const uint32_t i = k / 3, j = k - 3 * i;
    return tris[3 * (uint64_t)i + (j + 2) % 3];
}

__global__ void edge_finalize_kernel(const int32_t *__restrict__ tris, uint32_t num_tris, Table t,
                                     const uint32_t *__restrict__ slot_of, const uint32_t *__restrict__ is_first,
                                     const uint32_t *__restrict__ ids, int32_t *__restrict__ tri_edges,
                                     int32_t *__restrict__ tri_owned, int32_t *__restrict__ edge_verts)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_tris)
        return;
    int32_t owned[3] = {-1, -1, -1};
    int p = 0;
    for (int j = 0; j < 3; ++j)
    {
        const uint32_t k = 3 * i + j;
        const uint32_t s = slot_of[k];
        const uint32_t g = t.first[s];
        if (g >= 3 * num_tris)  // only after a full hash table (status bit set)
        {
            tri_edges[k] = -1;
            continue;
        }
        tri_edges[k] = (int32_t)ids[g];
        if (is_first[k])
        {
            const int32_t e = (int32_t)ids[k];
            owned[p++] = e;
            const unsigned long long key = t.keys[s];
            const uint32_t lp = t.last_pos[s], ln = t.last_neg[s];
            int4 rec;
            rec.x = lp ? opposite_vertex(tris, lp - 1) : -1;
            rec.y = (int32_t)(key >> 32);
            rec.z = (int32_t)(key & 0xffffffffull);
            rec.w = ln ? opposite_vertex(tris, ln - 1) : -1;
            reinterpret_cast<int4 *>(edge_verts)[e] = rec;
        }
    }
    tri_owned[3 * (uint64_t)i] = owned[0];
    tri_owned[3 * (uint64_t)i + 1] = owned[1];
    tri_owned[3 * (uint64_t)i + 2] = owned[2];
}

struct Layout
{
    size_t keys, first, last_pos, last_neg, slot_of, is_first, ids, scan, total;
};
inline Layout layout(uint32_t num_tris)
{
    const uint64_t cap = table_capacity(num_tris), occ = 3ull * num_tris;
    Layout l;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    l.keys = 0;
    l.first = l.keys + al(8 * cap);
    l.last_pos = l.first + al(4 * cap);
    l.last_neg = l.last_pos + al(4 * cap);
    l.slot_of = l.last_neg + al(4 * cap);
    l.is_first = l.slot_of + al(4 * occ);
    l.ids = l.is_first + al(4 * occ);
    l.scan = l.ids + al(4 * occ);
    l.total = l.scan + al(scan_flags_scratch_bytes(occ));
    return l;
}

}  // namespace

size_t topology_scratch_bytes(uint32_t num_tris) { return layout(num_tris).total; }

cudaError_t compute_topology(const int32_t *tris, uint32_t num_tris, int32_t *tri_edges, int32_t *tri_owned,
                             int32_t *edge_verts, uint32_t *num_edges, void *scratch, uint32_t *status,
                             cudaStream_t st)
{
    if (num_tris == 0)
        return cudaMemsetAsync(num_edges, 0, 4, st);
    const Layout l = layout(num_tris);
    char *base = static_cast<char *>(scratch);
    const uint32_t cap = table_capacity(num_tris), occ = 3 * num_tris;
    Table t;
    t.keys = reinterpret_cast<unsigned long long *>(base + l.keys);
    t.first = reinterpret_cast<uint32_t *>(base + l.first);
    t.last_pos = reinterpret_cast<uint32_t *>(base + l.last_pos);
    t.last_neg = reinterpret_cast<uint32_t *>(base + l.last_neg);
    t.cap_mask = cap - 1;
    uint32_t *slot_of = reinterpret_cast<uint32_t *>(base + l.slot_of);
    uint32_t *is_first = reinterpret_cast<uint32_t *>(base + l.is_first);
    uint32_t *ids = reinterpret_cast<uint32_t *>(base + l.ids);
    cudaError_t e;
    if ((e = cudaMemsetAsync(t.keys, 0xff, 8 * (size_t)cap, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(t.first, 0xff, 4 * (size_t)cap, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(t.last_pos, 0, (char *)slot_of - (char *)t.last_pos, st)) != cudaSuccess)
        return e;
    const int tb = 256;
    edge_insert_kernel<<<(occ + tb - 1) / tb, tb, 0, st>>>(tris, occ, t, slot_of, status);
    note_launch();
    edge_flag_kernel<<<(occ + tb - 1) / tb, tb, 0, st>>>(slot_of, occ, t, is_first);
    note_launch();
    if ((e = scan_flags(is_first, ids, occ, num_edges, base + l.scan, status, st)) != cudaSuccess)
        return e;
    edge_finalize_kernel<<<(num_tris + tb - 1) / tb, tb, 0, st>>>(tris, num_tris, t, slot_of, is_first, ids,
                                                                  tri_edges, tri_owned, edge_verts);
    note_launch();
    return cudaGetLastError();
}

}  // namespace snch
