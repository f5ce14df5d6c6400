// Single-pass flag scan and onesweep LSD radix sort for sm_103a.
//
// Both use decoupled look-back (Merrill & Garland 2016; Adinets & Merrill
// 2022): a block takes the next tile id from an atomic counter, publishes its
// local aggregate, then walks back over earlier tiles until it meets one that
// published an inclusive prefix. Tile ids follow block start order, so a block
// only waits on blocks that are already running; every wait is also bounded
// (kSpinLimit polls) and gives up by setting a status bit instead of hanging.
//
// The sort replaces thrust::stable_sort_by_key of the reference
// (include/snch_lbvh/core/bvh.cuh:452-454): it is stable, so equal Morton codes
// keep ascending object index exactly as the reference's sort does.
#include "common.cuh"
#include "internal.h"

namespace snch
{
namespace
{

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRounds = 16;  // keys per thread
static_assert(kThreads * kRounds == kSortTile, "tile size");
constexpr uint32_t kFlagA = 1u << 30;  // tile aggregate published
constexpr uint32_t kFlagP = 2u << 30;  // inclusive prefix published
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;

// exclusive scan of one value per thread over a 256-thread block
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *s_warp, uint32_t *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        s_warp[warp] = x;
    __syncthreads();
    uint32_t wsum = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w)
    {
        uint32_t t = s_warp[w];
        wsum += (w < warp) ? t : 0u;
        all += t;
    }
    __syncthreads();
    if (total)
        *total = all;
    return wsum + x - v;
}

// Walk back from tile-1 summing aggregates until an inclusive prefix is found.
__device__ __forceinline__ uint32_t look_back(const uint32_t *state, int64_t tile, int64_t stride, uint32_t *status)
{
    uint32_t prefix = 0, spins = 0;
    int64_t j = tile - 1;
    while (j >= 0)
    {
        const uint32_t s = ld_relaxed(state + j * stride);
        const uint32_t f = s & ~kCountMask;
        if (f == 0u)
        {
            if (++spins > kSpinLimit)
            {
                atomicOr(status, kStatusLookbackTimeout);
                break;
            }
            if (spins > 32)
                __nanosleep(64);
            continue;
        }
        prefix += s & kCountMask;
        if (f == kFlagP)
            break;
        --j;
    }
    return prefix;
}

__global__ void __launch_bounds__(kThreads) scan_flags_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                              uint32_t n, uint32_t *total, uint32_t *state,
                                                              uint32_t *tile_counter, uint32_t *status)
{
    __shared__ uint32_t s_tile, s_prefix, s_warp[kWarps];
    if (threadIdx.x == 0)
        s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * kSortTile + (uint64_t)threadIdx.x * kRounds;
    uint32_t v[kRounds], sum = 0;
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
    {
        v[r] = (base + r < n) ? in[base + r] : 0u;
        sum += v[r];
    }
    uint32_t block_total;
    const uint32_t excl = block_excl_scan(sum, s_warp, &block_total);
    if (threadIdx.x == 0)
    {
        uint32_t prefix = 0;
        if (tile == 0)
            st_relaxed(state, kFlagP | block_total);
        else
        {
            st_relaxed(state + tile, kFlagA | block_total);
            prefix = look_back(state, tile, 1, status);
            st_relaxed(state + tile, kFlagP | (prefix + block_total));
        }
        s_prefix = prefix;
        const uint32_t num_tiles = (n + kSortTile - 1) / kSortTile;
        if (total && tile == num_tiles - 1)
            *total = prefix + block_total;
    }
    __syncthreads();
    uint32_t run = s_prefix + excl;
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
    {
        if (base + r < n)
            out[base + r] = run;
        run += v[r];
    }
}

__global__ void radix_hist_kernel(const uint32_t *__restrict__ keys, uint32_t n, int passes, uint32_t *hist)
{
    __shared__ uint32_t s_hist[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
        (&s_hist[0][0])[i] = 0;
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint32_t k = keys[i];
        for (int p = 0; p < passes; ++p)
            atomicAdd(&s_hist[p][(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
    {
        const uint32_t c = (&s_hist[0][0])[i];
        if (c)
            atomicAdd(hist + i, c);
    }
}

// One 8-bit digit pass. Warp w ranks elements [tile*4096 + w*512, +512) in 16
// rounds of 32 with __match_any_sync, which keeps equal digits in input order;
// the block then stages the tile in shared memory in digit order and writes
// each digit run to its global position.
// (The compiler's 80 registers allow 3 blocks per SM. Compiled for 4 or 5 blocks,
// with the largest shared-memory carveout so that the 42 KB of shared memory
// per block fit, the 16M-pair sort took 0.576 / 0.586 against 0.570 ms.)
__global__ void __launch_bounds__(kThreads) onesweep_pass_kernel(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in, uint32_t *__restrict__ keys_out,
    uint32_t *__restrict__ vals_out, uint32_t n, int shift, const uint32_t *__restrict__ hist, uint32_t *lookback,
    uint32_t *tile_counter, uint32_t *status)
{
    __shared__ uint32_t s_warp_hist[kWarps][256];
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_local[256];
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp[kWarps];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0)
        s_tile = atomicAdd(tile_counter, 1u);
    for (int i = tid; i < kWarps * 256; i += kThreads)
        (&s_warp_hist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * kSortTile + (uint64_t)warp * (32 * kRounds);

    uint32_t k[kRounds], v[kRounds], rk[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
    {
        const uint64_t e = base + r * 32 + lane;
        const bool ok = e < n;
        k[r] = ok ? keys_in[e] : 0u;
        v[r] = ok ? vals_in[e] : 0u;
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
    {
        const uint64_t e = base + r * 32 + lane;
        const uint32_t d = (e < n) ? ((k[r] >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t cnt = 0;
        if (lane == leader && d < 256u)
        {
            cnt = s_warp_hist[warp][d];
            s_warp_hist[warp][d] = cnt + __popc(peers);
        }
        cnt = __shfl_sync(0xffffffffu, cnt, leader);
        rk[r] = cnt + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();

    const uint32_t d = tid;  // one digit per thread
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w)
    {
        const uint32_t c = s_warp_hist[w][d];
        s_warp_hist[w][d] = tot;
        tot += c;
    }
    uint32_t *mine = lookback + (uint64_t)tile * 256 + d;
    uint32_t prefix = 0;
    if (tile == 0)
        st_relaxed(mine, kFlagP | tot);
    else
    {
        st_relaxed(mine, kFlagA | tot);
        prefix = look_back(lookback + d, tile, 256, status);
        st_relaxed(mine, kFlagP | (prefix + tot));
    }
    const uint32_t g_excl = block_excl_scan(hist[d], s_warp, nullptr);
    const uint32_t l_excl = block_excl_scan(tot, s_warp, nullptr);
    s_base[d] = g_excl + prefix;
    s_local[d] = l_excl;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
    {
        const uint64_t e = base + r * 32 + lane;
        if (e < n)
        {
            const uint32_t dd = (k[r] >> shift) & 255u;
            const uint32_t pos = s_local[dd] + s_warp_hist[warp][dd] + rk[r];
            s_keys[pos] = k[r];
            s_vals[pos] = v[r];
        }
    }
    __syncthreads();
    const uint64_t tile_begin = (uint64_t)tile * kSortTile;
    const uint32_t tile_n = (uint32_t)((n - tile_begin) < (uint64_t)kSortTile ? (n - tile_begin) : kSortTile);
    for (uint32_t i = tid; i < tile_n; i += kThreads)
    {
        const uint32_t key = s_keys[i];
        const uint32_t dd = (key >> shift) & 255u;
        const uint32_t g = s_base[dd] + (i - s_local[dd]);
        if (g < n)  // only false after a look-back timeout (status bit set)
        {
            keys_out[g] = key;
            vals_out[g] = s_vals[i];
        }
    }
}

inline uint32_t num_tiles(uint64_t n) { return (uint32_t)((n + kSortTile - 1) / kSortTile); }

}  // namespace

size_t scan_flags_scratch_bytes(uint64_t n) { return 4 * (size_t)(num_tiles(n) + 1); }

cudaError_t scan_flags(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, void *scratch,
                       uint32_t *status, cudaStream_t st)
{
    if (n == 0)
        return total ? cudaMemsetAsync(total, 0, 4, st) : cudaSuccess;
    const uint32_t tiles = num_tiles(n);
    uint32_t *state = static_cast<uint32_t *>(scratch);
    uint32_t *counter = state + tiles;
    cudaError_t e = cudaMemsetAsync(state, 0, scan_flags_scratch_bytes(n), st);
    if (e != cudaSuccess)
        return e;
    scan_flags_kernel<<<tiles, kThreads, 0, st>>>(in, out, n, total, state, counter, status);
    note_launch();
    return cudaGetLastError();
}

// scratch: [hist passes*256][lookback passes*tiles*256][tile counters passes]
size_t sort_scratch_bytes(uint32_t n, int key_bits)
{
    const int passes = sort_passes(key_bits);
    return 4 * ((size_t)passes * 256 + (size_t)passes * num_tiles(n) * 256 + passes);
}

cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_tmp, uint32_t *vals_tmp, uint32_t n,
                             int key_bits, const uint32_t *hist, void *scratch, uint32_t *status, cudaStream_t st,
                             SortResult *result)
{
    if (result)
        *result = SortResult{keys, vals};
    if (n <= 1)
        return cudaSuccess;
    const int passes = sort_passes(key_bits);
    const uint32_t tiles = num_tiles(n);
    uint32_t *s_hist = static_cast<uint32_t *>(scratch);
    uint32_t *s_look = s_hist + passes * 256;
    uint32_t *s_count = s_look + (size_t)passes * tiles * 256;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sort_scratch_bytes(n, key_bits), st);
    if (e != cudaSuccess)
        return e;
    if (!hist)
    {
        const uint32_t blocks = tiles < 1024 ? tiles : 1024;
        radix_hist_kernel<<<blocks, 256, 0, st>>>(keys, n, passes, s_hist);
        note_launch();
        hist = s_hist;
    }
    uint32_t *ki = keys, *vi = vals, *ko = keys_tmp, *vo = vals_tmp;
    for (int p = 0; p < passes; ++p)
    {
        onesweep_pass_kernel<<<tiles, kThreads, 0, st>>>(ki, vi, ko, vo, n, 8 * p, hist + 256 * p,
                                                         s_look + (size_t)p * tiles * 256, s_count + p, status);
        note_launch();
        uint32_t *t = ki;
        ki = ko;
        ko = t;
        t = vi;
        vi = vo;
        vo = t;
    }
    e = cudaGetLastError();
    if (result)
        *result = SortResult{ki, vi};
    else if (e == cudaSuccess && ki != keys)
    {
        e = cudaMemcpyAsync(keys, ki, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(vals, vi, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
    }
    return e;
}

}  // namespace snch
