// Learned search radius: a small MLP over Fourier features of the query point
// that predicts log(distance to the nearest primitive) and log(distance to the
// nearest silhouette edge); its prediction seeds the traversals
// (snch_query_*_seeded), which stay exact through their unbounded fallback.
//
//   features  u = (p - centre) / half_extent, f_k = pi * 2^(k/4), k = 0..31:
//             [sin(f_k u_a), cos(f_k u_a)] for a = x, y, z      -> 192
//   layers    192 -> 64 -> 64 -> 64 -> 64 (ReLU), BF16 weights and activations,
//             FP32 accumulation in tensor memory (tcgen05.mma kind::f16)
//   head      64 -> 2 (FP32, CUDA cores): log d_nearest, log d_silhouette
//
// Kernels:
//   gemm_bf16_kernel   C[MxN] (+)= A[MxK] B[NxK]^T, tiles of 128 rows, operands
//                      loaded by TMA into a 4-stage shared-memory ring in the
//                      core-matrix layout, one thread issues the MMAs, the
//                      accumulator stays in TMEM across the K loop; optional
//                      bias + ReLU -> BF16 epilogue; used by training (forward
//                      layers, input and weight gradients)
//   mlp_radius_kernel  fused inference: features -> 4 tensor-core layers -> head
//                      -> radius, persistent CTAs with the weights resident in
//                      shared memory
//   small elementwise kernels for training (transposes, loss, ReLU backward, Adam)
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "internal.h"
#include "tcgen05.cuh"

namespace snch
{
namespace mlp
{

constexpr int kFreq = 32;
constexpr int kIn = 6 * kFreq;  // 192
constexpr int kHid = 64;
constexpr int kOut = 2;
constexpr uint32_t kWaitPolls = 1u << 24;
constexpr int kMaxWgradSplits = 64;  // the weight-gradient C slices: 64 x 256 x 64 floats

// parameter block offsets (floats)
constexpr int kW1 = 0, kB1 = kW1 + kHid * kIn;
constexpr int kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid, kB3 = kW3 + kHid * kHid;
constexpr int kW4 = kB3 + kHid, kB4 = kW4 + kHid * kHid;
constexpr int kW5 = kB4 + kHid, kB5 = kW5 + kOut * kHid;
constexpr int kNumParams = kB5 + kOut;

// feature k of axis a is sin / cos(pi * s_k * u_a) with s_k = 2^(k/4) rounded to
// float on the host (the same values the FP64 checker uses), via sincospif,
// whose range reduction is exact
__constant__ float c_scale[kFreq];

// The 24 features of octave j (frequencies k = 4j .. 4j+3, columns 24j .. 24j+23):
// f[6 kk + 2 a] = sin, f[6 kk + 2 a + 1] = cos of pi s_{4j+kk} u_a. Octave 0 comes
// from sincospif; every further octave doubles the angles (s_{k+4} = 2 s_k exactly):
// sin 2x = 2 sin x cos x, cos 2x = (cos x - sin x)(cos x + sin x). Seven doublings
// grow the absolute error to about 2^7 float ulps (~1e-5), far below the BF16
// spacing the features are stored with.
struct Octaves
{
    float s[12], c[12];  // [kk * 3 + a]
    __device__ __forceinline__ void init(const float u[3])
    {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                sincospif(c_scale[kk] * u[a], &s[kk * 3 + a], &c[kk * 3 + a]);
    }
    __device__ __forceinline__ void emit(float (&f)[24]) const
    {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                f[6 * kk + 2 * a] = s[kk * 3 + a];
                f[6 * kk + 2 * a + 1] = c[kk * 3 + a];
            }
    }
    __device__ __forceinline__ void next()
    {
#pragma unroll
        for (int i = 0; i < 12; ++i)
        {
            const float sn = 2.0f * s[i] * c[i];
            c[i] = (c[i] - s[i]) * (c[i] + s[i]);
            s[i] = sn;
        }
    }
};

// ------------------------------------------------------------------ generic GEMM
// C[M x N] (+)= A[M x K] * B[N x K]^T; A, B bf16 row-major (K contiguous), C fp32
// row-major. M % 128 == 0, K % 64 == 0, N in {64, 128, 192, 256}.
// Split K (blockIdx.y = split): split s sums K columns [s * k_split, (s + 1) * k_split)
// into its own slice C + s * M * N, so a reduction over the slices follows.
// With H non-null (forward layers, N = 64) the epilogue writes
// H = bf16(max(C + bias, 0)) instead of C.
//
// Operands arrive by TMA (cp.async.bulk.tensor.2d) in 64-column K chunks through
// a ring of kStages shared-memory stages: thread 0 produces (waits until a
// stage is free, then issues 8 boxes of 8 columns x R rows per operand, each box
// landing as one column of 8 x 16-byte core matrices), thread 32 consumes (waits
// for the stage's bytes, issues the four K=16 tcgen05.mma steps, and commits to
// the stage's "empty" barrier, which the tensor core signals once it has read
// the stage). Layout of an operand of R rows in a stage:
//   byte(r, k) = (k / 8) * (R * 16) + r * 16 + (k % 8) * 2
// i.e. core matrices with LBO = R * 16 (along K) and SBO = 128 (along rows).
// Every wait is bounded: on a timeout the block sets kStatusLookbackTimeout,
// lets the copies and MMAs it issued finish (bounded again) and writes nothing.
template <int N>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const __grid_constant__ CUtensorMap tm_a,
                                                        const __grid_constant__ CUtensorMap tm_b,
                                                        float *__restrict__ C, const float *__restrict__ bias,
                                                        __nv_bfloat16 *__restrict__ H, int K, int k_split,
                                                        int accumulate, uint32_t *status)
{
    constexpr int kChunk = 64;
    constexpr int kStages = 4;
    constexpr uint32_t kABytes = 128 * kChunk * 2, kBBytes = N * kChunk * 2, kStageBytes = kABytes + kBBytes;
    constexpr uint32_t kCols = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
    extern __shared__ __align__(128) uint8_t gemm_dyn[];
    // the stage ring, 1024-byte aligned inside the dynamic allocation (1 KB extra)
    uint8_t *smem = gemm_dyn + ((1024u - (tc::smem_u32(gemm_dyn) & 1023u)) & 1023u);
    __shared__ uint64_t full[kStages], empty[kStages], done;
    __shared__ uint32_t tmem_base;
    __shared__ int issued_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0)
    {
        tc::tmem_alloc(&tmem_base, kCols);
        tc::tmem_relinquish();
    }
    if (tid == 0)
    {
        for (int s = 0; s < kStages; ++s)
        {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&done, 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tmem_base;
    const int m0 = blockIdx.x * 128;
    const int k_begin = blockIdx.y * k_split, k_end = min(K, k_begin + k_split);
    const int nk = (k_end - k_begin) / kChunk;
    constexpr int stages = kStages;
    C += (int64_t)blockIdx.y * gridDim.x * 128 * N;
    bool ok = true;
    if (tid == 0)
    {
        // producer
        int issued = 0;
        for (int i = 0; i < nk; ++i)
        {
            const int s = i % stages;
            if (i >= stages && !tc::mbar_wait(&empty[s], (uint32_t)((i / stages - 1) & 1), kWaitPolls))
            {
                ok = false;
                break;
            }
            uint8_t *sa = smem + s * kStageBytes, *sb = sa + kABytes;
            tc::mbar_arrive_expect_tx(&full[s], kStageBytes);
            const int kc = k_begin + i * kChunk;
#pragma unroll
            for (int j = 0; j < kChunk / 8; ++j)
            {
                tc::tma_load_2d(sa + j * (128 * 16), &tm_a, kc + 8 * j, m0, &full[s]);
                tc::tma_load_2d(sb + j * (N * 16), &tm_b, kc + 8 * j, 0, &full[s]);
            }
            issued = i + 1;
        }
        issued_s = issued;
    }
    else if (tid == 32)
    {
        // MMA issuer
        constexpr uint32_t idesc = tc::idesc_bf16_f32(128, N);
        for (int i = 0; i < nk; ++i)
        {
            const int s = i % stages;
            if (!tc::mbar_wait(&full[s], (uint32_t)((i / stages) & 1), kWaitPolls))
            {
                ok = false;
                break;
            }
            tc::fence_after_sync();
            const uint32_t sa = tc::smem_u32(smem + s * kStageBytes), sb = sa + kABytes;
#pragma unroll
            for (int k16 = 0; k16 < kChunk / 16; ++k16)
                tc::mma_bf16(taddr, tc::smem_desc(sa + k16 * 2 * (128 * 16), 128 * 16, 128),
                             tc::smem_desc(sb + k16 * 2 * (N * 16), N * 16, 128), idesc,
                             (i > 0 || k16 > 0) ? 1u : 0u);
            tc::commit(&empty[s]);
        }
        tc::commit(&done);  // arrives when every MMA issued above has completed
    }
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    // the accumulator is complete once `done` fires (after a failure: the MMAs in flight have ended)
    ok = __syncthreads_and((tc::mbar_wait(&done, 0, kWaitPolls) && ok) ? 1 : 0) != 0;
    tc::fence_after_sync();
    if (!ok)
    {
        if (tid == 0)
        {
            atomicOr(status, kStatusLookbackTimeout);
            // the copies of the last issued round of every stage must land before the block exits
            for (int i = max(0, issued_s - stages); i < issued_s; ++i)
                tc::mbar_wait(&full[i % stages], (uint32_t)((i / stages) & 1), kWaitPolls);
        }
    }
    else
    {
        const int64_t row = m0 + 32 * warp + lane;
#pragma unroll
        for (int c = 0; c < N / 16; ++c)
        {
            float v[16];
            tc::tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + 16 * c, v);
            // 16-byte stores: a row's 16 columns are 64 (fp32) or 32 (bf16) contiguous bytes
            if (H)
            {
                __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    h[j] = __float2bfloat16_rn(fmaxf(v[j] + bias[16 * c + j], 0.0f));
                uint4 *dst = reinterpret_cast<uint4 *>(H + row * N + 16 * c);
                dst[0] = reinterpret_cast<const uint4 *>(h)[0];
                dst[1] = reinterpret_cast<const uint4 *>(h)[1];
            }
            else
            {
                float4 *dst = reinterpret_cast<float4 *>(C + row * N + 16 * c);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                {
                    float4 o = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                    if (accumulate)
                    {
                        const float4 a = dst[j];
                        o.x += a.x;
                        o.y += a.y;
                        o.z += a.z;
                        o.w += a.w;
                    }
                    dst[j] = o;
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0)
        tc::tmem_dealloc(taddr, kCols);
}

// ------------------------------------------------------------------ fused inference
struct RadiusArgs
{
    const float *params;  // fp32 master parameters (kNumParams)
    const float *pts;
    int64_t n;
    float center[3], inv_half[3];
    float margin, floor_;
    float *r_near, *r_sil;  // either may be null
    uint32_t *status;
};

__device__ __forceinline__ void store_bf16x8(uint8_t *dst, const float *v)
{
    __align__(16) __nv_bfloat162 h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(h);
}

// shared memory: W1 (64x192) | W2, W3, W4 (64x64 each) | X features (128x192), bf16.
// H (128x64, the hidden layer feeding the next MMA) reuses X's space: X is dead
// once the first layer's MMAs have completed. 96 KB: two CTAs per SM.
constexpr uint32_t kSmW1 = 0, kSmW2 = kSmW1 + 64 * 192 * 2, kSmW3 = kSmW2 + 64 * 64 * 2, kSmW4 = kSmW3 + 64 * 64 * 2;
constexpr uint32_t kSmX = kSmW4 + 64 * 64 * 2, kSmH = kSmX, kSmBytes = kSmX + 128 * 192 * 2;
constexpr uint32_t kSbo192 = (192 / 8) * 128, kSbo64 = (64 / 8) * 128;

__global__ void __launch_bounds__(128) mlp_radius_kernel(RadiusArgs a)
{
    extern __shared__ __align__(128) uint8_t smem[];
    __shared__ float s_bias[4][kHid];
    __shared__ float s_w5[kOut][kHid];
    __shared__ float s_b5[kOut];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    const float *P = a.params;
    // weights -> bf16 core-matrix layout, resident for the CTA's lifetime
    for (int i = tid; i < 64 * 192; i += 128)
    {
        const int r = i / 192, k = i % 192;
        *reinterpret_cast<__nv_bfloat16 *>(smem + kSmW1 + tc::core_offset(r, k, 128, kSbo192)) =
            __float2bfloat16_rn(P[kW1 + i]);
    }
    const int woff[3] = {kW2, kW3, kW4};
    const uint32_t soff[3] = {kSmW2, kSmW3, kSmW4};
    for (int l = 0; l < 3; ++l)
        for (int i = tid; i < 64 * 64; i += 128)
        {
            const int r = i / 64, k = i % 64;
            *reinterpret_cast<__nv_bfloat16 *>(smem + soff[l] + tc::core_offset(r, k, 128, kSbo64)) =
                __float2bfloat16_rn(P[woff[l] + i]);
        }
    if (tid < kHid)
    {
        s_bias[0][tid] = P[kB1 + tid];
        s_bias[1][tid] = P[kB2 + tid];
        s_bias[2][tid] = P[kB3 + tid];
        s_bias[3][tid] = P[kB4 + tid];
        s_w5[0][tid] = P[kW5 + tid];
        s_w5[1][tid] = P[kW5 + kHid + tid];
    }
    if (tid < kOut)
        s_b5[tid] = P[kB5 + tid];
    if (warp == 0)
    {
        tc::tmem_alloc(&tmem_base, 64);
        tc::tmem_relinquish();
    }
    if (tid == 0)
        tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tmem_base;
    const uint32_t my_lane_addr = taddr + ((uint32_t)(32 * warp) << 16);
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 64);
    const uint32_t sX = tc::smem_u32(smem + kSmX), sH = tc::smem_u32(smem + kSmH);
    const uint32_t sW1 = tc::smem_u32(smem + kSmW1);
    const uint32_t sWl[3] = {tc::smem_u32(smem + kSmW2), tc::smem_u32(smem + kSmW3), tc::smem_u32(smem + kSmW4)};
    uint32_t phase = 0;
    bool ok = true;
    const int64_t tiles = (a.n + 127) / 128;
    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x)
    {
        const int64_t q = tile * 128 + tid;
        const bool valid = q < a.n;
        // Fourier features of this thread's point -> row tid of X
        float u[3] = {0.f, 0.f, 0.f};
        if (valid)
            for (int c = 0; c < 3; ++c)
                u[c] = (__ldg(a.pts + 3 * q + c) - a.center[c]) * a.inv_half[c];
        Octaves oct;
        oct.init(u);
#pragma unroll 1
        for (int k = 0; k < kFreq; k += 4)  // one octave: 24 features = 3 core-matrix columns
        {
            float f[24];
            oct.emit(f);
            oct.next();
#pragma unroll
            for (int j = 0; j < 3; ++j)
                store_bf16x8(smem + kSmX + tc::core_offset(tid, 6 * k + 8 * j, 128, kSbo192), f + 8 * j);
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        // four tensor-core layers; the activations stay in shared memory / TMEM
        for (int layer = 0; layer < 4 && ok; ++layer)
        {
            if (tid == 0)
            {
                tc::fence_after_sync();
                if (layer == 0)
                {
#pragma unroll
                    for (int s = 0; s < kIn / 16; ++s)
                        tc::mma_bf16(taddr, tc::smem_desc(sX + 256 * s, 128, kSbo192),
                                     tc::smem_desc(sW1 + 256 * s, 128, kSbo192), idesc, s > 0 ? 1u : 0u);
                }
                else
                {
#pragma unroll
                    for (int s = 0; s < kHid / 16; ++s)
                        tc::mma_bf16(taddr, tc::smem_desc(sH + 256 * s, 128, kSbo64),
                                     tc::smem_desc(sWl[layer - 1] + 256 * s, 128, kSbo64), idesc, s > 0 ? 1u : 0u);
                }
                tc::commit(&mbar);
            }
            ok = __syncthreads_and(tc::mbar_wait(&mbar, phase, kWaitPolls) ? 1 : 0) != 0;
            if (!ok)
                break;
            phase ^= 1u;
            tc::fence_after_sync();
            if (layer < 3)
            {
                // h = relu(acc + b) -> bf16 row tid of H (the next layer's A)
#pragma unroll
                for (int c = 0; c < 4; ++c)
                {
                    float v[16];
                    tc::tmem_ld16(my_lane_addr + 16 * c, v);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        v[j] = fmaxf(v[j] + s_bias[layer][16 * c + j], 0.0f);
                    store_bf16x8(smem + kSmH + tc::core_offset(tid, 16 * c, 128, kSbo64), v);
                    store_bf16x8(smem + kSmH + tc::core_offset(tid, 16 * c + 8, 128, kSbo64), v + 8);
                }
                tc::fence_proxy_async();
                tc::fence_before_sync();
                __syncthreads();
            }
            else
            {
                float o0 = s_b5[0], o1 = s_b5[1];
#pragma unroll
                for (int c = 0; c < 4; ++c)
                {
                    float v[16];
                    tc::tmem_ld16(my_lane_addr + 16 * c, v);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                    {
                        const float h = fmaxf(v[j] + s_bias[3][16 * c + j], 0.0f);
                        o0 += h * s_w5[0][16 * c + j];
                        o1 += h * s_w5[1][16 * c + j];
                    }
                }
                if (valid)
                {
                    if (a.r_near)
                        a.r_near[q] = __expf(o0) * a.margin + a.floor_;
                    if (a.r_sil)
                        a.r_sil[q] = __expf(o1) * a.margin + a.floor_;
                }
                tc::fence_before_sync();
                __syncthreads();  // TMEM and X are rewritten by the next tile
            }
        }
    }
    if (!ok)
    {
        if (tid == 0)
            atomicOr(a.status, kStatusLookbackTimeout);
        tc::mbar_wait(&mbar, phase, kWaitPolls);  // the MMAs in flight finish before TMEM is freed
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0)
        tc::tmem_dealloc(taddr, 64);
}

// ------------------------------------------------------------------ training kernels
// Fourier features of B points -> X [B x 192] bf16 (rows beyond n are zero)
__global__ void features_kernel(const float *__restrict__ pts, int64_t n, int64_t rows, float3 center, float3 inv_half,
                                __nv_bfloat16 *__restrict__ X)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= rows)
        return;
    float u[3] = {0.f, 0.f, 0.f};
    if (i < n)
    {
        u[0] = (pts[3 * i] - center.x) * inv_half.x;
        u[1] = (pts[3 * i + 1] - center.y) * inv_half.y;
        u[2] = (pts[3 * i + 2] - center.z) * inv_half.z;
    }
    Octaves oct;
    oct.init(u);
    for (int k = 0; k < kFreq; k += 4)
    {
        float f[24];
        oct.emit(f);
        oct.next();
        for (int j = 0; j < 24; ++j)
            X[i * kIn + 6 * k + j] = __float2bfloat16_rn(i < n ? f[j] : 0.f);
    }
}

// H = relu(Z + b) (bf16) for a [B x 64] pre-activation
// dst[c][r] = src[r][c] (bf16), dst has dst_rows >= cols rows (the rest zero)
__global__ void transpose_bf16_kernel(const __nv_bfloat16 *__restrict__ src, int64_t rows, int cols, int dst_rows,
                                      __nv_bfloat16 *__restrict__ dst)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)dst_rows * rows)
        return;
    const int c = (int)(i / rows);
    const int64_t r = i % rows;
    dst[i] = c < cols ? src[r * cols + c] : __float2bfloat16_rn(0.0f);
}

__global__ void to_bf16_kernel(const float *__restrict__ src, int64_t n, __nv_bfloat16 *__restrict__ dst)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n)
        dst[i] = __float2bfloat16_rn(src[i]);
}

// W^T as bf16: dst[c][r] = W[r][c] for a rows x cols fp32 matrix
__global__ void weight_t_bf16_kernel(const float *__restrict__ W, int rows, int cols, __nv_bfloat16 *__restrict__ dst)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rows * cols)
    {
        const int c = i / rows, r = i % rows;
        dst[i] = __float2bfloat16_rn(W[r * cols + c]);
    }
}

// head forward + pinball loss gradient + head gradients + dZ4 (masked by ReLU):
// one thread per sample, 128 per block, block-reduced head gradients.
// target[b][0..1] = log distances (NaN = masked out).
__global__ void __launch_bounds__(128) head_loss_kernel(const __nv_bfloat16 *__restrict__ H4,
                                                        const float *__restrict__ params,
                                                        const float *__restrict__ target, int64_t n, int64_t rows,
                                                        float tau, float inv_count, float *__restrict__ grad,
                                                        __nv_bfloat16 *__restrict__ dZ4, float *__restrict__ loss)
{
    __shared__ float s_g[2 * kHid + 2 + 1];
    for (int i = threadIdx.x; i < 2 * kHid + 3; i += blockDim.x)
        s_g[i] = 0.f;
    __syncthreads();
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const float *W5 = params + kW5, *b5 = params + kB5;
    float h[kHid];
    float d0 = 0.f, d1 = 0.f, l = 0.f;
    if (b < rows)
    {
#pragma unroll
        for (int i = 0; i < kHid; ++i)
            h[i] = __bfloat162float(H4[b * kHid + i]);
        if (b < n)
        {
            float o[2] = {b5[0], b5[1]};
#pragma unroll
            for (int i = 0; i < kHid; ++i)
            {
                o[0] += h[i] * W5[i];
                o[1] += h[i] * W5[kHid + i];
            }
            float d[2];
            for (int c = 0; c < 2; ++c)
            {
                const float y = target[2 * b + c];
                if (isnan(y))
                {
                    d[c] = 0.f;
                    continue;
                }
                const float r = y - o[c];  // pinball: tau * r if r > 0 else (tau - 1) * r
                l += r > 0.f ? tau * r : (tau - 1.f) * r;
                d[c] = (r > 0.f ? -tau : 1.f - tau) * inv_count;
            }
            d0 = d[0];
            d1 = d[1];
        }
#pragma unroll
        for (int i = 0; i < kHid; ++i)
        {
            const float dh = d0 * W5[i] + d1 * W5[kHid + i];
            dZ4[b * kHid + i] = __float2bfloat16_rn(h[i] > 0.f ? dh : 0.f);
        }
    }
    if (d0 != 0.f || d1 != 0.f)
    {
#pragma unroll 8
        for (int i = 0; i < kHid; ++i)
        {
            atomicAdd(&s_g[i], d0 * h[i]);
            atomicAdd(&s_g[kHid + i], d1 * h[i]);
        }
        atomicAdd(&s_g[2 * kHid], d0);
        atomicAdd(&s_g[2 * kHid + 1], d1);
    }
    if (l != 0.f)
        atomicAdd(&s_g[2 * kHid + 2], l * inv_count);
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * kHid + 2; i += blockDim.x)
        if (s_g[i] != 0.f)
            atomicAdd(grad + kW5 + i, s_g[i]);  // kW5 .. kW5+127 then kB5, kB5+1 are contiguous
    if (threadIdx.x == 0 && s_g[2 * kHid + 2] != 0.f)
        atomicAdd(loss, s_g[2 * kHid + 2]);
}

// dZ = dH * (H > 0) as bf16; also accumulates the bias gradient (column sums)
__global__ void relu_back_kernel(const float *__restrict__ dH, const __nv_bfloat16 *__restrict__ H, int64_t rows,
                                 __nv_bfloat16 *__restrict__ dZ, float *__restrict__ db)
{
    __shared__ float s_db[kHid];
    if (threadIdx.x < kHid)
        s_db[threadIdx.x] = 0.f;
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < rows * kHid)
    {
        const float g = __bfloat162float(H[i]) > 0.f ? dH[i] : 0.f;
        dZ[i] = __float2bfloat16_rn(g);
        atomicAdd(&s_db[i % kHid], g);
    }
    __syncthreads();
    if (threadIdx.x < kHid && s_db[threadIdx.x] != 0.f)
        atomicAdd(db + threadIdx.x, s_db[threadIdx.x]);
}

// bias gradient of the last hidden layer from dZ4 (bf16)
__global__ void colsum_bf16_kernel(const __nv_bfloat16 *__restrict__ dZ, int64_t rows, float *__restrict__ db)
{
    __shared__ float s_db[kHid];
    if (threadIdx.x < kHid)
        s_db[threadIdx.x] = 0.f;
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < rows * kHid)
        atomicAdd(&s_db[i % kHid], __bfloat162float(dZ[i]));
    __syncthreads();
    if (threadIdx.x < kHid && s_db[threadIdx.x] != 0.f)
        atomicAdd(db + threadIdx.x, s_db[threadIdx.x]);
}

// dW[o][i] += sum over the K splits of C[s][i][o], for the first `in` rows of a
// split weight-gradient GEMM result (slices of split_stride floats, each rows x 64)
__global__ void add_wgrad_kernel(const float *__restrict__ C, int in, int splits, int64_t split_stride,
                                 float *__restrict__ dW)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < in * kHid)
    {
        const int o = t / in, i = t % in;
        float acc = 0.f;
        for (int s = 0; s < splits; ++s)
            acc += C[s * split_stride + i * kHid + o];
        dW[o * in + i] += acc;
    }
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float b1, float b2, float c1, float c2, float eps)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace mlp

// ------------------------------------------------------------------ host entry points (internal)
size_t mlp_num_params() { return mlp::kNumParams; }

namespace
{
// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}
// a rows x K bf16 row-major matrix, boxes of 8 columns (16 bytes) x box_rows rows
cudaError_t bf16_map(CUtensorMap *m, const void *base, int64_t rows, int64_t K, uint32_t box_rows)
{
    EncodeTiledFn f = encode_tiled();
    if (!f)
        return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {8, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = f(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}
}  // namespace

cudaError_t launch_gemm_bf16_ex(const void *A, const void *B, float *C, const float *bias, void *H, int64_t M,
                                int64_t N, int64_t K, int accumulate, uint32_t *status, cudaStream_t st, int splits)
{
    using namespace mlp;
    // TMA reads A and B, and the epilogue writes C / H, in 16-byte units
    if (M <= 0 || M % 128 || K <= 0 || K % 64 || (H && (N != 64 || !bias)) ||
        (reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B) | reinterpret_cast<uintptr_t>(C) |
         reinterpret_cast<uintptr_t>(H)) % 16)
        return cudaErrorInvalidValue;
    // every split gets at least one 64-column chunk, so every slice is written
    const int64_t chunks = K / 64;
    splits = (int)std::max<int64_t>(1, std::min<int64_t>(splits, chunks));
    const int k_split = (int)((chunks + splits - 1) / splits * 64);
    splits = (int)((K + k_split - 1) / k_split);
    // four stages (a ring sized to the chunks of a split, one stage for K = 64, measured
    // slower: more resident blocks, slower per launch)
    const size_t smem = 4 * ((size_t)128 * 64 * 2 + (size_t)N * 64 * 2) + 1024;
    const dim3 grid((unsigned)(M / 128), (unsigned)splits);
    CUtensorMap ta, tb;
    cudaError_t e = bf16_map(&ta, A, M, K, 128);
    if (e == cudaSuccess)
        e = bf16_map(&tb, B, N, K, (uint32_t)N);
    if (e != cudaSuccess)
        return e;
    auto *h = static_cast<__nv_bfloat16 *>(H);
    switch (N)
    {
#define SNCH_GEMM_CASE(NN)                                                                                          \
    case NN:                                                                                                        \
        e = cudaFuncSetAttribute(gemm_bf16_kernel<NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);     \
        if (e == cudaSuccess)                                                                                       \
            gemm_bf16_kernel<NN><<<grid, 128, smem, st>>>(ta, tb, C, bias, h, (int)K, k_split, accumulate, status); \
        break;
        SNCH_GEMM_CASE(64)
        SNCH_GEMM_CASE(128)
        SNCH_GEMM_CASE(192)
        SNCH_GEMM_CASE(256)
#undef SNCH_GEMM_CASE
    default:
        return cudaErrorInvalidValue;
    }
    note_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_gemm_bf16(const void *A, const void *B, float *C, int64_t M, int64_t N, int64_t K, int accumulate,
                             uint32_t *status, cudaStream_t st, int splits)
{
    return launch_gemm_bf16_ex(A, B, C, nullptr, nullptr, M, N, K, accumulate, status, st, splits);
}

cudaError_t set_mlp_scales(const float *scales)
{
    return cudaMemcpyToSymbol(mlp::c_scale, scales, sizeof(float) * mlp::kFreq);
}

cudaError_t launch_mlp_radius(const float *params, const float *pts, int64_t n, const float center[3],
                              const float inv_half[3], float margin, float floor_, float *r_near, float *r_sil,
                              uint32_t *status, cudaStream_t st)
{
    using namespace mlp;
    if (n <= 0)
        return cudaSuccess;
    RadiusArgs a;
    a.params = params;
    a.pts = pts;
    a.n = n;
    for (int c = 0; c < 3; ++c)
    {
        a.center[c] = center[c];
        a.inv_half[c] = inv_half[c];
    }
    a.margin = margin;
    a.floor_ = floor_;
    a.r_near = r_near;
    a.r_sil = r_sil;
    a.status = status;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(mlp_radius_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmBytes);
    if (e != cudaSuccess)
        return e;
    const int64_t tiles = (n + 127) / 128;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, (int64_t)sms * 2);
    mlp_radius_kernel<<<grid, 128, kSmBytes, st>>>(a);
    note_launch();
    return cudaGetLastError();
}

// One gradient evaluation over rows (multiple of 128) samples, n of them real:
// forward through the tensor-core GEMMs, pinball loss on the two log-distance
// outputs, backward (weight gradients dW^T = A^T dZ and input gradients dZ W
// on the tensor cores); the gradient is left in grad (fp32, kNumParams).
cudaError_t mlp_forward_backward(float *params, float *grad, const float *pts, const float *target, int64_t n,
                                 int64_t rows, const float center[3], const float inv_half[3], float tau,
                                 const MlpWorkspace &ws, float *loss, uint32_t *status, cudaStream_t st)
{
    using namespace mlp;
    cudaError_t e;
    const int T = 256;
    const float3 c3 = make_float3(center[0], center[1], center[2]);
    const float3 ih3 = make_float3(inv_half[0], inv_half[1], inv_half[2]);
    auto *X = static_cast<__nv_bfloat16 *>(ws.X);
    __nv_bfloat16 *H[4], *dZ[4];
    for (int l = 0; l < 4; ++l)
    {
        H[l] = static_cast<__nv_bfloat16 *>(ws.H[l]);
        dZ[l] = static_cast<__nv_bfloat16 *>(ws.dZ[l]);
    }
    auto *Tb = static_cast<__nv_bfloat16 *>(ws.T);
    auto *Tb2 = static_cast<__nv_bfloat16 *>(ws.T2);
    auto *Wt = static_cast<__nv_bfloat16 *>(ws.Wt);
    auto *Wb = static_cast<__nv_bfloat16 *>(ws.Wb);
    float *dH = ws.dH, *C = ws.C;
    if ((e = cudaMemsetAsync(grad, 0, sizeof(float) * kNumParams, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(loss, 0, sizeof(float), st)) != cudaSuccess)
        return e;
    // bf16 weights (row-major [out x in]) for the forward GEMMs
    const int woff[4] = {kW1, kW2, kW3, kW4};
    const int win[4] = {kIn, kHid, kHid, kHid};
    const int boff[4] = {kB1, kB2, kB3, kB4};
    const int64_t wbo[4] = {0, 64 * 192, 64 * 192 + 4096, 64 * 192 + 8192};
    for (int l = 0; l < 4; ++l)
    {
        to_bf16_kernel<<<blocks(64 * win[l], T), T, 0, st>>>(params + woff[l], 64 * win[l], Wb + wbo[l]);
        note_launch();
    }
    features_kernel<<<blocks(rows, T), T, 0, st>>>(pts, n, rows, c3, ih3, X);
    note_launch();
    // forward
    const __nv_bfloat16 *in = X;
    for (int l = 0; l < 4; ++l)
    {
        // H_l = bf16(max(in W_l^T + b_l, 0)), bias and ReLU in the GEMM's epilogue
        if ((e = launch_gemm_bf16_ex(in, Wb + wbo[l], nullptr, params + boff[l], H[l], rows, 64, win[l], 0, status,
                                     st, 1)) != cudaSuccess)
            return e;
        in = H[l];
    }
    head_loss_kernel<<<blocks(rows, 128), 128, 0, st>>>(H[3], params, target, n, rows, tau,
                                                         1.0f / (float)(n > 0 ? n : 1), grad, dZ[3], loss);
    note_launch();
    colsum_bf16_kernel<<<blocks(rows * 64, T), T, 0, st>>>(dZ[3], rows, grad + kB4);
    note_launch();
    // backward: weight gradients dW_l^T = A_{l-1}^T dZ_l and input gradients dH_{l-1} = dZ_l W_l
    for (int l = 3; l >= 0; --l)
    {
        const __nv_bfloat16 *Ain = l == 0 ? X : H[l - 1];
        const int inw = win[l];
        const int mpad = inw <= 128 ? 128 : 256;
        transpose_bf16_kernel<<<blocks((int64_t)mpad * rows, T), T, 0, st>>>(Ain, rows, inw, mpad, Tb);
        note_launch();
        transpose_bf16_kernel<<<blocks((int64_t)64 * rows, T), T, 0, st>>>(dZ[l], rows, 64, 64, Tb2);
        note_launch();
        const int splits = (int)std::min<int64_t>(kMaxWgradSplits, std::max<int64_t>(1, rows / 2048));
        if ((e = launch_gemm_bf16(Tb, Tb2, C, mpad, 64, rows, 0, status, st, splits)) != cudaSuccess)
            return e;
        const int64_t ch = rows / 64;  // the split count launch_gemm_bf16 settles on
        const int64_t ks = (ch + splits - 1) / splits;
        add_wgrad_kernel<<<blocks(inw * 64, T), T, 0, st>>>(C, inw, (int)((ch + ks - 1) / ks), (int64_t)mpad * 64,
                                                            grad + woff[l]);
        note_launch();
        if (l == 0)
            break;
        weight_t_bf16_kernel<<<blocks(64 * 64, T), T, 0, st>>>(params + woff[l], 64, 64, Wt);
        note_launch();
        if ((e = launch_gemm_bf16(dZ[l], Wt, dH, rows, 64, 64, 0, status, st)) != cudaSuccess)
            return e;
        relu_back_kernel<<<blocks(rows * 64, T), T, 0, st>>>(dH, H[l - 1], rows, dZ[l - 1], grad + boff[l - 1]);
        note_launch();
    }
    return cudaGetLastError();
}

cudaError_t mlp_adam(float *params, const float *grad, float *m, float *v, float lr, int step, cudaStream_t st)
{
    using namespace mlp;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<blocks(kNumParams, 256), 256, 0, st>>>(params, grad, m, v, kNumParams, lr, b1, b2, c1, c2, 1e-8f);
    note_launch();
    return cudaGetLastError();
}

}  // namespace snch
