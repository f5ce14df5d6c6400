// Wavefront walk-on-stars (Sawhney et al. 2023, "Walk on Stars") over the four
// queries of this library: the consumer the SNCH-LBVH exists for. Every step
// of every live walker issues one nearest-primitive query on the Dirichlet
// boundary, one nearest-silhouette query on the Neumann boundary, one ray
// inside the star and one SampleTriangleInSphere draw on the Neumann boundary;
// walkers that reach the Dirichlet shell leave, the rest are compacted so the
// next step's batches are dense. The kernels here are the walker updates
// between the batched queries (the queries themselves are the library's).
//
// The boundary data are those of the harmonic function u(x) = x_0 (the first
// coordinate): g = x_0 on the Dirichlet faces, h = n_0 (outward normal) on
// the Neumann faces, so every walker's estimate has expectation x_0 of its
// start point up to the epsilon-shell bias; this is what the tests check.
//
// Estimator per walk (star radius R = min(d_Dirichlet, d_silhouette)):
//   total += alpha G_R(x, y) h(y) / pdf(y)   (y: a Neumann point drawn in the ball,
//                                             alpha = 2 on the Neumann boundary, else 1,
//                                             G_R = (1/r - 1/R) / (4 pi))
//   x <- first Neumann hit of a uniform direction (hemisphere into the domain when
//        x is on the Neumann boundary) within R, else the point at distance R
//   at d_Dirichlet < epsilon: estimate = total + g(x)
#include "internal.h"

namespace snch
{
namespace
{

SNCH_DEV uint64_t wmix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// uniform in [0, 1) from (seed, walker, step, stream k)
SNCH_DEV float wrand(uint64_t seed, uint32_t id, uint32_t step, uint32_t k)
{
    const uint64_t h = wmix(seed ^ wmix(((uint64_t)id << 32) ^ ((uint64_t)step << 8) ^ k ^ 0x9E3779B97F4A7C15ull));
    return (float)(h >> 40) * (1.0f / 16777216.0f);
}

SNCH_DEV f3 face_normal(const float *verts, const int32_t *tris, int32_t t, float *area)
{
    const int32_t *f = tris + 3 * (int64_t)t;
    const f3 a = load_vert(verts, f[0]), b = load_vert(verts, f[1]), c = load_vert(verts, f[2]);
    const f3 n = cross3(sub(b, a), sub(c, a));
    const float l = len3(n);
    if (area)
        *area = 0.5f * l;
    return l > 0.f ? mk(n.x / l, n.y / l, n.z / l) : mk(0.f, 0.f, 0.f);
}

__global__ void wost_init_kernel(WalkState s, int64_t n, f3 center, float radius, uint64_t seed, float *start)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t id = (uint32_t)i;
    f3 p = mk(0.f, 0.f, 0.f);
    for (uint32_t k = 0; k < 64; ++k)  // rejection sampling of the unit ball (accepts 52 %)
    {
        const f3 q = mk(2.f * wrand(seed, id, 0xFFFFFFu, 3 * k) - 1.f, 2.f * wrand(seed, id, 0xFFFFFFu, 3 * k + 1) - 1.f,
                        2.f * wrand(seed, id, 0xFFFFFFu, 3 * k + 2) - 1.f);
        if (q.x * q.x + q.y * q.y + q.z * q.z <= 1.f)
        {
            p = q;
            break;
        }
    }
    const f3 x = mk(center.x + radius * p.x, center.y + radius * p.y, center.z + radius * p.z);
    s.x[3 * i] = x.x;
    s.x[3 * i + 1] = x.y;
    s.x[3 * i + 2] = x.z;
    s.on_b[i] = 0;
    s.total[i] = 0.f;
    s.id[i] = id;
    if (start)
    {
        start[3 * i] = x.x;
        start[3 * i + 1] = x.y;
        start[3 * i + 2] = x.z;
    }
}

// Termination test and, for the walkers that go on, compaction into `out`
// plus the inputs of the ray and sphere-sample batches.
__global__ void wost_prepare_kernel(WalkState in, int64_t n, const float *__restrict__ d_dir,
                                    const float *__restrict__ d_sil, WalkState out, WalkStep step_in, uint32_t step,
                                    uint32_t last_step, float eps, uint64_t seed, float *__restrict__ estimates,
                                    uint32_t *__restrict__ counts)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool live = false;
    f3 x = mk(0.f, 0.f, 0.f);
    float R = 0.f;
    uint32_t id = 0;
    if (i < n)
    {
        x = mk(in.x[3 * i], in.x[3 * i + 1], in.x[3 * i + 2]);
        id = in.id[i];
        const float dd = d_dir[i];
        const float ds = d_sil ? d_sil[i] : INFINITY;
        R = fminf(dd, ds);
        if (dd < eps || step >= last_step || !(R > 0.f))
        {
            estimates[id] = in.total[i] + x.x;  // g(x) = x_0 at the walk's last point
            if (dd < eps)
                atomicAdd(counts + 1, 1u);
        }
        else
            live = true;
    }
    // warp-aggregated append
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, live);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0 && mask)
        base = atomicAdd(counts, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (!live)
        return;
    const uint32_t j = base + __popc(mask & ((1u << lane) - 1u));
    const bool on_b = in.on_b[i] != 0;
    const f3 nb = on_b ? mk(in.nb[3 * i], in.nb[3 * i + 1], in.nb[3 * i + 2]) : mk(0.f, 0.f, 0.f);
    // uniform direction; on the Neumann boundary the hemisphere into the domain (-nb side)
    const float z = 1.f - 2.f * wrand(seed, id, step, 0), ph = 6.283185307f * wrand(seed, id, step, 1);
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    f3 d = mk(r * cosf(ph), r * sinf(ph), z);
    if (on_b && d.x * nb.x + d.y * nb.y + d.z * nb.z > 0.f)
        d = mk(-d.x, -d.y, -d.z);
    out.x[3 * j] = x.x;
    out.x[3 * j + 1] = x.y;
    out.x[3 * j + 2] = x.z;
    out.nb[3 * j] = nb.x;
    out.nb[3 * j + 1] = nb.y;
    out.nb[3 * j + 2] = nb.z;
    out.on_b[j] = on_b ? 1 : 0;
    out.total[j] = in.total[i];
    out.id[j] = id;
    step_in.dir[3 * j] = d.x;
    step_in.dir[3 * j + 1] = d.y;
    step_in.dir[3 * j + 2] = d.z;
    step_in.radius[j] = R;
    step_in.u[j] = wrand(seed, id, step, 2);
    step_in.su[j] = wrand(seed, id, step, 3);
    step_in.sv[j] = wrand(seed, id, step, 4);
}

// Neumann source term of the star and the move to the next point.
__global__ void wost_update_kernel(WalkState s, int64_t n, WalkStep st, const float *__restrict__ nverts,
                                   const int32_t *__restrict__ ntris)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const f3 x = mk(s.x[3 * i], s.x[3 * i + 1], s.x[3 * i + 2]);
    const float R = st.radius[i];
    float total = s.total[i];
    const bool on_b = s.on_b[i] != 0;
    if (st.smp_idx)
    {
        const int32_t t = st.smp_idx[i];
        const float pdf = st.smp_pdf[i];
        if (t >= 0 && pdf > 0.f)
        {
            const f3 y = mk(st.smp_pt[3 * i], st.smp_pt[3 * i + 1], st.smp_pt[3 * i + 2]);
            const float r = len3(sub(y, x));
            if (r > 0.f && r < R)
            {
                const f3 nrm = face_normal(nverts, ntris, t, nullptr);
                const float G = (1.f / r - 1.f / R) * (1.f / (4.f * 3.14159265358979f));
                total += (on_b ? 2.f : 1.f) * G * nrm.x / pdf;
            }
        }
    }
    const f3 d = mk(st.dir[3 * i], st.dir[3 * i + 1], st.dir[3 * i + 2]);
    f3 xn;
    if (st.hit && st.hit[i])
    {
        const float t = st.t[i];
        const f3 nb = face_normal(nverts, ntris, (int32_t)st.hit_idx[i], nullptr);
        // on the boundary, nudged into the domain so the next ray leaves it
        xn = mk(x.x + t * d.x - 1e-6f * nb.x, x.y + t * d.y - 1e-6f * nb.y, x.z + t * d.z - 1e-6f * nb.z);
        s.on_b[i] = 1;
        s.nb[3 * i] = nb.x;
        s.nb[3 * i + 1] = nb.y;
        s.nb[3 * i + 2] = nb.z;
    }
    else
    {
        xn = mk(x.x + R * d.x, x.y + R * d.y, x.z + R * d.z);
        s.on_b[i] = 0;
    }
    s.x[3 * i] = xn.x;
    s.x[3 * i + 1] = xn.y;
    s.x[3 * i + 2] = xn.z;
    s.total[i] = total;
}

inline unsigned wgrid(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

cudaError_t launch_wost_init(const WalkState &s, int64_t n, const float center[3], float radius, uint64_t seed,
                             float *start, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    const f3 c{center[0], center[1], center[2]};
    wost_init_kernel<<<wgrid(n), 256, 0, st>>>(s, n, c, radius, seed, start);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_wost_prepare(const WalkState &in, int64_t n, const float *d_dir, const float *d_sil,
                                const WalkState &out, const WalkStep &step_in, uint32_t step, uint32_t last_step,
                                float eps, uint64_t seed, float *estimates, uint32_t *counts, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    wost_prepare_kernel<<<wgrid(n), 256, 0, st>>>(in, n, d_dir, d_sil, out, step_in, step, last_step, eps, seed,
                                                  estimates, counts);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_wost_update(const WalkState &s, int64_t n, const WalkStep &step, const float *nverts,
                               const int32_t *ntris, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    wost_update_kernel<<<wgrid(n), 256, 0, st>>>(s, n, step, nverts, ntris);
    note_launch();
    return cudaGetLastError();
}

}  // namespace snch
