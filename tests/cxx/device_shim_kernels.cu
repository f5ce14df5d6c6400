// A caller's own kernels written against include/snch_device.cuh, in the call
// forms of the reference's per-thread device API (query.cuh:82-423,
// sample.cuh:10-91). Compiled by tests/test_gpu_device_shim.py with nvcc's
// default flags (FMA contraction on) into a shared library whose extern "C"
// launchers the test calls; the results must equal the library's own kernels.
#include <snch_device.cuh>

namespace
{
__device__ float3 f3at(const float *p, int i) { return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

__global__ void nearest_k(snch_traversal_view v, const float *pts, int n, unsigned *idx, float *dist)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const auto r = snch::query_device(v, snch::nearest(f3at(pts, i)), snch::scene3::distance_calculator());
    idx[i] = r.first;
    dist[i] = r.second;
}

__global__ void silhouette_k(snch_traversal_view v, const float *pts, const unsigned char *flip, int n, float *dist,
                             int *edge)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    // divergent on purpose: odd lanes use the reference's float-returning form,
    // even lanes the form that also returns the edge
    if (i & 1)
    {
        dist[i] = snch::query_device(v, snch::nearest_silhouette(f3at(pts, i), flip[i] != 0),
                                     snch::scene3::silhouette_distance_calculator());
        edge[i] = snch::query_device(v, snch::nearest_silhouette_edge(f3at(pts, i), flip[i] != 0)).second;
    }
    else
    {
        const auto r = snch::query_device(v, snch::nearest_silhouette_edge(f3at(pts, i), flip[i] != 0));
        dist[i] = r.first;
        edge[i] = r.second;
    }
}

__global__ void ray_k(snch_traversal_view v, const float *o, const float *d, const float *tmax, int n,
                      unsigned char *hit, float *t, float *uv, unsigned *idx, unsigned char *any)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const snch::ray r(f3at(o, i), f3at(d, i));
    const auto h = snch::query_device(v, snch::ray_intersect(r, tmax[i]), snch::scene3::intersect_test());
    hit[i] = thrust::get<0>(h) ? 1 : 0;
    t[i] = thrust::get<1>(h);
    uv[2 * i] = thrust::get<2>(h).x;
    uv[2 * i + 1] = thrust::get<2>(h).y;
    idx[i] = thrust::get<3>(h);
    any[i] = snch::query_device(v, snch::ray_intersect<true>(r, tmax[i])) ? 1 : 0;
}

__global__ void sample_k(snch_traversal_view v, const float *c, const float *rad, const float *u, const float *u2,
                         const float *v2, int n, int *idx, float *pdf, float *pt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const auto s = snch::sample_object_in_sphere(v, snch::sphere_intersect(snch::sphere(f3at(c, i), rad[i])),
                                                 snch::scene3::intersect_sphere(), snch::scene3::measurement_getter(),
                                                 snch::scene3::green_weight(), u[i]);
    idx[i] = s.first;
    pdf[i] = s.second;
    const float3 p = snch::sample_on_object(v, s.first, snch::scene3::sample_on_object(), u2[i], v2[i]);
    pt[3 * i] = p.x;
    pt[3 * i + 1] = p.y;
    pt[3 * i + 2] = p.z;
}

unsigned blocks(int n) { return (unsigned)((n + 127) / 128); }
}  // namespace

extern "C" {
int shim_nearest(const snch_traversal_view *v, const float *pts, int n, unsigned *idx, float *dist)
{
    if (n > 0)
        nearest_k<<<blocks(n), 128>>>(*v, pts, n, idx, dist);
    return (int)cudaDeviceSynchronize();
}
int shim_silhouette(const snch_traversal_view *v, const float *pts, const unsigned char *flip, int n, float *dist,
                    int *edge)
{
    if (n > 0)
        silhouette_k<<<blocks(n), 128>>>(*v, pts, flip, n, dist, edge);
    return (int)cudaDeviceSynchronize();
}
int shim_ray(const snch_traversal_view *v, const float *o, const float *d, const float *tmax, int n,
             unsigned char *hit, float *t, float *uv, unsigned *idx, unsigned char *any)
{
    if (n > 0)
        ray_k<<<blocks(n), 128>>>(*v, o, d, tmax, n, hit, t, uv, idx, any);
    return (int)cudaDeviceSynchronize();
}
int shim_sample(const snch_traversal_view *v, const float *c, const float *r, const float *u, const float *u2,
                const float *v2, int n, int *idx, float *pdf, float *pt)
{
    if (n > 0)
        sample_k<<<blocks(n), 128>>>(*v, c, r, u, u2, v2, n, idx, pdf, pt);
    return (int)cudaDeviceSynchronize();
}
}
