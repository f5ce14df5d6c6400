// The reference's own per-thread CUDA queries, wrapped in extern "C" kernels --
// TEST INFRASTRUCTURE ONLY (parity and the timed reference arm).
//
// Each kernel is the reference's benchmark pattern (benchmark.cu:400-405, one
// thread per query calling lbvh::query_device / sample_object_in_sphere with the
// scene<3> functors) compiled from the UNMODIFIED reference headers by
// oracle/Makefile into a device-only cubin for sm_103a with the reference's own
// flags (default -fmad, --extended-lambda --expt-relaxed-constexpr,
// CMakeLists.txt:35-44). The tree argument is the byte-compatible view that
// snch_get_bvh_view() returns, so the reference's traversal code runs over a
// tree built by this project.
#include <unordered_map>  // scene.cuh uses std::unordered_map without including it

#include "snch_lbvh/lbvh.cuh"
#include "snch_lbvh/scene.cuh"

using ref_view = lbvh::bvh_device<float, 3, lbvh::scene<3>::triangle>;

extern "C" __global__ void ref_nearest(ref_view bvh, const float3 *pts, int n, unsigned int *idx, float *dist)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const auto r = lbvh::query_device(bvh, lbvh::nearest(pts[i]), lbvh::scene<3>::distance_calculator());
    idx[i] = r.first;
    dist[i] = r.second;
}

extern "C" __global__ void ref_silhouette(ref_view bvh, const float3 *pts, const unsigned char *flip, int n,
                                          float *dist)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    dist[i] = lbvh::query_device(bvh, lbvh::nearest_silhouette(pts[i], flip ? flip[i] != 0 : false),
                                 lbvh::scene<3>::silhouette_distance_calculator());
}

extern "C" __global__ void ref_ray(ref_view bvh, const float3 *o, const float3 *d, const float *tmax, int n,
                                   unsigned char *hit, float *t, unsigned int *idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const auto r = lbvh::query_device(bvh, lbvh::ray_intersect(lbvh::ray<float, 3>(o[i], d[i]), tmax[i]),
                                      lbvh::scene<3>::intersect_test());
    hit[i] = thrust::get<0>(r) ? 1 : 0;
    t[i] = thrust::get<1>(r);
    idx[i] = thrust::get<3>(r);
}

extern "C" __global__ void ref_sample(ref_view bvh, const float3 *c, const float *r, const float *u, int n, int *idx,
                                      float *pdf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const auto s = lbvh::sample_object_in_sphere(bvh, lbvh::sphere_intersect(lbvh::sphere<float, 3>(c[i], r[i])),
                                                 lbvh::scene<3>::intersect_sphere(),
                                                 lbvh::scene<3>::measurement_getter(), lbvh::scene<3>::green_weight(),
                                                 u[i]);
    idx[i] = s.first;
    pdf[i] = s.first >= 0 ? s.second : 0.0f;
}
