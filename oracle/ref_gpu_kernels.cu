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

// The same query returning, besides the distance, the silhouette edge it ended
// on (the reference computes it but does not return it, query.cuh:382-386). The
// functor evaluates the owned edges exactly as silhouette_distance_calculator
// does (scene.cuh:978-1003, the reference's own find_closest_silhouette_point
// per edge) and repeats the traversal's own acceptance test
// (`found && dist <= best`, query.cuh:380) on the same values, so the edge it
// records is the one whose distance the traversal keeps.
struct edge_recording_calculator
{
    float *best;
    int *edge;
    __device__ bool operator()(const float3 origin, const lbvh::scene<3>::triangle &object,
                               const float max_radius_squared, float &distance, const bool flip,
                               const float min_radius_squared) const noexcept
    {
        float max_r2 = max_radius_squared;
        bool ret = false;
        int found_edge = -1;
        for (int i = 0; i < 3; ++i)
        {
            const int si = i == 0 ? object.silhouette_indices.x
                                  : (i == 1 ? object.silhouette_indices.y : object.silhouette_indices.z);
            if (si != -1 && object.silhouettes[si].find_closest_silhouette_point(origin, max_r2, distance, flip,
                                                                                 min_radius_squared))
            {
                ret = true;
                found_edge = si;
                max_r2 = distance * distance;
            }
        }
        if (ret && distance <= *best)
        {
            *best = distance;
            *edge = found_edge;
        }
        return ret;
    }
};

extern "C" __global__ void ref_silhouette_edge(ref_view bvh, const float3 *pts, const unsigned char *flip, int n,
                                               float *dist, int *edge)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float best = INFINITY;
    int e = -1;
    dist[i] = lbvh::query_device(bvh, lbvh::nearest_silhouette(pts[i], flip ? flip[i] != 0 : false),
                                 edge_recording_calculator{&best, &e});
    edge[i] = e;
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

// the same closest-hit query, also returning the hit's barycentric (u, v)
extern "C" __global__ void ref_ray_uv(ref_view bvh, const float3 *o, const float3 *d, const float *tmax, int n,
                                      unsigned char *hit, float *t, float2 *uv, unsigned int *idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const auto r = lbvh::query_device(bvh, lbvh::ray_intersect(lbvh::ray<float, 3>(o[i], d[i]), tmax[i]),
                                      lbvh::scene<3>::intersect_test());
    hit[i] = thrust::get<0>(r) ? 1 : 0;
    t[i] = thrust::get<1>(r);
    uv[i] = thrust::get<2>(r);
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
