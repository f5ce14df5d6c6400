// snch_gb300.hpp -- C++ host API over the C ABI (snch_gb300.h), shaped like
// the reference's lbvh::scene<3> (tyanyuy3125/snch-lbvh include/snch_lbvh/scene.cuh:704-1267)
// so that host code written against the reference switches by renaming the
// namespace: same member names, same call order, same error text.
//
//   snch::scene3 s(vertices.begin(), vertices.end(), faces.begin(), faces.end());
//   s.compute_silhouettes();
//   s.build_bvh();
//   const snch_bvh_view &v = s.get_bvh_device_ptr();   // reference device layout
//   s.query_nearest(d_points, n, d_index, d_dist);     // batched, on a stream
//
// Errors are thrown as std::runtime_error carrying snch_last_error(), as the
// reference throws std::runtime_error("BVH is not built yet.") (scene.cuh:1250).
#pragma once

#include <cstdint>
#include <iterator>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "snch_gb300.h"

namespace snch
{

inline void check(int rc)
{
    if (rc != SNCH_OK)
        throw std::runtime_error(snch_last_error());
}

class scene3
{
  public:
    scene3() = default;

    // scene<3>(vertices_first, vertices_last, indices_first, indices_last):
    // iterators over float3-like (x, y, z members) vertices and int3-like faces
    template <typename VertexIt, typename IndexIt>
    scene3(VertexIt vertices_first, VertexIt vertices_last, IndexIt indices_first, IndexIt indices_last)
    {
        std::vector<float> v;
        std::vector<int32_t> f;
        for (auto it = vertices_first; it != vertices_last; ++it)
        {
            v.push_back(static_cast<float>(it->x));
            v.push_back(static_cast<float>(it->y));
            v.push_back(static_cast<float>(it->z));
        }
        for (auto it = indices_first; it != indices_last; ++it)
        {
            f.push_back(static_cast<int32_t>(it->x));
            f.push_back(static_cast<int32_t>(it->y));
            f.push_back(static_cast<int32_t>(it->z));
        }
        check(snch_scene_create(v.data(), static_cast<int64_t>(v.size() / 3), f.data(),
                                static_cast<int64_t>(f.size() / 3), &h_));
    }

    // from flat arrays (xyz triples, index triples)
    scene3(const float *vertices_xyz, int64_t num_vertices, const int32_t *triangles, int64_t num_triangles)
    {
        check(snch_scene_create(vertices_xyz, num_vertices, triangles, num_triangles, &h_));
    }

    scene3(const scene3 &) = delete;
    scene3 &operator=(const scene3 &) = delete;
    scene3(scene3 &&o) noexcept : h_(std::exchange(o.h_, nullptr)), view_(o.view_) {}
    scene3 &operator=(scene3 &&o) noexcept
    {
        if (this != &o)
        {
            reset();
            h_ = std::exchange(o.h_, nullptr);
            view_ = o.view_;
        }
        return *this;
    }
    ~scene3() { reset(); }

    void compute_silhouettes(snch_stream_t stream = nullptr) { check(snch_compute_silhouettes(h_, stream)); }
    void build_bvh(snch_stream_t stream = nullptr)
    {
        check(snch_build_bvh(h_, stream));
        check(snch_get_bvh_view(h_, &view_));
    }
    // scene<3>::get_bvh_device_ptr(): throws "BVH is not built yet." before build_bvh()
    const snch_bvh_view &get_bvh_device_ptr()
    {
        check(snch_get_bvh_view(h_, &view_));
        return view_;
    }

    // batched device queries (query.cuh / sample.cuh semantics, see snch_gb300.h)
    void query_nearest(const float *points_xyz, int64_t n, uint32_t *index, float *distance,
                       snch_stream_t stream = nullptr) const
    {
        check(snch_query_nearest(h_, points_xyz, n, index, distance, stream));
    }
    void query_silhouette(const float *points_xyz, const uint8_t *flip, int64_t n, float *distance,
                          int32_t *edge = nullptr, snch_stream_t stream = nullptr) const
    {
        check(snch_query_silhouette(h_, points_xyz, flip, n, distance, edge, stream));
    }
    void query_ray(const float *origins_xyz, const float *dirs_xyz, const float *tmax, int64_t n, uint8_t *hit,
                   float *t, float *uv, uint32_t *index, snch_stream_t stream = nullptr) const
    {
        check(snch_query_ray(h_, origins_xyz, dirs_xyz, tmax, n, hit, t, uv, index, stream));
    }
    void sample_in_sphere(const float *centers_xyz, const float *radii, const float *u, int64_t n, int32_t *index,
                          float *pdf, snch_stream_t stream = nullptr) const
    {
        check(snch_sample_in_sphere(h_, centers_xyz, radii, u, n, index, pdf, stream));
    }
    void sample_on_object(const int32_t *index, const float *u, const float *v, int64_t n, float *points_xyz,
                          snch_stream_t stream = nullptr) const
    {
        check(snch_sample_on_object(h_, index, u, v, n, points_xyz, stream));
    }

    snch_scene_t handle() const { return h_; }

  private:
    void reset()
    {
        if (h_)
            snch_scene_destroy(h_);
        h_ = nullptr;
    }
    snch_scene_t h_ = nullptr;
    snch_bvh_view view_{};
};

}  // namespace snch
