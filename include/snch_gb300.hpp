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
    // ray_intersect<TestOnly = true>: occlusion test, hit flags only
    void query_ray_test(const float *origins_xyz, const float *dirs_xyz, const float *tmax, int64_t n, uint8_t *hit,
                        snch_stream_t stream = nullptr) const
    {
        check(snch_query_ray_test(h_, origins_xyz, dirs_xyz, tmax, n, hit, stream));
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

    // seeded forms: same results as query_nearest / query_silhouette for any radii
    void query_nearest_seeded(const float *points_xyz, const float *radius, int64_t n, uint32_t *index,
                              float *distance, uint32_t *num_fallback = nullptr, snch_stream_t stream = nullptr) const
    {
        check(snch_query_nearest_seeded(h_, points_xyz, radius, n, index, distance, num_fallback, stream));
    }
    void query_silhouette_seeded(const float *points_xyz, const uint8_t *flip, const float *radius, int64_t n,
                                 float *distance, int32_t *edge = nullptr, uint32_t *num_fallback = nullptr,
                                 snch_stream_t stream = nullptr) const
    {
        check(snch_query_silhouette_seeded(h_, points_xyz, flip, radius, n, distance, edge, num_fallback, stream));
    }
    void set_option(int option, int64_t value) { check(snch_set_option(h_, option, value)); }

    // query_device(overlaps(box)) / query_device(line_intersect(line)): the first
    // max_per_query results per query at [q * max_per_query ...], totals in count
    void query_overlap(const float *boxes_lo_hi, int64_t n, uint32_t max_per_query, uint32_t *index,
                       uint32_t *count, snch_stream_t stream = nullptr) const
    {
        check(snch_query_overlap(h_, boxes_lo_hi, n, max_per_query, index, count, stream));
    }
    void query_line(const float *origins_xyz, const float *dirs_xyz, int64_t n, uint32_t max_per_query,
                    uint32_t *index, float *t, uint32_t *count, snch_stream_t stream = nullptr) const
    {
        check(snch_query_line(h_, origins_xyz, dirs_xyz, n, max_per_query, index, t, count, stream));
    }

    // a built scene to / from a file (no rebuild on load)
    void save(const std::string &path, snch_stream_t stream = nullptr) const
    {
        check(snch_scene_save(h_, path.c_str(), stream));
    }
    static scene3 load(const std::string &path, snch_stream_t stream = nullptr)
    {
        snch_scene_t h = nullptr;
        check(snch_scene_load(path.c_str(), &h, stream));
        scene3 s(h);
        s.view_ = {};
        check(snch_get_bvh_view(h, &s.view_));
        return s;
    }

    snch_scene_t handle() const { return h_; }

  protected:
    explicit scene3(snch_scene_t h) : h_(h) {}
    void reset()
    {
        if (h_)
            snch_scene_destroy(h_);
        h_ = nullptr;
    }
    snch_scene_t h_ = nullptr;
    snch_bvh_view view_{};
};

// scene_loader<3>(filename) scene_loader.cuh:86-152: vertices (float3-like) and
// 0-based triangles (int3-like) of an OBJ file, throwing std::runtime_error as
// the reference does ("Could not open .obj file.")
template <typename Float3, typename Int3>
class scene_loader3
{
  public:
    explicit scene_loader3(const std::string &filename)
    {
        int64_t nv = 0, nt = 0;
        check(snch_obj_read(filename.c_str(), nullptr, 0, nullptr, 0, &nv, &nt));
        std::vector<float> v(static_cast<size_t>(3 * nv));
        std::vector<int32_t> t(static_cast<size_t>(3 * nt));
        check(snch_obj_read(filename.c_str(), v.data(), nv, t.data(), nt, &nv, &nt));
        for (int64_t i = 0; i < nv; ++i)
            vertices_.push_back(Float3{v[3 * i], v[3 * i + 1], v[3 * i + 2]});
        for (int64_t i = 0; i < nt; ++i)
            indices_.push_back(Int3{t[3 * i], t[3 * i + 1], t[3 * i + 2]});
    }
    const std::vector<Float3> &get_vertices() const { return vertices_; }
    const std::vector<Int3> &get_indices() const { return indices_; }
    std::size_t vertices_size() const { return vertices_.size(); }
    std::size_t primitives_size() const { return indices_.size(); }

  private:
    std::vector<Float3> vertices_;
    std::vector<Int3> indices_;
};

// lbvh::scene<2> (scene.cuh:287-703): line segments with silhouette vertices.
// Iterators over float2-like (x, y) vertices and int2-like (x, y) segments.
class scene2
{
  public:
    template <typename VertexIt, typename IndexIt>
    scene2(VertexIt vertices_first, VertexIt vertices_last, IndexIt indices_first, IndexIt indices_last)
    {
        std::vector<float> v;
        std::vector<int32_t> s;
        for (auto it = vertices_first; it != vertices_last; ++it)
        {
            v.push_back(static_cast<float>(it->x));
            v.push_back(static_cast<float>(it->y));
        }
        for (auto it = indices_first; it != indices_last; ++it)
        {
            s.push_back(static_cast<int32_t>(it->x));
            s.push_back(static_cast<int32_t>(it->y));
        }
        check(snch_scene2_create(v.data(), static_cast<int64_t>(v.size() / 2), s.data(),
                                 static_cast<int64_t>(s.size() / 2), &h_));
    }
    scene2(const scene2 &) = delete;
    scene2 &operator=(const scene2 &) = delete;
    scene2(scene2 &&o) noexcept : h_(std::exchange(o.h_, nullptr)), built_(o.built_) {}
    ~scene2()
    {
        if (h_)
            snch_scene2_destroy(h_);
    }
    // the silhouette vertices are derived on the GPU together with the tree
    void compute_silhouettes(snch_stream_t = nullptr) {}
    void build_bvh(snch_stream_t stream = nullptr)
    {
        check(snch_scene2_build(h_, stream));
        built_ = true;
    }
    void query_nearest(const float *points_xy, int64_t n, uint32_t *index, float *distance,
                       snch_stream_t stream = nullptr) const
    {
        check(snch_scene2_query_nearest(h_, points_xy, n, index, distance, stream));
    }
    void query_silhouette(const float *points_xy, const uint8_t *flip, int64_t n, float *distance,
                          int32_t *vertex = nullptr, snch_stream_t stream = nullptr) const
    {
        check(snch_scene2_query_silhouette(h_, points_xy, flip, n, distance, vertex, stream));
    }
    void query_ray(const float *origins_xy, const float *dirs_xy, const float *tmax, int64_t n, uint8_t *hit,
                   float *t, float *segment_param, uint32_t *index, snch_stream_t stream = nullptr) const
    {
        check(snch_scene2_query_ray(h_, origins_xy, dirs_xy, tmax, n, hit, t, segment_param, index, stream));
    }
    void query_ray_test(const float *origins_xy, const float *dirs_xy, const float *tmax, int64_t n, uint8_t *hit,
                        snch_stream_t stream = nullptr) const
    {
        check(snch_scene2_query_ray_test(h_, origins_xy, dirs_xy, tmax, n, hit, stream));
    }
    void sample_in_circle(const float *centers_xy, const float *radii, const float *u, int64_t n, int32_t *index,
                          float *pdf, snch_stream_t stream = nullptr) const
    {
        check(snch_scene2_sample_in_circle(h_, centers_xy, radii, u, n, index, pdf, stream));
    }
    void sample_on_object(const int32_t *index, const float *u, int64_t n, float *points_xy,
                          snch_stream_t stream = nullptr) const
    {
        check(snch_scene2_sample_on_object(h_, index, u, n, points_xy, stream));
    }
    snch_scene2_t handle() const { return h_; }

  private:
    snch_scene2_t h_ = nullptr;
    bool built_ = false;
};

// Many independent meshes in one scene (snch_batch_*): one build, one query
// launch per type; results per mesh as a scene3 of that mesh alone gives.
class batch3 : public scene3
{
  public:
    // concatenated vertices / triangles (per-mesh vertex indices) and num_meshes + 1
    // starts of each; device != 0: vertices and triangles are device buffers
    batch3(const float *vertices_xyz, int64_t num_vertices, const int32_t *triangles, int64_t num_triangles,
           const std::vector<int64_t> &mesh_vert_start, const std::vector<int64_t> &mesh_tri_start, int device = 0,
           snch_stream_t stream = nullptr)
        : scene3(create(vertices_xyz, num_vertices, triangles, num_triangles, mesh_vert_start, mesh_tri_start,
                        device, stream))
    {
    }
    int32_t num_meshes() const
    {
        int32_t m = 0;
        check(snch_batch_num_meshes(h_, &m));
        return m;
    }
    void query_nearest(const int32_t *mesh, const float *points_xyz, int64_t n, int32_t *index, float *distance,
                       snch_stream_t stream = nullptr) const
    {
        check(snch_batch_query_nearest(h_, mesh, points_xyz, n, index, distance, stream));
    }
    void query_silhouette(const int32_t *mesh, const float *points_xyz, const uint8_t *flip, int64_t n,
                          float *distance, int32_t *edge = nullptr, snch_stream_t stream = nullptr) const
    {
        check(snch_batch_query_silhouette(h_, mesh, points_xyz, flip, n, distance, edge, stream));
    }

  private:
    static snch_scene_t create(const float *v, int64_t nv, const int32_t *t, int64_t nt,
                               const std::vector<int64_t> &vs, const std::vector<int64_t> &ts, int device,
                               snch_stream_t stream)
    {
        if (vs.size() != ts.size() || vs.size() < 2)
            throw std::runtime_error("batch3: need num_meshes + 1 vertex and triangle starts");
        snch_scene_t h = nullptr;
        check(snch_batch_create(v, nv, t, nt, vs.data(), ts.data(), static_cast<int32_t>(vs.size() - 1), device, &h,
                                stream));
        return h;
    }
};

// Learned search radius (snch_mlp_*): train on (point, log distance) pairs,
// predict per-query radii for the seeded queries.
class learned_radius
{
  public:
    learned_radius(const float box_lo[3], const float box_hi[3], uint64_t seed = 0)
    {
        check(snch_mlp_create(box_lo, box_hi, seed, &h_));
    }
    learned_radius(const learned_radius &) = delete;
    learned_radius &operator=(const learned_radius &) = delete;
    ~learned_radius()
    {
        if (h_)
            snch_mlp_destroy(h_);
    }
    // device points (n x 3) and targets (n x 2: log nearest, log silhouette distance; NaN = none)
    float train(const float *points, const float *targets, int64_t n, int epochs = 1, int64_t batch = 65536,
                float lr = 2e-3f, float tau = 0.9f, snch_stream_t stream = nullptr)
    {
        float loss = 0.f;
        check(snch_mlp_train(h_, points, targets, n, epochs, batch, lr, tau, &loss, stream));
        return loss;
    }
    void predict(const float *points, int64_t n, float *radius_near, float *radius_sil, float margin = 1.5f,
                 float floor = 1e-4f, snch_stream_t stream = nullptr) const
    {
        check(snch_mlp_predict_radius(h_, points, n, margin, floor, radius_near, radius_sil, stream));
    }
    snch_mlp_t handle() const { return h_; }

  private:
    snch_mlp_t h_ = nullptr;
};

}  // namespace snch
