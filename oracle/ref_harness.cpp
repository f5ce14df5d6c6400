// Driver around the UNMODIFIED reference headers (tyanyuy3125/snch-lbvh,
// include/snch_lbvh/*.cuh) -- TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/Makefile with g++ and Thrust's CPP (host) backend, so the
// reference's own construction (bvh.cuh:380-613) and its own per-thread
// query_device / sample functions (query.cuh, sample.cuh) run on the CPU of
// this container and produce the golden vectors under tests/golden/.
// The reference compiles as host C++ after three shims defined here:
//   * atomicCAS / __threadfence used unguarded by the AABB refit (bvh.cuh:531, 548),
//     restated for a single host thread;
//   * thrust::min / thrust::max (bvh.cuh:125, 216, 220), absent from current CCCL;
//   * unqualified max() in green_weight (scene.cuh:1123) resolved to std::max.
// Where the reference leaves an output unset (sample pdf when no triangle is
// hit, sample.cuh:46; ray uv on a miss, query.cuh:100) this driver writes 0.
//
// Input/output: raw little-endian files, layout documented in
// tests/golden/make_golden.py (the only caller).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <unordered_map>
#include <string>
#include <vector>
using std::max;
using std::min;
namespace thrust
{
    using std::max;
    using std::min;
}
static inline int atomicCAS(int *address, int compare, int val)
{
    int old = *address;
    if (old == compare)
        *address = val;
    return old;
}
static inline void __threadfence() {}

#include "snch_lbvh/lbvh.cuh"
#include "snch_lbvh/scene.cuh"
#include "snch_lbvh/scene_loader.cuh"

namespace
{
    template <typename T>
    bool read_n(FILE *f, std::vector<T> &v, int64_t n)
    {
        v.resize(static_cast<size_t>(n));
        return n == 0 || fread(v.data(), sizeof(T), static_cast<size_t>(n), f) == static_cast<size_t>(n);
    }
    template <typename T>
    void write_n(FILE *f, const T *p, int64_t n)
    {
        if (n > 0)
            fwrite(p, sizeof(T), static_cast<size_t>(n), f);
    }
} // namespace

// --obj in.obj out.bin: the reference's own OBJ reader (scene_loader.cuh:86-152):
// int64 nv, nt, then nv x float3 and nt x int3
static int read_obj_mode(const char *obj, const char *out_path)
{
    lbvh::scene_loader<3> ld(obj);
    FILE *out = std::fopen(out_path, "wb");
    if (!out)
        return 6;
    const int64_t n[2] = {static_cast<int64_t>(ld.vertices_size()), static_cast<int64_t>(ld.primitives_size())};
    write_n(out, n, 2);
    for (const float3 &v : ld.get_vertices())
    {
        const float q[3] = {v.x, v.y, v.z};
        write_n(out, q, 3);
    }
    for (const int3 &t : ld.get_indices())
    {
        const int32_t q[3] = {t.x, t.y, t.z};
        write_n(out, q, 3);
    }
    std::fclose(out);
    return 0;
}

// --2d in.bin out.bin: the reference's scene<2> (scene.cuh:287-703), its 2D build
// and the four query templates over line segments. Input: int64 nv, nseg, n_near,
// n_sil, n_ray, n_smp; float2 verts, int2 segments, near points, silhouette points
// + uint8 flips, ray origins, directions, tmax, circle centres, radii, u.
// Output: silhouette vertices (nv x int4), owned vertices (nseg x int2), Morton
// codes, nodes, aabbs (upper.xy, lower.xy), cones (axis.xy, half, radius), then
// (two or more segments) nearest (uint32, float), silhouette (float), ray
// (uint8 hit, float t, float s, uint32 idx), sample (int32, float pdf).
static int scene2d_mode(const char *in_path, const char *out_path)
{
    FILE *in = std::fopen(in_path, "rb");
    if (!in)
        return 3;
    int64_t hdr[6];
    if (std::fread(hdr, sizeof(int64_t), 6, in) != 6)
        return 4;
    const int64_t nv = hdr[0], nt = hdr[1], n_near = hdr[2], n_sil = hdr[3], n_ray = hdr[4], n_smp = hdr[5];
    std::vector<float> verts, near_pts, sil_pts, ray_o, ray_d, ray_tmax, smp_c, smp_r, smp_u;
    std::vector<int32_t> segs;
    std::vector<uint8_t> sil_flip;
    bool ok = read_n(in, verts, nv * 2) && read_n(in, segs, nt * 2) && read_n(in, near_pts, n_near * 2) &&
              read_n(in, sil_pts, n_sil * 2) && read_n(in, sil_flip, n_sil) && read_n(in, ray_o, n_ray * 2) &&
              read_n(in, ray_d, n_ray * 2) && read_n(in, ray_tmax, n_ray) && read_n(in, smp_c, n_smp * 2) &&
              read_n(in, smp_r, n_smp) && read_n(in, smp_u, n_smp);
    std::fclose(in);
    if (!ok)
        return 5;
    std::vector<float2> v2(static_cast<size_t>(nv));
    for (int64_t i = 0; i < nv; ++i)
        v2[i] = make_float2(verts[2 * i], verts[2 * i + 1]);
    std::vector<int2> s2(static_cast<size_t>(nt));
    for (int64_t i = 0; i < nt; ++i)
        s2[i] = make_int2(segs[2 * i], segs[2 * i + 1]);
    lbvh::scene<2> sc(v2.data(), v2.data() + v2.size(), s2.data(), s2.data() + s2.size());
    sc.compute_silhouettes();
    sc.build_bvh();
    const auto bvh = sc.get_bvh_device_ptr();
    FILE *out = std::fopen(out_path, "wb");
    if (!out)
        return 6;
    for (int64_t i = 0; i < nv; ++i)
    {
        const auto &q = sc.silhouettes_h[i].indices;
        const int32_t w[4] = {q.x, q.y, q.z, q.w};
        write_n(out, w, 4);
    }
    for (int64_t i = 0; i < nt; ++i)
    {
        const int32_t w[2] = {sc.lines[i].silhouette_indices.x, sc.lines[i].silhouette_indices.y};
        write_n(out, w, 2);
    }
    {
        using box_t = lbvh::aabb<float, 2>;
        const float inf = std::numeric_limits<float>::infinity();
        box_t whole;
        whole.upper = make_float2(-inf, -inf);
        whole.lower = make_float2(inf, inf);
        std::vector<box_t> boxes(static_cast<size_t>(nt));
        for (int64_t i = 0; i < nt; ++i)
        {
            boxes[i] = lbvh::scene<2>::aabb_getter()(sc.lines[i]);
            whole = lbvh::merge(whole, boxes[i]);
        }
        lbvh::default_morton_code_calculator<float, 2, lbvh::scene<2>::line_segment> calc(whole);
        for (int64_t i = 0; i < nt; ++i)
        {
            const uint32_t m = calc(sc.lines[i], boxes[i]);
            write_n(out, &m, 1);
        }
    }
    const int64_t NN = bvh.num_nodes;
    for (int64_t i = 0; i < NN; ++i)
    {
        const auto &n = bvh.nodes[i];
        const uint32_t q[4] = {n.parent_idx, n.left_idx, n.right_idx, n.object_idx};
        write_n(out, q, 4);
    }
    for (int64_t i = 0; i < NN; ++i)
    {
        const auto &b = bvh.aabbs[i];
        const float q[4] = {b.upper.x, b.upper.y, b.lower.x, b.lower.y};
        write_n(out, q, 4);
    }
    for (int64_t i = 0; i < NN; ++i)
    {
        const auto &c = bvh.cones[i];
        const float q[4] = {c.axis.x, c.axis.y, c.half_angle, c.radius};
        write_n(out, q, 4);
    }
    if (nt >= 2)
    {
        for (int64_t q = 0; q < n_near; ++q)
        {
            const auto r = lbvh::query_device(bvh, lbvh::nearest(make_float2(near_pts[2 * q], near_pts[2 * q + 1])),
                                              lbvh::scene<2>::distance_calculator());
            const uint32_t idx = r.first;
            const float d = r.second;
            write_n(out, &idx, 1);
            write_n(out, &d, 1);
        }
        for (int64_t q = 0; q < n_sil; ++q)
        {
            const float2 p = make_float2(sil_pts[2 * q], sil_pts[2 * q + 1]);
            const float d = lbvh::query_device(bvh, lbvh::nearest_silhouette(p, sil_flip[q] != 0),
                                               lbvh::scene<2>::silhouette_distance_calculator());
            write_n(out, &d, 1);
        }
        for (int64_t q = 0; q < n_ray; ++q)
        {
            const float2 o = make_float2(ray_o[2 * q], ray_o[2 * q + 1]);
            const float2 d = make_float2(ray_d[2 * q], ray_d[2 * q + 1]);
            const auto r = lbvh::query_device(bvh, lbvh::ray_intersect(lbvh::ray<float, 2>(o, d), ray_tmax[q]),
                                              lbvh::scene<2>::intersect_test());
            const uint8_t hit = thrust::get<0>(r) ? 1 : 0;
            const float t = thrust::get<1>(r);
            const float sp = hit ? thrust::get<2>(r) : 0.0f;
            const uint32_t idx = thrust::get<3>(r);
            write_n(out, &hit, 1);
            write_n(out, &t, 1);
            write_n(out, &sp, 1);
            write_n(out, &idx, 1);
        }
        for (int64_t q = 0; q < n_smp; ++q)
        {
            const float2 c = make_float2(smp_c[2 * q], smp_c[2 * q + 1]);
            const auto r = lbvh::sample_object_in_sphere(
                bvh, lbvh::sphere_intersect(lbvh::sphere<float, 2>(c, smp_r[q])), lbvh::scene<2>::intersect_sphere(),
                lbvh::scene<2>::measurement_getter(), lbvh::scene<2>::green_weight(), smp_u[q]);
            const int32_t idx = r.first;
            const float pdf = idx >= 0 ? r.second : 0.0f;
            write_n(out, &idx, 1);
            write_n(out, &pdf, 1);
        }
    }
    std::fclose(out);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 4 && std::string(argv[1]) == "--obj")
        return read_obj_mode(argv[2], argv[3]);
    if (argc == 4 && std::string(argv[1]) == "--2d")
        return scene2d_mode(argv[2], argv[3]);
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE *in = std::fopen(argv[1], "rb");
    if (!in)
        return 3;
    int64_t hdr[10];
    if (std::fread(hdr, sizeof(int64_t), 10, in) != 10)
        return 4;
    const int64_t nv = hdr[0], nt = hdr[1], n_near = hdr[2], n_sil = hdr[3], n_ray = hdr[4], n_smp = hdr[5],
                  n_obj = hdr[6], n_box = hdr[7], n_line = hdr[8], max_out = hdr[9];
    std::vector<float> verts, near_pts, sil_pts, ray_o, ray_d, ray_tmax, smp_c, smp_r, smp_u, obj_u, obj_v, boxes,
        line_o, line_d;
    std::vector<int32_t> tris, obj_idx;
    std::vector<uint8_t> sil_flip;
    bool ok = read_n(in, verts, nv * 3) && read_n(in, tris, nt * 3) && read_n(in, near_pts, n_near * 3) &&
              read_n(in, sil_pts, n_sil * 3) && read_n(in, sil_flip, n_sil) && read_n(in, ray_o, n_ray * 3) &&
              read_n(in, ray_d, n_ray * 3) && read_n(in, ray_tmax, n_ray) && read_n(in, smp_c, n_smp * 3) &&
              read_n(in, smp_r, n_smp) && read_n(in, smp_u, n_smp) && read_n(in, obj_idx, n_obj) &&
              read_n(in, obj_u, n_obj) && read_n(in, obj_v, n_obj) && read_n(in, boxes, n_box * 6) &&
              read_n(in, line_o, n_line * 3) && read_n(in, line_d, n_line * 3);
    std::fclose(in);
    if (!ok)
        return 5;

    std::vector<float3> v3(static_cast<size_t>(nv));
    for (int64_t i = 0; i < nv; ++i)
        v3[i] = make_float3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    std::vector<int3> f3(static_cast<size_t>(nt));
    for (int64_t i = 0; i < nt; ++i)
        f3[i] = make_int3(tris[3 * i], tris[3 * i + 1], tris[3 * i + 2]);

    lbvh::scene<3> sc(v3.data(), v3.data() + v3.size(), f3.data(), f3.data() + f3.size());
    sc.compute_silhouettes();
    sc.build_bvh();
    const auto bvh = sc.get_bvh_device_ptr();

    FILE *out = std::fopen(argv[2], "wb");
    if (!out)
        return 6;
    const int64_t E = static_cast<int64_t>(sc.silhouettes_h.size());
    const int64_t NN = bvh.num_nodes;
    int64_t ohdr[2] = {E, NN};
    write_n(out, ohdr, 2);
    for (int64_t i = 0; i < nt; ++i)
    {
        int32_t e[3] = {sc.edge_indices_h[i].x, sc.edge_indices_h[i].y, sc.edge_indices_h[i].z};
        write_n(out, e, 3);
    }
    for (int64_t i = 0; i < nt; ++i)
    {
        const auto &t = sc.triangles[i];
        int32_t o[3] = {t.silhouette_indices.x, t.silhouette_indices.y, t.silhouette_indices.z};
        write_n(out, o, 3);
    }
    for (int64_t e = 0; e < E; ++e)
    {
        const auto &s = sc.silhouettes_h[e];
        int32_t q[4] = {s.indices.x, s.indices.y, s.indices.z, s.indices.w};
        write_n(out, q, 4);
    }
    // Morton codes in original order, from the reference's own calculator and
    // scene AABB (bvh.cuh:423-439).
    {
        using box_t = lbvh::aabb<float, 3>;
        const float inf = std::numeric_limits<float>::infinity();
        box_t whole;
        whole.upper = make_float3(-inf, -inf, -inf);
        whole.lower = make_float3(inf, inf, inf);
        std::vector<box_t> boxes(static_cast<size_t>(nt));
        for (int64_t i = 0; i < nt; ++i)
        {
            boxes[i] = lbvh::scene<3>::aabb_getter()(sc.triangles[i]);
            whole = lbvh::merge(whole, boxes[i]);
        }
        lbvh::default_morton_code_calculator<float, 3, lbvh::scene<3>::triangle> calc(whole);
        for (int64_t i = 0; i < nt; ++i)
        {
            uint32_t m = calc(sc.triangles[i], boxes[i]);
            write_n(out, &m, 1);
        }
    }
    for (int64_t i = 0; i < NN; ++i)
    {
        const auto &n = bvh.nodes[i];
        uint32_t q[4] = {n.parent_idx, n.left_idx, n.right_idx, n.object_idx};
        write_n(out, q, 4);
    }
    for (int64_t i = 0; i < NN; ++i)
    {
        const auto &b = bvh.aabbs[i];
        float q[6] = {b.upper.x, b.upper.y, b.upper.z, b.lower.x, b.lower.y, b.lower.z};
        write_n(out, q, 6);
    }
    for (int64_t i = 0; i < NN; ++i)
    {
        const auto &c = bvh.cones[i];
        float q[5] = {c.axis.x, c.axis.y, c.axis.z, c.half_angle, c.radius};
        write_n(out, q, 5);
    }
    // The reference's nearest / silhouette traversals read past the node array
    // for a one-triangle tree (bvh.cuh:388-390, query.cuh:265): not run there.
    const bool tree_ok = nt >= 2;
    for (int64_t q = 0; q < (tree_ok ? n_near : 0); ++q)
    {
        const float3 p = make_float3(near_pts[3 * q], near_pts[3 * q + 1], near_pts[3 * q + 2]);
        const auto r = lbvh::query_device(bvh, lbvh::nearest(p), lbvh::scene<3>::distance_calculator());
        uint32_t idx = r.first;
        float d = r.second;
        write_n(out, &idx, 1);
        write_n(out, &d, 1);
    }
    for (int64_t q = 0; q < (tree_ok ? n_sil : 0); ++q)
    {
        const float3 p = make_float3(sil_pts[3 * q], sil_pts[3 * q + 1], sil_pts[3 * q + 2]);
        float d = lbvh::query_device(bvh, lbvh::nearest_silhouette(p, sil_flip[q] != 0),
                                     lbvh::scene<3>::silhouette_distance_calculator());
        write_n(out, &d, 1);
    }
    for (int64_t q = 0; q < n_ray; ++q)
    {
        const float3 o = make_float3(ray_o[3 * q], ray_o[3 * q + 1], ray_o[3 * q + 2]);
        const float3 d = make_float3(ray_d[3 * q], ray_d[3 * q + 1], ray_d[3 * q + 2]);
        const auto r = lbvh::query_device(bvh, lbvh::ray_intersect(lbvh::ray<float, 3>(o, d), ray_tmax[q]),
                                          lbvh::scene<3>::intersect_test());
        uint8_t hit = thrust::get<0>(r) ? 1 : 0;
        float t = thrust::get<1>(r);
        float2 uv = hit ? thrust::get<2>(r) : make_float2(0.0f, 0.0f);
        uint32_t idx = thrust::get<3>(r);
        write_n(out, &hit, 1);
        write_n(out, &t, 1);
        write_n(out, &uv.x, 1);
        write_n(out, &uv.y, 1);
        write_n(out, &idx, 1);
    }
    for (int64_t q = 0; q < n_smp; ++q)
    {
        const float3 c = make_float3(smp_c[3 * q], smp_c[3 * q + 1], smp_c[3 * q + 2]);
        const auto r = lbvh::sample_object_in_sphere(
            bvh, lbvh::sphere_intersect(lbvh::sphere<float, 3>(c, smp_r[q])), lbvh::scene<3>::intersect_sphere(),
            lbvh::scene<3>::measurement_getter(), lbvh::scene<3>::green_weight(), smp_u[q]);
        int32_t idx = r.first;
        float pdf = idx >= 0 ? r.second : 0.0f;
        write_n(out, &idx, 1);
        write_n(out, &pdf, 1);
    }
    for (int64_t q = 0; q < n_obj; ++q)
    {
        const float3 p = lbvh::sample_on_object(bvh, obj_idx[q], lbvh::scene<3>::sample_on_object(), obj_u[q], obj_v[q]);
        float xyz[3] = {p.x, p.y, p.z};
        write_n(out, xyz, 3);
    }
    // AABB-overlap enumeration (query.cuh:177-231) and line enumeration
    // (query.cuh:15-77): up to max_out results in the reference's output order
    // and the total count it returns. Query boxes are given lower xyz, upper xyz.
    // The line query's element test is the caller's functor (the 3D scene ships
    // none): here the Moller-Trumbore arithmetic of scene<3>::intersect_test
    // (scene.cuh:1005-1052) without its t >= 0 condition -- a line, not a ray --
    // returning the line parameter t.
    if (tree_ok)
    {
        std::vector<uint32_t> found(static_cast<size_t>(max_out));
        for (int64_t q = 0; q < n_box; ++q)
        {
            lbvh::aabb<float, 3> b;
            b.lower = make_float3(boxes[6 * q], boxes[6 * q + 1], boxes[6 * q + 2]);
            b.upper = make_float3(boxes[6 * q + 3], boxes[6 * q + 4], boxes[6 * q + 5]);
            const uint32_t cnt =
                lbvh::query_device(bvh, lbvh::overlaps(b), found.data(), static_cast<unsigned int>(max_out));
            write_n(out, &cnt, 1);
            write_n(out, found.data(), std::min<int64_t>(cnt, max_out));
        }
        auto line_test = [](const lbvh::line<float, 3> &r, const lbvh::scene<3>::triangle &object) {
            const float3 v0 = object.vertices[object.vertex_indices.x];
            const float3 v1 = object.vertices[object.vertex_indices.y];
            const float3 v2 = object.vertices[object.vertex_indices.z];
            const float3 edge1 = {v1.x - v0.x, v1.y - v0.y, v1.z - v0.z};
            const float3 edge2 = {v2.x - v0.x, v2.y - v0.y, v2.z - v0.z};
            const float3 h = {r.dir.y * edge2.z - r.dir.z * edge2.y, r.dir.z * edge2.x - r.dir.x * edge2.z,
                              r.dir.x * edge2.y - r.dir.y * edge2.x};
            const float det = edge1.x * h.x + edge1.y * h.y + edge1.z * h.z;
            if (std::fabs(det) < lbvh::epsilon<float>())
                return thrust::make_pair(false, 0.0f);
            const float inv_det = 1.0f / det;
            const float3 sv = {r.origin.x - v0.x, r.origin.y - v0.y, r.origin.z - v0.z};
            const float u = (sv.x * h.x + sv.y * h.y + sv.z * h.z) * inv_det;
            if (u < 0.0f || u > 1.0f)
                return thrust::make_pair(false, 0.0f);
            const float3 qv = {sv.y * edge1.z - sv.z * edge1.y, sv.z * edge1.x - sv.x * edge1.z,
                               sv.x * edge1.y - sv.y * edge1.x};
            const float v = (r.dir.x * qv.x + r.dir.y * qv.y + r.dir.z * qv.z) * inv_det;
            if (v < 0.0f || u + v > 1.0f)
                return thrust::make_pair(false, 0.0f);
            return thrust::make_pair(true, (edge2.x * qv.x + edge2.y * qv.y + edge2.z * qv.z) * inv_det);
        };
        std::vector<thrust::pair<unsigned int, float>> hits(static_cast<size_t>(max_out));
        for (int64_t q = 0; q < n_line; ++q)
        {
            const float3 o = make_float3(line_o[3 * q], line_o[3 * q + 1], line_o[3 * q + 2]);
            const float3 d = make_float3(line_d[3 * q], line_d[3 * q + 1], line_d[3 * q + 2]);
            const uint32_t cnt = lbvh::query_device(bvh, lbvh::line_intersect(lbvh::line<float, 3>(o, d)), line_test,
                                                    hits.data(), static_cast<unsigned int>(max_out));
            write_n(out, &cnt, 1);
            for (int64_t k = 0; k < std::min<int64_t>(cnt, max_out); ++k)
            {
                write_n(out, &hits[k].first, 1);
                write_n(out, &hits[k].second, 1);
            }
        }
    }
    std::fclose(out);
    return 0;
}
