// Host C++ written against snch_gb300.hpp the way reference users write
// against lbvh::scene<3>: construct from vertex/face iterators, compute
// silhouettes, build, query. Unit icosahedron; the nearest distance from the
// origin is the inradius sqrt(3)/12 * (3 + sqrt(5)) * edge / 2... computed in double.
#include <cmath>
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "snch_gb300.hpp"

struct V3 { float x, y, z; };
struct I3 { int x, y, z; };

int main(int argc, char **argv)
{
    if (argc > 1 && std::string(argv[1]) == "--version")
    {
        std::printf("%s\n", snch_version());
        return 0;
    }
    const double t = (1.0 + std::sqrt(5.0)) / 2.0, s = 1.0 / std::sqrt(1.0 + t * t);
    std::vector<V3> v = {{-1, (float)t, 0}, {1, (float)t, 0}, {-1, (float)-t, 0}, {1, (float)-t, 0},
                         {0, -1, (float)t}, {0, 1, (float)t}, {0, -1, (float)-t}, {0, 1, (float)-t},
                         {(float)t, 0, -1}, {(float)t, 0, 1}, {(float)-t, 0, -1}, {(float)-t, 0, 1}};
    for (auto &p : v) { p.x *= (float)s; p.y *= (float)s; p.z *= (float)s; }
    std::vector<I3> f = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                         {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                         {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    snch::scene3 scene(v.begin(), v.end(), f.begin(), f.end());
    try
    {
        scene.get_bvh_device_ptr();
        std::printf("FAIL: expected \"BVH is not built yet.\"\n");
        return 1;
    }
    catch (const std::runtime_error &e)
    {
        if (std::string(e.what()) != "BVH is not built yet.")
            return 2;
    }
    scene.compute_silhouettes();
    scene.build_bvh();
    const snch_bvh_view &view = scene.get_bvh_device_ptr();
    if (view.num_objects != 20 || view.num_nodes != 39)
        return 3;
    float h_pts[3] = {0.f, 0.f, 0.f};
    float *d_pts = nullptr, *d_dist = nullptr;
    uint32_t *d_idx = nullptr;
    cudaMalloc(&d_pts, sizeof h_pts);
    cudaMalloc(&d_dist, 4);
    cudaMalloc(&d_idx, 4);
    cudaMemcpy(d_pts, h_pts, sizeof h_pts, cudaMemcpyHostToDevice);
    scene.query_nearest(d_pts, 1, d_idx, d_dist);
    float dist = 0;
    uint32_t idx = 0;
    cudaMemcpy(&dist, d_dist, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&idx, d_idx, 4, cudaMemcpyDeviceToHost);
    // inradius of the icosahedron with unit circumradius
    const double r_in = std::sqrt((5.0 + 2.0 * std::sqrt(5.0)) / 15.0);
    std::printf("nearest idx=%u dist=%.7f expected=%.7f\n", idx, dist, r_in);
    if (!(idx < 20 && std::fabs(dist - r_in) < 1e-5))
        return 4;

    // two copies of the icosahedron in one batch: the second shifted by +3 in x;
    // each query asks its own mesh and gets what a single scene of that mesh
    // gives. The centre is equidistant from all 20 faces and the shift rounds
    // the coordinates, so the shifted copy is compared with its own scene.
    std::vector<float> bv;
    std::vector<int32_t> bf;
    for (int m = 0; m < 2; ++m)
    {
        for (auto &p : v)
        {
            bv.push_back(p.x + 3.0f * m);
            bv.push_back(p.y);
            bv.push_back(p.z);
        }
        for (auto &q : f)
        {
            bf.push_back(q.x);
            bf.push_back(q.y);
            bf.push_back(q.z);
        }
    }
    snch::batch3 batch(bv.data(), 24, bf.data(), 40, {0, 12, 24}, {0, 20, 40});
    batch.compute_silhouettes();
    batch.build_bvh();
    if (batch.num_meshes() != 2)
        return 5;
    const float h2[6] = {0.f, 0.f, 0.f, 3.f, 0.f, 0.f};
    const int32_t hm[2] = {0, 1};
    float *d2 = nullptr, *dd = nullptr;
    int32_t *dm = nullptr, *di = nullptr;
    cudaMalloc(&d2, sizeof h2);
    cudaMalloc(&dd, 8);
    cudaMalloc(&dm, 8);
    cudaMalloc(&di, 8);
    cudaMemcpy(d2, h2, sizeof h2, cudaMemcpyHostToDevice);
    cudaMemcpy(dm, hm, sizeof hm, cudaMemcpyHostToDevice);
    batch.query_nearest(dm, d2, 2, di, dd);
    float bd[2];
    int32_t bi[2];
    cudaMemcpy(bd, dd, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(bi, di, 8, cudaMemcpyDeviceToHost);
    snch::scene3 shifted(bv.data() + 36, 12, bf.data() + 60, 20);
    shifted.compute_silhouettes();
    shifted.build_bvh();
    shifted.query_nearest(d2 + 3, 1, d_idx, d_dist);
    float sh_dist = 0;
    uint32_t sh_idx = 0;
    cudaMemcpy(&sh_dist, d_dist, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&sh_idx, d_idx, 4, cudaMemcpyDeviceToHost);
    std::printf("batched: idx=%d,%d dist=%.7f,%.7f single: idx=%u,%u dist=%.7f,%.7f\n", bi[0], bi[1], bd[0], bd[1],
                idx, sh_idx, dist, sh_dist);
    if (bi[0] != (int32_t)idx || bi[1] != (int32_t)sh_idx || bd[0] != dist || bd[1] != sh_dist)
        return 6;

    // learned radius (untrained) seeding the nearest query: same answer
    const float lo[3] = {-1.f, -1.f, -1.f}, hi[3] = {1.f, 1.f, 1.f};
    snch::learned_radius model(lo, hi, 7);
    float *dr = nullptr;
    cudaMalloc(&dr, 4);
    model.predict(d_pts, 1, dr, nullptr);
    scene.query_nearest_seeded(d_pts, dr, 1, d_idx, d_dist);
    float sdist = 0;
    uint32_t sidx = 0;
    cudaMemcpy(&sdist, d_dist, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&sidx, d_idx, 4, cudaMemcpyDeviceToHost);
    std::printf("seeded: idx=%u dist=%.7f\n", sidx, sdist);
    if (!(sidx == idx && sdist == dist))
        return 7;

    // scene_loader<3> round trip through an OBJ file, save / load of the built
    // scene, and an overlap query on the loaded one
    const std::string obj = "/tmp/snch_example_ico.obj", bin = "/tmp/snch_example_ico.snch";
    if (FILE *fo = std::fopen(obj.c_str(), "w"))
    {
        for (auto &p : v)
            std::fprintf(fo, "v %.9g %.9g %.9g\n", p.x, p.y, p.z);
        for (auto &q : f)
            std::fprintf(fo, "f %d %d %d\n", q.x + 1, q.y + 1, q.z + 1);
        std::fclose(fo);
    }
    snch::scene_loader3<V3, I3> loader(obj);
    if (loader.vertices_size() != 12 || loader.primitives_size() != 20 || loader.get_indices()[7].z != f[7].z)
        return 8;
    snch::scene3 from_file(loader.get_vertices().begin(), loader.get_vertices().end(), loader.get_indices().begin(),
                           loader.get_indices().end());
    from_file.compute_silhouettes();
    from_file.build_bvh();
    from_file.save(bin);
    snch::scene3 loaded = snch::scene3::load(bin);
    if (loaded.get_bvh_device_ptr().num_objects != 20)
        return 9;
    loaded.query_nearest(d_pts, 1, d_idx, d_dist);
    float ldist = 0;
    cudaMemcpy(&ldist, d_dist, 4, cudaMemcpyDeviceToHost);
    const float hb[6] = {-2.f, -2.f, -2.f, 2.f, 2.f, 2.f};
    float *dbox = nullptr;
    uint32_t *dcnt = nullptr, *didx = nullptr;
    cudaMalloc(&dbox, sizeof hb);
    cudaMalloc(&dcnt, 4);
    cudaMalloc(&didx, 4 * 32);
    cudaMemcpy(dbox, hb, sizeof hb, cudaMemcpyHostToDevice);
    loaded.query_overlap(dbox, 1, 32, didx, dcnt);
    uint32_t cnt = 0;
    cudaMemcpy(&cnt, dcnt, 4, cudaMemcpyDeviceToHost);
    std::printf("loaded: dist=%.7f overlap count=%u\n", ldist, cnt);
    for (void *q : {(void *)dbox, (void *)dcnt, (void *)didx})
        cudaFree(q);
    if (ldist != dist || cnt != 20)
        return 10;

    // scene<2>: a unit square; the nearest distance from its centre is 0.5
    struct V2 { float x, y; };
    struct I2 { int x, y; };
    const std::vector<V2> sq = {{0.f, 0.f}, {1.f, 0.f}, {1.f, 1.f}, {0.f, 1.f}};
    const std::vector<I2> sg = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
    snch::scene2 sq2(sq.begin(), sq.end(), sg.begin(), sg.end());
    sq2.compute_silhouettes();
    sq2.build_bvh();
    const float c2[2] = {0.5f, 0.5f};
    cudaMemcpy(d_pts, c2, sizeof c2, cudaMemcpyHostToDevice);
    sq2.query_nearest(d_pts, 1, d_idx, d_dist);
    float d2d = 0;
    cudaMemcpy(&d2d, d_dist, 4, cudaMemcpyDeviceToHost);
    std::printf("2d: dist=%.7f\n", d2d);
    if (d2d != 0.5f)
        return 11;
    for (void *q : {(void *)d_pts, (void *)d_dist, (void *)d_idx, (void *)d2, (void *)dd, (void *)dm, (void *)di,
                    (void *)dr})
        cudaFree(q);
    return 0;
}
