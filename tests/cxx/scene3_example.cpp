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
    cudaFree(d_pts);
    cudaFree(d_dist);
    cudaFree(d_idx);
    return (idx < 20 && std::fabs(dist - r_in) < 1e-5) ? 0 : 4;
}
