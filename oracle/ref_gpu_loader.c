/*
 * Loader of the reference's CUDA queries (oracle/_ref/ref_queries_sm103a.cubin,
 * built from oracle/ref_gpu_kernels.cu) -- TEST INFRASTRUCTURE ONLY.
 *
 * The cubin is device code only, so it is built where the reference headers
 * are and runs on any host architecture; this loader (host C over the CUDA
 * runtime's library API) is compiled on the machine that runs it.
 */
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

static cudaLibrary_t g_lib;
#define NK 6
static cudaKernel_t g_k[NK];
static const char *g_names[NK] = {"ref_nearest", "ref_silhouette", "ref_ray", "ref_sample", "ref_silhouette_edge", "ref_ray_uv"};

/* returns 0 on success, else the cudaError_t */
int rg_load(const char *cubin_path) {
    if (g_lib) return 0;
    cudaError_t e = cudaLibraryLoadFromFile(&g_lib, cubin_path, NULL, NULL, 0, NULL, NULL, 0);
    if (e != cudaSuccess) return (int)e;
    for (int i = 0; i < NK; ++i) {
        e = cudaLibraryGetKernel(&g_k[i], g_lib, g_names[i]);
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

typedef struct { unsigned char bytes[40]; } view40; /* snch_bvh_view == lbvh::bvh_device<float,3,triangle> */

static int launch(int k, int n, void **args, void *stream) {
    if (n <= 0) return 0;
    dim3 grid = {(unsigned)((n + 127) / 128), 1, 1}, block = {128, 1, 1};
    cudaError_t e = cudaLaunchKernel((const void *)g_k[k], grid, block, args, 0, (cudaStream_t)stream);
    return (int)e;
}

int rg_nearest(const void *view, const float *pts, int n, unsigned *idx, float *dist, void *stream) {
    view40 v = *(const view40 *)view;
    void *args[] = {&v, &pts, &n, &idx, &dist};
    return launch(0, n, args, stream);
}

int rg_silhouette(const void *view, const float *pts, const unsigned char *flip, int n, float *dist, void *stream) {
    view40 v = *(const view40 *)view;
    void *args[] = {&v, &pts, &flip, &n, &dist};
    return launch(1, n, args, stream);
}

int rg_ray(const void *view, const float *o, const float *d, const float *tmax, int n, unsigned char *hit, float *t,
           unsigned *idx, void *stream) {
    view40 v = *(const view40 *)view;
    void *args[] = {&v, &o, &d, &tmax, &n, &hit, &t, &idx};
    return launch(2, n, args, stream);
}

int rg_sample(const void *view, const float *c, const float *r, const float *u, int n, int *idx, float *pdf,
              void *stream) {
    view40 v = *(const view40 *)view;
    void *args[] = {&v, &c, &r, &u, &n, &idx, &pdf};
    return launch(3, n, args, stream);
}

int rg_silhouette_edge(const void *view, const float *pts, const unsigned char *flip, int n, float *dist, int *edge,
                       void *stream) {
    view40 v = *(const view40 *)view;
    void *args[] = {&v, &pts, &flip, &n, &dist, &edge};
    return launch(4, n, args, stream);
}

int rg_ray_uv(const void *view, const float *o, const float *d, const float *tmax, int n, unsigned char *hit, float *t,
              float *uv, unsigned *idx, void *stream) {
    view40 v = *(const view40 *)view;
    void *args[] = {&v, &o, &d, &tmax, &n, &hit, &t, &uv, &idx};
    return launch(5, n, args, stream);
}
