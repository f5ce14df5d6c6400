// snch_sort_pairs_noalloc: the library's stable radix sort for callers that
// cannot allocate GPU memory.
//
// Some callers may not call cudaMalloc or any allocating routine at the point
// where they need a sort: code between the frames of a real-time solver loop
// that must never stall (cudaMalloc/cudaFree can synchronise the whole
// device), host plug-ins whose GPU memory is owned and budgeted by the host
// application, and hooks that run while the application holds its own
// allocator lock. For them this entry point takes only the caller's input and
// output buffers and keeps every other byte it needs -- one ping-pong buffer,
// the decoupled look-back flags, the digit histograms and a status word -- in
// one file-scope __device__ array of fixed size. That array exists on every
// GPU that loads the library, from load until process exit; every call reuses
// it (and clears what must start at zero), so two calls that overlap on the
// GPU -- on different streams, or from different host threads -- race on it
// and must be ordered by the caller.
#include <cuda.h>

#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

namespace snch
{
namespace
{

constexpr int64_t kNoAllocMaxPairs = SNCH_SORT_NOALLOC_MAX_PAIRS;  // (key, value) pairs per call
constexpr size_t kNoAllocTmpBytes = 4 * (size_t)kNoAllocMaxPairs;
constexpr size_t kNoAllocSortBytes = size_t(2) << 20;  // covers sort_scratch_bytes(2^20, 32) (checked at set-up)
constexpr size_t kNoAllocBytes = 2 * kNoAllocTmpBytes + kNoAllocSortBytes + 256;

// [tmp keys | tmp values | look-back flags, histograms, tile counters | status word]
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of g_noalloc_scratch for the calling thread's current CUDA
// context. In host code the array's name is only a host-side stand-in; the
// address belongs to the module loaded in one context, not to a device
// ordinal: a host plug-in may run under a context of its own, and after a
// cudaDeviceReset the module is loaded again at a possibly different address.
// So the address is looked up again (cudaGetSymbolAddress, which allocates
// nothing) on every call whose stream is not being captured, and remembered per
// context for calls made during a capture. A call under capture in a context
// that has never made an uncaptured call looks it up too (the lookup can load
// the module, which is why the first call belongs before any capture).
using CtxGetCurrentFn = CUresult (*)(CUcontext *);

CtxGetCurrentFn ctx_get_current()
{
    static CtxGetCurrentFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    return fn;
}

struct ContextAddress
{
    CUcontext ctx;
    unsigned char *address;
};
std::mutex g_setup_mutex;
std::vector<ContextAddress> g_scratch_address;  // one entry per context seen

cudaError_t scratch_address(cudaStream_t st, unsigned char **out)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess)
        return e;
    CtxGetCurrentFn get = ctx_get_current();
    CUcontext ctx = nullptr;
    if (!get || get(&ctx) != CUDA_SUCCESS)
        ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ContextAddress *hit = nullptr;
    if (ctx)
        for (ContextAddress &c : g_scratch_address)
            if (c.ctx == ctx)
                hit = &c;
    if (hit && cs != cudaStreamCaptureStatusNone)
    {
        *out = hit->address;
        return cudaSuccess;
    }
    void *p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess)
        return e;
    if (!ctx && get && get(&ctx) != CUDA_SUCCESS)  // the lookup may have made the primary context current
        ctx = nullptr;
    if (hit)
        hit->address = static_cast<unsigned char *>(p);
    else if (ctx)
        g_scratch_address.push_back({ctx, static_cast<unsigned char *>(p)});
    *out = static_cast<unsigned char *>(p);
    return cudaSuccess;
}

}  // namespace
}  // namespace snch

using namespace snch;

extern "C" {

int snch_sort_pairs_noalloc(const uint32_t *keys_in, const uint32_t *values_in, uint32_t *keys_out,
                            uint32_t *values_out, int64_t n, int key_bits, uint32_t *device_status,
                            snch_stream_t stream)
{
    if (n < 0 || key_bits < 1 || key_bits > 32)
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "n < 0 or key_bits outside [1, 32]");
    if (n > kNoAllocMaxPairs)
        return report_error(SNCH_ERR_TOO_LARGE, "snch_sort_pairs_noalloc sorts at most " +
                                                    std::to_string(kNoAllocMaxPairs) + " pairs per call, got " +
                                                    std::to_string(n));
    if (n > 0 && (!keys_in || !values_in || !keys_out || !values_out))
        return report_error(SNCH_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (n == 0)
        return SNCH_OK;
    if (sort_scratch_bytes((uint32_t)kNoAllocMaxPairs, 32) > kNoAllocSortBytes)
        return report_error(SNCH_ERR_TOO_LARGE, "internal: static sort scratch is too small");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *base = nullptr;
    cudaError_t e = scratch_address(st, &base);
    if (e != cudaSuccess)
        return report_error(SNCH_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    uint32_t *tmp_keys = reinterpret_cast<uint32_t *>(base);
    uint32_t *tmp_vals = reinterpret_cast<uint32_t *>(base + kNoAllocTmpBytes);
    void *sort_scratch = base + 2 * kNoAllocTmpBytes;
    uint32_t *status = device_status ? device_status
                                     : reinterpret_cast<uint32_t *>(base + 2 * kNoAllocTmpBytes + kNoAllocSortBytes);
    // the status word of the shared array starts every call at zero (a caller's own word is the caller's)
    if (!device_status && (e = cudaMemsetAsync(status, 0, 4, st)) != cudaSuccess)
        return report_error(SNCH_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const size_t bytes = 4 * (size_t)n;
    if (keys_out != keys_in && (e = cudaMemcpyAsync(keys_out, keys_in, bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return report_error(SNCH_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    if (values_out != values_in &&
        (e = cudaMemcpyAsync(values_out, values_in, bytes, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return report_error(SNCH_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    // radix_sort_pairs clears its look-back flags, histograms and tile counters itself
    e = radix_sort_pairs(keys_out, values_out, tmp_keys, tmp_vals, (uint32_t)n, key_bits, nullptr, sort_scratch,
                         status, st);
    if (e != cudaSuccess)
        return report_error(SNCH_ERR_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
    return SNCH_OK;
}

}  // extern "C"
