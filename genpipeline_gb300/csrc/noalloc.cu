// noalloc.cu -- the OC update for callers that cannot allocate device memory.
//
// gbsimp_oc needs scratch (filter row sums, volume weights, reduction partials) from the
// caller. Some callers have no way to provide it: a host-language plugin that reaches the
// GPU only through this C ABI and owns no CUDA allocator, or a serving process whose device
// memory is fully reserved up front and must not grow or fragment per request. For them
// gbsimp_oc_noalloc takes its scratch from the fixed device array below instead.
#include <mutex>

#include "internal.h"

// Scratch of gbsimp_oc_noalloc: 16.1 MiB, enough for GBSIMP_OC_NOALLOC_MAX_ELEMENTS
// elements. It is a module-scope device array: every GPU that loads this library holds it
// until the process exits, whether or not the entry point is called.
#define GBS_OC_NOALLOC_BYTES (256 + 2 * (4 * GBSIMP_OC_NOALLOC_MAX_ELEMENTS) + 4 * 4096 * 8)
static __device__ __align__(256) unsigned char g_oc_noalloc_scratch[GBS_OC_NOALLOC_BYTES];

namespace {
std::mutex g_scratch_mu;
void *g_scratch_ptr[128];  // device address of the array, per device ordinal
}  // namespace

// The array's name is a host-side stand-in, not a device address: host code must ask the
// runtime for the address on the current device (once per device, cached).
static int scratch_on_current_device(const gbsimp_ctx *ctx, void **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gbs::cuda_error(e, "cudaGetDevice");
    if (dev != ctx->device) return gbs::set_error(GBS_EINVAL, "gbsimp_oc_noalloc: make the context's device current");
    if (dev < 0 || dev >= 128) return gbs::set_error(GBS_EINVAL, "gbsimp_oc_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_oc_noalloc_scratch);
        if (e != cudaSuccess || !p) return gbs::cuda_error(e, "cudaGetSymbolAddress(g_oc_noalloc_scratch)");
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return GBS_OK;
}

extern "C" int gbsimp_oc_noalloc(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin,
                                 const gbsimp_oc_params *prm, const float *x, const float *dc,
                                 const uint8_t *preserved, float *xnew, float *xphys, void *stream) {
    int rc = gbs::oc_check_args(ctx, nx, ny, nz, prm, x, dc, xnew, xphys);
    if (rc) return rc;
    const int64_t n = (int64_t)nx * ny * nz;
    if (n > GBSIMP_OC_NOALLOC_MAX_ELEMENTS)
        return gbs::set_error(GBS_EINVAL,
                              "gbsimp_oc_noalloc: %lld elements exceed its static scratch (at most %d elements); "
                              "use gbsimp_oc with a caller-provided workspace",
                              (long long)n, (int)GBSIMP_OC_NOALLOC_MAX_ELEMENTS);
    if (gbs::oc_ws_bytes_impl(n) > sizeof(g_oc_noalloc_scratch))
        return gbs::set_error(GBS_EINVAL, "gbsimp_oc_noalloc: scratch layout larger than the static array");
    void *ws = nullptr;
    rc = scratch_on_current_device(ctx, &ws);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // The array keeps the previous call's contents: the prepare step zeroes the reduction
    // scalars and recomputes the filter row sums and volume weights for this grid.
    rc = gbs::oc_prepare_impl(ctx, nx, ny, nz, rmin, preserved, ws, st);
    if (rc) return rc;
    return gbs::oc_run_impl(ctx, nx, ny, nz, rmin, prm, x, dc, preserved, xnew, xphys, ws, st);
}
