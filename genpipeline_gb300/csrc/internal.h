// internal.h -- functions shared between the translation units of libgbsimp.
#pragma once

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace gbs {
// A named NVTX range over a host scope: each phase of a SIMP iteration (solve with its outer
// rounds and inner PCGs, sensitivity, filter, OC update) shows as a span in a profiler's
// timeline. NVTX is header-only; with no tool attached a range costs one call.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Grids the kernels accept: positive extents and DOF indices that fit in 32 bits
// (3 (nx+1)(ny+1)(nz+1) < 2^31; node and DOF offsets are 32-bit in places). Each extent is
// widened before the +1 and bounded before the products, so no int or int64 arithmetic
// here can wrap (INT_MAX + 1, or three extents near 2^30 multiplied together).
inline bool grid_ok(int nx, int ny, int nz) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return false;
    const int64_t lim = (1LL << 31) / 3;
    const int64_t a = (int64_t)nx + 1, b = (int64_t)ny + 1, c = (int64_t)nz + 1;
    if (a >= lim || b >= lim || c >= lim) return false;
    const int64_t ab = a * b;  // < 2^62: no overflow
    if (ab >= lim) return false;
    return ab * c < lim;       // ab < 2^30 and c < 2^30: no overflow
}

int apply_f32(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
              const float *p, float *y, const uint8_t *mask, cudaStream_t st);
int apply_f64(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
              const double *p, double *y, const uint8_t *mask, cudaStream_t st);
int filter_launch(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, int mode, const float *hs,
                  const float *in, const uint8_t *preserved, float *out, cudaStream_t st);
// FP64 apply through the modal element form: an element pass writes the 24 corner
// contributions of every element to C (24 * n_elem doubles), a node pass sums them in a
// fixed order. Requires ctx->modal_ok.
size_t apply_f64_modal_ws_bytes(int nx, int ny, int nz);
int apply_f64_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                    const double *p, double *y, const uint8_t *mask, double *C, cudaStream_t st);
// Double-float element products (modal_dd.cuh). split_dd: udd = (h, l) split of u, fixed DOFs
// zero when mask is given. elem_dd_modal: the element pass of K(x) u from udd, corner
// contributions to C as (h, l) pairs in the layout of apply_f64_modal (24 * n_elem float2).
// Both require ctx->modal_ok for the element pass.
int split_dd(const gbsimp_ctx *ctx, int64_t nd, const double *u, const uint8_t *mask, float2 *udd, cudaStream_t st);
int elem_dd_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                  const float2 *udd, float2 *C, cudaStream_t st);
// gbsimp_warm_start without the argument checks (the native SIMP loop).
int warm_start_impl(const gbsimp_ctx *ctx, int64_t n, double *u, double *u_prev, double theta, cudaStream_t st);
// OC update with an explicit scratch pointer (layout of gbsimp_oc_ws_bytes).
size_t oc_ws_bytes_impl(int64_t n_elem);
// The filter row sums Hs inside an OC workspace (valid after oc_prepare_impl).
const float *oc_ws_hs(const void *ws, int64_t n_elem);
int oc_check_args(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_oc_params *prm, const float *x,
                  const float *dc, const float *xnew, const float *xphys);
int oc_prepare_impl(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const uint8_t *preserved, void *ws,
                    cudaStream_t st);
int oc_run_impl(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const gbsimp_oc_params *prm, const float *x,
                const float *dc, const uint8_t *preserved, float *xnew, float *xphys, void *ws, cudaStream_t st);
// A 4 KiB pinned host buffer private to the calling thread (for small status reads).
void *thread_pinned();
}  // namespace gbs
