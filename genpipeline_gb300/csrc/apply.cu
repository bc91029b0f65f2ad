// apply.cu -- C-ABI entry points of the element stiffness apply y = D K(x) D p.
#include "apply_modal.cuh"
#include "internal.h"

namespace gbs {

template <typename Tile, typename T, typename KeT>
int launch_apply_plain(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<T> &law, const KeT &ke,
                       const float *x, const T *p, T *y, const uint8_t *mask, cudaStream_t st) {
    TileArgs<T> A{nx, ny, nz, x, p, y, mask};
    PcgArgs pa{};
    const dim3 g = tile_grid<Tile>(nx, ny, nz), b = tile_block<Tile>();
    if (ctx->translation_free)
        apply_tile_kernel<T, KeT, Tile::X, Tile::Y, Tile::Z, true, MODE_PLAIN><<<g, b, 0, st>>>(A, law, ke, pa);
    else
        apply_tile_kernel<T, KeT, Tile::X, Tile::Y, Tile::Z, false, MODE_PLAIN><<<g, b, 0, st>>>(A, law, ke, pa);
    GBS_LAUNCH_CHECK("apply_tile_kernel");
    return GBS_OK;
}

int apply_f32(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
              const float *p, float *y, const uint8_t *mask, cudaStream_t st) {
    // the modal kernel copies p and writes y in aligned 16-byte groups
    if (ctx->modal_ok && modal_fits(nz) && !((uintptr_t)p & 15) && !((uintptr_t)y & 15))
        return launch_modal<MODE_PLAIN>(ctx, nx, ny, nz, make_law<float>(*law), x, p, y, mask, CgArgs{}, st);
    return launch_apply_plain<TileF, float, KeF>(ctx, nx, ny, nz, make_law<float>(*law), ctx->kef, x, p, y, mask,
                                                 st);
}

int apply_f64(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
              const double *p, double *y, const uint8_t *mask, cudaStream_t st) {
    return launch_apply_plain<TileD, double, KeD>(ctx, nx, ny, nz, make_law<double>(*law), ctx->ked, x, p, y,
                                                  mask, st);
}

// ---- arbitrary edof table (drop-in for cuda_kernels.fused_spmv / simp_sensitivity) ----
template <typename I>
__device__ __forceinline__ int64_t edof_at(const void *edof, int64_t i) {
    return (int64_t)((const I *)edof)[i];
}

__global__ void zero_f32_kernel(float *y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = 0.0f;
}

// One thread per element: gather p_e, y_e = E_e Ke p_e, scatter with atomics. Indices
// outside [0, n_dof) read as 0 and are not written (as the reference kernel clamps them,
// cuda_kernels/simp_sensitivity_ptx.cu:223-230).
template <typename I>
__global__ void apply_edof_kernel(int64_t n_elem, int64_t n_dof, const void *edof, Law<float> law, const KeF ke,
                                  const float *x, const float *p, float *y) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    int64_t idx[24];
    float pe[24];
#pragma unroll
    for (int q = 0; q < 24; ++q) {
        idx[q] = edof_at<I>(edof, e * 24 + q);
        pe[q] = (idx[q] >= 0 && idx[q] < n_dof) ? p[idx[q]] : 0.0f;
    }
    const float E = modulus(law, x[e]);
#pragma unroll
    for (int r = 0; r < 24; ++r) {
        float s = 0.0f;
#pragma unroll
        for (int q = 0; q < 24; ++q) s = fmaf(ke.k[r * 24 + q], pe[q], s);
        if (idx[r] >= 0 && idx[r] < n_dof) atomicAdd(&y[idx[r]], E * s);
    }
}

template <typename I>
__global__ void sens_edof_kernel(int64_t n_elem, int64_t n_dof, const void *edof, Law<float> law, const KeF ke,
                                 const float *x, const float *u, float *dc) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    float ue[24];
#pragma unroll
    for (int q = 0; q < 24; ++q) {
        const int64_t d = edof_at<I>(edof, e * 24 + q);
        ue[q] = (d >= 0 && d < n_dof) ? u[d] : 0.0f;
    }
    double ce = 0.0;
#pragma unroll
    for (int r = 0; r < 24; ++r) {
        float s = 0.0f;
#pragma unroll
        for (int q = 0; q < 24; ++q) s = fmaf(ke.k[r * 24 + q], ue[q], s);
        ce += (double)ue[r] * (double)s;
    }
    dc[e] = -dmodulus(law, x[e]) * (float)ce;
}

}  // namespace gbs

using namespace gbs;

extern "C" int gbsimp_apply_f32(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                                const float *p, float *y, const uint8_t *node_mask, void *stream) {
    if (!ctx || !law || !x || !p || !y || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_apply_f32: bad arguments");
    return apply_f32(ctx, nx, ny, nz, law, x, p, y, node_mask, (cudaStream_t)stream);
}

extern "C" int gbsimp_apply_path(const gbsimp_ctx *ctx, int nz) {
    if (!ctx) return -1;
    return (ctx->modal_ok && modal_fits(nz)) ? 1 : 0;
}

extern "C" int gbsimp_apply_f64(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                                const double *p, double *y, const uint8_t *node_mask, void *stream) {
    if (!ctx || !law || !x || !p || !y || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_apply_f64: bad arguments");
    return apply_f64(ctx, nx, ny, nz, law, x, p, y, node_mask, (cudaStream_t)stream);
}

extern "C" int gbsimp_apply_edof_f32(gbsimp_ctx *ctx, int64_t n_elem, int64_t n_dof, const void *edof,
                                     int edof_is_int64, const gbsimp_law *law, const float *x, const float *p,
                                     float *y, void *stream) {
    if (!ctx || !law || !edof || !x || !p || !y || n_elem < 0 || n_dof < 0)
        return set_error(GBS_EINVAL, "gbsimp_apply_edof_f32: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_dof > 0) {
        zero_f32_kernel<<<(unsigned)((n_dof + 255) / 256 < 65535 ? (n_dof + 255) / 256 : 65535), 256, 0, st>>>(y, n_dof);
        GBS_LAUNCH_CHECK("zero_f32_kernel");
    }
    if (n_elem == 0) return GBS_OK;
    const unsigned blocks = (unsigned)((n_elem + 127) / 128);
    if (edof_is_int64)
        apply_edof_kernel<int64_t><<<blocks, 128, 0, st>>>(n_elem, n_dof, edof, make_law<float>(*law), ctx->kef, x, p, y);
    else
        apply_edof_kernel<int32_t><<<blocks, 128, 0, st>>>(n_elem, n_dof, edof, make_law<float>(*law), ctx->kef, x, p, y);
    GBS_LAUNCH_CHECK("apply_edof_kernel");
    return GBS_OK;
}

extern "C" int gbsimp_sensitivity_edof_f32(gbsimp_ctx *ctx, int64_t n_elem, int64_t n_dof, const void *edof,
                                           int edof_is_int64, const gbsimp_law *law, const float *x,
                                           const float *u, float *dc, void *stream) {
    if (!ctx || !law || !edof || !x || !u || !dc || n_elem < 0 || n_dof < 0)
        return set_error(GBS_EINVAL, "gbsimp_sensitivity_edof_f32: bad arguments");
    if (n_elem == 0) return GBS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned blocks = (unsigned)((n_elem + 127) / 128);
    if (edof_is_int64)
        sens_edof_kernel<int64_t><<<blocks, 128, 0, st>>>(n_elem, n_dof, edof, make_law<float>(*law), ctx->kef, x, u, dc);
    else
        sens_edof_kernel<int32_t><<<blocks, 128, 0, st>>>(n_elem, n_dof, edof, make_law<float>(*law), ctx->kef, x, u, dc);
    GBS_LAUNCH_CHECK("sens_edof_kernel");
    return GBS_OK;
}
