// voxel.cu -- the evaluator's input step on the device.
//
// A decoded (D, H, W) density grid is resampled with linear interpolation, as
// scipy.ndimage.zoom(v, 0.5, order=1) does in VoxelFEMEvaluator.evaluate
// (fem/voxel_fem.py:457-459): output index o reads input coordinate o (n_in - 1) / (n_out - 1)
// (grid_mode off), weights (1 - w, w) on floor and floor + 1, nothing beyond the last input.
// It is then filtered as smooth_voxels does (pipeline_utils.py:55-76): a Gaussian of sigma
// voxels (radius int(4 sigma + 0.5), weights exp(-t^2 / (2 sigma^2)) normalised to sum 1,
// mirror boundary "reflect": d c b a | a b c d | d c b a), then the logistic
// 1 / (1 + exp(-sharpness (v - 0.5))).
//
// Both linear steps are separable, so each axis gets one banded n_out x n_in matrix
// A = G Z, built on the device in FP64, and a batch of volumes goes through three 1-D passes
// (z, y, x; FP64 sums, FP32 between passes, like the reference's float32 intermediates); the
// last pass applies the logistic.
#include <math.h>

#include "internal.h"

namespace gbs {

constexpr int kVoxBand = 32;      // nonzeros per row of A
constexpr int kVoxMaxExtent = 1024;

struct VoxRow {
    long long start;
    double w[kVoxBand];
};

static size_t al256v(size_t b) { return (b + 255) & ~(size_t)255; }

static inline int vox_radius(double sigma) { return sigma > 0.0 ? (int)(4.0 * sigma + 0.5) : 0; }

// Input span of one row of G Z (host check of the band).
static int vox_span(int n_in, int n_out, double sigma) {
    const double s = n_out > 1 ? (double)(n_in - 1) / (double)(n_out - 1) : 0.0;
    return (int)ceil(2.0 * vox_radius(sigma) * s) + 3;
}

__device__ __forceinline__ int vox_reflect(int j, int n) {
    // half-sample symmetric extension, repeated for offsets longer than the axis
    const int period = 2 * n;
    j %= period;
    if (j < 0) j += period;
    return j < n ? j : period - 1 - j;
}

// One thread per output row of one axis.
__global__ void vox_table_kernel(int n_in, int n_out, double sigma, VoxRow *rows) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_out) return;
    const int r = sigma > 0.0 ? (int)(4.0 * sigma + 0.5) : 0;
    const double s = n_out > 1 ? (double)(n_in - 1) / (double)(n_out - 1) : 0.0;
    double norm = 0.0;
    for (int t = -r; t <= r; ++t) norm += r > 0 ? exp(-0.5 / (sigma * sigma) * (double)(t * t)) : 1.0;
    long long lo = 1LL << 40;
    for (int t = -r; t <= r; ++t) {
        const int j = vox_reflect(o + t, n_out);
        const long long i0 = (long long)floor((double)j * s);
        lo = i0 < lo ? i0 : lo;
    }
    VoxRow &R = rows[o];
    R.start = lo;
    for (int k = 0; k < kVoxBand; ++k) R.w[k] = 0.0;
    for (int t = -r; t <= r; ++t) {
        const double g = (r > 0 ? exp(-0.5 / (sigma * sigma) * (double)(t * t)) : 1.0) / norm;
        const int j = vox_reflect(o + t, n_out);
        const double p = (double)j * s;
        const long long i0 = (long long)floor(p);
        const double w = p - (double)i0;
        const long long k0 = i0 - lo;
        if (k0 >= 0 && k0 < kVoxBand) R.w[k0] += g * (1.0 - w);
        if (i0 + 1 < n_in && k0 + 1 < kVoxBand) R.w[k0 + 1] += g * w;
    }
}

// out[b, a, o, c] = sum_k A[o][k] in[b, a, start_o + k, c] for an axis of length n_in with
// `outer` = batch x leading extent and `inner` = trailing extent (1 for the last axis).
__global__ void vox_pass_kernel(long long outer, int n_in, int n_out, long long inner, const float *__restrict__ in,
                                const VoxRow *__restrict__ rows, float *__restrict__ out, int logistic,
                                double sharpness) {
    const long long total = outer * n_out * inner;
    for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < total;
         id += (long long)gridDim.x * blockDim.x) {
        const long long c = id % inner;
        const long long rest = id / inner;
        const int o = (int)(rest % n_out);
        const long long a = rest / n_out;
        const VoxRow &R = rows[o];
        const float *src = in + a * n_in * inner + c;
        double acc = 0.0;
#pragma unroll 4
        for (int k = 0; k < kVoxBand; ++k) {
            const long long i = R.start + k;
            if (i >= 0 && i < n_in && R.w[k] != 0.0) acc += R.w[k] * (double)src[i * inner];
        }
        if (logistic) acc = 1.0 / (1.0 + exp(-sharpness * (acc - 0.5)));
        out[id] = (float)acc;
    }
}

static bool vox_dims_ok(int n_in, int n_out) {
    return n_in >= 1 && n_in <= kVoxMaxExtent && n_out >= 1 && n_out <= kVoxMaxExtent && (n_out >= 2 || n_in == 1);
}

static size_t vox_ws_bytes_impl(int batch, int D, int H, int W, int d, int h, int w) {
    return 256 + al256v(sizeof(VoxRow) * ((size_t)d + h + w)) + al256v(4 * (size_t)batch * D * H * w) +
           al256v(4 * (size_t)batch * D * h * w);
}

}  // namespace gbs

using namespace gbs;

extern "C" size_t gbsimp_voxel_prep_ws_bytes(int batch, int D, int H, int W, int d, int h, int w) {
    if (batch <= 0 || !vox_dims_ok(D, d) || !vox_dims_ok(H, h) || !vox_dims_ok(W, w)) return 0;
    return vox_ws_bytes_impl(batch, D, H, W, d, h, w);
}

extern "C" int gbsimp_voxel_prep(gbsimp_ctx *ctx, int batch, int D, int H, int W, const float *in, int d, int h,
                                 int w, float *out, double sigma, double sharpness, void *ws, size_t ws_bytes,
                                 void *stream) {
    if (!ctx || !in || !out || !ws || batch <= 0 || !vox_dims_ok(D, d) || !vox_dims_ok(H, h) ||
        !vox_dims_ok(W, w) || !(sigma >= 0.0) || !(sigma <= 64.0) || !isfinite(sharpness))
        return set_error(GBS_EINVAL, "gbsimp_voxel_prep: bad arguments");
    if (vox_span(D, d, sigma) > kVoxBand || vox_span(H, h, sigma) > kVoxBand || vox_span(W, w, sigma) > kVoxBand)
        return set_error(GBS_EINVAL, "gbsimp_voxel_prep: sigma %g with this zoom needs more than %d taps per row",
                         sigma, kVoxBand);
    if (ws_bytes < vox_ws_bytes_impl(batch, D, H, W, d, h, w))
        return set_error(GBS_EINVAL, "gbsimp_voxel_prep: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    char *p = (char *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
    VoxRow *rx = (VoxRow *)p, *ry = rx + d, *rz = ry + h;
    p += al256v(sizeof(VoxRow) * ((size_t)d + h + w));
    float *t1 = (float *)p;  // (batch, D, H, w)
    p += al256v(4 * (size_t)batch * D * H * w);
    float *t2 = (float *)p;  // (batch, D, h, w)
    vox_table_kernel<<<(d + 127) / 128, 128, 0, st>>>(D, d, sigma, rx);
    GBS_LAUNCH_CHECK("vox_table_kernel");
    vox_table_kernel<<<(h + 127) / 128, 128, 0, st>>>(H, h, sigma, ry);
    GBS_LAUNCH_CHECK("vox_table_kernel");
    vox_table_kernel<<<(w + 127) / 128, 128, 0, st>>>(W, w, sigma, rz);
    GBS_LAUNCH_CHECK("vox_table_kernel");
    auto blocks = [&](long long n) {
        long long b = (n + 255) / 256;
        const long long cap = 8LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
        return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
    };
    const long long B = batch;
    vox_pass_kernel<<<blocks(B * D * H * w), 256, 0, st>>>(B * D * H, W, w, 1, in, rz, t1, 0, 0.0);
    GBS_LAUNCH_CHECK("vox_pass_kernel");
    vox_pass_kernel<<<blocks(B * D * h * w), 256, 0, st>>>(B * D, H, h, w, t1, ry, t2, 0, 0.0);
    GBS_LAUNCH_CHECK("vox_pass_kernel");
    vox_pass_kernel<<<blocks(B * d * h * w), 256, 0, st>>>(B, D, d, (long long)h * w, t2, rx, out, 1, sharpness);
    GBS_LAUNCH_CHECK("vox_pass_kernel");
    return GBS_OK;
}
