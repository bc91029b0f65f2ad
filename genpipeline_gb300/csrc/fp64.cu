// fp64.cu -- FP64 element work through the modal form of the isotropic cube element
// (see apply_modal.cuh): the outer defect-correction residual f - K(x) u and the element
// energies of the sensitivity. GB300 runs FP64 at a small fraction of its FP32 rate, so the
// ~140-210 FP64 operations of the modal form per element replace 576 DFMA.
#include "apply_modal.cuh"
#include "internal.h"
#include "modal_dd.cuh"

namespace gbs {

// q = T^T v per component (Walsh-Hadamard; mode bit set = difference along that axis).
__device__ __forceinline__ void hadamard_fwd(double (&v)[8][3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double u0 = v[b][c], u1 = v[b | bit][c];
                v[b][c] = u0 + u1;
                v[b | bit][c] = u1 - u0;
            }
        }
    }
}

__device__ __forceinline__ void gather_corners64(int nx, int ny, int nz, int i, int j, int k, const double *p,
                                                 const uint8_t *mask, double (&v)[8][3]) {
    const int64_t NY = ny + 1, NZ = nz + 1;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int64_t n = ((int64_t)(i + (b >> 2)) * NY + (j + ((b >> 1) & 1))) * NZ + (k + (b & 1));
        const uint8_t m = mask ? mask[n] : (uint8_t)0;
#pragma unroll
        for (int c = 0; c < 3; ++c) v[b][c] = ((m >> c) & 1) ? 0.0 : p[3 * n + c];
    }
}

// Element pass: C[(b*3+c) * n_elem + e] = E_e (Ke p_e) at corner b (bit order), FP64.
__global__ void __launch_bounds__(128) modal_elem64_kernel(int nx, int ny, int nz, Law<double> law, const ModalKD km,
                                                           const float *__restrict__ x, const double *__restrict__ p,
                                                           const uint8_t *__restrict__ mask, double *C) {
    const int64_t n_elem = (int64_t)nx * ny * nz;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double v[8][3];
        gather_corners64(nx, ny, nz, i, j, k, p, mask, v);
        hadamard_fwd(v);
        double r[8][3];
#pragma unroll
        for (int m = 0; m < 8; ++m)
#pragma unroll
            for (int c = 0; c < 3; ++c) r[m][c] = 0.0;
#pragma unroll
        for (int q = 0; q < kModalNnz; ++q) {
            const int ro = modal_row(q), co = modal_col(q);
            r[ro / 3][ro % 3] = fma(km.v[q], v[co / 3][co % 3], r[ro / 3][ro % 3]);
        }
        const double E = modulus(law, (double)x[e]);
#pragma unroll
        for (int m = 1; m < 8; ++m)
#pragma unroll
            for (int c = 0; c < 3; ++c) r[m][c] *= E;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int bit = 1 << d;
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                if (b & bit) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const double r0 = r[b][c], r1 = r[b | bit][c];
                    r[b][c] = r0 - r1;
                    r[b | bit][c] = r0 + r1;
                }
            }
        }
#pragma unroll
        for (int b = 0; b < 8; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) C[(b * 3 + c) * n_elem + e] = r[b][c];
    }
}

// Node pass: y_n = sum over the (up to) 8 elements around n of their corner contribution,
// corners in the fixed order b = 0..7; masked DOFs are zero.
__global__ void __launch_bounds__(256) gather64_kernel(int nx, int ny, int nz, const double *__restrict__ C,
                                                       const uint8_t *__restrict__ mask, double *y) {
    const int64_t NY = ny + 1, NZ = nz + 1;
    const int64_t n_nodes = (int64_t)(nx + 1) * NY * NZ;
    const int64_t n_elem = (int64_t)nx * ny * nz;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(n / (NY * NZ)), j = (int)((n / NZ) % NY), k = (int)(n % NZ);
        double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const int ei = i - (b >> 2), ej = j - ((b >> 1) & 1), ek = k - (b & 1);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= nx || ej >= ny || ek >= nz) continue;
            const int64_t e = ((int64_t)ei * ny + ej) * nz + ek;
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] += C[(b * 3 + c) * n_elem + e];
        }
        const uint8_t m = mask ? mask[n] : (uint8_t)0;
#pragma unroll
        for (int c = 0; c < 3; ++c) y[3 * n + c] = ((m >> c) & 1) ? 0.0 : acc[c];
    }
}

size_t apply_f64_modal_ws_bytes(int nx, int ny, int nz) { return (size_t)24 * nx * ny * nz * sizeof(double); }

int apply_f64_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                    const double *p, double *y, const uint8_t *mask, double *C, cudaStream_t st) {
    const int64_t ne = (int64_t)nx * ny * nz, nn = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    const int64_t cap = 32LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    const unsigned b1 = (unsigned)((ne + 127) / 128 < cap ? (ne + 127) / 128 : cap);
    const unsigned b2 = (unsigned)((nn + 255) / 256 < cap ? (nn + 255) / 256 : cap);
    modal_elem64_kernel<<<b1, 128, 0, st>>>(nx, ny, nz, make_law<double>(*law), ctx->kmd, x, p, mask, C);
    GBS_LAUNCH_CHECK("modal_elem64_kernel");
    gather64_kernel<<<b2, 256, 0, st>>>(nx, ny, nz, C, mask, y);
    GBS_LAUNCH_CHECK("gather64_kernel");
    return GBS_OK;
}

// ---- double-float element products (the outer residual of defect correction) --------------
// udd = the double-float split of u (h = u rounded to FP32, l = the rest rounded), fixed DOFs
// zero when a mask is given.
__global__ void split_dd_kernel(int64_t nd, const double *__restrict__ u, const uint8_t *__restrict__ mask,
                                float2 *udd) {
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        const bool fx = mask && ((mask[d / 3] >> (int)(d % 3)) & 1);
        const ddv v = fx ? ddv{0.0f, 0.0f} : dd_split(u[d]);
        udd[d] = make_float2(v.h, v.l);
    }
}

// Element pass: C[(b*3+c) * n_elem + e] = E_e (Ke u_e) at corner b, as (h, l) pairs.
__global__ void __launch_bounds__(128) modal_elem_dd_kernel(int nx, int ny, int nz, const LawDD law,
                                                            const ModalKDD km, const FastDiv fy, const FastDiv fz,
                                                            const float *__restrict__ x,
                                                            const float2 *__restrict__ udd, float2 *__restrict__ C) {
    const int64_t n_elem = (int64_t)nx * ny * nz;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten3((uint32_t)e, fy, fz, i, j, k);
        ddv v[8][3], r[8][3];
        modal_fwd_dd(ny, nz, i, j, k, udd, v);
        modal_km_dd(km, v, r);
        const ddv E = modulus_dd(law, x[e]);
#pragma unroll
        for (int m = 1; m < 8; ++m)
#pragma unroll
            for (int c = 0; c < 3; ++c) r[m][c] = dd_mul(E.h, E.l, r[m][c]);
        modal_inv_dd(r);
#pragma unroll
        for (int b = 0; b < 8; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) C[(b * 3 + c) * n_elem + e] = make_float2(r[b][c].h, r[b][c].l);
    }
}

int split_dd(const gbsimp_ctx *ctx, int64_t nd, const double *u, const uint8_t *mask, float2 *udd, cudaStream_t st) {
    int64_t b = (nd + 255) / 256;  // about one DOF per thread (elementwise)
    const int64_t cap = 64LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    split_dd_kernel<<<(unsigned)(b < cap ? (b < 1 ? 1 : b) : cap), 256, 0, st>>>(nd, u, mask, udd);
    GBS_LAUNCH_CHECK("split_dd_kernel");
    return GBS_OK;
}

int elem_dd_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                  const float2 *udd, float2 *C, cudaStream_t st) {
    const int64_t ne = (int64_t)nx * ny * nz;
    const int64_t cap = 32LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    const unsigned b1 = (unsigned)((ne + 127) / 128 < cap ? (ne + 127) / 128 : cap);
    modal_elem_dd_kernel<<<b1, 128, 0, st>>>(nx, ny, nz, make_law_dd(*law), modal_kdd(ctx->kmd), fast_div(ny),
                                             fast_div(nz), x, udd, C);
    GBS_LAUNCH_CHECK("modal_elem_dd_kernel");
    return GBS_OK;
}

}  // namespace gbs
