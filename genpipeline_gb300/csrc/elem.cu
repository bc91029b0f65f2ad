// elem.cu -- element-wise kernels: sensitivity/compliance, density filter, OC bisection,
// FP64 dot. All reductions: per-block partials (FP64; double-float in the OC multisection),
// summed in a fixed order by the last block to finish (deterministic for a given launch
// shape).
#include <math.h>
#include <string.h>

#include <atomic>

#include "internal.h"
#include "modal_dd.cuh"

namespace gbs {

// ---- last-block reduction helper -----------------------------------------------------
// Every block calls it with its partial(s); returns true in the last block, whose threads
// then see the K sums of all partials in out[0..K-1] (shared). counter is reset.
template <int K>
__device__ bool last_block_reduce(const double (&v)[K], double *partials, unsigned *counter, double *out,
                                  double *sred) {
    __shared__ bool last;
    const int nblk = gridDim.x;
    double bs[K];
#pragma unroll
    for (int k = 0; k < K; ++k) bs[k] = block_sum(v[k], sred);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) partials[k * nblk + blockIdx.x] = bs[k];
        __threadfence();
        last = (atomicAdd(counter, 1u) == (unsigned)(nblk - 1));
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = 0.0;
        for (int i = threadIdx.x; i < nblk; i += blockDim.x) s += ((volatile double *)partials)[k * nblk + i];
        s = block_sum(s, sred);
        if (threadIdx.x == 0) out[k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = 0;
    return true;
}

inline unsigned reduce_blocks(const gbsimp_ctx *ctx, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = 4LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// ---- sensitivity ------------------------------------------------------------------------
// Thread per element: u_e gathered in FP64; ce = u_e^T Ke u_e through the modal form
// (q = T^T u_e, the 45 nonzeros of Km) when Ke has it, else the dense product (minus node 0's
// displacement when Ke annihilates translations); dc = -dE/dx ce, energy partial E ce.
__global__ void __launch_bounds__(128) sens_kernel(int nx, int ny, int nz, Law<double> law, const KeD ke, int sub,
                                                   int modal, const ModalKD kmd,
                                                   const float *__restrict__ x, const double *__restrict__ u,
                                                   float *dc, float *ce_out, double *partials, unsigned *counter,
                                                   double *energy_out) {
    __shared__ double sred[32];
    __shared__ double tot[1];
    const int64_t n_elem = (int64_t)nx * ny * nz;
    const int64_t NY = ny + 1, NZ = nz + 1;
    double part = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double ue[24];
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const int64_t m = ((int64_t)(i + corner_x(b)) * NY + (j + corner_y(b))) * NZ + (k + corner_z(b));
#pragma unroll
            for (int c = 0; c < 3; ++c) ue[3 * b + c] = u[3 * m + c];
        }
        double s = 0.0;
        if (modal) {
            // ce = q^T Km q with q = T^T u_e (Walsh-Hadamard of the corner values): the
            // translation modes drop out exactly and only the 45 nonzeros of Km are used.
            double q[8][3];
#pragma unroll
            for (int a = 0; a < 8; ++a) {
                const int b = corner_x(a) * 4 + corner_y(a) * 2 + corner_z(a);
#pragma unroll
                for (int c = 0; c < 3; ++c) q[b][c] = ue[3 * a + c];
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int bit = 1 << d;
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    if (b & bit) continue;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const double u0 = q[b][c], u1 = q[b | bit][c];
                        q[b][c] = u0 + u1;
                        q[b | bit][c] = u1 - u0;
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < kModalNnz; ++t) {
                const int ro = modal_row(t), co = modal_col(t);
                s = fma(kmd.v[t] * q[ro / 3][ro % 3], q[co / 3][co % 3], s);
            }
        } else {
            if (sub) {
                const double c0 = ue[0], c1 = ue[1], c2 = ue[2];
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    ue[3 * b] -= c0;
                    ue[3 * b + 1] -= c1;
                    ue[3 * b + 2] -= c2;
                }
            }
#pragma unroll
            for (int r = 0; r < 24; ++r) {
                double t = 0.0;
#pragma unroll
                for (int q = 0; q < 24; ++q) t = fma(ke.k[r * 24 + q], ue[q], t);
                s = fma(ue[r], t, s);
            }
        }
        const double xe = (double)x[e];
        if (dc) dc[e] = (float)(-dmodulus(law, xe) * s);
        if (ce_out) ce_out[e] = (float)s;
        part += modulus(law, xe) * s;
    }
    if (energy_out) {
        const double v[1] = {part};
        if (last_block_reduce<1>(v, partials, counter, tot, sred) && threadIdx.x == 0) *energy_out = tot[0];
    }
}

// The same through the double-float modal form (modal_dd.cuh), from the split displacements:
// ce = q^T Km q accumulated in double-float, then dc, ce and the energy partial as above.
__global__ void __launch_bounds__(128) sens_dd_kernel(int nx, int ny, int nz, Law<double> law, const ModalKDD km,
                                                      const FastDiv fy, const FastDiv fz,
                                                      const float *__restrict__ x, const float2 *__restrict__ udd,
                                                      float *dc, float *ce_out, double *partials, unsigned *counter,
                                                      double *energy_out) {
    __shared__ double sred[32];
    __shared__ double tot[1];
    const int64_t n_elem = (int64_t)nx * ny * nz;
    double part = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten3((uint32_t)e, fy, fz, i, j, k);
        ddv q[8][3], r[8][3];
        modal_fwd_dd(ny, nz, i, j, k, udd, q);
        modal_km_dd(km, q, r);
        ddv s{0.0f, 0.0f};
#pragma unroll
        for (int m = 1; m < 8; ++m)
#pragma unroll
            for (int c = 0; c < 3; ++c) s = dd_add(s, dd_mul(q[m][c].h, q[m][c].l, r[m][c]));
        const double ce = dd_value(s);
        const double xe = (double)x[e];
        if (dc) dc[e] = (float)(-dmodulus(law, xe) * ce);
        if (ce_out) ce_out[e] = (float)ce;
        part += modulus(law, xe) * ce;
    }
    if (energy_out) {
        const double v[1] = {part};
        if (last_block_reduce<1>(v, partials, counter, tot, sred) && threadIdx.x == 0) *energy_out = tot[0];
    }
}

// ---- density filter ---------------------------------------------------------------------
constexpr int kMaxStencil = 1024;
struct Stencil {
    int n;
    int r;
    int flat;              // 1: doff[] holds the flat offsets of this grid
    int off[kMaxStencil];  // dx, dy, dz packed as signed bytes
    float w[kMaxStencil];  // rmin - dist > 0
    int doff[kMaxStencil]; // (dx ny + dy) nz + dz: the element offset in x-y-z order
};

// The neighbourhood of simp_solver.py:1553-1565: offsets of the box of half-width
// ceil(rmin) with dist <= rmin; zero weights (dist == rmin) are dropped (they add nothing).
static int make_stencil(double rmin, Stencil *s) {
    if (!(rmin > 0.0) || rmin > 6.0) return set_error(GBS_EINVAL, "filter: rmin must be in (0, 6], got %g", rmin);
    const int r = (int)ceil(rmin);
    s->n = 0;
    s->r = r;
    s->flat = 0;
    for (int di = -r; di <= r; ++di)
        for (int dj = -r; dj <= r; ++dj)
            for (int dk = -r; dk <= r; ++dk) {
                const double d = sqrt((double)(di * di + dj * dj + dk * dk));
                if (d > rmin) continue;
                const double w = rmin - d;
                if (!(w > 0.0)) continue;
                if (s->n >= kMaxStencil) return set_error(GBS_EINVAL, "filter: stencil too large");
                s->off[s->n] = (int)(((unsigned)(uint8_t)(int8_t)di) | ((unsigned)(uint8_t)(int8_t)dj << 8) |
                                     ((unsigned)(uint8_t)(int8_t)dk << 16));
                s->w[s->n] = (float)w;
                ++s->n;
            }
    return GBS_OK;
}

// The flat element offsets of the stencil for a grid of ny x nz element rows, when every
// one fits in an int (s->flat = 1; otherwise the kernel uses the bounds-checked path only).
static void set_flat_offsets(int ny, int nz, Stencil *s) {
    const int64_t reach = (int64_t)s->r * ((int64_t)ny * nz + nz + 1);
    s->flat = reach < INT32_MAX ? 1 : 0;
    if (!s->flat) return;
    for (int q = 0; q < s->n; ++q) {
        const int o = s->off[q];
        const int di = (int)(int8_t)(o & 0xff), dj = (int)(int8_t)((o >> 8) & 0xff), dk = (int)(int8_t)((o >> 16) & 0xff);
        s->doff[q] = (int)(((int64_t)di * ny + dj) * nz + dk);
    }
}

__device__ __forceinline__ void neumaier_add(float &s, float &c, float v) {
    const float t = s + v;
    c += fabsf(s) >= fabsf(v) ? (s - t) + v : (v - t) + s;
    s = t;
}

__device__ __forceinline__ void unpack_off(int o, int &di, int &dj, int &dk) {
    di = (int)(int8_t)(o & 0xff);
    dj = (int)(int8_t)((o >> 8) & 0xff);
    dk = (int)(int8_t)((o >> 16) & 0xff);
}

// mode 0: out = (sum w v) / hs[e] (hs nullable: computed);  mode 1: out = sum w v/hs[e2];
// mode 2 (hs): out = sum w over in-bounds neighbours. preserved (mode 0): out = 1 there.
__global__ void __launch_bounds__(256) filter_kernel(int nx, int ny, int nz, const FastDiv fy, const FastDiv fz,
                                                     const Stencil st, int mode,
                                                     const float *__restrict__ hs, const float *__restrict__ in,
                                                     const uint8_t *__restrict__ preserved, float *out) {
    const int64_t n_elem = (int64_t)nx * ny * nz;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten3((uint32_t)e, fy, fz, i, j, k);
        // FP32 with compensated (Neumaier) summation in the fixed stencil order: error of a
        // few ulp whatever the stencil size (up to ~900 terms at rmin 6).
        float s = 0.0f, sc = 0.0f, ws = 0.0f, wc = 0.0f;
        // Away from the x and y faces only z can leave the grid: the same terms in the same
        // order, with one z test and a precomputed flat offset per term (a warp's elements
        // lie in one or two z columns, so the branch rarely splits a warp).
        if (st.flat && i >= st.r && i < nx - st.r && j >= st.r && j < ny - st.r) {
            for (int q = 0; q < st.n; ++q) {
                const int k2 = k + (int)(int8_t)((st.off[q] >> 16) & 0xff);
                if (k2 < 0 || k2 >= nz) continue;
                const int64_t e2 = e + st.doff[q];
                const float w = st.w[q];
                neumaier_add(ws, wc, w);
                if (mode == 0) neumaier_add(s, sc, w * in[e2]);
                else if (mode == 1) neumaier_add(s, sc, w * (in[e2] / hs[e2]));
            }
        } else {
            for (int q = 0; q < st.n; ++q) {
                int di, dj, dk;
                unpack_off(st.off[q], di, dj, dk);
                const int i2 = i + di, j2 = j + dj, k2 = k + dk;
                if (i2 < 0 || i2 >= nx || j2 < 0 || j2 >= ny || k2 < 0 || k2 >= nz) continue;
                const int64_t e2 = ((int64_t)i2 * ny + j2) * nz + k2;
                const float w = st.w[q];
                neumaier_add(ws, wc, w);
                if (mode == 0) neumaier_add(s, sc, w * in[e2]);
                else if (mode == 1) neumaier_add(s, sc, w * (in[e2] / hs[e2]));
            }
        }
        s += sc;
        ws += wc;
        float o;
        if (mode == 0) {
            const float h = hs ? hs[e] : ws;
            o = s / h;
            if (preserved && preserved[e]) o = 1.0f;
        } else if (mode == 1) {
            o = (float)s;
        } else {
            o = (float)ws;
        }
        out[e] = o;
    }
}

static unsigned elem_blocks(const gbsimp_ctx *ctx, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = 32LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

int filter_launch(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, int mode, const float *hs,
                  const float *in, const uint8_t *preserved, float *out, cudaStream_t st) {
    Stencil s;
    int rc = make_stencil(rmin, &s);
    if (rc) return rc;
    set_flat_offsets(ny, nz, &s);
    const int64_t n = (int64_t)nx * ny * nz;
    filter_kernel<<<elem_blocks(ctx, n, 256), 256, 0, st>>>(nx, ny, nz, fast_div(ny), fast_div(nz), s, mode, hs, in,
                                                            preserved, out);
    GBS_LAUNCH_CHECK("filter_kernel");
    return GBS_OK;
}

// ---- OC bisection -----------------------------------------------------------------------
struct OcScalars {
    double l1, l2, lfinal, npres;
    int steps, done;
    unsigned counter;
    unsigned bar;  // grid barrier of oc_coop_kernel (monotonic within one call)
    int status;    // GBS_ETIMEOUT when a barrier wait of oc_coop_kernel ran out
    int pad;
};

struct OcParams {
    float move, sqrt_floor;
    double tol, tol_eps, volfrac, l1, l2;
    int max_bisect;
};

// Workspace: [OcScalars (256 B)] [hs: n floats] [w: n floats] [partials: 4*cap doubles]
struct OcWs {
    OcScalars *sc;
    float *hs, *w;
    double *partials;
};

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static size_t oc_ws_bytes(int64_t n) {
    return 256 + 2 * align256((size_t)n * sizeof(float)) + align256(4 * 4096 * sizeof(double));
}

static OcWs oc_ws(void *ws, int64_t n) {
    char *p = (char *)ws;
    OcWs w;
    w.sc = (OcScalars *)p;
    p += 256;
    w.hs = (float *)p;
    p += align256((size_t)n * sizeof(float));
    w.w = (float *)p;
    p += align256((size_t)n * sizeof(float));
    w.partials = (double *)p;
    return w;
}

// w_e = sum_{e1 in ball(e), e1 not preserved} H[e1,e] / Hs[e1];  npres = #preserved.
__global__ void oc_weights_kernel(int nx, int ny, int nz, const Stencil st, const float *__restrict__ hs,
                                  const uint8_t *__restrict__ preserved, float *w, double *partials, OcScalars *sc) {
    __shared__ double sred[32];
    __shared__ double tot[1];
    const int64_t n_elem = (int64_t)nx * ny * nz;
    double np = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / ((int64_t)ny * nz)), j = (int)((e / nz) % ny), k = (int)(e % nz);
        double s = 0.0;
        for (int q = 0; q < st.n; ++q) {
            int di, dj, dk;
            unpack_off(st.off[q], di, dj, dk);
            const int i2 = i + di, j2 = j + dj, k2 = k + dk;
            if (i2 < 0 || i2 >= nx || j2 < 0 || j2 >= ny || k2 < 0 || k2 >= nz) continue;
            const int64_t e2 = ((int64_t)i2 * ny + j2) * nz + k2;
            if (preserved && preserved[e2]) continue;
            s += (double)st.w[q] / (double)hs[e2];
        }
        w[e] = (float)s;
        if (preserved && preserved[e]) np += 1.0;
    }
    const double v[1] = {np};
    if (last_block_reduce<1>(v, partials, &sc->counter, tot, sred) && threadIdx.x == 0) sc->npres = tot[0];
}

__device__ __forceinline__ float oc_trial(float x, float dc, float inv_l, const OcParams &P, bool pres) {
    float t = -dc * inv_l;
    t = t > P.sqrt_floor ? t : P.sqrt_floor;
    float v = x * sqrtf(t);
    v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    const float lo = x - P.move, hi = x + P.move;
    v = v < lo ? lo : v;
    v = v > hi ? hi : v;
    return pres ? 1.0f : v;
}

__global__ void oc_init_kernel(int64_t n, const OcParams P, const float *__restrict__ dc, double *partials,
                               OcScalars *sc) {
    sc->done = 0;  // every block writes the same values
    sc->steps = 0;
    sc->bar = 0;
    sc->status = 0;
    if (P.l2 >= 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            sc->l1 = P.l1;
            sc->l2 = P.l2;
            sc->lfinal = 0.5 * (P.l1 + P.l2);
        }
        return;
    }
    // l2 = 2 * max(max(-dc), 1)  (simp_solver_gpu.py:813); max via a sum of per-block maxima
    // would lose the max, so partials carry maxima and the last block takes their max.
    float m = -INFINITY;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, -dc[e]);
    m = warp_max(m);
    __shared__ float wm[32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wm[wid] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = -INFINITY;
        for (int i = 0; i < (int)((blockDim.x + 31) >> 5); ++i) b = fmaxf(b, wm[i]);
        partials[blockIdx.x] = (double)b;
        __threadfence();
        last = (atomicAdd(&sc->counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double mm = -INFINITY;
        for (unsigned i = 0; i < gridDim.x; ++i) mm = fmax(mm, ((volatile double *)partials)[i]);
        sc->counter = 0;
        sc->l1 = P.l1;
        sc->l2 = 2.0 * (mm > 1.0 ? mm : 1.0);
        sc->lfinal = 0.5 * (sc->l1 + sc->l2);
    }
}

// ---- multisection: kOcLevels bisection steps per launch ---------------------------------
// The bisection of simp_solver.py:229-247 visits one midpoint per step. One launch evaluates
// the volume at every midpoint the next kOcLevels steps could visit: the 2^kOcLevels - 1 nodes
// of the binary tree below (l1, l2), heap-ordered (node t: children 2t + 1 = [lo, mid] and
// 2t + 2 = [mid, hi]), each midpoint formed as bisection forms it, 0.5 (hi + lo) of its
// parent interval. The last block then walks the tree with bisection's tests (stop on
// (l2 - l1) / (l1 + l2 + eps) < tol, then vol > volfrac -> l1 = mid, else l2 = mid), so the
// sequence of intervals, lfinal and the step count are those of one launch per step (up to
// the rounding of the volume sums), in max_bisect / kOcLevels launches.
constexpr int kOcLevels = 5;
constexpr int kOcNodes = (1 << kOcLevels) - 1;
constexpr int kOcThreads = 256;

__global__ void __launch_bounds__(kOcThreads) oc_multi_kernel(int64_t n, const OcParams P, const float *__restrict__ x,
                                                              const float *__restrict__ dc,
                                                              const uint8_t *__restrict__ pres,
                                                              const float *__restrict__ w, float2 *partials,
                                                              OcScalars *sc) {
    __shared__ float s_sq[kOcNodes];    // sqrt(1 / mid) of node t
    __shared__ bool s_stop[kOcNodes];   // the stop test on node t's interval
    __shared__ double s_mid[kOcNodes];  // midpoint of node t
    __shared__ float s_part[kOcNodes][kOcThreads];
    __shared__ double s_tot[kOcNodes];
    __shared__ bool s_last;
    if (sc->done) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nblk = gridDim.x;
    if (tid < kOcNodes) {  // node tid: follow its path from the root (bits of tid + 1 below the leading one)
        double lo = sc->l1, hi = sc->l2;
        const int path = tid + 1, depth = 31 - __clz(path);
        for (int i = depth - 1; i >= 0; --i) {
            const double m = 0.5 * (hi + lo);
            if ((path >> i) & 1)
                lo = m;
            else
                hi = m;
        }
        const double m = 0.5 * (hi + lo);
        s_mid[tid] = m;
        s_sq[tid] = (float)sqrt(1.0 / m);
        s_stop[tid] = (hi - lo) / (lo + hi + P.tol_eps) < P.tol;
    }
    __syncthreads();
    // trial density of node t: x sqrt(max(-dc / mid, floor)) clamped, written as
    // x max(sqrt(-dc) sqrt(1 / mid), sqrt(floor)) (sqrt is monotone: one square root per element)
    float sq[kOcNodes], v[kOcNodes];
#pragma unroll
    for (int t = 0; t < kOcNodes; ++t) {
        sq[t] = s_sq[t];
        v[t] = 0.0f;
    }
    const float sfloor = sqrtf(P.sqrt_floor);
    for (int64_t e = blockIdx.x * (int64_t)kOcThreads + tid; e < n; e += (int64_t)nblk * kOcThreads) {
        const float we = w[e];
        if (pres && pres[e]) {  // xnew = 1
#pragma unroll
            for (int t = 0; t < kOcNodes; ++t) v[t] += we;
            continue;
        }
        const float xe = x[e], s0 = sqrtf(fmaxf(-dc[e], 0.0f));
        const float lo = xe - P.move, hi = xe + P.move;
#pragma unroll
        for (int t = 0; t < kOcNodes; ++t) {
            float tv = xe * fmaxf(s0 * sq[t], sfloor);
            tv = fminf(fmaxf(tv, 0.0f), 1.0f);
            tv = fminf(fmaxf(tv, lo), hi);
            v[t] = fmaf(we, tv, v[t]);
        }
    }
    // block sums: warp wi sums nodes wi, wi + 8, ... over the block's threads in double-float
#pragma unroll
    for (int t = 0; t < kOcNodes; ++t) s_part[t][tid] = v[t];
    __syncthreads();
    for (int t = warp; t < kOcNodes; t += kOcThreads / 32) {
        df32 a{0.0f, 0.0f};
        for (int j = lane; j < kOcThreads; j += 32) a = df_add(a, df32{s_part[t][j], 0.0f});
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            a = df_add(a, df32{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
        if (lane == 0) partials[t * nblk + blockIdx.x] = make_float2(a.hi, a.lo);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&sc->counter, 1u) == (unsigned)nblk - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int t = warp; t < kOcNodes; t += kOcThreads / 32) {
        df32 a{0.0f, 0.0f};
        for (int b = lane; b < nblk; b += 32) {
            const float2 p = __ldcg(&partials[t * nblk + b]);
            a = df_add(a, df32{p.x, p.y});
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            a = df_add(a, df32{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
        if (lane == 0) s_tot[t] = df_value(a);
    }
    __syncthreads();
    if (tid == 0) {
        double l1 = sc->l1, l2 = sc->l2, lfinal = sc->lfinal;
        int steps = sc->steps, done = 0, node = 0;
        const double target = P.volfrac * (double)n - sc->npres;  // vol > volfrac <=> sum > target
        for (int lvl = 0; lvl < kOcLevels; ++lvl) {
            const double m = s_mid[node];
            if (s_stop[node]) {
                lfinal = m;
                steps += 1;
                done = 1;
                break;
            }
            if (s_tot[node] > target) {
                l1 = m;
                node = 2 * node + 2;
            } else {
                l2 = m;
                node = 2 * node + 1;
            }
            lfinal = m;
            steps += 1;
            if (steps >= P.max_bisect) {
                done = 1;
                break;
            }
        }
        sc->l1 = l1;
        sc->l2 = l2;
        sc->lfinal = lfinal;
        sc->steps = steps;
        sc->done = done;
        sc->counter = 0;
    }
}

__device__ __forceinline__ unsigned long long oc_now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- multisection in one cooperative launch ----------------------------------------------
// The rounds of oc_multi_kernel without a launch per round. In each round every block
// evaluates the kOcNodes trial volumes on its elements and publishes its block sums (slot
// round & 1: a block rewrites a slot only after every block has left the barrier that read it),
// arrives on a monotonic counter and waits, bounded in time, for all blocks; then every block
// sums all partials in block order and walks the tree itself, so that all blocks hold the same
// (l1, l2, lfinal, steps, done) and no broadcast is needed. After the last round each block
// writes xnew for its elements (oc_final_kernel's step). A wait that runs out sets
// sc->status = GBS_ETIMEOUT and ends the rounds; the host reports it.
__global__ void __launch_bounds__(kOcThreads) oc_coop_kernel(int64_t n, const OcParams P, const float *__restrict__ x,
                                                             const float *__restrict__ dc,
                                                             const uint8_t *__restrict__ pres,
                                                             const float *__restrict__ w, float2 *partials,
                                                             OcScalars *sc, float *xnew, unsigned long long wait_ns) {
    __shared__ float s_sq[kOcNodes];
    __shared__ bool s_stop[kOcNodes];
    __shared__ double s_mid[kOcNodes];
    __shared__ float s_part[kOcNodes][kOcThreads + 8];  // rows padded: conflict-free column sums
    __shared__ double s_tot[kOcNodes];
    __shared__ double s_l1, s_l2, s_lfinal;
    __shared__ int s_steps, s_done, s_ok;
    const int tid = threadIdx.x;
    const int nblk = gridDim.x, bid = blockIdx.x;
    if (tid == 0) {
        s_l1 = sc->l1;
        s_l2 = sc->l2;
        s_lfinal = sc->lfinal;
        s_steps = sc->steps;
        s_done = sc->done;
        s_ok = 1;
    }
    __syncthreads();
    const float sfloor = sqrtf(P.sqrt_floor);
    const double target = P.volfrac * (double)n - sc->npres;  // vol > volfrac <=> sum > target
    // Rounds have two shapes. While l1 is still 0 the bisection's midpoints are l2/2, l2/4, ...
    // for as long as every volume stays at or below the target (each step sets l2 = mid); a
    // chain round evaluates the next kOcNodes midpoints of that all-left path, formed exactly
    // as bisection forms them (0.5 (hi + 0)), and ends at the first step that goes right. Once
    // l1 > 0, tree rounds evaluate the full kOcLevels-level tree. Each round advances the
    // bisection by at least one step, so max_bisect rounds bound the loop.
    for (int round = 0; round < P.max_bisect; ++round) {
        if (s_done || !s_ok) break;  // block-uniform: written before the last __syncthreads
        const bool chain = s_l1 == 0.0;
        if (tid < kOcNodes) {
            double lo = s_l1, hi = s_l2;
            if (chain) {
                // tid halvings 0.5 (hi + 0) of the all-left path: exact, so the same bits as that
                // loop of dependent FP64 operations (l2 <= 1e9 stays far above the subnormals)
                hi = ldexp(hi, -tid);
            } else {
                const int path = tid + 1, depth = 31 - __clz(path);
                for (int i = depth - 1; i >= 0; --i) {
                    const double m = 0.5 * (hi + lo);
                    if ((path >> i) & 1)
                        lo = m;
                    else
                        hi = m;
                }
            }
            const double m = 0.5 * (hi + lo);
            s_mid[tid] = m;
            s_sq[tid] = (float)sqrt(1.0 / m);
            s_stop[tid] = (hi - lo) / (lo + hi + P.tol_eps) < P.tol;
        }
        __syncthreads();
        float sq[kOcNodes], v[kOcNodes];
#pragma unroll
        for (int t = 0; t < kOcNodes; ++t) {
            sq[t] = s_sq[t];
            v[t] = 0.0f;
        }
        for (int64_t e = bid * (int64_t)kOcThreads + tid; e < n; e += (int64_t)nblk * kOcThreads) {
            const float we = w[e];
            if (pres && pres[e]) {
#pragma unroll
                for (int t = 0; t < kOcNodes; ++t) v[t] += we;
                continue;
            }
            const float xe = x[e], s0 = sqrtf(fmaxf(-dc[e], 0.0f));
            const float lo = xe - P.move, hi = xe + P.move;
#pragma unroll
            for (int t = 0; t < kOcNodes; ++t) {
                float tv = xe * fmaxf(s0 * sq[t], sfloor);
                tv = fminf(fmaxf(tv, 0.0f), 1.0f);
                tv = fminf(fmaxf(tv, lo), hi);
                v[t] = fmaf(we, tv, v[t]);
            }
        }
#pragma unroll
        for (int t = 0; t < kOcNodes; ++t) s_part[t][tid] = v[t];
        __syncthreads();
        // block sums: node t = tid / 8 summed by the 8 lanes tid % 8 (columns sub, sub + 8, ...),
        // then across those lanes; every sum in a fixed order
        float2 *part = partials + (size_t)(round & 1) * kOcNodes * nblk;
        const int t8 = tid >> 3, sub = tid & 7;
        {
            df32 a{0.0f, 0.0f};
            if (t8 < kOcNodes)
#pragma unroll 8
                for (int j = sub; j < kOcThreads; j += 8) a = df_add(a, df32{s_part[t8][j], 0.0f});
#pragma unroll
            for (int o = 4; o > 0; o >>= 1)
                a = df_add(a, df32{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
            if (t8 < kOcNodes && sub == 0) part[t8 * nblk + bid] = make_float2(a.hi, a.lo);
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(&sc->bar, 1u);
            const unsigned goal = (unsigned)nblk * (unsigned)(round + 1);
            const unsigned long long t0 = oc_now_ns();
            while (*(volatile unsigned *)&sc->bar < goal) {
                if (oc_now_ns() - t0 > wait_ns) {
                    s_ok = 0;
                    atomicExch(&sc->status, (int)GBS_ETIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
        }
        __syncthreads();
        if (!s_ok) break;
        // totals, the same way over the blocks' partials (loads issued eight at a time, added in
        // block order)
        {
            df32 a{0.0f, 0.0f};
            if (t8 < kOcNodes) {
                const float2 *pt = part + t8 * nblk;
                int b = sub;
                for (; b + 56 < nblk; b += 64) {
                    float2 pv[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) pv[q] = __ldcg(&pt[b + 8 * q]);
#pragma unroll
                    for (int q = 0; q < 8; ++q) a = df_add(a, df32{pv[q].x, pv[q].y});
                }
                for (; b < nblk; b += 8) {
                    const float2 p = __ldcg(&pt[b]);
                    a = df_add(a, df32{p.x, p.y});
                }
            }
#pragma unroll
            for (int o = 4; o > 0; o >>= 1)
                a = df_add(a, df32{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
            if (t8 < kOcNodes && sub == 0) s_tot[t8] = df_value(a);
        }
        __syncthreads();
        if (tid == 0) {  // bisection's tests along the chain or the tree (oc_multi_kernel's walk)
            double l1 = s_l1, l2 = s_l2, lfinal = s_lfinal;
            int steps = s_steps, done = 0, node = 0;
            for (int lvl = 0; lvl < (chain ? kOcNodes : kOcLevels); ++lvl) {
                const double m = s_mid[node];
                if (s_stop[node]) {
                    lfinal = m;
                    steps += 1;
                    done = 1;
                    break;
                }
                const bool right = s_tot[node] > target;
                if (right) {
                    l1 = m;
                    node = 2 * node + 2;
                } else {
                    l2 = m;
                    node = chain ? node + 1 : 2 * node + 1;
                }
                lfinal = m;
                steps += 1;
                if (steps >= P.max_bisect) {
                    done = 1;
                    break;
                }
                if (chain && right) break;  // off the all-left path: tree rounds from here
            }
            s_l1 = l1;
            s_l2 = l2;
            s_lfinal = lfinal;
            s_steps = steps;
            s_done = done;
        }
        __syncthreads();
    }
    if (bid == 0 && tid == 0) {
        sc->l1 = s_l1;
        sc->l2 = s_l2;
        sc->lfinal = s_lfinal;
        sc->steps = s_steps;
        sc->done = s_done;
    }
    const float inv_l = (float)(1.0 / s_lfinal);
    for (int64_t e = bid * (int64_t)kOcThreads + tid; e < n; e += (int64_t)nblk * kOcThreads)
        xnew[e] = oc_trial(x[e], dc[e], inv_l, P, pres && pres[e]);
}

__global__ void oc_final_kernel(int64_t n, const OcParams P, const float *__restrict__ x,
                                const float *__restrict__ dc, const uint8_t *__restrict__ pres, const OcScalars *sc,
                                float *xnew) {
    const float inv_l = (float)(1.0 / sc->lfinal);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        xnew[e] = oc_trial(x[e], dc[e], inv_l, P, pres && pres[e]);
}

// ---- FP64 dot ---------------------------------------------------------------------------
__global__ void dot_f64_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                               double *partials, unsigned *counter, double *out) {
    __shared__ double sred[32];
    __shared__ double tot[1];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    const double v[1] = {s};
    if (last_block_reduce<1>(v, partials, counter, tot, sred) && threadIdx.x == 0) *out = tot[0];
}

}  // namespace gbs

using namespace gbs;

// ---- C ABI ------------------------------------------------------------------------------
static size_t reduce_ws_bytes(int64_t nblocks) { return 256 + ((size_t)nblocks * 8 * 4 + 255) / 256 * 256; }

// [counter][partials][the double-float split of u (modal Ke)]
extern "C" size_t gbsimp_sensitivity_ws_bytes(int nx, int ny, int nz) {
    if (!grid_ok(nx, ny, nz)) return reduce_ws_bytes(4096);
    const size_t nd = 3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    return reduce_ws_bytes(4096) + (nd * sizeof(float2) + 255) / 256 * 256;
}

extern "C" int gbsimp_sensitivity(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                                  const double *u, float *dc, float *ce, double *energy_out, void *ws,
                                  size_t ws_bytes, void *stream) {
    NvtxRange range("gbsimp_sensitivity");
    if (!ctx || !law || !x || !u || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_sensitivity: bad arguments");
    if (energy_out && (!ws || ws_bytes < reduce_ws_bytes(4096)))
        return set_error(GBS_EINVAL, "gbsimp_sensitivity: workspace too small");
    const int64_t n = (int64_t)nx * ny * nz;
    const unsigned blocks = reduce_blocks(ctx, n, 128);
    unsigned *counter = (unsigned *)ws;
    double *partials = (double *)((char *)ws + 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (energy_out) GBS_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    // The double-float element products need the split of u in the workspace; without room
    // for it (a workspace sized for the energy sum only, or none) the FP64 pass runs.
    if (ctx->modal_ok && ws && ws_bytes >= gbsimp_sensitivity_ws_bytes(nx, ny, nz)) {
        float2 *udd = (float2 *)((char *)ws + reduce_ws_bytes(4096));
        int rc = split_dd(ctx, 3 * (int64_t)(nx + 1) * (ny + 1) * (nz + 1), u, nullptr, udd, st);
        if (rc) return rc;
        sens_dd_kernel<<<blocks, 128, 0, st>>>(nx, ny, nz, make_law<double>(*law), modal_kdd(ctx->kmd),
                                               fast_div(ny), fast_div(nz), x, udd, dc,
                                               ce, partials, counter, energy_out);
        GBS_LAUNCH_CHECK("sens_dd_kernel");
        return GBS_OK;
    }
    sens_kernel<<<blocks, 128, 0, st>>>(nx, ny, nz, make_law<double>(*law), ctx->ked, ctx->translation_free ? 1 : 0,
                                        ctx->modal_ok ? 1 : 0, ctx->kmd, x, u, dc, ce, partials, counter, energy_out);
    GBS_LAUNCH_CHECK("sens_kernel");
    return GBS_OK;
}

extern "C" int gbsimp_filter_hs(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, float *hs, void *stream) {
    if (!ctx || !hs || !grid_ok(nx, ny, nz)) return set_error(GBS_EINVAL, "gbsimp_filter_hs: bad arguments");
    return filter_launch(ctx, nx, ny, nz, rmin, 2, nullptr, nullptr, nullptr, hs, (cudaStream_t)stream);
}

extern "C" int gbsimp_filter(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const float *hs, const float *in,
                             float *out, int transpose, void *stream) {
    NvtxRange range("gbsimp_filter");
    if (!ctx || !in || !out || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_filter: bad arguments");
    if (transpose && !hs) return set_error(GBS_EINVAL, "gbsimp_filter: the transpose needs hs");
    return filter_launch(ctx, nx, ny, nz, rmin, transpose ? 1 : 0, hs, in, nullptr, out, (cudaStream_t)stream);
}

extern "C" size_t gbsimp_oc_ws_bytes(int nx, int ny, int nz) { return oc_ws_bytes((int64_t)nx * ny * nz); }

namespace gbs {

size_t oc_ws_bytes_impl(int64_t n) { return oc_ws_bytes(n); }

const float *oc_ws_hs(const void *ws, int64_t n) { return oc_ws(const_cast<void *>(ws), n).hs; }

int oc_prepare_impl(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const uint8_t *preserved, void *ws,
                    cudaStream_t st) {
    const int64_t n = (int64_t)nx * ny * nz;
    OcWs w = oc_ws(ws, n);
    GBS_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(OcScalars), st));
    int rc = filter_launch(ctx, nx, ny, nz, rmin, 2, nullptr, nullptr, nullptr, w.hs, st);
    if (rc) return rc;
    Stencil s;
    rc = make_stencil(rmin, &s);
    if (rc) return rc;
    oc_weights_kernel<<<reduce_blocks(ctx, n, 256), 256, 0, st>>>(nx, ny, nz, s, w.hs, preserved, w.w, w.partials, w.sc);
    GBS_LAUNCH_CHECK("oc_weights_kernel");
    return GBS_OK;
}

// Blocks of oc_coop_kernel that can be resident together on the context's device (cached per
// device), capped by the partials room; 0 when cooperative launches are unavailable.
static int oc_coop_blocks(const gbsimp_ctx *ctx) {
    static std::atomic<int> cache[64];
    const int dev = ctx->device;
    if (dev < 0 || dev >= 64) return 0;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v != 0) return v > 0 ? v : 0;
    int coop = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, oc_coop_kernel, kOcThreads, 0) != cudaSuccess ||
        per_sm < 1) {
        (void)cudaGetLastError();
        cache[dev].store(-1, std::memory_order_relaxed);
        return 0;
    }
    constexpr int kRoom = (4 * 4096 * (int)sizeof(double)) / (2 * kOcNodes * (int)sizeof(float2));
    v = per_sm * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    v = v < kRoom ? v : kRoom;
    cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

int oc_run_impl(const gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const gbsimp_oc_params *prm, const float *x,
                const float *dc, const uint8_t *preserved, float *xnew, float *xphys, void *ws, cudaStream_t st) {
    NvtxRange range("OC update");
    const int64_t n = (int64_t)nx * ny * nz;
    OcWs w = oc_ws(ws, n);
    OcParams P;
    P.move = (float)prm->move;
    P.sqrt_floor = (float)prm->sqrt_floor;
    P.tol = prm->tol;
    P.tol_eps = prm->tol_eps;
    P.volfrac = prm->volfrac;
    P.l1 = prm->l1;
    P.l2 = prm->l2;
    P.max_bisect = prm->max_bisect;
    const unsigned blocks = reduce_blocks(ctx, n, 256);
    oc_init_kernel<<<blocks, 256, 0, st>>>(n, P, dc, w.partials, w.sc);
    GBS_LAUNCH_CHECK("oc_init_kernel");
    // One cooperative launch for the multisection and xnew when its blocks can be resident
    // together (two slots of kOcNodes double-float partials per block fit the workspace).
    const int cb = oc_coop_blocks(ctx);
    if (cb > 0) {
        int64_t nb = (n + kOcThreads - 1) / kOcThreads;
        nb = nb > cb ? cb : (nb < 1 ? 1 : nb);
        float2 *parts = (float2 *)w.partials;
        unsigned long long wait_ns = 2000000000ull;  // 2 s per barrier wait
        void *args[] = {(void *)&n, (void *)&P, (void *)&x, (void *)&dc, (void *)&preserved, (void *)&w.w,
                        (void *)&parts, (void *)&w.sc, (void *)&xnew, (void *)&wait_ns};
        GBS_CUDA_TRY(cudaLaunchCooperativeKernel((void *)oc_coop_kernel, dim3((unsigned)nb), dim3(kOcThreads), args, 0,
                                                 st));
        GBS_LAUNCH_CHECK("oc_coop_kernel");
        return filter_launch(ctx, nx, ny, nz, rmin, 0, w.hs, xnew, preserved, xphys, st);
    }
    // kOcNodes double-float partials per block fit the 4 * 4096 doubles of the workspace
    int64_t mb = (n + kOcThreads - 1) / kOcThreads;
    const int64_t mcap = 2LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    mb = mb > mcap ? mcap : (mb < 1 ? 1 : mb);
    if (mb * kOcNodes > 4 * 4096) mb = (4 * 4096) / kOcNodes;
    for (int k = 0; k < prm->max_bisect; k += kOcLevels) {
        oc_multi_kernel<<<(unsigned)mb, kOcThreads, 0, st>>>(n, P, x, dc, preserved, w.w, (float2 *)w.partials, w.sc);
        GBS_LAUNCH_CHECK("oc_multi_kernel");
    }
    oc_final_kernel<<<elem_blocks(ctx, n, 256), 256, 0, st>>>(n, P, x, dc, preserved, w.sc, xnew);
    GBS_LAUNCH_CHECK("oc_final_kernel");
    return filter_launch(ctx, nx, ny, nz, rmin, 0, w.hs, xnew, preserved, xphys, st);
}

int oc_check_args(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_oc_params *prm, const float *x,
                  const float *dc, const float *xnew, const float *xphys) {
    if (!ctx || !prm || !x || !dc || !xnew || !xphys || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_oc: bad arguments");
    if (prm->max_bisect <= 0 || prm->max_bisect > 1000)
        return set_error(GBS_EINVAL, "gbsimp_oc: max_bisect out of range");
    if (x == xnew) return set_error(GBS_EINVAL, "gbsimp_oc: x and xnew must not alias");
    return GBS_OK;
}

}  // namespace gbs

extern "C" int gbsimp_oc_prepare(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const uint8_t *preserved,
                                 void *ws, size_t ws_bytes, void *stream) {
    if (!ctx || !grid_ok(nx, ny, nz) || !ws) return set_error(GBS_EINVAL, "gbsimp_oc_prepare: bad arguments");
    if (ws_bytes < oc_ws_bytes((int64_t)nx * ny * nz)) return set_error(GBS_EINVAL, "gbsimp_oc_prepare: workspace too small");
    return oc_prepare_impl(ctx, nx, ny, nz, rmin, preserved, ws, (cudaStream_t)stream);
}

extern "C" int gbsimp_oc(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const gbsimp_oc_params *prm,
                         const float *x, const float *dc, const uint8_t *preserved, float *xnew, float *xphys,
                         void *ws, size_t ws_bytes, void *stream) {
    int rc = oc_check_args(ctx, nx, ny, nz, prm, x, dc, xnew, xphys);
    if (rc) return rc;
    if (!ws || ws_bytes < oc_ws_bytes((int64_t)nx * ny * nz)) return set_error(GBS_EINVAL, "gbsimp_oc: workspace too small");
    return oc_run_impl(ctx, nx, ny, nz, rmin, prm, x, dc, preserved, xnew, xphys, ws, (cudaStream_t)stream);
}

extern "C" int gbsimp_oc_result(gbsimp_ctx *ctx, const void *ws, double *lambda_out, int *steps_out, void *stream) {
    if (!ctx || !ws) return set_error(GBS_EINVAL, "gbsimp_oc_result: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    OcScalars h;
    void *hp = thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "gbsimp_oc_result: no pinned staging buffer");
    GBS_CUDA_TRY(cudaMemcpyAsync(hp, ws, sizeof(OcScalars), cudaMemcpyDeviceToHost, st));
    GBS_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(&h, hp, sizeof h);
    if (lambda_out) *lambda_out = h.lfinal;
    if (steps_out) *steps_out = h.steps;
    if (h.status == GBS_ETIMEOUT)
        return set_error(GBS_ETIMEOUT, "gbsimp_oc_result: a grid barrier wait of the OC update ran out");
    return GBS_OK;
}

extern "C" int gbsimp_dot_f64(gbsimp_ctx *ctx, int64_t n, const double *a, const double *b, double *out, void *ws,
                              size_t ws_bytes, void *stream) {
    if (!ctx || !a || !b || !out || !ws || n < 0) return set_error(GBS_EINVAL, "gbsimp_dot_f64: bad arguments");
    if (ws_bytes < reduce_ws_bytes(4096)) return set_error(GBS_EINVAL, "gbsimp_dot_f64: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned *counter = (unsigned *)ws;
    double *partials = (double *)((char *)ws + 256);
    GBS_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    dot_f64_kernel<<<reduce_blocks(ctx, n, 256), 256, 0, st>>>(n, a, b, partials, counter, out);
    GBS_LAUNCH_CHECK("dot_f64_kernel");
    return GBS_OK;
}
