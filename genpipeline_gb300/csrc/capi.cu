// capi.cu -- context, error state and element stiffness of the gbsimp C ABI.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>

#include "internal.h"

namespace gbs {

static thread_local char g_err[512] = "";
static std::atomic<unsigned long long> g_launches{0};

static thread_local bool g_capturing = false;

// Launches enqueued while a graph is being captured are not executions; graph replays add
// their kernel count explicitly.
void count_launches(int n) {
    if (!g_capturing && n > 0) g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed);
}
void set_capturing(bool on) { g_capturing = on; }

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

int cuda_error(cudaError_t e, const char *what) {
    return set_error(GBS_ECUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

static const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// B^T D B summed over the 2x2x2 Gauss points of the unit cube. The integrand is
// polynomial of degree <= 2 per axis, so the two-point rule is exact.
static void ke_quadrature(double nu, double e0, double *ke) {
    const double lam = e0 * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double mu = e0 / (2.0 * (1.0 + nu));
    const double g[2] = {0.5 - 0.5 / sqrt(3.0), 0.5 + 0.5 / sqrt(3.0)};
    memset(ke, 0, 576 * sizeof(double));
    for (int q = 0; q < 8; ++q) {
        const double gx = g[q & 1], gy = g[(q >> 1) & 1], gz = g[(q >> 2) & 1];
        // grad N_a at the point, and the six strains (xx, yy, zz, xy, yz, zx) per DOF.
        double B[6][24];
        memset(B, 0, sizeof B);
        for (int a = 0; a < 8; ++a) {
            const double sx = kCorner[a][0] ? 1.0 : -1.0, sy = kCorner[a][1] ? 1.0 : -1.0,
                         sz = kCorner[a][2] ? 1.0 : -1.0;
            const double fx = kCorner[a][0] ? gx : 1.0 - gx, fy = kCorner[a][1] ? gy : 1.0 - gy,
                         fz = kCorner[a][2] ? gz : 1.0 - gz;
            const double dNx = sx * fy * fz, dNy = fx * sy * fz, dNz = fx * fy * sz;
            B[0][3 * a + 0] = dNx;
            B[1][3 * a + 1] = dNy;
            B[2][3 * a + 2] = dNz;
            B[3][3 * a + 0] = dNy;
            B[3][3 * a + 1] = dNx;
            B[4][3 * a + 1] = dNz;
            B[4][3 * a + 2] = dNy;
            B[5][3 * a + 0] = dNz;
            B[5][3 * a + 2] = dNx;
        }
        // D B with the isotropic D (lam + 2 mu on the normal diagonal, mu for shears).
        double DB[6][24];
        for (int c = 0; c < 24; ++c) {
            const double tr = B[0][c] + B[1][c] + B[2][c];
            for (int m = 0; m < 3; ++m) DB[m][c] = lam * tr + 2.0 * mu * B[m][c];
            for (int m = 3; m < 6; ++m) DB[m][c] = mu * B[m][c];
        }
        for (int r = 0; r < 24; ++r)
            for (int c = 0; c < 24; ++c) {
                double s = 0.0;
                for (int m = 0; m < 6; ++m) s += B[m][r] * DB[m][c];
                ke[r * 24 + c] += s * 0.125;
            }
    }
    for (int r = 0; r < 24; ++r)
        for (int c = r + 1; c < 24; ++c) {
            const double s = 0.5 * (ke[r * 24 + c] + ke[c * 24 + r]);
            ke[r * 24 + c] = ke[c * 24 + r] = s;
        }
}

namespace {
// Owner of one thread's pinned buffer: freed when the thread exits (every use copies into it
// and synchronises the stream before returning, so no copy is in flight by then).
struct ThreadPinned {
    void *p = nullptr;
    ~ThreadPinned() {
        if (p) cudaFreeHost(p);
    }
};
}  // namespace

void *thread_pinned() {
    // One small pinned buffer per host thread, so that threads sharing a context never
    // share a staging buffer.
    static thread_local ThreadPinned buf;
    if (!buf.p && cudaMallocHost(&buf.p, 4096) != cudaSuccess) buf.p = nullptr;
    return buf.p;
}

static void install_ke(gbsimp_ctx *ctx, const double *ke) {
    ctx->ke_version += 1;
    double mx = 0.0, tr = 0.0;
    for (int i = 0; i < 576; ++i) {
        ctx->ke[i] = ke[i];
        ctx->kef.k[i] = (float)ke[i];
        ctx->ked.k[i] = ke[i];
        mx = fmax(mx, fabs(ke[i]));
    }
    // Rigid translations in the kernel of Ke: sum over the 8 nodes of column block c.
    for (int r = 0; r < 24; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int b = 0; b < 8; ++b) s += ke[r * 24 + 3 * b + c];
            tr = fmax(tr, fabs(s));
        }
    ctx->translation_free = mx > 0.0 && tr <= 1e-12 * mx;
    // Modal form Km = T^T Ke T / 64 (T = T8 (x) I3, T8[a][m] = prod_d (m_d ? s(c_d(a)) : 1),
    // modes bit-ordered (x, y, z) = (4, 2, 1)); usable when Ke has no entry outside the
    // 45-entry pattern of an isotropic cube element.
    {
        double T8[8][8];
        for (int a = 0; a < 8; ++a)
            for (int m = 0; m < 8; ++m) {
                double v = 1.0;
                const int c[3] = {kCorner[a][0], kCorner[a][1], kCorner[a][2]};
                const int mb[3] = {(m >> 2) & 1, (m >> 1) & 1, m & 1};
                for (int d = 0; d < 3; ++d)
                    if (mb[d]) v *= c[d] ? 1.0 : -1.0;
                T8[a][m] = v;
            }
        double km[24][24];
        double kmax = 0.0;
        for (int r = 0; r < 24; ++r)
            for (int cc = 0; cc < 24; ++cc) {
                double s = 0.0;
                for (int a = 0; a < 8; ++a)
                    for (int b = 0; b < 8; ++b)
                        s += T8[a][r / 3] * ke[(3 * a + r % 3) * 24 + 3 * b + cc % 3] * T8[b][cc / 3];
                km[r][cc] = s / 64.0;
                kmax = fmax(kmax, fabs(km[r][cc]));
            }
        bool in_pattern[24][24] = {};
        int cls_first[kModalClasses];
        for (int k = kModalClasses - 1; k >= 0; --k)
            for (int i = kModalNnz - 1; i >= 0; --i)
                if (modal_class(i) == k) cls_first[k] = i;
        bool classes_ok = true;
        for (int i = 0; i < kModalNnz; ++i) {
            in_pattern[modal_row(i)][modal_col(i)] = true;
            const double kc = km[modal_row(cls_first[modal_class(i)])][modal_col(cls_first[modal_class(i)])];
            if (fabs(km[modal_row(i)][modal_col(i)] - kc) > 1e-9 * kmax) classes_ok = false;
            const float kf = (float)kc;
            ctx->km.c[modal_class(i)] = make_float2(kf, kf);
            ctx->kmd.v[i] = km[modal_row(i)][modal_col(i)];
        }
        bool ok = kmax > 0.0;
        for (int r = 0; r < 24 && ok; ++r)
            for (int cc = 0; cc < 24; ++cc)
                if (!in_pattern[r][cc] && fabs(km[r][cc]) > 1e-12 * kmax) {
                    ok = false;
                    break;
                }
        ctx->modal_ok = ok && classes_ok;
    }
    for (int i = 0; i < 24; ++i) {
        ctx->ke_diag_d[i] = ke[i * 25];
        ctx->ke_diag_f[i] = (float)ke[i * 25];
    }
}

}  // namespace gbs

using namespace gbs;

extern "C" int gbsimp_abi_version(void) { return GBSIMP_ABI_VERSION; }

extern "C" const char *gbsimp_last_error(void) { return g_err; }

extern "C" uint64_t gbsimp_launch_count(void) { return (uint64_t)g_launches.load(); }

extern "C" int gbsimp_ke_quadrature(double nu, double e0, double *ke576) {
    if (!ke576 || !(nu > -1.0 && nu < 0.5) || !(e0 > 0.0))
        return set_error(GBS_EINVAL, "gbsimp_ke_quadrature: need -1 < nu < 0.5, e0 > 0");
    ke_quadrature(nu, e0, ke576);
    return GBS_OK;
}

extern "C" int gbsimp_create(gbsimp_ctx **out) {
    if (!out) return set_error(GBS_EINVAL, "gbsimp_create: null out");
    *out = nullptr;
    gbsimp_ctx *c = (gbsimp_ctx *)calloc(1, sizeof(gbsimp_ctx));
    if (!c) return set_error(GBS_ENOMEM, "gbsimp_create: out of host memory");
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) {
        free(c);
        return cuda_error(e, "cudaGetDevice");
    }
    e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&c->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device);
    if (e != cudaSuccess) {
        free(c);
        return cuda_error(e, "cudaDeviceGetAttribute");
    }
    double ke[576];
    ke_quadrature(0.3, 1.0, ke);
    install_ke(c, ke);
    c->graphs = graph_cache_create();
    *out = c;
    return GBS_OK;
}

extern "C" int gbsimp_destroy(gbsimp_ctx *ctx) {
    if (!ctx) return GBS_OK;
    graph_cache_destroy(ctx->graphs);
    free(ctx);
    return GBS_OK;
}

extern "C" int gbsimp_set_ke(gbsimp_ctx *ctx, const double *ke576) {
    if (!ctx || !ke576) return set_error(GBS_EINVAL, "gbsimp_set_ke: bad arguments");
    for (int i = 0; i < 576; ++i)
        if (!isfinite(ke576[i])) return set_error(GBS_EINVAL, "gbsimp_set_ke: non-finite entry %d", i);
    install_ke(ctx, ke576);
    return GBS_OK;
}

extern "C" int gbsimp_get_ke(const gbsimp_ctx *ctx, double *ke576) {
    if (!ctx || !ke576) return set_error(GBS_EINVAL, "gbsimp_get_ke: bad arguments");
    memcpy(ke576, ctx->ke, sizeof ctx->ke);
    return GBS_OK;
}
