// runner.cu -- host-side drivers over the device calls: the SIMP loop in one call
// (gbsimp_simp_run) and the solve queue behind submit / poll (gbsimp_queue_*). Both only
// order existing stream work; neither launches kernels of its own.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <new>
#include <vector>

#include "internal.h"

using namespace gbs;

// ---- SIMP loop ------------------------------------------------------------------------
namespace {

constexpr size_t kAlign = 256;
size_t al(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }

// Workspace: [solve ws][OC ws (holds Hs)][sensitivity ws][dc][dcf][xnew][objective (double)]
// [the previous solution (FP64), for the extrapolated warm start]
struct SimpWs {
    void *solve, *oc, *sens;
    size_t solve_bytes, oc_bytes, sens_bytes;
    float *dc, *dcf, *xnew;
    double *obj, *u_prev;
};

// Warm start of solve k >= 3: u_{k-1} + theta (u_{k-1} - u_{k-2}) (gbsimp_warm_start).
constexpr double kWarmTheta = 0.5;

size_t simp_ws_bytes(int nx, int ny, int nz) {
    const size_t ne = (size_t)nx * ny * nz;
    return kAlign + al(gbsimp_solve_ws_bytes(nx, ny, nz)) + al(oc_ws_bytes_impl((int64_t)ne)) +
           al(gbsimp_sensitivity_ws_bytes(nx, ny, nz)) + 3 * al(ne * sizeof(float)) + al(sizeof(double)) +
           al(3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1) * sizeof(double));
}

SimpWs simp_ws(void *ws, int nx, int ny, int nz) {
    const size_t ne = (size_t)nx * ny * nz;
    char *p = (char *)(((uintptr_t)ws + kAlign - 1) & ~(uintptr_t)(kAlign - 1));
    SimpWs w;
    w.solve_bytes = gbsimp_solve_ws_bytes(nx, ny, nz);
    w.oc_bytes = oc_ws_bytes_impl((int64_t)ne);
    w.sens_bytes = gbsimp_sensitivity_ws_bytes(nx, ny, nz);
    w.solve = p;
    p += al(w.solve_bytes);
    w.oc = p;
    p += al(w.oc_bytes);
    w.sens = p;
    p += al(w.sens_bytes);
    w.dc = (float *)p;
    p += al(ne * sizeof(float));
    w.dcf = (float *)p;
    p += al(ne * sizeof(float));
    w.xnew = (float *)p;
    p += al(ne * sizeof(float));
    w.obj = (double *)p;
    p += al(sizeof(double));
    w.u_prev = (double *)p;
    return w;
}

}  // namespace

extern "C" size_t gbsimp_simp_run_ws_bytes(int nx, int ny, int nz) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
    return simp_ws_bytes(nx, ny, nz);
}

// SIMPSolver.run (simp_solver.py:56-79): solve, sensitivity, filter of dc, OC; the objective
// of iteration i is sum_e E_e ce_e at the xPhys that iteration's solve used (simp_solver.py:
// 216-218). The early-stop rule is SIMPSolverGPU.run's (simp_solver_gpu.py:111-125).
extern "C" int gbsimp_simp_run(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                               const gbsimp_simp_opts *opts, const double *f, const uint8_t *node_mask,
                               const uint8_t *preserved, float *x, float *xphys, double *u, double *compliance,
                               int32_t *iters_out, gbsimp_solve_stats *last_stats, void *ws, size_t ws_bytes,
                               void *stream) {
    NvtxRange range("gbsimp_simp_run");
    if (!ctx || !law || !opts || !f || !x || !xphys || !u || !ws || nx <= 0 || ny <= 0 || nz <= 0)
        return set_error(GBS_EINVAL, "gbsimp_simp_run: bad arguments");
    if (opts->n_iters < 0 || !(opts->rmin > 0.0) || !(opts->volfrac > 0.0 && opts->volfrac <= 1.0))
        return set_error(GBS_EINVAL, "gbsimp_simp_run: bad options");
    if (ws_bytes < simp_ws_bytes(nx, ny, nz)) return set_error(GBS_EINVAL, "gbsimp_simp_run: workspace too small");
    if (x == xphys) return set_error(GBS_EINVAL, "gbsimp_simp_run: x and xphys must not alias");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t ne = (int64_t)nx * ny * nz;
    const SimpWs w = simp_ws(ws, nx, ny, nz);
    gbsimp_oc_params prm = opts->oc;
    prm.volfrac = opts->volfrac;
    int rc = oc_check_args(ctx, nx, ny, nz, &prm, x, w.dc, w.xnew, xphys);
    if (rc) return rc;
    rc = oc_prepare_impl(ctx, nx, ny, nz, opts->rmin, preserved, w.oc, st);  // Hs and the volume weights
    if (rc) return rc;
    const float *hs = oc_ws_hs(w.oc, ne);  // Hs for the chain rule of the filter
    GBS_CUDA_TRY(cudaMemcpyAsync(xphys, x, (size_t)ne * sizeof(float), cudaMemcpyDeviceToDevice, st));
    if (iters_out) *iters_out = 0;
    float *xc = x, *xn = w.xnew;  // the design ping-pongs between the caller's x and xnew
    const bool need_obj = compliance != nullptr || opts->early_stop;
    double prev = 0.0;
    int below = 0, it = 0;
    gbsimp_solve_stats sstats = {};
    const int64_t nd = 3LL * (nx + 1) * (ny + 1) * (nz + 1);
    for (; it < opts->n_iters; ++it) {
        NvtxRange iteration("SIMP iteration");
        // u holds the last solution from the second iteration on, u_prev the one before from the
        // third on (the caller's initial u is not a solution of this loop)
        if (it >= 2) {
            rc = warm_start_impl(ctx, nd, u, w.u_prev, kWarmTheta, st);
        } else if (it == 1) {
            const cudaError_t e = cudaMemcpyAsync(w.u_prev, u, (size_t)nd * sizeof(double), cudaMemcpyDeviceToDevice, st);
            rc = e == cudaSuccess ? GBS_OK : cuda_error(e, "cudaMemcpyAsync(u_prev)");
        }
        if (rc) break;
        rc = gbsimp_solve(ctx, nx, ny, nz, law, xphys, f, node_mask, u, &opts->solve, &sstats, w.solve,
                          w.solve_bytes, stream);
        if (rc) break;
        if (sstats.status != GBS_OK && sstats.status != GBS_ENOTCONV) {
            rc = sstats.status;
            break;
        }
        rc = gbsimp_sensitivity(ctx, nx, ny, nz, law, xphys, u, w.dc, nullptr, need_obj ? w.obj : nullptr, w.sens,
                                w.sens_bytes, stream);
        if (rc) break;
        rc = gbsimp_filter(ctx, nx, ny, nz, opts->rmin, hs, w.dc, w.dcf, 1, stream);
        if (rc) break;
        rc = oc_run_impl(ctx, nx, ny, nz, opts->rmin, &prm, xc, w.dcf, preserved, xn, xphys, w.oc, st);
        if (rc) break;
        std::swap(xc, xn);
        if (need_obj) {
            double c = 0.0;
            void *hp = thread_pinned();
            if (!hp) {
                rc = set_error(GBS_ECUDA, "gbsimp_simp_run: no pinned staging buffer");
                break;
            }
            GBS_CUDA_TRY(cudaMemcpyAsync(hp, w.obj, sizeof(double), cudaMemcpyDeviceToHost, st));
            GBS_CUDA_TRY(cudaStreamSynchronize(st));
            c = *(const double *)hp;
            if (compliance) compliance[it] = c;
            if (opts->early_stop) {
                if (it > 0) below = std::abs(prev - c) / (prev + 1e-10) < 0.01 ? below + 1 : 0;
                prev = c;
                if (below >= 3) {
                    ++it;
                    break;
                }
            }
        }
    }
    if (iters_out) *iters_out = it;
    if (last_stats) *last_stats = sstats;
    if (xc != x) GBS_CUDA_TRY(cudaMemcpyAsync(x, xc, (size_t)ne * sizeof(float), cudaMemcpyDeviceToDevice, st));
    return rc;
}

// ---- solve queue ----------------------------------------------------------------------
struct gbsimp_queue {
    gbsimp_ctx *ctx;
    gbsimp_law law;
    gbsimp_solve_opts opts;
    std::mutex mu;
    std::vector<gbsimp_batch_item *> active;    // in the rounds
    std::vector<gbsimp_batch_item *> finished;  // done, not yet handed back
};

extern "C" int gbsimp_queue_create(gbsimp_ctx *ctx, const gbsimp_law *law, const gbsimp_solve_opts *opts,
                                   gbsimp_queue **out) {
    if (!ctx || !law || !opts || !out) return set_error(GBS_EINVAL, "gbsimp_queue_create: bad arguments");
    gbsimp_queue *q = new (std::nothrow) gbsimp_queue();
    if (!q) return set_error(GBS_ENOMEM, "gbsimp_queue_create: out of host memory");
    q->ctx = ctx;
    q->law = *law;
    q->opts = *opts;
    *out = q;
    return GBS_OK;
}

extern "C" int gbsimp_queue_destroy(gbsimp_queue *q) {
    delete q;
    return GBS_OK;
}

extern "C" int gbsimp_queue_submit(gbsimp_queue *q, gbsimp_batch_item *item) {
    if (!q || !item || !item->x || !item->f || !item->u || !item->ws || item->nx <= 0 || item->ny <= 0 ||
        item->nz <= 0)
        return set_error(GBS_EINVAL, "gbsimp_queue_submit: bad arguments");
    if (item->ws_bytes < gbsimp_solve_ws_bytes(item->nx, item->ny, item->nz))
        return set_error(GBS_EINVAL, "gbsimp_queue_submit: workspace too small");
    std::lock_guard<std::mutex> lock(q->mu);
    for (const gbsimp_batch_item *a : q->active)
        if (a == item) return set_error(GBS_EINVAL, "gbsimp_queue_submit: item already queued");
    item->state = 0;
    item->stats = gbsimp_solve_stats{};
    q->active.push_back(item);
    return GBS_OK;
}

extern "C" int gbsimp_queue_poll(gbsimp_queue *q, gbsimp_batch_item **done, int max_done, int *n_done,
                                 void *stream) {
    if (!q || !n_done || max_done < 0 || (max_done > 0 && !done))
        return set_error(GBS_EINVAL, "gbsimp_queue_poll: bad arguments");
    std::lock_guard<std::mutex> lock(q->mu);
    *n_done = 0;
    if (!q->active.empty()) {
        // gbsimp_batch_round takes an array of items: round on copies, then copy the results back
        std::vector<gbsimp_batch_item> items;
        items.reserve(q->active.size());
        for (const gbsimp_batch_item *a : q->active) items.push_back(*a);
        const int rc = gbsimp_batch_round(q->ctx, items.data(), (int)items.size(), &q->law, &q->opts, stream);
        if (rc) return rc;
        std::vector<gbsimp_batch_item *> still;
        for (size_t k = 0; k < items.size(); ++k) {
            *q->active[k] = items[k];
            (items[k].state != 0 ? q->finished : still).push_back(q->active[k]);
        }
        q->active.swap(still);
    }
    const int m = std::min(max_done, (int)q->finished.size());
    for (int k = 0; k < m; ++k) done[k] = q->finished[k];
    q->finished.erase(q->finished.begin(), q->finished.begin() + m);
    *n_done = m;
    return GBS_OK;
}

extern "C" int gbsimp_queue_size(const gbsimp_queue *q) {
    if (!q) return -1;
    std::lock_guard<std::mutex> lock(const_cast<gbsimp_queue *>(q)->mu);
    return (int)(q->active.size() + q->finished.size());
}
