/*
 * gbsimp.h -- C ABI of the GB300 (sm_103a) SIMP / voxel-FEM hot path.
 *
 * One shared library (genpipeline_gb300/libgbsimp.so). Plain C types only: every array
 * argument is a raw device pointer owned by the caller, every size is an explicit
 * integer, every call is ordered on the caller's CUDA stream (passed as void*) and none
 * of them synchronises the device unless its comment says it returns host-visible
 * results. Scratch memory is caller-owned too: each call that needs scratch takes
 * (ws, ws_bytes) and a *_ws_bytes() query says how much.
 *
 * Layout (identical to the reference genpipeline/topology/simp_solver.py:251-282):
 *   element e = i*ny*nz + j*nz + k   (0 <= i < nx, ...)
 *   node    n = i*(ny+1)*(nz+1) + j*(nz+1) + k
 *   DOF       = 3n + c  (c = x, y, z)
 *   element-local node a in the order (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),
 *   (1,1,1),(0,1,1); element-local DOF 3a + c; Ke is row-major 24x24.
 * Dirichlet masks are one byte per node: bit c set = DOF 3n+c is fixed (held at 0).
 * Grids: positive extents with fewer than 2^31 DOFs (3 (nx+1)(ny+1)(nz+1) < 2^31); the grid
 * entry points return GBS_EINVAL for anything else.
 *
 * Return values: GBS_OK or one of the GBS_E* codes; gbsimp_last_error() gives the
 * message of the last failure on the calling thread.
 */
#ifndef GBSIMP_H
#define GBSIMP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: gbsimp_solve_opts gained batch_share and batch_group; gbsimp_solve_stats names its two
 * library-owned fields (batched rounds with an iteration budget). The last field of
 * gbsimp_solve_opts, reserved (zero) before, selects the FP64 outer residual; zero keeps the
 * default. */
#define GBSIMP_ABI_VERSION 2

enum {
    GBS_OK = 0,
    GBS_EINVAL = 1,      /* bad argument (sizes, null pointers, too-small workspace) */
    GBS_ENOMEM = 2,      /* host allocation failed */
    GBS_ENOTCONV = 3,    /* iteration cap reached; the best iterate is still written */
    GBS_EBREAKDOWN = 4,  /* p^T K p <= 0 in CG (operator not SPD on the free DOFs) */
    GBS_ETIMEOUT = 5,    /* a bounded device-side wait expired */
    GBS_ECUDA = 6,       /* a CUDA runtime call failed */
    GBS_ENONFINITE = 7   /* NaN/Inf met in a residual or a reduction */
};

/* Stiffness law of one element: kind 0 ("ref", simp_solver.py:182-185)
 *   E = e0 * max(x, xmin)^penal,            dE/dx = e0 * penal * max(x, xmin)^(penal-1)
 * kind 1 ("modified", the SIMP law of simp_sensitivity_ptx.cu:20-26)
 *   E = emin + x^penal * (e0 - emin),       dE/dx = penal * x^(penal-1) * (e0 - emin)   */
typedef struct gbsimp_law {
    int32_t kind;
    int32_t reserved;
    double penal, e0, emin, xmin;
} gbsimp_law;

/* OC bisection parameters (simp_solver.py:225-249 = CPU variant:
 *   move 0.2, l1 0, l2 1e9, max_bisect 50, tol 1e-4, tol_eps 1e-12, sqrt_floor 1e-12;
 * simp_solver_gpu.py:801-841 = GPU variant: l2 < 0 requests l2 = 2*max(max(-dc), 1),
 *   max_bisect 30, tol 1e-5, tol_eps 1e-15, sqrt_floor 1e-15). */
typedef struct gbsimp_oc_params {
    double move, l1, l2, tol, tol_eps, sqrt_floor, volfrac;
    int32_t max_bisect;
    int32_t reserved;
} gbsimp_oc_params;

/* Options and results of the linear solves. */
typedef struct gbsimp_solve_opts {
    double rtol;          /* stop when ||D(f - K u)|| <= rtol * ||D f|| (outer residual, see gbsimp_solve) */
    double inner_rtol;    /* FP32 PCG reduction per outer correction (gbsimp_solve, batch); <= 0: 3e-5 */
    int32_t max_iter;     /* cap on the total FP32 PCG iterations */
    int32_t max_outer;    /* cap on outer defect corrections (gbsimp_solve, batched rounds) */
    int32_t check_every;  /* iterations between the host's checks where the host drives the
                             loop (profile, the CSR PCG); 0 = auto. Batched rounds: the inner
                             PCG iterations one round may run per item (rounded up to whole
                             graph-loop trips of 12 there), after which the round returns and the
                             paused solves resume in the next one; 0 = every inner PCG runs to
                             its tolerance within the round */
    int32_t fused;        /* 1 = persistent fused PCG kernel, 0 = graph loop, one launch per iteration */
    int32_t profile;      /* 1 = time every PCG apply launch with CUDA events (stats) */
    int32_t batch_share;  /* batched persistent launches: how the SMs are shared among the designs
                             of one launch. 0 = in proportion to element counts; 1 = in proportion
                             to element counts x longest grid extent (Jacobi-PCG iteration counts
                             grow about with it, so the designs of a launch finish together) */
    int32_t batch_group;  /* batched persistent launches: at most this many designs per launch
                             (0 or more than 24: 24) */
    int32_t residual_fp64; /* 1 = the outer residual's element products in FP64 at every rtol;
                              0 = in double-float for rtol >= 1e-9 (see gbsimp_solve) */
} gbsimp_solve_opts;

typedef struct gbsimp_solve_stats {
    int32_t status;       /* GBS_OK, GBS_ENOTCONV, GBS_EBREAKDOWN, GBS_ENONFINITE, GBS_ETIMEOUT */
    int32_t iterations;   /* FP32 PCG iterations (all outer corrections together) */
    int32_t outer;        /* outer residual evaluations */
    int32_t inner_active; /* batched rounds (library-owned, start at 0): 1 or 2 while an inner
                             PCG is paused by the round budget (persistent kernel / graph loop) */
    double relres;        /* last ||D(f - K u)|| / ||D f|| */
    double seconds;       /* host wall time of the call */
    double apply_seconds; /* device time of the PCG apply launches (opts->profile only) */
    int32_t apply_launches;
    int32_t inner_iters;  /* batched rounds (library-owned): iterations of the paused inner PCG
                             already counted in `iterations` */
} gbsimp_solve_stats;

typedef struct gbsimp_ctx gbsimp_ctx;

/* ---- context ---------------------------------------------------------------------- */
int gbsimp_abi_version(void);
/* Number of CUDA kernels this library has launched in the process (all threads). */
uint64_t gbsimp_launch_count(void);
const char *gbsimp_last_error(void);
/* Creates a context bound to the current CUDA device, holding the quadrature element
 * stiffness of (nu = 0.3, E = 1). No device memory is allocated. A context (and the CUDA
 * graphs it caches) belongs to the device's primary context: destroy it before any
 * cudaDeviceReset and create a new one afterwards. */
int gbsimp_create(gbsimp_ctx **out);
int gbsimp_destroy(gbsimp_ctx *ctx);
/* Unit-cube trilinear hexahedron by 2x2x2 Gauss quadrature of B^T D B (host, FP64). The
 * reference's own table (simp_solver.py:284-1543, reused by simp_solver_gpu.py:932-936)
 * is not symmetric positive semi-definite; this is the SPD matrix of the same element. */
int gbsimp_ke_quadrature(double nu, double e0, double *ke576);
/* Replaces the context's element stiffness (host pointer, 576 doubles, row-major). */
int gbsimp_set_ke(gbsimp_ctx *ctx, const double *ke576);
int gbsimp_get_ke(const gbsimp_ctx *ctx, double *ke576);

/* ---- element stiffness apply ------------------------------------------------------- */
/* y = D K(x) D p with K(x) = sum_e E(x_e) P_e^T Ke P_e; D zeroes the DOFs flagged in
 * node_mask (nullable: no masking). Replaces the COO assembly + SpMV of
 * simp_solver.py:200-205 / simp_solver_gpu.py:313-326 and fused_spmv_kernel
 * (cuda_kernels/simp_sensitivity_ptx.cu:301-373). Owner-computes, no atomics. */
int gbsimp_apply_f32(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                     const float *x, const float *p, float *y, const uint8_t *node_mask,
                     void *stream);
/* Which FP32 kernel serves gbsimp_apply_f32 / the PCG for this context and z extent:
 * 1 = modal (Hadamard) element kernel, used when Ke has the structure of an isotropic cube
 * element and nz <= 446; 0 = dense 24x24 node-gather kernel (any Ke); -1 = bad context. */
int gbsimp_apply_path(const gbsimp_ctx *ctx, int nz);
int gbsimp_apply_f64(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                     const float *x, const double *p, double *y, const uint8_t *node_mask,
                     void *stream);
/* Same operator over an arbitrary element->DOF table edof[n_elem][24] (int32 or int64 per
 * edof_is_int64), the contract of cuda_kernels.fused_spmv (cuda_kernels/__init__.py:329-368).
 * y (n_dof floats) is overwritten; contributions are summed with atomics. */
int gbsimp_apply_edof_f32(gbsimp_ctx *ctx, int64_t n_elem, int64_t n_dof, const void *edof,
                          int edof_is_int64, const gbsimp_law *law, const float *x,
                          const float *p, float *y, void *stream);

/* ---- element energy / sensitivity -------------------------------------------------- */
/* ce_e = u_e^T Ke u_e, dc_e = -dE/dx(x_e) * ce_e (simp_solver.py:215-218,
 * simp_sensitivity_kernel in cuda_kernels/simp_sensitivity_ptx.cu:163-270), from the FP64
 * displacement. dc and ce are nullable FP32 outputs; energy_out (nullable, device double)
 * receives sum_e E_e ce_e = u^T K u. With a workspace of gbsimp_sensitivity_ws_bytes and a
 * modal-form Ke the element products run in double-float (about 2^-46 relative rounding of
 * the element's displacement magnitudes); with a smaller workspace (at least the size the
 * energy sum needs, 256 + 4096 * 32 bytes) or none, in FP64. */
size_t gbsimp_sensitivity_ws_bytes(int nx, int ny, int nz);
int gbsimp_sensitivity(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                       const float *x, const double *u, float *dc, float *ce,
                       double *energy_out, void *ws, size_t ws_bytes, void *stream);
/* Arbitrary edof table and FP32 u (cuda_kernels.simp_sensitivity, __init__.py:286-326). */
int gbsimp_sensitivity_edof_f32(gbsimp_ctx *ctx, int64_t n_elem, int64_t n_dof,
                                const void *edof, int edof_is_int64, const gbsimp_law *law,
                                const float *x, const float *u, float *dc, void *stream);

/* ---- density filter ---------------------------------------------------------------- */
/* H[e1,e2] = rmin - dist(e1,e2) for dist <= rmin (clipped at the grid boundary),
 * Hs = row sums (simp_solver.py:1545-1567). transpose 0: out = H in / Hs (simp_solver.py:237);
 * transpose 1: out = H^T (in / Hs) (simp_solver.py:221-223). rmin <= 6. hs: nullable
 * precomputed row sums (from gbsimp_filter_hs), else computed on the fly. */
int gbsimp_filter_hs(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, float *hs,
                     void *stream);
int gbsimp_filter(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin, const float *hs,
                  const float *in, float *out, int transpose, void *stream);

/* ---- OC update --------------------------------------------------------------------- */
/* Bisection on the Lagrange multiplier (simp_solver.py:225-249; parameters above).
 * The volume of each trial is sum_e w_e xnew_e + n_preserved with the precomputed weights
 * w = H^T(m / Hs), m_e = 0 on preserved elements else 1 (same value as mean(H xnew / Hs)
 * with the preserved entries set to 1). Bisection runs on the device (no host sync).
 * Outputs: xnew, xphys (= H xnew / Hs, preserved -> 1), and in the workspace the final
 * multiplier and step count, copied to host by gbsimp_oc_result(). preserved nullable. */
size_t gbsimp_oc_ws_bytes(int nx, int ny, int nz);
int gbsimp_oc_prepare(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin,
                      const uint8_t *preserved, void *ws, size_t ws_bytes, void *stream);
int gbsimp_oc(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin,
              const gbsimp_oc_params *prm, const float *x, const float *dc,
              const uint8_t *preserved, float *xnew, float *xphys, void *ws, size_t ws_bytes,
              void *stream);
/* OC update that allocates nothing (no counterpart in the reference). It exists for callers
 * that cannot allocate device memory: a host-language plugin that reaches the GPU only
 * through this C ABI and has no CUDA allocator of its own, or a serving process whose device
 * memory is reserved up front and must not grow per request. Same inputs, outputs and
 * results as gbsimp_oc, but the scratch is a fixed 16.1 MiB device array inside the library
 * (held on every GPU that loads the library until the process exits), so grids above
 * GBSIMP_OC_NOALLOC_MAX_ELEMENTS elements are rejected with GBS_EINVAL. The first call on a
 * device looks up that array's device address (call it with the context's device current);
 * make that first call before any stream capture. All calls share the one array and each
 * call re-initialises what it reads: calls that overlap on the GPU (other streams, other
 * threads) race and must not be issued. The final multiplier and bisection step count stay in
 * that array, which gbsimp_oc_result cannot reach: they are not available from this entry
 * point. The array's address is cached per device for the life of the process, so, like
 * every context of this library, it must not be used across a cudaDeviceReset. */
#define GBSIMP_OC_NOALLOC_MAX_ELEMENTS 2097152
int gbsimp_oc_noalloc(gbsimp_ctx *ctx, int nx, int ny, int nz, double rmin,
                      const gbsimp_oc_params *prm, const float *x, const float *dc,
                      const uint8_t *preserved, float *xnew, float *xphys, void *stream);
/* Synchronises the stream; returns lambda and bisection steps of the last gbsimp_oc. */
int gbsimp_oc_result(gbsimp_ctx *ctx, const void *ws, double *lambda_out, int *steps_out,
                     void *stream);

/* ---- linear solves ----------------------------------------------------------------- */
/* FP32 Jacobi-PCG on the free DOFs (simp_solver_gpu.py:328-379, _solve :571-705):
 * u holds x0 on entry (fixed DOFs are zeroed), the solution on exit. The stop test is
 * ||r|| < rtol ||D b||, checked on the device every iteration. The iteration loop runs on
 * the device: a CUDA graph (cached per buffer set) whose WHILE node repeats 12 iterations
 * while the device-side stop flag is clear, with a hard cap derived from max_iter
 * (GBS_ETIMEOUT). With opts->profile the host launches the iterations instead, checking
 * every opts->check_every iterations, and times each apply launch. Synchronises the stream. */
size_t gbsimp_pcg_ws_bytes(int nx, int ny, int nz);
int gbsimp_pcg_f32(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                   const float *x, const float *b, const uint8_t *node_mask, float *u,
                   const gbsimp_solve_opts *opts, gbsimp_solve_stats *stats, void *ws,
                   size_t ws_bytes, void *stream);
/* Measures the kernel that dominates gbsimp_pcg_f32 and gbsimp_solve on the densities x:
 * one whole PCG iteration in one launch (modal element: the single-reduction pass that
 * stages s, r and u = M r, applies K to u, updates p and the iterate and sums r.u, w.u and
 * r.r; dense element: the apply fused with p = z + beta p, the iterate update and p.Ap),
 * with frozen scalars. reps back-to-back launches replayed from one CUDA graph, timed with
 * CUDA events on the stream; writes the mean device time per launch. Synchronises the
 * stream. */
size_t gbsimp_time_pcg_apply_ws_bytes(int nx, int ny, int nz);
int gbsimp_time_pcg_apply(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                          const float *x, const uint8_t *node_mask, int reps, void *ws,
                          size_t ws_bytes, double *seconds_per_launch, void *stream);
/* FP32 PCG inner solves with outer defect correction: r = D(f - K u), FP32 PCG on K d = r
 * from d = 0 to max(inner_rtol, rtol / (||r|| / ||D f||)), u += d (FP64), until
 * ||r|| <= rtol ||D f||. u (FP64) holds the warm start on entry. For rtol >= 1e-9 and a modal-form Ke, unless opts->residual_fp64 is set, the
 * residual runs in double-float arithmetic (FP32 pairs: rounding about 2^-46 of the
 * displacement magnitudes of an element, measured below 6.1e-13 ||D f|| on converged fields)
 * with FP64 u; otherwise its element products are FP64. Synchronises the stream. */
size_t gbsimp_solve_ws_bytes(int nx, int ny, int nz);
int gbsimp_solve(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                 const float *x, const double *f, const uint8_t *node_mask, double *u,
                 const gbsimp_solve_opts *opts, gbsimp_solve_stats *stats, void *ws,
                 size_t ws_bytes, void *stream);
/* Warm start of the next solve of a SIMP loop from the last two solutions: for each of the n
 * entries, t = u[i]; u[i] = t + theta (t - u_prev[i]); u_prev[i] = t (one FP64 fma). With
 * theta = 0.5 (the native loop's value) a 64^3 SIMP step needed 6.7% fewer PCG iterations than
 * with u alone; the solve still runs to its tolerance, so only the iterations change. */
int gbsimp_warm_start(gbsimp_ctx *ctx, int64_t n, double *u, double *u_prev, double theta,
                      void *stream);
/* ---- batched solves (many designs of different sizes in one launch) ------------------ */
/* One design of a batch. The caller fills the grid, the arrays (same meaning as in
 * gbsimp_solve) and a workspace of gbsimp_solve_ws_bytes(nx, ny, nz) bytes, sets state = 0
 * and zeroes stats; the library updates state (0 active, 1 converged, 2 stopped: see
 * stats.status) and accumulates stats across rounds. */
typedef struct gbsimp_batch_item {
    int32_t nx, ny, nz;
    int32_t state;
    const float *x;
    const double *f;
    const uint8_t *node_mask;
    double *u;
    void *ws;
    size_t ws_bytes;
    gbsimp_solve_stats stats;
} gbsimp_batch_item;

/* One round of the FP64 defect correction for every active item: FP64 residuals (one sync
 * for all), then the FP32 PCG of every item still above rtol, then the FP64 corrections.
 * With opts->fused the PCGs run as cooperative launches of a persistent kernel, up to 24
 * items per launch (packed greedily from the items that are resident together), each item on
 * its own share of the SMs with its own grid barrier and scalars, converging independently.
 * An item that fits no such launch, or any item when opts->fused is 0, runs its own
 * device-driven graph loop instead, enqueued on the same stream. With opts->check_every > 0 a
 * round runs at most that many inner iterations per item: an inner PCG still running then is
 * paused (stats.inner_active) and continues in the next round, so a round lasts a bounded time
 * whatever the grid sizes. Items may be added (state 0) or dropped between rounds: the serving
 * loop's continuous batching. Replaces one gbsimp_solve per design (the reference's one solve per
 * GPUVoxelFEM.solve, gpu_fem_solver.py:76-133, fed by evaluate_batch's thread pool,
 * voxel_fem.py:559-611). Synchronises the stream. */
int gbsimp_batch_round(gbsimp_ctx *ctx, gbsimp_batch_item *items, int n, const gbsimp_law *law,
                       const gbsimp_solve_opts *opts, void *stream);
/* Rounds until every item has state != 0. */
int gbsimp_batch_solve(gbsimp_ctx *ctx, gbsimp_batch_item *items, int n, const gbsimp_law *law,
                       const gbsimp_solve_opts *opts, void *stream);

/* ---- solve queue (continuous batching behind submit / poll) ---------------------------- */
/* A queue of solves advanced together by gbsimp_batch_round (one FP64 round per poll, with
 * the persistent batched PCG inside). Replaces the evaluator's thread pool of one solve per
 * design (voxel_fem.py:559-611 over gpu_fem_solver.py:76-133) for a serving loop: requests
 * join between rounds as they arrive and leave when they are done. The queue keeps pointers to
 * the submitted items; their buffers and workspaces stay the caller's until poll returns
 * them. All items of a queue share the law and the solve options given at creation.
 * submit, poll and size may be called from different threads: each takes the queue's lock,
 * and poll holds it for its whole round, so a submit during a round waits for that round
 * and joins the next. */
typedef struct gbsimp_queue gbsimp_queue;
int gbsimp_queue_create(gbsimp_ctx *ctx, const gbsimp_law *law, const gbsimp_solve_opts *opts,
                        gbsimp_queue **out);
int gbsimp_queue_destroy(gbsimp_queue *q);
/* Adds an item (its state is set to 0: it joins the next round). u holds its warm start. */
int gbsimp_queue_submit(gbsimp_queue *q, gbsimp_batch_item *item);
/* Runs one round for every queued item, then hands back up to max_done finished items
 * (state != 0, stats filled) in done[0..*n_done); finished items beyond max_done are handed
 * back by the next polls. Synchronises the stream. */
int gbsimp_queue_poll(gbsimp_queue *q, gbsimp_batch_item **done, int max_done, int *n_done,
                      void *stream);
/* Items queued or finished and not yet handed back. */
int gbsimp_queue_size(const gbsimp_queue *q);

/* ---- SIMP loop --------------------------------------------------------------------------- */
typedef struct gbsimp_simp_opts {
    double volfrac;            /* target volume fraction (replaces oc.volfrac) */
    double rmin;               /* density filter radius */
    int32_t n_iters;           /* OC iterations */
    int32_t early_stop;        /* 1: stop after three consecutive relative changes below 1% of
                                  the objective (the rule of SIMPSolverGPU.run,
                                  simp_solver_gpu.py:111-125, which tests a fresh compliance
                                  solve after each update; here each iteration's own objective,
                                  so the stop comes one design later) */
    gbsimp_oc_params oc;       /* the bisection (CPU or GPU variant parameters) */
    gbsimp_solve_opts solve;   /* the refined solves (gbsimp_solve) */
} gbsimp_simp_opts;
/* The SIMP loop of SIMPSolver.run (simp_solver.py:56-79) in one call: xphys = x, then per
 * iteration the solve K(xphys) u = f (from the third iteration on warm-started from
 * u_{k-1} + 0.5 (u_{k-1} - u_{k-2}), gbsimp_warm_start; before that from u), the element energies and
 * dc = -dE/dx ce at xphys, dc <- H^T(dc / Hs), and the OC update of x (xphys = H xnew / Hs,
 * preserved elements 1). x: initial design in, final design out; xphys: out; u: FP64 warm
 * start in, the last solve's displacement out. compliance (host, nullable, n_iters doubles)
 * receives sum_e E_e ce_e of each iteration (the reference's objective); reading it, and the
 * early stop, cost one stream synchronisation per iteration. *iters_out: iterations run.
 * *last_stats: the last solve. Stops with the solve's status on a failed solve. */
size_t gbsimp_simp_run_ws_bytes(int nx, int ny, int nz);
int gbsimp_simp_run(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law,
                    const gbsimp_simp_opts *opts, const double *f, const uint8_t *node_mask,
                    const uint8_t *preserved, float *x, float *xphys, double *u,
                    double *compliance, int32_t *iters_out, gbsimp_solve_stats *last_stats,
                    void *ws, size_t ws_bytes, void *stream);

/* Jacobi-PCG on a CSR matrix (int32 row_ptr/col_idx, FP32 values, FP32 diagonal), the
 * contract of cuda_kernels.pcg_solve_cuda (cuda_kernels/__init__.py:443-473,
 * simp_pcg_cuda.cu:66-124): x holds x0 on entry; fixed is a list of n_fixed DOF indices
 * whose residual entries are zeroed. Synchronises the stream. */
size_t gbsimp_pcg_csr_ws_bytes(int64_t n);
int gbsimp_pcg_csr_f32(gbsimp_ctx *ctx, int64_t n, const int32_t *row_ptr,
                       const int32_t *col_idx, const float *values, const float *diagonal,
                       const float *b, float *x, const int32_t *fixed, int64_t n_fixed,
                       const gbsimp_solve_opts *opts, gbsimp_solve_stats *stats, void *ws,
                       size_t ws_bytes, void *stream);

/* Diagnostic of the persistent kernels' grid barrier (no counterpart in the reference): one
 * cooperative launch (one block per SM) in which every block arrives once and waits, at most
 * wait_seconds (<= 2), for gridDim + extra_arrivals arrivals. *status_out is GBS_OK when the
 * barrier completed with the right sum (extra_arrivals = 0) and GBS_ETIMEOUT when the bounded
 * wait expired because the missing arrivals never came (extra_arrivals > 0); the context
 * stays usable either way. Synchronises the stream. */
size_t gbsimp_barrier_selftest_ws_bytes(void);
int gbsimp_barrier_selftest(gbsimp_ctx *ctx, int extra_arrivals, double wait_seconds, int *status_out,
                            void *ws, size_t ws_bytes, void *stream);

/* ---- reductions used by the host loops -------------------------------------------- */
/* out (device double) = sum_i a_i * b_i over n FP64 entries, fixed block order. */
int gbsimp_dot_f64(gbsimp_ctx *ctx, int64_t n, const double *a, const double *b,
                   double *out, void *ws, size_t ws_bytes, void *stream);

/* ---- evaluator input step ------------------------------------------------------------ */
/* A batch of (D, H, W) FP32 density grids -> (d, h, w): linear resampling as
 * scipy.ndimage.zoom(v, zoom, order=1) (output o reads input coordinate
 * o (n_in - 1) / (n_out - 1)), then smooth_voxels: Gaussian of `sigma` voxels (radius
 * int(4 sigma + 0.5), mirror "reflect" boundary) and the logistic
 * 1 / (1 + exp(-sharpness (v - 0.5))). Replaces the host-side zoom + smooth_voxels of
 * VoxelFEMEvaluator.evaluate (fem/voxel_fem.py:457-462, pipeline_utils.py:55-76); d = D etc.
 * gives smooth_voxels alone. Extents 1..1024 (an output extent of 1 only for an input
 * extent of 1); returns GBS_EINVAL when a row of the combined filter needs more than 32 taps.
 * Returns 0 from the size query for invalid extents. */
size_t gbsimp_voxel_prep_ws_bytes(int batch, int D, int H, int W, int d, int h, int w);
int gbsimp_voxel_prep(gbsimp_ctx *ctx, int batch, int D, int H, int W, const float *in, int d,
                      int h, int w, float *out, double sigma, double sharpness, void *ws,
                      size_t ws_bytes, void *stream);

/* ---- STL export step ------------------------------------------------------------------- */
/* Isosurface of an (nx, ny, nz) FP32 grid (C order) at `level`: marching cubes over the cells
 * between grid points, as density_to_stl extracts it before writing the STL
 * (topology/mesh_export.py:7-67, which uses skimage on the host). Corners with
 * value >= level are inside; ambiguous faces separate their inside corners (no cracks);
 * triangles point from inside to outside. Output: 9 floats per triangle (three vertices in
 * grid units times (sx, sy, sz)), in cell order. *n_tris receives the count; when tris is
 * NULL or max_tris < count nothing is written (size query). Synchronises the stream. */
size_t gbsimp_marching_cubes_ws_bytes(int nx, int ny, int nz);
int gbsimp_marching_cubes(gbsimp_ctx *ctx, int nx, int ny, int nz, const float *vol, double level,
                          double sx, double sy, double sz, float *tris, int64_t max_tris,
                          int64_t *n_tris, void *ws, size_t ws_bytes, void *stream);
/* The case table the kernel uses (host memory, no GPU needed): per case the triangle count
 * (ntri[256]), loop count (nloop[256]), loop lengths (len[256][4]) and the loops' cut-edge
 * indices (edge[256][12]). Any pointer may be NULL. Returns an upper bound on any case's
 * triangle count: 12, the number of cell edges (a loop of n cut edges gives at most n). */
int gbsimp_marching_cubes_table(unsigned char *ntri, unsigned char *nloop, unsigned char *len,
                                signed char *edge);

#ifdef __cplusplus
}
#endif
#endif /* GBSIMP_H */
