// pcg.cu -- Jacobi-PCG drivers: FP32 matrix-free PCG, FP32-inner / FP64-outer defect
// correction, and a CSR PCG for the pcg_solve_cuda contract.
//
// Two forms of the same Jacobi-PCG (simp_solver_gpu.py:328-379: z = r/diag, stop when
// ||r|| < rtol ||D b||):
// - modal element (isotropic cube Ke): one launch per iteration, the single-reduction form
//   (apply_modal.cuh, MODE_CG): the staging of the apply operand u_{i+1} = M r_{i+1} also
//   forms s_i and r_{i+1}, the owned nodes update p (and x on odd launches, two iterations
//   at once), and each block writes its sums of r.u, w.u and r.r; the next launch folds them
//   at its start (every block, in block order) into beta_{i+1} and alpha_{i+1}. Setup: r_0,
//   u_0, w_0 = A u_0, alpha_0 = (r_0.u_0) / (w_0.u_0).
// - dense element (any other Ke): two launches per iteration k (setup r_0, p_{-1} = 0):
//   K1  apply_tile_kernel<MODE_PCG>: p_k = z_k + beta_k p_{k-1} on the halo while staging,
//       x += alpha_{k-1} p_{k-1} on owned nodes, Ap_k = D K D p_k, p_k.Ap_k -> alpha_k.
//   K2  pcg_update_kernel: r_{k+1} = r_k - alpha_k Ap_k, ||r||^2 and r.z -> beta_{k+1}.
// Every scalar lives on the device; each kernel exits at once when the solve is done, so
// the host can launch whole chunks of iterations and look at the status once per chunk.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "apply_modal.cuh"
#include "internal.h"

namespace gbs {

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

static inline int64_t n_dof_of(int nx, int ny, int nz) { return 3LL * (nx + 1) * (ny + 1) * (nz + 1); }

// Blocks of 256 threads for a vector kernel that ends in a last-block reduction (at most 8 per
// SM: the partials hold 4096 per sum, and the last block sums them all).
static inline unsigned vec_blocks(const gbsimp_ctx *ctx, int64_t n) {
    int64_t b = (n + 255) / 256;
    const int64_t cap = 8LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}
// ... and for an elementwise kernel: about one element per thread, so that the loads of every
// element are in flight together rather than one grid-stride round trip after another.
static inline unsigned ew_blocks(const gbsimp_ctx *ctx, int64_t n) {
    int64_t b = (n + 255) / 256;
    const int64_t cap = 64LL * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    if (b > cap) b = cap;
    return (unsigned)(b < 1 ? 1 : b);
}

// ---- workspace of the FP32 PCG -----------------------------------------------------------
// Dense form: r, dinv, p0/p1 (p_k in p[k&1]), ap. Single-reduction form: r/r1 (r[i&1]),
// ap/p1/w2 (w[i%3]; the persistent kernel w[i&1]), s0/s1 (s[i&1]), p0 (p), dinv.
struct PcgWs {
    PcgScalars *sc;
    float *r, *dinv, *p0, *p1, *ap, *r1, *s0, *s1, *w2;
    double *partials;
    size_t partial_count;
    float *E;  // element moduli E(x_e) of the solve (single-reduction form: read by every launch)
};

static inline bool use_modal(const gbsimp_ctx *ctx, int nz) { return ctx->modal_ok && modal_fits(nz); }

// Partial sums (8 bytes each) of the workspace: one per CTA of the dense form; two slots of
// three per CTA of the one-kernel PCG, whose launch has tiles x segments <= max(tiles,
// one wave) CTAs (checked in pcg_setup); three per block of the vector reductions.
static size_t pcg_partials(int nx, int ny, int nz) {
    const dim3 g = tile_grid<TileF>(nx, ny, nz);
    size_t n = (size_t)g.x * g.y * g.z;
    if (modal_fits(nz)) {
        const int t = modal_tiles(ny, nz);
        const size_t m = 6 * (size_t)(t > kModalMaxWave ? t : kModalMaxWave);
        if (m > n) n = m;
    }
    return n > 3 * 4096 ? n : 3 * 4096;
}

// The one-kernel PCG's launch on this grid writes 6 partial sums per CTA: refuse a workspace
// that cannot hold them (a wave larger than kModalMaxWave CTAs).
static int check_modal_partials(const gbsimp_ctx *ctx, int nx, int ny, int nz, const PcgWs &w) {
    const int nblk = modal_blocks<MODE_CG>(ctx, nx, ny, nz);
    if (nblk < 0) return -nblk;
    if (6 * (size_t)nblk > w.partial_count)
        return set_error(GBS_EINVAL, "PCG: the launch needs more partial sums than the workspace holds");
    return GBS_OK;
}

static size_t pcg_ws_bytes_impl(int nx, int ny, int nz) {
    const size_t nd = (size_t)n_dof_of(nx, ny, nz);
    return 256 + al256(sizeof(PcgScalars)) + 9 * al256(nd * sizeof(float)) +
           al256(pcg_partials(nx, ny, nz) * sizeof(double)) + al256((size_t)nx * ny * nz * sizeof(float));
}

// Sub-buffers start on 256-byte boundaries whatever the alignment of `ws` (the size has
// 256 bytes of slack); the modal kernels copy vectors in aligned 16-byte groups.
static char *align256(void *ws) { return (char *)(((uintptr_t)ws + 255) & ~(uintptr_t)255); }

static PcgWs pcg_ws(void *ws, int nx, int ny, int nz) {
    const size_t nd = (size_t)n_dof_of(nx, ny, nz);
    char *p = align256(ws);
    PcgWs w;
    w.sc = (PcgScalars *)p;
    p += al256(sizeof(PcgScalars));
    float **v[9] = {&w.r, &w.dinv, &w.p0, &w.p1, &w.ap, &w.r1, &w.s0, &w.s1, &w.w2};
    for (int i = 0; i < 9; ++i) {
        *v[i] = (float *)p;
        p += al256(nd * sizeof(float));
    }
    w.partials = (double *)p;
    w.partial_count = pcg_partials(nx, ny, nz);
    p += al256(w.partial_count * sizeof(double));
    w.E = (float *)p;
    return w;
}

// E[e] = E(x_e): the single-reduction kernels read the moduli instead of evaluating the law
// per element and launch (the same FP32 function of the same inputs, so the same values).
__global__ void moduli_f32_kernel(int64_t n, Law<float> law, const float *__restrict__ x, float *E) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        E[e] = modulus(law, x[e]);
}

static CgArgs cg_args(const PcgWs &w, float *u) {
    CgArgs a;
    a.r[0] = w.r;
    a.r[1] = w.r1;
    a.w[0] = w.ap;
    a.w[1] = w.p1;
    a.w[2] = w.w2;
    a.s[0] = w.s0;
    a.s[1] = w.s1;
    a.p = w.p0;
    a.xu = u;
    a.dinv = w.dinv;
    a.partials = w.partials;
    a.sc = w.sc;
    return a;
}

__device__ __forceinline__ bool dof_fixed(const uint8_t *mask, int64_t d) {
    return mask && ((mask[d / 3] >> (int)(d % 3)) & 1);
}

// dinv = 1 / diag(K(x)) on free DOFs, 0 on fixed DOFs; diag_{n,c} = sum_{e ∋ n} E_e Ke[(a,c),(a,c)].
template <typename T>
__global__ void dinv_kernel(int nx, int ny, int nz, const FastDiv fNY, const FastDiv fNZ, Law<T> law, const KeF kd,
                            const float *__restrict__ x, const uint8_t *__restrict__ mask, float *dinv) {
    const int64_t NY = ny + 1, NZ = nz + 1;
    const int64_t n_nodes = (int64_t)(nx + 1) * NY * NZ;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten3((uint32_t)n, fNY, fNZ, i, j, k);
        // the 8 density loads first; an element outside the grid adds an exact zero
        float xe[8];
        bool in[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const int ei = i - corner_x(a), ej = j - corner_y(a), ek = k - corner_z(a);
            in[a] = ei >= 0 && ej >= 0 && ek >= 0 && ei < nx && ej < ny && ek < nz;
            xe[a] = in[a] ? x[((int64_t)ei * ny + ej) * nz + ek] : 0.0f;
        }
        T acc[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const T E = in[a] ? modulus(law, (T)xe[a]) : (T)0;
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] += E * (T)kd.k[(3 * a + c) * 25];
        }
        const uint8_t m = mask ? mask[n] : (uint8_t)0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            dinv[3 * n + c] = ((m >> c) & 1) || !(acc[c] > 0) ? 0.0f : (float)((T)1 / acc[c]);
    }
}

// Block sums of three quantities; the last block finishes the reduction.
__device__ bool last_block3(double a, double b, double c, double *partials, unsigned *counter, double *out) {
    __shared__ double sred[32];
    __shared__ bool last;
    const int nblk = gridDim.x;
    const double ba = block_sum(a, sred);
    const double bb = block_sum(b, sred);
    const double bc = block_sum(c, sred);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = ba;
        partials[nblk + blockIdx.x] = bb;
        partials[2 * nblk + blockIdx.x] = bc;
        __threadfence();
        last = (atomicAdd(counter, 1u) == (unsigned)(nblk - 1));
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        for (int i = threadIdx.x; i < nblk; i += blockDim.x) s += ((volatile double *)partials)[k * nblk + i];
        s = block_sum(s, sred);
        if (threadIdx.x == 0) out[k] = s;
    }
    if (threadIdx.x == 0) *counter = 0;
    return true;
}

// The same for FP32 per-thread partials, in double-float on the FP32 pipe (block sums, the
// per-block partials and the last block's sum in block order); the totals in out[] are valid
// in thread 0 of the last block.
__device__ bool last_block3_df(df32 a, df32 b, df32 c, float2 *partials, unsigned *counter, double *out) {
    __shared__ float2 sred[3 * 32];
    __shared__ bool last;
    const int nblk = gridDim.x;
    df32 v[3] = {a, b, c};
    block_sum_df<3>(v, sred);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) partials[k * nblk + blockIdx.x] = make_float2(v[k].hi, v[k].lo);
        __threadfence();
        last = (atomicAdd(counter, 1u) == (unsigned)(nblk - 1));
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    df32 s[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    for (int i = threadIdx.x; i < nblk; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float2 p = __ldcg(&partials[k * nblk + i]);
            s[k] = df_add(s[k], df32{p.x, p.y});
        }
    block_sum_df<3>(s, sred);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) out[k] = df_value(s[k]);
        *counter = 0;
    }
    return true;
}
__device__ __forceinline__ bool last_block3_df(float a, float b, float c, float2 *partials, unsigned *counter,
                                               double *out) {
    return last_block3_df(df32{a, 0.0f}, df32{b, 0.0f}, df32{c, 0.0f}, partials, counter, out);
}

// r = D b - q (q = D K D x0), x0 fixed entries zeroed, p_{-1} = 0; sums r.z, r.r, (Db).(Db).
__global__ void pcg_init_kernel(int64_t nd, const float *__restrict__ b, const float *__restrict__ q,
                                const uint8_t *__restrict__ mask, const float *__restrict__ dinv, float *r, float *pprev,
                                float *xu, double *partials, PcgScalars *sc, double tol, int max_iter,
                                int max_trips) {
    // per-thread partials in FP32 (a few terms each), block and grid sums in FP64
    float rz = 0.0f, rr = 0.0f, bb = 0.0f;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        const bool fx = dof_fixed(mask, d);
        const float bd = fx ? 0.0f : b[d];
        const float rd = fx ? 0.0f : bd - q[d];
        r[d] = rd;
        pprev[d] = 0.0f;
        if (fx) xu[d] = 0.0f;
        rz = fmaf(rd * dinv[d], rd, rz);
        rr = fmaf(rd, rd, rr);
        bb = fmaf(bd, bd, bb);
    }
    __shared__ double tot[3];
    if (last_block3(rz, rr, bb, partials, &sc->counter, tot) && threadIdx.x == 0) {
        sc->rz = tot[0];
        sc->rr = tot[1];
        sc->bnorm = sqrt(tot[2]);
        sc->alpha[0] = sc->alpha[1] = 0.0;
        sc->beta = 0.0;
        sc->tol = tol;
        sc->pap = 0.0;
        sc->iter = 0;
        sc->max_iter = max_iter;
        sc->trips = 0;
        sc->max_trips = max_trips;
        sc->status = GBS_OK;
        const bool fin = isfinite(tot[0]) && isfinite(tot[1]) && isfinite(tot[2]);
        sc->done = (!fin || sc->bnorm == 0.0 || sqrt(tot[1]) < tol * sc->bnorm || max_iter <= 0) ? 1 : 0;
        if (!fin) sc->status = GBS_ENONFINITE;
        else if (max_iter <= 0 && !(sqrt(tot[1]) < tol * sc->bnorm) && sc->bnorm != 0.0) sc->status = GBS_ENOTCONV;
    }
}

// Single-reduction setup, step 1: r_0 = D b - q (q = D K D x0, read from `qu`), u_0 = M r_0
// written over q, p_{-1} = s_{-1} = 0, fixed entries of x0 zeroed; sums r.u, r.r, (Db).(Db)
// and the stop test of the initial guess.
// x0_zero: x0 = 0 is known, q is not read (and x0 is written as zero).
__global__ void cg_init_kernel(int64_t nd, const float *__restrict__ b, float *qu, const uint8_t *__restrict__ mask,
                               const float *__restrict__ dinv, float *r, float *p, float *sprev, float *xu,
                               double *partials, PcgScalars *sc, double tol, int max_iter, int max_trips,
                               int x0_zero) {
    float ru = 0.0f, rr = 0.0f, bb = 0.0f;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        const bool fx = dof_fixed(mask, d);
        const float bd = fx ? 0.0f : b[d];
        const float rd = fx ? 0.0f : (x0_zero ? bd : bd - qu[d]);
        const float ud = dinv[d] * rd;
        r[d] = rd;
        qu[d] = ud;
        p[d] = 0.0f;
        sprev[d] = 0.0f;
        if (fx || x0_zero) xu[d] = 0.0f;
        ru = fmaf(rd, ud, ru);
        rr = fmaf(rd, rd, rr);
        bb = fmaf(bd, bd, bb);
    }
    __shared__ double tot[3];
    if (last_block3_df(ru, rr, bb, (float2 *)partials, &sc->counter, tot) && threadIdx.x == 0) {
        sc->rz = tot[0];
        sc->rr = tot[1];
        sc->bnorm = sqrt(tot[2]);
        sc->alpha[0] = sc->alpha[1] = 0.0;
        sc->beta = 0.0;
        sc->tol = tol;
        sc->pap = 0.0;
        sc->iter = 0;
        sc->max_iter = max_iter;
        sc->trips = 0;
        sc->max_trips = max_trips;
        sc->freeze = 0;
        sc->status = GBS_OK;
        const bool fin = isfinite(tot[0]) && isfinite(tot[1]) && isfinite(tot[2]);
        sc->done = (!fin || sc->bnorm == 0.0 || sqrt(tot[1]) < tol * sc->bnorm || max_iter <= 0) ? 1 : 0;
        if (!fin) sc->status = GBS_ENONFINITE;
        else if (max_iter <= 0 && !(sqrt(tot[1]) < tol * sc->bnorm) && sc->bnorm != 0.0) sc->status = GBS_ENOTCONV;
    }
}

// Single-reduction setup, step 2 (after w_0 = D K D u_0): alpha_0 = (r_0.u_0) / (w_0.u_0),
// beta_0 = 0.
__global__ void cg_start_kernel(int64_t nd, const float *__restrict__ w, const float *__restrict__ u,
                                double *partials, PcgScalars *sc) {
    if (sc->done) {  // the first launch reads state slot 1
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            CgState s = {};
            s.done = 1;
            s.status = sc->status;
            s.rr = df_from(sc->rr);
            s.gamma = df_from(sc->rz);
            sc->st[1] = s;
        }
        return;
    }
    float wu = 0.0f;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x)
        wu = fmaf(w[d], u[d], wu);
    __shared__ double tot[3];
    if (last_block3_df(wu, 0.0f, 0.0f, (float2 *)partials, &sc->counter, tot) && threadIdx.x == 0) {
        sc->pap = tot[0];
        if (!isfinite(tot[0])) {
            sc->done = 1;
            sc->status = GBS_ENONFINITE;
        } else if (!(tot[0] > 0.0)) {
            sc->done = 1;
            sc->status = GBS_EBREAKDOWN;
        } else {
            sc->alpha[0] = sc->rz / tot[0];
            sc->beta = 0.0;
        }
        const double stop = sc->tol * sc->bnorm;
        sc->rr_stop = (float)(stop * stop);
        CgState s = {};
        s.alpha = df_from(sc->alpha[0]);
        s.gamma = df_from(sc->rz);
        s.rr = df_from(sc->rr);
        s.pap = df_from(tot[0]);
        s.done = sc->done;
        s.status = sc->status;
        sc->st[1] = s;
    }
}

// After a run of one-kernel PCG launches (the last one of parity `last`): folds that launch's
// pending partial sums and publishes the state in the host-visible fields. A status already
// set on the host-visible side (the loop's trip cap) is kept.
__global__ void cg_fold_kernel(int nblk, int last, double *partials, PcgScalars *sc) {
    __shared__ float2 sred[3 * 32];
    CgState s = sc->st[last];
    const int pend = s.pending;
    if ((pend == CG_PENDING_STEP || pend == CG_PENDING_FIRST) && !s.done)
        cg_fold<256>(s, sc, (const float2 *)partials + last * 3 * nblk, nblk, sred);
    if (threadIdx.x == 0) {
        if (pend == CG_PENDING_FIRST) sc->bnorm = sqrt(df_value(s.rr));
        sc->st[last] = s;
        sc->iter = s.iter;
        sc->rz = df_value(s.gamma);
        sc->rr = df_value(s.rr);
        sc->pap = df_value(s.pap);
        sc->alpha[0] = df_value(s.alpha);
        // alpha of the last launched iteration (x may still owe its step: pcg_finalize_kernel)
        sc->alpha[1] = df_value(s.done ? s.alpha : s.alpha_prev);
        sc->beta = df_value(s.beta);
        if (sc->status == GBS_OK) sc->status = s.status;
        sc->done = sc->done || s.done;
    }
}

__global__ void __launch_bounds__(256) pcg_update_kernel(int64_t nd, const float *__restrict__ ap,
                                                         const float *__restrict__ dinv, float *r, double *partials,
                                                         PcgScalars *sc) {
    if (sc->done) return;
    const int it = sc->iter;
    const float alpha = (float)sc->alpha[it & 1];
    float rz = 0.0f, rr = 0.0f;  // per-thread FP32 partials, FP64 block and grid sums
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        const float rd = fmaf(-alpha, ap[d], r[d]);
        r[d] = rd;
        rr = fmaf(rd, rd, rr);
        rz = fmaf(rd * dinv[d], rd, rz);
    }
    __shared__ double tot[3];
    if (last_block3(rz, rr, 0.0, partials, &sc->counter, tot) && threadIdx.x == 0) {
        sc->iter = it + 1;
        sc->rr = tot[1];
        if (!isfinite(tot[0]) || !isfinite(tot[1])) {
            sc->done = 1;
            sc->status = GBS_ENONFINITE;
        } else if (sqrt(tot[1]) < sc->tol * sc->bnorm) {
            sc->done = 1;
        } else if (it + 1 >= sc->max_iter) {
            sc->done = 1;
            sc->status = GBS_ENOTCONV;
        }
        sc->beta = tot[0] / sc->rz;
        sc->rz = tot[0];
    }
}

// After the loop: x = 0 when D b = 0; otherwise the dense form (lazy = 1) adds alpha_last
// p_last (the iteration that met the stop test has not yet added its own step). The
// persistent single-reduction kernel (lazy = 0) has x complete already; the one-kernel form
// (lazy = 2) updates x on odd launches for two iterations at once, so when the last launched
// iteration was even (iter odd) x still owes alpha p of it (p0 holds that p, alpha[1] its
// alpha).
__global__ void pcg_finalize_kernel(int64_t nd, const float *p0, const float *p1, float *xu, const PcgScalars *sc,
                                    int lazy) {
    if (!sc->done) return;  // paused by a batched round's budget: the next round resumes it
    const int st = sc->status;
    const int it = sc->iter;
    const bool zero = sc->bnorm == 0.0;
    if (lazy == 2) {
        if (!zero && !((it & 1) && st != GBS_ENONFINITE)) return;
        const float a = (float)sc->alpha[1];
        for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x)
            xu[d] = zero ? 0.0f : fmaf(a, p0[d], xu[d]);
        return;
    }
    if (!zero && (!lazy || it == 0 || st == GBS_EBREAKDOWN || st == GBS_ENONFINITE)) return;
    const float alpha = (float)sc->alpha[(it - 1) & 1];
    const float *p = ((it - 1) & 1) ? p1 : p0;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x)
        xu[d] = zero ? 0.0f : fmaf(alpha, p[d], xu[d]);
}

static int read_scalars(const PcgScalars *d, PcgScalars *h, cudaStream_t st) {
    void *hp = thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "no pinned staging buffer");
    GBS_CUDA_TRY(cudaMemcpyAsync(hp, d, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    GBS_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(h, hp, sizeof(PcgScalars));
    return GBS_OK;
}

// Launches one iteration: the single-reduction kernel (modal element) or K1 + K2.
static int pcg_iteration(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                         const uint8_t *mask, float *u, const PcgWs &w, cudaStream_t st, cudaEvent_t after_k1,
                         int phase) {
    if (use_modal(ctx, nz)) {  // reads the moduli w.E of the setup, not x
        int rc = launch_modal<MODE_CG>(ctx, nx, ny, nz, law, w.E, nullptr, nullptr, mask, cg_args(w, u), st, phase);
        if (rc) return rc;
        if (after_k1) GBS_CUDA_TRY(cudaEventRecord(after_k1, st));
        return GBS_OK;
    }
    PcgArgs pa{w.r, w.dinv, w.p0, w.p1, u, w.partials, w.sc};
    {
        TileArgs<float> A{nx, ny, nz, x, nullptr, w.ap, mask};
        const dim3 g = tile_grid<TileF>(nx, ny, nz), b = tile_block<TileF>();
        if (ctx->translation_free)
            apply_tile_kernel<float, KeF, TileF::X, TileF::Y, TileF::Z, true, MODE_PCG><<<g, b, 0, st>>>(A, law, ctx->kef, pa);
        else
            apply_tile_kernel<float, KeF, TileF::X, TileF::Y, TileF::Z, false, MODE_PCG><<<g, b, 0, st>>>(A, law, ctx->kef, pa);
        GBS_LAUNCH_CHECK("apply_tile_kernel<PCG>");
    }
    if (after_k1) GBS_CUDA_TRY(cudaEventRecord(after_k1, st));
    const int64_t nd = n_dof_of(nx, ny, nz);
    pcg_update_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, w.ap, w.dinv, w.r, w.partials, w.sc);
    GBS_LAUNCH_CHECK("pcg_update_kernel");
    return GBS_OK;
}

// ---- persistent fused PCG: the whole solve in one cooperative launch ---------------------
// Every CTA keeps its (flat tile, x segment) of the modal apply for all iterations. One
// iteration = the single-reduction pass (apply_modal.cuh, MODE_CG_FUSED) -> one grid barrier
// that sums r.u, w.u and r.r -> the scalar step, which every CTA computes from the same
// totals. The barrier publishes per-block partials and every block sums them in block order
// (deterministic, no serial finisher). Each wait is bounded in time (%globaltimer): on expiry
// the CTA records GBS_ETIMEOUT, sets done and leaves.
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide sums at a barrier, in double-float. Each block publishes its K block sums in
// slot `slot` (two slots alternate: a block can only reach the next use of a slot after every
// block has left the barrier that last read it), arrives on a monotonic counter and waits for
// `target` arrivals; then every block sums all partials itself in block order, so every block
// holds the same totals (no serial finisher, deterministic). Waits are bounded by wait_ns.
template <int K>
__device__ bool grid_sums(const float (&v)[K], float2 *partials, int slot, unsigned *count, unsigned target, int nblk,
                          int bid, unsigned long long wait_ns, float2 *sred, df32 (&tot)[K]) {
    __shared__ bool s_ok;
    df32 bs[K];
#pragma unroll
    for (int k = 0; k < K; ++k) bs[k] = df32{v[k], 0.0f};
    block_sum_df<K>(bs, sred);
    float2 *part = partials + (size_t)slot * K * nblk;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) part[k * nblk + bid] = make_float2(bs[k].hi, bs[k].lo);
        __threadfence();
        atomicAdd(count, 1u);
        s_ok = true;
        const unsigned long long t0 = global_ns();
        while (*(volatile unsigned *)count < target) {
            if (global_ns() - t0 > wait_ns) {
                s_ok = false;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    if (!s_ok) return false;
    df32 s[K];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = df32{0.0f, 0.0f};
    for (int i = threadIdx.x; i < nblk; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 w = __ldcg(&part[k * nblk + i]);
            s[k] = df_add(s[k], df32{w.x, w.y});
        }
    block_sum_df<K>(s, sred);
    __shared__ df32 s_tot[K];
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) s_tot[k] = s[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) tot[k] = s_tot[k];
    return true;
}

// Self-test of the grid barrier above: every block arrives once and waits for
// gridDim.x + extra arrivals. With extra = 0 the barrier completes and every block sums the
// partials (one per block, 1.0 each); with extra > 0 nothing ever supplies the missing
// arrivals, so each block's bounded wait expires and the kernel records GBS_ETIMEOUT.
__global__ void barrier_selftest_kernel(double *partials, unsigned *count, int *status, unsigned extra,
                                        unsigned long long wait_ns) {
    __shared__ float2 sred[32];
    const float v[1] = {threadIdx.x == 0 ? 1.0f : 0.0f};  // 1.0 per block
    df32 tot[1];
    const bool ok = grid_sums<1>(v, (float2 *)partials, 0, count, gridDim.x + extra, (int)gridDim.x, (int)blockIdx.x,
                                 wait_ns, sred, tot);
    if (threadIdx.x == 0) {
        if (!ok) atomicExch(status, (int)GBS_ETIMEOUT);
        else if (df_value(tot[0]) != (double)gridDim.x) atomicExch(status, (int)GBS_EINVAL);
    }
}

// Designs of one cooperative launch. Each design owns the CTA range [block0, block0 + nblk)
// laid out as `tiles` flat tiles x (nblk / tiles) x segments, its own PCG state and barrier
// counter; designs advance independently.
constexpr int kMaxFused = 24;
struct FusedDesign {
    ModalGeom G;
    int tiles, block0, nblk, pad;
    const float *x;
    const uint8_t *mask;
    CgArgs ca;
};
struct FusedTable {
    int n, pad;
    FusedDesign d[kMaxFused];
};

template <int NT, int EPT, int MAXV>
__global__ void __launch_bounds__(NT, 2)
    pcg_fused_kernel(const __grid_constant__ FusedTable T, Law<float> law, const ModalK km,
                     unsigned long long wait_ns, int budget) {
    extern __shared__ float4 smem4[];
    __shared__ float2 sred[3 * 32];
    int di = 0;
    while (di + 1 < T.n && (int)blockIdx.x >= T.d[di + 1].block0) ++di;
    const FusedDesign &D = T.d[di];
    const ModalGeom &G = D.G;
    const CgArgs &ca = D.ca;
    const int bid = (int)blockIdx.x - D.block0;
    const int nblk = D.nblk;
    const int tile = bid % D.tiles, seg = bid / D.tiles;
    PcgScalars *sc = ca.sc;
    // The solve's scalars, identical in every block of the design (each block computes them).
    const volatile PcgScalars *vsc = sc;
    // Scalars in double-float (cg_scalar_step_df), as in the one-kernel-per-iteration form.
    int it = vsc->iter, done = vsc->done, status = vsc->status;
    df32 gamma_i = df_from(vsc->rz), alpha = df_from(vsc->alpha[0]), beta = df_from(vsc->beta);
    df32 rr = df_from(vsc->rr), delta = df_from(vsc->pap);
    const double stop = vsc->tol * vsc->bnorm;
    const float rr_stop = (float)(stop * stop);
    const int max_iter = vsc->max_iter;
    unsigned target = 0;
    // budget > 0: at most `budget` iterations in this launch; the state is written back with
    // `done` clear and the next launch resumes from it (iteration, scalars, buffer parity)
    const int it_end = budget > 0 ? it + budget : 0x7fffffff;
    while (!done && it < it_end) {
        const int c = it & 1, nc = c ^ 1;
        const CgPass cp{alpha.hi, beta.hi, ca.r[c], ca.w[c], ca.s[nc], ca.dinv, ca.r[nc], ca.s[c], ca.p, ca.xu, nullptr, ca.sc, 1};
        float sums[3];
        modal_pass<NT, EPT, MAXV, MODE_CG_FUSED>(G, D.x, nullptr, ca.w[nc], D.mask, law, km, cp, (float *)smem4, tile, seg,
                                                 sums, [](float &, float &, float &) { return true; });
        __threadfence();
        target += nblk;
        df32 tot[3];
        if (!grid_sums<3>(sums, (float2 *)ca.partials, it & 1, &sc->bar_count, target, nblk, bid, wait_ns, sred, tot)) {
            status = GBS_ETIMEOUT;
            break;
        }
        rr = tot[2];
        delta = tot[1];
        cg_scalar_step_df(tot[0], tot[1], tot[2], rr_stop, max_iter, it, done, status, gamma_i, alpha, beta);
    }
    if (status == GBS_ETIMEOUT) {
        if (threadIdx.x == 0) {
            atomicExch(&sc->status, (int)GBS_ETIMEOUT);
            atomicExch(&sc->done, 1);
        }
        return;
    }
    if (bid == 0 && threadIdx.x == 0) {
        sc->iter = it;
        sc->done = done;
        sc->status = status;
        sc->rz = df_value(gamma_i);
        sc->rr = df_value(rr);
        sc->pap = df_value(delta);
        sc->alpha[0] = df_value(alpha);
        sc->beta = df_value(beta);
    }
}

// One design of a batched inner solve: an initialised PCG state (pcg_run's setup done).
struct FusedItem {
    int nx, ny, nz;
    const float *x;
    const uint8_t *mask;
    float *u;
    PcgWs w;
};

// One cooperative launch of the persistent kernel over up to kMaxFused designs.
struct FusedPlan {
    void *kern;
    size_t smem;
    unsigned blocks;
    FusedTable T;
};

// Plans the launch of up to kMaxFused initialised designs: the CTAs of the GPU are shared in
// proportion to the designs' element counts (share 0) or element counts x longest extent
// (share 1: Jacobi-PCG iteration counts grow about with the longest extent, so the designs
// finish together instead of small ones leaving their SMs idle while a large one runs), at
// least one segment of flat tiles each. Returns GBS_EINVAL when the designs cannot all be
// resident at once (the caller then iterates them with the graph loop, or splits them over
// several launches). Host only. A paused design may be resumed under another plan: its state
// is the iteration's scalars and vectors, which do not depend on the segmentation.
static int fused_plan(const gbsimp_ctx *ctx, const FusedItem *items, int n, FusedPlan *plan, int share = 0) {
    if (n <= 0 || n > kMaxFused || !ctx->modal_ok) return GBS_EINVAL;
    bool small = true;
    int max_nz = 0;
    for (int i = 0; i < n; ++i) {
        if (!modal_fits(items[i].nz)) return GBS_EINVAL;
        small = small && modal_short(items[i].nz);
        max_nz = items[i].nz > max_nz ? items[i].nz : max_nz;
    }
    void *kern = small ? (void *)pcg_fused_kernel<kModalNT, kModalEPT, 2>
                       : (void *)pcg_fused_kernel<kModalNT, kModalEPT, 3>;
    static int ready_cache[2][128] = {};  // 1 = attribute set and cooperative launch supported, -1 = not
    static int reg_cache[2][128] = {};
    const int dev = ctx->device >= 0 && ctx->device < 128 ? ctx->device : 0;
    int &ready = ready_cache[small ? 0 : 1][dev];
    const size_t smem = modal_smem_bytes<kModalNT, kModalEPT>(max_nz, true);
    if (ready == 0) {
        const int smax = (int)modal_smem_bytes<kModalNT, kModalEPT>(446, true);
        int coop = 0;
        const bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax) == cudaSuccess &&
                        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop;
        cudaGetLastError();
        ready = ok ? 1 : -1;
    }
    if (ready < 0) return GBS_EINVAL;
    const int per_sm = modal_resident(ctx, kern, reg_cache[small ? 0 : 1][dev], smem);
    const int total = per_sm * (ctx->num_sms > 0 ? ctx->num_sms : 148);
    int tiles[kMaxFused], nseg[kMaxFused], seglen[kMaxFused];
    double weight[kMaxFused], wsum = 0.0;
    int need = 0;
    for (int i = 0; i < n; ++i) {
        const int F = kModalNT * kModalEPT - (items[i].nz + 2);
        const int S = (items[i].ny + 1) * (items[i].nz + 1);
        tiles[i] = (S + F - 1) / F;
        need += tiles[i];
        const int ext = std::max(items[i].nx, std::max(items[i].ny, items[i].nz));
        weight[i] = (double)items[i].nx * items[i].ny * items[i].nz * (share == 1 ? (double)ext : 1.0);
        wsum += weight[i];
    }
    if (need > total) return GBS_EINVAL;
    int used = 0;
    for (int i = 0; i < n; ++i) {
        int s = (int)((double)total * (weight[i] / wsum) / tiles[i]);
        s = s < 1 ? 1 : s;
        if (s > items[i].nx + 1) s = items[i].nx + 1;
        nseg[i] = s;
        used += tiles[i] * s;
    }
    while (used > total) {  // trim the design with the most segments
        int j = 0;
        for (int i = 1; i < n; ++i)
            if (nseg[i] > nseg[j]) j = i;
        if (nseg[j] <= 1) return GBS_EINVAL;
        nseg[j] -= 1;
        used -= tiles[j];
    }
    FusedTable &T = plan->T;
    memset(&T, 0, sizeof T);
    T.n = n;
    int block0 = 0;
    for (int i = 0; i < n; ++i) {
        const FusedItem &itm = items[i];
        seglen[i] = (itm.nx + 1 + nseg[i] - 1) / nseg[i];
        nseg[i] = (itm.nx + 1 + seglen[i] - 1) / seglen[i];
        FusedDesign &D = T.d[i];
        D.G = ModalGeom{itm.nx, itm.ny, itm.nz, nseg[i], seglen[i], 0};
        D.tiles = tiles[i];
        D.block0 = block0;
        D.nblk = tiles[i] * nseg[i];
        D.x = itm.w.E;  // the moduli of the design's setup
        D.mask = itm.mask;
        D.ca = cg_args(itm.w, itm.u);
        block0 += D.nblk;
        // the barrier writes two slots of three partial sums per CTA of the design
        if (6 * (size_t)D.nblk > itm.w.partial_count)
            return set_error(GBS_EINVAL, "fused PCG: a design's CTAs need more partial sums than its workspace holds");
    }
    plan->kern = kern;
    plan->smem = smem;
    plan->blocks = (unsigned)block0;
    return GBS_OK;
}

// Runs up to `budget` further PCG iterations (0: all that remain) of up to kMaxFused
// initialised designs in one cooperative launch (plan: fused_plan). A design that reaches the
// budget keeps `done` clear and resumes in the next launch; its barrier counter restarts here.
static int pcg_fused_batch(const gbsimp_ctx *ctx, const FusedItem *items, int n, const Law<float> &law,
                           cudaStream_t st, int budget = 0, int share = 0) {
    FusedPlan P;
    int rc = fused_plan(ctx, items, n, &P, share);
    if (rc) return rc;
    for (int i = 0; i < n; ++i)
        GBS_CUDA_TRY(cudaMemsetAsync(&items[i].w.sc->bar_count, 0, sizeof(unsigned), st));
    unsigned long long wait_ns = 2000000000ull;  // 2 s per barrier wait
    Law<float> lw = law;
    ModalK km = ctx->km;
    void *args[] = {&P.T, &lw, &km, &wait_ns, &budget};
    const cudaError_t e = cudaLaunchCooperativeKernel(P.kern, dim3(P.blocks), dim3(kModalNT), args, P.smem, st);
    if (e != cudaSuccess) {
        cudaGetLastError();  // a refused launch must not surface at the next launch check
        return set_error(GBS_EINVAL, "cooperative launch refused: %s", cudaGetErrorString(e));
    }
    count_launches(1);
    return GBS_OK;
}

// ---- device-driven PCG loop: one CUDA graph with a WHILE node ------------------------------
// Body: kLoopUnroll iterations (one kernel each, or K1 + K2 for the dense element) and a
// one-thread kernel that sets the loop condition from the device flag `done`. The iteration
// kernels return at once when done is set, so a finished solve costs at most kLoopUnroll-1
// empty iterations. The condition kernel also counts trips and stops
// the loop with GBS_ETIMEOUT after max_trips (set from max_iter), so the loop always ends.
constexpr int kLoopUnroll = 12;
static_assert(kLoopUnroll % 6 == 0, "a trip must end on launch phase 5 (parity 1, w index 2)");

static inline int launches_per_trip(const gbsimp_ctx *ctx, int nz) {
    return (use_modal(ctx, nz) ? 1 : 2) * kLoopUnroll + 1;
}

__global__ void pcg_loop_cond_kernel(cudaGraphConditionalHandle h, PcgScalars *sc) {
    const int trips = sc->trips + 1;
    sc->trips = trips;
    bool stop = sc->done != 0 || sc->st[1].done != 0;  // (a trip ends with a launch of parity 1)
    if (!stop && trips >= sc->max_trips) {
        sc->done = 1;
        sc->status = GBS_ETIMEOUT;
        stop = true;
    }
    // an iteration budget pauses the solve at a trip boundary (launch phase 5 done, so the
    // next launch of the same solve is phase 0 again); `done` stays clear
    if (!stop && sc->pause_trips > 0 && trips >= sc->pause_trips) stop = true;
    cudaGraphSetConditional(h, stop ? 0u : 1u);
}

// Before a graph-loop launch of a batched round: restarts the trip count (the cap max_trips
// then bounds every launch) and pauses after `trips` trips (0 = run to the end).
__global__ void pcg_set_pause_kernel(PcgScalars *sc, int trips) {
    sc->trips = 0;
    sc->pause_trips = trips;
}

struct GraphCache {
    std::mutex mu;
    std::unordered_map<std::string, cudaGraphExec_t> map;
    cudaStream_t cap = nullptr;  // private capture stream
};

void *graph_cache_create() { return new GraphCache(); }

void graph_cache_destroy(void *p) {
    GraphCache *gc = (GraphCache *)p;
    if (!gc) return;
    for (auto &kv : gc->map)
        if (kv.second) cudaGraphExecDestroy(kv.second);
    if (gc->cap) cudaStreamDestroy(gc->cap);
    delete gc;
}

struct LoopKey {
    const void *ws, *x, *mask, *u;
    int nx, ny, nz, kind;
    float penal, e0, emin, xmin;
    unsigned ke_version;
    int modal;
};

static int pcg_iteration(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                         const uint8_t *mask, float *u, const PcgWs &w, cudaStream_t st, cudaEvent_t after_k1,
                         int phase);

// Publishes the state after one-kernel PCG launches (last launch of parity `last`).
static int cg_publish(const gbsimp_ctx *ctx, int nx, int ny, int nz, const PcgWs &w, int last, cudaStream_t st) {
    if (!use_modal(ctx, nz)) return GBS_OK;
    const int nblk = modal_blocks<MODE_CG>(ctx, nx, ny, nz);
    if (nblk < 0) return -nblk;
    cg_fold_kernel<<<1, 256, 0, st>>>(nblk, last, w.partials, w.sc);
    GBS_LAUNCH_CHECK("cg_fold_kernel");
    return GBS_OK;
}

// Builds (or finds) the instantiated loop graph for this problem and buffer set and launches
// it on st, all under the cache's lock: another thread's eviction (the cache is emptied when
// full) can then never destroy a graph between its lookup and its launch, and CUDA defers
// the destruction of a graph that is still running. *built is false when no graph could be
// built (the error is returned; the caller may run the host loop instead).
static int launch_loop_graph(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                             const uint8_t *mask, float *u, const PcgWs &w, cudaStream_t st, bool *built) {
    *built = false;
    GraphCache *gc = (GraphCache *)ctx->graphs;
    if (!gc) return set_error(GBS_ECUDA, "no graph cache");
    const bool modal = use_modal(ctx, nz);
    LoopKey k;
    memset(&k, 0, sizeof k);
    k.ws = w.sc;
    k.x = x;
    k.mask = mask;
    k.u = u;
    k.nx = nx;
    k.ny = ny;
    k.nz = nz;
    k.kind = law.kind;
    k.penal = law.penal;
    k.e0 = law.e0;
    k.emin = law.emin;
    k.xmin = law.xmin;
    k.ke_version = ctx->ke_version;
    k.modal = modal ? 1 : 0;
    const std::string key((const char *)&k, sizeof k);
    std::lock_guard<std::mutex> lock(gc->mu);
    auto it = gc->map.find(key);
    if (it != gc->map.end()) {
        *built = true;
        GBS_CUDA_TRY(cudaGraphLaunch(it->second, st));
        return GBS_OK;
    }
    if (gc->map.size() >= 64) {
        for (auto &kv : gc->map) cudaGraphExecDestroy(kv.second);
        gc->map.clear();
    }
    if (modal) {
        const int r = modal_prepare<MODE_CG>(ctx, nz);
        if (r < 0) return -r;
    }
    if (!gc->cap) GBS_CUDA_TRY(cudaStreamCreateWithFlags(&gc->cap, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    GBS_CUDA_TRY(cudaGraphCreate(&g, 0));
    int rc = GBS_OK;
    cudaGraphExec_t exec = nullptr;
    do {
        cudaGraphConditionalHandle h;
        cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) {
            rc = cuda_error(e, "cudaGraphConditionalHandleCreate");
            break;
        }
        // cudaGraphNodeParams has a union with non-trivial members: zero-initialised storage.
        alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)] = {};
        cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(cp_buf);
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp);
        if (e != cudaSuccess) {
            rc = cuda_error(e, "cudaGraphAddNode(while)");
            break;
        }
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(gc->cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            rc = cuda_error(e, "cudaStreamBeginCaptureToGraph");
            break;
        }
        set_capturing(true);
        for (int i = 0; i < kLoopUnroll && rc == GBS_OK; ++i)
            rc = pcg_iteration(ctx, nx, ny, nz, law, x, mask, u, w, gc->cap, nullptr, i % 6);
        if (rc == GBS_OK) {
            pcg_loop_cond_kernel<<<1, 1, 0, gc->cap>>>(h, w.sc);
            e = cudaGetLastError();
            if (e != cudaSuccess) rc = cuda_error(e, "pcg_loop_cond_kernel");
        }
        set_capturing(false);
        cudaGraph_t captured = nullptr;
        e = cudaStreamEndCapture(gc->cap, &captured);
        if (rc == GBS_OK && e != cudaSuccess) rc = cuda_error(e, "cudaStreamEndCapture");
        if (rc != GBS_OK) break;
        e = cudaGraphInstantiate(&exec, g, 0);
        if (e != cudaSuccess) {
            rc = cuda_error(e, "cudaGraphInstantiate");
            exec = nullptr;
        }
    } while (0);
    cudaGraphDestroy(g);
    if (rc != GBS_OK) return rc;
    gc->map.emplace(key, exec);
    *built = true;
    GBS_CUDA_TRY(cudaGraphLaunch(exec, st));
    return GBS_OK;
}

// pcg_setup flags: the caller's start vector u is zero (q = 0, no apply), and the 1/diag in
// the workspace is already that of this x and mask (an earlier round of the same solve).
enum { SETUP_X0_ZERO = 1, SETUP_KEEP_DINV = 2 };

// 1/diag of K(x) on free DOFs and, for the modal kernels, the element moduli E(x_e).
static int setup_diag(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                      const uint8_t *mask, const PcgWs &w, cudaStream_t st) {
    const int64_t nd = n_dof_of(nx, ny, nz);
    dinv_kernel<float><<<ew_blocks(ctx, nd / 3), 256, 0, st>>>(nx, ny, nz, fast_div(ny + 1), fast_div(nz + 1), law,
                                                                 ctx->kef, x, mask, w.dinv);
    GBS_LAUNCH_CHECK("dinv_kernel");
    if (use_modal(ctx, nz)) {
        const int64_t ne = (int64_t)nx * ny * nz;
        moduli_f32_kernel<<<ew_blocks(ctx, ne), 256, 0, st>>>(ne, law, x, w.E);
        GBS_LAUNCH_CHECK("moduli_f32_kernel");
    }
    return GBS_OK;
}

// Start of a one-kernel PCG from x0 = 0 without a setup apply. r_0 = D b on free DOFs goes to
// the r buffer of the start pass (an odd launch, phase 5); x, p, the s it reads, the w it
// reads and the w it adds its output into are zeroed; the scalars are reset with the state
// marked CG_START_PASS. The start pass (alpha = beta = 0) then forms u_0 = M r_0,
// w_0 = D K D u_0 and the sums r_0.u_0, w_0.u_0, r_0.r_0, and the launch after it folds them
// into alpha_0 and the stop threshold (cg_first_step_df).
// The right-hand side is b, or with bdd given (h, l) pairs scaled by *bscale in FP32 (the
// outer residual r / ||r|| formed here instead of by a separate scale pass).
__global__ void cg_fresh_kernel(int64_t nd, const float *__restrict__ b, const float2 *__restrict__ bdd,
                                const double *bscale, const uint8_t *__restrict__ mask, float *r, float *p, float *sold,
                                float *w_in, float *w_out, float *x, PcgScalars *sc, double tol, int max_iter,
                                int max_trips) {
    const float bs = bdd ? (float)*bscale : 0.0f;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        float bv;
        if (bdd) {
            const float2 v = bdd[d];
            bv = fmaf(v.x, bs, v.y * bs);
        } else {
            bv = b[d];
        }
        r[d] = dof_fixed(mask, d) ? 0.0f : bv;
        p[d] = 0.0f;
        sold[d] = 0.0f;
        w_in[d] = 0.0f;
        w_out[d] = 0.0f;
        x[d] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        PcgScalars z = {};
        z.tol = tol;
        z.max_iter = max_iter;
        z.max_trips = max_trips;
        z.status = GBS_OK;
        z.st[0].pending = CG_START_PASS;
        z.st[0].status = GBS_OK;
        *sc = z;
    }
}


// PCG setup on the stream: zeroed scalars, 1/diag, q = D K D u, r = D b - q, then for the
// single-reduction form u_0 = M r_0, w_0 = D K D u_0 and alpha_0, for the dense form
// p_{-1} = 0; the first dot products and the stop test (nothing is read back).
static int pcg_setup(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *glaw, const float *x,
                     const float *b, const uint8_t *mask, float *u, double rtol, int max_iter, const PcgWs &w,
                     cudaStream_t st, unsigned flags = 0) {
    const int64_t nd = n_dof_of(nx, ny, nz);
    const Law<float> law = make_law<float>(*glaw);
    if (use_modal(ctx, nz)) {
        const int rc = check_modal_partials(ctx, nx, ny, nz, w);
        if (rc) return rc;
    }
    GBS_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(PcgScalars), st));
    if (!(flags & SETUP_KEEP_DINV)) {
        const int rc = setup_diag(ctx, nx, ny, nz, law, x, mask, w, st);
        if (rc) return rc;
    }
    const int max_trips = (max_iter + kLoopUnroll - 1) / kLoopUnroll + 2;
    // q = D K D u into `qbuf`, or zeros when u is known to be zero
    auto start_q = [&](float *qbuf) -> int {
        if (flags & SETUP_X0_ZERO) {
            GBS_CUDA_TRY(cudaMemsetAsync(qbuf, 0, (size_t)nd * sizeof(float), st));
            return GBS_OK;
        }
        return apply_f32(ctx, nx, ny, nz, glaw, x, u, qbuf, mask, st);
    };
    if (use_modal(ctx, nz)) {
        const CgArgs ca = cg_args(w, u);
        const int x0_zero = (flags & SETUP_X0_ZERO) ? 1 : 0;
        if (!x0_zero) {
            const int rc = start_q(ca.w[1]);
            if (rc) return rc;
        }
        cg_init_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, b, ca.w[1], mask, w.dinv, ca.r[0], ca.p, ca.s[1], u,
                                                           w.partials, w.sc, rtol, max_iter, max_trips, x0_zero);
        GBS_LAUNCH_CHECK("cg_init_kernel");
        int rc = apply_f32(ctx, nx, ny, nz, glaw, x, ca.w[1], ca.w[0], mask, st);
        if (rc) return rc;
        cg_start_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, ca.w[0], ca.w[1], w.partials, w.sc);
        GBS_LAUNCH_CHECK("cg_start_kernel");
        // u_0 in w[1] is no longer needed: the first launch adds its output into w[1] on the
        // segments' shared node planes, so w[1] starts at zero
        GBS_CUDA_TRY(cudaMemsetAsync(ca.w[1], 0, (size_t)nd * sizeof(float), st));
        return GBS_OK;
    }
    int rc = start_q(w.ap);
    if (rc) return rc;
    pcg_init_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, b, w.ap, mask, w.dinv, w.r, w.p1, u, w.partials, w.sc, rtol,
                                                        max_iter, max_trips);
    GBS_LAUNCH_CHECK("pcg_init_kernel");
    return GBS_OK;
}

// Whether pcg_run starts this solve with pcg_fresh_setup.
static inline bool fresh_start_ok(const gbsimp_ctx *ctx, int nz, int fused, int max_iter, unsigned flags) {
    return use_modal(ctx, nz) && (flags & SETUP_X0_ZERO) && !fused && max_iter > 0;
}

// pcg_setup for the one-kernel PCG from x0 = 0 (max_iter > 0): cg_fresh_kernel and the start
// pass, two launches instead of the setup's reductions and apply.
static int pcg_fresh_setup(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *glaw, const float *x,
                           const float *b, const float2 *bdd, const double *bscale, const uint8_t *mask, float *u,
                           double rtol, int max_iter, const PcgWs &w, cudaStream_t st, unsigned flags) {
    const int64_t nd = n_dof_of(nx, ny, nz);
    const Law<float> law = make_law<float>(*glaw);
    int rc = check_modal_partials(ctx, nx, ny, nz, w);
    if (rc) return rc;
    if (!(flags & SETUP_KEEP_DINV)) {
        rc = setup_diag(ctx, nx, ny, nz, law, x, mask, w, st);
        if (rc) return rc;
    }
    const int max_trips = (max_iter + kLoopUnroll - 1) / kLoopUnroll + 2;
    const CgArgs ca = cg_args(w, u);
    // phase 5 reads r[1], s[0], w[2] and adds into w[0] (the launch that precedes phase 0)
    cg_fresh_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, b, bdd, bscale, mask, ca.r[1], ca.p, ca.s[0], ca.w[2],
                                                         ca.w[0], u, w.sc, rtol, max_iter, max_trips);
    GBS_LAUNCH_CHECK("cg_fresh_kernel");
    return pcg_iteration(ctx, nx, ny, nz, law, x, mask, u, w, st, nullptr, 5);
}

// Optional profiling (prof != nullptr): CUDA events around every K1 launch; only the
// launches of iterations that actually ran (the device counter advanced) are summed.
struct ApplyProfile {
    double seconds = 0.0;
    int launches = 0;
};

// FP32 PCG. u: x0 in, solution out. Returns GBS_OK and fills *out (status inside).
// With out == nullptr (and no profiling) the solve is only enqueued: the device-driven paths
// need no host decision, and the caller reads the scalars later (w.sc of the workspace),
// together with its own.
int pcg_run(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *glaw, const float *x, const float *b,
            const uint8_t *mask, float *u, double rtol, int max_iter, int check_every, void *ws, PcgScalars *out,
            cudaStream_t st, ApplyProfile *prof = nullptr, int fused = 0, unsigned setup_flags = 0,
            const float2 *bdd = nullptr, const double *bscale = nullptr, bool *finish_left = nullptr) {
    const int64_t nd = n_dof_of(nx, ny, nz);
    PcgWs w = pcg_ws(ws, nx, ny, nz);
    const Law<float> law = make_law<float>(*glaw);
    // from x0 = 0 the one-kernel form starts with a start pass instead of the setup's apply
    // (the persistent kernel keeps the setup: it reads the scalars of iteration 0); only this
    // start takes the right-hand side as scaled (h, l) pairs
    const bool fresh = fresh_start_ok(ctx, nz, fused, max_iter, setup_flags);
    if (bdd && !fresh) return set_error(GBS_EINVAL, "pcg_run: a (h, l) right-hand side needs the fresh start");
    int rc = fresh ? pcg_fresh_setup(ctx, nx, ny, nz, glaw, x, b, bdd, bscale, mask, u, rtol, max_iter, w, st,
                                     setup_flags)
                   : pcg_setup(ctx, nx, ny, nz, glaw, x, b, mask, u, rtol, max_iter, w, st, setup_flags);
    if (rc) return rc;
    PcgScalars h;
    memset(&h, 0, sizeof h);
    const bool async = out == nullptr && !prof;
    if (!async) {
        rc = read_scalars(w.sc, &h, st);  // a solve that is done at setup skips the loops
        if (rc) return rc;
    }
    if (!prof && !h.done && fused) {
        const FusedItem item{nx, ny, nz, x, mask, u, w};
        if (pcg_fused_batch(ctx, &item, 1, law, st) == GBS_OK) {
            pcg_finalize_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, w.p0, w.p1, u, w.sc, 0);
            GBS_LAUNCH_CHECK("pcg_finalize_kernel");
            if (async) return GBS_OK;
            rc = read_scalars(w.sc, &h, st);
            if (rc) return rc;
            *out = h;
            return GBS_OK;
        }
        // the grid cannot be co-resident here: use the graph loop
    }
    if (!prof && !h.done) {
        bool built = false;
        const int lrc = launch_loop_graph(ctx, nx, ny, nz, law, x, mask, u, w, st, &built);
        if (built) {
            if (lrc) return lrc;  // the launch itself failed
            if (finish_left && async && use_modal(ctx, nz)) {
                // the caller publishes, finalizes and applies the correction in one pass
                *finish_left = true;
                return GBS_OK;
            }
            rc = cg_publish(ctx, nx, ny, nz, w, 1, st);
            if (rc) return rc;
            pcg_finalize_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, w.p0, w.p1, u, w.sc, use_modal(ctx, nz) ? 2 : 1);
            GBS_LAUNCH_CHECK("pcg_finalize_kernel");
            if (async) return GBS_OK;  // the caller counts the loop's launches from the scalars
            rc = read_scalars(w.sc, &h, st);
            if (rc) return rc;
            count_launches(h.trips * launches_per_trip(ctx, nz));
            *out = h;
            return GBS_OK;
        }
        // graph construction failed: fall through to host-launched iterations
    }
    if (async) {  // the host loop decides from the scalars
        rc = read_scalars(w.sc, &h, st);
        if (rc) return rc;
    }
    int chunk = check_every > 0 ? check_every : 16;
    const int max_chunk = check_every > 0 ? check_every : 128;
    std::vector<cudaEvent_t> ev;
    if (prof) {
        ev.resize(2 * (size_t)max_chunk);
        for (auto &e : ev) GBS_CUDA_TRY(cudaEventCreate(&e));
    }
    int launched = 0;
    while (!h.done && launched < max_iter) {
        const int n = (launched + chunk > max_iter) ? (max_iter - launched) : chunk;
        const int it0 = h.iter;
        for (int i = 0; i < n; ++i) {
            if (prof) GBS_CUDA_TRY(cudaEventRecord(ev[2 * i], st));
            rc = pcg_iteration(ctx, nx, ny, nz, law, x, mask, u, w, st, prof ? ev[2 * i + 1] : nullptr,
                               (launched + i) % 6);
            if (rc) return rc;
        }
        launched += n;
        rc = cg_publish(ctx, nx, ny, nz, w, (launched - 1) & 1, st);
        if (rc) return rc;
        rc = read_scalars(w.sc, &h, st);
        if (rc) return rc;
        if (prof) {
            int ran = h.iter - it0;
            // dense form: on breakdown K1 ran without K2
            if (!use_modal(ctx, nz) && (h.status == GBS_EBREAKDOWN || h.status == GBS_ENONFINITE)) ++ran;
            for (int i = 0; i < ran && i < n; ++i) {
                float ms = 0.0f;
                GBS_CUDA_TRY(cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]));
                prof->seconds += 1e-3 * ms;
                prof->launches += 1;
            }
        }
        if (check_every <= 0 && chunk < max_chunk) chunk *= 2;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    pcg_finalize_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, w.p0, w.p1, u, w.sc, use_modal(ctx, nz) ? 2 : 1);
    GBS_LAUNCH_CHECK("pcg_finalize_kernel");
    rc = read_scalars(w.sc, &h, st);
    if (rc) return rc;
    *out = h;
    return GBS_OK;
}

// ---- FP64 outer defect correction ---------------------------------------------------------
struct OuterScalars {
    double ff;      // ||D f||^2
    double rr;      // ||D(f - K u)||^2
    double scale;   // 1/||r|| used to form the FP32 right-hand side
    double rnorm;   // ||r||, the factor of the correction
    unsigned counter;
    float sigma;    // double-float residual: a power of two near 1/||D f||; FP32 sums of squares
                    // run on sigma r, which keeps them clear of the FP32 range limits
};

struct SolveWs {
    OuterScalars *os;
    double *r64;
    float *b32, *d32;
    double *partials;
    void *pcg;
    double *elem;  // 24 * n_elem corner contributions of the modal residual (FP64 or (h, l) float2)
    float2 *udd;   // double-float split of u (double-float residual)
    float2 *fdd;   // and of D f
};

static size_t solve_ws_bytes_impl(int nx, int ny, int nz) {
    const size_t nd = (size_t)n_dof_of(nx, ny, nz);
    return 256 + al256(sizeof(OuterScalars)) + al256(nd * 8) + 2 * al256(nd * 4) + al256(3 * 4096 * 8) +
           al256(pcg_ws_bytes_impl(nx, ny, nz)) + al256(apply_f64_modal_ws_bytes(nx, ny, nz)) + 2 * al256(nd * 8);
}

static SolveWs solve_ws(void *ws, int nx, int ny, int nz) {
    const size_t nd = (size_t)n_dof_of(nx, ny, nz);
    char *p = align256(ws);
    SolveWs w;
    w.os = (OuterScalars *)p;
    p += al256(sizeof(OuterScalars));
    w.r64 = (double *)p;
    p += al256(nd * 8);
    w.b32 = (float *)p;
    p += al256(nd * 4);
    w.d32 = (float *)p;
    p += al256(nd * 4);
    w.partials = (double *)p;
    p += al256(3 * 4096 * 8);
    w.pcg = p;
    p += al256(pcg_ws_bytes_impl(nx, ny, nz));
    w.elem = (double *)p;
    p += al256(apply_f64_modal_ws_bytes(nx, ny, nz));
    w.udd = (float2 *)p;
    p += al256(nd * 8);
    w.fdd = (float2 *)p;
    return w;
}

// The outer residual runs in double-float (modal_dd.cuh) for tolerances down to this one: its
// rounding, measured at most 6.1e-13 ||f|| on converged fields (32x16x16, 64^3), stays three
// orders of magnitude below. Tighter tolerances take the FP64 element pass.
constexpr double kDdMinRtol = 1e-9;
// The inner PCG's reduction per outer round when the options leave it at 0 (engine.INNER_RTOL).
constexpr double kInnerRtol = 3e-5;
static bool use_dd_residual(const gbsimp_ctx *ctx, const gbsimp_solve_opts *o) {
    return ctx->modal_ok && o->rtol >= kDdMinRtol && !o->residual_fp64;
}

// r = D f - q (q = D K D u); ||r||^2, ||D f||^2 -> os.
__global__ void resid64_kernel(int64_t nd, const double *__restrict__ f, const double *__restrict__ q,
                               const uint8_t *__restrict__ mask, double *r, double *partials, OuterScalars *os) {
    double rr = 0.0, ff = 0.0;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        const bool fx = dof_fixed(mask, d);
        const double fd = fx ? 0.0 : f[d];
        const double rd = fx ? 0.0 : fd - q[d];
        r[d] = rd;
        rr = fma(rd, rd, rr);
        ff = fma(fd, fd, ff);
    }
    __shared__ double tot[3];
    if (last_block3(rr, ff, 0.0, partials, &os->counter, tot) && threadIdx.x == 0) {
        os->rr = tot[0];
        os->ff = tot[1];
        os->rnorm = sqrt(tot[0]);
        os->scale = tot[0] > 0.0 ? 1.0 / sqrt(tot[0]) : 0.0;
    }
}

// The node pass of the double-float residual: q_n = the (up to) 8 corner contributions of the
// element pass summed in the fixed order b = 0..7 (double-float), then r = D(f - q) in FP64
// and ||r||^2, ||D f||^2 -> os.
// Once per solve, before the first double-float residual: fdd = the split of D f, and
// ||D f||^2 (FP64, from f itself) with sigma = 2^-round(log2 ||D f||); udd = the split of the
// start vector u (fixed DOFs zero).
__global__ void split_f_kernel(int64_t nd, const double *__restrict__ f, const uint8_t *__restrict__ mask, float2 *fdd,
                               double *partials, OuterScalars *os, const double *__restrict__ u, float2 *udd) {
    double ff = 0.0;
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < nd; d += (int64_t)gridDim.x * blockDim.x) {
        const bool fx = dof_fixed(mask, d);
        const double v = fx ? 0.0 : f[d];
        const ddv s = fx ? ddv{0.0f, 0.0f} : dd_split(v);
        fdd[d] = make_float2(s.h, s.l);
        ff = fma(v, v, ff);
        const ddv us = fx ? ddv{0.0f, 0.0f} : dd_split(u[d]);
        udd[d] = make_float2(us.h, us.l);
    }
    __shared__ double tot[3];
    const ddv fs = dd_split(ff);  // the thread's FP64 partial, summed on in double-float
    if (last_block3_df(df32{fs.h, fs.l}, df32{0.0f, 0.0f}, df32{0.0f, 0.0f}, (float2 *)partials, &os->counter, tot) &&
        threadIdx.x == 0) {
        os->ff = tot[0];
        int e = 0;
        if (tot[0] > 0.0 && isfinite(tot[0])) frexp(sqrt(tot[0]), &e);
        e = e < -120 ? -120 : (e > 120 ? 120 : e);
        os->sigma = ldexpf(1.0f, -e);
    }
}

__global__ void __launch_bounds__(256) resid_dd_kernel(int nx, int ny, int nz, const FastDiv fNY, const FastDiv fNZ,
                                                       const float2 *__restrict__ C,
                                                       const uint8_t *__restrict__ mask, const float2 *__restrict__ fdd,
                                                       float2 *r, double *partials, OuterScalars *os) {
    const int64_t NY = ny + 1, NZ = nz + 1;
    const int64_t n_nodes = (int64_t)(nx + 1) * NY * NZ;
    const int64_t n_elem = (int64_t)nx * ny * nz;
    const float sigma = os->sigma;
    float rr = 0.0f;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < n_nodes; n += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten3((uint32_t)n, fNY, fNZ, i, j, k);
        // all 24 loads first (zero outside the grid: adding an exact zero leaves a pair as it
        // is), then the sums in the fixed order b = 0..7
        float2 w[8][3];
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const int ei = i - (b >> 2), ej = j - ((b >> 1) & 1), ek = k - (b & 1);
            const bool in = ei >= 0 && ej >= 0 && ek >= 0 && ei < nx && ej < ny && ek < nz;
            const int64_t e = in ? ((int64_t)ei * ny + ej) * nz + ek : 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) w[b][c] = in ? __ldg(&C[(b * 3 + c) * n_elem + e]) : make_float2(0.0f, 0.0f);
        }
        const uint8_t m = mask ? mask[n] : (uint8_t)0;
        ddv acc[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll
        for (int b = 0; b < 8; ++b)
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] = dd_add(acc[c], ddv{w[b][c].x, w[b][c].y});
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const bool fx = (m >> c) & 1;
            const float2 fv = fdd[3 * n + c];
            const ddv rd = fx ? ddv{0.0f, 0.0f} : dd_add(ddv{fv.x, fv.y}, ddv{-acc[c].h, -acc[c].l});
            r[3 * n + c] = make_float2(rd.h, rd.l);
            // both parts: near convergence f and q agree in their leading parts and r lives in l
            const float rs = __fmul_rn(__fadd_rn(rd.h, rd.l), sigma);
            rr = fmaf(rs, rs, rr);
        }
    }
    __shared__ double tot[3];
    if (last_block3_df(rr, 0.0f, 0.0f, (float2 *)partials, &os->counter, tot) && threadIdx.x == 0) {
        const double s2 = (double)sigma * (double)sigma;
        os->rr = tot[0] / s2;
        os->rnorm = sqrt(tot[0]) / (double)sigma;
        os->scale = tot[0] > 0.0 ? (double)sigma / sqrt(tot[0]) : 0.0;
    }
}

// b = r / ||r|| in FP32 from the double-float residual.
__global__ void scale_dd_kernel(int64_t nd, const float2 *__restrict__ r, const OuterScalars *os, float *b) {
    const float s = (float)os->scale;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = r[i];
        b[i] = fmaf(v.x, s, v.y * s);
    }
}

// u += ||r|| d (one FP64 fma), fixed DOFs zero, and its double-float split for the next
// residual (integer conversions: f2d, dd_split).
__global__ void correct_dd_kernel(int64_t nd, const float *__restrict__ d, const OuterScalars *os,
                                  const uint8_t *__restrict__ mask, double *u, float2 *udd) {
    const double s = os->rnorm;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        const bool fx = dof_fixed(mask, i);
        const double v = fx ? 0.0 : fma(f2d(d[i]), s, u[i]);
        u[i] = v;
        const ddv w = fx ? ddv{0.0f, 0.0f} : dd_split(v);
        udd[i] = make_float2(w.h, w.l);
    }
}

// After a graph loop of one-kernel PCG launches that ended on launch parity `last`:
// cg_fold_kernel, pcg_finalize_kernel (one-kernel form) and correct_dd_kernel in one pass.
// Every block reads the state once and folds pending sums itself (the same totals in every
// block); block 0 publishes the host-visible fields. No block writes the state slot, and the
// done and status merges give the same value whether a block reads those fields before or after
// block 0 has written them. Each DOF then takes x's owed half step (finalize) and
// u += ||r|| x in FP64 with its split (correct).
__global__ void cg_finish_dd_kernel(int64_t nd, int nblk, int last, const double *partials, PcgScalars *sc,
                                    const float *__restrict__ p0, const float *__restrict__ xu,
                                    const OuterScalars *os, const uint8_t *__restrict__ mask, double *u,
                                    float2 *udd) {
    __shared__ float2 sred[3 * 32];
    __shared__ CgState s_state;
    __shared__ int s_done, s_status;
    __shared__ double s_bnorm;
    if (threadIdx.x == 0) s_state = sc->st[last];
    __syncthreads();
    CgState s = s_state;
    const int pend = s.pending;
    if ((pend == CG_PENDING_STEP || pend == CG_PENDING_FIRST) && !s.done)  // block-uniform
        cg_fold<256>(s, sc, (const float2 *)partials + last * 3 * nblk, nblk, sred);
    if (threadIdx.x == 0) {
        const int st0 = sc->status;
        s_status = st0 == GBS_OK ? s.status : st0;
        s_done = (sc->done || s.done) ? 1 : 0;
        s_bnorm = pend == CG_PENDING_FIRST ? sqrt(df_value(s.rr)) : sc->bnorm;
    }
    __syncthreads();
    const int status = s_status, done = s_done;
    const double bnorm = s_bnorm;
    const double a1 = df_value(s.done ? s.alpha : s.alpha_prev);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (pend == CG_PENDING_FIRST) sc->bnorm = bnorm;
        sc->iter = s.iter;
        sc->rz = df_value(s.gamma);
        sc->rr = df_value(s.rr);
        sc->pap = df_value(s.pap);
        sc->alpha[0] = df_value(s.alpha);
        sc->alpha[1] = a1;
        sc->beta = df_value(s.beta);
        sc->status = status;
        sc->done = done;
    }
    // pcg_finalize_kernel, one-kernel form: x = 0 when D b = 0; when the last launched
    // iteration was even (iter odd) x still owes alpha p of it
    const bool zero = bnorm == 0.0;
    const bool owe = done && !zero && (s.iter & 1) && status != GBS_ENONFINITE;
    const float a = (float)a1;
    const double rn = os->rnorm;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = (done && zero) ? 0.0f : (owe ? fmaf(a, p0[i], xu[i]) : xu[i]);
        const bool fx = dof_fixed(mask, i);
        const double v = fx ? 0.0 : fma(f2d(d), rn, u[i]);
        u[i] = v;
        const ddv w = fx ? ddv{0.0f, 0.0f} : dd_split(v);
        udd[i] = make_float2(w.h, w.l);
    }
}

__global__ void scale_to_f32_kernel(int64_t nd, const double *__restrict__ r, const OuterScalars *os, float *b,
                                    float *d) {
    const double s = os->scale;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x) {
        b[i] = (float)(r[i] * s);
        d[i] = 0.0f;
    }
}

__global__ void correct64_kernel(int64_t nd, const float *__restrict__ d, const OuterScalars *os,
                                 const uint8_t *__restrict__ mask, double *u) {
    const double s = os->rnorm;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nd; i += (int64_t)gridDim.x * blockDim.x)
        u[i] = dof_fixed(mask, i) ? 0.0 : fma((double)d[i], s, u[i]);
}

// The outer residual of u into w.r64 and w.os: double-float element products (udd current) or
// the FP64 element pass.
static int outer_residual(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                          const double *f, const uint8_t *mask, const double *u, bool dd, const SolveWs &w,
                          cudaStream_t st) {
    const int64_t nd = n_dof_of(nx, ny, nz);
    int rc;
    if (dd) {
        rc = elem_dd_modal(ctx, nx, ny, nz, law, x, w.udd, (float2 *)w.elem, st);
        if (rc) return rc;
        resid_dd_kernel<<<vec_blocks(ctx, nd / 3), 256, 0, st>>>(nx, ny, nz, fast_div(ny + 1), fast_div(nz + 1),
                                                                  (const float2 *)w.elem, mask, w.fdd,
                                                                  (float2 *)w.r64, w.partials, w.os);
        GBS_LAUNCH_CHECK("resid_dd_kernel");
        return GBS_OK;
    }
    rc = ctx->modal_ok ? apply_f64_modal(ctx, nx, ny, nz, law, x, u, w.r64, mask, w.elem, st)
                       : apply_f64(ctx, nx, ny, nz, law, x, u, w.r64, mask, st);
    if (rc) return rc;
    // resid64 reads q from r64 and overwrites it in place (element-wise, same index).
    resid64_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, f, w.r64, mask, w.r64, w.partials, w.os);
    GBS_LAUNCH_CHECK("resid64_kernel");
    return GBS_OK;
}

// u += d / scale, and with the double-float residual the split of the new u.
static int outer_correct(const gbsimp_ctx *ctx, int64_t nd, const uint8_t *mask, double *u, bool dd,
                         const SolveWs &w, cudaStream_t st) {
    if (dd) {
        correct_dd_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, w.d32, w.os, mask, u, w.udd);
        GBS_LAUNCH_CHECK("correct_dd_kernel");
    } else {
        correct64_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, w.d32, w.os, mask, u);
        GBS_LAUNCH_CHECK("correct64_kernel");
    }
    return GBS_OK;
}

// Before the first residual of a solve: the double-float splits of u and D f, ||D f||^2 (one
// pass).
static int outer_start(const gbsimp_ctx *ctx, int64_t nd, const double *u, const double *f, const uint8_t *mask,
                       bool dd, const SolveWs &w, cudaStream_t st) {
    if (!dd) return GBS_OK;
    split_f_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, f, mask, w.fdd, w.partials, w.os, u, w.udd);
    GBS_LAUNCH_CHECK("split_f_kernel");
    return GBS_OK;
}

// The FP32 right-hand side b32 = r / ||r|| of the next inner solve (its x0 = 0 is written by
// the PCG setup).
static int outer_scale(const gbsimp_ctx *ctx, int64_t nd, bool dd, const SolveWs &w, cudaStream_t st) {
    if (dd) {
        scale_dd_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, (const float2 *)w.r64, w.os, w.b32);
        GBS_LAUNCH_CHECK("scale_dd_kernel");
    } else {
        scale_to_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, w.r64, w.os, w.b32, w.d32);
        GBS_LAUNCH_CHECK("scale_to_f32_kernel");
    }
    return GBS_OK;
}

// One host read per defect-correction round: the outer scalars and, when a PCG ran since the
// last read, its scalars.
static int read_outer(const OuterScalars *d, OuterScalars *h, const PcgScalars *dp, PcgScalars *hpcg,
                      cudaStream_t st) {
    char *hp = (char *)thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "no pinned staging buffer");
    static_assert(sizeof(OuterScalars) <= 2048 && sizeof(PcgScalars) <= 2048, "pinned staging layout");
    GBS_CUDA_TRY(cudaMemcpyAsync(hp, d, sizeof(OuterScalars), cudaMemcpyDeviceToHost, st));
    if (dp) GBS_CUDA_TRY(cudaMemcpyAsync(hp + 2048, dp, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    GBS_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(h, hp, sizeof(OuterScalars));
    if (dp) memcpy(hpcg, hp + 2048, sizeof(PcgScalars));
    return GBS_OK;
}

int solve_run(const gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x, const double *f,
              const uint8_t *mask, double *u, const gbsimp_solve_opts *o, gbsimp_solve_stats *stats, void *ws,
              cudaStream_t st) {
    ApplyProfile prof;
    const int64_t nd = n_dof_of(nx, ny, nz);
    SolveWs w = solve_ws(ws, nx, ny, nz);
    GBS_CUDA_TRY(cudaMemsetAsync(w.os, 0, sizeof(OuterScalars), st));
    const unsigned vb = vec_blocks(ctx, nd);
    int total = 0, outer = 0, status = GBS_OK;
    double relres = 0.0;
    const int max_outer = o->max_outer > 0 ? o->max_outer : 20;
    const double inner = o->inner_rtol > 0.0 ? o->inner_rtol : kInnerRtol;
    // Each round: FP64 residual -> one host read (the outer scalars and the previous round's
    // PCG scalars) -> the decisions -> the inner PCG and the correction, enqueued without a
    // host read (the graph loop and the persistent kernel are device-driven).
    const bool async = !o->profile;
    const PcgScalars *pending = nullptr;
    const PcgWs pw = pcg_ws(w.pcg, nx, ny, nz);
    const bool dd = use_dd_residual(ctx, o);
    {
        int rc = outer_start(ctx, nd, u, f, mask, dd, w, st);
        if (rc) return rc;
    }
    for (;;) {
        OuterScalars h;
        PcgScalars ps;
        {
            NvtxRange range("outer residual");
            int rc = outer_residual(ctx, nx, ny, nz, law, x, f, mask, u, dd, w, st);
            if (rc) return rc;
            rc = read_outer(w.os, &h, pending, &ps, st);
            if (rc) return rc;
        }
        int rc = GBS_OK;
        ++outer;
        if (pending) {
            pending = nullptr;
            total += ps.iter;
            count_launches(ps.trips * launches_per_trip(ctx, nz));  // graph loop trips (0 for the persistent kernel)
            // a failed inner solve ends the loop; its correction (zero when it made no step)
            // is in u and the residual above is the one of the corrected u
            if (ps.status == GBS_EBREAKDOWN || ps.status == GBS_ENONFINITE || ps.status == GBS_ETIMEOUT)
                status = ps.status;
        }
        if (!isfinite(h.rr) || !isfinite(h.ff)) {
            status = GBS_ENONFINITE;
            break;
        }
        if (h.ff == 0.0) {
            GBS_CUDA_TRY(cudaMemsetAsync(u, 0, nd * sizeof(double), st));
            relres = 0.0;
            break;
        }
        relres = sqrt(h.rr / h.ff);
        if (status != GBS_OK) break;
        if (relres <= o->rtol) break;
        if (outer > max_outer || total >= o->max_iter) {
            status = GBS_ENOTCONV;
            break;
        }
        // the first round computes 1/diag, later rounds reuse it
        const unsigned flags = SETUP_X0_ZERO | (outer > 1 ? SETUP_KEEP_DINV : 0u);
        // the fresh start forms b = r / ||r|| itself from the double-float residual
        const bool scaled_in_start = dd && fresh_start_ok(ctx, nz, o->fused, o->max_iter - total, flags);
        if (!scaled_in_start) {
            rc = outer_scale(ctx, nd, dd, w, st);
            if (rc) return rc;
        }
        // Inner tolerance: enough to reach rtol from here, but not below what FP32 resolves.
        double itol = o->rtol / relres;
        if (itol < inner) itol = inner;
        // with the double-float residual the graph loop's publish, finalize and the correction
        // run as one pass (cg_finish_dd_kernel)
        bool finish_left = false;
        {
            NvtxRange range("inner PCG");
            rc = pcg_run(ctx, nx, ny, nz, law, x, w.b32, mask, w.d32, itol, o->max_iter - total, o->check_every, w.pcg,
                         async ? nullptr : &ps, st, o->profile ? &prof : nullptr, o->fused, flags,
                         scaled_in_start ? (const float2 *)w.r64 : nullptr, scaled_in_start ? &w.os->scale : nullptr,
                         dd ? &finish_left : nullptr);
        }
        if (rc) return rc;
        if (async) {
            pending = pw.sc;
        } else {
            total += ps.iter;
            if (ps.status == GBS_EBREAKDOWN || ps.status == GBS_ENONFINITE || ps.status == GBS_ETIMEOUT) {
                status = ps.status;
                if (ps.iter == 0) break;
            }
        }
        if (finish_left) {
            const int nblk = modal_blocks<MODE_CG>(ctx, nx, ny, nz);
            if (nblk < 0) return -nblk;
            // every block folds the ~300 partial sums itself: vec_blocks' cap (8 blocks per SM)
            // keeps those redundant reads small
            cg_finish_dd_kernel<<<vec_blocks(ctx, nd), 256, 0, st>>>(nd, nblk, 1, pw.partials, pw.sc, pw.p0, w.d32,
                                                                     w.os, mask, u, w.udd);
            GBS_LAUNCH_CHECK("cg_finish_dd_kernel");
        } else {
            rc = outer_correct(ctx, nd, mask, u, dd, w, st);
            if (rc) return rc;
        }
        if (status != GBS_OK) break;
    }
    if (stats) {
        stats->status = status;
        stats->iterations = total;
        stats->outer = outer;
        stats->relres = relres;
        stats->apply_seconds = prof.seconds;
        stats->apply_launches = prof.launches;
    }
    return GBS_OK;
}

// ---- warm start of a SIMP loop's next solve ---------------------------------------------------
__global__ void warm_start_kernel(int64_t n, double *__restrict__ u, double *__restrict__ up, double theta) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double t = u[i];
        u[i] = fma(theta, t - up[i], t);
        up[i] = t;
    }
}

int warm_start_impl(const gbsimp_ctx *ctx, int64_t n, double *u, double *u_prev, double theta, cudaStream_t st) {
    if (n <= 0) return GBS_OK;
    warm_start_kernel<<<ew_blocks(ctx, n), 256, 0, st>>>(n, u, u_prev, theta);
    GBS_LAUNCH_CHECK("warm_start_kernel");
    return GBS_OK;
}

// ---- CSR Jacobi-PCG (pcg_solve_cuda contract) -------------------------------------------------
struct CsrScalars {
    double rz, rr, bnorm, alpha, beta, pap;
    int iter, done, status, max_iter;
    double tol;
    unsigned counter;
    int pad;
};

// Warp per row.
__global__ void csr_spmv_kernel(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                                const float *__restrict__ v, const float *__restrict__ p, float *y) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < n; row += nw) {
        const int32_t b = rp[row], e = rp[row + 1];
        float s = 0.0f;
        for (int32_t k = b + lane; k < e; k += 32) {
            const int32_t c = ci[k];
            if (c >= 0 && c < n) s = fmaf(v[k], p[c], s);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) y[row] = s;
    }
}

__global__ void zero_list_kernel(int64_t m, const int32_t *__restrict__ idx, int64_t n, float *v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = idx[i];
        if (d >= 0 && d < n) v[d] = 0.0f;
    }
}

__global__ void csr_init_kernel(int64_t n, const float *__restrict__ b, const float *__restrict__ q, float *r,
                                double *partials, CsrScalars *sc) {
    double bb = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        r[i] = b[i] - q[i];
        bb += (double)b[i] * (double)b[i];
    }
    __shared__ double tot[3];
    if (last_block3(bb, 0.0, 0.0, partials, &sc->counter, tot) && threadIdx.x == 0) sc->bnorm = sqrt(tot[0]);
}

__global__ void csr_z_kernel(int64_t n, const float *__restrict__ r, const float *__restrict__ diag, float *z,
                             float *p, int set_p, double *partials, CsrScalars *sc) {
    if (!set_p && sc->done) return;
    double rz = 0.0;
    const float beta = set_p ? 0.0f : (float)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float zi = diag[i] != 0.0f ? r[i] / diag[i] : 0.0f;  // a zero diagonal entry (fixed row) gives z = 0
        z[i] = zi;
        rz += (double)r[i] * (double)zi;
    }
    __shared__ double tot[3];
    if (last_block3(rz, 0.0, 0.0, partials, &sc->counter, tot) && threadIdx.x == 0) {
        if (set_p) {
            sc->rz = tot[0];
        } else {
            sc->beta = tot[0] / sc->rz;
            sc->rz = tot[0];
        }
    }
    (void)p;
    (void)beta;
}

__global__ void csr_p_kernel(int64_t n, const float *__restrict__ z, float *p, int first, const CsrScalars *sc) {
    if (!first && sc->done) return;
    const float beta = first ? 0.0f : (float)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = first ? z[i] : fmaf(beta, p[i], z[i]);
}

__global__ void csr_pap_kernel(int64_t n, const float *__restrict__ p, const float *__restrict__ ap, double *partials,
                               CsrScalars *sc) {
    if (sc->done) return;
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)p[i] * (double)ap[i];
    __shared__ double tot[3];
    if (last_block3(s, 0.0, 0.0, partials, &sc->counter, tot) && threadIdx.x == 0) {
        sc->pap = tot[0];
        if (fabs(tot[0]) < 1e-30 || !isfinite(tot[0])) {  // simp_pcg_cuda.cu:102
            sc->done = 1;
            sc->status = isfinite(tot[0]) ? GBS_EBREAKDOWN : GBS_ENONFINITE;
        } else {
            sc->alpha = sc->rz / tot[0];
        }
    }
}

__global__ void csr_xr_kernel(int64_t n, const float *__restrict__ p, const float *__restrict__ ap, float *x, float *r,
                              const int32_t *__restrict__ fixed, int64_t n_fixed, CsrScalars *sc) {
    if (sc->done) return;
    const float a = (float)sc->alpha;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fmaf(a, p[i], x[i]);
        r[i] = fmaf(-a, ap[i], r[i]);
    }
    (void)fixed;
    (void)n_fixed;
}

__global__ void csr_check_kernel(int64_t n, const float *__restrict__ r, double *partials, CsrScalars *sc) {
    if (sc->done) return;
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)r[i] * (double)r[i];
    __shared__ double tot[3];
    if (last_block3(s, 0.0, 0.0, partials, &sc->counter, tot) && threadIdx.x == 0) {
        sc->rr = tot[0];
        sc->iter += 1;
        if (!isfinite(tot[0])) {
            sc->done = 1;
            sc->status = GBS_ENONFINITE;
        } else if (sqrt(tot[0]) < sc->tol * sc->bnorm) {
            sc->done = 1;
        } else if (sc->iter >= sc->max_iter) {
            sc->done = 1;
            sc->status = GBS_ENOTCONV;
        }
    }
}

struct CsrWs {
    CsrScalars *sc;
    float *r, *z, *p, *ap;
    double *partials;
};

static size_t csr_ws_bytes_impl(int64_t n) { return al256(sizeof(CsrScalars)) + 4 * al256((size_t)n * 4) + al256(3 * 4096 * 8); }

static CsrWs csr_ws(void *ws, int64_t n) {
    char *p = (char *)ws;
    CsrWs w;
    w.sc = (CsrScalars *)p;
    p += al256(sizeof(CsrScalars));
    float **v[4] = {&w.r, &w.z, &w.p, &w.ap};
    for (int i = 0; i < 4; ++i) {
        *v[i] = (float *)p;
        p += al256((size_t)n * 4);
    }
    w.partials = (double *)p;
    return w;
}

}  // namespace gbs

using namespace gbs;

extern "C" size_t gbsimp_pcg_ws_bytes(int nx, int ny, int nz) { return pcg_ws_bytes_impl(nx, ny, nz); }

extern "C" size_t gbsimp_time_pcg_apply_ws_bytes(int nx, int ny, int nz) {
    return pcg_ws_bytes_impl(nx, ny, nz) + al256((size_t)n_dof_of(nx, ny, nz) * sizeof(float));
}

__global__ void fill_f32_kernel(int64_t n, float v, float *a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void freeze_scalars_kernel(PcgScalars *sc) { sc->freeze = 1; }

extern "C" int gbsimp_time_pcg_apply(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *glaw, const float *x,
                                     const uint8_t *node_mask, int reps, void *ws, size_t ws_bytes,
                                     double *seconds_per_launch, void *stream) {
    if (!ctx || !glaw || !x || !ws || !seconds_per_launch || reps <= 0 || reps > 100000 || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_time_pcg_apply: bad arguments");
    if (ws_bytes < gbsimp_time_pcg_apply_ws_bytes(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_time_pcg_apply: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t nd = n_dof_of(nx, ny, nz);
    PcgWs w = pcg_ws(ws, nx, ny, nz);
    float *xu = (float *)(align256(ws) + pcg_ws_bytes_impl(nx, ny, nz) - 256);
    const Law<float> law = make_law<float>(*glaw);
    // A state on which every launch does the full work of one iteration and repeats it:
    // r = 1, everything else 0 (alpha = beta = 0), iteration 0. Single-reduction kernel: the
    // scalars are frozen, so no launch advances the iteration. Dense form: K2 never runs.
    const bool modal = use_modal(ctx, nz);
    if (modal) {
        const int rc = check_modal_partials(ctx, nx, ny, nz, w);
        if (rc) return rc;
    }
    GBS_CUDA_TRY(cudaMemsetAsync(w.sc, 0, sizeof(PcgScalars), st));
    dinv_kernel<float><<<ew_blocks(ctx, nd / 3), 256, 0, st>>>(nx, ny, nz, fast_div(ny + 1), fast_div(nz + 1), law,
                                                                 ctx->kef, x, node_mask, w.dinv);
    fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 1.0f, w.r);
    fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, w.p1);
    fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, xu);
    if (modal) {  // launches alternate the buffer parity: give both parities the same state
        const int64_t ne = (int64_t)nx * ny * nz;
        moduli_f32_kernel<<<ew_blocks(ctx, ne), 256, 0, st>>>(ne, law, x, w.E);
        fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 1.0f, w.r1);
        fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, w.ap);
        fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, w.s0);
        fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, w.s1);
        fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, w.p0);
        fill_f32_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, 0.0f, w.w2);
        freeze_scalars_kernel<<<1, 1, 0, st>>>(w.sc);
    }
    GBS_LAUNCH_CHECK("time_pcg_apply setup");
    if (modal) {
        const int r = modal_prepare<MODE_CG>(ctx, nz);
        if (r < 0) return -r;
    }
    GraphCache *gc = (GraphCache *)ctx->graphs;
    std::lock_guard<std::mutex> lock(gc->mu);
    if (!gc->cap) GBS_CUDA_TRY(cudaStreamCreateWithFlags(&gc->cap, cudaStreamNonBlocking));
    GBS_CUDA_TRY(cudaStreamBeginCapture(gc->cap, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    int rc = GBS_OK;
    PcgArgs pa{w.r, w.dinv, w.p0, w.p1, xu, w.partials, w.sc};
    for (int i = 0; i < reps && rc == GBS_OK; ++i) {
        if (modal) {
            rc = launch_modal<MODE_CG>(ctx, nx, ny, nz, law, w.E, nullptr, nullptr, node_mask, cg_args(w, xu), gc->cap,
                                       i % 6);
        } else {
            TileArgs<float> A{nx, ny, nz, x, nullptr, w.ap, node_mask};
            const dim3 g = tile_grid<TileF>(nx, ny, nz), b = tile_block<TileF>();
            if (ctx->translation_free)
                apply_tile_kernel<float, KeF, TileF::X, TileF::Y, TileF::Z, true, MODE_PCG><<<g, b, 0, gc->cap>>>(A, law, ctx->kef, pa);
            else
                apply_tile_kernel<float, KeF, TileF::X, TileF::Y, TileF::Z, false, MODE_PCG><<<g, b, 0, gc->cap>>>(A, law, ctx->kef, pa);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) rc = cuda_error(e, "apply_tile_kernel<PCG>");
        }
    }
    set_capturing(false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(gc->cap, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphInstantiate");
    cudaEvent_t e0, e1;
    GBS_CUDA_TRY(cudaEventCreate(&e0));
    GBS_CUDA_TRY(cudaEventCreate(&e1));
    rc = GBS_OK;
    float ms = 0.0f;
    if ((e = cudaGraphLaunch(exec, st)) != cudaSuccess ||       // warm-up replay
        (e = cudaEventRecord(e0, st)) != cudaSuccess || (e = cudaGraphLaunch(exec, st)) != cudaSuccess ||
        (e = cudaEventRecord(e1, st)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess ||
        (e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess)
        rc = cuda_error(e, "time_pcg_apply replay");
    count_launches(2 * reps);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(exec);
    if (rc) return rc;
    *seconds_per_launch = 1e-3 * ms / reps;
    return GBS_OK;
}

extern "C" size_t gbsimp_solve_ws_bytes(int nx, int ny, int nz) { return solve_ws_bytes_impl(nx, ny, nz); }

extern "C" size_t gbsimp_pcg_csr_ws_bytes(int64_t n) { return csr_ws_bytes_impl(n); }


extern "C" int gbsimp_pcg_f32(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                              const float *b, const uint8_t *node_mask, float *u, const gbsimp_solve_opts *opts,
                              gbsimp_solve_stats *stats, void *ws, size_t ws_bytes, void *stream) {
    auto t0 = std::chrono::steady_clock::now();
    if (!ctx || !law || !x || !b || !u || !opts || !ws || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_pcg_f32: bad arguments");
    if (ws_bytes < pcg_ws_bytes_impl(nx, ny, nz)) return set_error(GBS_EINVAL, "gbsimp_pcg_f32: workspace too small");
    if ((uintptr_t)u & 15) return set_error(GBS_EINVAL, "gbsimp_pcg_f32: u must be 16-byte aligned");
    PcgScalars h;
    ApplyProfile prof;
    int rc = pcg_run(ctx, nx, ny, nz, law, x, b, node_mask, u, opts->rtol, opts->max_iter, opts->check_every, ws, &h,
                     (cudaStream_t)stream, opts->profile ? &prof : nullptr, opts->fused);
    if (rc) return rc;
    if (stats) {
        stats->apply_seconds = prof.seconds;
        stats->apply_launches = prof.launches;
        stats->status = h.status;
        stats->iterations = h.iter;
        stats->outer = 0;
        stats->relres = h.bnorm > 0.0 ? sqrt(h.rr) / h.bnorm : 0.0;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return GBS_OK;
}

extern "C" int gbsimp_warm_start(gbsimp_ctx *ctx, int64_t n, double *u, double *u_prev, double theta,
                                 void *stream) {
    NvtxRange range("gbsimp_warm_start");
    if (!ctx || n < 0 || (n > 0 && (!u || !u_prev)) || !isfinite(theta))
        return set_error(GBS_EINVAL, "gbsimp_warm_start: bad arguments");
    return warm_start_impl(ctx, n, u, u_prev, theta, (cudaStream_t)stream);
}

extern "C" int gbsimp_solve(gbsimp_ctx *ctx, int nx, int ny, int nz, const gbsimp_law *law, const float *x,
                            const double *f, const uint8_t *node_mask, double *u, const gbsimp_solve_opts *opts,
                            gbsimp_solve_stats *stats, void *ws, size_t ws_bytes, void *stream) {
    auto t0 = std::chrono::steady_clock::now();
    if (!ctx || !law || !x || !f || !u || !opts || !ws || !grid_ok(nx, ny, nz))
        return set_error(GBS_EINVAL, "gbsimp_solve: bad arguments");
    NvtxRange range("gbsimp_solve");
    if (ws_bytes < solve_ws_bytes_impl(nx, ny, nz)) return set_error(GBS_EINVAL, "gbsimp_solve: workspace too small");
    gbsimp_solve_stats s{};
    int rc = solve_run(ctx, nx, ny, nz, law, x, f, node_mask, u, opts, &s, ws, (cudaStream_t)stream);
    if (rc) return rc;
    s.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = s;
    return GBS_OK;
}

extern "C" int gbsimp_pcg_csr_f32(gbsimp_ctx *ctx, int64_t n, const int32_t *row_ptr, const int32_t *col_idx,
                                  const float *values, const float *diagonal, const float *b, float *x,
                                  const int32_t *fixed, int64_t n_fixed, const gbsimp_solve_opts *opts,
                                  gbsimp_solve_stats *stats, void *ws, size_t ws_bytes, void *stream) {
    auto t0 = std::chrono::steady_clock::now();
    if (!ctx || n <= 0 || !row_ptr || !col_idx || !values || !diagonal || !b || !x || !opts || !ws ||
        (n_fixed > 0 && !fixed) || n >= (1LL << 31))
        return set_error(GBS_EINVAL, "gbsimp_pcg_csr_f32: bad arguments");
    if (ws_bytes < csr_ws_bytes_impl(n)) return set_error(GBS_EINVAL, "gbsimp_pcg_csr_f32: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    CsrWs w = csr_ws(ws, n);
    const unsigned vb = vec_blocks(ctx, n);
    unsigned sb = (unsigned)((n * 32 + 255) / 256);
    if (sb > 8u * (unsigned)ctx->num_sms) sb = 8u * (unsigned)ctx->num_sms;
    if (sb < 1) sb = 1;
    const unsigned fb = n_fixed > 0 ? vec_blocks(ctx, n_fixed) : 1;
    CsrScalars init{};
    init.tol = opts->rtol;
    init.max_iter = opts->max_iter;
    void *hp = thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "no pinned staging buffer");
    memcpy(hp, &init, sizeof init);
    GBS_CUDA_TRY(cudaMemcpyAsync(w.sc, hp, sizeof init, cudaMemcpyHostToDevice, st));
    // r = b - A x0; r[fixed] = 0; z = r/diag; p = z; rz = r.z
    csr_spmv_kernel<<<sb, 256, 0, st>>>(n, row_ptr, col_idx, values, x, w.ap);
    csr_init_kernel<<<vb, 256, 0, st>>>(n, b, w.ap, w.r, w.partials, w.sc);
    if (n_fixed > 0) zero_list_kernel<<<fb, 256, 0, st>>>(n_fixed, fixed, n, w.r);
    csr_z_kernel<<<vb, 256, 0, st>>>(n, w.r, diagonal, w.z, w.p, 1, w.partials, w.sc);
    csr_p_kernel<<<vb, 256, 0, st>>>(n, w.z, w.p, 1, w.sc);
    count_launches(4);
    GBS_LAUNCH_CHECK("csr setup");
    const int chunk = opts->check_every > 0 ? opts->check_every : 32;
    CsrScalars h{};
    int launched = 0;
    while (launched < opts->max_iter) {
        const int m = launched + chunk > opts->max_iter ? opts->max_iter - launched : chunk;
        for (int i = 0; i < m; ++i) {
            csr_spmv_kernel<<<sb, 256, 0, st>>>(n, row_ptr, col_idx, values, w.p, w.ap);
            if (n_fixed > 0) zero_list_kernel<<<fb, 256, 0, st>>>(n_fixed, fixed, n, w.ap);
            csr_pap_kernel<<<vb, 256, 0, st>>>(n, w.p, w.ap, w.partials, w.sc);
            csr_xr_kernel<<<vb, 256, 0, st>>>(n, w.p, w.ap, x, w.r, fixed, n_fixed, w.sc);
            if (n_fixed > 0) zero_list_kernel<<<fb, 256, 0, st>>>(n_fixed, fixed, n, w.r);
            csr_check_kernel<<<vb, 256, 0, st>>>(n, w.r, w.partials, w.sc);
            csr_z_kernel<<<vb, 256, 0, st>>>(n, w.r, diagonal, w.z, w.p, 0, w.partials, w.sc);
            csr_p_kernel<<<vb, 256, 0, st>>>(n, w.z, w.p, 0, w.sc);
        }
        count_launches(8 * m - 1);
        GBS_LAUNCH_CHECK("csr iteration");
        launched += m;
        GBS_CUDA_TRY(cudaMemcpyAsync(hp, w.sc, sizeof h, cudaMemcpyDeviceToHost, st));
        GBS_CUDA_TRY(cudaStreamSynchronize(st));
        memcpy(&h, hp, sizeof h);
        if (h.done) break;
    }
    if (stats) {
        stats->status = h.done ? h.status : GBS_ENOTCONV;
        stats->iterations = h.iter;
        stats->outer = 0;
        stats->relres = h.bnorm > 0.0 ? sqrt(h.rr) / h.bnorm : 0.0;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return GBS_OK;
}

// ---- batched rounds ------------------------------------------------------------------------
namespace gbs {

static int batch_round_impl(const gbsimp_ctx *ctx, gbsimp_batch_item *items, int n, const gbsimp_law *glaw,
                            const gbsimp_solve_opts *o, cudaStream_t st) {
    const Law<float> law = make_law<float>(*glaw);
    const int max_outer = o->max_outer > 0 ? o->max_outer : 20;
    const double inner = o->inner_rtol > 0.0 ? o->inner_rtol : kInnerRtol;
    // iteration budget of the inner PCGs in this round (0: each runs to its tolerance)
    const int budget = o->check_every > 0 ? o->check_every : 0;
    const bool dd = use_dd_residual(ctx, o);
    // act: every active item; res: those between inner solves, which get an outer residual
    // (the others resume their paused inner PCG)
    std::vector<int> act, res;
    for (int i = 0; i < n; ++i)
        if (items[i].state == 0) {
            act.push_back(i);
            if (items[i].stats.inner_active == 0) res.push_back(i);
        }
    if (act.empty()) return GBS_OK;
    // ---- FP64 residuals of the items between inner solves, one sync -------------------------
    void *hp = thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "no pinned staging buffer");
    const size_t per = sizeof(OuterScalars);
    for (size_t k = 0; k < res.size(); k += 4096 / per) {
        const size_t m = std::min(res.size() - k, (size_t)(4096 / per));
        for (size_t j = 0; j < m; ++j) {
            gbsimp_batch_item &it = items[res[k + j]];
            SolveWs w = solve_ws(it.ws, it.nx, it.ny, it.nz);
            if (it.stats.outer == 0) {
                GBS_CUDA_TRY(cudaMemsetAsync(w.os, 0, sizeof(OuterScalars), st));
                int rc = outer_start(ctx, n_dof_of(it.nx, it.ny, it.nz), it.u, it.f, it.node_mask, dd, w, st);
                if (rc) return rc;
            }
            int rc = outer_residual(ctx, it.nx, it.ny, it.nz, glaw, it.x, it.f, it.node_mask, it.u, dd, w, st);
            if (rc) return rc;
            GBS_CUDA_TRY(cudaMemcpyAsync((char *)hp + j * per, w.os, per, cudaMemcpyDeviceToHost, st));
        }
        GBS_CUDA_TRY(cudaStreamSynchronize(st));
        for (size_t j = 0; j < m; ++j) {
            gbsimp_batch_item &it = items[res[k + j]];
            OuterScalars h;
            memcpy(&h, (char *)hp + j * per, per);
            gbsimp_solve_stats &s = it.stats;
            s.outer += 1;
            if (!isfinite(h.rr) || !isfinite(h.ff)) {
                s.status = GBS_ENONFINITE;
                it.state = 2;
            } else if (h.ff == 0.0) {
                GBS_CUDA_TRY(cudaMemsetAsync(it.u, 0, n_dof_of(it.nx, it.ny, it.nz) * sizeof(double), st));
                s.relres = 0.0;
                s.status = GBS_OK;
                it.state = 1;
            } else {
                s.relres = sqrt(h.rr / h.ff);
                if (s.relres <= o->rtol) {
                    s.status = GBS_OK;
                    it.state = 1;
                } else if (s.outer > max_outer || s.iterations >= o->max_iter) {
                    s.status = GBS_ENOTCONV;
                    it.state = 2;
                }
            }
        }
    }
    // ---- new inner FP32 PCGs of the items still above rtol ------------------------------------
    std::vector<int> fresh;
    for (int i : res)
        if (items[i].state == 0) fresh.push_back(i);
    for (int i : fresh) {
        gbsimp_batch_item &it = items[i];
        const int64_t nd = n_dof_of(it.nx, it.ny, it.nz);
        SolveWs w = solve_ws(it.ws, it.nx, it.ny, it.nz);
        int src = outer_scale(ctx, nd, dd, w, st);
        if (src) return src;
        double itol = o->rtol / it.stats.relres;
        if (itol < inner) itol = inner;
        PcgWs pw = pcg_ws(w.pcg, it.nx, it.ny, it.nz);
        int rc = pcg_setup(ctx, it.nx, it.ny, it.nz, glaw, it.x, w.b32, it.node_mask, w.d32, itol,
                           o->max_iter - it.stats.iterations, pw, st, SETUP_X0_ZERO);
        if (rc) return rc;
    }
    // ---- run the inner PCGs: paused persistent solves, then the new ones ---------------------
    // A paused solve resumes in the form it started in (the persistent kernel and the graph loop
    // keep their scalars differently). New solves are packed greedily into persistent launches
    // of designs that are resident together; one that fits no launch runs its own graph loop.
    auto fitem = [&](int i) {
        gbsimp_batch_item &it = items[i];
        SolveWs w = solve_ws(it.ws, it.nx, it.ny, it.nz);
        return FusedItem{it.nx, it.ny, it.nz, it.x, it.node_mask, w.d32, pcg_ws(w.pcg, it.nx, it.ny, it.nz)};
    };
    const int group = o->batch_group > 0 && o->batch_group < kMaxFused ? o->batch_group : kMaxFused;
    const int share = o->batch_share == 1 ? 1 : 0;
    auto fits = [&](const std::vector<int> &c) {
        if (c.empty() || c.size() > (size_t)group) return false;
        FusedItem fi[kMaxFused];
        for (size_t j = 0; j < c.size(); ++j) fi[j] = fitem(c[j]);
        FusedPlan P;
        return fused_plan(ctx, fi, (int)c.size(), &P, share) == GBS_OK;
    };
    std::vector<int> order, graph_items;
    for (int i : act)
        if (items[i].state == 0 && items[i].stats.inner_active == 1) order.push_back(i);
    for (int i : act)
        if (items[i].state == 0 && items[i].stats.inner_active == 2) graph_items.push_back(i);
    for (int i : fresh) {
        if (o->fused && ctx->modal_ok) order.push_back(i);
        else graph_items.push_back(i);
    }
    std::vector<std::vector<int>> chunks;
    std::vector<int> cur;
    for (int i : order) {
        cur.push_back(i);
        if (fits(cur)) continue;
        cur.pop_back();
        if (!cur.empty()) chunks.push_back(cur);
        cur.assign(1, i);
        if (fits(cur)) continue;
        cur.clear();
        if (items[i].stats.inner_active == 1) {  // cannot happen: it ran in such a launch before
            items[i].stats.status = set_error(GBS_EINVAL, "gbsimp_batch: a paused solve no longer fits a launch");
            items[i].state = 2;
        } else {
            graph_items.push_back(i);
        }
    }
    if (!cur.empty()) chunks.push_back(cur);
    std::vector<int> fused_items;
    for (const auto &c : chunks) {
        FusedItem fi[kMaxFused];
        for (size_t j = 0; j < c.size(); ++j) fi[j] = fitem(c[j]);
        if (pcg_fused_batch(ctx, fi, (int)c.size(), law, st, budget, share) == GBS_OK) {
            fused_items.insert(fused_items.end(), c.begin(), c.end());
            continue;
        }
        for (int i : c) {  // launch refused
            if (items[i].stats.inner_active == 1) {
                items[i].stats.status = GBS_EINVAL;
                items[i].state = 2;
            } else {
                graph_items.push_back(i);
            }
        }
    }
    const int pause_trips = budget > 0 ? (budget + kLoopUnroll - 1) / kLoopUnroll : 0;
    for (int i : graph_items) {
        gbsimp_batch_item &it = items[i];
        SolveWs w = solve_ws(it.ws, it.nx, it.ny, it.nz);
        PcgWs pw = pcg_ws(w.pcg, it.nx, it.ny, it.nz);
        pcg_set_pause_kernel<<<1, 1, 0, st>>>(pw.sc, pause_trips);
        GBS_LAUNCH_CHECK("pcg_set_pause_kernel");
        bool built = false;
        int rc = launch_loop_graph(ctx, it.nx, it.ny, it.nz, law, it.x, it.node_mask, w.d32, pw, st, &built);
        if (rc) return rc;
        rc = cg_publish(ctx, it.nx, it.ny, it.nz, pw, 1, st);
        if (rc) return rc;
    }
    std::vector<int> inn(fused_items);
    inn.insert(inn.end(), graph_items.begin(), graph_items.end());
    if (inn.empty()) return GBS_OK;
    const size_t n_fused = fused_items.size();
    // finalize the solves that ended (a paused one is left as it is), read every item's PCG
    // scalars (one sync), correct u of the ended ones
    const size_t ps = sizeof(PcgScalars);
    for (size_t k = 0; k < inn.size(); k += 4096 / ps) {
        const size_t m = std::min(inn.size() - k, (size_t)(4096 / ps));
        for (size_t j = 0; j < m; ++j) {
            gbsimp_batch_item &it = items[inn[k + j]];
            const int64_t nd = n_dof_of(it.nx, it.ny, it.nz);
            SolveWs w = solve_ws(it.ws, it.nx, it.ny, it.nz);
            PcgWs pw = pcg_ws(w.pcg, it.nx, it.ny, it.nz);
            // one-kernel graph loop: x may owe a half step; persistent: complete
            const bool graph_loop = k + j >= n_fused;
            pcg_finalize_kernel<<<ew_blocks(ctx, nd), 256, 0, st>>>(nd, pw.p0, pw.p1, w.d32, pw.sc,
                                                                    use_modal(ctx, it.nz) ? (graph_loop ? 2 : 0) : 1);
            GBS_LAUNCH_CHECK("pcg_finalize_kernel");
            GBS_CUDA_TRY(cudaMemcpyAsync((char *)hp + j * ps, pw.sc, ps, cudaMemcpyDeviceToHost, st));
        }
        GBS_CUDA_TRY(cudaStreamSynchronize(st));
        for (size_t j = 0; j < m; ++j) {
            gbsimp_batch_item &it = items[inn[k + j]];
            const bool graph_loop = k + j >= n_fused;
            PcgScalars h;
            memcpy(&h, (char *)hp + j * ps, ps);
            if (graph_loop) count_launches(h.trips * launches_per_trip(ctx, it.nz));
            it.stats.iterations += h.iter - it.stats.inner_iters;
            if (!h.done) {  // paused by the budget: resumes next round, in the same form
                it.stats.inner_iters = h.iter;
                it.stats.inner_active = graph_loop ? 2 : 1;
                continue;
            }
            it.stats.inner_iters = 0;
            it.stats.inner_active = 0;
            if (h.status == GBS_EBREAKDOWN || h.status == GBS_ENONFINITE || h.status == GBS_ETIMEOUT) {
                it.stats.status = h.status;
                if (h.iter == 0 || h.status == GBS_ETIMEOUT) {
                    it.state = 2;
                    continue;
                }
            }
            SolveWs w = solve_ws(it.ws, it.nx, it.ny, it.nz);
            int rc = outer_correct(ctx, n_dof_of(it.nx, it.ny, it.nz), it.node_mask, it.u, dd, w, st);
            if (rc) return rc;
            if (it.stats.status != GBS_OK) it.state = 2;
        }
    }
    return GBS_OK;
}

}  // namespace gbs

static int check_batch(gbsimp_ctx *ctx, gbsimp_batch_item *items, int n, const gbsimp_law *law,
                       const gbsimp_solve_opts *opts) {
    if (!ctx || !law || !opts || n < 0 || (n > 0 && !items)) return set_error(GBS_EINVAL, "gbsimp_batch: bad arguments");
    for (int i = 0; i < n; ++i) {
        const gbsimp_batch_item &it = items[i];
        if (it.state != 0) continue;
        if (!it.x || !it.f || !it.u || !it.ws || !grid_ok(it.nx, it.ny, it.nz))
            return set_error(GBS_EINVAL, "gbsimp_batch: item %d has bad arguments", i);
        if (it.ws_bytes < solve_ws_bytes_impl(it.nx, it.ny, it.nz))
            return set_error(GBS_EINVAL, "gbsimp_batch: item %d workspace too small", i);
        if (it.stats.inner_active < 0 || it.stats.inner_active > 2 || it.stats.inner_iters < 0)
            return set_error(GBS_EINVAL, "gbsimp_batch: item %d has library-owned stats fields set (zero its stats)", i);
    }
    return GBS_OK;
}

extern "C" int gbsimp_batch_round(gbsimp_ctx *ctx, gbsimp_batch_item *items, int n, const gbsimp_law *law,
                                  const gbsimp_solve_opts *opts, void *stream) {
    NvtxRange range("gbsimp_batch_round");
    int rc = check_batch(ctx, items, n, law, opts);
    if (rc) return rc;
    return batch_round_impl(ctx, items, n, law, opts, (cudaStream_t)stream);
}

extern "C" int gbsimp_batch_solve(gbsimp_ctx *ctx, gbsimp_batch_item *items, int n, const gbsimp_law *law,
                                  const gbsimp_solve_opts *opts, void *stream) {
    int rc = check_batch(ctx, items, n, law, opts);
    if (rc) return rc;
    // every item ends within max_outer FP64 rounds; a round budget splits each inner solve over
    // at most max_iter / budget + 1 rounds
    int64_t max_rounds = (opts->max_outer > 0 ? opts->max_outer : 20) + 2;
    if (opts->check_every > 0) max_rounds *= 1 + (int64_t)(opts->max_iter > 0 ? opts->max_iter : 0) / opts->check_every;
    for (int64_t r = 0; r < max_rounds; ++r) {
        bool any = false;
        for (int i = 0; i < n; ++i) any = any || items[i].state == 0;
        if (!any) break;
        rc = batch_round_impl(ctx, items, n, law, opts, (cudaStream_t)stream);
        if (rc) return rc;
    }
    for (int i = 0; i < n; ++i)
        if (items[i].state == 0) {
            items[i].state = 2;
            items[i].stats.status = GBS_ENOTCONV;
        }
    return GBS_OK;
}

extern "C" size_t gbsimp_barrier_selftest_ws_bytes(void) { return 256 + 4096 * sizeof(double) + 256; }

extern "C" int gbsimp_barrier_selftest(gbsimp_ctx *ctx, int extra_arrivals, double wait_seconds, int *status_out,
                                       void *ws, size_t ws_bytes, void *stream) {
    if (!ctx || !status_out || !ws || extra_arrivals < 0 || extra_arrivals > 1024 || !(wait_seconds > 0.0) ||
        wait_seconds > 2.0 || ws_bytes < gbsimp_barrier_selftest_ws_bytes())
        return set_error(GBS_EINVAL, "gbsimp_barrier_selftest: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    char *p = align256(ws);
    unsigned *count = (unsigned *)p;
    int *status = (int *)(p + 64);
    double *partials = (double *)(p + 256);
    GBS_CUDA_TRY(cudaMemsetAsync(p, 0, 256, st));
    int coop = 0, per_sm = 0;
    GBS_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
    GBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, barrier_selftest_kernel, 128, 0));
    if (!coop || per_sm < 1) return set_error(GBS_EINVAL, "gbsimp_barrier_selftest: no cooperative launch");
    int nblk = ctx->num_sms > 0 ? ctx->num_sms : 1;  // one block per SM: all co-resident
    if (nblk > 4096) nblk = 4096;
    unsigned extra = (unsigned)extra_arrivals;
    unsigned long long wait_ns = (unsigned long long)(wait_seconds * 1e9);
    void *args[] = {&partials, &count, &status, &extra, &wait_ns};
    const cudaError_t e =
        cudaLaunchCooperativeKernel((void *)barrier_selftest_kernel, dim3((unsigned)nblk), dim3(128), args, 0, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_error(e, "barrier_selftest_kernel");
    }
    count_launches(1);
    void *hp = thread_pinned();
    if (!hp) return set_error(GBS_ECUDA, "no pinned staging buffer");
    GBS_CUDA_TRY(cudaMemcpyAsync(hp, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBS_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(status_out, hp, sizeof(int));
    return GBS_OK;
}
