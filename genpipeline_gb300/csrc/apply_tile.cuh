// apply_tile.cuh -- matrix-free K(x) p on brick tiles of nodes (owner computes, no atomics).
//
// Each CTA owns a TX x TY x TZ brick of NODES (threadIdx.x runs along z, the contiguous
// axis of the reference layout, so a warp reads/writes one 32-node z-run = 384 B of a
// 3-component vector). It stages in shared memory
//   * the vector p on the brick plus a one-node halo ((TX+2)(TY+2)(TZ+2) nodes x 3), and
//   * E(x_e) of the (TX+1)(TY+1)(TZ+1) elements that touch the brick (0 outside the grid),
// then every thread gathers its 27-node neighbourhood into registers and sums, over the 8
// elements around its node, E_e * (3 rows of Ke for the node's local position) . p_e.
// This is y_n = sum_{e ∋ n} E_e [Ke p_e]_{a(n,e)}, the row form of the COO assembly of
// genpipeline/topology/simp_solver.py:200-205; every output DOF is written by exactly one
// thread in a fixed summation order (deterministic, no atomics, no node colouring).
//
// SUB (valid only when Ke annihilates rigid translations, as the quadrature Ke does):
// p_m - p_n is used in place of p_m, which removes the translation part of the element
// displacement before the FP32 products and skips the node's own 3x3 block.
#pragma once

#include "common.cuh"

namespace gbs {

// MODE_PCG: K1 of the two-kernel PCG iteration (dense kernel). MODE_CG: the one-kernel
// single-reduction PCG iteration (modal kernel); MODE_CG_FUSED: the same pass inside the
// persistent kernel, where vectors that other CTAs rewrite between passes are read at L2
// (L1 is not coherent across SMs within one launch).
enum { MODE_PLAIN = 0, MODE_PCG = 1, MODE_CG = 3, MODE_CG_FUSED = 4 };

// State of the one-kernel PCG at the start of an iteration. Launch k writes slot k & 1 and
// reads slot (k & 1) ^ 1; `pending` marks a state whose pass has written block partial sums
// (slot k & 1 of the partials) that the next launch folds in before its own pass.
// The scalars are double-float (hi, lo) pairs; alpha_prev is the alpha of the iteration
// before (the odd launches' two-step update of x uses it).
struct CgState {
    df32 alpha, beta, gamma, rr, pap, alpha_prev;
    int iter, done, status, pending;
};

// Device-resident state of one Jacobi-PCG solve (FP32 vectors, FP64 scalars).
struct PcgScalars {
    double rz;        // r_k . z_k
    double alpha[2];  // alpha_k in slot k&1 (alpha_{-1} = 0)
    double beta;      // beta_k used by the step-k p update (beta_0 = 0)
    double bnorm;     // ||D b||
    double rr;        // ||r_k||^2
    double tol;       // rtol
    double pap;       // last p.Ap
    int iter;         // completed iterations
    int done;         // 1 = stop
    int status;       // GBS_OK / GBS_ENOTCONV / GBS_EBREAKDOWN / GBS_ENONFINITE
    int max_iter;
    unsigned counter; // blocks finished in the running kernel (last-block reductions)
    unsigned bar_count, bar_gen;  // grid barrier of the persistent kernel
    int trips;        // WHILE-loop trips run by the device-driven loop
    int max_trips;    // hard cap on those trips (the loop always ends)
    int pause_trips;  // > 0: the loop stops after this many trips without ending the solve
                      // (batched rounds with an iteration budget resume it in the next round)
    int freeze;       // 1 = kernels leave the scalars as they are (timing of one pass)
    float rr_stop;    // one-kernel PCG: (tol ||D b||)^2 in FP32, the stop test on r.r
    CgState st[2];    // one-kernel PCG: the state by launch parity
};

struct PcgArgs {
    const float *r;     // residual r_k (masked)
    const float *dinv;  // 1/diag(K) on free DOFs, 0 on fixed DOFs
    float *pbuf0;       // p_{k} lives in pbuf[k & 1]
    float *pbuf1;
    float *xu;          // iterate; K1 of step k adds alpha_{k-1} p_{k-1}
    double *partials;   // one double per block
    PcgScalars *sc;
};

// Buffers of the single-reduction PCG (MODE_CG). Iteration i reads r[i&1], w[i&1],
// s[(i+1)&1] and writes r[(i+1)&1], w[(i+1)&1], s[i&1]; p and x are updated in place.
struct CgArgs {
    float *r[2];        // r_i (masked residual)
    float *w[3];        // w_i = D K D u_i, u_i = M r_i: launch k reads w[k % 3], writes w[(k + 1) % 3]
                        // and clears the shared node planes of w[(k + 2) % 3], the next launch's
                        // output (the persistent kernel uses w[0], w[1] by iteration parity)
    float *s[2];        // s_i = D K D p_i
    float *p;           // search direction
    float *xu;          // iterate
    const float *dinv;  // M = 1/diag(K) on free DOFs, 0 on fixed DOFs
    double *partials;   // per block three double-float sums (float2 hi, lo) in two parity slots
    PcgScalars *sc;     // alpha[0] = alpha_i, beta = beta_i, rz = gamma_i = r_i.u_i
};

template <typename T>
struct TileArgs {
    int nx, ny, nz;
    const float *x;       // element densities (n_elem)
    const T *p;           // MODE_PLAIN input
    T *y;                 // output K p (masked)
    const uint8_t *mask;  // node Dirichlet bits (nullable)
};

template <typename T, typename KeT, int TX, int TY, int TZ, bool SUB, int MODE>
__global__ void __launch_bounds__(TX *TY *TZ)
    apply_tile_kernel(TileArgs<T> A, Law<T> law, const KeT ke, PcgArgs pa) {
    constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;
    constexpr int EX = TX + 1, EY = TY + 1, EZ = TZ + 1;
    constexpr int NT = TX * TY * TZ;
    __shared__ T sp[HX * HY * HZ * 3];
    __shared__ T se[EX * EY * EZ];
    __shared__ double sred[32];

    const int nx = A.nx, ny = A.ny, nz = A.nz;
    const int NY = ny + 1, NZ = nz + 1;
    const int tid = threadIdx.x + TZ * (threadIdx.y + TY * threadIdx.z);
    const int z0 = blockIdx.x * TZ, y0 = blockIdx.y * TY, x0 = blockIdx.z * TX;

    int it = 0;
    double beta = 0.0, alpha_prev = 0.0;
    const float *pold = nullptr;
    float *pnew = nullptr;
    if (MODE == MODE_PCG) {
        if (pa.sc->done) return;
        it = pa.sc->iter;
        beta = pa.sc->beta;
        alpha_prev = pa.sc->alpha[(it + 1) & 1];
        pold = (it & 1) ? pa.pbuf0 : pa.pbuf1;
        pnew = (it & 1) ? pa.pbuf1 : pa.pbuf0;
    }

    // ---- stage p (halo) and E(x): all global loads of a thread are issued before any
    // shared-memory store (unrolled, compile-time trip counts) so their latencies overlap.
    constexpr int NPV = HX * HY * HZ * 3;
    constexpr int IPV = (NPV + NT - 1) / NT;
    constexpr int NEV = EX * EY * EZ;
    constexpr int IEV = (NEV + NT - 1) / NT;
    T pv[IPV];
    float xv[IEV];
    bool xok[IEV];
#pragma unroll
    for (int q = 0; q < IPV; ++q) {
        const int t = tid + q * NT;
        const int c = t % 3;
        const int rest = t / 3;
        const int hz = rest % HZ;
        const int hy = (rest / HZ) % HY;
        const int hx = rest / (HZ * HY);
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
        T v = (T)0;
        if (t < NPV && gx >= 0 && gx <= nx && gy >= 0 && gy <= ny && gz >= 0 && gz <= nz) {
            const int64_t d = 3 * (((int64_t)gx * NY + gy) * NZ + gz) + c;
            if (MODE == MODE_PLAIN) {
                v = A.p[d];
                if (A.mask && ((A.mask[d / 3] >> c) & 1)) v = (T)0;
            } else {
                v = (T)fmaf((float)beta, pold[d], pa.r[d] * pa.dinv[d]);
            }
        }
        pv[q] = v;
    }
#pragma unroll
    for (int q = 0; q < IEV; ++q) {
        const int t = tid + q * NT;
        const int ez = t % EZ;
        const int ey = (t / EZ) % EY;
        const int ex = t / (EZ * EY);
        const int gx = x0 - 1 + ex, gy = y0 - 1 + ey, gz = z0 - 1 + ez;
        xok[q] = t < NEV && gx >= 0 && gx < nx && gy >= 0 && gy < ny && gz >= 0 && gz < nz;
        xv[q] = xok[q] ? A.x[((int64_t)gx * ny + gy) * nz + gz] : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < IPV; ++q) {
        const int t = tid + q * NT;
        if (t < NPV) sp[t] = pv[q];
    }
#pragma unroll
    for (int q = 0; q < IEV; ++q) {
        const int t = tid + q * NT;
        if (t < NEV) se[t] = xok[q] ? modulus(law, (T)xv[q]) : (T)0;  // no element: E = 0
    }
    __syncthreads();

    const int tz = threadIdx.x, ty = threadIdx.y, tx = threadIdx.z;
    const int gx = x0 + tx, gy = y0 + ty, gz = z0 + tz;
    const bool own = (gx <= nx && gy <= ny && gz <= nz);
    double part = 0.0;
    if (own) {
        T P[3][3][3][3];
#pragma unroll
        for (int dx = 0; dx < 3; ++dx)
#pragma unroll
            for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                for (int dz = 0; dz < 3; ++dz)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        P[dx][dy][dz][c] = sp[(((tx + dx) * HY + (ty + dy)) * HZ + (tz + dz)) * 3 + c];
        T ctr[3] = {P[1][1][1][0], P[1][1][1][1], P[1][1][1][2]};
        if (SUB) {
#pragma unroll
            for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                    for (int dz = 0; dz < 3; ++dz)
#pragma unroll
                        for (int c = 0; c < 3; ++c) P[dx][dy][dz][c] -= ctr[c];
        }
        T acc[3] = {(T)0, (T)0, (T)0};
#pragma unroll
        for (int a = 0; a < 8; ++a) {
            const T E = se[((tx + 1 - corner_x(a)) * EY + (ty + 1 - corner_y(a))) * EZ + (tz + 1 - corner_z(a))];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                T s = (T)0;
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    if (SUB && b == a) continue;
                    const int dx = corner_x(b) - corner_x(a) + 1;
                    const int dy = corner_y(b) - corner_y(a) + 1;
                    const int dz = corner_z(b) - corner_z(a) + 1;
#pragma unroll
                    for (int c2 = 0; c2 < 3; ++c2)
                        s = fma((T)ke.k[(3 * a + c) * 24 + 3 * b + c2], P[dx][dy][dz][c2], s);
                }
                acc[c] = fma(E, s, acc[c]);
            }
        }
        const int64_t n = ((int64_t)gx * NY + gy) * NZ + gz;
        const uint8_t m = A.mask ? A.mask[n] : (uint8_t)0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T yc = ((m >> c) & 1) ? (T)0 : acc[c];
            A.y[3 * n + c] = yc;
            if (MODE == MODE_PCG) {
                pnew[3 * n + c] = (float)ctr[c];
                part += (double)ctr[c] * (double)yc;
                pa.xu[3 * n + c] += (float)alpha_prev * pold[3 * n + c];
            }
        }
    }

    if (MODE == MODE_PCG) {
        // p.Ap: block partial -> last block reduces in block order, sets alpha_k.
        const double bs = block_sum(part, sred);
        const int nblk = gridDim.x * gridDim.y * gridDim.z;
        const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        __shared__ bool last;
        if (tid == 0) {
            pa.partials[bid] = bs;
            __threadfence();
            last = (atomicAdd(&pa.sc->counter, 1u) == (unsigned)(nblk - 1));
        }
        __syncthreads();
        if (last) {
            __threadfence();
            double s = 0.0;
            for (int i = tid; i < nblk; i += NT) s += ((volatile double *)pa.partials)[i];
            s = block_sum(s, sred);
            if (tid == 0) {
                PcgScalars *sc = pa.sc;
                sc->counter = 0;
                sc->pap = s;
                if (!(s > 0.0) || !isfinite(s)) {
                    sc->done = 1;
                    sc->status = isfinite(s) ? GBS_EBREAKDOWN : GBS_ENONFINITE;
                    sc->alpha[it & 1] = 0.0;
                } else {
                    sc->alpha[it & 1] = sc->rz / s;
                }
            }
        }
    }
}

// Tile shapes (node bricks) per precision.
struct TileF {
    static constexpr int X = 4, Y = 4, Z = 16;
};
struct TileD {
    static constexpr int X = 2, Y = 2, Z = 32;
};

template <typename Tile>
inline dim3 tile_grid(int nx, int ny, int nz) {
    return dim3((unsigned)((nz + 1 + Tile::Z - 1) / Tile::Z), (unsigned)((ny + 1 + Tile::Y - 1) / Tile::Y),
                (unsigned)((nx + 1 + Tile::X - 1) / Tile::X));
}
template <typename Tile>
inline dim3 tile_block() {
    return dim3(Tile::Z, Tile::Y, Tile::X);
}

}  // namespace gbs
