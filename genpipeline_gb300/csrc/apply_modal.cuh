// apply_modal.cuh -- K(x) p for the isotropic unit-cube element through its modal form.
//
// Let T = T8 (x) I3 with T8[a][m] = prod_d (m_d ? s(c_d(a)) : 1), s(0) = -1, s(1) = +1: the
// 2x2x2 Walsh-Hadamard basis of an element's corner values (mode m: bit 2 = x, bit 1 = y,
// bit 0 = z; bit set = "difference" along that axis). Since T^T T = 8 I,
//     Ke = T Km T^T   with   Km = T^T Ke T / 64.
// For any isotropic material on a cube, Km has the same 45 nonzeros (3 translation modes
// have zero rows and columns; constant strains couple the linear modes; bilinear and
// trilinear modes are nearly diagonal). So one element's product Ke p_e is
//     q = T^T p_e   (Hadamard butterflies: 72 add/sub),
//     r = E_e Km q  (45 FMA, 21 FMUL),
//     y = T r       (72 add/sub),
// about 210 FP32 operations against 576 FMA for the dense 24x24 product, and the
// translation part of p_e cancels exactly in the first butterfly (FP32-friendly).
//
// Data movement: a CTA owns F consecutive nodes of the flattened (y,z) node plane
// (flat = j*(nz+1) + k) and walks along x. Per step it computes one plane of the
// F + nz + 2 elements touching those nodes (elements with k = nz are empty padding) from two
// node planes held in shared memory (float4 per node, halo nz+2 on each side), while the
// next node plane is loaded into registers. Contributions go to a per-corner shared array;
// each owned node then sums the 4 (y,z) corners of element plane i (cx = 0) and keeps the
// 4 of the x+1 side in registers for the next plane: one writer per node and DOF, fixed
// summation order, no atomics.
#pragma once

#include "apply_tile.cuh"

namespace gbs {

struct ModalGeom {
    int nx, ny, nz;
    int nseg, seglen;  // x segments: node planes [s*seglen, min((s+1)*seglen, nx+1))
};


// Shared memory bytes of the modal kernel for a given z extent.
template <int NT, int EPT>
inline size_t modal_smem_bytes(int nz) {
    const int NE = NT * EPT, H = nz + 2, R = NE + H;
    return (size_t)3 * R * sizeof(float4) + (size_t)2 * NE * sizeof(float) + (size_t)24 * NE * sizeof(float);
}

// One element: corners P[b][c] (b = cx*4 + cy*2 + cz) -> y[b][c] = E (Ke p_e)_b,c.
__device__ __forceinline__ void modal_element(float (&v)[8][3], float E, const ModalK &km) {
    // forward Walsh-Hadamard per component: (u0, u1) -> (u0 + u1, u1 - u0)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float u0 = v[b][c], u1 = v[b | bit][c];
                v[b][c] = u0 + u1;
                v[b | bit][c] = u1 - u0;
            }
        }
    }
    // r = E Km q (translation mode 0 has no entries)
    float r[8][3];
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[m][c] = 0.0f;
#pragma unroll
    for (int i = 0; i < kModalNnz; ++i) {
        const int ro = modal_row(i), co = modal_col(i);
        r[ro / 3][ro % 3] = fmaf(km.v[i], v[co / 3][co % 3], r[ro / 3][ro % 3]);
    }
#pragma unroll
    for (int m = 1; m < 8; ++m)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[m][c] *= E;
    // inverse: (r0, r1) -> (r0 - r1, r0 + r1) along each axis
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float r0 = r[b][c], r1 = r[b | bit][c];
                r[b][c] = r0 - r1;
                r[b | bit][c] = r0 + r1;
            }
        }
    }
#pragma unroll
    for (int b = 0; b < 8; ++b)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[b][c] = r[b][c];
}

// PCG operands of one pass: p_new = r * dinv + beta * p_old is formed on the staged planes,
// x += alpha_prev * p_old on the owned nodes, p_new is written for the owned nodes.
struct PcgPass {
    float beta, alpha_prev;
    const float *r, *dinv, *pold;
    float *pnew, *xu;
};

template <int MODE>
__device__ __forceinline__ float ld_vec(const float *p) {
    if (MODE == MODE_FUSED) return __ldcg(p);
    return *p;
}

// One sliding-window pass of a CTA over its (flat tile, x segment): y = D K D p on the owned
// nodes. Returns this thread's share of p.y (PCG mode; 0 otherwise).
template <int NT, int EPT, int MAXN, int MODE>
__device__ __forceinline__ double modal_pass(const ModalGeom &G, const float *__restrict__ x,
                                             const float *__restrict__ p, float *__restrict__ y,
                                             const uint8_t *__restrict__ mask, const Law<float> &law,
                                             const ModalK &km, const PcgPass &pp, float4 *smem4, int tile,
                                             int seg) {
    constexpr int NE = NT * EPT;

    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const int NZ = nz + 1;
    const int S = (ny + 1) * NZ;  // nodes per x plane
    const int H = nz + 2;         // flat halo (one y row plus one node)
    const int R = NE + H;         // staged nodes per plane
    const int F = NE - H;         // owned nodes per plane
    const int F0 = tile * F;
    const int xs = seg * G.seglen;
    const int xe = min(xs + G.seglen, nx + 1);
    const int tid = threadIdx.x;

    float4 *Pn = smem4;                 // [3][R]  node planes (x, y, z, unused)
    float *Es = (float *)(Pn + 3 * R);  // [2][NE] element moduli
    float *Cc = Es + 2 * NE;            // [24][NE] element corner contributions

    const float beta = pp.beta, alpha_prev = pp.alpha_prev;
    const float *pold = pp.pold;
    float *pnew = pp.pnew;

    // ---- staging: issue the loads of a plane now, combine and store them later, so that
    // the element work of the current plane hides their latency ------------------------
    float ra[MAXN][3], rb[MAXN][3], rc[MAXN][3];  // PLAIN: p, -, -   PCG: r, dinv, p_old
    uint8_t rm[MAXN];
    float ex[EPT];
    bool eok[EPT];
    auto issue_plane = [&](int j) {
#pragma unroll
        for (int q = 0; q < MAXN; ++q) {
            const int l = tid + q * NT;
            const int flat = F0 - H + l;
            const bool ok = l < R && j >= 0 && j <= nx && flat >= 0 && flat < S;
            const int64_t n = ok ? (int64_t)j * S + flat : 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (MODE == MODE_PLAIN) {
                    ra[q][c] = ok ? p[3 * n + c] : 0.0f;
                } else {
                    ra[q][c] = ok ? ld_vec<MODE>(&pp.r[3 * n + c]) : 0.0f;
                    rb[q][c] = ok ? pp.dinv[3 * n + c] : 0.0f;
                    rc[q][c] = ok ? ld_vec<MODE>(&pold[3 * n + c]) : 0.0f;
                }
            }
            if (MODE == MODE_PLAIN) rm[q] = (ok && mask) ? mask[n] : (uint8_t)0;
        }
    };
    auto commit_plane = [&](int slot) {
#pragma unroll
        for (int q = 0; q < MAXN; ++q) {
            const int l = tid + q * NT;
            float v[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (MODE == MODE_PLAIN)
                    v[c] = ((rm[q] >> c) & 1) ? 0.0f : ra[q][c];
                else
                    v[c] = fmaf(beta, rc[q][c], ra[q][c] * rb[q][c]);
            }
            if (l < R) Pn[slot * R + l] = make_float4(v[0], v[1], v[2], 0.0f);
        }
    };
    auto issue_eplane = [&](int j) {
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            const int ef = F0 - H + tid + q * NT;
            const int ey = ef >= 0 ? ef / NZ : 0, ez = ef >= 0 ? ef - ey * NZ : 0;
            eok[q] = j >= 0 && j < nx && ef >= 0 && ey < ny && ez < nz;
            ex[q] = eok[q] ? x[((int64_t)j * ny + ey) * nz + ez] : 0.0f;
        }
    };
    auto commit_eplane = [&](int slot) {
#pragma unroll
        for (int q = 0; q < EPT; ++q) Es[slot * NE + tid + q * NT] = eok[q] ? modulus(law, ex[q]) : 0.0f;
    };

    // ---- prologue: node planes xs-1, xs and element plane xs-1 --------------------------
    issue_plane(xs - 1);
    commit_plane(0);
    issue_plane(xs);
    issue_eplane(xs - 1);
    commit_plane(1);
    commit_eplane(0);
    __syncthreads();

    float acc[EPT][3];
#pragma unroll
    for (int q = 0; q < EPT; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.0f;
    double part = 0.0;

    for (int i = xs - 1; i < xe; ++i) {  // modal_geom makes every segment non-empty
        const int k = i - (xs - 1);
        const int s0 = k % 3, s1 = (k + 1) % 3, s2 = (k + 2) % 3;
        const int es = k & 1;
        const bool more_nodes = i + 2 <= xe;
        const bool more_elems = i + 1 <= xe - 1;
        if (more_nodes) issue_plane(i + 2);
        if (more_elems) issue_eplane(i + 1);
        // owned-node operands of plane i, loaded before the element work as well
        const bool out_plane = i >= xs;
        uint8_t om[EPT];
        float ox[EPT][3], op[EPT][3];
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            const int t = tid + q * NT;
            const bool ok = out_plane && t < F && F0 + t < S;
            const int64_t n = ok ? (int64_t)i * S + F0 + t : 0;
            om[q] = (ok && mask) ? mask[n] : (uint8_t)0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (MODE != MODE_PLAIN) {
                    ox[q][c] = ok ? ld_vec<MODE>(&pp.xu[3 * n + c]) : 0.0f;
                    op[q][c] = ok ? ld_vec<MODE>(&pold[3 * n + c]) : 0.0f;
                } else {
                    ox[q][c] = op[q][c] = 0.0f;
                }
            }
        }

        // ---- element plane i -----------------------------------------------------------
        if (i >= 0 && i < nx) {
#pragma unroll 1
            for (int q = 0; q < EPT; ++q) {
                const int t = tid + q * NT;
                const float E = Es[es * NE + t];
                float v[8][3];
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const int cx = b >> 2, cy = (b >> 1) & 1, cz = b & 1;
                    const float4 w = Pn[(cx ? s1 : s0) * R + t + cy * NZ + cz];
                    v[b][0] = w.x;
                    v[b][1] = w.y;
                    v[b][2] = w.z;
                }
                modal_element(v, E, km);
#pragma unroll
                for (int b = 0; b < 8; ++b)
#pragma unroll
                    for (int c = 0; c < 3; ++c) Cc[(b * 3 + c) * NE + t] = v[b][c];
            }
        } else {
#pragma unroll 1
            for (int q = 0; q < EPT; ++q)
#pragma unroll
                for (int kk = 0; kk < 24; ++kk) Cc[kk * NE + tid + q * NT] = 0.0f;
        }
        if (more_nodes) commit_plane(s2);
        if (more_elems) commit_eplane(es ^ 1);
        __syncthreads();

        // ---- owned nodes of plane i ------------------------------------------------------
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            const int t = tid + q * NT;
            if (t < F) {
                const int te[4] = {t + H, t + H - 1, t + 1, t};  // (cy,cz) = 00, 01, 10, 11
                float yv[3], nacc[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float s = acc[q][c], a1 = 0.0f;
#pragma unroll
                    for (int yz = 0; yz < 4; ++yz) {
                        s += Cc[(yz * 3 + c) * NE + te[yz]];
                        a1 += Cc[((4 + yz) * 3 + c) * NE + te[yz]];
                    }
                    yv[c] = s;
                    nacc[c] = a1;
                }
                const int flat = F0 + t;
                if (out_plane && flat < S) {
                    const int64_t n = (int64_t)i * S + flat;
                    const float4 w = Pn[s0 * R + t + H];
                    const float pc[3] = {w.x, w.y, w.z};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float yc = ((om[q] >> c) & 1) ? 0.0f : yv[c];
                        y[3 * n + c] = yc;
                        if (MODE != MODE_PLAIN) {
                            pnew[3 * n + c] = pc[c];
                            part += (double)(pc[c] * yc);
                            pp.xu[3 * n + c] = fmaf(alpha_prev, op[q][c], ox[q][c]);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[q][c] = nacc[c];
            }
        }
        __syncthreads();
    }

    return part;
}

template <int NT, int EPT, int MAXN, int MODE>
__global__ void __launch_bounds__(NT, 2)
    apply_modal_kernel(ModalGeom G, const float *__restrict__ x, const float *__restrict__ p, float *__restrict__ y,
                       const uint8_t *__restrict__ mask, Law<float> law, const ModalK km, PcgArgs pa) {
    extern __shared__ float4 smem4[];
    __shared__ double sred[32];
    const int tid = threadIdx.x;
    int it = 0;
    PcgPass pp{0.0f, 0.0f, pa.r, pa.dinv, nullptr, nullptr, pa.xu};
    if (MODE == MODE_PCG) {
        if (pa.sc->done) return;
        it = pa.sc->iter;
        pp.beta = (float)pa.sc->beta;
        pp.alpha_prev = (float)pa.sc->alpha[(it + 1) & 1];
        pp.pold = (it & 1) ? pa.pbuf0 : pa.pbuf1;
        pp.pnew = (it & 1) ? pa.pbuf1 : pa.pbuf0;
    }
    const double part = modal_pass<NT, EPT, MAXN, MODE>(G, x, p, y, mask, law, km, pp, smem4, blockIdx.x, blockIdx.y);
    if (MODE == MODE_PCG) {
        const double bs = block_sum(part, sred);
        const int nblk = gridDim.x * gridDim.y;
        const int bid = blockIdx.x + gridDim.x * blockIdx.y;
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
            for (int b = tid; b < nblk; b += NT) s += ((volatile double *)pa.partials)[b];
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

// Launch geometry: NT = 256 threads, EPT = 2 (512 elements per plane step).
constexpr int kModalNT = 256;
constexpr int kModalEPT = 2;

inline bool modal_fits(int nz) { return nz + 2 <= kModalNT * kModalEPT - 64 && nz + 2 <= 2 * kModalNT; }

inline ModalGeom modal_geom(int nx, int ny, int nz, int num_sms, int blocks_per_sm) {
    const int NE = kModalNT * kModalEPT, H = nz + 2, F = NE - H;
    const int S = (ny + 1) * (nz + 1);
    const int tiles = (S + F - 1) / F;
    const int target = (num_sms > 0 ? num_sms : 148) * (blocks_per_sm > 0 ? blocks_per_sm : 1);
    // As many x segments as fit in one wave of resident CTAs (rounding down, so that the
    // re-rounded segment count never exceeds the target).
    int nseg = target / tiles;
    if (nseg > nx + 1) nseg = nx + 1;
    if (nseg < 1) nseg = 1;
    const int seglen = (nx + 1 + nseg - 1) / nseg;
    nseg = (nx + 1 + seglen - 1) / seglen;
    ModalGeom g{nx, ny, nz, nseg, seglen};
    return g;
}

inline dim3 modal_grid(const ModalGeom &g) {
    const int NE = kModalNT * kModalEPT, H = g.nz + 2, F = NE - H;
    const int S = (g.ny + 1) * (g.nz + 1);
    return dim3((unsigned)((S + F - 1) / F), (unsigned)g.nseg, 1);
}

// Sets the kernel's dynamic shared-memory limit and caches its occupancy for the device
// (host calls only; done before any graph capture). Returns resident CTAs per SM or < 0.
// Staged nodes per thread: R / NT = EPT + ceil((nz + 2) / NT).
inline bool modal_small_halo(int nz) { return nz + 2 <= kModalNT; }

template <int MODE, int MAXN>
inline int modal_prepare_one(const gbsimp_ctx *ctx) {
    auto kern = apply_modal_kernel<kModalNT, kModalEPT, MAXN, MODE>;
    static int per_sm_cache[128] = {};  // benign race: every thread stores the same value
    const int dev = ctx->device >= 0 && ctx->device < 128 ? ctx->device : 0;
    if (per_sm_cache[dev] > 0) return per_sm_cache[dev];
    const int smax = (int)modal_smem_bytes<kModalNT, kModalEPT>(446);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    if (e != cudaSuccess) return -cuda_error(e, "cudaFuncSetAttribute(apply_modal_kernel)");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kModalNT, smax) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    per_sm_cache[dev] = per_sm;
    return per_sm;
}

template <int MODE>
inline int modal_prepare(const gbsimp_ctx *ctx, int nz) {
    return modal_small_halo(nz) ? modal_prepare_one<MODE, kModalEPT + 1>(ctx) : modal_prepare_one<MODE, kModalEPT + 2>(ctx);
}

// Launches the modal kernel.
template <int MODE>
inline int launch_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                        const float *p, float *y, const uint8_t *mask, const PcgArgs &pa, cudaStream_t st) {
    const int per_sm = modal_prepare<MODE>(ctx, nz);
    if (per_sm < 0) return -per_sm;
    const size_t smem = modal_smem_bytes<kModalNT, kModalEPT>(nz);
    const ModalGeom g = modal_geom(nx, ny, nz, ctx->num_sms, per_sm);
    if (modal_small_halo(nz))
        apply_modal_kernel<kModalNT, kModalEPT, kModalEPT + 1, MODE>
            <<<modal_grid(g), kModalNT, smem, st>>>(g, x, p, y, mask, law, ctx->km, pa);
    else
        apply_modal_kernel<kModalNT, kModalEPT, kModalEPT + 2, MODE>
            <<<modal_grid(g), kModalNT, smem, st>>>(g, x, p, y, mask, law, ctx->km, pa);
    GBS_LAUNCH_CHECK("apply_modal_kernel");
    return GBS_OK;
}

}  // namespace gbs
