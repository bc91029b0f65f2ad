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


// Shared memory bytes of the modal kernel for a given z extent: three staged node planes
// (six for the PCG modes, which also keep M r of each plane), two planes of element moduli
// and the 24 corner contributions of every element of a plane.
template <int NT, int EPT>
inline size_t modal_smem_bytes(int nz, bool cg) {
    const int NE = NT * EPT, H = nz + 2, R = NE + H;
    return (size_t)(cg ? 6 : 3) * R * sizeof(float4) + (size_t)2 * NE * sizeof(float) +
           (size_t)24 * NE * sizeof(float);
}

// Packed FP32x2 helpers (sm_100+): lane .x belongs to one element, lane .y to another.
// a - b is fma(b, -1, a), which rounds exactly like the subtraction.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// Two elements at once: corners v[b][c] (b = cx*4 + cy*2 + cz) -> E (Ke p_e)_b,c for each
// lane. The operations and their order per lane are those of the scalar form: forward
// butterflies, r = Km q (each row summed in column order), r *= E, inverse butterflies.
__device__ __forceinline__ void modal_element2(float2 (&v)[8][3], float2 E, const ModalK &km) {
    // forward Walsh-Hadamard per component: (u0, u1) -> (u0 + u1, u1 - u0)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 u0 = v[b][c], u1 = v[b | bit][c];
                v[b][c] = add2(u0, u1);
                v[b | bit][c] = sub2(u1, u0);
            }
        }
    }
    // r = E Km q, one block at a time, in place (mode 0, the translations, has no entries)
#pragma unroll
    for (int bk = 0; bk < kModalBlocks; ++bk) {
        float2 t[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int ro = modal_block(bk, a);
            if (ro < 0) continue;
            float2 s = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int i = 0; i < kModalNnz; ++i) {
                if (modal_row(i) != ro) continue;
                const int co = modal_col(i);
                const float2 k = km.c[modal_class(i)];
                s = modal_row_first(i) ? __fmul2_rn(k, v[co / 3][co % 3]) : __ffma2_rn(k, v[co / 3][co % 3], s);
            }
            t[a] = __fmul2_rn(s, E);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int ro = modal_block(bk, a);
            if (ro >= 0) v[ro / 3][ro % 3] = t[a];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) v[0][c] = make_float2(0.0f, 0.0f);
    // inverse: (r0, r1) -> (r0 - r1, r0 + r1) along each axis
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 r0 = v[b][c], r1 = v[b | bit][c];
                v[b][c] = sub2(r0, r1);
                v[b | bit][c] = add2(r0, r1);
            }
        }
    }
}

// Operands of one pass of the single-reduction PCG iteration i (the Chronopoulos-Gear form of
// Jacobi-PCG: the same iterates as the textbook recurrence in exact arithmetic, with one
// grid-wide reduction per iteration instead of two). With u = M r (M = 1/diag) and
// w = D K D u:
//   staging (every staged node, halo included):
//       s_i = w_i + beta_i s_{i-1},   r_{i+1} = r_i - alpha_i s_i,   u_{i+1} = M r_{i+1}
//   owned nodes: p_i = M r_i + beta_i p_{i-1},   x_{i+1} = x_i + alpha_i p_i,
//       written: s_i, r_{i+1}, p_i, x_{i+1} and w_{i+1} = D K D u_{i+1}
//   sums: r_{i+1}.u_{i+1}, w_{i+1}.u_{i+1}, r_{i+1}.r_{i+1}
// r, w and s are double-buffered by iteration parity (neighbouring CTAs read the old ones at
// their halo while the owners write the new ones); p and x are touched by their owner only.
struct CgPass {
    float alpha, beta;
    const float *r, *w, *sold, *dinv;
    float *rnew, *snew, *p, *xu;
};

template <int MODE>
__device__ __forceinline__ float ld_vec(const float *p) {
    if (MODE == MODE_CG_FUSED) return __ldcg(p);
    return *p;
}

// One sliding-window pass of a CTA over its (flat tile, x segment): y = D K D p on the owned
// nodes (PLAIN), or one PCG iteration with y = w_{i+1} (CG modes). sums[] receives this
// thread's FP32 shares of r.u, w.u and r.r (CG modes).
template <int NT, int EPT, int MAXN, int MODE>
__device__ __forceinline__ void modal_pass(const ModalGeom &G, const float *__restrict__ x,
                                           const float *__restrict__ p, float *__restrict__ y,
                                           const uint8_t *__restrict__ mask, const Law<float> &law,
                                           const ModalK &km, const CgPass &cp, float4 *smem4, int tile, int seg,
                                           float (&sums)[3]) {
    constexpr int NE = NT * EPT;
    constexpr bool CG = MODE == MODE_CG || MODE == MODE_CG_FUSED;
    static_assert(EPT == 2, "two elements per thread (packed FP32x2)");
    static_assert(MODE == MODE_PLAIN || CG, "modal pass modes: PLAIN, CG, CG_FUSED");

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

    float4 *Pn = smem4;                               // [3][R] operand planes (x, y, z, unused)
    float4 *Zn = Pn + 3 * R;                          // [3][R] M r_i of the same planes (CG)
    float2 *Es2 = (float2 *)(Pn + (CG ? 6 : 3) * R);  // [2][NT] element moduli (tid, tid + NT)
    float2 *Cc2 = Es2 + 2 * NT;                       // [24][NT] corner contributions (tid, tid + NT)
    const float *Cc = (const float *)Cc2;

    const float alpha = cp.alpha, beta = cp.beta;
    float g_ru = 0.0f, g_wu = 0.0f, g_rr = 0.0f;  // FP32 per-thread partials

    // ---- staging: issue the loads of a plane now, combine and store them later, so that
    // the element work of the current plane hides their latency ------------------------
    float ra[MAXN][3], rb[MAXN][3], rc[MAXN][3], rd[MAXN][3];  // PLAIN: p; CG: r_i, w_i, s_{i-1}, M
    uint8_t rm[MAXN];
    float ex[EPT];
    bool eok[EPT];
    auto stage_node = [&](int l, int j, int64_t &n) -> bool {
        const int flat = F0 - H + l;
        const bool ok = l < R && j >= 0 && j <= nx && flat >= 0 && flat < S;
        n = ok ? (int64_t)j * S + flat : 0;
        return ok;
    };
    auto issue_plane = [&](int j) {
#pragma unroll
        for (int q = 0; q < MAXN; ++q) {
            int64_t n;
            const bool ok = stage_node(tid + q * NT, j, n);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (!CG) {
                    ra[q][c] = ok ? p[3 * n + c] : 0.0f;
                } else {
                    ra[q][c] = ok ? ld_vec<MODE>(&cp.r[3 * n + c]) : 0.0f;
                    rb[q][c] = ok ? ld_vec<MODE>(&cp.w[3 * n + c]) : 0.0f;
                    rc[q][c] = ok ? ld_vec<MODE>(&cp.sold[3 * n + c]) : 0.0f;
                    rd[q][c] = ok ? cp.dinv[3 * n + c] : 0.0f;
                }
            }
            if (!CG) rm[q] = (ok && mask) ? mask[n] : (uint8_t)0;
        }
    };
    auto commit_plane = [&](int slot, int j) {
#pragma unroll
        for (int q = 0; q < MAXN; ++q) {
            const int l = tid + q * NT;
            if (!CG) {
                float v[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = ((rm[q] >> c) & 1) ? 0.0f : ra[q][c];
                if (l < R) Pn[slot * R + l] = make_float4(v[0], v[1], v[2], 0.0f);
            } else {
                int64_t n;
                const bool ok = stage_node(l, j, n);
                const bool own = ok && l >= H && l < NE && j >= xs && j < xe;
                float u[3], z[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float s = fmaf(beta, rc[q][c], rb[q][c]);
                    const float rn = fmaf(-alpha, s, ra[q][c]);
                    u[c] = rd[q][c] * rn;
                    z[c] = rd[q][c] * ra[q][c];
                    if (own) {
                        cp.snew[3 * n + c] = s;
                        cp.rnew[3 * n + c] = rn;
                        g_ru = fmaf(rn, u[c], g_ru);
                        g_rr = fmaf(rn, rn, g_rr);
                    }
                }
                if (l < R) {
                    Pn[slot * R + l] = make_float4(u[0], u[1], u[2], 0.0f);
                    Zn[slot * R + l] = make_float4(z[0], z[1], z[2], 0.0f);
                }
            }
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
        Es2[slot * NT + tid] =
            make_float2(eok[0] ? modulus(law, ex[0]) : 0.0f, eok[1] ? modulus(law, ex[1]) : 0.0f);
    };

    // ---- prologue: node planes xs-1, xs and element plane xs-1 --------------------------
    issue_plane(xs - 1);
    commit_plane(0, xs - 1);
    issue_plane(xs);
    issue_eplane(xs - 1);
    commit_plane(1, xs);
    commit_eplane(0);
    __syncthreads();

    float acc[EPT][3];
#pragma unroll
    for (int q = 0; q < EPT; ++q) acc[q][0] = acc[q][1] = acc[q][2] = 0.0f;

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
                if (CG) {
                    ox[q][c] = ok ? ld_vec<MODE>(&cp.xu[3 * n + c]) : 0.0f;
                    op[q][c] = ok ? ld_vec<MODE>(&cp.p[3 * n + c]) : 0.0f;
                } else {
                    ox[q][c] = op[q][c] = 0.0f;
                }
            }
        }

        // ---- element plane i: elements tid and tid + NT as the two lanes of a float2 ----
        if (i >= 0 && i < nx) {
            const float2 E = Es2[es * NT + tid];
            float2 v[8][3];
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const int cx = b >> 2, cy = (b >> 1) & 1, cz = b & 1;
                const float4 *src = Pn + (cx ? s1 : s0) * R + tid + cy * NZ + cz;
                const float4 wa = src[0], wb = src[NT];
                v[b][0] = make_float2(wa.x, wb.x);
                v[b][1] = make_float2(wa.y, wb.y);
                v[b][2] = make_float2(wa.z, wb.z);
            }
            modal_element2(v, E, km);
#pragma unroll
            for (int b = 0; b < 8; ++b)
#pragma unroll
                for (int c = 0; c < 3; ++c) Cc2[(b * 3 + c) * NT + tid] = v[b][c];
        } else {
#pragma unroll
            for (int kk = 0; kk < 24; ++kk) Cc2[kk * NT + tid] = make_float2(0.0f, 0.0f);
        }
        if (more_nodes) commit_plane(s2, i + 2);
        if (more_elems) commit_eplane(es ^ 1);
        __syncthreads();

        // ---- owned nodes of plane i ------------------------------------------------------
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            const int t = tid + q * NT;
            if (t < F) {
                const int te[4] = {t + H, t + H - 1, t + 1, t};  // (cy,cz) = 00, 01, 10, 11
                int ce[4];  // float offset of element te in a Cc2 row
#pragma unroll
                for (int yz = 0; yz < 4; ++yz) ce[yz] = te[yz] >= NT ? 2 * (te[yz] - NT) + 1 : 2 * te[yz];
                float yv[3], nacc[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float s = acc[q][c], a1 = 0.0f;
#pragma unroll
                    for (int yz = 0; yz < 4; ++yz) {
                        s += Cc[(yz * 3 + c) * 2 * NT + ce[yz]];
                        a1 += Cc[((4 + yz) * 3 + c) * 2 * NT + ce[yz]];
                    }
                    yv[c] = s;
                    nacc[c] = a1;
                }
                const int flat = F0 + t;
                if (out_plane && flat < S) {
                    const int64_t n = (int64_t)i * S + flat;
                    float uc[3] = {0.0f, 0.0f, 0.0f}, zc[3] = {0.0f, 0.0f, 0.0f};
                    if (CG) {
                        const float4 wu = Pn[s0 * R + t + H], wz = Zn[s0 * R + t + H];
                        uc[0] = wu.x, uc[1] = wu.y, uc[2] = wu.z;
                        zc[0] = wz.x, zc[1] = wz.y, zc[2] = wz.z;
                    }
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float yc = ((om[q] >> c) & 1) ? 0.0f : yv[c];
                        y[3 * n + c] = yc;
                        if (CG) {
                            g_wu = fmaf(uc[c], yc, g_wu);
                            const float pc = fmaf(beta, op[q][c], zc[c]);
                            cp.p[3 * n + c] = pc;
                            cp.xu[3 * n + c] = fmaf(alpha, pc, ox[q][c]);
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[q][c] = nacc[c];
            }
        }
        __syncthreads();
    }
    sums[0] = g_ru;
    sums[1] = g_wu;
    sums[2] = g_rr;
}

// The scalar step at the end of PCG iteration i, from gamma = r_{i+1}.u_{i+1},
// delta = w_{i+1}.u_{i+1} and rho = r_{i+1}.r_{i+1} (all FP64). Returns the new state in
// (it, done, status, gamma_i -> gamma, alpha, beta):
//   stop when ||r_{i+1}|| < rtol ||D b|| (x_{i+1} is written), on a non-finite sum, or at
//   max_iter; otherwise beta_{i+1} = gamma_{i+1} / gamma_i and
//   alpha_{i+1} = gamma_{i+1} / (delta_{i+1} - beta_{i+1} gamma_{i+1} / alpha_i), whose
//   denominator is p_{i+1}.A p_{i+1} (breakdown when it is not positive).
__device__ __forceinline__ void cg_scalar_step(double gamma, double delta, double rho, double tol, double bnorm,
                                               int max_iter, int &it, int &done, int &status, double &gamma_i,
                                               double &alpha, double &beta) {
    it += 1;
    if (!isfinite(gamma) || !isfinite(delta) || !isfinite(rho)) {
        done = 1;
        status = GBS_ENONFINITE;
    } else if (sqrt(rho) < tol * bnorm) {
        done = 1;
    } else if (it >= max_iter) {
        done = 1;
        status = GBS_ENOTCONV;
    } else {
        const double b1 = gamma / gamma_i;
        const double den = delta - b1 * gamma / alpha;
        if (!(den > 0.0)) {
            done = 1;
            status = GBS_EBREAKDOWN;
        } else {
            alpha = gamma / den;
            beta = b1;
            gamma_i = gamma;
        }
    }
}

template <int NT, int EPT, int MAXN, int MODE>
__global__ void __launch_bounds__(NT, 2)
    apply_modal_kernel(ModalGeom G, const float *__restrict__ x, const float *__restrict__ p, float *__restrict__ y,
                       const uint8_t *__restrict__ mask, Law<float> law, const ModalK km, CgArgs ca) {
    extern __shared__ float4 smem4[];
    __shared__ double sred[32];
    const int tid = threadIdx.x;
    CgPass cp{0.0f, 0.0f, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int it = 0;
    if (MODE == MODE_CG) {
        const PcgScalars *sc = ca.sc;
        const int done = sc->done;
        it = sc->iter;
        const double a = sc->alpha[0], b = sc->beta;
        if (done) return;
        const int c = it & 1, nc = c ^ 1;
        cp = CgPass{(float)a, (float)b, ca.r[c], ca.w[c], ca.s[nc], ca.dinv, ca.r[nc], ca.s[c], ca.p, ca.xu};
        y = ca.w[nc];
    }
    float sums[3];
    modal_pass<NT, EPT, MAXN, MODE>(G, x, p, y, mask, law, km, cp, smem4, blockIdx.x, blockIdx.y, sums);
    if (MODE == MODE_CG) {
        const int nblk = gridDim.x * gridDim.y;
        const int bid = blockIdx.x + gridDim.x * blockIdx.y;
        double bs[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) bs[k] = block_sum((double)sums[k], sred);
        __shared__ bool last;
        if (tid == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) ca.partials[k * nblk + bid] = bs[k];
            __threadfence();
            last = (atomicAdd(&ca.sc->counter, 1u) == (unsigned)(nblk - 1));
        }
        __syncthreads();
        if (last) {
            __threadfence();
            double tot[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double s = 0.0;
                for (int b = tid; b < nblk; b += NT) s += ((volatile double *)ca.partials)[k * nblk + b];
                tot[k] = block_sum(s, sred);
            }
            if (tid == 0) {
                PcgScalars *sc = ca.sc;
                sc->counter = 0;
                if (!sc->freeze) {
                    int done = 0, status = GBS_OK;
                    double gamma_i = sc->rz, alpha = sc->alpha[0], beta = sc->beta;
                    cg_scalar_step(tot[0], tot[1], tot[2], sc->tol, sc->bnorm, sc->max_iter, it, done, status, gamma_i,
                                   alpha, beta);
                    sc->iter = it;
                    sc->rr = tot[2];
                    sc->pap = tot[1];
                    sc->rz = gamma_i;
                    sc->alpha[0] = alpha;
                    sc->beta = beta;
                    sc->status = status;
                    sc->done = done;
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

// Staged nodes per thread: R / NT = EPT + ceil((nz + 2) / NT).
inline bool modal_small_halo(int nz) { return nz + 2 <= kModalNT; }

// Resident CTAs per SM of a kernel that uses `smem` bytes of dynamic shared memory: the
// register limit (occupancy at no dynamic shared memory, queried once per device) and the
// shared-memory limit (1 KB of each CTA is reserved by the system).
inline int modal_resident(const gbsimp_ctx *ctx, const void *kern, int &reg_cache, size_t smem) {
    if (reg_cache == 0) {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, kModalNT, 0) != cudaSuccess || v < 1) v = 1;
        reg_cache = v;
    }
    int per_sm = reg_cache;
    if (ctx->smem_per_sm > 0) {
        const int by_smem = (int)((size_t)ctx->smem_per_sm / (smem + 1024));
        if (by_smem < per_sm) per_sm = by_smem;
    }
    return per_sm < 1 ? 1 : per_sm;
}

// Sets the kernel's dynamic shared-memory limit once per device (host calls only; done before
// any graph capture) and returns resident CTAs per SM for this z extent, or < 0 on error.
template <int MODE, int MAXN>
inline int modal_prepare_one(const gbsimp_ctx *ctx, int nz) {
    auto kern = apply_modal_kernel<kModalNT, kModalEPT, MAXN, MODE>;
    constexpr bool cg = MODE != MODE_PLAIN;
    static int set_cache[128] = {};  // benign races: every thread stores the same values
    static int reg_cache[128] = {};
    const int dev = ctx->device >= 0 && ctx->device < 128 ? ctx->device : 0;
    if (!set_cache[dev]) {
        const int smax = (int)modal_smem_bytes<kModalNT, kModalEPT>(446, cg);
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
        if (e != cudaSuccess) return -cuda_error(e, "cudaFuncSetAttribute(apply_modal_kernel)");
        set_cache[dev] = 1;
    }
    return modal_resident(ctx, (const void *)kern, reg_cache[dev], modal_smem_bytes<kModalNT, kModalEPT>(nz, cg));
}

template <int MODE>
inline int modal_prepare(const gbsimp_ctx *ctx, int nz) {
    return modal_small_halo(nz) ? modal_prepare_one<MODE, kModalEPT + 1>(ctx, nz)
                                : modal_prepare_one<MODE, kModalEPT + 2>(ctx, nz);
}

// Launches the modal kernel (MODE_PLAIN: y = D K D p; MODE_CG: one PCG iteration).
template <int MODE>
inline int launch_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                        const float *p, float *y, const uint8_t *mask, const CgArgs &ca, cudaStream_t st) {
    const int per_sm = modal_prepare<MODE>(ctx, nz);
    if (per_sm < 0) return -per_sm;
    const size_t smem = modal_smem_bytes<kModalNT, kModalEPT>(nz, MODE != MODE_PLAIN);
    const ModalGeom g = modal_geom(nx, ny, nz, ctx->num_sms, per_sm);
    if (modal_small_halo(nz))
        apply_modal_kernel<kModalNT, kModalEPT, kModalEPT + 1, MODE>
            <<<modal_grid(g), kModalNT, smem, st>>>(g, x, p, y, mask, law, ctx->km, ca);
    else
        apply_modal_kernel<kModalNT, kModalEPT, kModalEPT + 2, MODE>
            <<<modal_grid(g), kModalNT, smem, st>>>(g, x, p, y, mask, law, ctx->km, ca);
    GBS_LAUNCH_CHECK("apply_modal_kernel");
    return GBS_OK;
}

}  // namespace gbs
