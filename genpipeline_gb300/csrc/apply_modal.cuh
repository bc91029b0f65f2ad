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
// (flat = j*(nz+1) + k) and walks along x. A plane's R = F + 2(nz+2) staged nodes are one
// contiguous run of 3R words in every node vector, so one thread stages each vector's run
// with one bulk copy (cp.async.bulk, completion counted on an mbarrier) into a raw buffer,
// and every thread combines its 16-byte groups into the operand plane, kept in the staged
// word order, from which the element pair of a thread (tid, tid + NT) loads each corner
// value straight into the two lanes of a packed FP32x2 register. Per step the CTA computes
// one plane of elements from two operand planes while the copies of the plane after next
// are in flight. Each element's 24 corner contributions are combined along z with a warp
// shuffle (the element to the left is the lane to the left), along y through a 6-float
// shared slot per element, and along x in registers (the x+1 corners are carried to the
// next plane): one writer per node and DOF and a fixed summation order, except on the node
// planes that two x segments share in the one-kernel PCG, where the two halves are added
// onto zero (the same result in either order).
#pragma once

#include "apply_tile.cuh"

namespace gbs {

struct ModalGeom {
    int nx, ny, nz;
    // x segments: segment s covers planes [s seglen + min(s, rem), + seglen + (s < rem)) of the
    // nx + 1 node planes (nx element planes for MODE_CG)
    int nseg, seglen, rem;
};


// Row lengths of the shared-memory layout for R staged nodes per plane. A plane of R nodes
// takes ceil((3R + 3) / 4) float4 groups, at most MAXV per thread. The MAXV = 2 kernels lay
// out every R they take (R <= modal_r2) with the lengths of the largest one, so that the row
// offsets are compile-time immediates; the MAXV = 3 kernels size the rows to R.
template <int NT>
__host__ __device__ constexpr int modal_r2() { return (8 * NT - 5) / 3; }
__host__ __device__ constexpr int modal_rw(int R) { return 4 * ((3 * R + 6) / 4); }
template <int NT>
__host__ __device__ constexpr int modal_layout_r(int R) { return (3 * R + 6) / 4 <= 2 * NT ? modal_r2<NT>() : R; }

// Shared memory of the modal kernel for a given z extent (NT = 256, EPT = 2): four operand
// planes and the raw bulk-copy buffers (one per staged vector: p for the plain apply; r, w,
// s, 1/diag, p, x for the PCG modes), modal_rw floats each, two planes of element moduli, and
// two copies (by step parity) of the y-direction slots (3 floats per element) and of the
// warp-boundary contributions (6 floats per warp and lane).
template <int NT, int EPT>
inline size_t modal_smem_bytes(int nz, bool cg) {
    const int NE = NT * EPT, H = nz + 2, R = modal_layout_r<NT>(NE + H);
    const size_t RW = (size_t)modal_rw(R);
    return 4 * RW * sizeof(float) + (cg ? 6 : 1) * RW * sizeof(float) + (2 + 6) * (size_t)NT * sizeof(float2) +
           2 * (size_t)(NT / 32) * 6 * sizeof(float2);
}

// cp.async (sm_80+): 16-byte global -> shared copies through L2 that use no registers;
// src_bytes < 16 copies that many bytes and zero-fills the rest.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Bulk copies (sm_90+): one thread moves a contiguous range global -> shared (16-byte aligned
// addresses, size a multiple of 16); an mbarrier counts the bytes that have landed.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// The issuing thread's arrival, announcing the bytes its copies will deliver in this phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// Orders this thread's earlier shared-memory accesses before later bulk copies into them.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// A bulk prefetch of a global range into L2 (sm_90+; 16-byte aligned, a multiple of 16 bytes):
// no shared memory and no completion to wait for.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for phase `parity` of the barrier to complete, at most kBulkWaitTries polls (each
// poll suspends for a hardware-defined time); false when the limit ran out.
constexpr unsigned kBulkWaitTries = 1u << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    for (unsigned t = 0; t < kBulkWaitTries; ++t)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ float2 shfl_up2(float2 v) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
}

// Packed FP32x2 helpers (sm_100+): lane .x belongs to one element, lane .y to another.
// a - b is fma(b, -1, a), which rounds exactly like the subtraction.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// Two elements at once: corners v[b][c] (b = cx*4 + cy*2 + cz) -> E (Ke p_e)_b,c for each
// lane. The operations and their order per lane are those of the scalar form: forward
// butterflies, r = Km q (each row summed in column order), r *= E, inverse butterflies.
// With XONLY the inverse stops after its x stage: v[b] (b < 4) is then the (y, z)-modal cx = 0
// half and v[4 + b] the cx = 1 half, to be summed per node plane before yz_inverse2.
template <bool XONLY>
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
    // inverse: (r0, r1) -> (r0 - r1, r0 + r1) along each axis (x first; the stages commute)
#pragma unroll
    for (int dd = 0; dd < (XONLY ? 1 : 3); ++dd) {
        const int bit = 4 >> dd;
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

// The (y, z) stages of the inverse transform on one node plane's four corners
// (b = cy * 2 + cz): (r0, r1) -> (r0 - r1, r0 + r1) along z, then along y.
__device__ __forceinline__ void yz_inverse2(float2 (&h)[4][3]) {
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float2 r0 = h[b][c], r1 = h[b | bit][c];
                h[b][c] = sub2(r0, r1);
                h[b | bit][c] = add2(r0, r1);
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
    float *clear;     // MODE_CG: the next launch's output w (its shared node planes are zeroed here)
    PcgScalars *sc;   // MODE_CG: where a copy wait that ran out records GBS_ETIMEOUT
    // x update: 0 none; 1 x += alpha p_i every iteration; 2 two iterations at once,
    // x_{i+1} = x_{i-1} + (alpha_{i-1} + alpha_i beta_i) p_{i-1} + alpha_i u_i (the odd
    // launches of the one-kernel PCG; the even ones use 0)
    int xmode;
};

template <int MODE>
__device__ __forceinline__ float ld_vec(const float *p) {
    if (MODE == MODE_CG_FUSED) return __ldcg(p);
    return *p;
}

// One sliding-window pass of a CTA over its (flat tile, x segment): y = D K D p on the owned
// nodes (PLAIN; x = densities), or one PCG iteration with y = w_{i+1} (CG modes; x = the
// element moduli E(x_e), computed once per solve). sums[] receives this
// thread's FP32 shares of r.u, w.u and r.r (CG modes). Every node vector must be 16-byte
// aligned. pre(alpha, beta, alpha_prev) runs once the first plane's copies are in flight (the
// step's scalars can be formed meanwhile); when it returns false the pass stops there
// (returns false).
//
// Segments. PLAIN and CG_FUSED: segment s owns node planes [xs, xe) of nx + 1 and also
// computes element plane xs - 1 (a halo step) so that every owned node sums all its elements.
// CG: segment s computes element planes [xs, xe) of nx, owns node planes [xs, xe) (the last
// segment also node plane nx) and outputs node planes xs..xe. Node plane xs of s > 0 and node
// plane xe < nx each get one half from this segment and one from its neighbour; both add
// their halves into y, which the launch before cleared on those planes (cp.clear). Two
// additions onto zero give the same result in either order, so the sum stays deterministic,
// and the w.u shares add up the same way. That saves the halo step's element work and one
// staged plane per CTA.
template <int NT, int EPT, int MAXV, int MODE, typename Pre>
__device__ __forceinline__ bool modal_pass(const ModalGeom &G, const float *__restrict__ x,
                                           const float *__restrict__ p, float *__restrict__ y,
                                           const uint8_t *__restrict__ mask, const Law<float> &law,
                                           const ModalK &km, const CgPass &cp, float *smem, int tile, int seg,
                                           float (&sums)[3], Pre &&pre) {
    constexpr int NE = NT * EPT;
    constexpr bool CG = MODE == MODE_CG || MODE == MODE_CG_FUSED;
    constexpr int NR = CG ? 6 : 1;  // staged vectors
    static_assert(EPT == 2, "two elements per thread (packed FP32x2)");
    static_assert(NT % 32 == 0, "whole warps");
    static_assert(MODE == MODE_PLAIN || CG, "modal pass modes: PLAIN, CG, CG_FUSED");

    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const int NZ = nz + 1;
    const int S = (ny + 1) * NZ;  // nodes per x plane
    const int H = nz + 2;         // flat halo (one y row plus one node)
    const int R = NE + H;         // staged nodes per plane
    const int F = NE - H;         // owned nodes per plane (chunk positions [H, NE))
    const int F0 = tile * F;
    constexpr bool EDGE = MODE == MODE_CG;
    const int xs = seg * G.seglen + min(seg, G.rem);
    const int xe = min(xs + G.seglen + (seg < G.rem ? 1 : 0), EDGE ? nx : nx + 1);
    const int own_hi = (EDGE && xe == nx) ? nx + 1 : xe;  // owned node planes [xs, own_hi)
    const int x0 = EDGE ? xs : xs - 1;                     // first element plane of the pass
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    static_assert(MAXV == 2 || MAXV == 3, "two or three float4 groups per thread and plane");
    const int RL = MAXV == 2 ? modal_r2<NT>() : R;  // layout rows (constant for MAXV = 2)
    const int RW = modal_rw(RL);
    const int64_t NW = 3LL * (nx + 1) * S;  // words of a node vector

    // One barrier per plane step: the operand planes are a ring of four slots and the y-slots
    // and warp-boundary terms alternate by step parity, so that a step's writes never meet
    // the previous step's reads of the same buffer (a slot is rewritten two barriers after
    // its last read).
    float *Pn = smem;                           // [4][RW] operand planes in the staged word order
    float *Raw = Pn + 4 * RW;                   // [NR][RW] bulk-copy buffers
    float2 *Es2 = (float2 *)(Raw + NR * RW);    // [2][NT] element moduli (tid, tid + NT)
    float2 *Z1s = Es2 + 2 * NT;                 // [2][3][NT] y+1-side contributions (c) per element
    float2 *Bd = Z1s + 6 * NT;                  // [2][NT/32][6] z+1-side contributions (cy, c) of lane 31

    float alpha = cp.alpha, beta = cp.beta, alpha_prev = 0.0f, c1 = 0.0f;
    float g_ru = 0.0f, g_wu = 0.0f, g_rr = 0.0f;  // FP32 per-thread partials
    sums[0] = sums[1] = sums[2] = 0.0f;

    auto src_of = [&](int a) -> const float * {
        if (!CG) return p;
        return a == 0 ? cp.r : a == 1 ? cp.w : a == 2 ? cp.sold : a == 3 ? cp.dinv : a == 4 ? cp.p : cp.xu;
    };
    // Word geometry of node plane j: the chunk's words start at W0 = 3 (j S + F0 - H); group f
    // holds the aligned words [A + 4f, A + 4f + 4), chunk words 4f - pad .. 4f - pad + 3.
    struct PlaneW {
        int64_t A;
        int pad, nv, lo3, hi3, olo3, ohi3;
        bool pv, own;
    };
    // W0 mod 4 of node plane j (the PlaneW pad), in unsigned arithmetic (wraps mod 2^32)
    auto plane_pad = [&](int j) -> int {
        return (int)((3u * ((unsigned)j * (unsigned)S + (unsigned)(F0 - H))) & 3u);
    };
    auto plane_w = [&](int j) {
        PlaneW P;
        const int64_t W0 = 3 * ((int64_t)j * S + F0 - H);
        P.A = W0 & ~(int64_t)3;
        P.pad = (int)(W0 - P.A);
        P.nv = (P.pad + 3 * R + 3) / 4;
        P.pv = j >= 0 && j <= nx;
        P.lo3 = 3 * max(0, H - F0);          // chunk words of nodes inside the plane
        P.hi3 = 3 * min(R, S - F0 + H);
        P.own = j >= xs && j < own_hi;
        P.olo3 = 3 * H;                      // chunk words of owned nodes
        P.ohi3 = 3 * min(NE, S - F0 + H);
        return P;
    };

    // ---- staging ---------------------------------------------------------------------------
    // Bulk copies: thread 0 copies the plane's whole 16-byte groups of p (plain apply) or of r,
    // w, s and 1/diag, and the owned groups of p and x (PCG modes), one copy per vector, and an
    // mbarrier phase per plane counts the bytes. Only a group cut by the end of the vectors is
    // copied by its thread with cp.async (zero-filled). The raw buffers are rewritten only after
    // a block barrier that follows every thread's reads of the previous plane.
    constexpr int NF = CG ? 4 : 1;  // vectors staged over the whole plane
    __shared__ unsigned long long s_bar;
    unsigned bphase = 0;  // phase of the plane being committed
    bool bulk_ok = true;  // false once a wait ran out (then no further waits)
    if (tid == 0) mbar_init(&s_bar, 1);
    __syncthreads();
    auto bulk_wait = [&]() {
        if (bulk_ok && !mbar_wait(&s_bar, bphase)) {
            bulk_ok = false;
            if (cp.sc) {
                atomicExch(&cp.sc->status, (int)GBS_ETIMEOUT);
                atomicExch(&cp.sc->done, 1);
            }
        }
        bphase ^= 1u;
    };
    const int64_t full = NW & ~(int64_t)3;  // words of the vectors in whole 16-byte groups
    // Whole 16-byte groups of node plane j: [g0, g0 + nfull) of the plane-wide vectors and
    // [o0, o0 + nown) of the owned ones (p, x).
    auto plane_ranges = [&](int j, int64_t &g0, unsigned &nfull, int64_t &o0, unsigned &nown) {
        const PlaneW P = plane_w(j);
        nfull = 0;
        nown = 0;
        g0 = 0;
        o0 = 0;
        if (P.pv) {
            g0 = max(P.A, (int64_t)0);
            const int64_t g1 = min(P.A + 4 * (int64_t)P.nv, full);
            if (g1 > g0) nfull = (unsigned)(g1 - g0);
            if (CG && P.own) {  // groups that meet the owned words [olo3, ohi3)
                o0 = max(P.A + 4 * (int64_t)((P.olo3 + P.pad) >> 2), (int64_t)0);
                const int64_t o1 = min(P.A + 4 * (int64_t)((P.ohi3 + P.pad + 3) >> 2), full);
                if (o1 > o0) nown = (unsigned)(o1 - o0);
            }
        }
    };
    // L2 prefetch of node plane j (the plane after the one whose copies are in flight): its
    // DRAM reads start a step earlier than its copies into shared memory, with no shared memory
    // held for them.
    auto prefetch_plane = [&](int j) {
        int64_t g0, o0;
        unsigned nfull, nown;
        plane_ranges(j, g0, nfull, o0, nown);
        if (nfull)
#pragma unroll
            for (int a = 0; a < NF; ++a) bulk_prefetch_l2(src_of(a) + g0, 4u * nfull);
        if (CG && nown)
#pragma unroll
            for (int a = 4; a < 6; ++a)
                if (a == 4 || cp.xmode) bulk_prefetch_l2(src_of(a) + o0, 4u * nown);
    };
    auto issue_plane = [&](int j) {
        {
            if (tid == 0) {
                const PlaneW P = plane_w(j);
                int64_t g0, o0;
                unsigned nfull, nown;
                plane_ranges(j, g0, nfull, o0, nown);
                const unsigned nown_vec = cp.xmode ? 2u : 1u;  // p, and x when it is updated
                mbar_arrive_expect_tx(&s_bar, 4u * (NF * nfull + nown_vec * nown));
                fence_proxy_async();
                if (nfull)
#pragma unroll
                    for (int a = 0; a < NF; ++a)
                        bulk_copy_g2s(Raw + a * RW + (g0 - P.A), src_of(a) + g0, 4u * nfull, &s_bar);
                if (CG && nown)
#pragma unroll
                    for (int a = 4; a < 6; ++a)
                        if (a == 4 || cp.xmode)
                            bulk_copy_g2s(Raw + a * RW + (o0 - P.A), src_of(a) + o0, 4u * nown, &s_bar);
                // the PCG modes (several vectors per plane): the plain apply measured no gain
                if (CG && j + 1 <= xe) prefetch_plane(j + 1);  // xe: the segment's last staged plane
            }
            // the group cut by the end of the vectors: only the last node plane reaches it
            if (j == nx && full < NW) {
                const PlaneW P = plane_w(j);
                const int64_t ft = full >= P.A ? (full - P.A) >> 2 : (int64_t)P.nv;
                if (ft < P.nv && (int)(ft % NT) == tid) {
                    const int f = (int)ft, cw0 = 4 * f - P.pad;
                    const int nb = 4 * (int)(NW - full);
                    const bool ownable = P.own && cw0 + 4 > P.olo3 && cw0 < P.ohi3;
#pragma unroll
                    for (int a = 0; a < NR; ++a)
                        if (a < NF || (ownable && (a == 4 || cp.xmode)))
                            cp_async16(Raw + a * RW + 4 * f, src_of(a) + full, nb);
                }
            }
            cp_async_commit();
        }
    };
    // Combines the staged groups of plane j into operand slot
    // `slot`; in the PCG modes also updates s, r, p and x of the owned words. Interior groups
    // (all four words inside the plane, and all or none owned) take a branch-free path.
    auto commit_plane = [&](int slot, int j) {
        const PlaneW P = plane_w(j);
        cp_async_wait_all();
        bulk_wait();
        float *Pf = Pn + slot * RW;  // group f at Pf[4f]: component c of chunk node l at Pf[pad + 3 l + c]
#pragma unroll
        for (int q = 0; q < MAXV; ++q) {
            const int f = tid + q * NT;
            if (f < P.nv) {
                const int cw0 = 4 * f - P.pad;
                const int64_t gw = P.A + 4 * (int64_t)f;
                const bool in_all = P.pv && cw0 >= P.lo3 && cw0 + 4 <= P.hi3;
                const bool own_all = in_all && P.own && cw0 >= P.olo3 && cw0 + 4 <= P.ohi3;
                const bool own_none = !P.own || cw0 + 4 <= P.olo3 || cw0 >= P.ohi3;
                float val[4];
                if (!CG) {
                    const float4 a4 = *(const float4 *)(Raw + 4 * f);
                    const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int cw = cw0 + k;
                        const bool valid = in_all || (P.pv && cw >= P.lo3 && cw < P.hi3);
                        bool fixed = false;
                        if (mask && valid) {
                            const int l = cw / 3;
                            fixed = (mask[(int64_t)j * S + F0 - H + l] >> (cw - 3 * l)) & 1;
                        }
                        val[k] = valid && !fixed ? av[k] : 0.0f;
                    }
                } else {
                    const float4 r4 = *(const float4 *)(Raw + 0 * RW + 4 * f);
                    const float4 w4 = *(const float4 *)(Raw + 1 * RW + 4 * f);
                    const float4 s4 = *(const float4 *)(Raw + 2 * RW + 4 * f);
                    const float4 d4 = *(const float4 *)(Raw + 3 * RW + 4 * f);
                    const float rv[4] = {r4.x, r4.y, r4.z, r4.w}, wv[4] = {w4.x, w4.y, w4.z, w4.w};
                    const float sv[4] = {s4.x, s4.y, s4.z, s4.w}, dv[4] = {d4.x, d4.y, d4.z, d4.w};
                    float so[4], rno[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        so[k] = fmaf(beta, sv[k], wv[k]);
                        rno[k] = fmaf(-alpha, so[k], rv[k]);
                        val[k] = dv[k] * rno[k];
                    }
                    if (own_all) {
                        const float4 p4 = *(const float4 *)(Raw + 4 * RW + 4 * f);
                        const float4 x4 = cp.xmode ? *(const float4 *)(Raw + 5 * RW + 4 * f) : make_float4(0, 0, 0, 0);
                        const float pv[4] = {p4.x, p4.y, p4.z, p4.w}, xv[4] = {x4.x, x4.y, x4.z, x4.w};
                        float po[4], xo[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            const float ur = dv[k] * rv[k];  // u_i = M r_i
                            po[k] = fmaf(beta, pv[k], ur);
                            xo[k] = cp.xmode == 2 ? fmaf(c1, pv[k], fmaf(alpha, ur, xv[k])) : fmaf(alpha, po[k], xv[k]);
                            g_ru = fmaf(rno[k], val[k], g_ru);
                            g_rr = dv[k] != 0.0f ? fmaf(rno[k], rno[k], g_rr) : g_rr;  // free DOFs only
                        }
                        *(float4 *)(cp.snew + gw) = make_float4(so[0], so[1], so[2], so[3]);
                        *(float4 *)(cp.rnew + gw) = make_float4(rno[0], rno[1], rno[2], rno[3]);
                        *(float4 *)(cp.p + gw) = make_float4(po[0], po[1], po[2], po[3]);
                        if (cp.xmode) *(float4 *)(cp.xu + gw) = make_float4(xo[0], xo[1], xo[2], xo[3]);
                    } else if (!(in_all && own_none)) {
                        // edge group: word by word
                        const bool any_own = !own_none;
                        float pv[4] = {0.0f, 0.0f, 0.0f, 0.0f}, xv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                        if (any_own) {
                            const float4 p4 = *(const float4 *)(Raw + 4 * RW + 4 * f);
                            pv[0] = p4.x, pv[1] = p4.y, pv[2] = p4.z, pv[3] = p4.w;
                            if (cp.xmode) {
                                const float4 x4 = *(const float4 *)(Raw + 5 * RW + 4 * f);
                                xv[0] = x4.x, xv[1] = x4.y, xv[2] = x4.z, xv[3] = x4.w;
                            }
                        }
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            const int cw = cw0 + k;
                            const bool valid = P.pv && cw >= P.lo3 && cw < P.hi3;
                            const bool own = valid && any_own && cw >= P.olo3 && cw < P.ohi3;
                            if (!valid) val[k] = 0.0f;
                            if (own) {
                                const float ur = dv[k] * rv[k];
                                const float po = fmaf(beta, pv[k], ur);
                                cp.snew[gw + k] = so[k];
                                cp.rnew[gw + k] = rno[k];
                                cp.p[gw + k] = po;
                                if (cp.xmode)
                                    cp.xu[gw + k] =
                                        cp.xmode == 2 ? fmaf(c1, pv[k], fmaf(alpha, ur, xv[k])) : fmaf(alpha, po, xv[k]);
                                g_ru = fmaf(rno[k], val[k], g_ru);
                                g_rr = dv[k] != 0.0f ? fmaf(rno[k], rno[k], g_rr) : g_rr;
                            }
                        }
                    }
                }
                *(float4 *)(Pf + 4 * f) = make_float4(val[0], val[1], val[2], val[3]);
            }
        }
    };
    // Zeroes this CTA's owned words of node plane j in cp.clear (MODE_CG: a shared plane of the
    // next launch's output).
    auto clear_plane = [&](int j) {
        const PlaneW P = plane_w(j);
#pragma unroll
        for (int q = 0; q < MAXV; ++q) {
            const int f = tid + q * NT;
            const int cw0 = 4 * f - P.pad;
            if (f < P.nv && cw0 + 4 > P.olo3 && cw0 < P.ohi3) {
                const int64_t gw = P.A + 4 * (int64_t)f;
                if (cw0 >= P.olo3 && cw0 + 4 <= P.ohi3) {
                    *(float4 *)(cp.clear + gw) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (cw0 + k >= P.olo3 && cw0 + k < P.ohi3) cp.clear[gw + k] = 0.0f;
                }
            }
        }
    };
    float ex[EPT];
    bool eok[EPT];
    // (y, z) offset ey nz + ez of element tid + q NT within an element plane, -1 outside the
    // grid (loop-invariant: the integer division by NZ runs once per pass)
    int eoff[EPT];
#pragma unroll
    for (int q = 0; q < EPT; ++q) {
        const int ef = F0 - H + tid + q * NT;
        const int ey = ef >= 0 ? ef / NZ : 0, ez = ef >= 0 ? ef - ey * NZ : 0;
        eoff[q] = ef >= 0 && ey < ny && ez < nz ? ey * nz + ez : -1;
    }
    const int64_t eplane = (int64_t)ny * nz;
    auto issue_eplane = [&](int j) {
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            eok[q] = j >= 0 && j < nx && eoff[q] >= 0;
            ex[q] = eok[q] ? x[j * eplane + eoff[q]] : 0.0f;
        }
    };
    // PLAIN: x holds densities and the law gives the moduli; CG modes: x already holds the
    // moduli E(x_e) of the solve (issue_eplane leaves 0 outside the grid)
    auto commit_eplane = [&](int slot) {
        if (CG)
            Es2[slot * NT + tid] = make_float2(ex[0], ex[1]);
        else
            Es2[slot * NT + tid] =
                make_float2(eok[0] ? modulus(law, ex[0]) : 0.0f, eok[1] ? modulus(law, ex[1]) : 0.0f);
    };
    // Index in Bdf of the z+1-side contribution (cy, c = 0) of element e - 1, for an element e
    // in lane 0; component c adds 2 c.
    auto bd_index = [&](int e, int cy) -> int {
        const int pe = e - 1;
        const int pt = pe >= NT ? pe - NT : pe;
        return 2 * ((pt >> 5) * 6 + cy * 3) + (pe >= NT ? 1 : 0);
    };
    // Node-phase terms of node l = tid + q NT that come from other warps (loop-invariant):
    // bl[q] for lane 0 (element l - 1 in lane 31 of the previous warp), bm[q] for the node
    // whose y-neighbour element m = l - NZ sits in lane 0; -1 where there is none.
    int bl[EPT], bm[EPT];
    // node l of this thread: owned-range test (node_ok), slot of its y-neighbour element m in
    // the y-slots (zi), and its flat index in the plane (loop-invariant)
    int zi[EPT], nflat[EPT];
    bool node_ok[EPT];
#pragma unroll
    for (int q = 0; q < EPT; ++q) {
        const int l = tid + q * NT, mm = l - NZ;
        const bool node = l >= H;  // then l >= 1 and m >= 1
        bl[q] = node && lane == 0 ? bd_index(l, 0) : -1;
        bm[q] = node && (mm & 31) == 0 ? bd_index(mm, 1) : -1;
        nflat[q] = F0 - H + l;
        node_ok[q] = node && nflat[q] < S;
        zi[q] = mm >= NT ? 2 * (mm - NT) + 1 : 2 * mm;
    }

    // ---- prologue: node planes x0, x0 + 1 and element plane x0 (the raw buffers hold one
    // plane: the second plane's copies go out after the first plane is combined) ----------
    issue_plane(x0);
    issue_eplane(x0);
    if (!pre(alpha, beta, alpha_prev)) {
        cp_async_wait_all();  // no copy may land after the CTA has left
        bulk_wait();
        return false;
    }
    c1 = fmaf(alpha, beta, alpha_prev);  // the two-step x update's coefficient of p_{i-1}
    commit_plane(0, x0);
    __syncthreads();  // every thread's reads of the raw buffers before they are refilled
    issue_plane(x0 + 1);
    commit_eplane(0);
    commit_plane(1, x0 + 1);
    if (EDGE && xs > 0) clear_plane(xs);
    __syncthreads();

    // x-direction carry: the cx = 1 half of element plane i - 1 in the (y, z) modal basis,
    // which belongs to node plane i together with the cx = 0 half of element plane i
    float2 g1[4][3];
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int c = 0; c < 3; ++c) g1[b][c] = make_float2(0.0f, 0.0f);

    // steps x0..xlast: element plane i (while i < xe, or i < nx with a halo step) and node
    // plane i out (from xs on)
    const int xlast = EDGE ? xe : xe - 1;
    for (int i = x0; i <= xlast; ++i) {  // modal_geom makes every segment non-empty
        const int k = i - x0;
        const int s0 = k & 3, s1 = (k + 1) & 3, s2 = (k + 2) & 3;
        // component c of chunk node l: plane i at P0[3 l + c], plane i + 1 at P1[3 l + c]
        const float *P0 = Pn + s0 * RW + plane_pad(i), *P1 = Pn + s1 * RW + plane_pad(i + 1);
        float2 *Z1k = Z1s + (k & 1) * 3 * NT, *Bdk = Bd + (k & 1) * (NT / 32) * 6;
        const int es = k & 1;
        const bool more_nodes = i + 2 <= xe;
        const bool more_elems = i + 1 <= xe - 1;
        if (more_nodes) issue_plane(i + 2);
        if (more_elems) issue_eplane(i + 1);
        const bool out_plane = EDGE || i >= xs;
        const bool shared = EDGE && ((i == xs && xs > 0) || (i == xe && xe < nx));  // added, not stored
        uint8_t om[EPT];
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            const int l = tid + q * NT;
            const bool ok = out_plane && l >= H && F0 - H + l < S;
            om[q] = (!CG && ok && mask) ? mask[(int64_t)i * S + F0 - H + l] : (uint8_t)0;
        }

        // ---- element plane i: elements tid and tid + NT as the two lanes of a float2 ----
        // h: the contributions of element planes i - 1 (carried) and i to node plane i, summed
        // in the (y, z) modal basis, then transformed back
        float2 h[4][3];
        if (EDGE ? i < xe : (i >= 0 && i < nx)) {
            const float2 E = Es2[es * NT + tid];
            float2 v[8][3];
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const int cx = b >> 2, cy = (b >> 1) & 1, cz = b & 1;
                const float *src = (cx ? P1 : P0) + 3 * (tid + cy * NZ + cz);
#pragma unroll
                for (int c = 0; c < 3; ++c) v[b][c] = make_float2(src[c], src[c + 3 * NT]);
            }
            modal_element2<true>(v, E, km);
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    h[b][c] = add2(v[b][c], g1[b][c]);
                    g1[b][c] = v[4 + b][c];
                }
        } else {
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    h[b][c] = g1[b][c];
                    g1[b][c] = make_float2(0.0f, 0.0f);
                }
        }
        yz_inverse2(h);  // h[cy * 2 + cz]: contribution to corner (cy, cz) of node plane i
        // z: the cz = 1 corners of element e - 1 (lane - 1) join the cz = 0 corners of e
        float2 z0[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            float2 a1 = shfl_up2(h[1][c]), b1 = shfl_up2(h[3][c]);
            if (lane == 0) a1 = b1 = make_float2(0.0f, 0.0f);
            z0[c] = add2(h[0][c], a1);
            Z1k[c * NT + tid] = add2(h[2][c], b1);
        }
        if (lane == 31) {
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                for (int c = 0; c < 3; ++c) Bdk[warp * 6 + cy * 3 + c] = h[cy * 2 + 1][c];
        }
        if (more_nodes) commit_plane(s2, i + 2);
        if (more_elems) commit_eplane(es ^ 1);
        __syncthreads();

        // ---- nodes of plane i: node l = element l of this thread, stored straight to y -----
        const float *Pu = P0;
        const float *Z1f = (const float *)Z1k, *Bdf = (const float *)Bdk;
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
            const int l = tid + q * NT;
            if (node_ok[q] && out_plane) {
                // zi[q]: the y+1 corners of element l - NZ (>= 1), which touch node l
                float yc[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    float s = (q ? z0[c].y : z0[c].x) + Z1f[c * 2 * NT + zi[q]];
                    const float tl = Bdf[max(bl[q], 0) + 2 * c], tm = Bdf[max(bm[q], 0) + 2 * c];
                    s += bl[q] >= 0 ? tl : 0.0f;
                    s += bm[q] >= 0 ? tm : 0.0f;
                    // PCG modes leave w unmasked: 1/diag = 0 keeps u, p and x at zero on fixed
                    // DOFs whatever w holds there, and r.r skips them (the plain apply masks)
                    yc[c] = (!CG && ((om[q] >> c) & 1)) ? 0.0f : s;
                }
                if (CG) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) g_wu = fmaf(Pu[3 * l + c], yc[c], g_wu);
                }
                float *yo = y + 3 * ((int64_t)i * S + nflat[q]);
                if (shared) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) atomicAdd(yo + c, yc[c]);
                } else {
#pragma unroll
                    for (int c = 0; c < 3; ++c) yo[c] = yc[c];
                }
            }
        }
    }
    sums[0] = g_ru;
    sums[1] = g_wu;
    sums[2] = g_rr;
    return true;
}

// The scalar step at the end of PCG iteration i, from gamma = r_{i+1}.u_{i+1},
// delta = w_{i+1}.u_{i+1} and rho = r_{i+1}.r_{i+1}, all in double-float. Returns the new
// state in (it, done, status, gamma_i -> gamma, alpha, beta):
//   stop when r.r < rr_stop = (rtol ||D b||)^2 (x_{i+1} is written; r.r = 0 also stops, for a
//   threshold below the FP32 range), on a non-finite sum, or at max_iter; otherwise
//   beta_{i+1} = gamma_{i+1} / gamma_i and
//   alpha_{i+1} = gamma_{i+1} / (delta_{i+1} - beta_{i+1} gamma_{i+1} / alpha_i), whose
//   denominator is p_{i+1}.A p_{i+1} (breakdown when it is not positive).
__device__ __forceinline__ void cg_scalar_step_df(df32 gamma, df32 delta, df32 rho, float rr_stop, int max_iter,
                                                  int &it, int &done, int &status, df32 &gamma_i, df32 &alpha,
                                                  df32 &beta) {
    it += 1;
    if (!isfinite(gamma.hi) || !isfinite(delta.hi) || !isfinite(rho.hi)) {
        done = 1;
        status = GBS_ENONFINITE;
    } else if (rho.hi < rr_stop || rho.hi == 0.0f) {
        done = 1;
    } else if (it >= max_iter) {
        done = 1;
        status = GBS_ENOTCONV;
    } else {
        const df32 b1 = df_div(gamma, gamma_i);
        const df32 den = df_add(delta, df_neg(df_mul(b1, df_div(gamma, alpha))));
        if (!(den.hi > 0.0f)) {
            done = 1;
            status = GBS_EBREAKDOWN;
        } else {
            alpha = df_div(gamma, den);
            beta = b1;
            gamma_i = gamma;
        }
    }
}

// The scalars of iteration 0 from the sums of a start pass (alpha = beta = 0 from x0 = 0:
// gamma = r_0.u_0, delta = w_0.u_0, rho = r_0.r_0 = ||D b||^2): alpha_0 = gamma / delta,
// beta_0 = 0. Stops at once on a non-finite sum, on D b = 0, or when rtol > 1 (x0 = 0 already
// meets ||r|| < rtol ||D b||); breakdown when delta is not positive.
__device__ __forceinline__ void cg_first_step_df(df32 gamma, df32 delta, df32 rho, double tol, int &done,
                                                 int &status, df32 &gamma_i, df32 &alpha, df32 &beta) {
    if (!isfinite(gamma.hi) || !isfinite(delta.hi) || !isfinite(rho.hi)) {
        done = 1;
        status = GBS_ENONFINITE;
    } else if (rho.hi == 0.0f || tol > 1.0) {
        done = 1;
    } else if (!(delta.hi > 0.0f)) {
        done = 1;
        status = GBS_EBREAKDOWN;
    } else {
        alpha = df_div(gamma, delta);
        beta = df32{0.0f, 0.0f};
        gamma_i = gamma;
    }
}

// CgState.pending: the sums of the pass that wrote the state are still to be folded (1); the
// same for a start pass (2: cg_first_step_df instead of the scalar step); the next launch is
// the start pass itself (3: nothing to fold, it runs with alpha = beta = 0).
enum { CG_PENDING_STEP = 1, CG_PENDING_FIRST = 2, CG_START_PASS = 3 };

// Folds the block partial sums (r.u, w.u, r.r; double-float, slot layout [k][nblk]) of the
// pass that started from state s into s: the scalar step of that iteration (of a start pass:
// the scalars of iteration 0). Every block of the next launch does it, in the same order
// (deterministic), instead of a last block of the pass. All threads of the block take part;
// nothing runs on the FP64 pipe.
template <int NT>
__device__ __forceinline__ void cg_fold(CgState &s, const PcgScalars *sc, const float2 *partials, int nblk,
                                        float2 *sred) {
    __shared__ CgState sh;
    df32 tot[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    for (int b = threadIdx.x; b < nblk; b += NT)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float2 v = __ldcg(&partials[k * nblk + b]);
            tot[k] = df_add(tot[k], df32{v.x, v.y});
        }
    block_sum_df<3>(tot, sred);
    if (threadIdx.x == 0) {
        int it = s.iter, done = 0, status = s.status;
        const df32 a_before = s.alpha;
        if (s.pending == CG_PENDING_FIRST)
            cg_first_step_df(tot[0], tot[1], tot[2], sc->tol, done, status, s.gamma, s.alpha, s.beta);
        else
            cg_scalar_step_df(tot[0], tot[1], tot[2], sc->rr_stop, sc->max_iter, it, done, status, s.gamma,
                              s.alpha, s.beta);
        if (!done) s.alpha_prev = a_before;
        s.iter = it;
        s.done = done;
        s.status = status;
        s.rr = tot[2];
        s.pap = tot[1];
        s.pending = 0;
        sh = s;
    }
    __syncthreads();
    s = sh;
}

// phase: k mod 6 for the k-th launch of a solve (the graph loop and the host loops know it
// statically); par = k & 1. MODE_CG reads state slot par ^ 1 and partial slot par ^ 1, writes
// state slot par (block 0) and partial slot par; w rotates by k mod 3 (CgArgs).
template <int NT, int EPT, int MAXV, int MODE>
__global__ void __launch_bounds__(NT, 2)
    apply_modal_kernel(ModalGeom G, const float *__restrict__ x, const float *__restrict__ p, float *__restrict__ y,
                       const uint8_t *__restrict__ mask, Law<float> law, const ModalK km, CgArgs ca, int phase) {
    extern __shared__ float4 smem4[];
    __shared__ float2 sred[3 * 32];
    const int tid = threadIdx.x;
    const int nblk = gridDim.x * gridDim.y;
    const int bid = blockIdx.x + gridDim.x * blockIdx.y;
    const int par = phase & 1;
    CgPass cp{0.0f, 0.0f, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    if (MODE == MODE_CG) {
        // Launch k runs iteration k while the solve lasts, so the vector parity is the launch
        // parity (and w cycles with k mod 3): the first plane's copies go out before the state
        // is known. Selects, not dynamic indices (those would copy the parameter arrays to the
        // stack).
        const bool odd = par;
        const int w3 = phase >= 3 ? phase - 3 : phase;
        float *r_c = odd ? ca.r[1] : ca.r[0], *r_n = odd ? ca.r[0] : ca.r[1];
        float *s_c = odd ? ca.s[1] : ca.s[0], *s_n = odd ? ca.s[0] : ca.s[1];
        float *w_c = w3 == 0 ? ca.w[0] : w3 == 1 ? ca.w[1] : ca.w[2];
        float *w_n = w3 == 0 ? ca.w[1] : w3 == 1 ? ca.w[2] : ca.w[0];
        float *w_z = w3 == 0 ? ca.w[2] : w3 == 1 ? ca.w[0] : ca.w[1];
        // x is updated on odd launches only, two iterations at a time
        cp = CgPass{0.0f, 0.0f, r_c, w_c, s_n, ca.dinv, r_n, s_c, ca.p, ca.xu, w_z, ca.sc, odd ? 2 : 0};
        y = w_n;
    }
    auto pre = [&](float &alpha, float &beta, float &alpha_prev) -> bool {
        if (MODE != MODE_CG) return true;
        const PcgScalars *sc = ca.sc;
        CgState s = sc->st[par ^ 1];
        if (!sc->freeze) {
            const int pend = s.pending;
            if ((pend == CG_PENDING_STEP || pend == CG_PENDING_FIRST) && !s.done) {
                cg_fold<NT>(s, sc, (const float2 *)ca.partials + (par ^ 1) * 3 * nblk, nblk, sred);
                if (pend == CG_PENDING_FIRST && bid == 0 && tid == 0) {
                    // the stop threshold (rtol ||D b||)^2 of the later folds, ||D b||^2 = r_0.r_0
                    const double bn = sqrt(df_value(s.rr));
                    const double stop = sc->tol * bn;
                    ca.sc->bnorm = bn;
                    ca.sc->rr_stop = (float)(stop * stop);
                }
            }
            if (bid == 0 && tid == 0) {
                CgState o = s;
                o.pending = s.done ? 0 : (pend == CG_START_PASS ? CG_PENDING_FIRST : CG_PENDING_STEP);
                ca.sc->st[par] = o;
            }
        }
        alpha = s.alpha.hi;
        beta = s.beta.hi;
        alpha_prev = s.alpha_prev.hi;
        return !s.done;
    };
    float sums[3];
    if (!modal_pass<NT, EPT, MAXV, MODE>(G, x, p, y, mask, law, km, cp, (float *)smem4, blockIdx.x, blockIdx.y, sums,
                                         pre))
        return;
    if (MODE == MODE_CG) {
        df32 bs[3] = {{sums[0], 0.0f}, {sums[1], 0.0f}, {sums[2], 0.0f}};
        block_sum_df<3>(bs, sred);
        if (tid == 0) {
            float2 *part = (float2 *)ca.partials + par * 3 * nblk;
#pragma unroll
            for (int k = 0; k < 3; ++k) part[k * nblk + bid] = make_float2(bs[k].hi, bs[k].lo);
        }
    }
}

// Launch geometry: NT = 256 threads, EPT = 2 (512 elements per plane step).
constexpr int kModalNT = 256;
constexpr int kModalEPT = 2;

inline bool modal_fits(int nz) { return nz + 2 <= kModalNT * kModalEPT - 64 && nz + 2 <= 2 * kModalNT; }

// edge: segments over the nx element planes (MODE_CG, shared boundary node planes), else
// over the nx + 1 node planes (a halo element plane per segment).
inline ModalGeom modal_geom(int nx, int ny, int nz, int num_sms, int blocks_per_sm, bool edge = false) {
    const int NE = kModalNT * kModalEPT, H = nz + 2, F = NE - H;
    const int S = (ny + 1) * (nz + 1);
    const int tiles = (S + F - 1) / F;
    const int planes = edge ? nx : nx + 1;
    const int target = (num_sms > 0 ? num_sms : 148) * (blocks_per_sm > 0 ? blocks_per_sm : 1);
    // As many x segments as fit in one wave of resident CTAs, of lengths that differ by at
    // most one plane (64 element planes in 30 segments: 4 of 3 planes and 26 of 2, rather
    // than 22 of 3).
    int nseg = target / tiles;
    if (nseg > planes) nseg = planes;
    if (nseg < 1) nseg = 1;
    ModalGeom g{nx, ny, nz, nseg, planes / nseg, planes % nseg};
    return g;
}

// Flat tiles of one (y, z) node plane: the CTAs of one x segment (modal_fits(nz) holds).
inline int modal_tiles(int ny, int nz) {
    const int F = kModalNT * kModalEPT - (nz + 2);
    return ((ny + 1) * (nz + 1) + F - 1) / F;
}

// Upper bound on one wave of resident modal CTAs (SMs x CTAs per SM) that workspaces are
// sized for; a launch of max(tiles, wave) CTAs beyond what a workspace holds is refused.
constexpr int kModalMaxWave = 2048;

inline dim3 modal_grid(const ModalGeom &g) { return dim3((unsigned)modal_tiles(g.ny, g.nz), (unsigned)g.nseg, 1); }

// 16-byte groups of a staged plane per thread: 2 when 4 * ceil((3R + 3) / 4) <= 8 NT words
// (nz <= 167), else 3 (modal_fits bounds nz).
inline bool modal_short(int nz) { return (3 * (kModalNT * kModalEPT + nz + 2) + 6) / 4 <= 2 * kModalNT; }

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
template <int MODE, int MAXV>
inline int modal_prepare_one(const gbsimp_ctx *ctx, int nz) {
    auto kern = apply_modal_kernel<kModalNT, kModalEPT, MAXV, MODE>;
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
    return modal_short(nz) ? modal_prepare_one<MODE, 2>(ctx, nz) : modal_prepare_one<MODE, 3>(ctx, nz);
}

// CTAs of the modal kernel's launch for a grid (the partial sums of one MODE_CG pass).
template <int MODE>
inline int modal_blocks(const gbsimp_ctx *ctx, int nx, int ny, int nz) {
    const int per_sm = modal_prepare<MODE>(ctx, nz);
    if (per_sm < 0) return per_sm;
    const dim3 g = modal_grid(modal_geom(nx, ny, nz, ctx->num_sms, per_sm, MODE == MODE_CG));
    return (int)(g.x * g.y);
}

// Launches the modal kernel (MODE_PLAIN: y = D K D p; MODE_CG: one PCG iteration, phase =
// launch index mod 6).
template <int MODE>
inline int launch_modal(const gbsimp_ctx *ctx, int nx, int ny, int nz, const Law<float> &law, const float *x,
                        const float *p, float *y, const uint8_t *mask, const CgArgs &ca, cudaStream_t st,
                        int phase = 0) {
    const int per_sm = modal_prepare<MODE>(ctx, nz);
    if (per_sm < 0) return -per_sm;
    const size_t smem = modal_smem_bytes<kModalNT, kModalEPT>(nz, MODE != MODE_PLAIN);
    const ModalGeom g = modal_geom(nx, ny, nz, ctx->num_sms, per_sm, MODE == MODE_CG);
    if (modal_short(nz))
        apply_modal_kernel<kModalNT, kModalEPT, 2, MODE>
            <<<modal_grid(g), kModalNT, smem, st>>>(g, x, p, y, mask, law, ctx->km, ca, phase);
    else
        apply_modal_kernel<kModalNT, kModalEPT, 3, MODE>
            <<<modal_grid(g), kModalNT, smem, st>>>(g, x, p, y, mask, law, ctx->km, ca, phase);
    GBS_LAUNCH_CHECK("apply_modal_kernel");
    return GBS_OK;
}

}  // namespace gbs
