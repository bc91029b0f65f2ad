// modal_dd.cuh -- the modal element form (apply_modal.cuh) in unnormalised double-float
// arithmetic (common.cuh: ddv): the element products of the outer residual and of the
// sensitivities. GB300 issues FP64 at about 1/64 of its FP32 rate; these run on the FP32 pipe
// with about 2^-46 relative rounding of the magnitudes involved instead of FP64's 2^-53.
#pragma once

#include "common.cuh"

namespace gbs {

// Double-float pairs of the 45 Km coefficients (host side).
inline ModalKDD modal_kdd(const ModalKD &k) {
    ModalKDD d;
    for (int t = 0; t < kModalNnz; ++t) {
        d.h[t] = (float)k.v[t];
        d.l[t] = (float)(k.v[t] - (double)d.h[t]);
    }
    return d;
}

// The stiffness law for double-float element moduli: e0, emin, e0 - emin and xmin as (h, l)
// pairs of their FP64 values, and the FP64 law for penalties that are not small integers.
struct LawDD {
    int kind, pint;
    ddv e0, emin, span, xmin;
    Law<double> law;
};
inline ddv dd_host(double v) {
    const float h = (float)v;
    return ddv{h, (float)(v - (double)h)};
}
inline LawDD make_law_dd(const gbsimp_law &l) {
    LawDD d;
    d.law = make_law<double>(l);
    d.kind = d.law.kind;
    d.pint = d.law.pint;
    d.e0 = dd_host(l.e0);
    d.emin = dd_host(l.emin);
    d.span = dd_host(l.e0 - l.emin);
    d.xmin = dd_host(l.xmin);
    return d;
}

// E(x) of modulus() in double-float from an FP32 density: x^p by exact first product and
// double-float products after it (integer p <= 4), the law's constants as pairs; about 2^-48
// relative. Other penalties: the FP64 law, split.
__device__ __forceinline__ ddv modulus_dd(const LawDD &L, float x) {
    if (L.pint < 0) return dd_split(modulus(L.law, (double)x));
    ddv base{x, 0.0f};
    if (L.kind == 0 && !(x > L.xmin.h || (x == L.xmin.h && L.xmin.l < 0.0f))) base = L.xmin;  // max(x, xmin)
    ddv p{1.0f, 0.0f};
    for (int i = 0; i < L.pint; ++i) p = i == 0 ? base : dd_mul(base.h, base.l, p);
    if (L.kind == 0) return dd_mul(L.e0.h, L.e0.l, p);
    return dd_add(L.emin, dd_mul(L.span.h, L.span.l, p));
}

// q = T^T u_e of element (i, j, k): corners in bit order (x, y, z) = (4, 2, 1), from the
// split displacements udd (h, l per DOF).
__device__ __forceinline__ void modal_fwd_dd(int ny, int nz, int i, int j, int k, const float2 *__restrict__ udd,
                                             ddv (&v)[8][3]) {
    const int64_t NY = ny + 1, NZ = nz + 1;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const int64_t n = ((int64_t)(i + (b >> 2)) * NY + (j + ((b >> 1) & 1))) * NZ + (k + (b & 1));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 w = __ldg(&udd[3 * n + c]);
            v[b][c] = ddv{w.x, w.y};
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if (b & bit) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) dd_fwd(v[b][c], v[b | bit][c]);
        }
    }
}

// r = Km q over the 45 nonzeros; the rows of mode 0 (translations) are zero.
__device__ __forceinline__ void modal_km_dd(const ModalKDD &km, const ddv (&q)[8][3], ddv (&r)[8][3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) r[0][c] = ddv{0.0f, 0.0f};
#pragma unroll
    for (int t = 0; t < kModalNnz; ++t) {
        const int ro = modal_row(t), co = modal_col(t);
        const ddv p = dd_mul(km.h[t], km.l[t], q[co / 3][co % 3]);
        r[ro / 3][ro % 3] = modal_row_first(t) ? p : dd_add(r[ro / 3][ro % 3], p);
    }
}

// y_e = T r per corner (bit order); r[0] is zero, so the first stage's pairs (0, 1) are
// (-r1, r1) without rounding.
__device__ __forceinline__ void modal_inv_dd(ddv (&r)[8][3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) r[0][c] = ddv{-r[1][c].h, -r[1][c].l};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int bit = 1 << d;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if ((b & bit) || (d == 0 && b == 0)) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) dd_inv(r[b][c], r[b | bit][c]);
        }
    }
}

}  // namespace gbs
