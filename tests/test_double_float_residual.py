"""The double-float outer residual (csrc/modal_dd.cuh, fp64.cu modal_elem_dd_kernel, pcg.cu
resid_dd_kernel), emulated operation for operation in numpy float32 and checked against the FP64
residual of the oracle on oracle-solved displacements.

Emulated: u split into (h, l) = (RN32(u), RN32(u - h)); the forward Walsh-Hadamard butterflies
(a, b) -> (a + b, b - a) with exact two-sums on the h parts and plain FP32 adds of the l parts and
the two-sum errors; r = Km q row by row with products (ch + cl)(qh + ql) = ch qh exactly (its
error as an fma would give it) + ch ql + cl qh; r *= E; the inverse butterflies (a - b, a + b);
node sums in corner order b = 0..7 with two-sums; r = f - q. The FP32 products of two FP32
values are exact in float64, which gives the fma's error term exactly.
"""
import numpy as np
import pytest

from genpipeline_gb300 import bcs
from oracle import oracle as O

f32, f64 = np.float32, np.float64
# corner order of the reference's element (node a at corner (cx, cy, cz))
CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def km_of(ke):
    """Km = T^T Ke T / 64 in mode-major (mode * 3 + component) order, modes bit-ordered
    (x, y, z) = (4, 2, 1)."""
    t8 = np.zeros((8, 8))
    for a, c in enumerate(CORNERS):
        for m in range(8):
            bits = ((m >> 2) & 1, (m >> 1) & 1, m & 1)
            t8[a, m] = np.prod([(1.0 if c[d] else -1.0) if bits[d] else 1.0 for d in range(3)])
    t = np.kron(t8, np.eye(3))
    return t.T @ ke @ t / 64.0


def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def split(x):
    h = x.astype(f32)
    return h, (x - h.astype(f64)).astype(f32)


def fma32(a, b, c):
    return (a.astype(f64) * b.astype(f64) + c.astype(f64)).astype(f32)


def dd_mul(ch, cl, qh, ql):
    p = ch * qh
    e = (ch.astype(f64) * qh.astype(f64) - p.astype(f64)).astype(f32)
    return p, fma32(cl, qh, fma32(ch, ql, e))


def residual_dd(grid, ke, E, u, f, node_mask):
    nx, ny, nz = grid
    km = km_of(ke)
    kmax = np.abs(km).max()
    ny1, nz1 = ny + 1, nz + 1
    i, j, k = (a.ravel() for a in np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"))
    uh, ul = split(u)
    nodes = [((i + (b >> 2)) * ny1 + (j + ((b >> 1) & 1))) * nz1 + (k + (b & 1)) for b in range(8)]
    v = {}
    for b in range(8):
        for c in range(3):
            fx = (node_mask[nodes[b]] >> c) & 1
            v[b, c] = [np.where(fx, f32(0), uh[3 * nodes[b] + c]), np.where(fx, f32(0), ul[3 * nodes[b] + c])]
    for d in range(3):
        bit = 1 << d
        for b in range(8):
            if b & bit:
                continue
            for c in range(3):
                a0, a1 = v[b, c], v[b | bit, c]
                s, e = two_sum(a0[0], a1[0])
                t, g = two_sum(a1[0], -a0[0])
                v[b, c] = [s, (a0[1] + a1[1]) + e]
                v[b | bit, c] = [t, (a1[1] - a0[1]) + g]
    eh, el = split(E)
    r = {}
    for ro in range(24):
        acc = None
        for co in range(24):
            if abs(km[ro, co]) <= 1e-12 * kmax:
                continue
            ch, cl = split(np.array([km[ro, co]]))
            q = v[co // 3, co % 3]
            p, e = dd_mul(np.full_like(q[0], ch[0]), np.full_like(q[0], cl[0]), q[0], q[1])
            if acc is None:
                acc = [p, e]
            else:
                s, g = two_sum(acc[0], p)
                acc = [s, (acc[1] + e) + g]
        if acc is None:
            acc = [np.zeros_like(eh), np.zeros_like(eh)]
        r[ro // 3, ro % 3] = list(dd_mul(eh, el, acc[0], acc[1]))
    for d in range(3):
        bit = 1 << d
        for b in range(8):
            if b & bit:
                continue
            for c in range(3):
                a0, a1 = r[b, c], r[b | bit, c]
                s, e = two_sum(a0[0], -a1[0])
                t, g = two_sum(a0[0], a1[0])
                r[b, c] = [s, (a0[1] - a1[1]) + e]
                r[b | bit, c] = [t, (a0[1] + a1[1]) + g]
    nn = (nx + 1) * ny1 * nz1
    qh, ql = np.zeros(3 * nn, f32), np.zeros(3 * nn, f32)
    for b in range(8):  # each node receives its corners in the order b = 0..7
        for c in range(3):
            idx = 3 * nodes[b] + c
            s, g = two_sum(qh[idx], r[b, c][0])
            ql[idx] = (ql[idx] + r[b, c][1]) + g
            qh[idx] = s
    q = qh.astype(f64) + ql.astype(f64)
    fixed = (np.repeat(node_mask, 3) >> np.tile(np.arange(3), nn)) & 1
    return np.where(fixed, 0.0, f - q)


@pytest.mark.parametrize("grid,load,law", [((16, 8, 8), "cantilever", "modified"), ((12, 12, 8), "top_patch", "ref")])
def test_double_float_residual_matches_fp64(grid, load, law):
    f, fixed = bcs.LOAD_CASES[load](*grid)
    node_mask = bcs.node_mask(*grid, fixed)
    dof_mask = bcs.dof_mask(*grid, fixed)
    rng = np.random.default_rng(3)
    x = rng.uniform(0.05, 1.0, int(np.prod(grid)))
    ke = O.ke_quadrature()
    E = O.moduli(x, O.Material(law, 3.0))
    u, _, _ = O.pcg(grid, ke, E, f, dof_mask, tol=1e-11)
    r64 = f - O.apply(grid, ke, E, u, dof_mask)
    r64[dof_mask.astype(bool)] = 0.0
    rdd = residual_dd(grid, ke, E, u, f, node_mask)
    fn = np.linalg.norm(np.where(dof_mask.astype(bool), 0.0, f))
    # measured 5e-13..6e-13 on converged 32x16x16 and 64^3 fields; the solver uses it for rtol >= 1e-9
    assert np.linalg.norm(rdd - r64) <= 2e-12 * fn
    assert np.linalg.norm(r64) <= 1e-10 * fn  # the field is converged: the test sees the rounding, not r
