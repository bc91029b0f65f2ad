"""Marching cubes restated in numpy for the STL export row. Test infrastructure only: the
tests and ``__graft_entry__.smoke()`` use it as the checker; the package never imports it.

The reference extracts the surface with skimage's marching cubes on the host
(``genpipeline/topology/mesh_export.py:7-67``). skimage is not installed here or on the GPU
machine, so its exact triangulation cannot be recorded: parity of triangles is against this
restatement of the algorithm the device kernel uses (same case rule, same cell and table
order), and the surface itself is checked against analytic shapes (area, enclosed volume,
closedness, outward normals).

Case rule: corners with value >= level are inside; on every cell face the cut edges are
joined by segments, a face with four cut edges separating its two inside corners; the
segments close into loops, each oriented so that its normal points from the inside to the
outside corners. A loop of three is one triangle; a longer loop is fanned around the mean of
its vertices. Vertices interpolate the level linearly along the cut edge from its lower grid
point.
"""
from __future__ import annotations

import numpy as np

CORNER = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
EDGE = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
FACE = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (3, 2, 6, 7), (0, 3, 7, 4), (1, 2, 6, 5)]


def _edge(a, b):
    for e, (p, q) in enumerate(EDGE):
        if (p, q) in ((a, b), (b, a)):
            return e
    raise ValueError((a, b))


def case_loops(cs: int):
    inside = [(cs >> c) & 1 for c in range(8)]
    nbr = {}

    def link(e0, e1):
        nbr.setdefault(e0, []).append(e1)
        nbr.setdefault(e1, []).append(e0)

    for q in FACE:
        sides = [s for s in range(4) if inside[q[s]] != inside[q[(s + 1) % 4]]]
        if len(sides) == 2:
            link(_edge(q[sides[0]], q[(sides[0] + 1) % 4]), _edge(q[sides[1]], q[(sides[1] + 1) % 4]))
        elif len(sides) == 4:
            for s in range(4):
                if inside[q[s]]:
                    link(_edge(q[(s + 3) % 4], q[s]), _edge(q[s], q[(s + 1) % 4]))
    loops, used = [], set()
    for e0 in range(12):
        if e0 not in nbr or e0 in used:
            continue
        loop, prev, cur = [], None, e0
        while True:
            loop.append(cur)
            used.add(cur)
            a, b = nbr[cur]
            nxt = a if a != prev else b
            prev, cur = cur, nxt
            if cur == e0:
                break
        mid = [0.5 * (np.array(CORNER[EDGE[e][0]]) + np.array(CORNER[EDGE[e][1]])) for e in loop]
        n = np.zeros(3)
        d = np.zeros(3)
        for t, e in enumerate(loop):
            p, q = mid[t], mid[(t + 1) % len(loop)]
            n += [(p[1] - q[1]) * (p[2] + q[2]), (p[2] - q[2]) * (p[0] + q[0]), (p[0] - q[0]) * (p[1] + q[1])]
            a, b = EDGE[e]
            ci, co = (a, b) if inside[a] else (b, a)
            d += np.array(CORNER[co]) - np.array(CORNER[ci])
        if n @ d < 0:
            loop = [loop[0]] + loop[1:][::-1]
        loops.append(loop)
    return loops


TABLE = [case_loops(cs) for cs in range(256)]


def n_triangles(cs: int) -> int:
    return sum(1 if len(lp) == 3 else len(lp) for lp in TABLE[cs])


def _vertex(e, i, j, k, c, level):
    a, b = EDGE[e]
    pa, pb = np.array(CORNER[a]), np.array(CORNER[b])
    if pa.sum() > pb.sum():
        a, b, pa, pb = b, a, pb, pa
    t = (level - c[a]) / (c[b] - c[a])
    return np.array([i, j, k], dtype=np.float64) + pa + t * (pb - pa)


def marching_cubes(vol: np.ndarray, level: float, spacing=(1.0, 1.0, 1.0)) -> np.ndarray:
    """(n_tri, 3, 3) triangles in cell order (C order of the cell index), then table order."""
    v = np.asarray(vol, dtype=np.float64)
    nx, ny, nz = v.shape
    out = []
    corner = np.array(CORNER)
    for i in range(nx - 1):
        for j in range(ny - 1):
            for k in range(nz - 1):
                c = [v[i + cx, j + cy, k + cz] for cx, cy, cz in corner]
                cs = sum(1 << q for q in range(8) if c[q] >= level)
                for loop in TABLE[cs]:
                    p = [_vertex(e, i, j, k, c, level) * spacing for e in loop]
                    if len(p) == 3:
                        out.append(p)
                    else:
                        mid = sum(p) / len(p)
                        out.extend([mid, p[t], p[(t + 1) % len(p)]] for t in range(len(p)))
    return np.array(out, dtype=np.float64).reshape(-1, 3, 3)


def area(tris: np.ndarray) -> float:
    return float(0.5 * np.linalg.norm(np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0]), axis=1).sum())


def enclosed_volume(tris: np.ndarray) -> float:
    """Divergence theorem over a closed, outward-oriented surface."""
    return float(np.einsum("ij,ij->i", tris[:, 0], np.cross(tris[:, 1], tris[:, 2])).sum() / 6.0)


def open_edges(tris: np.ndarray, decimals: int = 5) -> int:
    """Undirected edges not shared by exactly two triangles (0 for a closed surface)."""
    from collections import Counter

    q = np.round(tris, decimals)
    cnt = Counter()
    for t in q:
        for r in range(3):
            a, b = tuple(t[r]), tuple(t[(r + 1) % 3])
            cnt[(a, b) if a < b else (b, a)] += 1
    return sum(1 for v in cnt.values() if v != 2)
