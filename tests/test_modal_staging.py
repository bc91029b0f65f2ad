"""CPU check of the modal kernels' staging arithmetic (issue_plane / commit_plane of
genpipeline_gb300/csrc/apply_modal.cuh), restated here, over every tile and node plane of many
grids, for both kernel forms (two 16-byte groups per thread and plane for nz <= 167, three
above) and both modes (plain apply: one vector over the whole plane; PCG: four whole-plane
vectors plus the owned groups of p and x).

For every copy: the source range lies inside the node vector (3 (nx+1)(ny+1)(nz+1) words),
starts on a 16-byte boundary and spans whole 16-byte groups; the destination lies inside its
RW-word raw buffer, on a 16-byte boundary; the group cut by the end of the vector goes to a
whole group of the raw buffer. Every staged group is combined by some thread (nv <= groups
per thread x 256) and the operand planes and element reads stay inside one RW-word slot.
The x segments of modal_geom partition the planes (restated too).
"""
import numpy as np
import pytest

NT, NE = 256, 512


def _check(nx, ny, nz, cg):
    H, NZ = nz + 2, nz + 1
    R, F, S = NE + H, NE - H, (ny + 1) * (nz + 1)
    maxv = 2 if (3 * R + 6) // 4 <= 2 * NT else 3
    rl = (8 * NT - 5) // 3 if maxv == 2 else R
    rw = 4 * ((3 * rl + 6) // 4)
    nw = 3 * (nx + 1) * S
    full = nw & ~3
    assert rw % 4 == 0
    for tile in range(-(-S // F)):
        f0 = tile * F
        for j in range(-1, nx + 3):
            w0 = 3 * (j * S + f0 - H)
            a = w0 & ~3
            pad = w0 - a
            nv = (pad + 3 * R + 3) // 4
            assert nv <= maxv * NT and 4 * nv <= rw
            # corner reads of the element pass: chunk node tid + cy NZ + cz (+ NT), 3 words each
            assert pad + 3 * ((NT - 1) + NZ + 1 + NT) + 2 < rw
            if not 0 <= j <= nx:
                continue
            g0, g1 = max(a, 0), min(a + 4 * nv, full)
            if g1 > g0:
                assert g0 % 4 == 0 and (g1 - g0) % 4 == 0 and g1 <= nw
                assert (g0 - a) % 4 == 0 and (g0 - a) + (g1 - g0) <= rw
            if cg:
                olo3, ohi3 = 3 * H, 3 * min(NE, S - f0 + H)
                o0 = max(a + 4 * ((olo3 + pad) >> 2), 0)
                o1 = min(a + 4 * ((ohi3 + pad + 3) >> 2), full)
                if o1 > o0:
                    assert o0 % 4 == 0 and (o1 - o0) % 4 == 0 and o1 <= nw
                    assert (o0 - a) + (o1 - o0) <= rw
            if full < nw and full >= a:
                ft = (full - a) >> 2
                if ft < nv:
                    assert 4 * ft + 4 <= rw and 0 < nw - full < 4
                    if j < nx:
                        # the kernel copies the cut group for the last node plane only: in an
                        # earlier plane's chunk its words lie past the plane's own nodes (never used)
                        assert full - (a + pad) >= 3 * min(R, S - f0 + H)


@pytest.mark.parametrize("cg", [False, True])
def test_staging_in_bounds_for_every_z_extent(cg):
    for nz in range(1, 447):
        for ny in (1, 2, 7):
            _check(2, ny, nz, cg)


@pytest.mark.parametrize("cg", [False, True])
@pytest.mark.parametrize("grid", [(64, 64, 64), (192, 96, 96), (64, 32, 32), (40, 20, 100), (4, 3, 167),
                                  (4, 3, 168), (3, 5, 300), (2, 2, 446), (8, 4, 200), (3, 2, 446), (1, 300, 446),
                                  (17, 9, 37), (1, 1, 1)])
def test_staging_in_bounds_for_test_and_bench_grids(grid, cg):
    _check(*grid, cg)


def _segments(nx, ny, nz, sms, per_sm, edge):
    """modal_geom's x segments: [xs, xe) per segment (restated)."""
    f = NE - (nz + 2)
    tiles = -(-(ny + 1) * (nz + 1) // f)
    planes = nx if edge else nx + 1
    nseg = max(1, min((sms * per_sm) // tiles, planes))
    seglen, rem = planes // nseg, planes % nseg
    out = []
    for s in range(nseg):
        xs = s * seglen + min(s, rem)
        out.append((xs, min(xs + seglen + (1 if s < rem else 0), planes)))
    return tiles, out


@pytest.mark.parametrize("edge", [False, True])
def test_segments_partition_the_planes(edge):
    """Segments tile [0, planes) exactly, each non-empty, lengths within one plane of each
    other; the launch (tiles x segments) fills at most one wave unless one plane's tiles
    alone exceed it."""
    rng = np.random.default_rng(2)
    cases = [(64, 64, 64, 152, 2), (192, 96, 96, 152, 2), (3, 2, 446, 152, 1), (1, 300, 446, 152, 2)]
    cases += [(int(rng.integers(1, 300)), int(rng.integers(1, 200)), int(rng.integers(1, 447)), 152,
               int(rng.integers(1, 3))) for _ in range(300)]
    for nx, ny, nz, sms, per_sm in cases:
        tiles, segs = _segments(nx, ny, nz, sms, per_sm, edge)
        planes = nx if edge else nx + 1
        assert segs[0][0] == 0 and segs[-1][1] == planes
        assert all(a[1] == b[0] for a, b in zip(segs, segs[1:]))
        lens = [xe - xs for xs, xe in segs]
        assert min(lens) >= 1 and max(lens) - min(lens) <= 1
        assert tiles * len(segs) <= max(sms * per_sm, tiles)
    tiles, segs = _segments(64, 64, 64, 152, 2, True)  # the 64^3 PCG launch: 10 tiles x 30 segments
    assert (tiles, len(segs), sorted({b - a for a, b in segs})) == (10, 30, [2, 3])


def test_random_grids():
    rng = np.random.default_rng(1)
    for _ in range(200):
        _check(int(rng.integers(1, 40)), int(rng.integers(1, 300)), int(rng.integers(1, 447)), bool(rng.integers(2)))
