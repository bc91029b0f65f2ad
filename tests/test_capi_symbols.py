"""CPU checks of the C ABI: the library builds/loads and exports every declared symbol;
host-only entry points work without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from genpipeline_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gbsimp_\w+)\s*\(", src))
    return names


def test_every_declared_symbol_is_exported_and_bound():
    lib = L.load()
    names = _declared()
    assert len(names) >= 25
    for n in sorted(names):
        assert hasattr(lib, n), n
    # the Python binding covers the whole header
    assert names <= set(L.SIGNATURES), sorted(names - set(L.SIGNATURES))


def test_abi_version_and_errors():
    lib = L.load()
    assert lib.gbsimp_abi_version() == 2
    with pytest.raises(L.GbsimpError) as ei:
        L.check(lib.gbsimp_ke_quadrature(0.6, 1.0, None))
    assert ei.value.code == L.GBS_EINVAL


def test_library_ke_matches_oracle_and_reference_quadrature(golden):
    from oracle import oracle as O
    from genpipeline_gb300.engine import Engine

    k = Engine.ke_quadrature(0.3, 1.0)
    np.testing.assert_allclose(k, O.ke_quadrature(0.3), rtol=0, atol=2e-16)
    np.testing.assert_allclose(k, golden("ke")["ke_quadrature"], rtol=0, atol=2e-16)
    k2 = Engine.ke_quadrature(0.25, 2.0)
    np.testing.assert_allclose(k2, O.ke_quadrature(0.25, 2.0), rtol=0, atol=1e-15)


def test_workspace_queries_are_host_only():
    lib = L.load()
    for grid in ((1, 1, 1), (64, 64, 64), (192, 96, 96)):
        nd = 3 * (grid[0] + 1) * (grid[1] + 1) * (grid[2] + 1)
        assert lib.gbsimp_pcg_ws_bytes(*grid) >= 5 * 4 * nd
        assert lib.gbsimp_solve_ws_bytes(*grid) >= lib.gbsimp_pcg_ws_bytes(*grid) + 16 * nd
        assert lib.gbsimp_oc_ws_bytes(*grid) >= 8 * grid[0] * grid[1] * grid[2]
    assert lib.gbsimp_pcg_csr_ws_bytes(1000) >= 16000


def test_pcg_workspace_holds_the_one_kernel_partials():
    """The one-kernel PCG writes two slots of three partial sums (8 bytes each) per CTA; its
    launch is tiles x segments CTAs, tiles = ceil((ny+1)(nz+1) / (512 - (nz+2))) per plane and
    segments filling one wave (at least one). The workspace's partials region must hold them
    for waves up to 2048 CTAs, including planes of thousands of tiles (large ny with nz near
    the modal limit of 446)."""
    lib = L.load()

    def al(b):
        return (b + 255) // 256 * 256

    # the scalars block: total - slack - 9 vectors - partials - the element moduli (1 element)
    sc = lib.gbsimp_pcg_ws_bytes(1, 1, 1) - 256 - 9 * al(4 * 24) - al(8 * 12288) - al(4)
    assert sc > 0 and sc % 256 == 0
    rng = np.random.default_rng(0)
    shapes = [(64, 64, 64), (192, 96, 96), (1, 300, 446), (2, 2000, 446), (1, 600, 400), (3, 1, 446), (1, 1, 1)]
    shapes += [(int(rng.integers(1, 64)), int(rng.integers(1, 2500)), int(rng.integers(1, 447))) for _ in range(300)]
    for nx, ny, nz in shapes:
        nd = 3 * (nx + 1) * (ny + 1) * (nz + 1)
        part = lib.gbsimp_pcg_ws_bytes(nx, ny, nz) - 256 - sc - 9 * al(4 * nd) - al(4 * nx * ny * nz)
        f = 512 - (nz + 2)
        tiles = -(-(ny + 1) * (nz + 1) // f)
        for wave in (1, 152, 304, 608, 2048):
            nblk = tiles * max(1, min(wave // tiles, nx))
            assert part >= 48 * nblk, (nx, ny, nz, wave)


def test_grids_beyond_32_bit_dof_indices_are_refused():
    """3 (nx+1)(ny+1)(nz+1) must stay below 2^31 for every grid entry point; the argument
    checks run before the context is used (the placeholder context is never dereferenced)."""
    lib = L.load()
    ctx = C.c_void_p(16)
    buf = C.c_void_p(256)
    law = L.make_law("modified", 3.0)
    big = (900, 900, 900)  # 3 * 901^3 > 2^31 DOFs
    prm = L.OcParams()
    calls = {
        "gbsimp_apply_f32": lambda g: lib.gbsimp_apply_f32(ctx, *g, C.byref(law), buf, buf, buf, None, None),
        "gbsimp_apply_f64": lambda g: lib.gbsimp_apply_f64(ctx, *g, C.byref(law), buf, buf, buf, None, None),
        "gbsimp_sensitivity": lambda g: lib.gbsimp_sensitivity(ctx, *g, C.byref(law), buf, buf, buf, None, None, None, 0,
                                                               None),
        "gbsimp_filter_hs": lambda g: lib.gbsimp_filter_hs(ctx, *g, 1.5, buf, None),
        "gbsimp_filter": lambda g: lib.gbsimp_filter(ctx, *g, 1.5, buf, buf, buf, 0, None),
        "gbsimp_oc_prepare": lambda g: lib.gbsimp_oc_prepare(ctx, *g, 1.5, None, buf, 1 << 62, None),
        "gbsimp_oc": lambda g: lib.gbsimp_oc(ctx, *g, 1.5, C.byref(prm), buf, buf, None, buf, buf, buf, 1 << 62, None),
    }
    int_max = 2**31 - 1
    # Extents whose +1 or whose products would wrap in 32- or 64-bit arithmetic, and the exact
    # boundary: (461+1)(4680+1)(330+1) = 715,827,882 = floor(2^31 / 3) nodes, the first count
    # refused (2*3*7*11 = 462, 31*151 = 4681, 331).
    wrap = [(int_max, 1, 1), (1, int_max, 1), (1, 1, int_max), (int_max, int_max, int_max),
            (2**30, 2**30, 2**30), (2**21, 2**21, 2**21), (461, 4680, 330), (330, 461, 4680)]
    for name, call in calls.items():
        assert call(big) == L.GBS_EINVAL, name
        assert b"bad arguments" in lib.gbsimp_last_error(), name
        assert call((0, 4, 4)) == L.GBS_EINVAL, name
        for g in wrap:
            assert call(g) == L.GBS_EINVAL, (name, g)


def test_every_status_entry_point_rejects_null_arguments():
    """Every status-returning call, given a NULL context, zero sizes and NULL pointers, returns
    GBS_EINVAL with a message before touching the device (no GPU here)."""
    lib = L.load()
    no_status = {"gbsimp_abi_version", "gbsimp_launch_count", "gbsimp_last_error", "gbsimp_create",
                 "gbsimp_destroy", "gbsimp_queue_destroy", "gbsimp_queue_size", "gbsimp_apply_path",
                 "gbsimp_marching_cubes_table"}
    checked = 0
    for name, (res, args) in sorted(L.SIGNATURES.items()):
        if name in no_status or res is not L._I:
            continue
        vals = [0 if a in (L._I, L._I64, L._SZ, C.c_int32) else 0.0 if a is L._D else None for a in args]
        assert getattr(lib, name)(*vals) == L.GBS_EINVAL, name
        assert lib.gbsimp_last_error(), name
        checked += 1
    assert checked >= 28
    assert lib.gbsimp_apply_path(None, 64) == -1
    ntri = (C.c_ubyte * 256)()
    assert lib.gbsimp_marching_cubes_table(ntri, None, None, None) == 12 >= max(ntri) > 0


def test_queue_and_simp_run_argument_checks_without_gpu():
    """Host-only paths of the queue and the SIMP loop: size queries and argument errors."""
    lib = L.load()
    assert lib.gbsimp_simp_run_ws_bytes(0, 4, 4) == 0
    assert lib.gbsimp_simp_run_ws_bytes(8, 4, 4) > lib.gbsimp_solve_ws_bytes(8, 4, 4)
    assert lib.gbsimp_queue_size(None) == -1
    n = C.c_int(7)
    assert lib.gbsimp_queue_poll(None, None, 0, C.byref(n), None) == L.GBS_EINVAL
    assert lib.gbsimp_queue_submit(None, None) == L.GBS_EINVAL
    assert lib.gbsimp_queue_create(None, None, None, None) == L.GBS_EINVAL
    assert C.sizeof(L.SimpOpts) == 16 + 8 + C.sizeof(L.OcParams) + C.sizeof(L.SolveOpts)
