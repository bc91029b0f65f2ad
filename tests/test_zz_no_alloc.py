"""The allocation-free OC update (gbsimp_oc_noalloc) against gbsimp_oc.

gbsimp_oc_noalloc serves callers that cannot allocate device memory -- a plugin reaching the
GPU only through the C ABI with no CUDA allocator, or a serving process with a fixed device
budget -- by taking its scratch from a static array inside the library. It must give the
results of gbsimp_oc (which uses a caller-provided workspace) on every call, including
consecutive calls that leave the shared array holding the previous call's contents.

This file sorts after the other kernel tests (only the full-size checks follow it), so that a
run stopping at its first failure has run them.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from genpipeline_gb300 import _lib as L
from genpipeline_gb300.engine import Engine

pytestmark = pytest.mark.gpu

# Same kernels in the same order as gbsimp_oc: results agree to the OC tests' tolerance.
RTOL, ATOL = 1e-6, 1e-7


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _noalloc(eng, grid, rmin, volfrac, x, dc, pres, variant):
    xn = torch.empty_like(x)
    xp = torch.empty_like(x)
    prm = L.make_oc(volfrac, variant)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(eng.lib.gbsimp_oc_noalloc(eng.ctx, *grid, float(rmin), C.byref(prm), _ptr(x), _ptr(dc), _ptr(pres),
                                      _ptr(xn), _ptr(xp), stream))
    return xn, xp


def _case(grid, seed, with_preserved):
    rng = np.random.default_rng(seed)
    n = int(np.prod(grid))
    x = torch.as_tensor(rng.uniform(0.01, 1.0, n).astype(np.float32), device="cuda")
    dc = torch.as_tensor((-rng.gamma(2.0, 1.0, n) * 10 ** rng.uniform(-3, 0, n)).astype(np.float32), device="cuda")
    pres = None
    if with_preserved:
        pres = torch.as_tensor((rng.random(n) < 0.05).astype(np.uint8), device="cuda")
    return x, dc, pres


def test_noalloc_oc_matches_oc_on_consecutive_calls():
    eng = Engine()
    calls = [((40, 20, 24), 2.0, 0.3, 1, True, L.OC_CPU),
             ((33, 17, 9), 1.5, 0.45, 2, False, L.OC_GPU),
             ((64, 32, 32), 3.0, 0.25, 3, True, L.OC_CPU)]
    for grid, rmin, vf, seed, with_pres, variant in calls:
        x, dc, pres = _case(grid, seed, with_pres)
        xn_ref, xp_ref = eng.oc(grid, rmin, vf, x, dc, pres, variant)
        xn, xp = _noalloc(eng, grid, rmin, vf, x, dc, pres, variant)
        torch.cuda.synchronize()
        np.testing.assert_allclose(xn.cpu().numpy(), xn_ref.cpu().numpy(), rtol=RTOL, atol=ATOL)
        np.testing.assert_allclose(xp.cpu().numpy(), xp_ref.cpu().numpy(), rtol=RTOL, atol=ATOL)


def test_noalloc_oc_allocates_no_device_memory():
    """After one call per variant (which loads the array's address and the kernels), further
    calls leave the device's free memory unchanged: the scratch is the library's own array."""
    eng = Engine()
    grid, rmin, vf = (48, 24, 20), 2.0, 0.3
    x, dc, pres = _case(grid, 5, True)
    xn, xp = torch.empty_like(x), torch.empty_like(x)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call(variant, p):
        prm = L.make_oc(vf, variant)
        L.check(eng.lib.gbsimp_oc_noalloc(eng.ctx, *grid, float(rmin), C.byref(prm), _ptr(x), _ptr(dc), _ptr(p),
                                          _ptr(xn), _ptr(xp), stream))

    for variant in (L.OC_CPU, L.OC_GPU):
        for p in (pres, None):
            call(variant, p)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        for variant in (L.OC_CPU, L.OC_GPU):
            for p in (pres, None):
                call(variant, p)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    xn_ref, xp_ref = eng.oc(grid, rmin, vf, x, dc, None, L.OC_GPU)
    torch.cuda.synchronize()
    np.testing.assert_allclose(xn.cpu().numpy(), xn_ref.cpu().numpy(), rtol=RTOL, atol=ATOL)
    np.testing.assert_allclose(xp.cpu().numpy(), xp_ref.cpu().numpy(), rtol=RTOL, atol=ATOL)


def test_noalloc_oc_rejects_grids_above_its_limit():
    eng = Engine()
    x, dc, xn, xp = (torch.zeros(8, device="cuda") for _ in range(4))  # never touched: rejected first
    prm = L.make_oc(0.3)
    grid = (256, 128, 65)  # 2,129,920 elements > 2,097,152
    assert np.prod(grid) > 2097152
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = eng.lib.gbsimp_oc_noalloc(eng.ctx, *grid, 1.5, C.byref(prm), _ptr(x), _ptr(dc), None, _ptr(xn),
                                   _ptr(xp), stream)
    assert rc == L.GBS_EINVAL
    assert b"static scratch" in eng.lib.gbsimp_last_error()
