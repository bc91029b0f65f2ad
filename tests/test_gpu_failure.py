"""Failure detection on the GPU without a fault: the persistent kernels' grid barrier gives
up after its bounded wait and reports GBS_ETIMEOUT when arrivals never come, and the context
keeps working afterwards."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_barrier_times_out_and_context_survives():
    from genpipeline_gb300 import _lib as L
    from genpipeline_gb300.engine import get_engine

    eng = get_engine()
    lib = eng.lib
    nb = int(lib.gbsimp_barrier_selftest_ws_bytes())
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    st = C.c_int(-1)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(lib.gbsimp_barrier_selftest(eng.ctx, 0, 1.0, C.byref(st), C.c_void_p(ws.data_ptr()), nb, stream))
    assert st.value == L.GBS_OK
    L.check(lib.gbsimp_barrier_selftest(eng.ctx, 1, 2e-3, C.byref(st), C.c_void_p(ws.data_ptr()), nb, stream))
    assert st.value == L.GBS_ETIMEOUT
    # the device still answers: a normal apply right after
    grid = (6, 5, 4)
    x = torch.rand(np.prod(grid), device="cuda")
    p = torch.randn(3 * 7 * 6 * 5, device="cuda")
    y = eng.apply(grid, L.make_law("modified", 3.0), x, p)
    torch.cuda.synchronize()
    assert torch.isfinite(y).all()
