"""Host-side generators of the batched and serving workloads."""
import numpy as np
import pytest

from genpipeline_gb300 import designs as D
from genpipeline_gb300.serve import request_stream


def test_grf_density_is_seeded_and_bounded():
    a = D.grf_density((24, 20, 16), 5)
    b = D.grf_density((24, 20, 16), 5)
    c = D.grf_density((24, 20, 16), 6)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.dtype == np.float32 and a.min() >= 1e-3 and a.max() <= 1.0
    rng = np.random.Generator(np.random.PCG64(5))
    rng.standard_normal((24, 20, 16))
    m = rng.uniform(0.2, 0.5)
    assert a.mean() == pytest.approx(m, abs=0.02)  # clipping at 1 moves the mean only slightly


def test_grf_density_length_scale():
    """Correlation length of the field: neighbours much closer than 6 voxels are correlated."""
    x = D.grf_density((64, 64, 64), 1).astype(np.float64)
    z = x - x.mean()
    c1 = np.mean(z[1:] * z[:-1]) / z.var()
    c20 = np.mean(z[20:] * z[:-20]) / z.var()
    assert c1 > 0.9 and abs(c20) < 0.3


def test_request_stream_statistics():
    reqs = request_stream(2000, rate=200.0)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert 2000 / t[-1] == pytest.approx(200.0, rel=0.08)
    assert set(r.n for r in reqs) == {24, 32, 48, 64, 96}
    assert set(r.load for r in reqs) == set(D.LOADS)
    rep = sum(r.repeat for r in reqs) / len(reqs)
    assert 0.07 < rep < 0.13
    assert request_stream(50)[7].seed == request_stream(50)[7].seed


def test_attached_payloads_are_the_seeded_densities():
    from genpipeline_gb300.serve import attach_payloads

    reqs = attach_payloads(request_stream(40, rate=200.0, edges=(8, 12, 16), repeat_frac=0.2, seed=3), workers=4)
    assert any(r.repeat for r in reqs)
    first = {}
    for r in reqs:
        assert r.density.shape == (r.n, r.n, r.n) and r.density.dtype == np.float32
        np.testing.assert_array_equal(r.density, D.grf_density((r.n, r.n, r.n), r.seed))
        first.setdefault((r.n, r.seed), r.density)
        assert r.density is first[(r.n, r.seed)]  # a repeated design shares its source's array
