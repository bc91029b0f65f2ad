"""CPU checks (FP64 numpy) of two algebraic rearrangements the GPU kernels rely on.

1. The one-kernel PCG (single-reduction Chronopoulos-Gear form) updates x only on odd
   iterations, two steps at once: x_{i+1} = x_{i-1} + (alpha_{i-1} + alpha_i beta_i) p_{i-1}
   + alpha_i u_i, and a solve that stops after an even iteration adds its alpha p. That must
   give the x of the every-iteration update.
2. The OC update evaluates five bisection levels per launch: the 31 midpoints of the binary
   tree below (l1, l2), each formed as bisection forms it, walked with bisection's tests.
   That must reproduce plain bisection's intervals, multiplier and step count.
"""
import numpy as np


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n))
    return a @ a.T + n * np.eye(n) * rng.uniform(0.5, 2.0, n)


def _cg(A, b, iters, two_step):
    """Single-reduction Jacobi-PCG (s_i = w_i + beta s_{i-1}, r_{i+1} = r_i - alpha s_i,
    u = M r, p_i = u_i + beta p_{i-1}, w = A u) with the x update every iteration or every
    other iteration; returns x after `iters` iterations."""
    m = 1.0 / np.diag(A)
    x = np.zeros_like(b)
    r = b.copy()
    u = m * r
    w = A @ u
    gamma = r @ u
    alpha, beta = gamma / (w @ u), 0.0
    alpha_prev = 0.0
    s = np.zeros_like(b)
    p = np.zeros_like(b)
    for i in range(iters):
        s = w + beta * s
        p_old = p
        p = u + beta * p_old
        if not two_step:
            x = x + alpha * p
        elif i % 2 == 1:
            x = x + (alpha_prev + alpha * beta) * p_old + alpha * u
        r = r - alpha * s
        u = m * r
        w = A @ u
        g_new, delta = r @ u, w @ u
        beta_new = g_new / gamma
        alpha_new = g_new / (delta - beta_new * g_new / alpha)
        alpha_prev, alpha, beta, gamma = alpha, alpha_new, beta_new, g_new
    if two_step and iters % 2 == 1:  # the last iteration (even index) still owes alpha p
        x = x + alpha_prev * p
    return x


def test_two_step_x_update_equals_every_iteration_update():
    for seed, n in [(0, 30), (1, 57), (2, 12)]:
        A = _spd(n, seed)
        b = np.random.default_rng(100 + seed).standard_normal(n)
        for iters in (1, 2, 3, 8, 13, 20):
            x1 = _cg(A, b, iters, two_step=False)
            x2 = _cg(A, b, iters, two_step=True)
            np.testing.assert_allclose(x2, x1, rtol=0, atol=1e-12 * np.abs(x1).max())
        # and the iteration converges to the solution
        np.testing.assert_allclose(_cg(A, b, 4 * n, two_step=True), np.linalg.solve(A, b), rtol=1e-8, atol=1e-10)


def _bisection(vol, l1, l2, tol, eps, max_steps):
    steps, lfinal = 0, 0.5 * (l1 + l2)
    while steps < max_steps:
        m = 0.5 * (l2 + l1)
        if (l2 - l1) / (l1 + l2 + eps) < tol:
            return m, steps + 1, (l1, l2)
        if vol(m) > 0.0:
            l1 = m
        else:
            l2 = m
        lfinal, steps = m, steps + 1
    return lfinal, steps, (l1, l2)


def _multisection(vol, l1, l2, tol, eps, max_steps, levels=5):
    nodes = (1 << levels) - 1
    steps, lfinal = 0, 0.5 * (l1 + l2)
    while steps < max_steps:
        mids, stop = [], []
        for t in range(nodes):  # node t: path bits of t + 1 below its leading one
            lo, hi = l1, l2
            path = t + 1
            for i in range(path.bit_length() - 2, -1, -1):
                m = 0.5 * (hi + lo)
                lo, hi = (m, hi) if (path >> i) & 1 else (lo, m)
            mids.append(0.5 * (hi + lo))
            stop.append((hi - lo) / (lo + hi + eps) < tol)
        vols = [vol(m) for m in mids]  # one pass over the elements on the GPU
        node = 0
        for _ in range(levels):
            m = mids[node]
            if stop[node]:
                return m, steps + 1, (l1, l2)
            if vols[node] > 0.0:
                l1, node = m, 2 * node + 2
            else:
                l2, node = m, 2 * node + 1
            lfinal, steps = m, steps + 1
            if steps >= max_steps:
                return lfinal, steps, (l1, l2)
    return lfinal, steps, (l1, l2)


def test_multisection_reproduces_bisection():
    rng = np.random.default_rng(5)
    for trial in range(20):
        x = rng.uniform(0.01, 1.0, 500)
        dc = -rng.gamma(2.0, 1.0, x.size) * 10 ** rng.uniform(-3, 0, x.size)
        volfrac = rng.uniform(0.2, 0.5)

        def vol(lam):  # the CPU variant's trial densities, simp_solver.py:229-247 (no filter)
            t = np.maximum(-dc / lam, 1e-12)
            xn = np.clip(np.clip(x * np.sqrt(t), 0.0, 1.0), x - 0.2, x + 0.2)
            return xn.mean() - volfrac

        for (l1, l2, tol, eps, cap) in [(0.0, 1e9, 1e-4, 1e-12, 50), (0.0, 2.0 * max(-dc.min(), 1.0), 1e-5, 1e-15, 30),
                                        (0.0, 1e9, 1e-4, 1e-12, 7)]:
            assert _multisection(vol, l1, l2, tol, eps, cap) == _bisection(vol, l1, l2, tol, eps, cap)
