"""The algebraic forms the point kernel evaluates, against the reference's own forms (CPU).

csrc/xc_functionals.cuh evaluates B88's term as beta g x / D instead of the
reference's beta 2^(4/3 log2 rho + 2 log2 x - log2 D) (popular_functionals.py:52-103),
and LYP's rho^(-1/3), rho^(-5/3), rho^(8/3) (popular_functionals.py:197-269) from cube
roots.  These are the same functions; this test pins the restatements, in float64 with
torch autograd for the partials, against the oracle's log form over densities and
gradients spanning the clip (1e-30) to 1e3.  The CUDA kernel itself is compared with the
oracle by the GPU parity tests.
"""
import numpy as np
import torch

import oracle as O

F64 = torch.float64
CLIP = 1e-30


def b88_direct(rho, grad_rho, clip_cte=CLIP):
    """B88 as csrc/xc_functionals.cuh:b88_x_e evaluates it (g = |grad rho|, x = g / rho^(4/3))."""
    beta = 0.0042
    rho = torch.clamp(rho, min=clip_cte)
    g = torch.sqrt(torch.clamp(torch.sum(grad_rho ** 2, axis=-1), min=clip_cte))
    rc = torch.clamp(rho, min=clip_cte)
    x = g / (rc * torch.pow(rc, 1.0 / 3.0))
    return -(beta * (g * x) / (1 + 6 * beta * x * torch.asinh(x))).sum(axis=1)


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    rho = 10.0 ** rng.uniform(-34, 3, (n, 2))
    rho[:8] = [[0.0, 0.0], [CLIP, CLIP], [1e-31, 1.0], [1.0, 1e-31], [2e-30, 5e-30], [1e3, 1e3], [1e-10, 1e-12],
               [0.5, 0.25]]
    grad = rng.standard_normal((n, 2, 3)) * 10.0 ** rng.uniform(-17, 3, (n, 2, 1))
    grad[:2] = 0.0
    return (torch.tensor(rho, dtype=F64, requires_grad=True), torch.tensor(grad, dtype=F64, requires_grad=True))


def _rel(a, b):
    a, b = a.detach(), b.detach()
    return float(((a - b).abs() / b.abs().clamp(min=1e-300)).max())


def test_b88_direct_form_matches_log_form():
    rho, grad = _inputs(50_000, 0)
    e_log = O.b88_x_e(rho, grad)
    e_dir = b88_direct(rho, grad)
    assert _rel(e_dir, e_log) < 1e-12
    g_log = torch.autograd.grad(e_log.sum(), (rho, grad))
    g_dir = torch.autograd.grad(e_dir.sum(), (rho, grad))
    for a, b in zip(g_dir, g_log):
        # Both forms are analytic; where the log form's partial is exactly zero (clipped
        # inputs) the direct one is too, elsewhere they agree to the log form's own
        # rounding (base-2 exponents of size ~100 lose about 1e-14 relative).
        assert torch.equal(a == 0, b == 0)
        scale = b.abs().max()
        assert float((a - b).abs().max()) <= 1e-11 * float(scale)
        nz = b != 0
        assert _rel(a[nz], b[nz]) < 1e-10


def test_third_powers_from_cube_roots():
    rng = np.random.default_rng(1)
    x = torch.tensor(10.0 ** rng.uniform(-30, 3, 100_000), dtype=F64)
    cb = torch.pow(x, 1.0 / 3.0)
    rcb = 1.0 / cb
    for n, got in ((-1, rcb), (-5, rcb * rcb / x), (4, x * cb), (8, (x * x) * (cb * cb))):
        assert _rel(got, x ** (n / 3.0)) < 5e-14, n
