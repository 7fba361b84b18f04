"""Host-side pieces of the learned initial guess (no GPU): the training-body
generator and the CPU oracle of the network."""
import numpy as np
import pytest

from oracle import net_oracle as no


def test_random_bodies_leave_no_isolated_fluid_cell():
    from flowfpmpp_gb300 import learned as lg
    rng = np.random.default_rng(3)
    ax, ay, az = lg.training_grid(32, 32, 16)
    for _ in range(25):
        solid = lg.random_bodies(rng, ax, ay, az)
        fl = np.pad(~solid, 1)
        nb = sum(np.roll(fl, s, a) for a in range(3) for s in (1, -1))[1:-1, 1:-1, 1:-1]
        assert solid.any()
        assert not np.any(~solid & (nb == 0))


def test_oracle_gradient_matches_finite_differences():
    """The oracle's autograd gradient of the loss against central differences
    on a few parameters (BF16 rounding switched off by smooth perturbations
    that are exact in BF16: the check uses the unrounded float64 network)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    nx, ny, nz = 8, 8, 8
    fluid = np.ones((nx, ny, nz), dtype=np.uint8)
    fluid[3:5, 3:5, 3:5] = 0
    mx, my, mz = (np.linspace(0.5, 1.0, n).astype(np.float32) for n in (nx, ny, nz))
    rhs = rng.standard_normal((nx, ny, nz)).astype(np.float32)
    target = rng.standard_normal((nx, ny, nz)).astype(np.float32)
    p = rng.normal(0, 0.1, no.param_count())
    saved = no.bf
    no.bf = lambda x: x  # exact float64 network for the finite-difference check

    class _Id(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.view_as(x)

        @staticmethod
        def backward(ctx, g):
            return g

    saved_rg = no._RoundGrad
    no._RoundGrad = _Id
    try:
        _, L, g = no.output_and_grads(p, fluid, mx, my, mz, rhs, target)
        for q in rng.choice(no.param_count(), 6, replace=False):
            h = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[q] += h
            pm[q] -= h
            lp = no.output_and_grads(pp, fluid, mx, my, mz, rhs, target)[1]
            lm = no.output_and_grads(pm, fluid, mx, my, mz, rhs, target)[1]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[q]) <= 1e-5 * max(1.0, abs(g[q])) + 1e-7, (q, fd, g[q])
    finally:
        no.bf = saved
        no._RoundGrad = saved_rg
