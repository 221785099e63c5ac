"""Known answers for the shape-target loss restatement (no GPU)."""
import numpy as np

from oracle import deform as OD


def test_grid_mass_conserves_mass():
    rng = np.random.default_rng(0)
    x = rng.uniform(0.3, 0.7, (500, 3))
    m = OD.grid_mass(x, 0.01, 1.0 / 16, (16, 16, 16))
    assert np.isclose(m.sum(), 500 * 0.01)


def test_target_sdf_is_distance_to_a_single_seed():
    n = (12, 12, 12)
    t = np.zeros(n)
    t[6, 6, 6] = 1.0
    dx = 0.1
    sdf = OD.target_sdf(t, dx, 24)
    ii = np.stack(np.meshgrid(*[np.arange(v) for v in n], indexing="ij"), -1)
    exact = np.sqrt((((ii - 6) * dx) ** 2).sum(-1) + 1e-8)
    exact[6, 6, 6] = 0.0
    assert np.allclose(sdf, exact, rtol=1e-12, atol=1e-12)


def test_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    x = rng.uniform(0.35, 0.65, (200, 3))
    dx, n, pm = 1.0 / 16, (16, 16, 16), 0.01
    target = OD.grid_mass(x + 0.02, pm, dx, n)
    sdf = OD.target_sdf(target, dx, 32)
    m = OD.grid_mass(x, pm, dx, n)
    g = OD.loss_grad_x(x, pm, dx, m, target, sdf, 0.5, 1.0)
    d = 1e-3 * rng.standard_normal(x.shape)
    eps = 1e-4
    f = lambda y: OD.loss(OD.grid_mass(y, pm, dx, n), target, sdf, 0.5, 1.0)  # noqa: E731
    fd = (f(x + eps * d) - f(x - eps * d)) / (2 * eps)
    assert abs((g * d).sum() - fd) <= 1e-6 * abs(fd)
