"""ORACLE (test infrastructure only): float64 numpy restatement of the shape-target loss
(difftactile/tasks/deform_loss.py:8-146) and the mass-only P2G it reads
(compute_grid_m_kernel, difftactile/object_model/mpm_plastic.py:169-178).  Pinned against the
reference's own methods run on a numpy stand-in for Taichi (tests/golden/make_deform.py,
tests/test_golden_deform.py: grid mass, distance field and loss to float64 rounding) and by the
known answers in tests/test_oracle_deform.py; the gradient by finite differences."""
from __future__ import annotations

import numpy as np


def _weights(x, inv_dx):
    base = (x * inv_dx - 0.5).astype(np.int64)  # truncation toward zero, as cast(int)
    fx = x * inv_dx - base
    w = np.stack([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2], 1)  # [N, 3, 3]
    dw = np.stack([fx - 1.5, -2.0 * (fx - 1.0), fx - 0.5], 1)
    return base, w, dw


def grid_mass(x, p_mass, dx, n):
    x = np.asarray(x, np.float64)
    base, w, _ = _weights(x, 1.0 / dx)
    m = np.zeros(n)
    for a in range(3):
        for b in range(3):
            for c in range(3):
                W = w[:, a, 0] * w[:, b, 1] * w[:, c, 2] * p_mass
                np.add.at(m, (base[:, 0] + a, base[:, 1] + b, base[:, 2] + c), W)
    return m


def loss(m, target, sdf, wd, ws):
    return wd * np.abs(m - target).sum() + ws * (sdf * m).sum()


def loss_grad_x(x, p_mass, dx, m, target, sdf, wd, ws):
    x = np.asarray(x, np.float64)
    inv_dx = 1.0 / dx
    base, w, dw = _weights(x, inv_dx)
    g = wd * np.sign(m - target) + ws * sdf
    out = np.zeros_like(x)
    for a in range(3):
        for b in range(3):
            for c in range(3):
                gm = g[base[:, 0] + a, base[:, 1] + b, base[:, 2] + c] * p_mass
                out[:, 0] += gm * dw[:, a, 0] * w[:, b, 1] * w[:, c, 2]
                out[:, 1] += gm * w[:, a, 0] * dw[:, b, 1] * w[:, c, 2]
                out[:, 2] += gm * w[:, a, 0] * w[:, b, 1] * dw[:, c, 2]
    return inv_dx * out


def target_sdf(target, dx, passes):
    """update_target x passes: nearest-seed propagation over offsets in [-3, 3)^3 \\ {0}."""
    n = target.shape
    ii = np.stack(np.meshgrid(*[np.arange(v) for v in n], indexing="ij"), -1)
    gp = ii * dx
    inf = 1000.0
    sdf_c = np.full(n, inf)
    near_c = np.zeros(n + (3,))
    seed = target > 1e-4
    offs = [(a, b, c) for a in range(-3, 3) for b in range(-3, 3) for c in range(-3, 3) if (a, b, c) != (0, 0, 0)]
    for _ in range(passes):
        sdf = np.full(n, inf)
        near = np.zeros(n + (3,))
        for a, b, c in offs:  # loop order of ti.ndrange: first minimum wins
            v = ii + np.array([a, b, c])
            ok = np.all((v >= 0) & (v < np.array(n)), -1)
            vv = np.where(ok[..., None], v, 0)
            q_sdf = sdf_c[vv[..., 0], vv[..., 1], vv[..., 2]]
            q_near = near_c[vv[..., 0], vv[..., 1], vv[..., 2]]
            cand = ok & (q_sdf < inf)
            d = np.sqrt(((gp - q_near) ** 2).sum(-1) + 1e-8)
            better = cand & (d < sdf)
            sdf = np.where(better, d, sdf)
            near = np.where(better[..., None], q_near, near)
        sdf = np.where(seed, 0.0, sdf)
        near = np.where(seed[..., None], gp, near)
        sdf_c, near_c = sdf, near
    return sdf_c
