"""Rigid shape matching readout (multi_obj.py:309-340) on the GPU: H against numpy, and the angle
loss gradient with respect to both frames' particle positions against float64 finite differences
(2e-3 relative)."""
import numpy as np
import pytest
import torch

from difftactile_gb300 import scene as S
from difftactile_gb300.rigid import RigidMatch
from difftactile_gb300.world import World
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4


def ref_H(x0, x1, rigid):
    N_ = len(x0)
    c0 = x0[rigid].sum(0) / N_
    c1 = x1[rigid].sum(0) / N_
    return np.einsum("pi,pj->ij", x0[rigid] - c0, x1[rigid] - c1)


def angle_of(H):
    U, _, Vt = np.linalg.svd(H)
    R = Vt.T @ U.T
    return np.arctan2(R[1, 0], R[1, 1])


def test_rigid_match_and_angle_gradient(cuda_lib):
    env = SS.elastic_cube(n=32, side_cells=6, gravity=(0.0, 0.0, 0.0))
    x = env.x.astype(np.float64)
    c = x.mean(0)
    omega = 50.0  # spin about z: 5e-3 rad per substep
    v = np.stack([-omega * (x[:, 1] - c[1]), omega * (x[:, 0] - c[0]), np.zeros(len(x))], 1)
    # the whole object is the rigid material (the box-opening case): the reference divides the rigid
    # sums by the object's particle count, which is the centre of mass only when all are rigid
    core = np.ones(len(x), bool)
    env = env.replace(v=v.astype(np.float32), mat=core.astype(np.int32),
                      materials=[S.Material(5e3, 0.3), S.Material(5e5, 0.3)])
    w = World([env], n_frames=2, dt=DT)
    w.step_begin()
    w.substep(0)
    rm = RigidMatch(w, 0, mat=1)
    c0, c1, H = rm.H(0)
    torch.cuda.synchronize()
    x0 = w.particles(0)["x"].double().cpu().numpy()
    x1 = w.particles(1)["x"].double().cpu().numpy()
    Hr = ref_H(x0, x1, core)
    assert SS.rel_err(H.cpu().numpy(), Hr) < 1e-4
    # loss = angle^2: d/dH by autograd, then back to the particles of both frames
    Ht = H.double().cpu().requires_grad_(True)
    ang = RigidMatch.angle(RigidMatch.rotation(Ht))
    assert abs(float(ang.detach()) - angle_of(Hr)) < 1e-3 * abs(angle_of(Hr))
    (Hb,) = torch.autograd.grad(ang ** 2, Ht)
    w.adj_clear()
    rm.backward(0, Hb, 0)
    rm.backward(0, Hb, 1)
    torch.cuda.synchronize()
    g0 = w.particle_adjoint(0)["x"].double().cpu().numpy()
    g1 = w.particle_adjoint(1)["x"].double().cpu().numpy()
    rng = np.random.default_rng(3)
    for trial in range(3):
        d0, d1 = 1e-4 * rng.standard_normal(x0.shape), 1e-4 * rng.standard_normal(x1.shape)
        L = lambda s: angle_of(ref_H(x0 + s * d0, x1 + s * d1, core)) ** 2  # noqa: E731
        eps = 1e-2
        fd = (L(eps) - L(-eps)) / (2 * eps)
        pred = float((g0 * d0).sum() + (g1 * d1).sum())
        assert abs(pred - fd) <= 2e-3 * abs(fd) + 1e-12, (trial, pred, fd)
