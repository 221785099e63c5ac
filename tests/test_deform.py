"""Shape-target loss on the GPU (Deform_Loss, tasks/deform_loss.py:8-146) against the float64 numpy
restatement: mass grid and loss within 1e-5 relative, target distance field within 1e-5, the
particle-position adjoint within 1e-4."""
import numpy as np
import pytest
import torch

from difftactile_gb300.deform import DeformLoss
from difftactile_gb300.world import World
from oracle import deform as OD
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu


def test_deform_loss_matches_oracle(cuda_lib):
    env = SS.elastic_cube(n=32, side_cells=8)
    w = World([env], n_frames=2, dt=1e-4)
    x = env.x.astype(np.float64)
    n = tuple(env.n_grid)
    target = OD.grid_mass(x + np.array([0.04, -0.02, 0.01]), env.p_mass, env.dx, n)
    dl = DeformLoss(w, 0, sdf_weight=1.0, density_weight=0.5)
    dl.initialize(target)
    sdf_ref = OD.target_sdf(target, env.dx, 2 * max(n))
    assert SS.rel_err(dl.to_dense(dl.sdf).cpu().numpy(), sdf_ref) < 1e-5
    loss = float(dl.compute_loss(0).item())
    m_ref = OD.grid_mass(x, env.p_mass, env.dx, n)
    assert SS.rel_err(dl.to_dense(dl.m).cpu().numpy(), m_ref) < 1e-5
    L_ref = OD.loss(m_ref, target, sdf_ref, 0.5, 1.0)
    assert abs(loss - L_ref) <= 1e-5 * abs(L_ref)
    w.adj_clear()
    dl.compute_loss_grad(0, 1.0)
    torch.cuda.synchronize()
    g = w.particle_adjoint(0)["x"].double().cpu().numpy()
    g_ref = OD.loss_grad_x(x, env.p_mass, env.dx, m_ref, target, sdf_ref, 0.5, 1.0)
    assert SS.rel_err(g, g_ref) < 1e-4
    # soft IoU (deform_loss.py:128-142): I = sum(a b) / (max a max b), U = sum a / max a + sum b / max b
    a, b = m_ref, target
    inter = (a * b).sum() / a.max() / b.max()
    iou_ref = inter / (a.sum() / a.max() + b.sum() / b.max() - inter)
    assert abs(dl.iou() - iou_ref) <= 1e-5 * abs(iou_ref)
