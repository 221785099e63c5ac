"""Configurations end to end on the GPU: reduced-size configuration 3 (gripper, core/shell sphere)
and configuration 5 (ropes under large pads, several environments) roll out and back-propagate to
finite action gradients; configuration 1's loss (final centre-of-mass height) differentiated with
respect to the initial velocity matches float64 finite differences of the oracle (2e-3)."""
import numpy as np
import pytest
import torch

from difftactile_gb300 import configs
from difftactile_gb300 import scene as S
from difftactile_gb300.trajectory import GripperTrajectory, PoseTrajectory, Trajectory
from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu


def test_grasp_sphere_reduced_rolls_out_and_back(cuda_lib):
    cfg, kin = configs.grasp_sphere(n_steps=2, substeps=5, n_grid=64, n_core=2000, n_shell=18000, pad=(8, 8, 2),
                                    ckpt_every=1)
    env = cfg.envs[0]
    terms = tuple((s, int(sp.layer.max()), np.zeros(sp.verts.shape)) for s, sp in enumerate(env.sensors))
    w = World(cfg.envs, n_frames=Trajectory.frames_needed(2, 5, 1), dt=cfg.dt)
    tr = GripperTrajectory(w, 2, kin, (0, 1), 1, terms)
    loss = tr.forward(torch.as_tensor(cfg.actions, dtype=torch.float64, device=w.device))
    g = tr.backward()
    torch.cuda.synchronize()
    assert w.error_word() == 0
    assert torch.isfinite(loss).all() and torch.isfinite(g).all()
    assert float(g.abs().sum()) > 0


def test_rope_pads_reduced_rolls_out_and_back(cuda_lib):
    cfg = configs.rope_pads(n_envs=2, n_steps=2, substeps=5, n_rope=200, pad=(10, 10, 2), n_particles=4000,
                            n_grid=64)
    rng = np.random.default_rng(0)
    terms = tuple((e, int(env.sensors[0].layer.max()), 1e-4 * rng.standard_normal(env.sensors[0].verts.shape))
                  for e, env in enumerate(cfg.envs))
    w = World(cfg.envs, n_frames=Trajectory.frames_needed(2, 5, 0), dt=cfg.dt)
    tr = PoseTrajectory(w, 2, 0, terms)
    loss = tr.forward(torch.as_tensor(cfg.actions, dtype=torch.float64, device=w.device))
    g = tr.backward()
    torch.cuda.synchronize()
    assert w.error_word() == 0
    assert torch.isfinite(loss).all() and torch.isfinite(g).all()
    assert float(g.abs().sum()) > 0
    rs = w.rope_state(2 * 5, 0)
    assert torch.isfinite(rs["pos"]).all()


def test_elastic_cube_com_gradient_wrt_initial_velocity(cuda_lib):
    """Configuration 1's task in small: loss = final centre-of-mass height, gradient with respect to
    a uniform initial velocity (grasp_plastic.py:259-261 readout through the full adjoint)."""
    env = SS.elastic_cube(n=32, side_cells=6, model=S.MODEL_NEOHOOKEAN, bc=S.BC_STICKY_FLOOR,
                          center=(0.5, 0.25, 0.5))
    env = env.replace(eps=1e-3 * env.p_mass)
    n_sub = 20
    w = World([env], n_frames=n_sub + 1, dt=1e-4, grad_clip=0.0)
    w.step_begin()
    for f in range(n_sub):
        w.substep(f)
    com = w.com(n_sub)
    w.adj_clear()
    gb = torch.zeros((1, 4), device=w.device)
    gb[0, 1] = 1.0
    assert w.lib.dt_com_bwd(w.wp, n_sub, gb.data_ptr(), w.stream) == 0
    w.substeps_bwd(n_sub, 0)
    torch.cuda.synchronize()
    gv = w.particle_adjoint(0)["v"].double().cpu().numpy()
    d = np.array([0.3, -1.0, 0.2])
    pred = float((gv * d).sum())
    o = O.Oracle(env, 1e-4, np.float64)

    def L(eps):
        st = o.initial_state()
        st["v"] = st["v"] + eps * d
        for _ in range(n_sub):
            st, _ = o.substep(st)
        return float(st["x"][:, 1].mean())

    e = 1e-3
    fd = (L(e) - L(-e)) / (2 * e)
    assert abs(float(com[0, 1]) - L(0.0)) < 1e-5
    assert abs(pred - fd) <= 2e-3 * abs(fd), (pred, fd)
