"""Pose control of every sensor in one launch: dt_pose_control_vel_all and
dt_pose_control_vel_bwd_all give the per-sensor entry points' control velocities, step-transform
adjoints and virtual-position adjoints (set_pose_control + set_control_vel, fem_sensor.py:229-266),
on three environments with one or two pads each (sensor boundaries inside CTAs and warps)."""
import numpy as np
import pytest
import torch

from difftactile_gb300 import _native as N
from difftactile_gb300.world import World
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu


def world():
    envs = [SS.pad_over_box(seed=1, two_pads=True), SS.pad_over_box(seed=2), SS.pad_over_box(seed=3, two_pads=True)]
    return World(envs, n_frames=6, dt=1e-4)


def transforms(n, seed=4):
    rng = np.random.default_rng(seed)
    Ab = np.zeros((n, 12), np.float32)
    Ab[:, [0, 5, 10]] = 1.0
    Ab += 1e-3 * rng.standard_normal((n, 12)).astype(np.float32)
    return torch.as_tensor(Ab, device="cuda")


def test_forward_all_matches_per_sensor(cuda_lib):
    w = world()
    Ab = transforms(w.n_sensors)
    inv_T = 1.0 / (w.dt * 5)
    for s in range(w.n_sensors):
        N.check(w.lib.dt_pose_control_vel(w.wp, s, Ab[s].data_ptr(), inv_T, 0, 6, w.stream), "cv")
    per = w.t["v_cv"].clone()
    w.t["v_cv"].zero_()
    N.check(w.lib.dt_pose_control_vel_all(w.wp, Ab.data_ptr(), inv_T, 0, 6, w.stream), "cv all")
    torch.cuda.synchronize()
    assert torch.equal(per, w.t["v_cv"])


def test_adjoint_all_matches_per_sensor(cuda_lib):
    w = world()
    Ab = transforms(w.n_sensors)
    inv_T = 1.0 / (w.dt * 5)
    rng = np.random.default_rng(9)
    seed = torch.as_tensor(rng.standard_normal(tuple(w.t["v_adj_cv"].shape)).astype(np.float32), device="cuda")
    seed[..., 3] = 0.0
    out = []
    for mode in ("per", "all"):
        w.adj_clear()
        w.t["v_adj_cv"].copy_(seed)
        bar = torch.zeros((w.n_sensors, 12), device="cuda")
        if mode == "per":
            for s in range(w.n_sensors):
                N.check(w.lib.dt_pose_control_vel_bwd(w.wp, s, Ab[s].data_ptr(), inv_T, bar[s].data_ptr(), 0, 6,
                                                      w.stream), "cv bwd")
        else:
            N.check(w.lib.dt_pose_control_vel_bwd_all(w.wp, Ab.data_ptr(), inv_T, bar.data_ptr(), 0, 6, w.stream),
                    "cv bwd all")
        torch.cuda.synchronize()
        assert float(w.t["v_adj_cv"].abs().max()) == 0.0  # consumed
        out.append((bar.cpu().numpy(), w.t["v_adj_vpos"][0].cpu().numpy()))
    assert SS.rel_err(out[1][0], out[0][0]) < 1e-5
    assert SS.rel_err(out[1][1], out[0][1]) < 1e-5
    assert np.abs(out[0][0]).min() > 0.0  # every sensor received an adjoint
