"""Pose control against the reference's own methods (tests/golden/make_pose.py runs
FEMDomeSensor.set_pose_control / set_control_vel of fem_sensor.py in float64 on the reference dome):
the step transforms of trajectory.PoseTrajectory (all steps and sensors in one batch) and of
api.FEMDomeSensor.set_pose_control equal the reference's dtrans_h, and the control velocity the
device computes from them (cv = ((A vp + b) - vp) / (dt S)) equals the reference's per vertex."""
import os
import types

import numpy as np
import torch

from difftactile_gb300.api import FEMDomeSensor
from difftactile_gb300.trajectory import PoseTrajectory
from tests.golden.make_pose import ACTIONS, DT, SUB, sensor

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pose_ref.npz")


def test_pose_control_matches_reference():
    g = np.load(GOLDEN)
    sp = sensor()
    S = SUB - 1
    M = np.asarray(sp.trans_world, np.float64)
    tr = PoseTrajectory.__new__(PoseTrajectory)  # the action model only: no world, nothing launches
    tr.w, tr.S = types.SimpleNamespace(dt=DT), S
    tr.TW = torch.as_tensor(M[None])
    tr.TW_inv = torch.as_tensor(np.linalg.inv(M)[None])
    Ab = tr.step_transforms(torch.tensor(ACTIONS, dtype=torch.float64)[:, None]).numpy()  # [2, 1, 12]
    assert np.abs(Ab[:, 0] - g["dtrans"][:, :3].reshape(2, 12)).max() < 1e-12
    world = types.SimpleNamespace(sensor_specs=[sp], dt=DT, device="cpu")
    shim = FEMDomeSensor(types.SimpleNamespace(world=world, sub_steps=SUB), 0)
    vp = g["vpos"].astype(np.float64)
    for t, a in enumerate(ACTIONS):
        shim.set_pose_control(a[0:3], a[3:6])
        assert np.abs(shim.dtrans.numpy().reshape(3, 4) - g["dtrans"][t, :3]).max() < 1e-6  # float32 copy
        A, b = Ab[t, 0].reshape(3, 4)[:, :3], Ab[t, 0].reshape(3, 4)[:, 3]
        cv = ((vp @ A.T + b) - vp) / (DT * S)
        assert np.abs(cv - g["cv"][t]).max() < 1e-9 * np.abs(g["cv"][t]).max()
        assert abs(shim.inv_T - 1.0 / (DT * S)) < 1e-9
