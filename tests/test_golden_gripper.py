"""The gripper's action model against the reference's own methods (tests/golden/make_gripper.py runs
Gripper.init_params / kinematic of gripper_kinematics.py in float64): the host kinematic chain
(trajectory.GripperKinematics.rollout) gives the reference's finger poses at every substep of a control
step, and GripperTrajectory.controls, applied as the device kernel applies it (v = D [x_rest, 1]),
gives the reference's per-vertex control velocities of both finger pads."""
import os
import types

import numpy as np
import torch

from difftactile_gb300.trajectory import GripperTrajectory
from tests.golden.make_gripper import ACTION, DT, SUB, kinematics, pads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gripper_ref.npz")


def test_gripper_chain_and_control_velocities_match_reference():
    g = np.load(GOLDEN)
    kin = kinematics()
    S = SUB - 1
    acts = torch.tensor([ACTION], dtype=torch.float64)
    F = kin.rollout(acts, S)[0].numpy()              # [2, S + 1, 4, 4]
    assert np.abs(F[0] - g["finger1"]).max() < 1e-12 and np.abs(F[1] - g["finger2"]).max() < 1e-12
    tr = GripperTrajectory.__new__(GripperTrajectory)  # the action model only: no world, nothing launches
    tr.kin, tr.T, tr.S = kin, 1, S
    tr.w = types.SimpleNamespace(dt=DT)
    tr.T0_inv = [torch.linalg.inv(F0) for F0 in kin.finger_poses0()]
    D = tr.controls(acts)[0].reshape(2, S, 3, 4).numpy()
    for i, sp in enumerate(pads(kin)):
        src = np.concatenate([np.asarray(sp.verts, np.float64), np.ones((len(sp.verts), 1))], 1)
        cv = np.einsum("fab,vb->fva", D[i], src)
        ref = g[f"cv{i + 1}"]
        assert np.abs(ref).max() > 0.1
        assert np.abs(cv - ref).max() < 1e-9 * np.abs(ref).max(), i
