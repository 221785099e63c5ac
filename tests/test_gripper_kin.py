"""Gripper kinematic chain (gripper_kinematics.py:120-194) on the host (no GPU)."""
import numpy as np
import torch

from difftactile_gb300.trajectory import GripperKinematics, eul2mat_xyz


def test_eul2mat_xyz_is_rx_ry_rz():
    from scipy.spatial.transform import Rotation
    rng = np.random.default_rng(0)
    for _ in range(5):
        a = rng.uniform(-180, 180, 3)
        M = eul2mat_xyz(torch.as_tensor(a), torch.tensor([1.0, 2.0, 3.0], dtype=torch.float64)).numpy()
        R = Rotation.from_euler("XYZ", a, degrees=True).as_matrix()  # intrinsic x-y-z = Rx Ry Rz
        assert np.allclose(M[:3, :3], R, atol=1e-12)
        assert np.allclose(M[:3, 3], [1, 2, 3])


def test_no_action_keeps_the_fingers_still():
    k = GripperKinematics([10.0, 0.0, 5.0], [0.5, 0.5, 0.5], 0.07, 1e-4, base_height=0.02, base_width=0.3,
                          finger_height=0.1)
    F = k.rollout(torch.zeros((2, 7), dtype=torch.float64), 3)
    F0 = torch.stack(k.finger_poses0())
    assert torch.allclose(F, F0[None, :, None].expand_as(F))


def test_grip_moves_each_finger_along_its_local_y():
    dt, S, dg = 1e-3, 4, 2.0
    k = GripperKinematics([0.0, 0.0, 0.0], [0.5, 0.5, 0.5], 0.07, dt, base_height=0.02, base_width=0.3,
                          finger_height=0.1)
    a = torch.zeros((1, 7), dtype=torch.float64)
    a[0, 6] = dg
    F = k.rollout(a, S)[0]
    for i in range(2):
        y = F[i, 0, :3, 1]
        assert torch.allclose(F[i, -1, :3, 3] - F[i, 0, :3, 3], S * dg * dt * y)
    # the fingers approach each other
    gap0 = (F[1, 0, :3, 3] - F[0, 0, :3, 3]).norm()
    gap1 = (F[1, -1, :3, 3] - F[0, -1, :3, 3]).norm()
    assert torch.isclose(gap0 - gap1, torch.tensor(2 * S * dg * dt, dtype=torch.float64))


def test_end_effector_translation_carries_both_fingers():
    dt, S = 1e-3, 3
    k = GripperKinematics([0.0, 0.0, 0.0], [0.5, 0.5, 0.5], 0.07, dt, base_height=0.02, base_width=0.3,
                          finger_height=0.1)
    a = torch.zeros((2, 7), dtype=torch.float64)
    a[:, 1] = -0.5
    F = k.rollout(a, S)
    for i in range(2):
        d = F[-1, i, -1, :3, 3] - F[0, i, 0, :3, 3]
        assert torch.allclose(d, torch.tensor([0.0, -0.5 * dt * 2 * S, 0.0], dtype=torch.float64))
