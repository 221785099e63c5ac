"""Golden gripper kinematics computed by the reference's own methods.

Gripper of sensor_model/gripper_kinematics.py (eul2mat, init_params, pos_transformation,
grip_kinematic, fem_sensor1/2_set_control_vel, kinematic; :122-296) read out of the reference source
with `ast` and run in float64 through the stand-in `ti` module of this folder (ti_numpy.py): one
control step of a tilted gripper (end-effector pose, finger offsets) with a seeded action, its
finger poses over the step's substeps and the control velocities of two finger pads.  Inputs and
outputs go to tests/golden/gripper_ref.npz.

    python tests/golden/make_gripper.py REFERENCE_ROOT
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from tests.golden import ti_numpy as ti  # noqa: E402

DT, SUB = 1e-3, 5                      # sub_steps = 5: four substeps per control step
ROT, TRANS, GRIP = (10.0, -20.0, 30.0), (0.5, 0.45, 0.55), 0.075
BASE_H, BASE_W, FINGER_H = 0.02, 0.3, 0.1
ACTION = (0.3, -0.2, 0.1, 20.0, -15.0, 10.0, -0.4)  # d_pos, d_ori (deg per unit time), d_gripper


def pads(kin):
    """Two finger pads placed at the fingers' start poses (also rebuilt by tests/test_golden_gripper.py)."""
    from difftactile_gb300 import scene as S
    return [S.finger_pad_sensor(F.numpy(), nx=3, nz=3, ny=2, h=0.01) for F in kin.finger_poses0()]


def kinematics():
    from difftactile_gb300.trajectory import GripperKinematics
    return GripperKinematics(ROT, TRANS, GRIP, DT, base_height=BASE_H, base_width=BASE_W, finger_height=FINGER_H)


def main():
    ref = reference_root()
    src = os.path.join(ref, "difftactile", "sensor_model", "gripper_kinematics.py")
    sens = []
    for sp, F0 in zip(pads(kinematics()), kinematics().finger_poses0()):
        V = len(sp.verts)
        Fi = np.linalg.inv(F0.numpy())
        s = types.SimpleNamespace(n_verts=V, dt=DT, init_x=ti.Field((V,), (3,)), control_vel=ti.Field((SUB, V), (3,)))
        s.init_x.a[:] = (Fi[:3, :3] @ np.asarray(sp.verts, np.float64).T).T + Fi[:3, 3]  # the pad's local frame
        sens.append(s)
    g = types.SimpleNamespace(dt=DT, base_width=BASE_W, base_height=BASE_H, finger_height=FINGER_H,
                              fem_sensor1=sens[0], fem_sensor2=sens[1], d_pos=ti.Field((), (3,)),
                              d_ori=ti.Field((), (3,)), d_gripper=ti.scalar(ACTION[6]), ee_world=ti.Field((), (4, 4)),
                              finger1_t=ti.Field((), (4, 4)), finger2_t=ti.Field((), (4, 4)),
                              grip_delta=ti.Field((SUB,)))
    for k in ("ee_local", "ee", "ee_delta", "finger1_local", "finger2_local", "finger1_ee", "finger2_ee",
              "finger1_delta", "finger2_delta"):
        setattr(g, k, ti.Field((SUB,), (4, 4)))
    g.d_pos[None], g.d_ori[None] = ACTION[0:3], ACTION[3:6]
    ti.methods(src, "Gripper", ["eul2mat", "init_params", "pos_transformation", "grip_kinematic",
                                "fem_sensor1_set_control_vel", "fem_sensor2_set_control_vel", "kinematic"], g)
    g.init_params(ti.Vector(list(ROT)), ti.Vector(list(TRANS)), GRIP)
    for f in range(SUB - 1):
        g.kinematic(f)
    np.savez_compressed(os.path.join(HERE, "gripper_ref.npz"), finger1=g.finger1_ee.a, finger2=g.finger2_ee.a,
                        cv1=sens[0].control_vel.a[:SUB - 1], cv2=sens[1].control_vel.a[:SUB - 1])
    print("finger travel", np.linalg.norm(g.finger1_ee.a[-1, :3, 3] - g.finger1_ee.a[0, :3, 3]),
          "control speed", np.abs(sens[0].control_vel.a[:SUB - 1]).max())


if __name__ == "__main__":
    main()
