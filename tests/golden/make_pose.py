"""Golden pose control computed by the reference's own methods.

FEMDomeSensor.eul2mat, set_pose_control and set_control_vel (sensor_model/fem_sensor.py:196-266) read
out of the reference source with `ast` and run in float64 through the stand-in `ti` module of this
folder (ti_numpy.py): the reference dome of the dome parity scene (its world pose trans_world), two
seeded actions applied one after the other, the step transform dtrans_h of each and the control
velocity of every vertex from the virtual positions.  Inputs and outputs go to
tests/golden/pose_ref.npz.

    python tests/golden/make_pose.py REFERENCE_ROOT
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from tests import small_scenes as SS  # noqa: E402
from tests.golden import ti_numpy as ti  # noqa: E402

DT, SUB = 1e-4, 21                        # sub_steps = 21: 20 substeps per control step
ACTIONS = ((0.3, -0.5, 0.2, 10.0, -20.0, 5.0), (-0.1, 0.4, 0.0, -3.0, 0.0, 12.0))  # d_pos, d_ori (deg/s)


def sensor():
    """The dome of the dome parity scene (also rebuilt by tests/test_golden_pose.py)."""
    return SS.dome_over_box().sensors[0]


def main():
    ref = reference_root()
    src = os.path.join(ref, "difftactile", "sensor_model", "fem_sensor.py")
    sp = sensor()
    M = np.asarray(sp.trans_world, np.float64)
    V = len(sp.verts)
    rng = np.random.default_rng(4)
    vpos = np.asarray(np.asarray(sp.verts, np.float64) + 1e-3 * rng.standard_normal((V, 3)), np.float32)
    s = types.SimpleNamespace(dt=DT, sub_steps=SUB, n_verts=V, d_pos=ti.Field((), (3,)), d_ori=ti.Field((), (3,)),
                              virtual_pos=ti.Field((1, V), (3,)), control_vel=ti.Field((V,), (3,)))
    for k in ("dtrans_h", "trans_world", "trans_local", "trans_h", "inv_trans_h"):
        setattr(s, k, ti.Field((), (4, 4)))
    for k in ("rot_world", "rot_local", "rot_h", "inv_rot"):
        setattr(s, k, ti.Field((), (3, 3)))
    s.trans_world[None], s.trans_local[None] = M, np.eye(4)
    s.rot_world[None], s.rot_local[None] = M[:3, :3], np.eye(3)
    s.virtual_pos.a[0] = vpos
    ti.methods(src, "FEMDomeSensor", ["eul2mat", "set_pose_control", "set_control_vel"], s)
    dtrans, cv, trans_h = [], [], []
    for a in ACTIONS:
        s.d_pos[None], s.d_ori[None] = a[0:3], a[3:6]
        s.set_pose_control()
        s.set_control_vel(0)
        dtrans.append(s.dtrans_h.a.copy())
        cv.append(s.control_vel.a.copy())
        trans_h.append(s.trans_h.a.copy())
    np.savez_compressed(os.path.join(HERE, "pose_ref.npz"), vpos=vpos, dtrans=np.stack(dtrans), cv=np.stack(cv),
                        trans_h=np.stack(trans_h))
    print("control speed", [float(np.abs(c).max()) for c in cv])


if __name__ == "__main__":
    main()
