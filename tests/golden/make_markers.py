"""Golden marker readout computed by the reference's own code.

FEMDomeSensor.init_cam_model (sensor_model/fem_sensor.py:130-159: the outer layer's nodes projected
by project_points_to_pix, every marker interpolated from its 5 nearest projected nodes) and
extract_markers (:161-187, with project_3d_2d of sensor_model/fisheye_model.py:12-30) are read out
of the reference source with `ast` and run in float64 through the stand-in `ti` module of this folder
(ti_numpy.py).  The OpenCV detection of the marker pixels in init.png that init_cam_model starts
from is replaced by a seeded marker set (its only output).  The sensor is the reference's dome in
the dome parity scene of tests/small_scenes.py; the readout runs on a displaced surface and a moved
sensor pose.  Inputs and outputs go to tests/golden/markers_ref.npz.

    python tests/golden/make_markers.py REFERENCE_ROOT
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


def sensor():
    """The dome of the dome parity scene (also rebuilt by tests/test_golden_markers.py)."""
    return SS.dome_over_box().sensors[0]


def pose_shift():
    """World-to-sensor transform of the readout: the rest pose moved by a small rotation about z and
    a translation."""
    c, s = np.cos(0.02), np.sin(0.02)
    D = np.array([[c, -s, 0, 0.003], [s, c, 0, -0.002], [0, 0, 1, 0.001], [0, 0, 0, 1.0]])
    return D


def main():
    ref = reference_root()
    fem = os.path.join(ref, "difftactile", "sensor_model", "fem_sensor.py")
    fish = os.path.join(ref, "difftactile", "sensor_model", "fisheye_model.py")
    sp = sensor()
    M = np.asarray(sp.trans_world, np.float64)
    Mi = np.linalg.inv(M)
    verts = np.asarray(sp.verts, np.float64)
    local = (Mi[:3, :3] @ verts.T).T + Mi[:3, 3]
    layer = np.asarray(sp.layer)
    rng = np.random.default_rng(3)

    fns = ti.functions(fish, ["project_3d_2d", "project_points_to_pix"])
    surf = np.where(layer == 3)[0]  # fem_sensor.py:55, N_t - 1 = 3
    pix = fns["project_points_to_pix"](local[surf][:, [0, 2, 1]].copy())
    lo, hi = pix.min(0), pix.max(0)
    markers = lo + (hi - lo) * (0.15 + 0.7 * rng.random((40, 2)))  # seeded stand-in for the detection

    cam = types.SimpleNamespace(all_nodes=local, surface_id_np=surf, num_k_closest=5)
    ti.methods(fem, "FEMDomeSensor", ["init_cam_model"], cam,
               extra={"cv2": types.SimpleNamespace(imread=lambda path: None),
                      "get_marker_image": lambda img: markers,
                      "project_points_to_pix": fns["project_points_to_pix"]})
    surf_2d, interp_idx, interp_weight = cam.init_cam_model()

    V, S_, Mk = len(verts), len(surf), len(markers)
    s = types.SimpleNamespace(num_surface=S_, num_markers=Mk, num_k_closest=5, surface_id=ti.Field((S_,), (), np.int64),
                              pos=ti.Field((1, V), (3,)), virtual_pos=ti.Field((1, V), (3,)),
                              inv_trans_h=ti.Field((), (4, 4)), surface_cam_loc=ti.Field((S_,), (2,)),
                              surface_cam_virtual_loc=ti.Field((S_,), (2,)),
                              interp_idx=ti.Field((Mk,), (5,), np.int64), interp_weight=ti.Field((Mk,), (5,)),
                              predict_markers=ti.Field((Mk,), (2,)), virtual_markers=ti.Field((Mk,), (2,)))
    s.surface_id.a[:] = surf
    pos = np.asarray(verts + 2e-3 * rng.standard_normal(verts.shape), np.float32).astype(np.float64)
    s.pos.a[0], s.virtual_pos.a[0] = pos, verts
    inv_trans = np.linalg.inv(M @ pose_shift())
    s.inv_trans_h[None] = inv_trans
    s.interp_idx.a[:], s.interp_weight.a[:] = interp_idx, interp_weight
    ti.methods(fem, "FEMDomeSensor", ["extract_markers"], s, extra={"project_3d_2d": fns["project_3d_2d"]})
    s.extract_markers(0)
    np.savez_compressed(os.path.join(HERE, "markers_ref.npz"), markers=markers, surf=surf.astype(np.int32),
                        surf_2d=surf_2d, idx=interp_idx.astype(np.int32), wts=interp_weight, pos=pos,
                        inv_trans=inv_trans, pred=s.predict_markers.a, virt=s.virtual_markers.a)
    shift = np.linalg.norm(s.predict_markers.a - s.virtual_markers.a, axis=1)
    print(f"{Mk} markers over {S_} surface nodes, marker shift {shift.mean():.3g} px mean")


if __name__ == "__main__":
    main()
