"""Fisheye projection against golden vectors of the reference's own code (tests/golden/
make_fisheye.py runs project_points_to_pix of difftactile/sensor_model/fisheye_model.py:32-51 on
seeded camera-frame points).  The package's host projection is that function (agreement to 1e-9
px); the oracle's restatement of the kernel-side project_3d_2d (fisheye_model.py:12-30, the one
the CUDA marker readout follows) differs from it only by its 1e-10 norm and 1e-8 atan2 guards
(agreement to 1e-3 px), which pins the projection the GPU readout is checked against."""
import os

import numpy as np

from difftactile_gb300 import markers
from oracle import markers as OM

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fisheye_ref.npz")


def test_host_projection_matches_reference():
    g = np.load(GOLDEN)
    assert g["points"].shape == (512, 3)
    pix = markers.project_points_to_pix(g["points"])
    assert np.abs(pix - g["pix"]).max() < 1e-9


def test_oracle_kernel_projection_matches_reference():
    g = np.load(GOLDEN)
    pix = OM.project_3d_2d(g["points"], markers.DEFAULT_CAM)
    err = np.abs(pix - g["pix"]).max()
    assert err < 1e-3, err
    # the fixture spans the image: angles all around the axis and radii out to the pad's edge
    r = np.linalg.norm(g["pix"] - np.array([markers.DEFAULT_CAM["cx"], markers.DEFAULT_CAM["cy"]]), axis=1)
    assert r.max() > 50.0 and r.min() < 20.0
