"""The marker readout against the reference's own code (tests/golden/make_markers.py runs
FEMDomeSensor.init_cam_model and extract_markers of fem_sensor.py with fisheye_model.py's
projections, in float64): the package's host set-up (markers.MarkerModel: surface nodes, projected
positions, 5 nearest nodes and inverse-distance weights of every marker) and the oracle's readout of
a displaced surface under a moved pose (oracle/markers.py, the restatement the CUDA readout is
checked against) agree to float64 rounding."""
import os
import types

import numpy as np

from difftactile_gb300.markers import MarkerModel
from oracle import markers as OM
from tests.golden.make_markers import sensor

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "markers_ref.npz")


def test_marker_setup_and_readout_match_reference():
    g = np.load(GOLDEN)
    sp = sensor()
    world = types.SimpleNamespace(sensor_specs=[sp], device="cpu")  # host set-up only, nothing launches
    mm = MarkerModel(world, 0, markers_2d=g["markers"], k=5)
    assert np.array_equal(mm.surf, g["surf"])
    assert np.array_equal(mm.idx, g["idx"])
    assert np.allclose(mm.wts, g["wts"], rtol=1e-12, atol=0)
    surf_2d = (mm.wts[:, :, None] * mm.cam_points[mm.idx]).sum(1)
    assert np.allclose(surf_2d, g["surf_2d"], rtol=1e-12, atol=0)
    pred, virt = OM.extract_markers(g["pos"], sp.verts.astype(np.float64), mm.surf, mm.idx, mm.wts, g["inv_trans"],
                                    mm.cam)
    assert np.abs(pred - g["pred"]).max() < 1e-9 and np.abs(virt - g["virt"]).max() < 1e-9
    assert np.abs(g["pred"] - g["virt"]).max() > 0.5  # the displaced surface moves the markers
