"""Known answers for the readout restatements (no GPU): fisheye projection, IDW marker set-up,
contact-force sum."""
import numpy as np

from difftactile_gb300 import configs
from difftactile_gb300.markers import DEFAULT_CAM, idw_weights, project_points_to_pix
from oracle import markers as OM


def test_fisheye_axis_and_radius():
    cam = DEFAULT_CAM
    # on the optical axis: the principal point (up to the 1e-10 guard in the norm: ~0.01 px)
    p = OM.project_3d_2d(np.array([[0.0, 0.0, 0.1]]), cam)
    assert np.allclose(p, [[cam["cx"], cam["cy"]]], atol=0.05)
    # at angle theta from the axis: radius m f theta, angle omega = atan2(y, x) + pi
    th = 0.3
    d = 0.05
    a = np.array([[d * np.sin(th), 0.0, d * np.cos(th) - cam["plane"]]])
    p = OM.project_3d_2d(a, cam)
    r = cam["m"] * cam["f"] * th
    assert np.allclose(p, [[cam["cx"] - r, cam["cy"]]], rtol=1e-6)


def test_host_projection_matches_device_formula_away_from_guards():
    rng = np.random.default_rng(0)
    a = rng.uniform(-0.05, 0.05, (50, 3))
    assert np.allclose(project_points_to_pix(a.copy()), OM.project_3d_2d(a.copy(), DEFAULT_CAM), rtol=1e-4)


def test_idw_weights_reproduce_the_nodes_they_sit_on():
    pts = np.random.default_rng(1).uniform(0, 100, (40, 2))
    idx, w = idw_weights(pts[:5] + 1e-9, pts, k=5)
    assert np.allclose(w.sum(1), 1.0)
    loc = (w[:, :, None] * pts[idx]).sum(1)
    assert np.allclose(loc, pts[:5], atol=1e-6)


def test_contact_force_sum_is_half_the_vertex_sum_on_a_closed_fan():
    # every vertex of a triangle fan around a centre node: sum of 1/6 per incidence
    ext = np.arange(12, dtype=np.float64).reshape(4, 3)
    tris = np.array([[0, 1, 2], [0, 2, 3], [0, 3, 1]])
    got = OM.contact_force_sum(ext, tris)
    inc = np.array([3, 2, 2, 2])
    assert np.allclose(got, (inc[:, None] * ext).sum(0) / 6)


def test_press_pad_marker_model_geometry():
    from difftactile_gb300.markers import MarkerModel

    class FakeWorld:  # the set-up needs only the sensor specs and a device
        device = "cpu"
        sensor_specs = configs.sensor_press(n_steps=1).envs[0].sensors
        lib = None

    m = MarkerModel(FakeWorld(), 0)  # host set-up only; no readout call
    assert len(m.surf) == 21 * 21
    assert m.markers_2d.shape == (136, 2)
    assert np.allclose(m.wts.sum(1), 1.0)
