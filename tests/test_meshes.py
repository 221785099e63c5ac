"""The mesh-to-particles sampling of the reference's ObjLoader.generate_particles (object_model/
obj_loader.py:22-60) on the host: normalisation to the unit extent and the regular sample grid, an
OBJ box (polygon faces) and a triangulated sphere (particle count within 2% of the sphere's volume on
the grid), and the reference-shaped MPMObj construction on top of it (grid spacing, particle volume,
the init transform)."""
import numpy as np

from difftactile_gb300 import meshes
from difftactile_gb300.api import FEMDomeSensor, GripperFEMSensor, MPMObj
from tests.test_api import _sphere_obj


def test_box_obj_fills_the_normalised_box(tmp_path):
    p = tmp_path / "box.obj"
    V = [[x, y, z] for x in (0, 2) for y in (0, 1) for z in (0, 1)]
    quads = [[0, 1, 3, 2], [4, 6, 7, 5], [0, 4, 5, 1], [2, 3, 7, 6], [0, 2, 6, 4], [1, 5, 7, 3]]
    p.write_text("".join(f"v {a} {b} {c}\n" for a, b, c in V) + "".join(
        "f " + " ".join(str(i + 1) for i in q) + "\n" for q in quads))
    x = meshes.generate_particles(str(p), 20)
    # 2 x 1 x 1 scaled to 1 x 0.5 x 0.5 about the origin; samples on faces counted on one side only
    assert len(x) == 20 * 10 * 10
    assert np.allclose(x.min(0), [-0.5, -0.25, -0.25]) and np.all(x.max(0) < [0.5, 0.25, 0.25])


def test_sphere_obj_volume(tmp_path):
    p = tmp_path / "ball.obj"
    _sphere_obj(str(p), n_lat=30, n_lon=60)
    d = 38
    x = meshes.generate_particles(str(p), d)
    expect = 4.0 / 3.0 * np.pi * 0.5 ** 3 * d ** 3
    assert abs(len(x) - expect) < 0.02 * expect
    assert np.linalg.norm(x, axis=1).max() <= 0.5 + 1e-6


def test_reference_shaped_objects_on_the_host(tmp_path):
    p = tmp_path / "ball.obj"
    _sphere_obj(str(p))
    mo = MPMObj(dt=5e-5, sub_steps=5, obj_name=str(p), space_scale=10.0, obj_scale=4.0, density=1.5, rho=4.0)
    assert mo.particle_density == 64 * 1.5 * 4.0 / 10.0 and mo.dx_0 == 10.0 / 64 and mo.rho == 16.0
    assert abs(mo.p_mass - (10.0 / 64 * 4.0) ** 3 * 16.0) < 1e-12 and mo.E_0 == 4e4 and mo.nu_0 == 0.4
    assert np.abs(mo.particles).max() <= 2.0 + 1e-6   # unit extent times obj_scale
    mo.init([5.5, 2.3, 5.8], [0.0, 0.0, 90.0], [0.1, 0.0, 0.0])
    R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])  # 90 degrees about z
    assert np.allclose(mo.x_init, mo.particles @ R.T + [5.5, 2.3, 5.8], atol=1e-5)
    assert np.allclose(mo.v_init, [0.1, 0.0, 0.0])
    s = FEMDomeSensor(dt=5e-5, sub_steps=5)
    s.init(180.0, 0.0, 0.0, 1.0, 2.0, 3.0)
    assert np.allclose(s.spec.out_dir, [0.0, -1.0, 0.0], atol=1e-12) and s.spec.carry == 0
    assert np.allclose(s.spec.verts[:, 1].max(), 2.0, atol=1e-5)   # the dome's base plane at y = 2
    g = GripperFEMSensor(dt=5e-5, sub_steps=5)
    M = np.eye(4)
    M[:3, 3] = [1.0, 2.0, 3.0]
    g.init(M)
    assert g.spec.carry == 1 and np.allclose(g.spec.verts, g.all_nodes + [1.0, 2.0, 3.0], atol=1e-5)
