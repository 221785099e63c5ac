"""The dome sensor mesh against golden vectors of the reference's own generator
(tests/golden/make_dome.py runs FEMDomeSensor.fibonacci_sphere / init_mesh of
difftactile/sensor_model/fem_sensor.py:280-322): identical nodes and layer indices, and the same
tets and surface triangles as sets of vertex tuples (Qhull may order simplices differently across
versions)."""
import os

import numpy as np

from difftactile_gb300 import scene as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dome_ref.npz")


def as_set(simplices):
    return {tuple(sorted(int(i) for i in s)) for s in simplices}


def test_dome_mesh_matches_reference_generator():
    g = np.load(GOLDEN)
    nodes, tets, tris, layers = S.dome_mesh()
    assert nodes.shape == g["nodes"].shape == (1910, 3)
    assert np.array_equal(nodes, g["nodes"])
    assert np.array_equal(layers, g["layers"])
    assert len(tets) == len(g["tets"]) == 8198 and as_set(tets) == as_set(g["tets"])
    assert len(tris) == len(g["tris"]) == 1543 and as_set(tris) == as_set(g["tris"])
