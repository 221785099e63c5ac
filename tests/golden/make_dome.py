"""Golden dome-sensor mesh computed by the reference's own code.

FEMDomeSensor.init_mesh and fibonacci_sphere (difftactile/sensor_model/fem_sensor.py:280-322) are
numpy + scipy; their module needs taichi, which this environment lacks, so the two methods are
taken out of the reference source with `ast` and run on a stand-in object carrying the sensor's
constructor constants (N_node 200, N_t 4, t_res 0.25, inner_radius 0.75, fem_sensor.py:24-27).

    python tests/golden/make_dome.py REFERENCE_ROOT     # writes tests/golden/dome_ref.npz
"""
import ast
import os
import sys
import types

import numpy as np
from scipy.spatial import Delaunay

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402


def source():
    return os.path.join(reference_root(), "difftactile", "sensor_model", "fem_sensor.py")


def reference_methods():
    SRC = source()
    tree = ast.parse(open(SRC).read())
    cls = next(n for n in tree.body if isinstance(n, ast.ClassDef) and n.name == "FEMDomeSensor")
    fns = [n for n in cls.body if isinstance(n, ast.FunctionDef) and n.name in ("fibonacci_sphere", "init_mesh")]
    for fn in fns:
        fn.decorator_list = []
    ns = {"np": np, "Delaunay": Delaunay}
    exec(compile(ast.Module(body=fns, type_ignores=[]), SRC, "exec"), ns)
    return ns["fibonacci_sphere"], ns["init_mesh"]


def main():
    fib, init_mesh = reference_methods()
    me = types.SimpleNamespace(N_node=200, N_t=4, t_res=0.25, inner_radius=0.75)
    me.fibonacci_sphere = types.MethodType(fib, me)
    nodes, tets, tris, layers = init_mesh(me)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dome_ref.npz")
    np.savez_compressed(out, nodes=nodes, tets=tets.astype(np.int32), tris=tris.astype(np.int32),
                        layers=layers.astype(np.int32))
    print("wrote", out, nodes.shape, tets.shape, tris.shape)


if __name__ == "__main__":
    main()
