"""Golden vectors of the reference's fisheye projection, computed by the reference's own code.

`project_points_to_pix` (difftactile/sensor_model/fisheye_model.py:32-51) is plain numpy, but its
module imports cv2 and taichi at the top, which this environment lacks; the function is therefore
taken out of the reference source with `ast` and run alone with numpy.  Camera-frame points are
seeded (the size of the sensor pad seen by its camera: x, y within 12 mm of the axis, 8-20 mm in
front of the image plane once the plane offset is added).

    python tests/golden/make_fisheye.py REFERENCE_ROOT     # writes tests/golden/fisheye_ref.npz
"""
import ast
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402


def source():
    return os.path.join(reference_root(), "difftactile", "sensor_model", "fisheye_model.py")


def reference_function():
    SRC = source()
    tree = ast.parse(open(SRC).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "project_points_to_pix")
    ns = {"np": np}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), SRC, "exec"), ns)
    return ns["project_points_to_pix"]


def main():
    rng = np.random.default_rng(17)
    n = 512
    pts = np.stack([rng.uniform(-0.012, 0.012, n), rng.uniform(-0.012, 0.012, n), rng.uniform(-0.012, 0.0, n)], 1)
    pix = reference_function()(pts.copy())  # the function shifts z in place
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fisheye_ref.npz")
    np.savez(out, points=pts, pix=pix)
    print("wrote", out, pix.shape)


if __name__ == "__main__":
    main()
