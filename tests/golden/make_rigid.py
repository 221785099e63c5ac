"""Golden rigid shape matching computed by the reference's own methods.

MultiObj.compute_COM, compute_H, compute_H_svd and compute_R of object_model/multi_obj.py:309-334 read
out of the reference source with `ast` and run in float64 through the stand-in `ti` module of this
folder (ti_numpy.py): a seeded particle cloud of which 60% carry the rigid material tag, moved over
one substep by a rotation about z plus noise; the centres (divided by the whole particle count, as the
reference does), the covariance H and R = V U^T go to tests/golden/rigid_ref.npz.

    python tests/golden/make_rigid.py REFERENCE_ROOT
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from tests.golden import ti_numpy as ti  # noqa: E402

DT = 1e-4


def main():
    ref = reference_root()
    src = os.path.join(ref, "difftactile", "object_model", "multi_obj.py")
    rng = np.random.default_rng(8)
    N = 300
    x0 = np.asarray(rng.uniform(0.4, 0.6, (N, 3)), np.float32).astype(np.float64)
    rigid = rng.random(N) < 0.6
    c, s = np.cos(0.05), np.sin(0.05)
    Rz = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    x1 = (x0 - 0.5) @ Rz.T + 0.5 + 1e-4 * rng.standard_normal((N, 3))
    v1 = np.asarray((x1 - x0) / DT, np.float32).astype(np.float64)     # x_{f+1} = x_f + dt v_{f+1}
    o = types.SimpleNamespace(n_particles=N, dt=DT, titles=ti.Field((N,), (1,), np.int64), x_0=ti.Field((2, N), (3,)),
                              v_0=ti.Field((2, N), (3,)), COM_t0=ti.Field((1,), (3,)), COM_t1=ti.Field((1,), (3,)))
    for k in ("H", "U", "S", "V", "R"):
        setattr(o, k, ti.Field((1,), (3, 3)))
    o.titles.a[:, 0] = np.where(rigid, 2, 1)
    o.x_0.a[0], o.v_0.a[1] = x0, v1
    ti.methods(src, "MultiObj", ["compute_COM", "compute_H", "compute_H_svd", "compute_R"], o)
    for name in ("compute_COM", "compute_H", "compute_H_svd", "compute_R"):
        getattr(o, name)(0)
    np.savez_compressed(os.path.join(HERE, "rigid_ref.npz"), x0=x0, v1=v1, rigid=rigid, c0=o.COM_t0.a[0],
                        c1=o.COM_t1.a[0], H=o.H.a[0], R=o.R.a[0])
    print("det H", np.linalg.det(o.H.a[0]), "angle", np.arctan2(o.R.a[0][1, 0], o.R.a[0][1, 1]))


if __name__ == "__main__":
    main()
