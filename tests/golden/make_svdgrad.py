"""Golden SVD adjoint computed by the reference's own method.

MPMObj.single_svd_grad and clamp of object_model/mpm_elastic.py:145-173 (the hand-written adjoint of
ti.svd) read out of the reference source with `ast` and run in float64 through the stand-in `ti`
module of this folder (ti_numpy.py), on 64 seeded decompositions with seeded adjoints of U, S
(diagonal, as the substep produces it) and V.  Inputs and outputs go to tests/golden/svdgrad_ref.npz.

    python tests/golden/make_svdgrad.py REFERENCE_ROOT
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from tests.golden import ti_numpy as ti  # noqa: E402


def main():
    ref = reference_root()
    src = os.path.join(ref, "difftactile", "object_model", "mpm_elastic.py")
    rng = np.random.default_rng(9)
    n = 64
    F = np.eye(3) + 0.3 * rng.standard_normal((n, 3, 3))
    o = types.SimpleNamespace(U_svd=ti.Field((1, n), (3, 3)), S_svd=ti.Field((1, n), (3, 3)),
                              V_svd=ti.Field((1, n), (3, 3)))
    o.U_svd.grad, o.S_svd.grad, o.V_svd.grad = (ti.Field((1, n), (3, 3)) for _ in range(3))
    for p in range(n):
        o.U_svd[0, p], o.S_svd[0, p], o.V_svd[0, p] = ti.svd(F[p])
    o.U_svd.grad.a[0] = rng.standard_normal((n, 3, 3))
    o.V_svd.grad.a[0] = rng.standard_normal((n, 3, 3))
    o.S_svd.grad.a[0] = np.einsum("ni,ij->nij", rng.standard_normal((n, 3)), np.eye(3))
    ti.methods(src, "MPMObj", ["single_svd_grad", "clamp"], o)
    Fb = np.stack([o.single_svd_grad(0, p) for p in range(n)])
    np.savez_compressed(os.path.join(HERE, "svdgrad_ref.npz"), U=o.U_svd.a[0], S=o.S_svd.a[0], V=o.V_svd.a[0],
                        Ub=o.U_svd.grad.a[0], Sb=o.S_svd.grad.a[0], Vb=o.V_svd.grad.a[0], Fb=Fb)
    print("cases", n, "max |F_bar|", np.abs(Fb).max())


if __name__ == "__main__":
    main()
