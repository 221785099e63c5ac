"""The oracle's SVD adjoint against the reference's own single_svd_grad (tests/golden/make_svdgrad.py
runs mpm_elastic.py:145-173 in float64 on seeded decompositions and adjoints of U, S and V): both of
the oracle's forms agree with it when no adjoint reaches R = U V^T directly (the divided form differs
from the reference's only in how it takes that adjoint)."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "svdgrad_ref.npz")


@pytest.mark.parametrize("mode", [0, 1])
def test_svd_adjoint_matches_reference(mode):
    g = np.load(GOLDEN)
    s = np.einsum("nii->ni", g["S"])
    sb = np.einsum("nii->ni", g["Sb"])
    Fb = O.svd_grad(g["U"], s, g["V"], g["Ub"], sb, g["Vb"], np.zeros_like(g["U"]), mode)
    err = np.abs(Fb - g["Fb"]).max(axis=(1, 2)) / np.maximum(np.abs(g["Fb"]).max(axis=(1, 2)), 1e-30)
    assert err.max() < 1e-11, err.max()
