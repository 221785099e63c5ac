"""Rigid shape matching against the reference's own methods (tests/golden/make_rigid.py runs
MultiObj.compute_COM / compute_H / compute_H_svd / compute_R of multi_obj.py in float64): the
covariance restatement the GPU test checks dt_rigid_match against (test_rigid.ref_H, centres divided
by the whole particle count as the reference does) equals the reference's H, and the host rotation
and angle (rigid.RigidMatch.rotation / angle) give its R and compute_angle's increment."""
import os

import numpy as np
import torch

from difftactile_gb300.rigid import RigidMatch
from tests.golden.make_rigid import DT
from tests.test_rigid import ref_H

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rigid_ref.npz")


def test_rigid_match_matches_reference():
    g = np.load(GOLDEN)
    x0, x1, rigid = g["x0"], g["x0"] + DT * g["v1"], g["rigid"]
    N = len(x0)
    assert np.allclose(x0[rigid].sum(0) / N, g["c0"], rtol=1e-13, atol=0)
    assert np.allclose(x1[rigid].sum(0) / N, g["c1"], rtol=1e-13, atol=0)
    H = ref_H(x0, x1, rigid)
    assert np.abs(H - g["H"]).max() < 1e-12 * np.abs(g["H"]).max()
    R = RigidMatch.rotation(torch.as_tensor(g["H"])).numpy()
    assert np.abs(R - g["R"]).max() < 1e-12
    ang = float(RigidMatch.angle(torch.as_tensor(g["R"])))
    assert abs(ang - np.arctan2(g["R"][1, 0], g["R"][1, 1])) < 1e-15 and abs(ang) > 0.01
