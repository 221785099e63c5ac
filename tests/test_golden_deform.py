"""The deform-loss oracle against the reference's own methods (tests/golden/make_deform.py runs
Deform_Loss of tasks/deform_loss.py over compute_grid_m_kernel of object_model/mpm_plastic.py in
float64): the particles' grid mass, the target's distance field after update_target's 2 n passes,
and the weighted loss with its density and distance parts agree to float64 rounding."""
import os

import numpy as np

from oracle import deform as OD
from tests.golden.make_deform import DX, N_GRID, P_MASS, W_DENSITY, W_SDF, cloud

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "deform_ref.npz")


def test_deform_loss_matches_reference_methods():
    g = np.load(GOLDEN)
    x = cloud(0)
    n = (N_GRID,) * 3
    target = OD.grid_mass(x + 0.03, P_MASS, DX, n)
    assert np.allclose(target, g["target"], rtol=1e-13, atol=1e-16)
    m = OD.grid_mass(x, P_MASS, DX, n)
    assert np.allclose(m, g["mass"], rtol=1e-13, atol=1e-16)
    sdf = OD.target_sdf(g["target"], DX, 2 * N_GRID)
    assert np.allclose(sdf, g["sdf"], rtol=1e-13, atol=0)
    assert (g["sdf"] > 0).any() and (g["sdf"] < 1000).all()
    L = OD.loss(m, g["target"], sdf, W_DENSITY, W_SDF)
    dens = np.abs(m - g["target"]).sum()
    assert np.allclose([L, dens, (sdf * m).sum()], g["loss"], rtol=1e-12, atol=0)
