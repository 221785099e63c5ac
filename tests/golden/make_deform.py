"""Golden shape-target loss computed by the reference's own methods.

Deform_Loss of tasks/deform_loss.py (update_target_sdf / update_target, compute_density_loss_kernel,
compute_sdf_loss_kernel, sum_up_loss_kernel, compute_loss_kernel; :56-124) over the mass-only P2G
compute_grid_m_kernel of object_model/mpm_plastic.py:169-178, read out of the reference source with
`ast` and run in float64 on numpy fields through the stand-in `ti` module of this folder
(ti_numpy.py).  A seeded particle cloud on a 12^3 grid and a target density made from a shifted copy
of it; the target's distance field (2 n passes of the nearest-seed propagation, as update_target
runs them), the particles' grid mass and the weighted loss go to tests/golden/deform_ref.npz.

    python tests/golden/make_deform.py REFERENCE_ROOT
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from tests.golden import ti_numpy as ti  # noqa: E402

N_GRID = 12
DX = 1.0 / N_GRID
P_MASS = 0.01
W_DENSITY, W_SDF = 0.5, 2.0


def cloud(seed):
    """Particles of the fixture (also rebuilt by tests/test_golden_deform.py)."""
    rng = np.random.default_rng(seed)
    return np.asarray(rng.uniform(0.35, 0.6, (150, 3)), np.float32).astype(np.float64)


def grid_mass(x, mpm_src):
    o = types.SimpleNamespace(n_particles=len(x), inv_dx_0=1.0 / DX, p_mass=P_MASS, x_0=ti.Field((1, len(x)), (3,)),
                              grid_m_s=ti.Field((N_GRID,) * 3))
    o.x_0.a[0] = x
    ti.methods(mpm_src, "MPMObj", ["compute_grid_m_kernel"], o)
    return o


def main():
    ref = reference_root()
    mpm_src = os.path.join(ref, "difftactile", "object_model", "mpm_plastic.py")
    loss_src = os.path.join(ref, "difftactile", "tasks", "deform_loss.py")
    x = cloud(0)
    tgt = grid_mass(x + 0.03, mpm_src)          # target density: the cloud shifted by 0.03
    tgt.compute_grid_m_kernel(0)
    obj = grid_mass(x, mpm_src)
    res = (N_GRID,) * 3
    d = types.SimpleNamespace(dtype=ti.f64, n_grid=N_GRID, dx_0=DX, dim=3, inf=1000, grid_mass=obj.grid_m_s,
                              compute_grid_mass=obj.compute_grid_m_kernel,
                              target_density=ti.Field(res), target_sdf=ti.Field(res), target_sdf_copy=ti.Field(res),
                              nearest_point=ti.Field(res, (3,)), nearest_point_copy=ti.Field(res, (3,)),
                              sdf_loss=ti.scalar(0.0), density_loss=ti.scalar(0.0), loss=ti.scalar(0.0),
                              sdf_weight=ti.scalar(W_SDF), density_weight=ti.scalar(W_DENSITY))
    d.target_density.a[:] = tgt.grid_m_s.a
    ti.methods(loss_src, "Deform_Loss", ["norm", "update_target_sdf", "update_target", "compute_density_loss_kernel",
                                         "compute_sdf_loss_kernel", "sum_up_loss_kernel", "compute_loss_kernel"], d)
    d.update_target()
    d.compute_loss_kernel(0)
    np.savez_compressed(os.path.join(HERE, "deform_ref.npz"), target=d.target_density.a, sdf=d.target_sdf.a,
                        mass=d.grid_mass.a, loss=np.array([d.loss[None], d.density_loss[None], d.sdf_loss[None]]))
    reached = (d.target_sdf.a < 1000).mean()
    print(f"seeds {(d.target_density.a > 1e-4).sum()}, reached {reached:.2f}, loss {d.loss[None]:.6g}")


if __name__ == "__main__":
    main()
