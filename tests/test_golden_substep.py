"""The oracle's substep against golden substeps of the reference's own simulation methods
(tests/golden/make_substep.py runs MPMObj of mpm_elastic.py / mpm_plastic.py, FEMDomeSensor of
fem_sensor.py and Contact.update of grasp_plastic.py, taken out of the reference source, in float64
on numpy fields).  Same states, same constants, one substep: particles, the grid at every occupied
node, the contact argmin, the sensors' elastic velocities, contact forces and next frame agree to
float64 rounding (1e-9 relative, norm-wise), and the rest-shape inverses B to 1e-12."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import small_scenes as SS
from tests.golden.make_substep import DT, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "substep_ref.npz")
TOL = 1e-9


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _case(g, name):
    return {k.split("/", 1)[1]: g[k] for k in g.files if k.startswith(name + "/")}


@pytest.mark.parametrize("name", ["corotated_cube", "plastic_pads"])
def test_oracle_substep_matches_reference_methods(golden, name):
    env = scenes()[name]
    r = _case(golden, name)
    m = env.materials[0]
    consts = [DT, env.dx, env.volume, env.p_mass, env.eps, env.bound, *m.mu_lam, m.yield_stress, env.kn, env.kd,
              env.kt, env.mu_t]
    assert np.allclose(r["consts"], consts, rtol=1e-15, atol=0)  # the scene builders still build these scenes
    NS = len(env.sensors)
    st = {k: r[k].astype(np.float64) for k in ("x", "v", "C", "F")}
    st["pos"] = [r[f"s{s}_pos"].astype(np.float64) for s in range(NS)]
    st["vel"] = [r[f"s{s}_vel"].astype(np.float64) for s in range(NS)]
    st["vpos"] = [r[f"s{s}_vpos"].astype(np.float64) for s in range(NS)]
    cv = [r[f"s{s}_cv"].astype(np.float64) for s in range(NS)]
    for s, sp in enumerate(env.sensors):
        assert SS.rel_err(sp.rest_inverse().astype(np.float64), r[f"s{s}_B"]) < 1e-12
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    out, dbg = o.substep(st, cv=cv if NS else None, cv1=cv if NS else None)
    for a, b in (("x1", "x"), ("v1", "v"), ("C1", "C"), ("F1", "F")):
        assert SS.rel_err(out[b], r[a]) < TOL, a
    i, j, k = r["occ"].T
    assert np.array_equal(np.argwhere(dbg["grid_m"] > env.eps), r["occ"])  # the same occupied nodes
    for key in ("grid_m", "grid_v_in", "grid_v_out", "grid_f"):
        assert SS.rel_err(dbg[key][i, j, k], r[key]) < TOL, key
    if not NS:
        return
    assert np.array_equal(dbg["cidx"][i, j, k, :NS], r["cidx"])
    assert float(np.abs(r["grid_f"]).max()) > 0 and all((r[f"s{s}_ext"] != 0).any() for s in range(NS))
    for s in range(NS):
        assert SS.rel_err(dbg["vel_mid"][s], r[f"s{s}_vel_mid"]) < TOL, s
        assert SS.rel_err(dbg["ext"][s], r[f"s{s}_ext"]) < TOL, s
        assert SS.rel_err(out["pos"][s], r[f"s{s}_pos1"]) < TOL, s
        assert SS.rel_err(out["vel"][s], r[f"s{s}_vel1"]) < TOL, s
        assert SS.rel_err(out["vpos"][s], r[f"s{s}_vpos1"]) < TOL, s


def test_fixture_exercises_both_return_map_branches(golden):
    """Half of the plastic box's particles start beyond the von Mises yield surface, half inside."""
    r = _case(golden, "plastic_pads")
    env = scenes()["plastic_pads"]
    m = env.materials[0]
    Fn = (np.eye(3)[None] + DT * r["C"].astype(np.float64)) @ r["F"].astype(np.float64)
    eps = np.log(np.maximum(np.linalg.svd(Fn, compute_uv=False), 0.05))
    dg = np.sqrt(((eps - eps.mean(1, keepdims=True)) ** 2).sum(1) + 1e-8) - m.yield_stress / (2 * m.mu_lam[0])
    assert 0.3 < (dg > 0).mean() < 0.7
