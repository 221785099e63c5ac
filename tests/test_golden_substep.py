"""The oracle's substep against golden substeps of the reference's own simulation methods
(tests/golden/make_substep.py runs MPMObj of mpm_elastic.py / mpm_plastic.py, MultiObj of
multi_obj.py, FEMDomeSensor of
fem_sensor.py / gripper_fem.py, PBDRope of PBD_rope.py and Contact.update of grasp_plastic.py and
cable_straightening.py, taken out of the reference source, in float64 on numpy fields).  Same
states, same constants, one substep: particles, the grid at every occupied node, the contact argmin,
the sensors' elastic velocities, contact forces and next frame, and the rope's next frame, contact
impulses, contact indices and travel flags agree to float64 rounding (1e-9 relative, norm-wise);
the rest-shape inverses B (float32 fields in the reference) are equal."""
import os

import numpy as np
import pytest

from oracle import markers as OM
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


def _sensors_agree(r, out, dbg, NS):
    for s in range(NS):
        assert SS.rel_err(dbg["vel_mid"][s], r[f"s{s}_vel_mid"]) < TOL, s
        assert SS.rel_err(dbg["ext"][s], r[f"s{s}_ext"]) < TOL, s
        assert SS.rel_err(out["pos"][s], r[f"s{s}_pos1"]) < TOL, s
        assert SS.rel_err(out["vel"][s], r[f"s{s}_vel1"]) < TOL, s
        assert SS.rel_err(out["vpos"][s], r[f"s{s}_vpos1"]) < TOL, s


def _sensor_state(env, r):
    NS = len(env.sensors)
    f64 = lambda k: [r[f"s{s}_{k}"].astype(np.float64) for s in range(NS)]  # noqa: E731
    for s, sp in enumerate(env.sensors):  # float32 fields in the reference and on the device alike
        assert np.array_equal(sp.rest_inverse().astype(np.float64), r[f"s{s}_B"])
    return {"pos": f64("pos"), "vel": f64("vel"), "vpos": f64("vpos")}, f64("cv"), f64("cv1")


def test_oracle_rope_substep_matches_reference_methods(golden):
    """Contact.update of tasks/cable_straightening.py:166-173 (two gripper pads of gripper_fem.py with
    per-frame control velocities; PBDRope.update of PBD_rope.py:112-180; the rope collision
    :288-319 with its contact-force variant :212-224)."""
    env = scenes()["rope_pads"]
    r = _case(golden, "rope_pads")
    st, cv, cv1 = _sensor_state(env, r)
    st.update(x=np.zeros((0, 3)), v=np.zeros((0, 3)), C=np.zeros((0, 3, 3)), F=np.zeros((0, 3, 3)),
              rpos=[r["rpos"].astype(np.float64)], rvel=[r["rvel"].astype(np.float64)],
              rtrav=[r["rtrav"].astype(np.float64)])
    out, dbg = O.Oracle(env, DT, np.float64, grad_clip=0.0).substep(st, cv=cv, cv1=cv1)
    assert np.array_equal(dbg["rope_cidx"][0][:, :2], r["rcidx"])
    assert (r["rext"] != 0).any() and np.array_equal(out["rtrav"][0], r["rtrav1"])
    assert SS.rel_err(dbg["rope_ext"][0], r["rext"]) < TOL
    assert SS.rel_err(out["rpos"][0], r["rpos1"]) < TOL
    assert SS.rel_err(out["rvel"][0], r["rvel1"]) < TOL
    _sensors_agree(r, out, dbg, 2)


@pytest.mark.parametrize("name", ["corotated_cube", "plastic_pads", "multi_material_cube"])
def test_oracle_substep_matches_reference_methods(golden, name):
    env = scenes()[name]
    r = _case(golden, name)
    m = env.materials[0]
    consts = [DT, env.dx, env.volume, env.p_mass, env.eps, env.bound, *m.mu_lam, m.yield_stress, env.kn, env.kd,
              env.kt, env.mu_t]
    assert np.allclose(r["consts"], consts, rtol=1e-15, atol=0)  # the scene builders still build these scenes
    NS = len(env.sensors)
    st, cv, _ = _sensor_state(env, r)
    st.update({k: r[k].astype(np.float64) for k in ("x", "v", "C", "F")})
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
    _sensors_agree(r, out, dbg, NS)
    # the grasp task's readouts: summed surface force of each pad, centre of mass of the next frame
    for s, sp in enumerate(env.sensors):
        assert SS.rel_err(OM.contact_force_sum(dbg["ext"][s], sp.tris), r["contact_force"][s]) < TOL, s
    assert SS.rel_err(out["x"].mean(0), r["com1"]) < TOL


def test_oracle_rope_chain_matches_reference_methods(golden):
    """Five substeps of the cable task's Contact.update with ramping control velocities (frame f:
    cv + f (cv1 - cv)), each oracle substep fed the previous one's output: rope and pads at the end."""
    from tests.golden.make_substep import CHAIN
    env = scenes()["rope_pads_chain"]
    r = _case(golden, "rope_pads_chain")
    st, cv, cv1 = _sensor_state(env, r)
    st.update(x=np.zeros((0, 3)), v=np.zeros((0, 3)), C=np.zeros((0, 3, 3)), F=np.zeros((0, 3, 3)),
              rpos=[r["rpos"].astype(np.float64)], rvel=[r["rvel"].astype(np.float64)],
              rtrav=[r["rtrav"].astype(np.float64)])
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    ramp = lambda f: [a + f * (b - a) for a, b in zip(cv, cv1)]  # noqa: E731
    for f in range(CHAIN):
        st, _ = o.substep(st, cv=ramp(f), cv1=ramp(f + 1))
    assert np.array_equal(st["rtrav"][0], r["rtravN"]) and r["rtravN"].sum() > r["rtrav"].sum()
    assert SS.rel_err(st["rpos"][0], r["rposN"]) < TOL and SS.rel_err(st["rvel"][0], r["rvelN"]) < TOL
    for s in range(len(env.sensors)):
        for a, b in (("posN", "pos"), ("velN", "vel"), ("vposN", "vpos")):
            assert SS.rel_err(st[b][s], r[f"s{s}_{a}"]) < TOL, (s, a)


@pytest.mark.parametrize("name", ["corotated_cube", "plastic_pads", "multi_material_cube"])
def test_float32_oracle_is_within_the_one_substep_tolerance(golden, name):
    """In float32 (the CUDA path's arithmetic) the oracle's substep stays within 1e-5 relative of the
    reference's float64 step for x, v, C, F and the sensors' positions (worst 4e-6: v and C of the
    three-material cube, whose stiffest layer has E = 4e5)."""
    env = scenes()[name]
    r = _case(golden, name)
    st, cv, _ = _sensor_state(env, r)
    st.update({k: r[k].astype(np.float64) for k in ("x", "v", "C", "F")})
    NS = len(env.sensors)
    out, _ = O.Oracle(env, DT, np.float32, grad_clip=0.0).substep(st, cv=cv if NS else None, cv1=cv if NS else None)
    for a, b in (("x1", "x"), ("v1", "v"), ("C1", "C"), ("F1", "F")):
        assert SS.rel_err(out[b].astype(np.float64), r[a]) < 1e-5, a
    for s in range(NS):
        assert SS.rel_err(out["pos"][s].astype(np.float64), r[f"s{s}_pos1"]) < 1e-5, s


def test_oracle_chain_matches_reference_methods(golden):
    """Five substeps of the grasp task's Contact.update, each oracle substep fed the previous one's
    output: the particles and both pads at the last frame."""
    from tests.golden.make_substep import CHAIN
    env = scenes()["plastic_pads_chain"]
    r = _case(golden, "plastic_pads_chain")
    st, cv, _ = _sensor_state(env, r)
    st.update({k: r[k].astype(np.float64) for k in ("x", "v", "C", "F")})
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    for _ in range(CHAIN):
        st, _ = o.substep(st, cv=cv, cv1=cv)
    for a, b in (("xN", "x"), ("vN", "v"), ("CN", "C"), ("FN", "F")):
        assert SS.rel_err(st[b], r[a]) < TOL, a
    for s in range(len(env.sensors)):
        for a, b in (("posN", "pos"), ("velN", "vel"), ("vposN", "vpos")):
            assert SS.rel_err(st[b][s], r[f"s{s}_{a}"]) < TOL, (s, a)


def test_fixture_exercises_both_return_map_branches(golden):
    """Half of the plastic box's particles start beyond the von Mises yield surface, half inside."""
    r = _case(golden, "plastic_pads")
    env = scenes()["plastic_pads"]
    m = env.materials[0]
    Fn = (np.eye(3)[None] + DT * r["C"].astype(np.float64)) @ r["F"].astype(np.float64)
    eps = np.log(np.maximum(np.linalg.svd(Fn, compute_uv=False), 0.05))
    dg = np.sqrt(((eps - eps.mean(1, keepdims=True)) ** 2).sum(1) + 1e-8) - m.yield_stress / (2 * m.mu_lam[0])
    assert 0.3 < (dg > 0).mean() < 0.7
