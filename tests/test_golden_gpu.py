"""The CUDA path against the golden substeps of the reference's own simulation methods, with no oracle
in between.

tests/golden/make_substep.py ran the reference's MPMObj / MultiObj / FEMDomeSensor / PBDRope methods
and the grasp and cable tasks' Contact.update (taken out of the reference source, in float64 on numpy
fields) on seeded float32 states; this file loads the same float32 states into a World, runs the
substeps through the C ABI and compares with the fixture's outputs.

Bounds (norm-wise relative, float32 arithmetic against the float64 reference):
  one substep   x, v, F, the sensors' next positions: 1e-5; C and the sensors' velocities, elastic
                velocities and contact forces: 1e-4 (sums of atomically accumulated contributions
                whose order the atomics choose); the grid at every occupied node (mass, momentum,
                velocity): 1e-5; the occupied set and the contact argmin of every occupied node and
                rope particle: exact;
  five substeps (chains): 1e-4 on every state, except the rope's velocity (2e-4): PBD velocities are
                position differences over dt = 1e-4, and float32 rounding of the positions alone puts
                the float32 oracle 1.2e-4 from this fixture after five substeps.
Each test prints its measured errors (pytest -s shows them).
"""
import numpy as np
import pytest
import torch

from difftactile_gb300.world import World
from tests import small_scenes as SS
from tests.golden.make_substep import CHAIN, DT, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "substep_ref.npz"))


def _case(g, name):
    return {k.split("/", 1)[1]: g[k] for k in g.files if k.startswith(name + "/")}


def _load(env, r, n_frames, ramp=False):
    """World holding the fixture's float32 state in frame 0 and its control velocities per frame."""
    w = World([env], n_frames=n_frames, dt=DT, grad_clip=0.0)
    if env.n_particles:
        w.set_particles(0, x=r["x"], v=r["v"], C=r["C"], F=r["F"])
    for s in range(len(env.sensors)):
        sl = w.vslice(s)
        for name, key in (("v_pos", "pos"), ("v_vel", "vel"), ("v_vpos", "vpos")):
            w.t[name][0, sl, :3] = torch.as_tensor(r[f"s{s}_{key}"], device=w.device)
        cv, cv1 = r[f"s{s}_cv"].astype(np.float64), r[f"s{s}_cv1"].astype(np.float64)
        if ramp:  # frame f: cv + f (cv1 - cv)
            frames = np.stack([cv + f * (cv1 - cv) for f in range(n_frames)])
        elif env.sensors[s].carry:  # the gripper form reads frames f and f + 1
            frames = np.stack([cv, cv1] + [cv1] * (n_frames - 2))
        else:
            frames = np.broadcast_to(cv, (n_frames,) + cv.shape)
        w.set_control_velocity(s, frames.astype(np.float32))
    for rr in range(len(env.ropes)):
        w.set_rope_state(0, rr, pos=r["rpos"], vel=r["rvel"], trav=r["rtrav"])
    w.step_begin()
    return w


def _check(errs, bounds):
    print({k: f"{v:.2e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if not v <= bounds[k]}
    assert not bad, f"beyond bounds: {bad} (all: {errs})"


ONE = {"x": 1e-5, "v": 1e-5, "F": 1e-5, "C": 1e-4, "pos": 1e-5, "vel": 1e-4, "vpos": 1e-5, "vel_mid": 1e-4,
       "ext": 1e-4, "grid_m": 1e-5, "grid_v_in": 1e-5, "grid_v_out": 1e-5, "contact_force": 1e-4, "com": 1e-5,
       "rpos": 1e-5, "rvel": 1e-4, "rext": 1e-4}


@pytest.mark.parametrize("name", ["corotated_cube", "plastic_pads", "multi_material_cube"])
def test_cuda_substep_matches_reference_fixture(cuda_lib, golden, name):
    env = scenes()[name]
    r = _case(golden, name)
    w = _load(env, r, 2)
    w.substep(0)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    P = {k: v.double().cpu().numpy() for k, v in w.particles(1).items()}
    errs = {k: SS.rel_err(P[k], r[k + "1"]) for k in ("x", "v", "C", "F")}
    # the grid at every occupied node: the same occupied set, mass, momentum and velocity
    g = w.dense_grid(0)
    m = g["m"].double().cpu().numpy()
    assert np.array_equal(np.argwhere(m > env.eps), r["occ"])
    i, j, k = r["occ"].T
    errs["grid_m"] = SS.rel_err(m[i, j, k], r["grid_m"])
    errs["grid_v_in"] = SS.rel_err(g["mv"].double().cpu().numpy()[i, j, k], r["grid_v_in"])
    errs["grid_v_out"] = SS.rel_err(g["v_out"].double().cpu().numpy()[i, j, k], r["grid_v_out"])
    NS = len(env.sensors)
    if NS:
        # contact argmin of every occupied node, per sensor slot: exact
        assert np.array_equal(g["cidx"].cpu().numpy()[i, j, k, :NS], r["cidx"])
        for key, name_ in (("pos", "v_pos"), ("vel", "v_vel"), ("vpos", "v_vpos")):
            errs[key] = max(SS.rel_err(w.sensor_frame(name_, 1, s).double().cpu().numpy(), r[f"s{s}_{key}1"])
                            for s in range(NS))
        errs["vel_mid"] = max(SS.rel_err(w.sensor_frame("v_velmid", 0, s).double().cpu().numpy(), r[f"s{s}_vel_mid"])
                              for s in range(NS))
        errs["ext"] = max(SS.rel_err(w.sensor_frame("v_ext", 0, s).double().cpu().numpy(), r[f"s{s}_ext"])
                          for s in range(NS))
        # the grasp task's readouts: summed surface force per pad, centre of mass of the next frame
        cf = []
        for s in range(NS):
            out = torch.zeros(4, device=w.device)
            w.call("dt_contact_force", s, 0, out.data_ptr())
            cf.append(out[:3].double().cpu().numpy())
        errs["contact_force"] = SS.rel_err(np.stack(cf), r["contact_force"])
        errs["com"] = SS.rel_err(w.com(1)[0].double().cpu().numpy(), r["com1"])
    _check(errs, ONE)


def test_cuda_rope_substep_matches_reference_fixture(cuda_lib, golden):
    """The cable task's Contact.update: a rope under two gripper pads (control-velocity carry)."""
    env = scenes()["rope_pads"]
    r = _case(golden, "rope_pads")
    w = _load(env, r, 2)
    w.substep(0)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    rs = {k: v.double().cpu().numpy() for k, v in w.rope_state(1, 0).items()}
    assert np.array_equal(w.t["r_cidx"][0, :, :2].cpu().numpy(), r["rcidx"])
    assert np.array_equal(rs["trav"], r["rtrav1"])
    errs = {"rpos": SS.rel_err(rs["pos"], r["rpos1"]), "rvel": SS.rel_err(rs["vel"], r["rvel1"]),
            "rext": SS.rel_err(w.t["r_ext"][0, :, :3].double().cpu().numpy(), r["rext"])}
    for key, name_ in (("pos", "v_pos"), ("vel", "v_vel"), ("vpos", "v_vpos")):
        errs[key] = max(SS.rel_err(w.sensor_frame(name_, 1, s).double().cpu().numpy(), r[f"s{s}_{key}1"])
                        for s in range(2))
    errs["vel_mid"] = max(SS.rel_err(w.sensor_frame("v_velmid", 0, s).double().cpu().numpy(), r[f"s{s}_vel_mid"])
                          for s in range(2))
    errs["ext"] = max(SS.rel_err(w.sensor_frame("v_ext", 0, s).double().cpu().numpy(), r[f"s{s}_ext"])
                      for s in range(2))
    _check(errs, ONE)


CHAINED = dict({k: 1e-4 for k in ("x", "v", "C", "F", "pos", "vel", "vpos", "rpos")}, rvel=2e-4)


def test_cuda_chain_matches_reference_fixture(cuda_lib, golden):
    """Five substeps of the grasp task's Contact.update, frame to frame on the device."""
    env = scenes()["plastic_pads_chain"]
    r = _case(golden, "plastic_pads_chain")
    w = _load(env, r, CHAIN + 1)
    for f in range(CHAIN):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    P = {k: v.double().cpu().numpy() for k, v in w.particles(CHAIN).items()}
    errs = {k: SS.rel_err(P[k], r[k + "N"]) for k in ("x", "v", "C", "F")}
    for key, name_ in (("pos", "v_pos"), ("vel", "v_vel"), ("vpos", "v_vpos")):
        errs[key] = max(SS.rel_err(w.sensor_frame(name_, CHAIN, s).double().cpu().numpy(), r[f"s{s}_{key}N"])
                        for s in range(2))
    _check(errs, CHAINED)


def test_cuda_rope_chain_matches_reference_fixture(cuda_lib, golden):
    """Five substeps of the cable task's Contact.update with ramping control velocities."""
    env = scenes()["rope_pads_chain"]
    r = _case(golden, "rope_pads_chain")
    w = _load(env, r, CHAIN + 1, ramp=True)
    for f in range(CHAIN):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    rs = {k: v.double().cpu().numpy() for k, v in w.rope_state(CHAIN, 0).items()}
    assert np.array_equal(rs["trav"], r["rtravN"])
    errs = {"rpos": SS.rel_err(rs["pos"], r["rposN"]), "rvel": SS.rel_err(rs["vel"], r["rvelN"])}
    for key, name_ in (("pos", "v_pos"), ("vel", "v_vel"), ("vpos", "v_vpos")):
        errs[key] = max(SS.rel_err(w.sensor_frame(name_, CHAIN, s).double().cpu().numpy(), r[f"s{s}_{key}N"])
                        for s in range(2))
    _check(errs, CHAINED)
