"""The reference-named interface (api.Simulation: MPMObj / FEMDomeSensor / Contact methods of
tasks/grasp_plastic.py:151-178) and the torch.autograd.Function over substeps, on the GPU."""
import numpy as np
import pytest
import torch

from difftactile_gb300.api import Simulation, simulate
from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4


def grasp_sequence(sim, f):
    """Contact.update of grasp_plastic.py:151-164, call for call (two sensors)."""
    m = sim.mpm_object
    m.compute_new_F(f)
    m.svd(f)
    m.p2g(f)
    for s in sim.sensors:
        s.update(f)
    m.check_grid_occupy(f)
    sim.check_collision(f)
    sim.collision(f)
    m.grid_op(f)
    m.g2p(f)
    for s in sim.sensors:
        s.update2(f)


def test_reference_call_sequence_matches_fused_substeps(cuda_lib):
    env = SS.pad_over_box(two_pads=True)
    cv = [SS.control_velocity(sp, seed=3 + i) for i, sp in enumerate(env.sensors)]
    S = 4
    sim = Simulation([env], n_frames=S, dt=DT)
    ref = World([env], n_frames=S, dt=DT)
    for s, c in enumerate(cv):
        sim.world.set_control_velocity(s, c)
        ref.set_control_velocity(s, c)
    sim.reset()
    ref.step_begin()
    for f in range(S - 1):
        grasp_sequence(sim, f)
        grasp_sequence(sim, f)  # a repeated call sequence is a no-op until the next reset
        ref.substep(f)
    torch.cuda.synchronize()
    a, b = sim.world.particles(S - 1), ref.particles(S - 1)
    for k in ("x", "v", "C", "F"):
        assert SS.rel_err(a[k].cpu().numpy(), b[k].cpu().numpy()) < 1e-6, k
    for s in range(2):
        assert SS.rel_err(sim.sensors[s].pos(S - 1).cpu().numpy(), ref.sensor_frame("v_pos", S - 1, s).cpu().numpy()) < 1e-6
    # checkpoint round trip: frame 0 restored exactly, the last frame moved to frame 0 before
    x_last = sim.world.particles(S - 1)["x"].clone()
    x0 = sim.world.particles(0)["x"].clone()
    sim.mpm_object.memory_to_cache(0)
    for s in sim.sensors:
        s.memory_to_cache(0)  # once per object in the reference: no second move
    assert torch.equal(sim.world.particles(0)["x"], x_last)
    sim.memory_from_cache(0)
    assert torch.equal(sim.world.particles(0)["x"], x0)


def test_substep_segment_gradients_match_oracle_adjoint(cuda_lib):
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = World([env], n_frames=2, dt=DT, grad_clip=0.0)
    w.set_control_velocity(0, cv[0])
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    st0 = o.initial_state()
    dev = w.device
    t = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.float32, device=dev).requires_grad_(True)  # noqa: E731
    ins = [t(st0["x"]), t(st0["v"]), t(st0["C"]), t(st0["F"]), t(st0["pos"][0]), t(st0["vel"][0]), t(st0["vpos"][0])]
    outs = simulate(w, 0, 1, *ins)
    rng = np.random.default_rng(1)
    Ws = [rng.standard_normal(tuple(o_.shape)) for o_ in outs]
    loss = sum((torch.as_tensor(Wk, dtype=torch.float32, device=dev) * o_).sum() for Wk, o_ in zip(Ws, outs))
    grads = torch.autograd.grad(loss, ins)
    adj1 = {"x": Ws[0], "v": Ws[1], "C": Ws[2], "F": Ws[3], "pos": [Ws[4]], "vel": [Ws[5]], "vpos": [Ws[6]]}
    ref = o.substep_bwd(st0, adj1, cv=[c.astype(np.float64) for c in cv], cv1=[c.astype(np.float64) for c in cv])
    names = ["x", "v", "C", "F", "pos", "vel", "vpos"]
    for k, g in zip(names, grads):
        r = ref[k][0] if isinstance(ref[k], list) else ref[k]
        assert SS.rel_err(g.cpu().numpy(), r) < 1e-3, k


def _sphere_obj(path, n_lat=16, n_lon=32):
    """A closed latitude-longitude sphere of radius 1 as an OBJ file."""
    V = [[0.0, 1.0, 0.0]]
    for i in range(1, n_lat):
        th = np.pi * i / n_lat
        for j in range(n_lon):
            ph = 2 * np.pi * j / n_lon
            V.append([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)])
    V.append([0.0, -1.0, 0.0])
    F, last = [], len(V) - 1
    for j in range(n_lon):
        F.append([0, 1 + (j + 1) % n_lon, 1 + j])
    for i in range(n_lat - 2):
        for j in range(n_lon):
            a, b = 1 + i * n_lon + j, 1 + i * n_lon + (j + 1) % n_lon
            F += [[a, b, b + n_lon], [a, b + n_lon, a + n_lon]]
    for j in range(n_lon):
        F.append([last, 1 + (n_lat - 2) * n_lon + j, 1 + (n_lat - 2) * n_lon + (j + 1) % n_lon])
    with open(path, "w") as fh:
        fh.writelines(f"v {x} {y} {z}\n" for x, y, z in V)
        fh.writelines(f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in F)


def test_reference_shaped_construction_runs_the_task_loop(cuda_lib, tmp_path):
    """Objects made as a reference task makes them (tasks/grasp_plastic.py:31-48, 118-136):
    MPMObj(dt, sub_steps, obj_name, space_scale, obj_scale, density, rho).init(position, orientation,
    velocity), FEMDomeSensor(dt, sub_steps).init(rot_x, rot_y, rot_z, t_dx, t_dy, t_dz), set_pose_control /
    set_control_vel, then the reference's Contact.update call sequence for every substep and
    Contact.update_grad back down: the same frames as a World of the equivalent scene stepped with the
    fused substep, and finite adjoints."""
    from difftactile_gb300.api import FEMDomeSensor, MPMObj
    from difftactile_gb300.scene import EnvSpec
    obj = str(tmp_path / "ball.obj")
    _sphere_obj(obj)
    dt, S = 5e-5, 5
    mo = MPMObj(dt=dt, sub_steps=S, obj_name=obj, space_scale=10.0, obj_scale=4.0, density=1.5, rho=4.0, plastic=True)
    assert mo.n_particles > 10_000 and abs(mo.dx_0 - 10.0 / 64) < 1e-12 and abs(mo.p_vol - (mo.dx_0 * 4.0) ** 3) < 1e-12
    mo.init([5.5, 2.3, 5.8], [-90.0, 0.0, 0.0], [0.0, 0.0, 0.0])
    top = float(mo.x_init[:, 1].max())
    s = FEMDomeSensor(dt=dt, sub_steps=S)
    s.init(180.0, 0.0, 0.0, 5.5, top + 1.5 + 0.05, 5.8)  # apex down, just above the ball
    sim = Simulation.from_objects(mo, [s])
    w = sim.world
    assert w.n_particles == mo.n_particles and w.n_sensors == 1
    assert np.allclose(mo.state(0)["x"].cpu().numpy(), mo.x_init)
    s.set_pose_control([0.0, 8.0, 0.0], [0.0, 0.0, 0.0])  # +y: the dome's out-direction, into the ball
    s.set_control_vel(0)
    # the same scene as specs, stepped with the fused substep
    env = EnvSpec(x=mo.x_init, v=mo.v_init, materials=[mo.material()], n_grid=(64,) * 3, dx=mo.dx_0, p_vol=mo.p_vol,
                  rho=mo.rho, sensors=[s.spec], kn=34.53, kd=269.44, kt=154.78, mu_t=53.85)
    ref = World([env], n_frames=S, dt=dt)
    ref.t["v_cv"].copy_(w.t["v_cv"])
    sim.reset()
    ref.step_begin()
    for f in range(S - 1):
        grasp_sequence(sim, f)
        ref.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    assert float(w.t["v_ext"][: S - 1, :, :3].abs().sum()) > 0  # the dome touched the ball
    # a second fused run gives the atomic-ordering spread (C of a ball nearly at rest is mostly that noise)
    ref2 = World([env], n_frames=S, dt=dt)
    ref2.t["v_cv"].copy_(w.t["v_cv"])
    ref2.step_begin()
    for f in range(S - 1):
        ref2.substep(f)
    torch.cuda.synchronize()
    a, b, c = w.particles(S - 1), ref.particles(S - 1), ref2.particles(S - 1)
    for k in ("x", "v", "C", "F"):
        spread = SS.rel_err(c[k].cpu().numpy(), b[k].cpu().numpy())
        assert SS.rel_err(a[k].cpu().numpy(), b[k].cpu().numpy()) <= max(10 * spread, 1e-6), (k, spread)
    assert SS.rel_err(s.pos(S - 1).cpu().numpy(), ref.sensor_frame("v_pos", S - 1, 0).cpu().numpy()) < 1e-6
    # Contact.update_grad down the frames from a centre-of-mass loss
    sim.clear_all_grad()
    gb = torch.zeros((1, 4), device=w.device)
    gb[0, 1] = 1.0
    assert w.lib.dt_com_bwd(w.wp, S - 1, gb.data_ptr(), w.stream) == 0
    for f in reversed(range(S - 1)):
        sim.update_grad(f)
    torch.cuda.synchronize()
    g = w.particle_adjoint(0)
    assert all(torch.isfinite(g[k]).all() for k in g) and float(g["v"].abs().sum()) > 0
