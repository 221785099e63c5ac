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
