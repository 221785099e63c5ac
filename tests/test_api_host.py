"""The reference-named interface's bookkeeping on the host (api.Simulation over a stand-in world, no
GPU): the per-object methods of Contact.update (tasks/grasp_plastic.py:151-164) issue each fused launch
once per frame until the next reset, memory_to_cache / memory_from_cache (mpm_elastic.py:300-320,
fem_sensor.py:501-521) act once per step however many objects call them, and a checkpointed backward
sweep written with those calls gives torch autograd's initial-state gradient for odd and even
sub_steps (memory_from_cache moves frame 0's adjoint to the last frame's buffer)."""
import pytest
import torch

from difftactile_gb300.api import FEMDomeSensor, MPMObj, PBDRope, Simulation
from tests.test_checkpoint_schedule import FakeWorld, System


class CallWorld(FakeWorld):
    """FakeWorld that also logs the fused launches the shims issue, and runs one adjoint substep."""

    n_sensors, n_ropes = 2, 1

    def __init__(self, n_frames, sys):
        super().__init__(n_frames, sys)
        self.log = []

    def call(self, name, *args):
        self.log.append((name,) + tuple(args))
        if name == "dt_g2p":          # the pieces of a frame together advance it; g2p writes frame f + 1
            FakeWorld.substep(self, args[0])

    def substep(self, f):
        self.log.append(("dt_substep_fwd", f))
        super().substep(f)

    def substep_bwd(self, f):
        self.substeps_bwd(f + 1, f)


def simulation(sub_steps, sys=None):
    sim = Simulation.__new__(Simulation)
    sim.world = CallWorld(sub_steps, sys or System())
    sim.sub_steps = sub_steps
    sim._done, sim._cache, sim._last_cache_op = set(), {}, None
    sim.mpm_object = MPMObj(sim)
    sim.sensors = [FEMDomeSensor(sim, s) for s in range(2)]
    sim.ropes = [PBDRope(sim, 0)]
    return sim


def grasp_sequence(sim, f):
    """Contact.update (grasp_plastic.py:151-164) with the cable task's rope update, call for call."""
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
    for r in sim.ropes:
        r.update(f)
    m.g2p(f)
    for s in sim.sensors:
        s.update2(f)


FUSED = ["dt_p2g", "dt_fem_update", "dt_grid_op", "dt_rope_update", "dt_g2p", "dt_fem_update2"]


def test_each_fused_launch_runs_once_per_frame():
    sim = simulation(4)
    sim.reset()
    for f in range(3):
        grasp_sequence(sim, f)
        grasp_sequence(sim, f)  # repeated: nothing more
    assert sim.world.log == [(n, f) for f in range(3) for n in FUSED]
    sim.world.log.clear()
    sim.reset()
    grasp_sequence(sim, 0)
    assert sim.world.log == [(n, 0) for n in FUSED]
    sim.world.log.clear()
    sim.reset()
    sim.update(0)           # the single fused call marks every piece of the frame done
    grasp_sequence(sim, 0)
    assert sim.world.log == [("dt_substep_fwd", 0)]


def test_cache_calls_act_once_per_step():
    sim = simulation(4)
    w = sim.world
    for f in range(4):
        w.set_z(f, torch.full((w.z(0).numel(),), float(f)))
    sim.mpm_object.memory_to_cache(0)
    for s in sim.sensors:
        s.memory_to_cache(0)    # every object calls it in the reference: one move only
    sim.ropes[0].memory_to_cache(0)
    assert float(w.z(0)[0]) == 3.0 and float(sim._cache[0]["p_state"].flatten()[0]) == 0.0
    w.set_z(0, torch.full((w.z(0).numel(),), 7.0))
    sim.mpm_object.memory_from_cache(0)
    for s in sim.sensors:
        s.memory_from_cache(0)
    assert float(w.z(0).abs().max()) == 0.0  # the cached start of step 0, once


@pytest.mark.parametrize("sub_steps", [4, 5])
def test_checkpointed_backward_through_the_reference_calls(sub_steps):
    """T steps of sub_steps - 1 substeps each; forward caches each step's start, backward restores it,
    recomputes the step and runs update_grad down to frame 0."""
    T = 3
    sys = System(seed=sub_steps)
    sim = simulation(sub_steps, sys)
    w = sim.world
    w.set_z(0, sys.z0.float())
    for t in range(T):
        sim.reset()
        for f in range(sub_steps - 1):
            grasp_sequence(sim, f)
        sim.memory_to_cache(t)   # start of step t kept; the last frame becomes frame 0
    L = float(sys.loss(w.z(0).double()))
    sim.clear_all_grad()
    w.set_adj(0, sys.q + w.z(0).double())       # loss adjoint of the final state, now frame 0
    for t in reversed(range(T)):
        sim.memory_from_cache(t)
        sim.reset()
        for f in range(sub_steps - 1):
            sim.update(f)
        for f in reversed(range(sub_steps - 1)):
            sim.update_grad(f)
    z = sys.z0.clone().requires_grad_(True)
    zz = z
    for _ in range(T * (sub_steps - 1)):
        zz = sys.step(zz, torch.zeros(3, dtype=torch.float64))
    Lr = sys.loss(zz)
    (gz,) = torch.autograd.grad(Lr, z)
    assert abs(L - float(Lr.detach())) <= 1e-4 * abs(float(Lr.detach()))
    g = w.adj(0).double()
    assert float((g - gz).norm() / gz.norm()) < 1e-4
