"""Reference-facing interface: the object and method names a DiffTactile task script calls, on top
of the fused CUDA substep, plus a torch.autograd.Function over a segment of substeps.

The reference's objects (MPMObj, FEMDomeSensor, PBDRope, the task's Contact) each own Taichi fields
and launch one kernel per method (tasks/grasp_plastic.py:151-178).  Here one World owns every buffer
and a substep is three fused launches; the shims map each reference method onto them:

  MPMObj.compute_new_F(f), svd(f), p2g(f)        -> dt_p2g (F update, SVD and scatter fused)
  FEMDomeSensor.update(f)                        -> dt_fem_update (all sensors' tets, once per frame)
  MPMObj.check_grid_occupy(f), Contact.check_collision(f), collision(f), MPMObj.grid_op(f)
                                                 -> dt_grid_op (+ dt_rope_update when ropes exist)
  PBDRope.update(f)                              -> dt_rope_update (once per frame)
  MPMObj.g2p(f)                                  -> dt_g2p
  FEMDomeSensor.update2(f)                       -> dt_fem_update2 (all sensors, once per frame)
  Contact.update(f)                              -> dt_substep_fwd
  Contact.update_grad(f)                         -> dt_substep_bwd (g2p.grad ... compute_new_F.grad, with
                                                    clamp_grid and svd_grad inside)
  memory_to_cache(t) / memory_from_cache(t)      -> device checkpoints of frame 0 (HBM, not host RAM)

A fused launch covers all objects, so it runs once per frame until the next reset(): the
reference calls update(f) per sensor, the second call finds the frame done.  Methods whose work
lives inside a fused launch (compute_new_F, svd, check_grid_occupy, check_collision, collision,
clamp_grid, svd_grad) only mark their place in the sequence.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from .world import World


class Simulation:
    """One World with reference-named views: ``mpm_object``, ``sensors`` (FEMDomeSensor-like),
    ``ropes`` (PBDRope-like), and the task-level Contact methods on the Simulation itself."""

    def __init__(self, envs, n_frames: int, dt: float, device="cuda", **world_kw):
        self.world = World(envs, n_frames=n_frames, dt=dt, device=device, **world_kw)
        self.sub_steps = n_frames
        self._done: set = set()
        self._cache: dict = {}
        self._last_cache_op = None  # the reference calls memory_to/from_cache once per object
        self.mpm_object = MPMObj(self)
        self.sensors = [FEMDomeSensor(self, s) for s in range(self.world.n_sensors)]
        self.ropes = [PBDRope(self, r) for r in range(self.world.n_ropes)]

    # ---- fused launches, once per frame between resets ----
    def _once(self, key, f, name):
        if (key, f) in self._done:
            return
        self.world.call(name, int(f))
        self._done.add((key, f))

    # ---- Contact (task) methods, grasp_plastic.py:151-178, 192-202, 259-261, 386-403 ----
    def reset(self):
        """Contact.reset: the grid and the sensors' contact forces of a new step (dt_step_begin)."""
        self.world.step_begin()
        self._done.clear()
        self._last_cache_op = None

    def update(self, f):
        self._last_cache_op = None
        self.world.substep(int(f))
        self._done.update({("p2g", f), ("fem", f), ("grid", f), ("rope", f), ("g2p", f), ("fem2", f)})

    def update_grad(self, f):
        self.world.substep_bwd(int(f))

    def check_collision(self, f):
        """Argmin search; fused into grid_op (dt_grid_op)."""

    def collision(self, f):
        """Contact forces; fused into grid_op (dt_grid_op)."""

    def clamp_grid(self, f):
        """Gradient clamp; applied inside update_grad (world grad_clip)."""

    def compute_obj_pos(self, f) -> torch.Tensor:
        """Centre of mass of each environment's object at frame f ([n_envs, 3])."""
        return self.world.com(int(f))

    def compute_contact_force(self, f, s=0) -> torch.Tensor:
        out = torch.zeros(4, device=self.world.device)
        N.check(self.world.lib.dt_contact_force(self.world.wp, int(s), int(f), out.data_ptr(), self.world.stream),
                "contact force")
        return out[:3]

    def memory_to_cache(self, t):
        """Keep frame 0 as the start of step t (device), then move the last frame to frame 0."""
        if self._last_cache_op == ("to", t):
            return
        self._last_cache_op = ("to", t)
        w = self.world
        self._cache[t] = {k: w.t[k][0].clone() for k in ("p_state", "v_pos", "v_vel", "v_vpos", "r_state")}
        w.copy_frame(self.sub_steps - 1, 0)

    def memory_from_cache(self, t):
        """Restore the start of step t into frame 0, moving frame 0's adjoint to the last frame's
        buffer (copy_grad) so that the backward sweep continues from it."""
        if self._last_cache_op == ("from", t):
            return
        self._last_cache_op = ("from", t)
        w = self.world
        last = (self.sub_steps - 1) & 1
        if last != 0:
            for k in ("p_adj", "v_adj_pos", "v_adj_vel", "v_adj_vpos", "r_adj"):
                w.t[k][last].copy_(w.t[k][0])
        for k, v in self._cache[t].items():
            w.t[k][0].copy_(v)
        self._done.clear()

    def clear_all_grad(self):
        self.world.adj_clear()


class MPMObj:
    """MPM object methods (object_model/mpm_elastic.py:117-344)."""

    def __init__(self, sim: Simulation):
        self.sim = sim

    def compute_new_F(self, f):
        """F_new = (I + dt C) F; fused into p2g."""

    def svd(self, f):
        """SVD of F_new; fused into p2g."""

    def p2g(self, f):
        self.sim._once("p2g", f, "dt_p2g")

    def check_grid_occupy(self, f):
        """Occupancy m > eps; fused into grid_op."""

    def grid_op(self, f):
        self.sim._once("grid", f, "dt_grid_op")
        self.sim._once("rope", f, "dt_rope_update")

    def g2p(self, f):
        self.sim._once("g2p", f, "dt_g2p")

    def svd_grad(self, f):
        """SVD adjoint; part of Contact.update_grad (dt_substep_bwd)."""

    def reset(self):
        self.sim.reset()

    def copy_frame(self, source, target):
        self.sim.world.copy_frame(int(source), int(target))

    def memory_to_cache(self, t):
        self.sim.memory_to_cache(t)

    def memory_from_cache(self, t):
        self.sim.memory_from_cache(t)

    def clear_loss_grad(self):
        self.sim.world.adj_clear()

    def clear_step_grad(self, f):
        self.sim.world.adj_clear()

    # fields read by task code: x_0, v_0, C_0, F_0 of frame f (user particle order)
    def state(self, f):
        return self.sim.world.particles(int(f))

    def init(self, x, v=None):
        self.sim.world.set_particles(0, x=x, v=np.zeros_like(x) if v is None else v)


class FEMDomeSensor:
    """FEM sensor methods (sensor_model/fem_sensor.py:212-521, gripper_fem.py)."""

    def __init__(self, sim: Simulation, s: int):
        self.sim, self.s = sim, s
        self.dtrans = None

    def update(self, f):
        self.sim._once("fem", f, "dt_fem_update")

    def update2(self, f):
        self.sim._once("fem2", f, "dt_fem_update2")

    def reset_contact(self):
        """Contact forces are cleared per frame by the substep itself."""

    def set_pose_control(self, d_pos, d_ori, steps: int | None = None):
        """dtrans_h = T_world eul2mat(d_ori dt (S-1), d_pos dt (S-1)) T_world^-1 (fem_sensor.py:229-245)."""
        from .trajectory import eul2mat_zyx
        w = self.sim.world
        S = (self.sim.sub_steps - 1) if steps is None else steps
        sp = w.sensor_specs[self.s]
        TW = np.eye(4) if sp.trans_world is None else np.asarray(sp.trans_world, np.float64)
        M = eul2mat_zyx(torch.as_tensor(d_ori, dtype=torch.float64) * w.dt * S,
                        torch.as_tensor(d_pos, dtype=torch.float64) * w.dt * S).numpy()
        D = TW @ M @ np.linalg.inv(TW)
        self.dtrans = torch.as_tensor(D[:3].reshape(-1), dtype=torch.float32, device=w.device)
        self.inv_T = 1.0 / (w.dt * S)

    def set_control_vel(self, f=0):
        """Control velocity of the base layer from dtrans_h and the virtual positions of frame f,
        written to every frame (fem_sensor.py:259-266)."""
        w = self.sim.world
        N.check(w.lib.dt_pose_control_vel(w.wp, self.s, self.dtrans.data_ptr(), self.inv_T, int(f),
                                          w.n_frames - int(f), w.stream), "set_control_vel")

    def set_vel(self, f):
        """vel[f] = control_vel[f] (gripper_fem.py:194-196)."""
        w = self.sim.world
        sl = w.vslice(self.s)
        w.t["v_vel"][f, sl] = w.t["v_cv"][f, sl]
        w.t["v_velmid"][f, sl] = w.t["v_cv"][f, sl]

    def pos(self, f):
        return self.sim.world.sensor_frame("v_pos", int(f), self.s)

    def vel(self, f):
        return self.sim.world.sensor_frame("v_vel", int(f), self.s)

    def virtual_pos(self, f):
        return self.sim.world.sensor_frame("v_vpos", int(f), self.s)

    def extract_markers(self, f, model=None, inv_trans=None):
        """(predicted, virtual) marker pixels of frame f (fem_sensor.py:161-187)."""
        from .markers import MarkerModel
        if model is None:
            model = getattr(self, "_markers", None) or MarkerModel(self.sim.world, self.s)
            self._markers = model
        return model.readout(int(f), inv_trans)

    def memory_to_cache(self, t):
        self.sim.memory_to_cache(t)

    def memory_from_cache(self, t):
        self.sim.memory_from_cache(t)


class PBDRope:
    """PBD rope methods (object_model/PBD_rope.py:112-258)."""

    def __init__(self, sim: Simulation, r: int):
        self.sim, self.r = sim, r

    def update(self, f):
        self.sim._once("rope", f, "dt_rope_update")

    def copy_frame(self, source, target):
        self.sim.world.copy_frame(int(source), int(target))

    def state(self, f):
        return self.sim.world.rope_state(int(f), self.r)

    def memory_to_cache(self, t):
        self.sim.memory_to_cache(t)

    def memory_from_cache(self, t):
        self.sim.memory_from_cache(t)


# -------------------------------------------------------------------------------------------------
class SubstepSegment(torch.autograd.Function):
    """Substeps f0 .. f0 + n - 1 of a World as one differentiable torch op.

    Inputs: particle x, v, C, F (user order, [N,3] / [N,3,3]) and the sensors' pos, vel, vpos
    ([V,3], all sensors flattened) of frame f0, and optionally the materials' Lame parameters
    ``lame`` [n_materials, 2] (mu, lambda; mpm_elastic.py:64-71, multi_obj.py:65-74), written into the
    world's material table.  Outputs the same state quantities at frame f0 + n.  The world's control
    velocities are constants here.  Backward seeds the world's adjoint buffers of frame f0 + n with the
    output gradients, runs dt_substep_bwd down to f0 and returns the adjoints of frame f0 and, for
    ``lame``, the material adjoint the substeps accumulated (dt_world.mat_adj).

    The backward reads the frames and grid tape the forward left in the world.  If any of frames
    f0 .. f0 + n was rewritten in between (another segment, a rollout, set_particles, a step_begin) or
    the material table changed, the backward raises instead of returning another rollout's gradient."""

    @staticmethod
    def forward(ctx, world: World, f0: int, n: int, x, v, C, F, pos, vel, vpos, lame=None):
        w = world
        if lame is not None:
            lt = lame.detach().double().cpu()
            if lt.shape != (w.n_materials, 2):
                raise ValueError(f"lame: {tuple(lt.shape)}, expected ({w.n_materials}, 2)")
            for m in range(w.n_materials):
                w.set_material(m, mu=float(lt[m, 0]), lam=float(lt[m, 1]))
        w.set_particles(f0, x=x.detach(), v=v.detach(), C=C.detach(), F=F.detach())
        for name, a in (("v_pos", pos), ("v_vel", vel), ("v_vpos", vpos)):
            w.t[name][f0, :, :3] = a.detach().to(torch.float32)
        if f0 == 0:
            w.step_begin()
        else:
            w.t["v_velmid"][f0] = w.t["v_vel"][f0]
            w.t["v_ext"][f0].zero_()
            w.t["tape_bcount"][f0:f0 + n].zero_()
        for f in range(f0, f0 + n):
            w.substep(f)
        ctx.world, ctx.f0, ctx.n = w, f0, n
        ctx.gen = w.frame_gen[f0:f0 + n + 1].copy()
        ctx.mgen = w.material_gen
        ctx.lame = None if lame is None else (lame.dtype, lame.device)
        out = w.particles(f0 + n)
        return (out["x"], out["v"], out["C"], out["F"], w.t["v_pos"][f0 + n, :, :3].clone(),
                w.t["v_vel"][f0 + n, :, :3].clone(), w.t["v_vpos"][f0 + n, :, :3].clone())

    @staticmethod
    def backward(ctx, gx, gv, gC, gF, gpos, gvel, gvpos):
        w, f0, n = ctx.world, ctx.f0, ctx.n
        fe = f0 + n
        if not np.array_equal(w.frame_gen[f0:fe + 1], ctx.gen) or w.material_gen != ctx.mgen:
            raise RuntimeError(f"frames {f0}..{fe} of the world (or its material table) were rewritten after this "
                               "segment's forward; its backward would differentiate another rollout")
        w.adj_clear()
        z = lambda g, shape: torch.zeros(shape, device=w.device) if g is None else g  # noqa: E731
        Np, V = w.n_particles, w.n_verts
        w.set_particle_adjoint(fe, x=z(gx, (Np, 3)), v=z(gv, (Np, 3)), C=z(gC, (Np, 3, 3)), F=z(gF, (Np, 3, 3)))
        b = fe & 1
        for name, g in (("v_adj_pos", gpos), ("v_adj_vel", gvel), ("v_adj_vpos", gvpos)):
            w.t[name][b, :, :3] = z(g, (V, 3))
        for f in reversed(range(f0, fe)):
            w.substep_bwd(f)
        a = w.particle_adjoint(f0)
        b0 = f0 & 1
        glame = None
        if ctx.lame is not None:
            glame = w.material_adjoint().to(dtype=ctx.lame[0], device=ctx.lame[1])
        return (None, None, None, a["x"], a["v"], a["C"], a["F"], w.t["v_adj_pos"][b0, :, :3].clone(),
                w.t["v_adj_vel"][b0, :, :3].clone(), w.t["v_adj_vpos"][b0, :, :3].clone(), glame)


def simulate(world: World, f0: int, n: int, x, v, C, F, pos, vel, vpos, lame=None):
    """Functional form of SubstepSegment (see there)."""
    return SubstepSegment.apply(world, f0, n, x, v, C, F, pos, vel, vpos, lame)
