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

    @classmethod
    def from_objects(cls, mpm_object, sensors=(), ropes=(), *, kn=34.53, kd=269.44, kt=154.78, friction=53.85,
                     device="cuda", **world_kw):
        """The device world of objects made the reference's way (MPMObj(...).init(...),
        FEMDomeSensor(...).init(...), PBDRope(...).init(...)), as a task's Contact holds them
        (tasks/grasp_plastic.py:31-150): one environment, the object's 64^3 grid, the sensors in the given
        order, the contact parameters of the grasp task (kn, kd, kt, friction coefficient; :61-64).  The
        objects become views of the returned simulation, so their reference methods run on the device.
        The world holds ``sub_steps`` frames, as the reference's fields do."""
        from .scene import EnvSpec
        mo = mpm_object
        if mo.x_init is None:
            raise RuntimeError("call mpm_object.init(position, orientation, velocity) first")
        for sp in sensors:
            if sp.spec is None:
                raise RuntimeError("place every sensor first (init)")
        env = EnvSpec(x=mo.x_init, v=mo.v_init, materials=[mo.material()], n_grid=(mo.n_grid,) * 3, dx=mo.dx_0,
                      p_vol=mo.p_vol, rho=mo.rho, gravity=mo.gravity, bound=mo.bound, eps=mo.eps,
                      sensors=[sp.spec for sp in sensors], ropes=[r.spec for r in ropes], kn=kn, kd=kd, kt=kt,
                      mu_t=friction)
        sim = cls([env], n_frames=mo.sub_steps, dt=mo.dt, device=device, **world_kw)
        mo.sim = sim
        sim.mpm_object = mo
        for i, sp in enumerate(sensors):
            sp.sim, sp.s = sim, i
        for i, r in enumerate(ropes):
            r.sim, r.r = sim, i
        sim.sensors = list(sensors)
        sim.ropes = list(ropes)
        return sim

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


def _rotvec_deg(r) -> np.ndarray:
    """Rotation matrix of a rotation vector given in degrees (scipy's Rotation.from_rotvec of the
    radians, as the reference's init methods: mpm_elastic.py:95-96, fem_sensor.py:113-114)."""
    from scipy.spatial.transform import Rotation
    return Rotation.from_rotvec(np.deg2rad(np.asarray(r, np.float64))).as_matrix()


class MPMObj:
    """MPM object (object_model/mpm_elastic.py, mpm_plastic.py).  Two ways to make one:

    - as the reference does, ``MPMObj(dt, sub_steps, obj_name, space_scale, obj_scale, density, rho)``
      (mpm_elastic.py:19): a 64^3 grid of spacing space_scale / 64, the object's particles sampled from
      ``obj_name`` (a mesh file, see meshes.object_particles) at particle_density = 64 density
      obj_scale / space_scale and scaled by obj_scale, p_vol = (dx obj_scale)^3, rho = rho obj_scale,
      E = 4e3 space_scale, nu = 0.4, grid-mass epsilon 1e-5; ``plastic=True`` gives mpm_plastic.py's
      von Mises object (yield stress 1000).  Then ``init(position, orientation, velocity)``, and
      ``Simulation.from_objects`` builds the device world around it;
    - as a view of a built ``Simulation`` (``MPMObj(sim)``).
    Once bound to a simulation the reference's methods (p2g, grid_op, g2p, ...) run on the device."""

    def __init__(self, dt=5e-5, sub_steps=80, obj_name=None, space_scale=1.0, obj_scale=1.0, density=2, rho=1, *,
                 plastic=False, n_grid=64):
        self.particles = None
        if hasattr(dt, "world"):  # a view of a built simulation
            self.sim = dt
            return
        from . import meshes
        from .scene import MODEL_COROTATED, MODEL_VON_MISES
        self.sim = None
        self.dt, self.sub_steps = float(dt), int(sub_steps)
        self.n_grid, self.bound, self.dim = int(n_grid), 3, 3
        self.space_scale, self.obj_scale = float(space_scale), float(obj_scale)
        self.rho = rho * self.obj_scale
        self.particle_density = self.n_grid * density * self.obj_scale / self.space_scale
        self.obj_name = obj_name
        self.particles = meshes.object_particles(obj_name, int(self.particle_density)) * np.float32(self.obj_scale)
        self.n_particles = len(self.particles)
        self.dx_0 = float(self.space_scale / self.n_grid)
        self.inv_dx_0 = 1.0 / self.dx_0
        self.p_vol = (self.dx_0 * self.obj_scale) ** 3
        self.p_mass = self.p_vol * self.rho
        self.eps = 1e-5
        self.gravity = (0.0, -9.8, 0.0)
        self.E_0, self.nu_0 = 4e3 * self.space_scale, 0.4
        self.yield_stress = 1000.0 if plastic else 0.0
        self.model = MODEL_VON_MISES if plastic else MODEL_COROTATED
        self.x_init = self.v_init = None

    @property
    def mu_0(self):
        return self.E_0 / 2 / (1 + self.nu_0)

    @property
    def lambda_0(self):
        return self.E_0 * self.nu_0 / (1 + self.nu_0) / (1 - 2 * self.nu_0)

    def set_material_params(self, E, nu):
        """Young's modulus and Poisson's ratio (mu_0, lambda_0 follow, mpm_elastic.py:64-71)."""
        self.E_0, self.nu_0 = float(E), float(nu)
        if self.sim is not None:
            self.sim.world.set_material(0, E=self.E_0, nu=self.nu_0)

    def material(self):
        from .scene import Material
        return Material(self.E_0, self.nu_0, self.yield_stress, self.model)

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

    def init(self, *args):
        """``init(position, orientation, velocity)`` (mpm_elastic.py:90-114): x = R(orientation) p +
        position for the object's particles p, v = velocity, F = I, of frame 0.  A view of a simulation
        built from environment specs (no particles of its own) takes ``init(x, v=None)`` with the
        particles' positions instead."""
        if self.particles is not None and len(args) == 3 and np.asarray(args[0]).shape == (3,):
            position, orientation, velocity = args
            R = _rotvec_deg(orientation)
            self.x_init = (self.particles.astype(np.float64) @ R.T + np.asarray(position, np.float64)).astype(np.float32)
            self.v_init = np.broadcast_to(np.asarray(velocity, np.float32), self.x_init.shape).copy()
            x, v = self.x_init, self.v_init
        else:
            x = np.asarray(args[0], np.float32)
            v = np.zeros_like(x) if len(args) < 2 or args[1] is None else np.asarray(args[1], np.float32)
        if self.sim is not None:
            n = len(x)
            self.sim.world.set_particles(0, x=x, v=v, C=np.zeros((n, 3, 3), np.float32),
                                         F=np.broadcast_to(np.eye(3, dtype=np.float32), (n, 3, 3)))


class FEMDomeSensor:
    """FEM dome sensor (sensor_model/fem_sensor.py).  Two ways to make one:

    - as the reference does, ``FEMDomeSensor(dt, sub_steps, init_img_path)`` (fem_sensor.py:20): the
      dome elastomer (fibonacci hemisphere layers, Delaunay tets; N_node 200, N_t 4, t_res 0.25, inner
      radius 0.75), node mass 2 pi r^2 / N_node t_res rho with rho 2000, E 0.8e4, nu 0.43; then
      ``init(rot_x, rot_y, rot_z, t_dx, t_dy, t_dz)`` places it (fem_sensor.py:112-128) and
      ``Simulation.from_objects`` builds the device world.  ``init_img_path`` (the camera image whose
      marker blobs OpenCV detects) is not read: markers.MarkerModel holds a stored marker set;
    - as a view of sensor ``s`` of a built ``Simulation`` (``FEMDomeSensor(sim, s)``)."""

    carry = 0  # control-velocity carry of the gripper pads' update2 (gripper_fem.py:415)

    def __init__(self, dt=5e-5, sub_steps=50, init_img_path=None):
        self.dtrans = None
        self.spec = None
        if hasattr(dt, "world"):  # a view of a built simulation
            self.sim, self.s = dt, int(sub_steps)
            return
        from .scene import dome_mesh
        self.sim, self.s = None, None
        self.dt, self.sub_steps = float(dt), int(sub_steps)
        self.N_node, self.N_t, self.t_res, self.inner_radius = 200, 4, 0.25, 0.75
        self.all_nodes, self.all_f2v, self.surface_f2v, self.layer_idxs = dome_mesh(
            self.N_node, self.N_t, self.t_res, self.inner_radius)
        self.n_verts, self.n_cells, self.num_triangles = len(self.all_nodes), len(self.all_f2v), len(self.surface_f2v)
        self.dx = 2 * np.pi * self.inner_radius ** 2 / self.N_node
        self.vol = self.dx * self.t_res
        self.rho = 2000.0
        self.mass = self.vol * self.rho
        self.E_init, self.nu_init = 0.8e4, 0.43
        self.trans_world = None

    @property
    def mu(self):
        return self.E_init / 2 / (1 + self.nu_init)

    @property
    def lam(self):
        return self.E_init * self.nu_init / (1 + self.nu_init) / (1 - 2 * self.nu_init)

    def set_material_params(self, E, nu):
        """Young's modulus and Poisson's ratio of the elastomer (fem_sensor.py:190-193)."""
        self.E_init, self.nu_init = float(E), float(nu)

    def init(self, rot_x, rot_y, rot_z, t_dx, t_dy, t_dz):
        """Place the sensor: trans_world = [R | t] with R the rotation vector (rot_x, rot_y, rot_z) in
        degrees (fem_sensor.py:112-128); the rest positions are trans_world applied to the dome."""
        M = np.eye(4)
        M[:3, :3] = _rotvec_deg([rot_x, rot_y, rot_z])
        M[:3, 3] = [t_dx, t_dy, t_dz]
        self._place(M)

    def _place(self, M):
        from .scene import SensorSpec
        if self.sim is not None:
            raise RuntimeError("the sensor is already part of a simulation; place it before Simulation.from_objects")
        self.trans_world = np.asarray(M, np.float64)
        world = (self.trans_world[:3, :3] @ self.all_nodes.T).T + self.trans_world[:3, 3]
        out_dir = self.trans_world[:3, :3] @ np.array([0.0, 1.0, 0.0])
        self.spec = SensorSpec(verts=world.astype(np.float32), tets=self.all_f2v, tris=self.surface_f2v,
                               layer=self.layer_idxs, mass=self.mass, E=self.E_init, nu=self.nu_init,
                               out_dir=tuple(out_dir), carry=self.carry, trans_world=self.trans_world)

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


class GripperFEMSensor(FEMDomeSensor):
    """A gripper finger's dome sensor (sensor_model/gripper_fem.py): the same elastomer, placed by
    ``init(matrix)`` (gripper_fem.py:102-108, the finger's 4x4 pose) and integrated with the control
    velocity carried over between frames (update2, gripper_fem.py:404-418)."""

    carry = 1

    def init(self, matrix):
        self._place(np.asarray(matrix, np.float64))


class PBDRope:
    """PBD rope (object_model/PBD_rope.py).  Two ways to make one:

    - as the reference does, ``PBDRope(dt, sub_steps, p_rad, p_rho, n_particles, table_height,
      rest_length)`` (PBD_rope.py:16-60) then ``init(pos, ori)`` (:74-87), and
      ``Simulation.from_objects``;
    - as a view of rope ``r`` of a built ``Simulation`` (``PBDRope(sim, r)``)."""

    def __init__(self, dt=5e-5, sub_steps=80, p_rad=0.05, p_rho=1.0, n_particles=10, table_height=0.0,
                 rest_length=None):
        if hasattr(dt, "world"):  # a view of a built simulation
            self.sim, self.r = dt, int(sub_steps)
            self.spec = None
            return
        from .scene import RopeSpec
        self.sim, self.r = None, None
        self.dt, self.sub_steps = float(dt), int(sub_steps)
        self.spec = RopeSpec(n=int(n_particles), rad=float(p_rad), rho=float(p_rho), rest_length=rest_length,
                             table_h=float(table_height))
        self.n_particles = int(n_particles)

    def init(self, pos, ori):
        """Node 0 at ``pos`` (pinned), the others along ``ori`` at the rest length (PBD_rope.py:74-87)."""
        self.spec = self.spec.replace(pos=tuple(float(c) for c in pos), ori=tuple(float(c) for c in ori))
        if self.sim is not None:
            self.sim.world.set_rope_state(0, self.r, pos=self.spec.init_positions(),
                                          vel=np.zeros((self.spec.n, 3), np.float32),
                                          trav=np.zeros(self.spec.n, np.float32))

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
