"""Seeded synthetic scenes with the shapes of the benchmark configurations.

Physical parameters the configuration text leaves open are fixed here (and only here):
object density 1000 kg/m^3 (so that the reference's absolute grid-mass epsilon of 1e-5 stays far
below node masses and the penalty contact of stiffness 1e4 N/m per node stays explicit-stable at
dt = 1e-4), contact damping 100, friction coefficient 0.5, and the tangential stiffness kt of the
friction (calculate_contact_force, grasp_plastic.py:205-216) per environment from the mass of a grid
node of one cell, kt = 0.2 rho dx^3 / dt (``friction_stiffness``).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import scene as S


def friction_stiffness(rho, dx, dt=1e-4, gain=0.2):
    """Tangential stiffness of the contact friction for grid nodes of mass ~ rho dx^3.  While a contact
    sticks (kt |v_t| below the Coulomb cap) the explicit friction removes kt dt / m of the relative
    tangential velocity per substep; above 1 it overshoots.  The forward stays bounded by the cap, but
    the adjoint runs through the sticking branch's Jacobian with gain |1 - kt dt / m| per substep: with
    kt = 100 on nodes of ~1e-3 kg (gain ~ 9) the 25,000-substep adjoint of the grasp rollout overflows
    float32.  ``gain`` = kt dt / m for a node of one cell's mass."""
    return gain * rho * dx ** 3 / dt


@dataclass
class Config:
    name: str
    envs: list
    dt: float
    substeps: int
    n_steps: int
    actions: np.ndarray | None = None   # [n_steps, n_sensors, 6]
    loss_terms: tuple = ()
    ckpt_every: int = 1        # 0: full tape (every frame kept, no recompute)
    tape_blocks: int | None = None  # grid-tape capacity per frame (active 4^3-node blocks)
    rope_terms: tuple = ()     # (rope, target [3]): squared distance of the rope's tip from the target

    @property
    def n_particles(self):
        return sum(e.n_particles for e in self.envs)

    def build(self, device="cuda", rebin_every: int = 0, **world_kw):
        """World sized for this configuration's rollout and its PoseTrajectory (``rebin_every``: see
        Trajectory; checkpointed configurations only)."""
        from .trajectory import PoseTrajectory
        from .world import World
        nf = PoseTrajectory.frames_needed(self.n_steps, self.substeps, self.ckpt_every)
        w = World(self.envs, n_frames=nf, dt=self.dt, device=device, tape_blocks=self.tape_blocks, **world_kw)
        return w, PoseTrajectory(w, self.n_steps, self.ckpt_every, self.loss_terms, rope_terms=self.rope_terms,
                                 rebin_every=rebin_every)


def _press_env(n_grid=96, box_cells=20, pad=(20, 20, 5), pad_h=0.0125, seed=1, yield_stress=50.0, E=5e3, nu=0.3,
               center=(0.5, 0.5), gap_cells=0.37):
    dx = 1.0 / n_grid
    cx, cz = center
    lo = np.array([cx * n_grid - box_cells / 2, 4.0, cz * n_grid - box_cells / 2]) * dx
    hi = lo + box_cells * dx
    x = S.box_particles(lo, hi, dx, 8, seed)
    # pad density scaled as h^-2: a tet's stiffness grows as E h and a node's mass as rho h^3, so the
    # pad keeps the stiffness-to-mass ratio, and with it the explicit stability margin at dt = 1e-4,
    # of the 0.0125 m pad (the elastomer has no damping; with node masses held fixed instead, pads
    # of 0.023 m hexes oscillate with growing amplitude and turn non-finite within 170 control
    # steps).  Node masses then grow in proportion to h, and the penalty contact (stiffness 1e4 per
    # node) keeps k dt^2 / m below 0.2 down to the smallest pads of the population (0.005 m)
    rho_pad = 1000.0 * (0.0125 / pad_h) ** 2
    # configuration 2's pad is linear corotated (its text), configuration 4 takes the same pad
    sp = S.hex_pad_sensor([cx, hi[1] + gap_cells * dx, cz], nx=pad[0], nz=pad[1], ny=pad[2], h=pad_h, E=1.5e5,
                          nu=0.45, rho=rho_pad, model=S.FEM_LINEAR_COROTATED)
    env = S.EnvSpec(x=x, materials=[S.Material(E, nu, yield_stress, S.MODEL_VON_MISES)],
                    n_grid=(n_grid, n_grid, n_grid), dx=dx, rho=1000.0, sensors=[sp],
                    kn=1e4, kd=100.0, kt=friction_stiffness(1000.0, dx), mu_t=0.5)
    return env, sp


def press_actions(n_steps, n_sensors=1, seed=2, press=0.15, slide=0.1, noise=0.01):
    """Press for the first 60% of the steps, then slide along +x; N(0, noise) on all 6 DoF.  Pose actions
    act in the sensor's own frame (set_pose_control, fem_sensor.py:229-245), whose +y is the pad's
    out-direction, towards the object: the press is +y.  ``press`` is a speed (m/s) or one per sensor."""
    rng = np.random.default_rng(seed)
    a = noise * rng.standard_normal((n_steps, n_sensors, 6))
    n_press = int(0.6 * n_steps)
    a[:n_press, :, 1] += np.broadcast_to(np.asarray(press, np.float64), (n_sensors,))
    a[n_press:, :, 0] += slide
    return a


def sensor_press(n_steps=100, substeps=20, seed=1) -> Config:
    """Config 2: FEM pad (20x20x5 hex, 6 tets/hex: 2646 nodes, 12000 tets, 800 surface triangles,
    linear corotated, E 1.5e5, nu 0.45, driven base layer) pressing and sliding on a von-Mises elastoplastic box of
    64,000 particles (20^3 cells x 8) on a 96^3 grid, yield stress 50, penalty contact 1e4;
    100 steps x 20 substeps, actions ~ N(0, 0.01) around press-and-slide; loss = L2 of the surface
    nodes' displacement field against a seeded target field.

    The whole rollout is kept on the device (2001 frames: 12.3 GB of particle records, a grid tape
    of 1024 active blocks per frame, 6.3 GB), so the backward needs no recompute."""
    env, sp = _press_env(seed=seed)
    rng = np.random.default_rng(3)
    target = 1e-3 * rng.standard_normal(sp.verts.shape)
    surf = int(sp.layer.max())
    return Config("sensor_press", [env], 1e-4, substeps, n_steps, press_actions(n_steps, 1), ((0, surf, target),),
                  ckpt_every=0, tape_blocks=1024)


def elastic_cube(substeps=200, seed=0) -> Config:
    """Config 1: elastic cube (side 0.25 at (0.5, 0.6, 0.5), 8 particles/cell jittered, 32,768
    particles) on 64^3, Neo-Hookean E 5e3, nu 0.3, rho 1, p_vol (dx/2)^3, gravity, sticky floor,
    dt 1e-4, 200 substeps.  Grid-mass epsilon scaled to 1e-3 particle masses (rho = 1 makes node
    masses ~1e-6, below the reference's absolute 1e-5)."""
    dx = 1.0 / 64
    x = S.cube_particles([0.5, 0.6, 0.5], 0.25, dx, 8, seed)
    env = S.EnvSpec(x=x, materials=[S.Material(5e3, 0.3, 0.0, S.MODEL_NEOHOOKEAN)], n_grid=(64, 64, 64), dx=dx,
                    rho=1.0, bc=S.BC_STICKY_FLOOR)
    env = env.replace(eps=1e-3 * env.p_mass)
    return Config("elastic_cube", [env], 1e-4, substeps, 1)


def batched_population(n_envs=64, substeps=20, n_steps=200, seed=6, lo=8_000, hi=128_000) -> Config:
    """Config 4: independent environments with particle counts log-uniform in [8k, 128k], grids
    48^3..128^3 sized to the object, per-env materials, one config-2 pad each.

    Each pad starts 2.07 cells above its box, clear of the grid nodes the box occupies (a pad started
    inside that band takes a penalty impulse on its first substep which, with no damping in the
    elastomer, rings on for the whole rollout and drives pads of some environments to non-finite
    values within 200 steps), and presses at a speed that takes it through the gap and 25% of the
    box's height by the end of the press phase of the 200-step rollout (120 steps; the boxes, yield
    stress 20-100 Pa, also slump under gravity).  Shorter rollouts keep these speeds, so their steps
    are the first steps of the full one."""
    rng = np.random.default_rng(seed)
    envs, press = [], []
    gap = 2.07
    n_press = 120
    for e in range(n_envs):
        n_p = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        cells = max(4, int(round((n_p / 8) ** (1 / 3))))
        need = 4 * int(np.ceil((cells * 1.5 + 12) / 4))
        n_grid = int(np.clip(max(need, 4 * int(rng.uniform(48, 128) / 4)), 48, 128))
        Ev = float(np.exp(rng.uniform(np.log(2e3), np.log(2e4))))
        env, _ = _press_env(n_grid=n_grid, box_cells=cells, pad=(20, 20, 5), pad_h=cells / n_grid / 16,
                            seed=seed * 1000 + e, E=Ev, yield_stress=float(rng.uniform(20, 100)), gap_cells=gap)
        envs.append(env)
        press.append((gap + 0.25 * cells) / n_grid / (n_press * 1e-4 * substeps))
    acts = press_actions(n_steps, n_envs, press=np.array(press))
    terms = []
    for e, env in enumerate(envs):
        sp = env.sensors[0]
        tg = 1e-3 * np.random.default_rng(100 + e).standard_normal(sp.verts.shape)
        terms.append((e, int(sp.layer.max()), tg))
    # grid tape: ~14,500 of the 843,000 blocks are active per frame for 64 environments; 32,768 reserved
    tape = 32768 if n_envs >= 64 else max(1024, 512 * n_envs)
    return Config("batched_population", envs, 1e-4, substeps, n_steps, acts, tuple(terms), tape_blocks=tape)


def grasp_sphere(n_steps=1000, substeps=25, seed=4, n_grid=128, n_core=20_000, n_shell=180_000, pad=(20, 20, 5),
                 ckpt_every=50) -> "tuple[Config, object]":
    """Config 3: a parallel-jaw gripper whose two finger pads (configuration 2's 20x20x5 hex pad each)
    squeeze a sphere of a stiff core (``n_core`` particles) and a soft shell (``n_shell``, E log-uniform
    in [1e3, 1e5], seed 4) on an ``n_grid``^3 grid; ``n_steps`` x ``substeps`` with a checkpoint every
    ``ckpt_every`` steps.  Returns (config, gripper kinematics); the actions are [n_steps, 7] (d_pos,
    d_ori, d_gripper): close for the first half, then lift."""
    from .trajectory import GripperKinematics
    rng = np.random.default_rng(seed)
    dx = 1.0 / n_grid
    # sphere radius from the particle count (8 per cell): volume = (n_core + n_shell) / 8 cells
    vol = (n_core + n_shell) / 8 * dx ** 3
    R = (3 * vol / (4 * np.pi)) ** (1 / 3)
    r_core = R * (n_core / (n_core + n_shell)) ** (1 / 3)
    c = np.array([0.5, 0.08 + R + 4 * dx, 0.5])
    x = S.sphere_particles(c, R, dx, 8, seed)
    core = np.linalg.norm(x - c, axis=1) < r_core
    E_shell = float(np.exp(rng.uniform(np.log(1e3), np.log(1e5))))
    mats = [S.Material(E_shell, 0.3, 0.0, S.MODEL_COROTATED), S.Material(1e6, 0.3, 0.0, S.MODEL_COROTATED)]
    h = 2 * R / pad[0]
    grip = 0.5 * (0.3 - 2 * R) + 0.1 * h  # pads start just inside the sphere's silhouette
    kin = GripperKinematics([0.0, 0.0, 0.0], [0.5, c[1] + 0.12, 0.5], grip, 1e-4, base_height=0.02, base_width=0.3,
                            finger_height=0.1)
    pads = [S.finger_pad_sensor(f.numpy(), nx=pad[0], nz=pad[1], ny=pad[2], h=h, rho=1000.0 * (0.0125 / h) ** 2,
                                shift=(0.13 * dx, -0.21 * dx))
            for f in kin.finger_poses0()]
    env = S.EnvSpec(x=x, materials=mats, mat=core.astype(np.int32), n_grid=(n_grid,) * 3, dx=dx, rho=1000.0,
                    sensors=pads, kn=1e4, kd=100.0, kt=friction_stiffness(1000.0, dx), mu_t=0.5,
                    bc=S.BC_STICKY_FLOOR)
    acts = np.zeros((n_steps, 7))
    acts[: n_steps // 2, 6] = 0.05
    acts[n_steps // 2:, 1] = 0.05
    acts += 0.01 * rng.standard_normal(acts.shape)
    return Config("grasp_sphere", [env], 1e-4, substeps, n_steps, acts, (), ckpt_every), kin


def rope_pads(n_envs=16, n_steps=500, substeps=20, seed=5, n_rope=2000, pad=(40, 40, 5), n_particles=512_000,
              n_grid=160, rope_len=0.6, iters=50, ckpt_every=10, yield_stress=50.0) -> Config:
    """Config 5: ``n_envs`` environments, each a 40x40x5 hex pad (10,086 nodes, 48,000 tets) pressing a
    PBD rope of ``n_rope`` particles (``rope_len`` long, compliance 1e-6, ``iters`` stretch + bending pass
    pairs per substep) into an elastoplastic slab (von Mises, yield stress 50) of ``n_particles`` MPM
    particles (4 cells thick) on an ``n_grid``^3 grid; ``n_steps`` x ``substeps``, a checkpoint every
    ``ckpt_every`` steps (16 x 512k particles: 786 MB per frame).  The loss is the squared distance of
    each rope's tip from a seeded target.

    Each pad starts 2.07 cells above the slab, clear of the grid nodes it occupies (see
    batched_population), and presses at a speed that takes its surface one cell below the slab's top
    by the end of the press phase of the 500-step rollout (300 steps); shorter rollouts keep that
    speed.  The rope-pad contact stiffness is scaled to the rope particles' mass (k dt^2 / m = 0.2) so
    that the explicit penalty contact stays stable for thin ropes."""
    rng = np.random.default_rng(seed)
    envs = []
    dx = 1.0 / n_grid
    dt = 1e-4
    gap = 2.07
    press = (gap + 1.0) * dx / (300 * dt * substeps)
    for e in range(n_envs):
        sx = max(2, int(round(np.sqrt(n_particles / 8 / 4))))   # cells of a 4-cell-thick slab, 8 per cell
        sz = max(2, int(round(n_particles / 8 / 4 / sx)))
        lo = np.array([0.5 - sx * dx / 2, 4 * dx, 0.5 - sz * dx / 2])
        x = S.box_particles(lo, lo + np.array([sx, 4, sz]) * dx, dx, 8, seed * 100 + e)
        top = float(x[:, 1].max())
        rest = rope_len / max(n_rope - 1, 1)
        rad = rest / 1.6
        xs = np.stack([0.5 - rope_len / 2 + rest * np.arange(n_rope), np.full(n_rope, top + rad),
                       np.full(n_rope, 0.5 + 0.01 * rng.standard_normal())], 1)
        mass = 1000.0 * (np.pi * 4.0 / 3.0) * rad ** 3
        kn = 0.2 * mass / dt ** 2
        rope = S.RopeSpec(n=n_rope, rad=rad, rho=1000.0, rest_length=rest, pos=tuple(xs[0]), ori=(1.0, 0.0, 0.0),
                          table_h=top, x=xs.astype(np.float32), stretch_compliance=1e-6, bend_compliance=1e-6,
                          kn=kn, kd=0.01 * kn * dt, kt=0.2 * mass / dt, mu_t=0.5, iters=iters)
        h = min(1.2 * rope_len, 0.9) / pad[0]
        sp = S.hex_pad_sensor([0.5 + 0.13 * dx, top + gap * dx, 0.5 - 0.21 * dx], nx=pad[0], nz=pad[1], ny=pad[2],
                              h=h, rho=1000.0 * (0.0125 / h) ** 2)
        envs.append(S.EnvSpec(x=x, materials=[S.Material(5e3, 0.3, yield_stress, S.MODEL_VON_MISES)],
                              n_grid=(n_grid,) * 3, dx=dx, rho=1000.0, sensors=[sp], ropes=[rope], kn=1e4, kd=100.0,
                              kt=friction_stiffness(1000.0, dx), mu_t=0.5))
    rope_terms = tuple((e, xs_tip) for e, xs_tip in enumerate(
        [np.asarray(env.ropes[0].x[-1], np.float64) + np.array([0.0, 0.0, 0.05]) for env in envs]))
    # grid tape: a 512k-particle slab touches ~3,000 of the 64,000 blocks of its 160^3 grid per frame
    tape = 8192 * n_envs
    return Config("rope_pads", envs, dt, substeps, n_steps, press_actions(n_steps, n_envs, press=press), (),
                  ckpt_every=ckpt_every, tape_blocks=tape, rope_terms=rope_terms)
