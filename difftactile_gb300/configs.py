"""Seeded synthetic scenes with the shapes of the benchmark configurations.

Physical parameters the configuration text leaves open are fixed here (and only here):
object density 1000 kg/m^3 (so that the reference's absolute grid-mass epsilon of 1e-5 stays far
below node masses and the penalty contact of stiffness 1e4 N/m per node stays explicit-stable at
dt = 1e-4), contact damping 100, tangential stiffness 100, friction coefficient 0.5.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import scene as S


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

    @property
    def n_particles(self):
        return sum(e.n_particles for e in self.envs)

    def build(self, device="cuda", **world_kw):
        """World sized for this configuration's rollout and its PoseTrajectory."""
        from .trajectory import PoseTrajectory
        from .world import World
        nf = PoseTrajectory.frames_needed(self.n_steps, self.substeps, self.ckpt_every)
        w = World(self.envs, n_frames=nf, dt=self.dt, device=device, tape_blocks=self.tape_blocks, **world_kw)
        return w, PoseTrajectory(w, self.n_steps, self.ckpt_every, self.loss_terms)


def _press_env(n_grid=96, box_cells=20, pad=(20, 20, 5), pad_h=0.0125, seed=1, yield_stress=50.0, E=5e3, nu=0.3,
               center=(0.5, 0.5)):
    dx = 1.0 / n_grid
    cx, cz = center
    lo = np.array([cx * n_grid - box_cells / 2, 4.0, cz * n_grid - box_cells / 2]) * dx
    hi = lo + box_cells * dx
    x = S.box_particles(lo, hi, dx, 8, seed)
    # pad density scaled so that node masses stay those of the 0.0125 m pad: the explicit penalty
    # contact (stiffness 1e4 per node) needs k dt^2 / m well below 1 on the pad's vertices too
    rho_pad = 1000.0 * (0.0125 / pad_h) ** 3
    sp = S.hex_pad_sensor([cx, hi[1] + 0.37 * dx, cz], nx=pad[0], nz=pad[1], ny=pad[2], h=pad_h, E=1.5e5, nu=0.45,
                          rho=rho_pad)
    env = S.EnvSpec(x=x, materials=[S.Material(E, nu, yield_stress, S.MODEL_VON_MISES)],
                    n_grid=(n_grid, n_grid, n_grid), dx=dx, rho=1000.0, sensors=[sp],
                    kn=1e4, kd=100.0, kt=100.0, mu_t=0.5)
    return env, sp


def press_actions(n_steps, n_sensors=1, seed=2, press=0.15, slide=0.1, noise=0.01):
    """Press for the first 60% of the steps, then slide along +x; N(0, noise) on all 6 DoF."""
    rng = np.random.default_rng(seed)
    a = noise * rng.standard_normal((n_steps, n_sensors, 6))
    n_press = int(0.6 * n_steps)
    a[:n_press, :, 1] -= press
    a[n_press:, :, 0] += slide
    return a


def sensor_press(n_steps=100, substeps=20, seed=1) -> Config:
    """Config 2: FEM pad (20x20x5 hex, 6 tets/hex: 2646 nodes, 12000 tets, 800 surface triangles,
    E 1.5e5, nu 0.45, driven base layer) pressing and sliding on a von-Mises elastoplastic box of
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
    48^3..128^3 sized to the object, per-env materials, one config-2 pad each."""
    rng = np.random.default_rng(seed)
    envs = []
    for e in range(n_envs):
        n_p = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        cells = max(4, int(round((n_p / 8) ** (1 / 3))))
        need = 4 * int(np.ceil((cells * 1.5 + 12) / 4))
        n_grid = int(np.clip(max(need, 4 * int(rng.uniform(48, 128) / 4)), 48, 128))
        Ev = float(np.exp(rng.uniform(np.log(2e3), np.log(2e4))))
        env, _ = _press_env(n_grid=n_grid, box_cells=cells, pad=(20, 20, 5), pad_h=cells / n_grid / 16,
                            seed=seed * 1000 + e, E=Ev, yield_stress=float(rng.uniform(20, 100)))
        envs.append(env)
    acts = press_actions(n_steps, n_envs)
    terms = []
    for e, env in enumerate(envs):
        sp = env.sensors[0]
        tg = 1e-3 * np.random.default_rng(100 + e).standard_normal(sp.verts.shape)
        terms.append((e, int(sp.layer.max()), tg))
    # grid tape: ~14,500 of the 843,000 blocks are active per frame; 32,768 reserved
    return Config("batched_population", envs, 1e-4, substeps, n_steps, acts, tuple(terms), tape_blocks=32768)
