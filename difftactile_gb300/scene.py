"""Scene specification and seeded synthetic scene generators.

A scene is a list of environments.  Each environment holds one MPM object (particles with
per-particle material ids, on its own dense grid) and the FEM sensors that touch it.  The
reference builds objects by voxelising meshes (object_model/obj_loader.py:25-65, trimesh +
mesh_to_sdf) and sensors with a scipy Delaunay dome (sensor_model/fem_sensor.py:280-322); here the
objects are seeded lattice fills of analytic shapes and the sensors are either that dome (restated
below) or a structured hex pad split into tets.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

import numpy as np

MODEL_COROTATED, MODEL_VON_MISES, MODEL_NEOHOOKEAN = 0, 1, 2
# elastomer force models of the FEM sensors: the reference's (fem_sensor.py:424-435) and linear corotated
FEM_REFERENCE, FEM_LINEAR_COROTATED = 0, 1
BC_SLIP_WALLS, BC_STICKY_FLOOR = 0, 1


def lame(E: float, nu: float) -> tuple[float, float]:
    """(mu, lambda) from Young's modulus and Poisson's ratio (mpm_elastic.py:70-71)."""
    E, nu = float(np.float32(E)), float(np.float32(nu))
    return E / 2 / (1 + nu), E * nu / (1 + nu) / (1 - 2 * nu)


def lame_grad_to_E_nu(E: float, nu: float, g_mu, g_lam):
    """Chain rule of lame(): gradients with respect to (mu, lambda) -> gradients with respect to
    (E, nu).  mu = E / (2 (1 + nu)), lambda = E nu / ((1 + nu)(1 - 2 nu)) (mpm_elastic.py:70-71)."""
    a, b = 1.0 + nu, 1.0 - 2.0 * nu
    dmu_dE, dmu_dnu = 1.0 / (2.0 * a), -E / (2.0 * a * a)
    dlam_dE, dlam_dnu = nu / (a * b), E * (1.0 + 2.0 * nu * nu) / (a * b) ** 2
    return g_mu * dmu_dE + g_lam * dlam_dE, g_mu * dmu_dnu + g_lam * dlam_dnu


@dataclass
class Material:
    E: float
    nu: float
    yield_stress: float = 0.0
    model: int = MODEL_COROTATED
    mu: float | None = None    # explicit Lame parameters override E, nu (tasks set them directly,
    lam: float | None = None   # grasp_plastic.py:65-68)

    @property
    def mu_lam(self):
        if self.mu is not None and self.lam is not None:
            return float(self.mu), float(self.lam)
        return lame(self.E, self.nu)


@dataclass
class SensorSpec:
    """FEM elastomer.  ``verts`` are world-space rest positions; layer 0 is kinematically driven;
    ``tris`` are the contact-surface triangles (local vertex ids)."""
    verts: np.ndarray          # [V,3] float
    tets: np.ndarray           # [T,4] int
    tris: np.ndarray           # [S,3] int
    layer: np.ndarray          # [V] int
    mass: float                # node mass
    E: float = 1.5e5
    nu: float = 0.45
    mu: float | None = None    # explicit Lame parameters override E, nu (tasks set them directly)
    lam: float | None = None
    out_dir: tuple = (0.0, 1.0, 0.0)
    carry: int = 0             # gripper_fem.py:415 control-velocity carry term
    trans_world: np.ndarray | None = None  # 4x4 sensor pose used by pose control
    model: int = FEM_REFERENCE  # FEM_* elastomer force model

    def lame(self):
        if self.mu is not None and self.lam is not None:
            return float(self.mu), float(self.lam)
        return lame(self.E, self.nu)

    def rest_inverse(self) -> np.ndarray:
        """B = Dm^-1 per tet from the rest positions (fem_sensor.py:334-338), float32 [T,3,3]."""
        p = self.verts.astype(np.float32)
        t = self.tets
        D = np.stack([p[t[:, 0]] - p[t[:, 3]], p[t[:, 1]] - p[t[:, 3]], p[t[:, 2]] - p[t[:, 3]]], axis=2)
        return np.linalg.inv(D.astype(np.float64)).astype(np.float32)


@dataclass
class RopeSpec:
    """PBD rope (PBDRope.__init__ / init, PBD_rope.py:18-99): ``n`` particles of radius ``rad`` laid out
    from ``pos`` along ``ori`` at the rest length; node 0 stays pinned at ``pos``.  ``kn, kd, kt, mu_t``
    are the rope-sensor contact parameters (cable_straightening.py:212-224)."""
    n: int = 50
    rad: float = 0.25
    rho: float = 10.0
    rest_length: float | None = 0.1    # None: 2 rad (bending 4 rad), else bending 2 rest_length
    pos: tuple = (0.0, 0.0, 0.0)
    ori: tuple = (0.0, 0.0, 1.0)
    table_h: float = 0.0
    stretch_compliance: float | None = None  # default 1e-5 / rho
    bend_compliance: float | None = None     # default 1e-5 / rho
    stretch_relax: float = 0.3
    bend_relax: float = 0.1
    iters: int = 1                     # stretch + bending pass pairs per substep (the reference: one)
    friction: float = 0.995
    gravity: tuple = (0.0, -9.8, 0.0)
    kn: float = 1e4
    kd: float = 100.0
    kt: float = 100.0
    mu_t: float = 1.0
    x: np.ndarray | None = None        # [n,3] initial positions overriding the straight layout
    v: np.ndarray | None = None        # [n,3] initial velocities (default 0)

    @property
    def mass(self):
        return self.rho * (np.pi * 4.0 / 3.0) * self.rad ** 3

    @property
    def rest(self):
        return 2 * self.rad if self.rest_length is None else self.rest_length

    @property
    def bend(self):
        return 4 * self.rad if self.rest_length is None else 2 * self.rest_length

    @property
    def compliance(self):
        cs = 1e-5 / self.rho if self.stretch_compliance is None else self.stretch_compliance
        cb = 1e-5 / self.rho if self.bend_compliance is None else self.bend_compliance
        return cs, cb

    def init_positions(self) -> np.ndarray:
        if self.x is not None:
            return np.asarray(self.x, np.float32)
        i = np.arange(self.n, dtype=np.float64)[:, None]
        return (np.asarray(self.pos, np.float64) + np.asarray(self.ori, np.float64) * self.rest * i).astype(np.float32)

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)


@dataclass
class EnvSpec:
    x: np.ndarray                      # [N,3] particle positions
    materials: list                    # list[Material]
    n_grid: tuple = (64, 64, 64)
    dx: float = 1.0 / 64
    p_vol: float | None = None         # default (dx/2)^3
    rho: float = 1.0
    v: np.ndarray | None = None        # [N,3] initial velocities (default 0)
    mat: np.ndarray | None = None      # [N] material ids (default 0)
    gravity: tuple = (0.0, -9.8, 0.0)
    bound: int = 3
    bc: int = BC_SLIP_WALLS
    eps: float = 1e-5
    sensors: list = field(default_factory=list)   # list[SensorSpec]
    kn: float = 1e4
    kd: float = 100.0
    kt: float = 100.0
    mu_t: float = 1.0
    ropes: list = field(default_factory=list)     # list[RopeSpec]

    @property
    def n_particles(self):
        return int(self.x.shape[0])

    @property
    def inv_dx(self):
        return 1.0 / self.dx

    @property
    def volume(self):
        return self.p_vol if self.p_vol is not None else (self.dx / 2) ** 3

    @property
    def p_mass(self):
        return self.volume * self.rho

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)


# ------------------------------------------------------------------------------------------------
# particle fills
# ------------------------------------------------------------------------------------------------
def box_particles(lo, hi, dx, ppc=8, seed=0) -> np.ndarray:
    """Cells of size dx filling the box [lo, hi), ``ppc`` points per cell jittered uniformly
    inside the cell (seeded)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    nc = np.maximum(np.round((hi - lo) / dx).astype(int), 1)
    ii = np.stack(np.meshgrid(*[np.arange(n) for n in nc], indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    j = rng.random((ii.shape[0], ppc, 3))
    pts = lo + (ii[:, None, :] + j) * dx
    return pts.reshape(-1, 3).astype(np.float32)


def cube_particles(center, side, dx, ppc=8, seed=0):
    c = np.asarray(center, np.float64)
    return box_particles(c - side / 2, c + side / 2, dx, ppc, seed)


def sphere_particles(center, radius, dx, ppc=8, seed=0, r_in=0.0):
    c = np.asarray(center, np.float64)
    pts = box_particles(c - radius, c + radius, dx, ppc, seed)
    r = np.linalg.norm(pts - c, axis=1)
    return pts[(r < radius) & (r >= r_in)]


# ------------------------------------------------------------------------------------------------
# sensor meshes
# ------------------------------------------------------------------------------------------------
def eul2mat_zyx(rot_deg, trans):
    """4x4 transform with R = Rz Ry Rx (fem_sensor.py:196-210)."""
    rx, ry, rz = np.deg2rad(np.asarray(rot_deg, np.float64))
    Rx = np.array([[1, 0, 0], [0, np.cos(rx), -np.sin(rx)], [0, np.sin(rx), np.cos(rx)]])
    Ry = np.array([[np.cos(ry), 0, np.sin(ry)], [0, 1, 0], [-np.sin(ry), 0, np.cos(ry)]])
    Rz = np.array([[np.cos(rz), -np.sin(rz), 0], [np.sin(rz), np.cos(rz), 0], [0, 0, 1]])
    M = np.eye(4)
    M[:3, :3] = Rz @ Ry @ Rx
    M[:3, 3] = trans
    return M


def hex_pad_local(nx=20, nz=20, ny=5, h=0.0125):
    """Structured hex pad in local coordinates: x in [0, nx h], z in [0, nz h], thickness along +y
    with layer 0 (driven base) at y = 0 and the contact surface at y = ny h.  Each hex is split
    into 6 tets sharing its main diagonal; the contact surface is 2 triangles per top quad."""
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    I, J, K = np.meshgrid(np.arange(NX), np.arange(NY), np.arange(NZ), indexing="ij")
    verts = np.stack([I, J, K], -1).reshape(-1, 3).astype(np.float64) * h
    vid = lambda i, j, k: (i * NY + j) * NZ + k  # noqa: E731
    layer = J.reshape(-1)
    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    # cube corners c[b] with bit 0 -> x, bit 1 -> y, bit 2 -> z
    c = [vid(ci + (b & 1), cj + ((b >> 1) & 1), ck + ((b >> 2) & 1)) for b in range(8)]
    # Kuhn split along the 0-7 diagonal: paths through x, y, z in every order
    paths = [(1, 3), (1, 5), (2, 3), (2, 6), (4, 5), (4, 6)]
    tets = np.concatenate([np.stack([c[0], c[a], c[b], c[7]], -1) for a, b in paths], 0)
    ti, tk = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    ti, tk = ti.ravel(), tk.ravel()
    a, b_, c_, d = vid(ti, ny, tk), vid(ti + 1, ny, tk), vid(ti + 1, ny, tk + 1), vid(ti, ny, tk + 1)
    tris = np.concatenate([np.stack([a, b_, c_], -1), np.stack([a, c_, d], -1)], 0)
    return verts, tets.astype(np.int32), tris.astype(np.int32), layer.astype(np.int32)


def hex_pad_sensor(center_bottom, nx=20, nz=20, ny=5, h=0.0125, rho=1000.0, E=1.5e5, nu=0.45, model=FEM_REFERENCE):
    """Pad pressing down: the local pad is flipped by 180 deg about x so that its contact surface
    faces -y, and placed with the centre of that surface at ``center_bottom``."""
    v, tets, tris, layer = hex_pad_local(nx, nz, ny, h)
    v = v - np.array([nx * h / 2, 0.0, nz * h / 2])
    v[:, 1] -= ny * h  # contact surface at local y = 0 ... after the flip it faces -y
    M = eul2mat_zyx([180.0, 0.0, 0.0], center_bottom)
    world = (M[:3, :3] @ v.T).T + M[:3, 3]
    out_dir = M[:3, :3] @ np.array([0.0, 1.0, 0.0])
    vol = (nx * h) * (nz * h) * (ny * h)
    mass = rho * vol / len(v)
    return SensorSpec(verts=world.astype(np.float32), tets=tets, tris=tris, layer=layer, mass=mass, E=E, nu=nu,
                      out_dir=tuple(out_dir), trans_world=M, model=model)


def finger_pad_sensor(pose, nx=6, nz=6, ny=2, h=1.0 / 32, rho=1000.0, E=1.5e5, nu=0.45, shift=(0.0, 0.0)):
    """Hex pad on a gripper finger (gripper_fem.py's sensor placed by init(matrix)): in the finger's
    frame the pad is centred in x and z with its contact surface at y = 0 facing +y (towards the
    other finger); ``pose`` is the finger's 4x4 pose, ``shift`` moves the pad within its surface
    (local x, z).  Velocity carry of gripper_fem.py:415."""
    pose = np.asarray(pose, np.float64)
    v, tets, tris, layer = hex_pad_local(nx, nz, ny, h)
    v = v - np.array([nx * h / 2 - shift[0], ny * h, nz * h / 2 - shift[1]])
    world = (pose[:3, :3] @ v.T).T + pose[:3, 3]
    out_dir = pose[:3, :3] @ np.array([0.0, 1.0, 0.0])
    vol = (nx * h) * (nz * h) * (ny * h)
    return SensorSpec(verts=world.astype(np.float32), tets=tets, tris=tris, layer=layer, mass=rho * vol / len(v), E=E,
                      nu=nu, out_dir=tuple(out_dir), trans_world=pose, carry=1)


def fibonacci_hemisphere(samples, scale=1.0):
    """Points evenly spread on a hemisphere (fem_sensor.py:280-291)."""
    phi = np.pi * (np.sqrt(5.0) - 1.0)
    idx = np.arange(samples).astype(float)
    y = 1 - (idx / (samples - 1))
    radius = np.sqrt(1 - y * y)
    theta = phi * idx
    return scale * np.vstack((np.cos(theta) * radius, y, np.sin(theta) * radius)).T


def dome_mesh(N_node=200, N_t=4, t_res=0.25, inner_radius=0.75):
    """The reference's dome elastomer mesh (fem_sensor.py:293-322): N_t fibonacci hemisphere layers,
    tets from a Delaunay triangulation of (x, layer height, z), surface triangles from a Delaunay
    triangulation of the outer layer's (x, z)."""
    from scipy.spatial import Delaunay

    nodes, heights, layers = [], [], []
    surface = None
    cur = 0
    for i in range(N_t):
        rad = inner_radius + i * t_res
        n = int(N_node * (rad ** 2) / (inner_radius ** 2))
        pts = fibonacci_hemisphere(n, rad)
        nodes.append(pts)
        heights.append([rad] * n)
        layers.append([i] * n)
        if i == N_t - 1:
            surface = cur + Delaunay(np.vstack((pts[:, 0], pts[:, 2])).T).simplices
        cur += n
    heights = np.concatenate(heights)
    nodes = np.concatenate(nodes, 0)
    tets = Delaunay(np.array([nodes[:, 0], heights, nodes[:, 2]]).T).simplices
    return nodes, tets.astype(np.int32), surface.astype(np.int32), np.concatenate(layers).astype(np.int32)


def dome_sensor(trans=np.eye(4), dt_rho=2000.0, N_node=200, N_t=4, t_res=0.25, inner_radius=0.75):
    nodes, tets, tris, layer = dome_mesh(N_node, N_t, t_res, inner_radius)
    world = (trans[:3, :3] @ nodes.T).T + trans[:3, 3]
    dxa = 2 * np.pi * inner_radius ** 2 / N_node
    mass = dxa * t_res * dt_rho  # fem_sensor.py:35-38
    out_dir = trans[:3, :3] @ np.array([0.0, 1.0, 0.0])
    return SensorSpec(verts=world.astype(np.float32), tets=tets, tris=tris, layer=layer, mass=mass, E=0.8e4, nu=0.43,
                      out_dir=tuple(out_dir), trans_world=np.asarray(trans, np.float64))
