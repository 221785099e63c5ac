"""Small seeded scenes the oracle finishes in seconds (parity cases)."""
import numpy as np

from difftactile_gb300 import scene as S


def elastic_cube(n=32, side_cells=6, ppc=8, seed=0, v=(0.0, 0.0, 0.0), model=S.MODEL_COROTATED, gravity=(0, -9.8, 0),
                 rho=1000.0, E=5e3, nu=0.3, bc=S.BC_SLIP_WALLS, center=(0.5, 0.5, 0.5)):
    dx = 1.0 / n
    x = S.cube_particles(center, side_cells * dx, dx, ppc, seed)
    rng = np.random.default_rng(seed + 100)
    vv = np.asarray(v, np.float32) + 0.05 * rng.standard_normal(x.shape).astype(np.float32)
    return S.EnvSpec(x=x, v=vv, materials=[S.Material(E, nu, 50.0, model)], n_grid=(n, n, n), dx=dx, rho=rho,
                     gravity=gravity, bc=bc)


def pad_over_box(n=32, box_cells=(6, 4, 6), pad=(6, 6, 2), ppc=8, seed=1, model=S.MODEL_VON_MISES, yield_stress=5.0,
                 two_pads=False):
    """An elastoplastic box resting low in the domain with a hex pad whose contact surface is 0.37
    cell above the box top, so that grid nodes above the box start inside the pad.  The offset is not
    a multiple of half a cell: a surface through node centres ((j + 0.5) dx) would put nodes exactly
    at sdf = 0, where the contact force has a kink and finite differences are meaningless."""
    dx = 1.0 / n
    lo = np.array([n / 2 - box_cells[0] / 2, 4, n / 2 - box_cells[2] / 2]) * dx
    hi = lo + np.array(box_cells) * dx
    x = S.box_particles(lo, hi, dx, ppc, seed)
    rng = np.random.default_rng(seed + 7)
    v = 0.02 * rng.standard_normal(x.shape).astype(np.float32)
    sensors = []
    top = hi[1]
    sp = S.hex_pad_sensor([0.5 + 0.13 * dx, top + 0.37 * dx, 0.5 - 0.21 * dx], nx=pad[0], nz=pad[1], ny=pad[2], h=dx)
    sensors.append(sp)
    if two_pads:
        sp2 = S.hex_pad_sensor([0.5 - 0.07 * dx, top + 0.83 * dx, 0.5 + 0.11 * dx], nx=pad[0] - 2, nz=pad[1] - 2, ny=pad[2],
                               h=dx)
        sensors.append(sp2)
    return S.EnvSpec(x=x, v=v, materials=[S.Material(5e3, 0.3, yield_stress, model)], n_grid=(n, n, n), dx=dx,
                     rho=1000.0, sensors=sensors, kn=1e4, kd=100.0, kt=100.0, mu_t=1.0)


def control_velocity(sp, seed=3, scale=0.05, down=-0.1):
    rng = np.random.default_rng(seed)
    base = np.array([0.0, down, 0.0]) + scale * rng.standard_normal(3)
    return np.broadcast_to(base, sp.verts.shape).astype(np.float32).copy()


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(np.linalg.norm(b), 1e-30)
    return float(np.linalg.norm(a - b) / den)


def aligned_pad_over_box(n=32, box_cells=(8, 4, 8), seed=4):
    """Pad vertices on grid-node planes in x and z: node centres project onto quad diagonals, where the
    two triangles' centroids are equidistant (exact argmin ties, resolved to the first index)."""
    dx = 1.0 / n
    lo = np.array([n / 2 - box_cells[0] / 2, 4, n / 2 - box_cells[2] / 2]) * dx
    hi = lo + np.array(box_cells) * dx
    x = S.box_particles(lo, hi, dx, 8, seed)
    sp = S.hex_pad_sensor([0.5, hi[1] + 0.37 * dx, 0.5], nx=10, nz=10, ny=2, h=dx)
    return S.EnvSpec(x=x, materials=[S.Material(5e3, 0.3)], n_grid=(n, n, n), dx=dx, rho=1000.0, sensors=[sp],
                     kn=1e4, kd=100.0, kt=100.0, mu_t=1.0)


def dome_over_box(n=40, seed=5):
    """The reference's dome elastomer (Delaunay mesh, spatially unordered triangles), scaled to
    radius 0.15 and pressed with its apex into a box."""
    dx = 1.0 / n
    lo = np.array([0.5 - 0.12, 4 * dx, 0.5 - 0.12])
    hi = np.array([0.5 + 0.12, 4 * dx + 0.2, 0.5 + 0.12])
    x = S.box_particles(lo, hi, dx, 8, seed)
    nodes, tets, tris, layer = S.dome_mesh()
    scale = 0.15 / 1.5
    # dome apex (outer layer, y max) pointing down into the box top
    M = S.eul2mat_zyx([180.0, 0.0, 0.0], [0.5, hi[1] + 1.5 * scale - 0.3 * dx, 0.5])
    world = (M[:3, :3] @ (scale * nodes).T).T + M[:3, 3]
    sp = S.SensorSpec(verts=world.astype(np.float32), tets=tets, tris=tris, layer=layer, mass=1e-3, E=8e3,
                      nu=0.43, out_dir=tuple(M[:3, :3] @ np.array([0.0, 1.0, 0.0])), trans_world=M)
    return S.EnvSpec(x=x, materials=[S.Material(5e3, 0.3)], n_grid=(n, n, n), dx=dx, rho=1000.0, sensors=[sp],
                     kn=1e4, kd=100.0, kt=100.0, mu_t=1.0)


def rope_under_pad(n_rope=16, rad=0.01, seed=9, pad=(6, 6, 2), press=0.3, table=True):
    """A PBD rope lying along x on the table (y = 0) with a hex pad above it whose contact surface
    is ``press`` radii into the rope's contact band (no MPM particles)."""
    from difftactile_gb300 import scene as S_
    rng = np.random.default_rng(seed)
    rest = 1.6 * rad
    x0 = 0.5 - rest * (n_rope - 1) / 2
    pts = np.stack([x0 + rest * np.arange(n_rope), np.full(n_rope, rad), np.full(n_rope, 0.5)], 1)
    pts[1:] += 0.1 * rad * rng.standard_normal((n_rope - 1, 3))
    rope = S_.RopeSpec(n=n_rope, rad=rad, rho=1000.0, rest_length=rest, pos=tuple(pts[0]), ori=(1.0, 0.0, 0.0),
                       table_h=0.0 if table else -1.0, x=pts.astype(np.float32), kn=1e4, kd=10.0, kt=10.0, mu_t=0.5)
    h = 0.012
    surf_y = 2 * rad - press * rad
    sp = S_.hex_pad_sensor([0.5 + 0.13 * h, surf_y, 0.5 - 0.21 * h], nx=pad[0], nz=pad[1], ny=pad[2], h=h)
    return S_.EnvSpec(x=np.zeros((0, 3), np.float32), materials=[S_.Material(5e3, 0.3)], n_grid=(16, 16, 16),
                      dx=1.0 / 16, rho=1000.0, sensors=[sp], ropes=[rope])


def gripper_box(n=32, seed=11, grip_width=0.075):
    """A box held between the two finger pads of a parallel-jaw gripper (end effector at
    (0.5, 0.5, 0.5), fingers 0.3 apart minus twice the grip width); the pads start 0.1 cell inside
    the box's faces.  Returns (env, kinematics)."""
    from difftactile_gb300.trajectory import GripperKinematics
    dx = 1.0 / n
    kin = GripperKinematics([0.0, 0.0, 0.0], [0.5, 0.5, 0.5], grip_width, 1e-4, base_height=0.02, base_width=0.3,
                            finger_height=0.1)
    F = [f.numpy() for f in kin.finger_poses0()]
    lo = np.array([0.5 - 2.5 * dx, 0.33, 0.5 - 2.5 * dx])
    x = S.box_particles(lo, lo + np.array([5, 4, 5]) * dx, dx, 8, seed)
    # pads shifted off the node planes: node centres must not project onto the quads' diagonals
    pads = [S.finger_pad_sensor(Fi, nx=6, nz=6, ny=2, h=dx, shift=(0.13 * dx, -0.21 * dx)) for Fi in F]
    env = S.EnvSpec(x=x, materials=[S.Material(5e3, 0.3, 5.0, S.MODEL_VON_MISES)], n_grid=(n, n, n), dx=dx,
                    rho=1000.0, sensors=pads, kn=1e4, kd=100.0, kt=100.0, mu_t=1.0, gravity=(0.0, 0.0, 0.0))
    return env, kin
