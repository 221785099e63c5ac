"""Golden substeps computed by the reference's own simulation methods.

The reference's substep is Taichi code (taichi is absent here and not installable), so its methods
are read out of the reference source with `ast` and run, in float64, on numpy fields through the
stand-in `ti` module of this folder (ti_numpy.py, which lists the semantics it takes for Taichi's
primitives).  Five cases on seeded states, one substep each except the chained one:

  corotated_cube  MPMObj of object_model/mpm_elastic.py (compute_new_F, svd, p2g, check_grid_occupy,
                  grid_op, g2p; :134-260), a fixed-corotated cube falling into the floor band of a 16^3
                  grid (wall rule of grid_op);
  plastic_pads    Contact.update of tasks/grasp_plastic.py:151-164 (check_collision, collision,
                  calculate_contact_force; :205-299) and its readouts compute_contact_force and
                  compute_obj_pos (:218-229, :259-261) over MPMObj of object_model/mpm_plastic.py (the
                  von Mises p2g; :140-310) and two FEMDomeSensor pads of sensor_model/fem_sensor.py
                  (init_pos, find_closest, find_sdf, update_contact_force, update, update2; :325-457),
                  a plastic box pressed by two hex pads (half of its particles beyond the yield surface);
  multi_material_cube  MultiObj of object_model/multi_obj.py (per-particle Lame parameters by material
                  tag in p2g; :168-305), a cube of three material layers;
  plastic_pads_chain  the plastic_pads scene over five substeps of the grasp task's Contact.update
                  (frame-to-frame carry of particles, sensor state and per-frame grids);
  rope_pads       Contact.update of tasks/cable_straightening.py:166-173 (check_collision, collision and
                  its calculate_contact_force variant; :212-319) over PBDRope of object_model/PBD_rope.py
                  (update, update_contact_force; :108-180) and two FEMDomeSensor pads of
                  sensor_model/gripper_fem.py (per-frame control velocities, the carry term of update2),
                  a rope pressed by a pad along ten of its sixteen particles;
  rope_pads_chain the rope_pads scene over five substeps, the pads' control velocities ramping.

The scenes come from tests/small_scenes.py (the parity scenes); states, constants and the outputs
(particles, the grid at occupied nodes, contact indices, the sensors' forces and next frame) go to
tests/golden/substep_ref.npz.

    python tests/golden/make_substep.py REFERENCE_ROOT
"""
import dataclasses
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from tests import small_scenes as SS  # noqa: E402
from tests.golden import ti_numpy as ti  # noqa: E402

DT = 1e-4
CHAIN = 5   # substeps of the chained case
PKG = None  # the reference's package folder, set by main()


def scenes():
    """The parity scenes (also rebuilt by tests/test_golden_substep.py)."""
    from difftactile_gb300 import scene as S
    cube = SS.elastic_cube(n=16, side_cells=4, center=(0.5, 3.5 / 16, 0.5), v=(0.0, -0.5, 0.0))
    pads = SS.pad_over_box(two_pads=True, box_cells=(4, 3, 4), yield_stress=2.0)
    rope = SS.rope_under_pad(pad=(16, 4, 2), press=0.5)  # 11 of the 16 rope particles under the pad
    # the cable task's two gripper pads (control-velocity carry of gripper_fem.update2): the parity
    # scene's pad pressing the rope, and a second one well above it
    far = S.hex_pad_sensor([0.5, 0.3, 0.5], nx=4, nz=4, ny=2, h=0.012)
    rope = rope.replace(sensors=[dataclasses.replace(rope.sensors[0], carry=1), dataclasses.replace(far, carry=1)])
    # three materials by particle (MultiObj's lower / middle / upper parts, E 4e5 / 4e1 / 4e3, nu 0.4)
    mats = [S.Material(4e5, 0.4), S.Material(4e1, 0.4), S.Material(4e3, 0.4)]
    tri = SS.elastic_cube(n=16, side_cells=4, center=(0.5, 0.5, 0.5), v=(0.0, 0.0, 0.0), seed=2)
    layer = np.digitize(tri.x[:, 1], np.quantile(tri.x[:, 1], [1 / 3, 2 / 3])).astype(np.int32)
    tri = tri.replace(materials=mats, mat=layer)
    return {"corotated_cube": cube, "plastic_pads": pads, "rope_pads": rope, "multi_material_cube": tri,
            "plastic_pads_chain": pads, "rope_pads_chain": rope}


def seeded_state(env, seed, jitter):
    """Seeded float32 state; sensor vertices displaced by ``jitter`` x N(0, 1) from rest."""
    rng = np.random.default_rng(seed)
    N = env.n_particles
    r32 = lambda a: np.asarray(a, np.float32).astype(np.float64)  # noqa: E731
    F = np.eye(3) + 0.05 * rng.standard_normal((N, 3, 3))
    F[1::2] = (np.eye(3) + 1e-4 * rng.standard_normal((N, 3, 3)))[1::2]  # inside the yield surface
    st = {"x": r32(env.x), "v": r32(env.v if env.v is not None else np.zeros((N, 3))),
          "C": r32(0.3 * rng.standard_normal((N, 3, 3))), "F": r32(F)}
    st["pos"] = [r32(sp.verts + jitter * rng.standard_normal(sp.verts.shape)) for sp in env.sensors]
    st["vel"] = [r32(0.01 * rng.standard_normal(sp.verts.shape)) for sp in env.sensors]
    st["vpos"] = [r32(sp.verts) for sp in env.sensors]
    st["cv"] = [r32(SS.control_velocity(sp, seed=11 + i)) for i, sp in enumerate(env.sensors)]
    st["cv1"] = [r32(c + 0.01 * rng.standard_normal(c.shape)) for c in st["cv"]]  # frame f + 1 (gripper)
    st["rpos"] = [r32(rp.init_positions()) for rp in env.ropes]
    st["rvel"] = [r32(0.01 * rng.standard_normal((rp.n, 3))) for rp in env.ropes]
    st["rtrav"] = [r32(rng.integers(0, 2, rp.n)) for rp in env.ropes]
    return st


def mpm_object(env, st, src, plastic, cls="MPMObj", frames=2):
    n = env.n_grid[0]
    N = env.n_particles
    m = env.materials[0]
    mu, lam = m.mu_lam
    o = types.SimpleNamespace(
        n_particles=N, n_grid=n, dim=3, bound=env.bound, dt=DT, dx_0=env.dx, inv_dx_0=1.0 / env.dx,
        p_vol=env.volume, p_mass=env.p_mass, eps=env.eps, dtype=ti.f32, gravity=ti.Vector(list(env.gravity)),
        mu_0=ti.scalar(mu), lambda_0=ti.scalar(lam), yield_stress=ti.scalar(m.yield_stress))
    for k, e in (("x_0", (3,)), ("v_0", (3,)), ("C_0", (3, 3)), ("F_new", (3, 3)), ("F_0", (3, 3)),
                 ("U_svd", (3, 3)), ("V_svd", (3, 3)), ("S_svd", (3, 3))):
        setattr(o, k, ti.Field((frames, N), e))
    for k, e in (("grid_v_in", (3,)), ("grid_v_out", (3,)), ("grid_m", ()), ("grid_f", (3,))):
        setattr(o, k, ti.Field((frames, n, n, n), e))
    o.grid_occupy = ti.Field((frames, n, n, n), (), np.int64)
    o.x_0.a[0], o.v_0.a[0], o.C_0.a[0], o.F_0.a[0] = st["x"], st["v"], st["C"], st["F"]
    names = ["compute_new_F", "svd", "p2g", "check_grid_occupy", "grid_op", "g2p", "update_contact_force"]
    if plastic:
        names += ["norm", "make_matrix_from_diag", "compute_von_mises"]
    return ti.methods(src, cls, names, o)


def sensor_object(sp, pos, vel, vpos, cv, src, cls="FEMDomeSensor", frames=2):
    V, T = len(sp.verts), len(sp.tets)
    mu, lam = sp.lame()
    M = np.eye(4) if sp.trans_world is None else np.asarray(sp.trans_world, np.float64)
    s = types.SimpleNamespace(n_verts=V, n_cells=T, num_triangles=len(sp.tris), dt=DT, mass=float(sp.mass), eps=1e-10,
                              mu=ti.scalar(mu), lam=ti.scalar(lam), trans_h=ti.Field((), (4, 4)),
                              rot_h=ti.Field((), (3, 3)), out_direction=ti.Field((), (3,)))
    s.trans_h[None] = np.eye(4)
    s.rot_h[None] = M[:3, :3]
    s.init_x = ti.Field((V,), (3,))
    s.init_x.a[:] = np.asarray(sp.verts, np.float64)
    for k in ("pos", "vel", "virtual_pos", "external_force_field"):
        setattr(s, k, ti.Field((frames, V), (3,)))
    s.control_vel = ti.Field((V,), (3,))
    s.B = ti.Field((T,), (3, 3))
    s.f2v = ti.Field((T,), (4,), np.int64)
    s.f2v.a[:] = sp.tets
    s.contact_seg = ti.Field((len(sp.tris),), (3,), np.int64)
    s.contact_seg.a[:] = sp.tris
    s.layer_id = ti.Field((V,), (), np.int64)
    s.layer_id.a[:] = sp.layer
    ti.methods(src, cls, ["init_pos", "find_closest", "find_sdf", "update_contact_force", "update", "update2"], s)
    s.init_pos()  # rest-shape inverses B from the rest positions, out_direction = rot_h e_y
    s.B.a[:] = s.B.a.astype(np.float32)  # B is a float32 field in the reference (and on the device)
    s.pos.a[0], s.vel.a[0], s.virtual_pos.a[0] = pos, vel, vpos
    s.control_vel.a[:] = cv
    return s


def gripper_sensor_object(sp, pos, vel, vpos, cvs, src):
    """A gripper pad (sensor_model/gripper_fem.py: per-frame control velocities ``cvs`` [frames][V][3])."""
    s = sensor_object(sp, pos, vel, vpos, cvs[0], src, cls="FEMDomeSensor", frames=len(cvs))
    s.control_vel = ti.Field((len(cvs), len(sp.verts)), (3,))
    s.control_vel.a[:] = cvs
    return s


def rope_object(rp, pos, vel, trav, src, frames=2):
    n = rp.n
    cs, cb = rp.compliance
    o = types.SimpleNamespace(n_particles=n, n_segments=n - 1, dt=DT, p_rad=rp.rad, p_mass=rp.mass,
                              invM=1.0 / rp.mass, gravity=ti.Vector(list(rp.gravity)), eps=1e-10,
                              table_height=rp.table_h, rest_length=rp.rest, bending_length=rp.bend,
                              stretch_compliance=ti.scalar(cs), bending_compliance=ti.scalar(cb),
                              stretch_relaxation=ti.scalar(rp.stretch_relax),
                              bending_relaxation=ti.scalar(rp.bend_relax), floor_friction=rp.friction,
                              floor_normal=ti.Field((), (3,)), init_pos=ti.Field((n,), (3,)),
                              travel_info=ti.Field((frames, n), (1,)))
    o.floor_normal[None] = [0.0, 1.0, 0.0]
    o.init_pos.a[:] = rp.init_positions()
    for k in ("tmp_pos", "tmp_vel", "dpos", "pos", "vel", "ext_f"):
        setattr(o, k, ti.Field((frames, n), (3,)))
    o.pos.a[0], o.vel.a[0], o.travel_info.a[0, :, 0] = pos, vel, trav
    return ti.methods(src, "PBDRope", ["update", "update_contact_force"], o)


def occupied(o):
    occ = np.argwhere(o.grid_occupy.a[0] == 1)
    i, j, k = occ.T
    return occ, o.grid_m.a[0][i, j, k], o.grid_v_in.a[0][i, j, k], o.grid_v_out.a[0][i, j, k], o.grid_f.a[0][i, j, k]


def run_cube(env, st):
    o = mpm_object(env, st, os.path.join(PKG, "object_model", "mpm_elastic.py"), plastic=False)
    for name in ("compute_new_F", "svd", "p2g", "check_grid_occupy", "grid_op", "g2p"):
        getattr(o, name)(0)
    return o, []


def run_multi(env, st):
    o = mpm_object(env, st, os.path.join(PKG, "object_model", "multi_obj.py"), plastic=False, cls="MultiObj")
    mu, lam = zip(*[m.mu_lam for m in env.materials])
    o.mu_0, o.lamda_0 = ti.Field((len(mu),)), ti.Field((len(mu),))
    o.mu_0.a[:], o.lamda_0.a[:] = mu, lam
    o.titles = ti.Field((env.n_particles,), (), np.int64)
    o.titles.a[:] = env.mat
    for name in ("compute_new_F", "svd", "p2g", "check_grid_occupy", "grid_op", "g2p"):
        getattr(o, name)(0)
    return o, []


def run_pads(env, st, n_sub=1):
    fr = n_sub + 1
    o = mpm_object(env, st, os.path.join(PKG, "object_model", "mpm_plastic.py"), plastic=True, frames=fr)
    sens = [sensor_object(sp, st["pos"][i], st["vel"][i], st["vpos"][i], st["cv"][i],
                          os.path.join(PKG, "sensor_model", "fem_sensor.py"), frames=fr)
            for i, sp in enumerate(env.sensors)]
    n = env.n_grid[0]
    c = types.SimpleNamespace(mpm_object=o, gripper=types.SimpleNamespace(fem_sensor1=sens[0], fem_sensor2=sens[1]),
                              kn=ti.scalar(env.kn), kd=ti.scalar(env.kd), kt=ti.scalar(env.kt),
                              friction_coeff=ti.scalar(env.mu_t), norm_eps=1e-11,
                              contact_idx=ti.Field((fr, n, n, n), (2,), np.int64))
    c.contact_force1, c.contact_force2, c.predict_obj_pos = ti.Field((), (3,)), ti.Field((), (3,)), ti.Field((), (3,))
    ti.methods(os.path.join(PKG, "tasks", "grasp_plastic.py"), "Contact",
               ["update", "check_collision", "collision", "calculate_contact_force", "compute_contact_force",
                "compute_obj_pos"], c)
    for f in range(n_sub):
        c.update(f)
    c.compute_contact_force(0)  # the readouts of the grasp task's losses (:218-229, :259-261)
    c.compute_obj_pos(1)
    return o, sens, c


def run_rope(env, st, n_sub=1):
    fem = os.path.join(PKG, "sensor_model", "gripper_fem.py")
    fr = n_sub + 1
    cvs = [np.stack([st["cv"][i] + f * (st["cv1"][i] - st["cv"][i]) for f in range(fr)]) for i in range(len(env.sensors))]
    sens = [gripper_sensor_object(sp, st["pos"][i], st["vel"][i], st["vpos"][i], cvs[i], fem)
            for i, sp in enumerate(env.sensors)]
    rp = env.ropes[0]
    ro = rope_object(rp, st["rpos"][0], st["rvel"][0], st["rtrav"][0], os.path.join(PKG, "object_model", "PBD_rope.py"),
                     frames=fr)
    c = types.SimpleNamespace(rope_object=ro, gripper=types.SimpleNamespace(fem_sensor1=sens[0], fem_sensor2=sens[1]),
                              kn=ti.scalar(rp.kn), kd=ti.scalar(rp.kd), kt=ti.scalar(rp.kt),
                              friction_coeff=ti.scalar(rp.mu_t), norm_eps=1e-11,
                              contact_idx=ti.Field((fr, rp.n), (2,), np.int64),
                              contact_flag=ti.Field((fr, rp.n), (), np.int64))
    ti.methods(os.path.join(PKG, "tasks", "cable_straightening.py"), "Contact",
               ["update", "check_collision", "collision", "calculate_contact_force"], c)
    for f in range(n_sub):
        c.update(f)
    return ro, sens, c


def main():
    global PKG
    PKG = os.path.join(reference_root(), "difftactile")
    f32 = lambda a: np.asarray(a, np.float32)  # noqa: E731 - the inputs are float32 values
    out = {}
    for name, env in scenes().items():
        seed = {"corotated_cube": 5, "plastic_pads": 6, "rope_pads": 7, "multi_material_cube": 8,
                "plastic_pads_chain": 9, "rope_pads_chain": 10}[name]
        st = seeded_state(env, seed=seed,
                          jitter=0.02 * (0.012 if name == "rope_pads" else env.dx))  # 2% of a hex edge
        rec = {"consts": np.array([DT, env.dx, env.volume, env.p_mass, env.eps, env.bound, *env.materials[0].mu_lam,
                                   env.materials[0].yield_stress, env.kn, env.kd, env.kt, env.mu_t])}
        if name == "plastic_pads_chain":
            o, sens, c = run_pads(env, st, n_sub=CHAIN)
            rec.update(x=f32(st["x"]), v=f32(st["v"]), C=f32(st["C"]), F=f32(st["F"]),
                       xN=o.x_0.a[CHAIN], vN=o.v_0.a[CHAIN], CN=o.C_0.a[CHAIN], FN=o.F_0.a[CHAIN])
            for s_, so in enumerate(sens):
                for key, val in (("pos", f32(st["pos"][s_])), ("vel", f32(st["vel"][s_])),
                                 ("vpos", f32(st["vpos"][s_])), ("cv", f32(st["cv"][s_])), ("cv1", f32(st["cv1"][s_])),
                                 ("B", so.B.a), ("posN", so.pos.a[CHAIN]), ("velN", so.vel.a[CHAIN]),
                                 ("vposN", so.virtual_pos.a[CHAIN])):
                    rec[f"s{s_}_{key}"] = val
            out.update({f"{name}/{k}": v for k, v in rec.items()})
            print(name + ":", f"{CHAIN} substeps")
            continue
        if name == "rope_pads_chain":  # control velocities ramp linearly: frame f = cv + f (cv1 - cv)
            ro, sens, c = run_rope(env, st, n_sub=CHAIN)
            rec.update(rpos=f32(st["rpos"][0]), rvel=f32(st["rvel"][0]), rtrav=f32(st["rtrav"][0]),
                       rposN=ro.pos.a[CHAIN], rvelN=ro.vel.a[CHAIN], rtravN=ro.travel_info.a[CHAIN, :, 0])
            for s_, so in enumerate(sens):
                for key, val in (("pos", f32(st["pos"][s_])), ("vel", f32(st["vel"][s_])),
                                 ("vpos", f32(st["vpos"][s_])), ("cv", f32(st["cv"][s_])), ("cv1", f32(st["cv1"][s_])),
                                 ("B", so.B.a), ("posN", so.pos.a[CHAIN]), ("velN", so.vel.a[CHAIN]),
                                 ("vposN", so.virtual_pos.a[CHAIN])):
                    rec[f"s{s_}_{key}"] = val
            out.update({f"{name}/{k}": v for k, v in rec.items()})
            print(name + ":", f"{CHAIN} substeps, {int(ro.travel_info.a[CHAIN, :, 0].sum())} rope particles travelled")
            continue
        if name == "rope_pads":
            ro, sens, c = run_rope(env, st)
            rec.update(rpos=f32(st["rpos"][0]), rvel=f32(st["rvel"][0]), rtrav=f32(st["rtrav"][0]),
                       rpos1=ro.pos.a[1], rvel1=ro.vel.a[1], rtrav1=ro.travel_info.a[1, :, 0], rext=ro.ext_f.a[0],
                       rcidx=c.contact_idx.a[0].astype(np.int32))
            summary = f"{env.ropes[0].n} rope particles, {int((ro.ext_f.a[0] != 0).any(1).sum())} in contact"
        else:
            run = {"corotated_cube": run_cube, "multi_material_cube": run_multi}.get(name)
            o, sens, c = run(env, st) + (None,) if run else run_pads(env, st)
            occ, gm, gvi, gvo, gf = occupied(o)
            rec.update(x=f32(st["x"]), v=f32(st["v"]), C=f32(st["C"]), F=f32(st["F"]), x1=o.x_0.a[1], v1=o.v_0.a[1],
                       C1=o.C_0.a[1], F1=o.F_0.a[1], occ=occ.astype(np.int32), grid_m=gm, grid_v_in=gvi,
                       grid_v_out=gvo, grid_f=gf)
            if c is not None:
                i, j, k = occ.T
                rec["cidx"] = c.contact_idx.a[0][i, j, k].astype(np.int32)
                rec["contact_force"] = np.stack([c.contact_force1.a, c.contact_force2.a])
                rec["com1"] = c.predict_obj_pos.a
            summary = f"{env.n_particles} particles, {len(occ)} occupied nodes"
        for s, so in enumerate(sens):
            for key, val in (("pos", f32(st["pos"][s])), ("vel", f32(st["vel"][s])), ("vpos", f32(st["vpos"][s])),
                             ("cv", f32(st["cv"][s])), ("cv1", f32(st["cv1"][s])), ("B", so.B.a),
                             ("vel_mid", so.vel.a[0]), ("ext", so.external_force_field.a[0]), ("pos1", so.pos.a[1]),
                             ("vel1", so.vel.a[1]), ("vpos1", so.virtual_pos.a[1])):
                rec[f"s{s}_{key}"] = val
            summary += f", sensor {s}: {int((so.external_force_field.a[0] != 0).any(1).sum())} vertices in contact"
        out.update({f"{name}/{k}": v for k, v in rec.items()})
        print(name + ":", summary)
    np.savez_compressed(os.path.join(HERE, "substep_ref.npz"), **out)


if __name__ == "__main__":
    main()
