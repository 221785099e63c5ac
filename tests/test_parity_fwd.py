"""Forward-substep parity of the CUDA path (through the C ABI) against the CPU oracle.

Tolerances (fp32, norm-wise relative): state after one substep within 1e-5 (x, v, F, sensor pos)
and 1e-4 for C and the sensor velocities (sums of 27 atomically accumulated, partly cancelling
contributions whose order the atomics choose); the contact argmin is compared bit-exactly; drift
after 100 substeps is bounded by 1e-3.  Each comparison prints its measured errors (pytest -s).
"""
import numpy as np
import pytest
import torch

from difftactile_gb300 import scene as S
from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4


def run_gpu(envs, n_sub, cvs=None, **world_kw):
    w = World(envs, n_frames=n_sub + 1, dt=DT, **world_kw)
    if cvs is not None:
        for s, cv in enumerate(cvs):
            w.set_control_velocity(s, cv)
    w.step_begin()
    for f in range(n_sub):
        w.substep(f)
    torch.cuda.synchronize()
    return w


def run_oracle(env, n_sub, cvs=None):
    o = O.Oracle(env, DT)
    st = o.initial_state()
    dbgs = []
    for _ in range(n_sub):
        st, d = o.substep(st, cv=cvs, cv1=cvs)
        dbgs.append(d)
    return st, dbgs


def sensor_state(w, f, s):
    return {k: w.sensor_frame(n, f, s).cpu().numpy() for k, n in (("pos", "v_pos"), ("vel", "v_vel"), ("vpos", "v_vpos"))}


def compare(w, f, st, env_idx=0, sensor_base=0, tol_x=1e-5, tol_v=1e-5, tol_c=1e-4):
    got = {k: v.cpu().numpy() for k, v in w.particles(f).items()}
    row = w.env_rows[env_idx]
    sl = slice(row.p_begin, row.p_end)
    errs = {k: SS.rel_err(got[k][sl], st[k]) for k in ("x", "v", "C", "F")}
    for s in range(len(st.get("pos", []))):
        ss = sensor_state(w, f, sensor_base + s)
        errs[f"pos{s}"] = SS.rel_err(ss["pos"], st["pos"][s])
        errs[f"vel{s}"] = SS.rel_err(ss["vel"], st["vel"][s])
    def tol(k):
        if k in ("x", "F") or k.startswith("pos"):
            return tol_x
        return tol_v if k == "v" else tol_c
    print("parity", {k: f"{e:.2e}" for k, e in errs.items()})
    bad = {k: e for k, e in errs.items() if e > tol(k)}
    assert not bad, f"parity errors {errs}"
    return errs


@pytest.mark.parametrize("model", [S.MODEL_COROTATED, S.MODEL_VON_MISES, S.MODEL_NEOHOOKEAN])
def test_one_substep_elastic_cube(cuda_lib, model):
    env = SS.elastic_cube(model=model)
    w = run_gpu([env], 1)
    st, _ = run_oracle(env, 1)
    assert w.error_word() == 0
    compare(w, 1, st)


@pytest.mark.parametrize("lanes", [8, 4])
def test_one_substep_pad_contact_and_grid(cuda_lib, lanes):
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = run_gpu([env], 1, cv, contact_lanes=lanes)
    st, dbg = run_oracle(env, 1, cv)
    assert w.error_word() == 0
    compare(w, 1, st)
    g = w.dense_grid(0)
    d = dbg[0]
    occ = d["grid_m"] > env.eps
    assert np.array_equal(g["m"].cpu().numpy() > env.eps, occ)
    assert SS.rel_err(g["m"].cpu().numpy(), d["grid_m"]) < 1e-5
    assert SS.rel_err(g["v_out"].cpu().numpy(), d["grid_v_out"]) < 1e-4
    # contact argmin: bit-exact on occupied nodes (same float ops, every operation rounded)
    ci = g["cidx"].cpu().numpy()[..., :1]
    assert np.array_equal(ci[occ], d["cidx"][occ])
    # contact actually happened and the sensor received the reaction
    assert np.abs(d["grid_f"]).sum() > 0


def test_two_pads_one_env(cuda_lib):
    env = SS.pad_over_box(two_pads=True)
    cv = [SS.control_velocity(sp, seed=s) for s, sp in enumerate(env.sensors)]
    w = run_gpu([env], 1, cv)
    st, _ = run_oracle(env, 1, cv)
    compare(w, 1, st)


def test_multi_material_particles(cuda_lib):
    env = SS.elastic_cube()
    rng = np.random.default_rng(5)
    env = env.replace(mat=rng.integers(0, 3, env.n_particles).astype(np.int32),
                      materials=[S.Material(5e3, 0.3), S.Material(4e5, 0.4), S.Material(2e3, 0.3, 5.0, S.MODEL_VON_MISES)])
    w = run_gpu([env], 1)
    st, _ = run_oracle(env, 1)
    compare(w, 1, st)


def test_batched_uneven_envs_match_each_env_alone(cuda_lib):
    envs = [SS.pad_over_box(n=32, box_cells=(6, 4, 6), seed=1),
            SS.elastic_cube(n=24, side_cells=5, seed=2, model=S.MODEL_NEOHOOKEAN),
            SS.pad_over_box(n=40, box_cells=(8, 5, 7), pad=(8, 8, 2), seed=3)]
    cvs = [SS.control_velocity(sp, seed=9) for e in envs for sp in e.sensors]
    w = run_gpu(envs, 1, cvs)
    s0 = 0
    for e, env in enumerate(envs):
        ncv = [SS.control_velocity(sp, seed=9) for sp in env.sensors]
        st, _ = run_oracle(env, 1, ncv if env.sensors else None)
        compare(w, 1, st, env_idx=e, sensor_base=s0)
        s0 += len(env.sensors)


def test_reference_method_sequence_equals_fused_substep(cuda_lib):
    """p2g; fem.update; grid_op (occupancy + check_collision + collision + grid_op); g2p; fem.update2
    (grasp_plastic.py:151-164) gives the fused substep's result."""
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w1 = run_gpu([env], 1, cv)
    w2 = World([env], n_frames=2, dt=DT)
    w2.set_control_velocity(0, cv[0])
    w2.step_begin()
    for name in ("dt_p2g", "dt_fem_update", "dt_grid_op", "dt_g2p", "dt_fem_update2"):
        w2.call(name, 0)
    torch.cuda.synchronize()
    a, b = w1.particles(1), w2.particles(1)
    for k in a:
        assert SS.rel_err(a[k].cpu().numpy(), b[k].cpu().numpy()) < 1e-5


def test_drift_after_100_substeps(cuda_lib):
    env = SS.pad_over_box(n=32, box_cells=(6, 4, 6))
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    n = 100
    w = run_gpu([env], n, cv)
    st, _ = run_oracle(env, n, cv)
    assert w.error_word() == 0
    errs = compare(w, n, st, tol_x=1e-3, tol_v=1e-3, tol_c=1e-3)
    print("drift after 100 substeps:", errs)


def test_oob_particle_sets_error_and_is_skipped(cuda_lib):
    env = SS.elastic_cube()
    x = env.x.copy()
    x[0] = [0.999, 0.5, 0.5]  # stencil base + 2 would be past the last node
    env = env.replace(x=x)
    w = run_gpu([env], 1)
    assert w.error_word() & 1
    got = w.particles(1)["x"].cpu().numpy()
    assert np.array_equal(got[0], x[0])
    w.clear_error()
    assert w.error_word() == 0


@pytest.mark.parametrize("lanes", [8, 4])
@pytest.mark.parametrize("maker", [SS.aligned_pad_over_box, SS.dome_over_box])
def test_contact_argmin_ties_and_unordered_meshes(cuda_lib, maker, lanes):
    """Exact first-minimum argmin on exact ties (grid-aligned pad) and on a spatially unordered
    triangle list (Delaunay dome), against the oracle's sequential scan, with 8 and 4 lanes per node."""
    env = maker()
    w = run_gpu([env], 1, contact_lanes=lanes)
    _, dbg = run_oracle(env, 1)
    g = w.dense_grid(0)
    occ = dbg[0]["grid_m"] > env.eps
    assert occ.sum() > 100
    ci = g["cidx"].cpu().numpy()[..., 0]
    assert np.array_equal(ci[occ], dbg[0]["cidx"][..., 0][occ])


@pytest.mark.parametrize("lanes", [8, 4])
def test_contact_argmin_large_pad(cuda_lib, lanes):
    """A 40x40 pad (3,200 surface triangles, 100 groups of centroids) over a box: the grid kernel
    searches per-block candidate groups; the argmin stays bit-exact with the oracle's scan."""
    env = SS.pad_over_box(n=64, box_cells=(16, 4, 16), pad=(40, 40, 2))
    assert len(env.sensors[0].tris) > 32 * 32
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = run_gpu([env], 1, cv, contact_lanes=lanes)
    st, dbg = run_oracle(env, 1, cv)
    assert w.error_word() == 0
    compare(w, 1, st)
    g = w.dense_grid(0)
    occ = dbg[0]["grid_m"] > env.eps
    assert occ.sum() > 1000
    ci = g["cidx"].cpu().numpy()[..., 0]
    assert np.array_equal(ci[occ], dbg[0]["cidx"][..., 0][occ])


def test_one_substep_linear_corotated_pad(cuda_lib):
    """The pad's elastomer with the linear corotated force (configuration 2's model): one substep in
    contact against the oracle."""
    import dataclasses
    env = SS.pad_over_box()
    env = env.replace(sensors=[dataclasses.replace(env.sensors[0], model=S.FEM_LINEAR_COROTATED)])
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = run_gpu([env], 2, cv)
    st, _ = run_oracle(env, 2, cv)
    assert w.error_word() == 0
    compare(w, 2, st)
