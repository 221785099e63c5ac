"""PBD rope (PBDRope.update, PBD_rope.py:112-180) with its sensor contact
(cable_straightening.py:288-319) on the GPU, through the C ABI, against the oracle.

Tolerances: state after 3 substeps within 1e-5 relative (positions) and 1e-4 (velocities, contact
sums); the rope argmin triangle bit-exact; adjoint of one substep within 1e-3 relative of the
oracle's float64 adjoint (itself checked against finite differences in test_oracle_rope.py).
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


def run_gpu(envs, n_sub, cvs=None, **kw):
    w = World(envs, n_frames=n_sub + 1, dt=DT, **kw)
    if cvs is not None:
        for s, cv in enumerate(cvs):
            w.set_control_velocity(s, cv)
    w.step_begin()
    for f in range(n_sub):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    return w


def oracle_run(env, n_sub, cvs=None, dtype=np.float32):
    o = O.Oracle(env, DT, dtype)
    st = o.initial_state()
    dbgs = []
    for _ in range(n_sub):
        st, d = o.substep(st, cv=cvs, cv1=cvs)
        dbgs.append(d)
    return st, dbgs


def test_rope_under_pad_forward(cuda_lib):
    env = SS.rope_under_pad()
    cv = [SS.control_velocity(sp, scale=0.02, down=-0.05) for sp in env.sensors]
    n_sub = 3
    w = run_gpu([env], n_sub, cv)
    st, dbgs = oracle_run(env, n_sub, cv)
    rs = {k: v.cpu().numpy() for k, v in w.rope_state(n_sub, 0).items()}
    assert SS.rel_err(rs["pos"], st["rpos"][0]) < 1e-5
    assert SS.rel_err(rs["vel"], st["rvel"][0]) < 1e-4
    assert np.array_equal(rs["trav"], st["rtrav"][0])
    for f, d in enumerate(dbgs):
        cid = w.t["r_cidx"][f, :, 0].cpu().numpy()
        assert np.array_equal(cid, d["rope_cidx"][0][:, 0]), f
        re = w.t["r_ext"][f, :, :3].cpu().numpy()
        assert SS.rel_err(re, d["rope_ext"][0]) < 1e-4, f
    ps = w.sensor_frame("v_pos", n_sub, 0).cpu().numpy()
    vs = w.sensor_frame("v_vel", n_sub, 0).cpu().numpy()
    assert SS.rel_err(ps, st["pos"][0]) < 1e-5
    assert SS.rel_err(vs, st["vel"][0]) < 1e-4


def test_free_rope_sags_like_the_oracle_over_50_substeps(cuda_lib):
    rp = S.RopeSpec(n=40, rad=0.01, rho=1000.0, rest_length=0.012, pos=(0.3, 0.5, 0.5), ori=(1.0, 0.0, 0.0),
                    table_h=0.45)
    env = S.EnvSpec(x=np.zeros((0, 3), np.float32), materials=[S.Material(5e3, 0.3)], n_grid=(16, 16, 16),
                    dx=1.0 / 16, ropes=[rp])
    w = run_gpu([env], 50)
    st, _ = oracle_run(env, 50)
    rs = w.rope_state(50, 0)
    assert SS.rel_err(rs["pos"].cpu().numpy(), st["rpos"][0]) < 1e-5
    assert SS.rel_err(rs["vel"].cpu().numpy(), st["rvel"][0]) < 1e-3


def test_ropes_in_two_envs_beside_an_mpm_env(cuda_lib):
    e0 = SS.rope_under_pad(n_rope=70, seed=1)         # two contact CTAs
    e1 = SS.pad_over_box()
    e2 = SS.rope_under_pad(n_rope=9, seed=2, press=0.5)
    cvs = [SS.control_velocity(e.sensors[0], seed=5 + i, scale=0.02, down=-0.05) for i, e in enumerate((e0, e1, e2))]
    w = run_gpu([e0, e1, e2], 2, cvs)
    for r, (e, cv) in enumerate(((e0, cvs[0]), (e2, cvs[2]))):
        st, _ = oracle_run(e, 2, [cv])
        rs = w.rope_state(2, r)
        assert SS.rel_err(rs["pos"].cpu().numpy(), st["rpos"][0]) < 1e-5, r
        assert SS.rel_err(rs["vel"].cpu().numpy(), st["rvel"][0]) < 1e-4, r


def test_rope_solver_on_the_second_stream_matches_one_stream(cuda_lib):
    """The rope solver on the world's second stream beside G2P, and its adjoint beside the MPM adjoint
    stages (World(overlap_ropes=True), the default), against everything on one stream: four substeps
    of two rope environments (six pass pairs each) beside an MPM environment, then the adjoint sweep
    down to frame 0 from seeded adjoints.  The two differ only in the atomics' summation order."""
    e0 = SS.rope_under_pad(n_rope=70, seed=1)
    e0 = e0.replace(ropes=[e0.ropes[0].replace(iters=6)])
    e1 = SS.pad_over_box()
    e2 = SS.rope_under_pad(n_rope=9, seed=2, press=0.5)
    cvs = [SS.control_velocity(e.sensors[0], seed=5 + i, scale=0.02, down=-0.05) for i, e in enumerate((e0, e1, e2))]
    n = 4
    out = {}
    for overlap in (False, True):
        w = World([e0, e1, e2], n_frames=n + 1, dt=DT, grad_clip=0.0, overlap_ropes=overlap)
        assert bool(w.w.aux_stream) == overlap
        for s, cv in enumerate(cvs):
            w.set_control_velocity(s, cv)
        w.step_begin()
        for f in range(n):
            w.substep(f)
        w.adj_clear()
        g = torch.Generator(device=w.device).manual_seed(3)
        for name in ("r_adj", "v_adj_pos", "v_adj_vel"):
            w.t[name][n & 1].copy_(torch.randn(w.t[name][n & 1].shape, device=w.device, generator=g))
        w.substeps_bwd(n, 0)
        torch.cuda.synchronize()
        assert w.error_word() == 0
        out[overlap] = {"rstate": w.t["r_state"][n].clone(), "r_adj": w.t["r_adj"][0].clone(),
                        "v_adj_pos": w.t["v_adj_pos"][0].clone(), "p_adj": w.t["p_adj"][0].clone()}
    errs = {k: SS.rel_err(out[True][k].cpu().numpy(), out[False][k].cpu().numpy()) for k in out[True]}
    print("second stream vs one stream", errs)
    assert max(errs.values()) < 1e-5, errs


@pytest.mark.parametrize("iters", [1, 6])
def test_rope_adjoint_matches_oracle(cuda_lib, iters):
    """One pass pair (the reference's PBDRope.update) and six (the adjoint recomputes the pass inputs
    into the dt_world.r_work workspace)."""
    env = SS.rope_under_pad()
    env = env.replace(ropes=[env.ropes[0].replace(iters=iters)])
    rng = np.random.default_rng(4)
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    st0 = o.initial_state()
    st0["rvel"] = [(0.05 * rng.standard_normal(a.shape)).astype(np.float32).astype(np.float64) for a in st0["rvel"]]
    st0["vel"] = [(0.01 * rng.standard_normal(a.shape)).astype(np.float32).astype(np.float64) for a in st0["vel"]]
    W = {k: [rng.standard_normal(a.shape) for a in st0[k]] for k in ("pos", "vel", "vpos", "rpos", "rvel")}
    adj1 = {"x": np.zeros((0, 3)), "v": np.zeros((0, 3)), "C": np.zeros((0, 3, 3)), "F": np.zeros((0, 3, 3))}
    adj1.update(W)
    ref = o.substep_bwd(st0, adj1)

    w = World([env], n_frames=2, dt=DT, grad_clip=0.0)
    sl = w.vslice(0)
    w.t["v_vel"][0, sl, :3] = torch.as_tensor(st0["vel"][0], dtype=torch.float32, device=w.device)
    w.set_rope_state(0, 0, vel=st0["rvel"][0])
    w.step_begin()
    w.substep(0)
    w.adj_clear()
    for name, k in (("v_adj_pos", "pos"), ("v_adj_vel", "vel"), ("v_adj_vpos", "vpos")):
        w.t[name][1, sl, :3] = torch.as_tensor(W[k][0], dtype=torch.float32, device=w.device)
    w.set_rope_adjoint(1, 0, pos=W["rpos"][0], vel=W["rvel"][0])
    w.substep_bwd(0)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    ra = w.rope_adjoint(0, 0)
    errs = {"rpos": SS.rel_err(ra["pos"].cpu().numpy(), ref["rpos"][0]),
            "rvel": SS.rel_err(ra["vel"].cpu().numpy(), ref["rvel"][0]),
            "pos": SS.rel_err(w.t["v_adj_pos"][0, sl, :3].cpu().numpy(), ref["pos"][0]),
            "vel": SS.rel_err(w.t["v_adj_vel"][0, sl, :3].cpu().numpy(), ref["vel"][0])}
    assert max(errs.values()) < 1e-3, errs


def test_rope_argmin_on_a_large_pad(cuda_lib):
    """A 40x40 pad (3,200 surface triangles, 100 groups of centroids: the per-CTA candidate search)
    over a 48-particle rope: argmin bit-exact and state as the oracle's."""
    env = SS.rope_under_pad(n_rope=48, pad=(40, 40, 2))
    assert len(env.sensors[0].tris) > 32 * 32
    cv = [SS.control_velocity(sp, scale=0.02, down=-0.05) for sp in env.sensors]
    n_sub = 2
    w = run_gpu([env], n_sub, cv)
    st, dbgs = oracle_run(env, n_sub, cv)
    for f, d in enumerate(dbgs):
        cid = w.t["r_cidx"][f, :, 0].cpu().numpy()
        assert np.array_equal(cid, d["rope_cidx"][0][:, 0]), f
    rs = {k: v.cpu().numpy() for k, v in w.rope_state(n_sub, 0).items()}
    assert SS.rel_err(rs["pos"], st["rpos"][0]) < 1e-5


def test_rope_iterations_forward_match_the_oracle(cuda_lib):
    """50 pass pairs per substep (configuration 5's solver) over three substeps under the pad: state as
    the oracle's, and the stretch constraints closer to their rest length than with one pair."""
    env = SS.rope_under_pad(n_rope=40)
    cv = [SS.control_velocity(sp, scale=0.02, down=-0.05) for sp in env.sensors]
    res = {}
    for iters in (1, 50):
        e = env.replace(ropes=[env.ropes[0].replace(iters=iters)])
        w = run_gpu([e], 3, cv)
        st, _ = oracle_run(e, 3, cv)
        rs = {k: v.cpu().numpy() for k, v in w.rope_state(3, 0).items()}
        assert SS.rel_err(rs["pos"], st["rpos"][0]) < 1e-5, iters
        assert SS.rel_err(rs["vel"], st["rvel"][0]) < 1e-3, iters
        L = np.linalg.norm(np.diff(rs["pos"], axis=0), axis=1)[1:]
        res[iters] = float(np.abs(L - e.ropes[0].rest).max())
    assert res[50] < res[1], res
