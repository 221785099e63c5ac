"""Adjoint parity: the CUDA backward substeps (through the C ABI) against central finite differences
of the float64 oracle, on random directions over every input of the substep: particle x, v, C, F;
sensor pos, vel, virtual pos; per-frame control velocities; material mu, lambda.

Tolerance: directional derivatives within 1e-3 relative (fp32 adjoint vs fp64 finite differences).
The grasp task's gradient clamp (grasp_plastic.py:192-202) is disabled so that the adjoint is exact.
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
GROUPS = ("x", "v", "C", "F", "pos", "vel", "vpos", "cv", "mu", "lam")
SCALE = {"x": 2e-4, "v": 1e-2, "C": 1e-1, "F": 1e-3, "pos": 2e-4, "vel": 1e-2, "vpos": 1e-3, "cv": 1e-2}


def base_point(env, seed):
    rng = np.random.default_rng(seed)
    N = env.n_particles
    st = {"x": env.x.astype(np.float64), "v": env.v.astype(np.float64),
          "C": 0.3 * rng.standard_normal((N, 3, 3)),
          "F": np.eye(3) + 0.05 * rng.standard_normal((N, 3, 3))}
    st["pos"] = [sp.verts.astype(np.float64) for sp in env.sensors]
    st["vel"] = [0.01 * rng.standard_normal(sp.verts.shape) for sp in env.sensors]
    st["vpos"] = [sp.verts.astype(np.float64) for sp in env.sensors]
    cv = [SS.control_velocity(sp, seed=11 + i).astype(np.float64) for i, sp in enumerate(env.sensors)]
    # round the base point to float32 so that the GPU and the oracle start from the same values
    for k in ("x", "v", "C", "F"):
        st[k] = st[k].astype(np.float32).astype(np.float64)
    for k in ("pos", "vel", "vpos"):
        st[k] = [a.astype(np.float32).astype(np.float64) for a in st[k]]
    cv = [a.astype(np.float32).astype(np.float64) for a in cv]
    return st, cv


def loss_weights(env, n_particles, seed):
    rng = np.random.default_rng(seed)
    W = {"x": rng.standard_normal((n_particles, 3)), "v": rng.standard_normal((n_particles, 3)),
         "C": 1e-2 * rng.standard_normal((n_particles, 3, 3)), "F": rng.standard_normal((n_particles, 3, 3))}
    W["pos"] = [rng.standard_normal(sp.verts.shape) for sp in env.sensors]
    W["vel"] = [rng.standard_normal(sp.verts.shape) for sp in env.sensors]
    W["vpos"] = [rng.standard_normal(sp.verts.shape) for sp in env.sensors]
    return W


def oracle_loss(env, st0, cv, W, n_sub, mu_lam=None):
    if mu_lam is not None:
        m = env.materials[0]
        env = env.replace(materials=[S.Material(m.E, m.nu, m.yield_stress, m.model, mu=mu_lam[0], lam=mu_lam[1])])
    o = O.Oracle(env, DT, np.float64)
    st = {k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}
    for _ in range(n_sub):
        st, _ = o.substep(st, cv=cv, cv1=cv)
    L = sum(float((W[k] * st[k]).sum()) for k in ("x", "v", "C", "F"))
    for k in ("pos", "vel", "vpos"):
        L += sum(float((a * b).sum()) for a, b in zip(W[k], st[k]))
    return L


def gpu_grads(env, st0, cv, W, n_sub, **world_kw):
    world_kw.setdefault("grad_clip", 0.0)
    w = World([env], n_frames=n_sub + 1, dt=DT, **world_kw)
    w.set_particles(0, x=st0["x"], v=st0["v"], C=st0["C"], F=st0["F"])
    for s in range(len(env.sensors)):
        sl = w.vslice(s)
        for name, k in (("v_pos", "pos"), ("v_vel", "vel"), ("v_vpos", "vpos")):
            w.t[name][0, sl, :3] = torch.as_tensor(st0[k][s], dtype=torch.float32, device=w.device)
        w.set_control_velocity(s, cv[s])
    w.step_begin()
    for f in range(n_sub):
        w.substep(f)
    w.adj_clear()
    w.set_particle_adjoint(n_sub, x=W["x"], v=W["v"], C=W["C"], F=W["F"])
    nb = n_sub & 1
    for s in range(len(env.sensors)):
        sl = w.vslice(s)
        for name, k in (("v_adj_pos", "pos"), ("v_adj_vel", "vel"), ("v_adj_vpos", "vpos")):
            w.t[name][nb, sl, :3] = torch.as_tensor(W[k][s], dtype=torch.float32, device=w.device)
    for f in reversed(range(n_sub)):
        w.substep_bwd(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    g = {k: v.double().cpu().numpy() for k, v in w.particle_adjoint(0).items()}
    for name, k in (("v_adj_pos", "pos"), ("v_adj_vel", "vel"), ("v_adj_vpos", "vpos")):
        g[k] = [w.t[name][0, w.vslice(s), :3].double().cpu().numpy() for s in range(len(env.sensors))]
    g["cv"] = [w.t["v_adj_cv"][:, w.vslice(s), :3].double().sum(0).cpu().numpy() for s in range(len(env.sensors))]
    ma = w.t["mat_adj"][0].double().cpu().numpy()
    g["mu"], g["lam"] = ma[0], ma[1]
    return g


def directional(env, st0, cv, W, g, n_sub, groups, seed, eps=1e-4):
    rng = np.random.default_rng(seed)
    mu0, lam0 = env.materials[0].mu_lam
    d = {}
    for k in ("x", "v", "C", "F"):
        d[k] = SCALE[k] * rng.standard_normal(st0[k].shape) if k in groups else np.zeros_like(st0[k])
    for k in ("pos", "vel", "vpos"):
        d[k] = [SCALE[k] * rng.standard_normal(a.shape) if k in groups else np.zeros_like(a) for a in st0[k]]
    d["cv"] = [SCALE["cv"] * rng.standard_normal(a.shape) if "cv" in groups else np.zeros_like(a) for a in cv]
    d["mu"] = 1e-2 * mu0 * rng.standard_normal() if "mu" in groups else 0.0
    d["lam"] = 1e-2 * lam0 * rng.standard_normal() if "lam" in groups else 0.0
    pred = sum(float((g[k] * d[k]).sum()) for k in ("x", "v", "C", "F"))
    for k in ("pos", "vel", "vpos", "cv"):
        pred += sum(float((a * b).sum()) for a, b in zip(g[k], d[k]))
    pred += g["mu"] * d["mu"] + g["lam"] * d["lam"]

    def shifted(sgn):
        st = {k: st0[k] + sgn * eps * d[k] for k in ("x", "v", "C", "F")}
        for k in ("pos", "vel", "vpos"):
            st[k] = [a + sgn * eps * b for a, b in zip(st0[k], d[k])]
        c = [a + sgn * eps * b for a, b in zip(cv, d["cv"])]
        return oracle_loss(env, st, c, W, n_sub, (mu0 + sgn * eps * d["mu"], lam0 + sgn * eps * d["lam"]))

    fd = (shifted(1) - shifted(-1)) / (2 * eps)
    return pred, fd


@pytest.mark.parametrize("model,ys", [(S.MODEL_COROTATED, 50.0), (S.MODEL_VON_MISES, 2.0),
                                      (S.MODEL_NEOHOOKEAN, 50.0)])
def test_adjoint_matches_finite_differences(cuda_lib, model, ys):
    env = SS.pad_over_box(model=model, yield_stress=ys)
    n_sub = 2
    st0, cv = base_point(env, 3)
    W = loss_weights(env, env.n_particles, 4)
    g = gpu_grads(env, st0, cv, W, n_sub)
    failures = []
    for i, groups in enumerate([(k,) for k in GROUPS] + [GROUPS] * 3):
        pred, fd = directional(env, st0, cv, W, g, n_sub, groups, seed=100 + i)
        rel = abs(pred - fd) / max(abs(fd), 1e-9)
        if rel > 1e-3:
            failures.append((groups if len(groups) == 1 else "all", pred, fd, rel))
    assert not failures, failures


@pytest.mark.parametrize("model,ys,fem", [(S.MODEL_COROTATED, 50.0, S.FEM_REFERENCE), (S.MODEL_VON_MISES, 2.0, S.FEM_REFERENCE),
                                          (S.MODEL_VON_MISES, 2.0, S.FEM_LINEAR_COROTATED)])
def test_adjoint_matches_oracle_adjoint(cuda_lib, model, ys, fem):
    """Whole adjoint arrays of one substep against the oracle's float64 adjoint (norm-wise 1e-3), with the
    reference's elastomer force and with the linear corotated one."""
    import dataclasses
    env = SS.pad_over_box(n=40, box_cells=(10, 6, 10), pad=(10, 10, 3), model=model, yield_stress=ys)
    env = env.replace(sensors=[dataclasses.replace(sp, model=fem) for sp in env.sensors])
    st0, cv = base_point(env, 7)
    W = loss_weights(env, env.n_particles, 8)
    g = gpu_grads(env, st0, cv, W, 1)
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    ref = o.substep_bwd({k: (v if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}, W,
                        cv=cv, cv1=cv)
    errs = {k: SS.rel_err(g[k], ref[k]) for k in ("x", "v", "C", "F")}
    for k in ("pos", "vel", "vpos"):
        errs[k] = SS.rel_err(g[k][0], ref[k][0])
    errs["cv"] = SS.rel_err(g["cv"][0], ref["cv"][0] + ref["cv1"][0])
    errs["mu"] = abs(g["mu"] - ref["mat"][0, 0]) / abs(ref["mat"][0, 0])
    errs["lam"] = abs(g["lam"] - ref["mat"][0, 1]) / abs(ref["mat"][0, 1])
    assert max(errs.values()) < 1e-3, errs


def test_clamp_grid_fires_and_matches_oracle(cuda_lib):
    """The grasp task's clamp_grid (grasp_plastic.py:192-202: grid_m.grad and the sensors' pos / vel
    grads clipped to +-c in the backward pass) with a clip small enough to fire on most nodes and
    vertices: the clipped CUDA adjoint of one substep against the oracle's float64 adjoint with the same
    clip (norm-wise 1e-3), and far from the unclipped one (the clip changed the result)."""
    env = SS.pad_over_box(n=40, box_cells=(10, 6, 10), pad=(10, 10, 3), model=S.MODEL_VON_MISES, yield_stress=2.0)
    st0, cv = base_point(env, 7)
    W = loss_weights(env, env.n_particles, 8)
    clip = 0.05
    g = gpu_grads(env, st0, cv, W, 1, grad_clip=clip)
    g0 = gpu_grads(env, st0, cv, W, 1, grad_clip=0.0)
    copy = lambda: {k: (v if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}  # noqa: E731
    ref = O.Oracle(env, DT, np.float64, grad_clip=clip).substep_bwd(copy(), W, cv=cv, cv1=cv)
    errs = {k: SS.rel_err(g[k], ref[k]) for k in ("x", "v", "C", "F")}
    for k in ("pos", "vel", "vpos"):
        errs[k] = SS.rel_err(g[k][0], ref[k][0])
    changed = {"x": SS.rel_err(g["x"], g0["x"])}
    changed["pos"] = SS.rel_err(g["pos"][0], g0["pos"][0])
    print("clipped vs oracle", errs, "clipped vs unclipped", changed)
    assert max(errs.values()) < 1e-3, errs
    assert min(changed.values()) > 1e-2, changed


def test_multi_substep_backward_equals_substep_sequence(cuda_lib):
    """dt_substeps_bwd (restores fused into the previous stage 3) == dt_substep_bwd per substep, on
    one forward tape; the bound is ten times the run-to-run spread of two unfused sweeps (atomic
    accumulation order), at least 1e-6."""
    env = SS.pad_over_box()
    n_sub = 4
    st0, cv = base_point(env, 5)
    W = loss_weights(env, env.n_particles, 6)
    w = World([env], n_frames=n_sub + 1, dt=DT, grad_clip=0.0)
    w.set_particles(0, x=st0["x"], v=st0["v"], C=st0["C"], F=st0["F"])
    w.set_control_velocity(0, cv[0])
    w.step_begin()
    for f in range(n_sub):
        w.substep(f)
    outs = []
    for fused in (False, False, True):
        w.adj_clear()
        w.set_particle_adjoint(n_sub, x=W["x"], v=W["v"], C=W["C"], F=W["F"])
        if fused:
            w.substeps_bwd(n_sub, 0)
        else:
            for f in reversed(range(n_sub)):
                w.substep_bwd(f)
        torch.cuda.synchronize()
        outs.append({k: v.double().cpu().numpy() for k, v in w.particle_adjoint(0).items()})
    for k in ("x", "v", "C", "F"):
        spread = SS.rel_err(outs[1][k], outs[0][k])
        assert SS.rel_err(outs[2][k], outs[0][k]) <= max(10 * spread, 1e-6), (k, spread)


def test_adjoint_mid_rollout_plastic_state(cuda_lib):
    """One adjoint substep from a mid-rollout state of compressed plastic material (the pad pressing
    a box of yield stress 2 for 16 substeps: every particle yielding, most with two singular values
    of F_new within 0.1% of each other) against the float64 oracle's adjoint of the same substep from
    the same float32 state.  The CUDA return-map adjoint forms the rotation part with divided
    differences, so it stays precise where the generic SVD adjoint's 1 / (s_j^2 - s_i^2) would
    amplify float32 rounding; only particles within 1e-6 of the yield surface (whose branch flips
    under rounding) are excepted.  Tolerance 1e-3 relative on every adjoint."""
    env = SS.pad_over_box(yield_stress=2.0)
    cv = [SS.control_velocity(sp, down=-0.3) for sp in env.sensors]
    n = 16
    w = World([env], n_frames=n + 2, dt=DT, grad_clip=0.0)
    for s, c in enumerate(cv):
        w.set_control_velocity(s, c)
    w.step_begin()
    for f in range(n + 1):
        w.substep(f)
    f = n
    P = w.particles(f)
    st = {k: P[k].double().cpu().numpy() for k in ("x", "v", "C", "F")}
    sl = w.vslice(0)
    fem = lambda name, fr: w.t[name][fr, sl, :3].double().cpu().numpy()  # noqa: E731
    st["pos"], st["vel"], st["vpos"] = [fem("v_pos", f)], [fem("v_vel", f)], [fem("v_vpos", f)]
    W = {k: v.astype(np.float32) for k, v in loss_weights(env, env.n_particles, 31).items() if k in ("x", "v", "C", "F")}
    w.adj_clear()
    w.set_particle_adjoint(f + 1, **W)
    w.substep_bwd(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    g = {k: v.double().cpu().numpy() for k, v in w.particle_adjoint(f).items()}
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    ref = o.substep_bwd(st, {k: W[k].astype(np.float64) for k in W}, cv=[fem("v_cv", f)], cv1=[fem("v_cv", f + 1)])
    m = env.materials[0]
    Fn = (np.eye(3)[None] + DT * st["C"]) @ st["F"]
    eps = np.log(np.maximum(np.linalg.svd(Fn, compute_uv=False), 0.05))
    dgam = np.linalg.norm(eps - eps.mean(1, keepdims=True), axis=1) - m.yield_stress / (2.0 * m.mu_lam[0])
    assert (dgam > 0).mean() > 0.5, "the state should be mostly yielding"
    keep = np.abs(dgam) >= 1e-6
    errs = {k: SS.rel_err(g[k][keep], ref[k][keep]) for k in ("x", "v", "C", "F")}
    assert max(errs.values()) < 1e-3, errs
