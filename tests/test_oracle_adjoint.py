"""The oracle's adjoint substep (float64) against central finite differences of its forward
substep, on random directions over every input group, for each material model and on the other
parity scenes (two pads, the dome, the gripper, the sticky floor, a three-substep chain)."""
import numpy as np
import pytest

from difftactile_gb300 import scene as S
from oracle import oracle as O
from tests import small_scenes as SS
from tests import test_parity_bwd as T


@pytest.mark.parametrize("model,ys", [(0, 50.0), (1, 2.0), (2, 50.0)])
def test_oracle_adjoint_matches_finite_differences(model, ys):
    env = SS.pad_over_box(model=model, yield_stress=ys)
    st0, cv = T.base_point(env, 3)
    W = T.loss_weights(env, env.n_particles, 4)
    o = O.Oracle(env, T.DT, np.float64, grad_clip=0.0)
    adj = o.substep_bwd({k: (v if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}, W,
                        cv=cv, cv1=cv)
    g = {k: adj[k] for k in ("x", "v", "C", "F", "pos", "vel", "vpos")}
    g["cv"] = [a + b for a, b in zip(adj["cv"], adj["cv1"])]
    g["mu"], g["lam"] = adj["mat"][0]
    bad = []
    for i, groups in enumerate([(k,) for k in T.GROUPS] + [T.GROUPS]):
        pred, fd = T.directional(env, st0, cv, W, g, 1, groups, seed=100 + i)
        rel = abs(pred - fd) / max(abs(fd), 1e-12)
        if rel > 1e-5:
            bad.append((groups, pred, fd, rel))
    assert not bad, bad


def _scene(name):
    if name == "two_pads":
        return SS.pad_over_box(two_pads=True), 1
    if name == "dome":
        return SS.dome_over_box(), 1
    if name == "gripper":
        return SS.gripper_box()[0], 1
    if name == "sticky_floor":  # cube resting in the floor band: sticky-floor nodes (grid_op's floor rule)
        return SS.elastic_cube(center=(0.5, 4.5 / 32, 0.5), v=(0.0, -0.5, 0.0), bc=S.BC_STICKY_FLOOR), 1
    if name == "pad_3_substeps":
        return SS.pad_over_box(yield_stress=50.0), 3
    if name == "linear_corotated_pad":  # the pad's elastomer with the linear corotated force
        import dataclasses
        env = SS.pad_over_box()
        return env.replace(sensors=[dataclasses.replace(env.sensors[0], model=S.FEM_LINEAR_COROTATED)]), 2
    raise KeyError(name)


@pytest.mark.parametrize("name", ["two_pads", "dome", "gripper", "sticky_floor", "pad_3_substeps",
                                  "linear_corotated_pad"])
def test_oracle_adjoint_matches_finite_differences_per_scene(name):
    """The same check on the other parity scenes: two pads in one environment, the reference's dome
    (unordered triangles, tilted contact normal), the gripper's two finger pads, a cube on the sticky
    floor, a three-substep chain (the adjoint carried through the per-frame grid and sensor state) and the
    pad with the linear corotated elastomer force."""
    env, n_sub = _scene(name)
    if env.v is None:
        env = env.replace(v=np.zeros_like(env.x))
    st0, cv = T.base_point(env, 5)
    W = T.loss_weights(env, env.n_particles, 6)
    o = O.Oracle(env, T.DT, np.float64, grad_clip=0.0)
    st = {k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}
    sts = [st]
    for _ in range(n_sub - 1):
        st, _ = o.substep({k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v])
                           for k, v in st.items()}, cv=cv, cv1=cv)
        sts.append(st)
    g = {k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v]) for k, v in W.items()}
    g["cv"] = [np.zeros_like(a) for a in cv]
    g["mu"] = g["lam"] = 0.0
    for i in reversed(range(n_sub)):
        Wi = {k: g[k] for k in ("x", "v", "C", "F", "pos", "vel", "vpos")}
        stc = {k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v]) for k, v in sts[i].items()}
        adj = o.substep_bwd(stc, Wi, cv=cv, cv1=cv)
        cvs = [c + a + b for c, a, b in zip(g["cv"], adj["cv"], adj["cv1"])]
        mu, lam = g["mu"] + adj["mat"][0][0], g["lam"] + adj["mat"][0][1]
        g = {k: adj[k] for k in ("x", "v", "C", "F", "pos", "vel", "vpos")}
        g["cv"], g["mu"], g["lam"] = cvs, mu, lam
    groups = [(k,) for k in T.GROUPS if env.sensors or k not in ("pos", "vel", "vpos", "cv")] + [T.GROUPS]
    bad = []
    for i, gr in enumerate(groups):
        # small steps: the dome's contact set changes within 1e-3 of the state directions (a vertex
        # crossing the contact band); a 1e-6 relative step of mu or lambda moves the loss by ~1e-9 of
        # its size, within reach of its float64 rounding, so those step further (the stress is
        # linear in both)
        eps = 1e-3 if gr in (("mu",), ("lam",)) else 1e-5
        pred, fd = T.directional(env, st0, cv, W, g, n_sub, gr, seed=200 + i, eps=eps)
        rel = abs(pred - fd) / max(abs(fd), 1e-12)
        if rel > 1e-5:
            bad.append((gr, pred, fd, rel))
    assert not bad, bad


def test_oracle_multithreaded_forward_matches_sequential():
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    a = O.Oracle(env, T.DT, np.float64, n_threads=1)
    b = O.Oracle(env, T.DT, np.float64, n_threads=4)
    sa, _ = a.substep(a.initial_state(), cv=cv, cv1=cv)
    sb, _ = b.substep(b.initial_state(), cv=cv, cv1=cv)
    for k in ("x", "v", "C", "F"):
        assert SS.rel_err(sb[k], sa[k]) < 1e-12


def test_return_map_adjoint_is_stable_at_coinciding_singular_values():
    """Compressed plastic material (a pad pressing a box of yield stress 2 for 16 substeps: most
    particles have two singular values of F_new within 0.1% of each other): with the divided-
    difference form of the return map's rotation adjoint (svd_grad_mode 0) the float32 adjoint
    agrees with the float64 one to 1e-4; the reference's generic formula (mode 1) amplifies float32
    rounding there by orders of magnitude more."""
    from oracle import oracle as O
    from tests.test_parity_bwd import loss_weights
    dt = 1e-4
    env = SS.pad_over_box(yield_stress=2.0)
    cv = [SS.control_velocity(sp, down=-0.3) for sp in env.sensors]
    o32 = O.Oracle(env, dt, np.float32, grad_clip=0.0)
    st = o32.initial_state()
    for _ in range(16):
        st, _ = o32.substep(st, cv=cv, cv1=cv)
    st = {k: (v.astype(np.float64) if not isinstance(v, list) else [a.astype(np.float64) for a in v])
          for k, v in st.items()}
    W = {k: v.astype(np.float32).astype(np.float64)
         for k, v in loss_weights(env, env.n_particles, 31).items() if k in ("x", "v", "C", "F")}
    err = {}
    for mode in (0, 1):
        r64 = O.Oracle(env, dt, np.float64, grad_clip=0.0).substep_bwd(st, W, cv=cv, cv1=cv, svd_grad_mode=mode)
        r32 = O.Oracle(env, dt, np.float32, grad_clip=0.0).substep_bwd(st, W, cv=cv, cv1=cv, svd_grad_mode=mode)
        err[mode] = SS.rel_err(r32["F"], r64["F"])
    assert err[0] < 1e-4, err
    assert err[1] > 10 * err[0], err
