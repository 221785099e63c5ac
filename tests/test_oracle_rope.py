"""CPU restatement of the PBD rope (PBDRope.update, PBD_rope.py:112-180) and its sensor contact
(cable_straightening.py:288-319): known answers, more solver iterations converging the constraints,
and the hand-written adjoint against central finite differences in float64."""
import numpy as np

from difftactile_gb300 import scene as S
from oracle import oracle as O
from tests import small_scenes as SS

DT = 1e-4


def free_rope(n=8, gravity=(0.0, 0.0, 0.0), table_h=-1.0, x=None):
    rp = S.RopeSpec(n=n, rad=0.01, rho=1000.0, rest_length=0.016, pos=(0.3, 0.5, 0.5), ori=(1.0, 0.0, 0.0),
                    table_h=table_h, gravity=gravity, x=x)
    return S.EnvSpec(x=np.zeros((0, 3), np.float32), materials=[S.Material(5e3, 0.3)], n_grid=(16, 16, 16),
                     dx=1.0 / 16, ropes=[rp])


def test_straight_rope_at_rest_length_stays():
    env = free_rope()
    o = O.Oracle(env, DT, np.float64)
    st = o.initial_state()
    st1, _ = o.substep(st)
    # rest lengths hold up to the float32 rounding of the initial layout (~1e-9)
    assert np.abs(st1["rpos"][0] - st["rpos"][0]).max() < 1e-7
    assert np.abs(st1["rvel"][0]).max() < 1e-3


def test_pinned_node_and_sag_under_gravity():
    env = free_rope(gravity=(0.0, -9.8, 0.0))
    o = O.Oracle(env, DT, np.float64)
    st = o.initial_state()
    for _ in range(5):
        st, _ = o.substep(st)
    p = st["rpos"][0]
    assert np.allclose(p[0], env.ropes[0].init_positions()[0])
    assert (p[1:, 1] < 0.5).all()


def test_floor_removes_normal_velocity_and_damps_tangential():
    x = np.stack([0.3 + 0.016 * np.arange(4), np.full(4, 1e-6), np.full(4, 0.5)], 1).astype(np.float32)
    env = free_rope(n=4, gravity=(0.0, -9.8, 0.0), table_h=0.0, x=x)
    env = env.replace(ropes=[env.ropes[0].replace(v=np.tile([0.1, -0.5, 0.0], (4, 1)))])
    o = O.Oracle(env, DT, np.float64)
    st = o.initial_state()
    st1, _ = o.substep(st)
    v = st1["rvel"][0]
    # straight chain at rest length: no constraint corrections; node 0 pinned
    assert np.allclose(v[1:, 1], 0.0, atol=1e-9)
    assert np.allclose(v[1:, 0], 0.1 * 0.995, rtol=1e-3)  # float32 layout rounding perturbs rest lengths


def test_rope_presses_into_pad_and_pad_feels_it():
    env = SS.rope_under_pad()
    o = O.Oracle(env, DT, np.float64)
    st = o.initial_state()
    st1, dbg = o.substep(st)
    assert (dbg["rope_cidx"][0] >= 0).all()
    assert np.abs(dbg["rope_ext"][0]).sum() > 0
    assert np.abs(dbg["ext"][0]).sum() > 0
    # equal and opposite: rope impulse sum = - dt * total sensor force
    assert np.allclose(dbg["rope_ext"][0].sum(0), -DT * dbg["ext"][0].sum(0), rtol=1e-9, atol=1e-15)
    assert (st1["rtrav"][0][dbg["rope_ext"][0].any(1)] == 1).all()


def _loss(o, st0, W, n_sub):
    st = {k: (v if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}
    for _ in range(n_sub):
        st, _ = o.substep(st)
    L = 0.0
    for k in ("pos", "vel", "vpos", "rpos", "rvel"):
        L += sum(float((a * b).sum()) for a, b in zip(W[k], st[k]))
    return L


import pytest  # noqa: E402


@pytest.mark.parametrize("iters", [1, 4])
def test_rope_adjoint_matches_finite_differences(iters):
    """One stretch + bending pass pair (the reference) and four of them per substep."""
    env = SS.rope_under_pad()
    env = env.replace(ropes=[env.ropes[0].replace(iters=iters)])
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    st0 = o.initial_state()
    rng = np.random.default_rng(3)
    st0["rvel"] = [0.05 * rng.standard_normal(a.shape) for a in st0["rvel"]]
    st0["vel"] = [0.01 * rng.standard_normal(a.shape) for a in st0["vel"]]
    W = {k: [rng.standard_normal(a.shape) for a in st0[k]] for k in ("pos", "vel", "vpos", "rpos", "rvel")}
    # one substep adjoint
    adj1 = {"x": np.zeros((0, 3)), "v": np.zeros((0, 3)), "C": np.zeros((0, 3, 3)), "F": np.zeros((0, 3, 3))}
    for k in ("pos", "vel", "vpos", "rpos", "rvel"):
        adj1[k] = W[k]
    g = o.substep_bwd(st0, adj1)
    for trial in range(4):
        d = {k: [1e-3 * rng.standard_normal(a.shape) for a in st0[k]] for k in ("pos", "vel", "rpos", "rvel")}
        pred = sum(float((ga * da).sum()) for k in d for ga, da in zip(g[k], d[k]))
        eps = 1e-4

        def shifted(sgn):
            st = dict(st0)
            for k in d:
                st[k] = [a + sgn * eps * b for a, b in zip(st0[k], d[k])]
            return _loss(o, st, W, 1)

        fd = (shifted(1) - shifted(-1)) / (2 * eps)
        assert abs(pred - fd) <= 1e-6 * max(abs(fd), 1e-9), (trial, pred, fd)


def test_more_iterations_converge_the_stretch_constraints():
    """A rope stretched by 20% relaxes towards its rest length faster with more pass pairs (the
    compliance-weighted Jacobi passes converge); one pair is the reference's single pass.  The first
    segment is left out: node 0 is put back on its pin after the passes (PBD_rope.py:174-177)."""
    n = 8
    x = np.stack([0.3 + 1.2 * 0.016 * np.arange(n), np.full(n, 0.5), np.full(n, 0.5)], 1).astype(np.float32)
    errs = []
    for iters in (1, 5, 50):
        env = free_rope(n=n, x=x)
        env = env.replace(ropes=[env.ropes[0].replace(iters=iters)])
        st1, _ = O.Oracle(env, DT, np.float64).substep(O.Oracle(env, DT, np.float64).initial_state())
        L = np.linalg.norm(np.diff(st1["rpos"][0], axis=0), axis=1)
        errs.append(float(np.abs(L[1:] - 0.016).max()))
    assert errs[0] > errs[1] > errs[2], errs
