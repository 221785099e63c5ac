"""The oracle's adjoint against derivatives of the reference's own substep (tests/golden/
make_gradient.py: central differences of the grasp task's Contact.update, run from the reference
source in float64, along seeded directions of every input group): the oracle's adjoint substep,
contracted with the same directions, gives the same directional derivatives (1e-5 relative).  The
reference's own gradients are Taichi autodiff; differences of its forward are what can run here."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.make_gradient import base, directions
from tests.golden.make_substep import DT

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gradient_ref.npz")


def test_oracle_adjoint_matches_reference_derivatives():
    fd = np.load(GOLDEN)["fd"]
    env, st, W = base()
    cv = st["cv"]
    adj = O.Oracle(env, DT, np.float64, grad_clip=0.0).substep_bwd(
        {k: (st[k] if not isinstance(st[k], list) else list(st[k])) for k in ("x", "v", "C", "F", "pos", "vel", "vpos")},
        W, cv=cv, cv1=cv)
    g = {k: adj[k] for k in ("x", "v", "C", "F", "pos", "vel", "vpos")}
    g["cv"] = [a + b for a, b in zip(adj["cv"], adj["cv1"])]
    g["mu"], g["lam"] = adj["mat"][0]
    ds = directions(env, st, seed=300)
    assert len(ds) == len(fd)
    bad = []
    for (gr, d), ref in zip(ds, fd):
        pred = sum(float((g[k] * d[k]).sum()) for k in ("x", "v", "C", "F"))
        pred += sum(float((a * b).sum()) for k in ("pos", "vel", "vpos", "cv") for a, b in zip(g[k], d[k]))
        pred += g["mu"] * d["mu"] + g["lam"] * d["lam"]
        if abs(pred - ref) > 1e-5 * abs(ref):
            bad.append((gr, pred, ref))
    assert not bad, bad


def test_oracle_rope_adjoint_matches_reference_derivatives():
    """The cable task's substep (PBD rope under a gripper pad, both frames' control velocities)."""
    from tests.golden.make_gradient import ROPE_GROUPS, rope_base, rope_directions
    fd = np.load(GOLDEN)["fd_rope"]
    env, st, W = rope_base()
    z3, z33 = np.zeros((0, 3)), np.zeros((0, 3, 3))
    s = {"x": z3, "v": z3, "C": z33, "F": z33, **{k: st[k] for k in ("pos", "vel", "vpos", "rpos", "rvel", "rtrav")}}
    adj1 = {"x": z3, "v": z3, "C": z33, "F": z33, **W}
    adj = O.Oracle(env, DT, np.float64, grad_clip=0.0).substep_bwd(s, adj1, cv=st["cv"], cv1=st["cv1"])
    ds = rope_directions(st, seed=400)
    assert len(ds) == len(fd)
    bad = []
    for (gr, d), ref in zip(ds, fd):
        pred = sum(float((a * b).sum()) for k in ROPE_GROUPS for a, b in zip(adj[k], d[k]))
        if abs(pred - ref) > 1e-5 * abs(ref):
            bad.append((gr, pred, ref))
    assert not bad, bad
