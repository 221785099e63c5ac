"""The oracle's adjoint substep (float64) against central finite differences of its forward
substep, on random directions over every input group, for each material model."""
import numpy as np
import pytest

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


def test_oracle_multithreaded_forward_matches_sequential():
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    a = O.Oracle(env, T.DT, np.float64, n_threads=1)
    b = O.Oracle(env, T.DT, np.float64, n_threads=4)
    sa, _ = a.substep(a.initial_state(), cv=cv, cv1=cv)
    sb, _ = b.substep(b.initial_state(), cv=cv, cv1=cv)
    for k in ("x", "v", "C", "F"):
        assert SS.rel_err(sb[k], sa[k]) < 1e-12
