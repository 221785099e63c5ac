"""Golden directional derivatives of the reference's own substep.

The reference's gradients are Taichi autodiff, which cannot run here; central differences of its
own forward methods stand in for them.  The grasp task's Contact.update (the plastic_pads case of
make_substep.py: von Mises box, two hex pads, contact) is run in float64 through the stand-in `ti`
module of this folder from perturbed copies of a seeded state, and the derivative of a seeded
linear loss of the next frame (particles x, v, C, F and both pads' pos, vel, virtual pos) is taken
along seeded directions of each input group (particle state, pad state, control velocities, the
material's mu and lambda) and of all of them at once; likewise the cable task's Contact.update (the
rope_pads case: PBD rope under a gripper pad) along the rope's and the pads' state and both frames'
control velocities.  Derivatives go to tests/golden/gradient_ref.npz (the directions are rebuilt from
their seeds).

    python tests/golden/make_gradient.py REFERENCE_ROOT
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.refroot import reference_root  # noqa: E402

from difftactile_gb300 import scene as S  # noqa: E402
from tests.golden import make_substep as MS  # noqa: E402

GROUPS = ("x", "v", "C", "F", "pos", "vel", "vpos", "cv", "mu", "lam")
SCALE = {"x": 2e-4, "v": 1e-2, "C": 1e-1, "F": 1e-3, "pos": 2e-4, "vel": 1e-2, "vpos": 1e-3, "cv": 1e-2}
EPS = 1e-5


def base():
    """Scene, state and loss weights of the fixture (also rebuilt by tests/test_golden_gradient.py)."""
    env = MS.scenes()["plastic_pads"]
    st = MS.seeded_state(env, seed=6, jitter=0.02 * env.dx)
    rng = np.random.default_rng(12)
    N = env.n_particles
    W = {"x": rng.standard_normal((N, 3)), "v": rng.standard_normal((N, 3)), "C": 1e-2 * rng.standard_normal((N, 3, 3)),
         "F": rng.standard_normal((N, 3, 3))}
    for k in ("pos", "vel", "vpos"):
        W[k] = [rng.standard_normal(sp.verts.shape) for sp in env.sensors]
    return env, st, W


def directions(env, st, seed):
    """One seeded direction per group and one over all groups."""
    out = []
    mu0, lam0 = env.materials[0].mu_lam
    for i, gr in enumerate([(k,) for k in GROUPS] + [GROUPS]):
        rng = np.random.default_rng(seed + i)
        d = {k: (SCALE[k] * rng.standard_normal(st[k].shape) if k in gr else np.zeros_like(st[k]))
             for k in ("x", "v", "C", "F")}
        for k in ("pos", "vel", "vpos", "cv"):
            d[k] = [SCALE[k] * rng.standard_normal(a.shape) if k in gr else np.zeros_like(a) for a in st[k]]
        d["mu"] = 1e-2 * mu0 * rng.standard_normal() if "mu" in gr else 0.0
        d["lam"] = 1e-2 * lam0 * rng.standard_normal() if "lam" in gr else 0.0
        out.append((gr, d))
    return out


def loss(env, st, W, d, h):
    """The loss after one reference substep from st + h d."""
    m = env.materials[0]
    mu, lam = m.mu_lam
    e = env.replace(materials=[S.Material(m.E, m.nu, m.yield_stress, m.model, mu=mu + h * d["mu"],
                                          lam=lam + h * d["lam"])])
    s = {k: st[k] + h * d[k] for k in ("x", "v", "C", "F")}
    for k in ("pos", "vel", "vpos", "cv"):
        s[k] = [a + h * b for a, b in zip(st[k], d[k])]
    o, sens, _ = MS.run_pads(e, s)
    L = sum(float((W[k] * getattr(o, f).a[1]).sum()) for k, f in (("x", "x_0"), ("v", "v_0"), ("C", "C_0"), ("F", "F_0")))
    for k, f in (("pos", "pos"), ("vel", "vel"), ("vpos", "virtual_pos")):
        L += sum(float((w * getattr(so, f).a[1]).sum()) for w, so in zip(W[k], sens))
    return L


ROPE_GROUPS = ("rpos", "rvel", "pos", "vel", "vpos", "cv", "cv1")
ROPE_SCALE = {"rpos": 2e-4, "rvel": 1e-2, "pos": 2e-4, "vel": 1e-2, "vpos": 1e-3, "cv": 1e-2, "cv1": 1e-2}


def rope_base():
    """The cable case (rope_pads of make_substep.py), its state and loss weights of the next frame
    (rope pos, vel; both gripper pads' pos, vel, virtual pos)."""
    env = MS.scenes()["rope_pads"]
    st = MS.seeded_state(env, seed=7, jitter=0.02 * 0.012)
    rng = np.random.default_rng(13)
    W = {"rpos": [rng.standard_normal((rp.n, 3)) for rp in env.ropes],
         "rvel": [rng.standard_normal((rp.n, 3)) for rp in env.ropes]}
    for k in ("pos", "vel", "vpos"):
        W[k] = [rng.standard_normal(sp.verts.shape) for sp in env.sensors]
    return env, st, W


def rope_directions(st, seed):
    out = []
    for i, gr in enumerate([(k,) for k in ROPE_GROUPS] + [ROPE_GROUPS]):
        rng = np.random.default_rng(seed + i)
        out.append((gr, {k: [ROPE_SCALE[k] * rng.standard_normal(a.shape) if k in gr else np.zeros_like(a)
                             for a in st[k]] for k in ROPE_GROUPS}))
    return out


def rope_loss(env, st, W, d, h):
    s = dict(st)
    for k in ROPE_GROUPS:
        s[k] = [a + h * b for a, b in zip(st[k], d[k])]
    ro, sens, _ = MS.run_rope(env, s)
    L = float((W["rpos"][0] * ro.pos.a[1]).sum()) + float((W["rvel"][0] * ro.vel.a[1]).sum())
    for k, f in (("pos", "pos"), ("vel", "vel"), ("vpos", "virtual_pos")):
        L += sum(float((w * getattr(so, f).a[1]).sum()) for w, so in zip(W[k], sens))
    return L


def main():
    MS.PKG = os.path.join(reference_root(), "difftactile")
    env, st, W = base()
    fd = []
    for gr, d in directions(env, st, seed=300):
        # step EPS along the direction; mu or lambda alone move one substep's loss so little that a
        # step that short meets the loss's float64 rounding, so those step 1e-3 (the stress is linear
        # in both)
        h = 1e-3 if gr in (("mu",), ("lam",)) else EPS
        fd.append((loss(env, st, W, d, h) - loss(env, st, W, d, -h)) / (2 * h))
    env, st, W = rope_base()
    fd_rope = [(rope_loss(env, st, W, d, EPS) - rope_loss(env, st, W, d, -EPS)) / (2 * EPS)
               for gr, d in rope_directions(st, seed=400)]
    np.savez_compressed(os.path.join(HERE, "gradient_ref.npz"), fd=np.array(fd), fd_rope=np.array(fd_rope))
    print(np.array(fd), np.array(fd_rope))


if __name__ == "__main__":
    main()
