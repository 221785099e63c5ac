"""Gripper-driven rollouts on the GPU: a box squeezed between the two finger sensors of a
parallel-jaw gripper (gripper_kinematics.py, per-substep finger control velocities, set_sensor_vel
at every step start).  The full-tape and checkpointed sweeps agree; d loss / d actions matches the
oracle's float64 adjoint composed through the same rollout within 2e-3 relative (norm), and central
finite differences (eps 1e-4: contact flags switch as the pads slide, so the loss is only piecewise
smooth and larger steps cross kinks) within 5e-3 per direction."""
import numpy as np
import pytest
import torch

from difftactile_gb300.trajectory import GripperTrajectory, Trajectory
from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4
T_STEPS, SUB = 3, 4


def setup():
    env, kin = SS.gripper_box()
    rng = np.random.default_rng(12)
    terms = tuple((s, int(sp.layer.max()), 1e-4 * rng.standard_normal(sp.verts.shape))
                  for s, sp in enumerate(env.sensors))
    return env, kin, terms


def actions(seed=6):
    rng = np.random.default_rng(seed)
    a = np.zeros((T_STEPS, 7))
    a[:, 0:3] = 0.05 * rng.standard_normal((T_STEPS, 3))
    a[:, 3:6] = 20.0 * rng.standard_normal((T_STEPS, 3))
    a[:, 6] = 0.2 + 0.05 * rng.standard_normal(T_STEPS)
    return a


def gpu_rollout(env, kin, terms, acts, ckpt_every):
    nf = Trajectory.frames_needed(T_STEPS, SUB, ckpt_every)
    w = World([env], n_frames=nf, dt=DT, grad_clip=0.0)
    tr = GripperTrajectory(w, T_STEPS, kin, (0, 1), ckpt_every, terms)
    loss = float(tr.forward(torch.as_tensor(acts, dtype=torch.float64, device=w.device)).item())
    g = tr.backward().cpu().numpy()
    torch.cuda.synchronize()
    assert w.error_word() == 0
    return loss, g


def finger_cvs(env, kin, acts_t):
    """Per step and finger, the control velocities of frames 0..S (frame S zero)."""
    F = kin.rollout(acts_t, SUB)
    T0i = [torch.linalg.inv(f) for f in kin.finger_poses0()]
    rest = [torch.cat([torch.as_tensor(sp.verts.astype(np.float32), dtype=torch.float64),
                       torch.ones((len(sp.verts), 1), dtype=torch.float64)], 1) for sp in env.sensors]
    out = []
    for t in range(T_STEPS):
        per = []
        for i in range(2):
            c = [((F[t, i, f + 1] - F[t, i, f]) @ T0i[i] @ rest[i].T).T[:, :3] / DT for f in range(SUB)]
            c.append(torch.zeros_like(c[0]))
            per.append(c)
        out.append(per)
    return out


def loss_grad_state(env, terms, st):
    g = {"pos": [np.zeros_like(a) for a in st["pos"]], "vpos": [np.zeros_like(a) for a in st["vpos"]]}
    for s, layer, tg in terms:
        sel = env.sensors[s].layer == layer
        d = st["pos"][s] - st["vpos"][s] - tg
        g["pos"][s][sel] += 2 * d[sel]
        g["vpos"][s][sel] -= 2 * d[sel]
    return g


def oracle_grad(env, kin, terms, acts):
    """d loss / d actions from the oracle's float64 adjoint substeps, chained through the
    kinematics with torch autograd."""
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    a = torch.as_tensor(acts, dtype=torch.float64).requires_grad_(True)
    cvt = finger_cvs(env, kin, a)
    cv = [[[c.detach().numpy() for c in cvt[t][i]] for i in range(2)] for t in range(T_STEPS)]
    st = o.initial_state()
    tape = []
    for t in range(T_STEPS):
        st["vel"] = [cv[t][0][0].copy(), cv[t][1][0].copy()]
        for f in range(SUB):
            tape.append((t, f, {k: (v if not isinstance(v, list) else [x.copy() for x in v]) for k, v in st.items()}))
            st, _ = o.substep(st, cv=[cv[t][0][f], cv[t][1][f]], cv1=[cv[t][0][f + 1], cv[t][1][f + 1]])
    g = loss_grad_state(env, terms, st)
    N_ = env.n_particles
    adj = {"x": np.zeros((N_, 3)), "v": np.zeros((N_, 3)), "C": np.zeros((N_, 3, 3)), "F": np.zeros((N_, 3, 3)),
           "pos": g["pos"], "vel": [np.zeros_like(x) for x in g["pos"]], "vpos": g["vpos"]}
    cvb = [[[np.zeros_like(c) for c in cv[t][i]] for i in range(2)] for t in range(T_STEPS)]
    for t, f, st_f in reversed(tape):
        out = o.substep_bwd(st_f, adj, cv=[cv[t][0][f], cv[t][1][f]], cv1=[cv[t][0][f + 1], cv[t][1][f + 1]])
        for i in range(2):
            cvb[t][i][f] += out["cv"][i]
            cvb[t][i][f + 1] += out["cv1"][i]
        adj = {k: out[k] for k in ("x", "v", "C", "F", "pos", "vel", "vpos")}
        if f == 0:  # set_sensor_vel(0): the overwritten velocity gets no adjoint
            for i in range(2):
                cvb[t][i][0] += adj["vel"][i]
                adj["vel"][i] = np.zeros_like(adj["vel"][i])
    outs = [cvt[t][i][f] for t in range(T_STEPS) for i in range(2) for f in range(SUB)]
    bars = [torch.as_tensor(cvb[t][i][f]) for t in range(T_STEPS) for i in range(2) for f in range(SUB)]
    (ga,) = torch.autograd.grad(outs, a, bars)
    return ga.numpy()


def oracle_loss(env, kin, terms, acts):
    o = O.Oracle(env, DT, np.float64)
    st = o.initial_state()
    cvt = finger_cvs(env, kin, torch.as_tensor(acts, dtype=torch.float64))
    for t in range(T_STEPS):
        cvs = [[c.numpy() for c in cvt[t][i]] for i in range(2)]
        st["vel"] = [cvs[0][0].copy(), cvs[1][0].copy()]  # set_sensor_vel(0)
        for f in range(SUB):
            st, _ = o.substep(st, cv=[cvs[0][f], cvs[1][f]], cv1=[cvs[0][f + 1], cvs[1][f + 1]])
    L = 0.0
    for s, layer, tg in terms:
        sel = env.sensors[s].layer == layer
        d = st["pos"][s] - st["vpos"][s] - tg
        L += float((d[sel] ** 2).sum())
    return L


def test_gripper_full_tape_matches_checkpoints():
    env, kin, terms = setup()
    a = actions()
    lf, gf = gpu_rollout(env, kin, terms, a, 0)
    for k in (1, 2):
        lk, gk = gpu_rollout(env, kin, terms, a, k)
        assert abs(lk - lf) <= 1e-5 * abs(lf), (k, lk, lf)
        assert SS.rel_err(gk, gf) < 1e-4, k


def test_gripper_action_gradient_vs_oracle():
    env, kin, terms = setup()
    a = actions()
    loss, g = gpu_rollout(env, kin, terms, a, 0)
    L0 = oracle_loss(env, kin, terms, a)
    assert abs(loss - L0) <= 1e-3 * abs(L0), (loss, L0)
    go = oracle_grad(env, kin, terms, a)
    assert SS.rel_err(g, go) < 2e-3
    rng = np.random.default_rng(9)
    for trial in range(3):
        d = rng.standard_normal(a.shape)
        d[:, 3:6] *= 100.0
        eps = 1e-4
        fd = (oracle_loss(env, kin, terms, a + eps * d) - oracle_loss(env, kin, terms, a - eps * d)) / (2 * eps)
        pred = float((g * d).sum())
        assert abs(pred - fd) <= 5e-3 * abs(fd) + 1e-12, (trial, pred, fd)
