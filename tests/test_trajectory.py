"""Trajectory-level gradients: pose-controlled rollouts of several control steps, actions ->
step transforms -> per-vertex control velocities -> substeps -> marker loss, and back.

* the full-tape sweep (no recompute) and the checkpointed sweeps (k = 1, 2) agree;
* d loss / d actions from the CUDA adjoint matches central finite differences of a float64
  restatement of the same rollout on the oracle (pose control as in set_pose_control +
  set_control_vel, fem_sensor.py:229-266), within 2e-3 relative per direction;
* the same for the cable task's rope-tip loss (a rope of five stretch + bending pass pairs per
  substep under the pad), full tape and checkpointed.
"""
import numpy as np
import pytest
import torch

from difftactile_gb300 import scene as S
from difftactile_gb300.trajectory import PoseTrajectory
from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4
T_STEPS, SUB = 3, 4


def scene():
    env = SS.pad_over_box(n=32)
    sp = env.sensors[0]
    rng = np.random.default_rng(21)
    target = 1e-4 * rng.standard_normal(sp.verts.shape)
    return env, ((0, int(sp.layer.max()), target),)


def actions(seed=5):
    rng = np.random.default_rng(seed)
    a = np.zeros((T_STEPS, 1, 6))
    a[:, 0, 1] = -0.2
    a[:, 0, :3] += 0.05 * rng.standard_normal((T_STEPS, 3))
    a[:, 0, 3:] += 20.0 * rng.standard_normal((T_STEPS, 3))  # degrees per second
    return a


def gpu_rollout(env, terms, acts, ckpt_every):
    nf = PoseTrajectory.frames_needed(T_STEPS, SUB, ckpt_every)
    w = World([env], n_frames=nf, dt=DT, grad_clip=0.0)
    tr = PoseTrajectory(w, T_STEPS, ckpt_every, terms)
    loss = float(tr.forward(torch.as_tensor(acts, dtype=torch.float64, device=w.device)).item())
    g = tr.backward().cpu().numpy()
    torch.cuda.synchronize()
    assert w.error_word() == 0
    return loss, g


def oracle_loss(env, terms, acts, rope_terms=()):
    o = O.Oracle(env, DT, np.float64)
    st = o.initial_state()
    inv_T = 1.0 / (DT * SUB)
    for t in range(T_STEPS):
        cv = []
        for s, sp in enumerate(env.sensors):
            a = acts[t, s]
            M = S.eul2mat_zyx(a[3:6] * DT * SUB, a[0:3] * DT * SUB)
            TW = sp.trans_world if sp.trans_world is not None else np.eye(4)
            D = TW @ M @ np.linalg.inv(TW)
            p = st["vpos"][s]
            cv.append(((p @ D[:3, :3].T + D[:3, 3]) - p) * inv_T)
        for _ in range(SUB):
            st, _ = o.substep(st, cv=cv, cv1=cv)
    L = 0.0
    for s, layer, tg in terms:
        sel = env.sensors[s].layer == layer
        d = st["pos"][s] - st["vpos"][s] - tg
        L += float((d[sel] ** 2).sum())
    for r, tg in rope_terms:
        L += float(((st["rpos"][r][-1] - tg) ** 2).sum())
    return L


def test_full_tape_matches_checkpoints():
    env, terms = scene()
    a = actions()
    lf, gf = gpu_rollout(env, terms, a, 0)
    for k in (1, 2):
        lk, gk = gpu_rollout(env, terms, a, k)
        assert abs(lk - lf) <= 1e-5 * abs(lf), (k, lk, lf)
        assert SS.rel_err(gk, gf) < 1e-4, k


def test_action_gradient_vs_oracle_fd():
    env, terms = scene()
    a = actions()
    loss, g = gpu_rollout(env, terms, a, 0)
    L0 = oracle_loss(env, terms, a)
    assert abs(loss - L0) <= 1e-3 * abs(L0), (loss, L0)
    rng = np.random.default_rng(8)
    for trial in range(3):
        d = rng.standard_normal(a.shape)
        d[..., 3:] *= 100.0  # rotations are in degrees per second: probe them at a comparable scale
        eps = 1e-3
        fd = (oracle_loss(env, terms, a + eps * d) - oracle_loss(env, terms, a - eps * d)) / (2 * eps)
        pred = float((g * d).sum())
        assert abs(pred - fd) <= 2e-3 * abs(fd) + 1e-12, (trial, pred, fd)


def test_rope_tip_loss_gradient_vs_oracle_fd():
    """The cable task's loss, the rope tip's squared distance from a target, through five pass pairs of
    the PBD solver per substep: checkpointed (k = 1) and full-tape sweeps agree, and d loss / d actions
    matches central finite differences of the oracle's float64 rollout (2e-3 per direction)."""
    env = SS.rope_under_pad(n_rope=16)
    env = env.replace(ropes=[env.ropes[0].replace(iters=5)])
    tip = env.ropes[0].init_positions()[-1].astype(np.float64)
    rope_terms = ((0, tip + np.array([0.003, 0.002, -0.001])),)
    a = actions()
    a[:, 0, 1] = 0.2  # +y: the pad's out-direction, onto the rope
    res = {}
    for k in (0, 1):
        nf = PoseTrajectory.frames_needed(T_STEPS, SUB, k)
        w = World([env], n_frames=nf, dt=DT, grad_clip=0.0)
        tr = PoseTrajectory(w, T_STEPS, k, (), rope_terms=rope_terms)
        loss = float(tr.forward(torch.as_tensor(a, dtype=torch.float64, device=w.device)).item())
        g = tr.backward().cpu().numpy()
        torch.cuda.synchronize()
        assert w.error_word() == 0
        res[k] = (loss, g)
    assert abs(res[1][0] - res[0][0]) <= 1e-5 * abs(res[0][0])
    assert SS.rel_err(res[1][1], res[0][1]) < 1e-4
    loss, g = res[0]
    L0 = oracle_loss(env, (), a, rope_terms)
    assert abs(loss - L0) <= 1e-3 * abs(L0), (loss, L0)
    assert np.abs(g).sum() > 0
    rng = np.random.default_rng(8)
    for trial in range(3):
        d = rng.standard_normal(a.shape)
        d[..., 3:] *= 100.0
        eps = 1e-3
        fd = (oracle_loss(env, (), a + eps * d, rope_terms) - oracle_loss(env, (), a - eps * d, rope_terms)) / (2 * eps)
        pred = float((g * d).sum())
        print("rope tip", trial, pred, fd)
        assert abs(pred - fd) <= 2e-3 * abs(fd) + 1e-12, (trial, pred, fd)
