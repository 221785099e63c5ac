"""Gradients with respect to material parameters through the training API, on the GPU.

- SubstepSegment with the materials' Lame parameters as an input (mpm_elastic.py:64-71,
  multi_obj.py:65-74): d loss / d (mu, lambda) of two materials against central finite differences of
  the float64 oracle (1e-3 relative per direction).
- A reduced configuration 3 (gripper fingers squeezing a sphere of a stiff core and a soft shell,
  GripperTrajectory on a full tape): d loss / d (actions, log E_shell), E_shell through the chain rule of
  mu(E, nu), lambda(E, nu), against central finite differences of the float64 oracle's rollout along 8
  random directions and along log E_shell alone (5e-3 relative: contact flags switch as the pads move,
  so the loss is piecewise smooth).
- The segment's backward refuses frames that another forward overwrote in between.
"""
import numpy as np
import pytest
import torch

from difftactile_gb300 import configs
from difftactile_gb300 import scene as S
from difftactile_gb300.api import simulate
from difftactile_gb300.trajectory import GripperTrajectory, Trajectory
from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4


def two_material_scene():
    env = SS.pad_over_box(n=32, box_cells=(6, 4, 6), yield_stress=2.0)
    mats = [S.Material(5e3, 0.3, 2.0, S.MODEL_VON_MISES), S.Material(2e4, 0.35, 6.0, S.MODEL_VON_MISES)]
    mat = (env.x[:, 0] > np.median(env.x[:, 0])).astype(np.int32)
    return env.replace(materials=mats, mat=mat)


def test_segment_material_gradient_matches_oracle_fd(cuda_lib):
    env = two_material_scene()
    n_sub = 2
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = World([env], n_frames=n_sub + 1, dt=DT, grad_clip=0.0)
    for s, c in enumerate(cv):
        w.set_control_velocity(s, c)
    dev = w.device
    rng = np.random.default_rng(3)
    N = env.n_particles
    x0 = torch.as_tensor(env.x, dtype=torch.float32, device=dev)
    v0 = torch.as_tensor(env.v, dtype=torch.float32, device=dev)
    C0 = torch.as_tensor(0.3 * rng.standard_normal((N, 3, 3)), dtype=torch.float32, device=dev)
    F0 = torch.as_tensor(np.eye(3) + 0.05 * rng.standard_normal((N, 3, 3)), dtype=torch.float32, device=dev)
    sp = env.sensors[0]
    pos = torch.as_tensor(sp.verts, dtype=torch.float32, device=dev)
    vel = torch.zeros_like(pos)
    lame = w.lame_table().requires_grad_(True)
    Wx, Wv, WF = (torch.as_tensor(rng.standard_normal(s), dtype=torch.float64, device=dev)
                  for s in ((N, 3), (N, 3), (N, 3, 3)))
    Wp = torch.as_tensor(rng.standard_normal(pos.shape), dtype=torch.float64, device=dev)
    out = simulate(w, 0, n_sub, x0, v0, C0, F0, pos, vel, pos.clone(), lame)
    L = (Wx * out[0]).sum() + (Wv * out[1]).sum() + (WF * out[3]).sum() + (Wp * out[4]).sum()
    L.backward()
    g = lame.grad.cpu().numpy()
    assert np.isfinite(g).all() and np.abs(g).sum() > 0

    st0 = {"x": env.x.astype(np.float64), "v": env.v.astype(np.float64), "C": C0.double().cpu().numpy(),
           "F": F0.double().cpu().numpy(), "pos": [sp.verts.astype(np.float64)], "vel": [np.zeros(sp.verts.shape)],
           "vpos": [sp.verts.astype(np.float64)]}
    W = {k: a.cpu().numpy() for k, a in (("x", Wx), ("v", Wv), ("F", WF))}
    Wpos = Wp.cpu().numpy()
    base = np.array([m.mu_lam for m in env.materials])

    def oracle_L(ml):
        mats = [S.Material(m.E, m.nu, m.yield_stress, m.model, mu=ml[i, 0], lam=ml[i, 1])
                for i, m in enumerate(env.materials)]
        o = O.Oracle(env.replace(materials=mats), DT, np.float64, grad_clip=0.0)
        st = {k: (v.copy() if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}
        for _ in range(n_sub):
            st, _ = o.substep(st, cv=cv, cv1=cv)
        return float((W["x"] * st["x"]).sum() + (W["v"] * st["v"]).sum() + (W["F"] * st["F"]).sum()
                     + (Wpos * st["pos"][0]).sum())

    failures = []
    for trial in range(4):
        d = rng.standard_normal(base.shape) * 1e-2 * base
        eps = 1e-3
        fd = (oracle_L(base + eps * d) - oracle_L(base - eps * d)) / (2 * eps)
        pred = float((g * d).sum())
        print("lame", trial, pred, fd)
        if abs(pred - fd) > 1e-3 * abs(fd):
            failures.append((trial, pred, fd))
    assert not failures, failures


def test_segment_backward_refuses_overwritten_frames(cuda_lib):
    env = SS.pad_over_box()
    w = World([env], n_frames=5, dt=DT, grad_clip=0.0)
    w.set_control_velocity(0, SS.control_velocity(env.sensors[0]))
    dev = w.device
    N = env.n_particles
    x = torch.as_tensor(env.x, dtype=torch.float32, device=dev).requires_grad_(True)
    v = torch.as_tensor(env.v, dtype=torch.float32, device=dev)
    C = torch.zeros((N, 3, 3), device=dev)
    F = torch.eye(3, device=dev).expand(N, 3, 3).contiguous()
    pos = torch.as_tensor(env.sensors[0].verts, dtype=torch.float32, device=dev)
    z = torch.zeros_like(pos)
    a = simulate(w, 0, 2, x, v, C, F, pos, z, pos)
    # a second segment over frames 1..3 rewrites frames 1 and 2 of the first
    simulate(w, 1, 2, a[0].detach(), a[1].detach(), a[2].detach(), a[3].detach(), a[4], a[5], a[6])
    with pytest.raises(RuntimeError, match="rewritten"):
        a[0].sum().backward()
    # an untouched segment differentiates
    x.grad = None
    b = simulate(w, 0, 2, x, v, C, F, pos, z, pos)
    b[0].sum().backward()
    assert x.grad is not None and torch.isfinite(x.grad).all()


T_STEPS, SUB = 2, 4


def reduced_grasp():
    cfg, kin = configs.grasp_sphere(n_steps=T_STEPS, substeps=SUB, n_grid=32, n_core=250, n_shell=2250,
                                    pad=(4, 4, 2), ckpt_every=0)
    env = cfg.envs[0]
    rng = np.random.default_rng(12)
    terms = tuple((s, int(sp.layer.max()), 1e-4 * rng.standard_normal(sp.verts.shape))
                  for s, sp in enumerate(env.sensors))
    a = np.zeros((T_STEPS, 7))
    a[:, 0:3] = 0.05 * rng.standard_normal((T_STEPS, 3))
    a[:, 3:6] = 20.0 * rng.standard_normal((T_STEPS, 3))
    a[:, 6] = 0.3 + 0.05 * rng.standard_normal(T_STEPS)
    return env, kin, terms, a


def finger_cvs(env, kin, acts_t):
    """Per step and finger the control velocities of frames 0..S (frame S zero), as GripperTrajectory."""
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


def oracle_loss(env, kin, terms, acts, E_shell):
    m0, m1 = env.materials
    env = env.replace(materials=[S.Material(E_shell, m0.nu, m0.yield_stress, m0.model), m1])
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
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


def test_reduced_grasp_sphere_shell_E_gradient_vs_fd(cuda_lib):
    """Configuration 3 in small: d loss / d actions and d loss / d log E_shell (material 0, the shell;
    material 1 is the stiff core) against the float64 oracle's central differences on 8 random
    directions of (actions, log E_shell)."""
    env, kin, terms, a = reduced_grasp()
    E0 = float(env.materials[0].E)
    w = World([env], n_frames=Trajectory.frames_needed(T_STEPS, SUB, 0), dt=DT, grad_clip=0.0)
    tr = GripperTrajectory(w, T_STEPS, kin, (0, 1), 0, terms)
    loss = float(tr.forward(torch.as_tensor(a, dtype=torch.float64, device=w.device)).item())
    ga = tr.backward().cpu().numpy()
    gE = float(tr.material_grad_E_nu()[0, 0])
    torch.cuda.synchronize()
    assert w.error_word() == 0
    L0 = oracle_loss(env, kin, terms, a, E0)
    assert abs(loss - L0) <= 1e-3 * abs(L0), (loss, L0)
    assert gE != 0.0
    rng = np.random.default_rng(5)
    failures = []
    eps = 1e-4
    for trial in range(8):
        da = rng.standard_normal(a.shape)
        da[:, 3:6] *= 100.0
        dl = rng.standard_normal()
        fd = (oracle_loss(env, kin, terms, a + eps * da, E0 * np.exp(eps * dl))
              - oracle_loss(env, kin, terms, a - eps * da, E0 * np.exp(-eps * dl))) / (2 * eps)
        pred = float((ga * da).sum()) + gE * E0 * dl
        print("direction", trial, pred, fd, "E part", gE * E0 * dl)
        if abs(pred - fd) > 5e-3 * abs(fd) + 1e-12:
            failures.append((trial, pred, fd))
    # the shell's modulus alone (along the mixed directions above its share is small)
    for eps_l in (1e-3, 2e-3):
        fd = (oracle_loss(env, kin, terms, a, E0 * np.exp(eps_l)) - oracle_loss(env, kin, terms, a, E0 * np.exp(-eps_l))) \
            / (2 * eps_l)
        pred = gE * E0
        print("log E_shell", eps_l, pred, fd)
        if abs(pred - fd) > 5e-3 * abs(fd):
            failures.append(("E", eps_l, pred, fd))
    assert not failures, failures
