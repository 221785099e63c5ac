"""Differentiable rollouts, either on a full device tape (every frame of the rollout kept in HBM, no
recompute) or with device checkpoints (forward keeps the start state of every k-th control step;
backward recomputes each segment, then each step's substep tape, and runs the adjoint substeps in
reverse).

The reference keeps the start of every step in host RAM (memory_to_cache / memory_from_cache,
object_model/mpm_elastic.py:300-320, sensor_model/fem_sensor.py:501-521) and recomputes the
substeps of one step during the backward sweep (tasks/grasp_plastic.py:594-648); that is k = 1.
Here the checkpoints stay in HBM and k is a parameter; k = 0 keeps the whole tape.

Actions are per step and per pose-controlled sensor: (d_pos[3], d_ori[3]) as in
set_pose_control (fem_sensor.py:229-245): rot_v = d_ori dt S, trans_v = d_pos dt S, the step
transform dtrans_h = T_world eul2mat(rot_v, trans_v) T_world^-1 drives the base layer through the
control velocity (fem_sensor.py:259-266).  The 4x4 algebra runs in float64 torch on the device;
the per-vertex control velocities and everything after them are CUDA kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from .world import World


def eul2mat_zyx(rot_deg: torch.Tensor, trans: torch.Tensor) -> torch.Tensor:
    """Batched 4x4 transforms with R = Rz Ry Rx (fem_sensor.py:196-210); [..., 3] -> [..., 4, 4]."""
    r = torch.deg2rad(rot_deg)
    cx, cy, cz = torch.cos(r[..., 0]), torch.cos(r[..., 1]), torch.cos(r[..., 2])
    sx, sy, sz = torch.sin(r[..., 0]), torch.sin(r[..., 1]), torch.sin(r[..., 2])
    o, z = torch.ones_like(cx), torch.zeros_like(cx)
    Rx = torch.stack([o, z, z, z, cx, -sx, z, sx, cx], -1).reshape(*cx.shape, 3, 3)
    Ry = torch.stack([cy, z, sy, z, o, z, -sy, z, cy], -1).reshape(*cx.shape, 3, 3)
    Rz = torch.stack([cz, -sz, z, sz, cz, z, z, z, o], -1).reshape(*cx.shape, 3, 3)
    R = Rz @ Ry @ Rx
    top = torch.cat([R, trans[..., :, None]], -1)
    bottom = torch.zeros(*cx.shape, 1, 4, dtype=R.dtype, device=R.device)
    bottom[..., 0, 3] = 1
    return torch.cat([top, bottom], -2)


class PoseTrajectory:
    """T control steps x S substeps of a World whose sensors are pose-controlled.

    ``ckpt_every`` = k >= 1: the world holds one control step (n_frames = S + 1); the forward keeps
    the start state of every k-th step and the backward recomputes.  ``ckpt_every`` = 0 (full tape):
    the world holds the whole rollout (n_frames = T S + 1, step t on frames [t S, t S + S]) and the
    backward runs straight down the tape with no recompute, which is what the reference's
    gradient tape would do if it fitted in memory; on a 280 GB device it does for the tasks here.

    ``loss_terms``: list of (sensor, layer, target [nv,3]) marker-displacement terms read at the
    final frame.
    """

    def __init__(self, world: World, n_steps: int, ckpt_every: int = 1, loss_terms=()):
        self.w = world
        self.T = int(n_steps)
        self.full = int(ckpt_every) == 0
        if self.full:
            if (world.n_frames - 1) % self.T:
                raise ValueError(f"full tape: n_frames - 1 = {world.n_frames - 1} is not a multiple of T = {self.T}")
            self.S = (world.n_frames - 1) // self.T
            self.k = self.T
            self.n_ck = 0
        else:
            self.S = world.n_frames - 1
            self.k = int(ckpt_every)
            self.n_ck = (self.T + self.k - 1) // self.k
        self.f_end = self.T * self.S if self.full else self.S  # frame holding the final state
        dev = world.device
        Np, V = world.n_particles, world.n_verts
        if not self.full:
            self.ck_p = torch.zeros((self.n_ck, 6, Np, 4), device=dev)
            self.ck_v = torch.zeros((self.n_ck, 3, V, 4), device=dev)
        if not self.full and self.k > 1:
            self.seg_p = torch.zeros((self.k, 6, Np, 4), device=dev)
            self.seg_v = torch.zeros((self.k, 3, V, 4), device=dev)
        self.inv_T = 1.0 / (world.dt * self.S)
        self.TW, self.TW_inv = [], []
        for sp in world.sensor_specs:
            M = sp.trans_world if sp.trans_world is not None else np.eye(4)
            self.TW.append(torch.as_tensor(M, dtype=torch.float64, device=dev))
            self.TW_inv.append(torch.as_tensor(np.linalg.inv(M), dtype=torch.float64, device=dev))
        self.loss_terms = []
        for s, layer, target in loss_terms:
            tg = torch.zeros((world.sensor_rows[s].nv, 4), device=dev)
            tg[:, :3] = torch.as_tensor(np.asarray(target), dtype=torch.float32, device=dev)
            self.loss_terms.append((s, int(layer), tg))
        self.loss = torch.zeros(1, device=dev)
        self.Ab = None
        self.Ab_bar = None
        self.launches = 0

    @staticmethod
    def frames_needed(n_steps: int, substeps: int, ckpt_every: int) -> int:
        """World n_frames for a trajectory of ``n_steps`` x ``substeps`` with ``ckpt_every``."""
        return n_steps * substeps + 1 if ckpt_every == 0 else substeps + 1

    # ------------------------------------------------------------------ state save / load
    def _save(self, P, Vv, i):
        t = self.w.t
        P[i].copy_(t["p_state"][0])
        Vv[i, 0].copy_(t["v_pos"][0])
        Vv[i, 1].copy_(t["v_vel"][0])
        Vv[i, 2].copy_(t["v_vpos"][0])

    def _load(self, P, Vv, i):
        t = self.w.t
        t["p_state"][0].copy_(P[i])
        t["v_pos"][0].copy_(Vv[i, 0])
        t["v_vel"][0].copy_(Vv[i, 1])
        t["v_vpos"][0].copy_(Vv[i, 2])

    # ------------------------------------------------------------------ actions
    def step_transforms(self, actions: torch.Tensor) -> torch.Tensor:
        """actions [T, n_sensors, 6] (float64) -> Ab [T, n_sensors, 12] (float64, differentiable)."""
        S = self.S
        out = []
        for s in range(self.w.n_sensors):
            a = actions[:, s]
            M = eul2mat_zyx(a[:, 3:6] * self.w.dt * S, a[:, 0:3] * self.w.dt * S)
            D = self.TW[s] @ M @ self.TW_inv[s]
            out.append(D[:, :3, :].reshape(-1, 12))
        return torch.stack(out, 1)

    # ------------------------------------------------------------------ one control step
    def _f0(self, t):
        return t * self.S if self.full else 0

    def _step(self, t, copy_end=True):
        w = self.w
        st = w.stream
        f0 = self._f0(t)
        for s in range(w.n_sensors):
            N.check(w.lib.dt_pose_control_vel(w.wp, s, self.Ab32[t, s].data_ptr(), self.inv_T, f0, self.S + 1, st),
                    "pose cv")
        self.launches += w.n_sensors
        if not self.full:
            w.step_begin()
            self.launches += 1
        for f in range(f0, f0 + self.S):
            w.substep(f)
        self.launches += 3 * self.S
        if copy_end and not self.full:
            w.copy_frame(self.S, 0)

    def forward(self, actions: torch.Tensor) -> torch.Tensor:
        """Roll out; returns the final-frame loss (device scalar)."""
        self.actions = actions.detach().double().requires_grad_(True)
        self.Ab = self.step_transforms(self.actions)
        self.Ab32 = self.Ab.detach().float().contiguous()
        if self.full:
            self.w.step_begin()
            self.launches += 1
        for t in range(self.T):
            if not self.full and t % self.k == 0:
                self._save(self.ck_p, self.ck_v, t // self.k)
            self._step(t)
        return self.readout()

    def readout(self) -> torch.Tensor:
        w = self.w
        self.loss.zero_()
        f = self.f_end if self.full else 0  # the checkpointed world copied the final frame to 0
        for s, layer, tg in self.loss_terms:
            N.check(w.lib.dt_marker_loss(w.wp, s, f, layer, tg.data_ptr(), self.loss.data_ptr(), w.stream), "loss")
            self.launches += 1
        return self.loss

    def _step_bwd(self, t):
        w = self.w
        f0 = self._f0(t)
        for f in reversed(range(f0, f0 + self.S)):
            w.substep_bwd(f)
        for s in range(w.n_sensors):
            N.check(w.lib.dt_pose_control_vel_bwd(w.wp, s, self.Ab32[t, s].data_ptr(), self.inv_T,
                                                  self.Ab_bar[t, s].data_ptr(), f0, self.S + 1, w.stream),
                    "pose cv bwd")
        self.launches += 4 * self.S + w.n_sensors

    def backward(self, loss_bar: float = 1.0) -> torch.Tensor:
        """Adjoint sweep; returns d loss / d actions [T, n_sensors, 6] (float64).  Initial-state
        adjoints are left in the world's frame-0 adjoint buffers, material grads in mat_adj."""
        w = self.w
        st = w.stream
        w.adj_clear()
        for s, layer, tg in self.loss_terms:
            N.check(w.lib.dt_marker_loss_bwd(w.wp, s, self.f_end, layer, tg.data_ptr(), float(loss_bar), st),
                    "loss bwd")
        self.Ab_bar = torch.zeros_like(self.Ab32)
        if self.full:
            for t in reversed(range(self.T)):
                self._step_bwd(t)
        for seg in reversed(range(self.n_ck)):
            t0, t1 = seg * self.k, min((seg + 1) * self.k, self.T)
            self._load(self.ck_p, self.ck_v, seg)
            if self.k > 1:
                for t in range(t0, t1):
                    self._save(self.seg_p, self.seg_v, t - t0)
                    if t + 1 < t1:
                        self._step(t)
            for t in reversed(range(t0, t1)):
                if self.k > 1:
                    self._load(self.seg_p, self.seg_v, t - t0)
                self._step(t, copy_end=False)
                self._step_bwd(t)
                if self.S & 1:  # frame 0's adjoint (buffer 0) is frame S's of the previous step (buffer 1)
                    for name in ("p_adj", "v_adj_pos", "v_adj_vel", "v_adj_vpos"):
                        w.t[name][1].copy_(w.t[name][0])
        (g,) = torch.autograd.grad(self.Ab, self.actions, self.Ab_bar.double())
        return g
