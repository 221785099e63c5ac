"""Differentiable rollouts, either on a full device tape (every frame of the rollout kept in HBM, no
recompute) or with device checkpoints (forward keeps the start state of every k-th control step;
backward recomputes each segment, then each step's substep tape, and runs the adjoint substeps in
reverse).

The reference keeps the start of every step in host RAM (memory_to_cache / memory_from_cache,
object_model/mpm_elastic.py:300-320, sensor_model/fem_sensor.py:501-521) and recomputes the
substeps of one step during the backward sweep (tasks/grasp_plastic.py:594-648); that is k = 1.
Here the checkpoints stay in HBM and k is a parameter; k = 0 keeps the whole tape.

Two action models drive the sensors' base layers through per-vertex control velocities:
  PoseTrajectory     per step and pose-controlled sensor (d_pos[3], d_ori[3]) as in set_pose_control
                     (fem_sensor.py:229-245): rot_v = d_ori dt S, trans_v = d_pos dt S, the step
                     transform dtrans_h = T_world eul2mat(rot_v, trans_v) T_world^-1 and the control
                     velocity (fem_sensor.py:259-266);
  GripperTrajectory  per step (d_pos[3], d_ori[3], d_gripper) of a parallel-jaw gripper whose two
                     fingers carry sensors (gripper_kinematics.py:120-216): per-substep finger poses
                     and control velocities, the sensors' velocities reset to them at every step start
                     (set_sensor_vel).
The 4x4 algebra runs in float64 torch on the device with autograd; the per-vertex control
velocities and everything after them are CUDA kernels with hand-written adjoints.
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


class Trajectory:
    """T control steps x S substeps of a World whose sensors are driven by actions (subclasses
    define the action model through controls / _apply / _apply_bwd).

    ``ckpt_every`` = k >= 1: the world holds one control step (n_frames = S + 1); the forward keeps
    the start state of every k-th step and the backward recomputes.  ``ckpt_every`` = 0 (full tape):
    the world holds the whole rollout (n_frames = T S + 1, step t on frames [t S, t S + S]) and the
    backward runs straight down the tape with no recompute, which is what the reference's
    gradient tape would do if it fitted in memory; on a 280 GB device it does for the tasks here.

    ``loss_terms``: list of (sensor, layer, target [nv,3]) marker-displacement terms read at the
    final frame; ``rope_terms``: list of (rope, target [3]) terms |tip - target|^2 of the rope's last
    particle at the final frame (the cable task's tip-position loss).

    ``rebin_every`` = r >= 1 (checkpointed trajectories only): at the start of every r-th segment after
    the first, before its checkpoint is saved, the particles are sorted by cell again (World.rebin), so
    that the scatters' same-cell runs survive long horizons; the permutation of each such checkpoint is
    kept, and the backward sweep, having reached the segment's first frame, maps the particle adjoint
    (and the material index) back to the previous segment's order.  0: the construction order is kept.

    ``graph``: the launch sequence of a forward (and of a backward) is the same on every call, so the
    first call runs eagerly and then records it as a CUDA graph; later calls copy the new controls
    into the recorded buffer and replay the graph (one launch from the host per rollout).  The
    recorded graphs hold the world's and this trajectory's device pointers: state set through the
    world's tensors in place is seen by the replays, reallocated tensors are not.
    """

    def __init__(self, world: World, n_steps: int, ckpt_every: int = 1, loss_terms=(), graph: bool = False,
                 rope_terms=(), rebin_every: int = 0):
        self.w = world
        self.graph = bool(graph)
        self._graphs = {}     # "fwd" / ("bwd", loss_bar) -> torch.cuda.CUDAGraph
        self._graph_launches = {}
        self._pool = None
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
        Np, V, NR = world.n_particles, world.n_verts, world.n_rope_particles
        if not self.full:
            self.ck_p = torch.zeros((self.n_ck, 6, Np, 4), device=dev)
            self.ck_v = torch.zeros((self.n_ck, 3, V, 4), device=dev)
            self.ck_r = torch.zeros((self.n_ck, 2, NR, 4), device=dev)
        self.rebin_every = int(rebin_every)
        if self.rebin_every < 0 or (self.rebin_every and self.full):
            raise ValueError("rebin_every needs a checkpointed trajectory (ckpt_every >= 1) and must be >= 0")
        self.ck_src = (torch.zeros((self.n_ck, Np), dtype=torch.int32, device=dev) if self.rebin_every else None)
        self._epoch = 0  # the re-binned segment (0: none) whose particle order the world holds
        self._fin = None  # checkpointed: a copy of the final frame (the backward sweep overwrites it)
        self._fin_live = False
        if not self.full and self.k > 1:
            self.seg_p = torch.zeros((self.k, 6, Np, 4), device=dev)
            self.seg_v = torch.zeros((self.k, 3, V, 4), device=dev)
            self.seg_r = torch.zeros((self.k, 2, NR, 4), device=dev)
        self.loss_terms = []
        for s, layer, target in loss_terms:
            tg = torch.zeros((world.sensor_rows[s].nv, 4), device=dev)
            tg[:, :3] = torch.as_tensor(np.asarray(target), dtype=torch.float32, device=dev)
            self.loss_terms.append((s, int(layer), tg))
        self.rope_terms = []
        for r, target in rope_terms:
            row = world.rope_rows[r]
            self.rope_terms.append((row.p_off + row.n - 1,
                                    torch.as_tensor(np.asarray(target), dtype=torch.float32, device=dev).reshape(3)))
        self.loss = torch.zeros(1, device=dev)
        self.ctrl = None
        self.ctrl_bar = None
        self.launches = 0

    @staticmethod
    def frames_needed(n_steps: int, substeps: int, ckpt_every: int) -> int:
        """World n_frames for a trajectory of ``n_steps`` x ``substeps`` with ``ckpt_every``."""
        return n_steps * substeps + 1 if ckpt_every == 0 else substeps + 1

    # ------------------------------------------------------------------ action model (subclasses)
    def controls(self, actions: torch.Tensor) -> torch.Tensor:
        """actions (float64, differentiable) -> per-step control tensor [T, ...] (float64)."""
        raise NotImplementedError

    def _apply(self, t: int, f0: int):
        """Launch the control velocities of step t, whose first frame is f0."""
        raise NotImplementedError

    def _apply_bwd(self, t: int, f0: int):
        """Adjoint of _apply: accumulate into self.ctrl_bar[t] (after the step's adjoint substeps)."""
        raise NotImplementedError

    # ------------------------------------------------------------------ state save / load
    def _save(self, P, Vv, Rr, i):
        t = self.w.t
        P[i].copy_(t["p_state"][0])
        Vv[i, 0].copy_(t["v_pos"][0])
        Vv[i, 1].copy_(t["v_vel"][0])
        Vv[i, 2].copy_(t["v_vpos"][0])
        Rr[i].copy_(t["r_state"][0])

    def _load(self, P, Vv, Rr, i):
        t = self.w.t
        t["p_state"][0].copy_(P[i])
        t["v_pos"][0].copy_(Vv[i, 0])
        t["v_vel"][0].copy_(Vv[i, 1])
        t["v_vpos"][0].copy_(Vv[i, 2])
        t["r_state"][0].copy_(Rr[i])

    # ------------------------------------------------------------------ particle order (rebin_every)
    def _rebinned(self, seg: int) -> bool:
        return self.rebin_every > 0 and seg > 0 and seg % self.rebin_every == 0

    def _epoch_of(self, seg: int) -> int:
        """The re-binned segment whose order segment ``seg`` runs in (0: the rollout's start order)."""
        return (seg // self.rebin_every) * self.rebin_every if self.rebin_every else 0

    def _to_epoch(self, e: int):
        """Bring the world's material index and slot maps (not its state or adjoints) to the order of
        re-binned segment ``e``, through the stored permutations of the segments in between."""
        while self._epoch < e:
            self._epoch += self.rebin_every
            self.w.rebin_permute(self.ck_src[self._epoch], inverse=False)
            self.launches += 1
        while self._epoch > e:
            self.w.rebin_permute(self.ck_src[self._epoch], inverse=True)
            self.launches += 1
            self._epoch -= self.rebin_every

    def _final_frame_ready(self):
        """A checkpointed backward sweep recomputes each step on the world's frames and so overwrites
        the final frame the loss adjoint is seeded from: keep a copy of it before the first sweep after
        a forward, put it back before every later one (a second backward, or one after adjoint_at)."""
        if self.full:
            return
        if self._fin_live:
            if self._fin is None:
                dev, Np, V, NR = self.w.device, self.w.n_particles, self.w.n_verts, self.w.n_rope_particles
                self._fin = (torch.zeros((1, 6, Np, 4), device=dev), torch.zeros((1, 3, V, 4), device=dev),
                             torch.zeros((1, 2, NR, 4), device=dev))
            self._save(*self._fin, 0)  # the forward left the final state in frames 0 and S
            self._fin_live = False
        elif self._fin is not None:
            self._load(*self._fin, 0)
            self.w.copy_frame(0, self.S)
        else:
            raise RuntimeError("the backward sweep needs a forward rollout first")

    def _leave_segment(self, seg: int):
        """The backward sweep reached segment ``seg``'s first frame: map the adjoint of that frame (the
        buffer the previous segment's last step reads) and the material index back to the order the
        previous segment ran in."""
        if self._rebinned(seg):
            self.w.rebin_permute(self.ck_src[seg], inverse=True, adj_buf=self.S & 1)
            self.launches += 1
            self._epoch = self._epoch_of(seg - 1)

    # ------------------------------------------------------------------ one control step
    def _f0(self, t):
        return t * self.S if self.full else 0

    def _step(self, t, copy_end=True, tape=True):
        """Control step t.  ``tape`` = False: its substeps write no grid or SVD tape (a checkpointed
        rollout's forward pass, whose backward sweep recomputes the step with its tape)."""
        w = self.w
        f0 = self._f0(t)
        self._apply(t, f0)
        if not self.full:
            w.step_begin()
            self.launches += 1
        w.set_tape(tape)
        try:
            for f in range(f0, f0 + self.S):
                w.substep(f)
        finally:
            w.set_tape(True)
        self.launches += 3 * self.S
        if copy_end and not self.full:
            w.copy_frame(self.S, 0)

    # ------------------------------------------------------------------ CUDA graphs
    def _capture(self, key, body):
        """Record ``body``'s launches (already run once eagerly) as a CUDA graph under ``key``."""
        if self.w.stream_override is not None:
            raise RuntimeError("graph capture needs the world to launch on torch's current stream")
        torch.cuda.synchronize(self.w.device)
        g = torch.cuda.CUDAGraph()
        n0 = self.launches
        with torch.cuda.graph(g, pool=self._pool):
            body()
        self._graph_launches[key] = self.launches - n0
        self.launches = n0
        self._pool = g.pool()
        self._graphs[key] = g

    def _replay(self, key):
        self.w.touch()  # the replay rewrites the world's frames
        self._graphs[key].replay()
        self.launches += self._graph_launches[key]

    def reset_graphs(self):
        """Drop the recorded graphs (after reallocating world tensors or changing launch settings)."""
        self._graphs.clear()
        self._graph_launches.clear()
        if self.w.probe is not None:
            self.w.probe_graph_events = []

    def _forward_body(self):
        if self.full:
            self.w.step_begin()
            self.launches += 1
        for t in range(self.T):
            if not self.full and t % self.k == 0:
                if self._rebinned(t // self.k):
                    self.w.rebin(0, self.ck_src[t // self.k])
                    self._epoch = t // self.k
                    self.launches += 8
                self._save(self.ck_p, self.ck_v, self.ck_r, t // self.k)
            self._step(t, tape=self.full)  # checkpointed: the backward sweep recomputes each step's tape
        self.readout()

    def forward(self, actions: torch.Tensor) -> torch.Tensor:
        """Roll out; returns the final-frame loss (device scalar)."""
        if actions.shape[0] != self.T:
            raise ValueError(f"actions hold {actions.shape[0]} control steps, the trajectory {self.T}")
        self.actions = actions.detach().double().requires_grad_(True)
        self.ctrl = self.controls(self.actions)
        c32 = self.ctrl.detach().float().contiguous()
        self._epoch = 0  # the world's present particle order is this rollout's start order
        if self.graph and "fwd" in self._graphs:
            self.ctrl32.copy_(c32)
            self._replay("fwd")
            self._epoch = self._epoch_of(self.n_ck - 1)
            self._fin_live = True
            return self.loss
        self.ctrl32 = c32
        self._forward_body()
        if self.graph:
            self._capture("fwd", self._forward_body)
        self._fin_live = True
        return self.loss

    def readout(self) -> torch.Tensor:
        w = self.w
        self.loss.zero_()
        f = self.f_end if self.full else 0  # the checkpointed world copied the final frame to 0
        for s, layer, tg in self.loss_terms:
            N.check(w.lib.dt_marker_loss(w.wp, s, f, layer, tg.data_ptr(), self.loss.data_ptr(), w.stream), "loss")
            self.launches += 1
        for tip, tg in self.rope_terms:
            self.loss += ((w.t["r_state"][f, 0, tip, :3] - tg) ** 2).sum()
        return self.loss

    def _seed_rope_terms(self, loss_bar):
        """Adjoint of the rope-tip terms into the rope adjoint of the final frame."""
        w = self.w
        for tip, tg in self.rope_terms:
            w.t["r_adj"][self.f_end & 1, 0, tip, :3] += (2.0 * float(loss_bar)) * (
                w.t["r_state"][self.f_end, 0, tip, :3] - tg)

    def _step_bwd(self, t):
        w = self.w
        f0 = self._f0(t)
        w.substeps_bwd(f0 + self.S, f0)
        self.launches += 3 * self.S + 1
        self._apply_bwd(t, f0)

    def backward(self, loss_bar: float = 1.0) -> torch.Tensor:
        """Adjoint sweep; returns d loss / d actions (float64, the actions' shape).  Initial-state
        adjoints are left in the world's frame-0 adjoint buffers, material grads in mat_adj."""
        key = ("bwd", float(loss_bar))
        self._to_epoch(self._epoch_of(self.n_ck - 1))  # after adjoint_at the world may hold an earlier order
        self._final_frame_ready()
        if self.graph and key in self._graphs:
            self._replay(key)
            self._epoch = 0
        else:
            if self.ctrl_bar is None or self.ctrl_bar.shape != self.ctrl32.shape:
                self.ctrl_bar = torch.zeros_like(self.ctrl32)
            self._backward_body(loss_bar)
            if self.graph:
                self._capture(key, lambda: self._backward_body(loss_bar))
        # the action -> control graph is kept: a second sweep of the same forward differentiates it again
        (g,) = torch.autograd.grad(self.ctrl, self.actions, self.ctrl_bar.double(), retain_graph=True)
        return g

    def material_grad(self) -> torch.Tensor:
        """d loss / d (mu, lambda) of every material of the world, [n_materials, 2] float64, from the
        last backward (the adjoint substeps accumulate it over the whole rollout)."""
        return self.w.material_adjoint()

    def material_grad_E_nu(self) -> torch.Tensor:
        """d loss / d (E, nu) of every material, [n_materials, 2] float64, by the chain rule of
        mu(E, nu), lambda(E, nu) (mpm_elastic.py:70-71) applied to material_grad(); for materials
        given by E and nu (not by explicit Lame parameters)."""
        from .scene import lame_grad_to_E_nu
        g = self.material_grad()
        out = torch.zeros_like(g)
        for m, mat in enumerate(self.w.materials):
            gE, gnu = lame_grad_to_E_nu(float(mat.E), float(mat.nu), g[m, 0], g[m, 1])
            out[m, 0], out[m, 1] = gE, gnu
        return out

    def adjoint_at(self, t: int, f: int, loss_bar: float = 1.0) -> int:
        """Run the backward sweep of the last forward from the loss down to frame ``f`` + 1 of step
        ``t`` (host-launched, no graph) and stop there: the step's forward tape (frames of step t, its
        grid tape) is valid and the adjoint of its frame f + 1 is in the world's adjoint buffers
        ((f + 1) & 1).  Returns the world frame index of step t's frame f.  For inspecting gradients
        mid-rollout (the adjoint of one substep from a real loss); a following backward() starts over
        (from the final frame of the last forward, which is kept for it)."""
        if not (0 <= t < self.T and 0 <= f < self.S):
            raise ValueError(f"(t, f) = ({t}, {f}) outside [0, {self.T}) x [0, {self.S})")
        w = self.w
        self._to_epoch(self._epoch_of(self.n_ck - 1))
        self._final_frame_ready()
        w.adj_clear()
        for s, layer, tg in self.loss_terms:
            N.check(w.lib.dt_marker_loss_bwd(w.wp, s, self.f_end, layer, tg.data_ptr(), float(loss_bar), w.stream),
                    "loss bwd")
        self._seed_rope_terms(loss_bar)
        if self.ctrl_bar is None or self.ctrl_bar.shape != self.ctrl32.shape:
            self.ctrl_bar = torch.zeros_like(self.ctrl32)
        self.ctrl_bar.zero_()

        def stop(tt):
            f0 = self._f0(tt)
            if f + 1 < self.S:  # (f = S - 1: the adjoint of frame S is the step's incoming one)
                w.substeps_bwd(f0 + self.S, f0 + f + 1)
            return f0 + f

        if self.full:
            for tt in reversed(range(t + 1, self.T)):
                self._step_bwd(tt)
            return stop(t)
        for seg in reversed(range(self.n_ck)):
            t0, t1 = seg * self.k, min((seg + 1) * self.k, self.T)
            if t1 <= t:
                break
            self._load(self.ck_p, self.ck_v, self.ck_r, seg)
            if self.k > 1:
                for tt in range(t0, t1):
                    self._save(self.seg_p, self.seg_v, self.seg_r, tt - t0)
                    if tt + 1 < t1:
                        self._step(tt, tape=False)
            for tt in reversed(range(max(t0, t), t1)):
                if self.k > 1:
                    self._load(self.seg_p, self.seg_v, self.seg_r, tt - t0)
                self._step(tt, copy_end=False)
                if tt == t:
                    return stop(tt)
                self._step_bwd(tt)
                if self.S & 1:
                    for name in ("p_adj", "v_adj_pos", "v_adj_vel", "v_adj_vpos", "r_adj"):
                        w.t[name][1].copy_(w.t[name][0])
            self._leave_segment(seg)
        raise AssertionError("unreachable")

    def _backward_body(self, loss_bar):
        w = self.w
        st = w.stream
        w.adj_clear()
        for s, layer, tg in self.loss_terms:
            N.check(w.lib.dt_marker_loss_bwd(w.wp, s, self.f_end, layer, tg.data_ptr(), float(loss_bar), st),
                    "loss bwd")
        self._seed_rope_terms(loss_bar)
        self.ctrl_bar.zero_()
        if self.full:
            for t in reversed(range(self.T)):
                self._step_bwd(t)
        for seg in reversed(range(self.n_ck)):
            t0, t1 = seg * self.k, min((seg + 1) * self.k, self.T)
            self._load(self.ck_p, self.ck_v, self.ck_r, seg)
            if self.k > 1:
                for t in range(t0, t1):
                    self._save(self.seg_p, self.seg_v, self.seg_r, t - t0)
                    if t + 1 < t1:
                        self._step(t, tape=False)
            for t in reversed(range(t0, t1)):
                if self.k > 1:
                    self._load(self.seg_p, self.seg_v, self.seg_r, t - t0)
                self._step(t, copy_end=False)
                self._step_bwd(t)
                if self.S & 1:  # frame 0's adjoint (buffer 0) is frame S's of the previous step (buffer 1)
                    for name in ("p_adj", "v_adj_pos", "v_adj_vel", "v_adj_vpos", "r_adj"):
                        w.t[name][1].copy_(w.t[name][0])
            self._leave_segment(seg)


class PoseTrajectory(Trajectory):
    """Pose-controlled sensors (dome sensor, set_pose_control / set_control_vel): actions
    [T, n_sensors, 6] = (d_pos[3], d_ori[3] in degrees per unit time)."""

    def __init__(self, world: World, n_steps: int, ckpt_every: int = 1, loss_terms=(), graph: bool = False,
                 rope_terms=(), rebin_every: int = 0):
        super().__init__(world, n_steps, ckpt_every, loss_terms, graph, rope_terms, rebin_every)
        dev = world.device
        self.inv_T = 1.0 / (world.dt * self.S)
        Ms = [sp.trans_world if sp.trans_world is not None else np.eye(4) for sp in world.sensor_specs]
        self.TW = torch.as_tensor(np.stack(Ms) if Ms else np.zeros((0, 4, 4)), dtype=torch.float64, device=dev)
        self.TW_inv = torch.as_tensor(np.stack([np.linalg.inv(M) for M in Ms]) if Ms else np.zeros((0, 4, 4)),
                                      dtype=torch.float64, device=dev)

    def step_transforms(self, actions: torch.Tensor) -> torch.Tensor:
        """actions [T, n_sensors, 6] (float64) -> Ab [T, n_sensors, 12] (float64, differentiable); all
        sensors and steps in one batch of 4x4 products."""
        k = self.w.dt * self.S
        M = eul2mat_zyx(actions[..., 3:6] * k, actions[..., 0:3] * k)  # [T, n_sensors, 4, 4]
        D = self.TW @ M @ self.TW_inv
        return D[..., :3, :].reshape(actions.shape[0], actions.shape[1], 12)

    controls = step_transforms

    # every sensor is pose-controlled: one launch for all of them (rows of ctrl32[t] are per sensor)
    def _apply(self, t, f0):
        w = self.w
        N.check(w.lib.dt_pose_control_vel_all(w.wp, self.ctrl32[t].data_ptr(), self.inv_T, f0, self.S + 1, w.stream),
                "pose cv")
        self.launches += 1

    def _apply_bwd(self, t, f0):
        w = self.w
        N.check(w.lib.dt_pose_control_vel_bwd_all(w.wp, self.ctrl32[t].data_ptr(), self.inv_T,
                                                  self.ctrl_bar[t].data_ptr(), f0, self.S + 1, w.stream),
                "pose cv bwd")
        self.launches += 1

    # names kept for callers of the earlier interface
    @property
    def Ab(self):
        return self.ctrl

    @property
    def Ab32(self):
        return self.ctrl32

    @property
    def Ab_bar(self):
        return self.ctrl_bar


class GripperTrajectory(Trajectory):
    """Two finger sensors of a parallel-jaw gripper (Gripper, gripper_kinematics.py:68-296): actions
    [T, 7] = (d_pos[3], d_ori[3] in degrees per unit time, d_gripper).  ``kin`` is a
    GripperKinematics; ``fingers`` the two sensors' indices in the world."""

    def __init__(self, world: World, n_steps: int, kin, fingers=(0, 1), ckpt_every: int = 1, loss_terms=(),
                 graph: bool = False, rope_terms=(), rebin_every: int = 0):
        super().__init__(world, n_steps, ckpt_every, loss_terms, graph, rope_terms, rebin_every)
        self.kin = kin
        self.fingers = tuple(fingers)
        dev = world.device
        rest = torch.zeros((world.n_verts, 4), dtype=torch.float32, device=dev)
        rest[:, :3] = torch.as_tensor(world.rest_verts, device=dev)
        self.rest = rest
        self.T0_inv = [torch.linalg.inv(F.cpu()).to(dev) for F in kin.finger_poses0()]
        self.zero_cv = torch.zeros((1, 4), device=dev)

    def controls(self, actions: torch.Tensor) -> torch.Tensor:
        """actions [T, 7] -> D [T, 2, S, 12]: rows 0..2 of (F_{f+1} - F_f) T0^-1 / dt per finger and
        substep (fem_sensor1/2_set_control_vel, gripper_kinematics.py:196-216)."""
        frames = self.kin.rollout(actions, self.S)  # [T, 2, S + 1, 4, 4]
        dt = self.w.dt
        out = []
        for i in range(2):
            Fi = frames[:, i]
            D = (Fi[:, 1:] - Fi[:, :-1]) @ self.T0_inv[i].to(Fi.dtype) / dt
            out.append(D[..., :3, :].reshape(self.T, self.S, 12))
        return torch.stack(out, 1)

    def _apply(self, t, f0):
        w = self.w
        for i, s in enumerate(self.fingers):
            N.check(w.lib.dt_affine_control_vel(w.wp, s, self.ctrl32[t, i].data_ptr(), self.rest.data_ptr(), f0,
                                                self.S, w.stream), "affine cv")
            sl = w.vslice(s)
            # frame f0 + S: the next step's first control velocity (written by its own _apply); zero
            # at the end of the rollout, as the reference never sets control_vel[sub_steps - 1]
            w.t["v_cv"][f0 + self.S, sl] = 0.0
            # set_sensor_vel(0) (gripper_fem.py:194-196): the sensor starts the step at its control velocity
            w.t["v_vel"][f0, sl] = w.t["v_cv"][f0, sl]
            w.t["v_velmid"][f0, sl] = w.t["v_cv"][f0, sl]
        self.launches += 2

    def _apply_bwd(self, t, f0):
        w = self.w
        b = f0 & 1
        for i, s in enumerate(self.fingers):
            sl = w.vslice(s)
            # adjoint of set_sensor_vel: the velocity that was overwritten gets none
            w.t["v_adj_cv"][f0, sl] += w.t["v_adj_vel"][b, sl]
            w.t["v_adj_vel"][b, sl] = 0.0
            w.t["v_adj_cv"][f0 + self.S, sl] = 0.0
            N.check(w.lib.dt_affine_control_vel_bwd(w.wp, s, self.rest.data_ptr(), f0, self.S,
                                                    self.ctrl_bar[t, i].data_ptr(), w.stream), "affine cv bwd")
        self.launches += 2


# ---------------------------------------------------------------------------------------------
# gripper kinematics
# ---------------------------------------------------------------------------------------------
def eul2mat_xyz(rot_deg: torch.Tensor, trans: torch.Tensor) -> torch.Tensor:
    """4x4 transforms with R = Rx Ry Rz (the gripper's eul2mat, gripper_kinematics.py:280-296)."""
    r = torch.deg2rad(rot_deg)
    cx, cy, cz = torch.cos(r[..., 0]), torch.cos(r[..., 1]), torch.cos(r[..., 2])
    sx, sy, sz = torch.sin(r[..., 0]), torch.sin(r[..., 1]), torch.sin(r[..., 2])
    o, z = torch.ones_like(cx), torch.zeros_like(cx)
    Rx = torch.stack([o, z, z, z, cx, -sx, z, sx, cx], -1).reshape(*cx.shape, 3, 3)
    Ry = torch.stack([cy, z, sy, z, o, z, -sy, z, cy], -1).reshape(*cx.shape, 3, 3)
    Rz = torch.stack([cz, -sz, z, sz, cz, z, z, z, o], -1).reshape(*cx.shape, 3, 3)
    R = Rx @ Ry @ Rz
    top = torch.cat([R, trans[..., :, None]], -1)
    bottom = torch.zeros(*cx.shape, 1, 4, dtype=R.dtype, device=R.device)
    bottom[..., 0, 3] = 1
    return torch.cat([top, bottom], -2)


class GripperKinematics:
    """Kinematic chain of the parallel-jaw gripper (Gripper.init_params / pos_transformation /
    grip_kinematic, gripper_kinematics.py:120-194), in float64 torch with autograd.

    The end effector sits at ee_world = eul2mat(rot, trans); finger i's pose is
    ee ee_to_finger_i finger_local_i with ee_to_finger_1 = eul2mat((-90, 0, -90),
    (-base_width/2 + grip_width, -base_height - finger_height, 0)) and ee_to_finger_2 =
    eul2mat((-90, 0, 90), (base_width/2 - grip_width, ...)).  Per substep the end effector moves by
    eul2mat(d_ori dt, d_pos dt) in its own frame and each finger by (0, d_gripper dt, 0) in its own."""

    def __init__(self, rot, trans, grip_width, dt, base_height=2.0, base_width=14.0, finger_height=7.5,
                 device="cpu"):
        self.dt = float(dt)
        self.dev = torch.device(device)
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.ee_world = eul2mat_xyz(torch.as_tensor(rot, **f64), torch.as_tensor(trans, **f64))
        bw, bh, fh, gw = base_width, base_height, finger_height, grip_width
        self.e2f = [eul2mat_xyz(torch.tensor([-90.0, 0.0, -90.0], **f64),
                                torch.tensor([-bw / 2 + gw, -bh - fh, 0.0], **f64)),
                    eul2mat_xyz(torch.tensor([-90.0, 0.0, 90.0], **f64),
                                torch.tensor([bw / 2 - gw, -bh - fh, 0.0], **f64))]

    def finger_poses0(self):
        """Finger poses at the start (the sensors are placed with them: init_fem_sensor)."""
        return [self.ee_world @ e for e in self.e2f]

    def rollout(self, actions: torch.Tensor, S: int) -> torch.Tensor:
        """actions [T, 7] -> finger poses [T, 2, S + 1, 4, 4] of every step's frames 0..S (frame 0 of
        step t is frame S of step t - 1)."""
        T = actions.shape[0]
        dt = self.dt
        eye = torch.eye(4, dtype=torch.float64, device=actions.device)
        ee_world = self.ee_world.to(actions.device)
        e2f = [e.to(actions.device) for e in self.e2f]
        ee_local, fl = eye, [eye, eye]
        F = [ee_world @ e2f[0], ee_world @ e2f[1]]
        out = []
        for t in range(T):
            a = actions[t]
            E = eul2mat_xyz(a[3:6] * dt, a[0:3] * dt)
            z = torch.zeros_like(a[6])
            G = eul2mat_xyz(torch.stack([z, z, z]), torch.stack([z, a[6] * dt, z]))
            frames = [[F[0]], [F[1]]]
            for _ in range(S):
                ee_local = E @ ee_local
                ee = ee_world @ ee_local
                for i in range(2):
                    fl[i] = G @ fl[i]
                    F[i] = ee @ e2f[i] @ fl[i]
                    frames[i].append(F[i])
            out.append(torch.stack([torch.stack(frames[0]), torch.stack(frames[1])]))
        return torch.stack(out)
