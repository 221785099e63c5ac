"""Vectorised tactile environments: many independent scenes stepped together in one World.

The reference trains its RL / CMA baselines through a gym environment that wraps one task scene
(TactileEnv, baseline/tactile_env.py:23-243) and vectorises it with a sequential DummyVecEnv
(baseline/training_rl.py:95): one scene per launch sequence.  BatchedTactileEnv keeps the same
reset / step / observation / reward shape but holds all scenes in one World, so every substep stage
is one launch for all of them.

Actions: per environment (d_pos[3], d_ori[3]) for its first sensor, applied as pose control over one
control step (set_pose_control + set_control_vel, fem_sensor.py:229-266; one launch for all sensors).
Observations: per environment the displacement (pos - virtual pos) of a fixed sample of the sensor's
surface nodes (the tactile signal the reference reads through its markers) and the object's centre
of mass.  Reward: scale - |centre of mass - target|^2 per environment (the COM readout of the tasks,
grasp_plastic.py:259-261).  Episodes end at ``time_limit`` steps; an environment whose observation
is not finite is truncated.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from .trajectory import eul2mat_zyx
from .world import World


class BatchedTactileEnv:
    def __init__(self, envs, substeps: int = 20, dt: float = 1e-4, time_limit: int = 100, n_obs_nodes: int = 32,
                 targets=None, reward_scale: float = 1.0, device="cuda", seed: int = 0, graph: bool = False):
        self.w = World(envs, n_frames=substeps + 1, dt=dt, device=device)
        # graph: the first step runs eagerly and records its launches (control velocities, S substeps,
        # frame copy) as one CUDA graph that later steps replay
        self.graph = bool(graph)
        self._graph = None
        w = self.w
        self.n_envs = len(envs)
        self.S = int(substeps)
        self.time_limit = int(time_limit)
        self.reward_scale = float(reward_scale)
        self.inv_T = 1.0 / (dt * self.S)
        dev = w.device
        # first sensor of every environment
        first = []
        for e in range(self.n_envs):
            row = w.env_rows[e]
            if row.s_end <= row.s_begin:
                raise ValueError(f"environment {e} has no sensor to drive")
            first.append(row.s_begin)
        self.first = first
        rng = np.random.default_rng(seed)
        idx = []
        for s in first:
            sp, r = w.sensor_specs[s], w.sensor_rows[s]
            surf = np.where(np.asarray(sp.layer) == np.asarray(sp.layer).max())[0]
            pick = rng.choice(surf, size=min(n_obs_nodes, len(surf)), replace=len(surf) < n_obs_nodes)
            idx.append(r.v_off + np.sort(pick))
        self.obs_idx = torch.as_tensor(np.stack(idx), dtype=torch.long, device=dev)  # [n_envs, k]
        self.TW = torch.stack([torch.as_tensor(w.sensor_specs[s].trans_world if w.sensor_specs[s].trans_world is not None
                                               else np.eye(4), dtype=torch.float64) for s in range(w.n_sensors)]).to(dev)
        self.TW_inv = torch.linalg.inv(self.TW.cpu()).to(dev)
        self.targets = (torch.zeros((self.n_envs, 3), device=dev) if targets is None
                        else torch.as_tensor(np.asarray(targets), dtype=torch.float32, device=dev))
        t = w.t
        self.init = [t["p_state"][0].clone(), t["v_pos"][0].clone(), t["v_vel"][0].clone(), t["v_vpos"][0].clone(),
                     t["r_state"][0].clone()]
        self.Ab = torch.zeros((w.n_sensors, 12), dtype=torch.float32, device=dev)
        self.Ab[:, 0] = self.Ab[:, 5] = self.Ab[:, 10] = 1.0  # identity for undriven sensors
        self.time_step = 0

    @property
    def obs_dim(self):
        return 3 * self.obs_idx.shape[1] + 3

    def get_observations(self) -> torch.Tensor:
        t = self.w.t
        disp = (t["v_pos"][0, :, :3] - t["v_vpos"][0, :, :3])[self.obs_idx]  # [n_envs, k, 3]
        com = self.w.com(0)[:, :3]
        return torch.cat([disp.reshape(self.n_envs, -1), com], 1)

    def reset(self, seed=None, options=None):
        t = self.w.t
        for k, v in zip(("p_state", "v_pos", "v_vel", "v_vpos", "r_state"), self.init):
            t[k][0].copy_(v)
        self.time_step = 0
        return self.get_observations(), {}

    def _advance(self):
        w = self.w
        N.check(w.lib.dt_pose_control_vel_all(w.wp, self.Ab.data_ptr(), self.inv_T, 0, self.S + 1, w.stream),
                "pose cv")
        w.step_begin()
        for f in range(self.S):
            w.substep(f)
        w.copy_frame(self.S, 0)

    def step(self, actions):
        """actions [n_envs, 6] (d_pos, d_ori in degrees per unit time) -> (obs, rewards, dones,
        truncated, infos), all per environment (device tensors)."""
        w = self.w
        a = torch.as_tensor(actions, dtype=torch.float64, device=w.device).reshape(self.n_envs, 6)
        s = torch.as_tensor(self.first, device=w.device)
        M = eul2mat_zyx(a[:, 3:6] * w.dt * self.S, a[:, 0:3] * w.dt * self.S)
        D = self.TW[s] @ M @ self.TW_inv[s]
        self.Ab[s] = D[:, :3, :].reshape(self.n_envs, 12).float()
        if self._graph is not None:
            self._graph.replay()
        else:
            self._advance()
            if self.graph:
                torch.cuda.synchronize(w.device)
                self._graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(self._graph):
                    self._advance()
        self.time_step += 1
        obs = self.get_observations()
        com = obs[:, -3:]
        rewards = self.reward_scale - ((com - self.targets) ** 2).sum(1)
        finite = torch.isfinite(obs).all(1)
        dones = torch.full((self.n_envs,), self.time_step >= self.time_limit, device=w.device)
        truncated = dones | ~finite
        obs = torch.where(finite[:, None], obs, torch.zeros_like(obs))
        return obs, rewards, dones, truncated, {}
