"""Vectorised environments (BatchedTactileEnv): stepping several scenes in one World gives each
scene's observations and rewards as stepping it alone (1e-5 relative)."""
import numpy as np
import pytest
import torch

from difftactile_gb300.envs import BatchedTactileEnv
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu


def test_batched_env_matches_envs_stepped_alone(cuda_lib):
    scenes = [SS.pad_over_box(seed=1), SS.pad_over_box(seed=2, box_cells=(5, 4, 5)), SS.dome_over_box()]
    rng = np.random.default_rng(0)
    acts = 0.05 * rng.standard_normal((3, len(scenes), 6))
    acts[..., 1] -= 0.1
    batched = BatchedTactileEnv(scenes, substeps=4, time_limit=3, n_obs_nodes=8, seed=1)
    obs_b, _ = batched.reset()
    assert obs_b.shape == (3, batched.obs_dim)
    outs = []
    for t in range(3):
        outs.append(batched.step(acts[t]))
    assert bool(outs[-1][2].all()) and not bool(outs[0][2].any())
    for e, sc in enumerate(scenes):
        alone = BatchedTactileEnv([sc], substeps=4, time_limit=3, n_obs_nodes=8, seed=1)
        alone.obs_idx = batched.obs_idx[e:e + 1] - batched.w.sensor_rows[batched.first[e]].v_off + \
            alone.w.sensor_rows[alone.first[0]].v_off
        alone.reset()
        for t in range(3):
            o, r, d, tr, _ = alone.step(acts[t, e:e + 1])
            ob, rb = outs[t][0][e], outs[t][1][e]
            assert SS.rel_err(ob.cpu().numpy(), o[0].cpu().numpy()) < 1e-5, (e, t)
            assert abs(float(rb) - float(r[0])) <= 1e-5 * max(abs(float(r[0])), 1.0), (e, t)
