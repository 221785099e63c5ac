"""The three 27-node scatter strategies (shared-memory gather, per-particle global REDs, warp
segmented reduction over runs of particles sharing a base cell) give the oracle's forward state
and adjoint, with particles in Morton order (long runs) and in the user's order (runs of one),
and across environment boundaries inside a warp."""
import numpy as np
import pytest
import torch

from difftactile_gb300.world import World
from oracle import oracle as O
from tests import small_scenes as SS
from tests.test_parity_bwd import base_point, gpu_grads, loss_weights
from tests.test_parity_fwd import compare, run_oracle

pytestmark = pytest.mark.gpu
DT = 1e-4
MODES = {"tile": 0, "global": 1, "warp": 2, "smem": 3}


@pytest.mark.parametrize("sort", [True, False])
@pytest.mark.parametrize("mode", list(MODES))
def test_forward_three_substeps(cuda_lib, mode, sort):
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = World([env], n_frames=4, dt=DT, scatter_mode=MODES[mode], sort_particles=sort)
    for s, c in enumerate(cv):
        w.set_control_velocity(s, c)
    w.step_begin()
    for f in range(3):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    st, _ = run_oracle(env, 3, cv)
    compare(w, 3, st)


@pytest.mark.parametrize("mode", list(MODES))
def test_adjoint_one_substep(cuda_lib, mode):
    env = SS.pad_over_box()
    st0, cv = base_point(env, 7)
    W = loss_weights(env, env.n_particles, 8)
    g = gpu_grads(env, st0, cv, W, 1, scatter_mode=MODES[mode])
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    ref = o.substep_bwd({k: (v if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}, W,
                        cv=cv, cv1=cv)
    errs = {k: SS.rel_err(g[k], ref[k]) for k in ("x", "v", "C", "F")}
    errs["pos"] = SS.rel_err(g["pos"][0], ref["pos"][0])
    assert max(errs.values()) < 1e-3, errs


def test_warp_runs_across_env_boundaries(cuda_lib):
    """Env sizes that are not multiples of 32 put two environments in one warp; equal cells of
    different environments must not merge into one run."""
    e0 = SS.elastic_cube(n=32, side_cells=3, ppc=3, seed=1)
    e1 = SS.elastic_cube(n=32, side_cells=3, ppc=3, seed=2)
    assert e0.n_particles % 32 and e0.n_particles == e1.n_particles
    w = World([e0, e1], n_frames=3, dt=DT, scatter_mode=MODES["warp"])
    w.step_begin()
    for f in range(2):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    for e, env in enumerate((e0, e1)):
        st, _ = run_oracle(env, 2)
        compare(w, 2, st, env_idx=e)


@pytest.mark.parametrize("mode,p_block,depth,ppt,adj", [
    ("warp", 64, 0, 1, 0), ("warp", 256, 0, 1, 0), ("global", 64, 0, 1, 0), ("global", 256, 0, 1, 0),
    ("warp", 128, 1, 1, 0), ("warp", 128, 2, 1, 0), ("warp", 256, 1, 1, 0), ("warp", 128, 1, 2, 0),
    ("warp", 64, 0, 2, 0), ("global", 256, 0, 2, 0), ("tile", 128, 0, 2, 0), ("smem", 128, 0, 1, 0),
    ("smem", 128, 0, 2, 0), ("smem", 64, 0, 1, 0), ("smem", 256, 0, 2, 0),
    ("warp", 64, 1, 2, 2), ("warp", 64, 1, 2, 3), ("warp", 128, 0, 1, 1), ("global", 128, 0, 1, 2)])
def test_particle_block_sizes(cuda_lib, mode, p_block, depth, ppt, adj):
    """Particle-role CTAs of 64 and 256 threads, capped segmented reductions, two chunks of particles
    per CTA and a G2P adjoint scatter of another depth than the P2G's (scatter_depth_adj: 1, 2, or 3
    for whole runs; ignored outside the warp scatter) — the autotuner's other shapes; 1,152
    particles: an odd number of chunks, so the last two-chunk CTA has one — give the oracle's forward
    state after three substeps and its one-substep adjoint."""
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    kw = dict(scatter_mode=MODES[mode], p_block=p_block, scatter_depth=depth, p_per_thread=ppt, scatter_depth_adj=adj)
    w = World([env], n_frames=4, dt=DT, **kw)
    for s, c in enumerate(cv):
        w.set_control_velocity(s, c)
    w.step_begin()
    for f in range(3):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    st, _ = run_oracle(env, 3, cv)
    compare(w, 3, st)
    st0, cv0 = base_point(env, 7)
    W = loss_weights(env, env.n_particles, 8)
    g = gpu_grads(env, st0, cv0, W, 1, **kw)
    o = O.Oracle(env, DT, np.float64, grad_clip=0.0)
    ref = o.substep_bwd({k: (v if not isinstance(v, list) else [a.copy() for a in v]) for k, v in st0.items()}, W,
                        cv=cv0, cv1=cv0)
    errs = {k: SS.rel_err(g[k], ref[k]) for k in ("x", "v", "C", "F")}
    assert max(errs.values()) < 1e-3, errs
