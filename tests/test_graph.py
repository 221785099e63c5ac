"""CUDA-graph replay of rollouts.

A trajectory recorded as CUDA graphs on its first forward / backward and replayed on later calls
with new actions gives the loss and action gradient of the same trajectory launched from the host
(pose-driven full tape and checkpointed, gripper-driven full tape); a batched environment replaying
its recorded step gives the observations and rewards of host-launched stepping.  The bound is the
run-to-run spread of the host-launched path (the scatters' atomic summation order differs between
runs) with a floor of 1e-5 (loss, observations) / 1e-4 (gradients) relative.  CUDA-event probes
recorded inside a graph time every replay's launches.
"""
import numpy as np
import pytest
import torch

from difftactile_gb300.envs import BatchedTactileEnv
from difftactile_gb300.trajectory import GripperTrajectory, PoseTrajectory, Trajectory
from difftactile_gb300.world import World
from tests import small_scenes as SS
from tests import test_gripper as TG
from tests import test_trajectory as TT

pytestmark = pytest.mark.gpu
STATE = ("p_state", "v_pos", "v_vel", "v_vpos", "v_cv", "r_state")


def snapshot(w):
    return {k: w.t[k][0].clone() for k in STATE}


def restore(w, snap):
    for k, v in snap.items():
        w.t[k][0].copy_(v)


def run(tr, w, snap, acts):
    restore(w, snap)
    loss = float(tr.forward(torch.as_tensor(acts, dtype=torch.float64, device=w.device)).item())
    g = tr.backward().cpu().numpy()
    torch.cuda.synchronize()
    assert w.error_word() == 0
    return loss, g


def compare(make_eager, make_graph, w, acts_list):
    snap = snapshot(w)
    eager, graph = make_eager(), make_graph()
    for i, acts in enumerate(acts_list):
        l0, g0 = run(eager, w, snap, acts)
        l1, g1 = run(eager, w, snap, acts)  # run-to-run spread of the host-launched path
        lg, gg = run(graph, w, snap, acts)
        tol_l = max(1e-5, 4 * abs(l1 - l0) / max(abs(l0), 1e-30))
        tol_g = max(1e-4, 4 * SS.rel_err(g1, g0))
        assert abs(lg - l0) <= tol_l * max(abs(l0), 1e-30), (i, lg, l0)
        assert SS.rel_err(gg, g0) <= tol_g, (i, SS.rel_err(gg, g0), tol_g)
    assert "fwd" in graph._graphs and ("bwd", 1.0) in graph._graphs
    return graph


@pytest.mark.parametrize("ckpt", [0, 2])
def test_pose_trajectory_graph_replay(cuda_lib, ckpt):
    env, terms = TT.scene()
    nf = PoseTrajectory.frames_needed(TT.T_STEPS, TT.SUB, ckpt)
    w = World([env], n_frames=nf, dt=TT.DT, grad_clip=0.0)
    graph = compare(lambda: PoseTrajectory(w, TT.T_STEPS, ckpt, terms),
                    lambda: PoseTrajectory(w, TT.T_STEPS, ckpt, terms, graph=True),
                    w, [TT.actions(s) for s in (5, 6, 7)])
    assert graph.launches > 0


@pytest.mark.parametrize("ckpt", [0, 1])
def test_rope_trajectory_graph_replay(cuda_lib, ckpt):
    """A pad pressing a rope of five pass pairs per substep, rope-tip loss: the rope solver and its
    adjoint run on the world's second stream (forked and joined inside every substep call), which the
    recorded graph holds as a branch; replays give the host-launched loss and gradient."""
    env = SS.rope_under_pad(n_rope=16)
    env = env.replace(ropes=[env.ropes[0].replace(iters=5)])
    tip = env.ropes[0].init_positions()[-1].astype(np.float64)
    rope_terms = ((0, tip + np.array([0.003, 0.002, -0.001])),)
    nf = PoseTrajectory.frames_needed(TT.T_STEPS, TT.SUB, ckpt)
    w = World([env], n_frames=nf, dt=TT.DT, grad_clip=0.0)
    assert w.w.aux_stream
    acts = []
    for s in (5, 6):
        a = TT.actions(s)
        a[:, 0, 1] = 0.2
        acts.append(a)
    compare(lambda: PoseTrajectory(w, TT.T_STEPS, ckpt, (), rope_terms=rope_terms),
            lambda: PoseTrajectory(w, TT.T_STEPS, ckpt, (), rope_terms=rope_terms, graph=True), w, acts)


def test_gripper_trajectory_graph_replay(cuda_lib):
    env, kin, terms = TG.setup()
    nf = Trajectory.frames_needed(TG.T_STEPS, TG.SUB, 0)
    w = World([env], n_frames=nf, dt=TG.DT, grad_clip=0.0)
    compare(lambda: GripperTrajectory(w, TG.T_STEPS, kin, ckpt_every=0, loss_terms=terms),
            lambda: GripperTrajectory(w, TG.T_STEPS, kin, ckpt_every=0, loss_terms=terms, graph=True),
            w, [TG.actions(s) for s in (6, 7)])


def test_probe_events_inside_graph(cuda_lib):
    env, terms = TT.scene()
    w = World([env], n_frames=TT.T_STEPS * TT.SUB + 1, dt=TT.DT, grad_clip=0.0)
    tr = PoseTrajectory(w, TT.T_STEPS, 0, terms, graph=True)
    acts = torch.as_tensor(TT.actions(), dtype=torch.float64, device=w.device)
    w.set_probe("fwd", 0, every=2)
    tr.forward(acts)  # host-launched, then recorded with the event pairs as graph nodes
    n_probed = (TT.T_STEPS * TT.SUB + 1) // 2
    assert len(w.probe_events) == n_probed and len(w.probe_graph_events) == n_probed
    w.probe_events.clear()
    for _ in range(2):
        tr.forward(acts)
        ms, n = w.probe_ms()
        assert n == n_probed and np.isfinite(ms) and 0.0 < ms < 100.0
    w.set_probe(None)


def test_sampled_backward_probe_keeps_the_adjoint(cuda_lib):
    """Probing every third backward substep splits the fused adjoint runs around the probed frames;
    the action gradient stays that of the unprobed sweep."""
    env, terms = TT.scene()
    w = World([env], n_frames=TT.T_STEPS * TT.SUB + 1, dt=TT.DT, grad_clip=0.0)
    snap = snapshot(w)
    tr = PoseTrajectory(w, TT.T_STEPS, 0, terms)
    acts = TT.actions()
    _, g0 = run(tr, w, snap, acts)
    _, g1 = run(tr, w, snap, acts)
    w.set_probe("bwd", 3, every=3)
    _, gp = run(tr, w, snap, acts)
    ms, n = w.probe_ms()
    w.set_probe(None)
    assert n == len(range(0, TT.T_STEPS * TT.SUB, 3)) and np.isfinite(ms)
    assert SS.rel_err(gp, g0) <= max(1e-4, 4 * SS.rel_err(g1, g0))


def test_batched_env_graph_replay(cuda_lib):
    scenes = [SS.pad_over_box(seed=1), SS.pad_over_box(seed=2, box_cells=(5, 4, 5))]
    rng = np.random.default_rng(3)
    acts = 0.05 * rng.standard_normal((4, len(scenes), 6))
    acts[..., 1] -= 0.1
    out = []
    for graph in (False, False, True):
        env = BatchedTactileEnv(scenes, substeps=4, time_limit=4, n_obs_nodes=8, seed=1, graph=graph)
        env.reset()
        out.append([tuple(x.cpu().numpy() for x in env.step(acts[t])[:2]) for t in range(4)])
        assert env.w.error_word() == 0
        assert (env._graph is not None) == graph
    for t in range(4):
        spread = SS.rel_err(out[1][t][0], out[0][t][0])
        assert SS.rel_err(out[2][t][0], out[0][t][0]) <= max(1e-5, 4 * spread), t
        assert np.allclose(out[2][t][1], out[0][t][1], rtol=1e-5, atol=1e-6), t
