"""Re-binning of the particles by cell (dt_rebin, dt_rebin_permute; Trajectory(rebin_every=r)).

* dt_rebin on a world whose particles start in a random slot order: src is a permutation; in the new
  order every environment's slots are sorted by the grid node of their base cell (the key computed
  here on the host), ties by old slot; every particle stays in its environment's range; the state in
  the caller's order, the material index of every particle and the records themselves are unchanged;
* dt_rebin_permute and its inverse restore an adjoint buffer, the material index and the slot maps;
* a checkpointed pose-controlled rollout that re-bins at every checkpoint gives the loss, the action
  gradient, the initial-state adjoint and the material gradient of the same rollout without
  re-binning (the two differ only in the order the atomics add: 1e-5 on the loss, 1e-3 on gradients).
"""
import numpy as np
import pytest
import torch

from difftactile_gb300 import scene as S
from difftactile_gb300.trajectory import PoseTrajectory
from difftactile_gb300.world import World
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4


def two_envs():
    a = SS.pad_over_box(n=32)
    b = SS.elastic_cube(n=24, side_cells=6, seed=3, v=(0.3, -0.2, 0.1))
    layer = (b.x[:, 1] > np.median(b.x[:, 1])).astype(np.int32)
    b = b.replace(materials=[S.Material(5e3, 0.3, 50.0, S.MODEL_COROTATED), S.Material(2e4, 0.3, 50.0, S.MODEL_COROTATED)],
                  mat=layer)
    return [a, b]


def host_keys(w, x):
    """base grid node of each slot (x: [N,3] slots), the layout of the header's grid comment"""
    keys = np.zeros(len(x), np.int64)
    for r in w.env_rows:
        sl = slice(r.p_begin, r.p_end)
        n = np.array(r.n[:])
        nb = np.array(r.nb[:])
        c = np.clip(np.floor(x[sl].astype(np.float32) * np.float32(r.inv_dx) - np.float32(0.5)), 0, n - 1).astype(np.int64)
        b = ((c[:, 0] >> 2) * nb[1] + (c[:, 1] >> 2)) * nb[2] + (c[:, 2] >> 2)
        keys[sl] = r.node_off + 64 * b + 16 * (c[:, 0] & 3) + 4 * (c[:, 1] & 3) + (c[:, 2] & 3)
    return keys


def test_rebin_sorts_by_cell_and_keeps_every_particle(cuda_lib):
    rng = np.random.default_rng(0)
    envs = []
    for e in two_envs():  # particles in a random order, kept as given (no sort at construction)
        o = rng.permutation(e.n_particles)
        envs.append(e.replace(x=e.x[o], v=None if e.v is None else e.v[o], mat=None if e.mat is None else e.mat[o]))
    w = World(envs, n_frames=2, dt=DT, sort_particles=False)
    N = w.n_particles
    before = {k: v.clone() for k, v in w.particles(0).items()}
    mat_before = w.t["p_mat"][w._inv_perm_t].clone()
    state0, perm0, mat0 = w.t["p_state"][0].clone(), w._perm_t.clone(), w.t["p_mat"].clone()
    src = torch.empty(N, dtype=torch.int32, device=w.device)
    w.rebin(0, src)
    torch.cuda.synchronize()
    s = src.cpu().numpy().astype(np.int64)
    assert np.array_equal(np.sort(s), np.arange(N))
    keys = host_keys(w, w.t["p_state"][0, 0, :, :3].cpu().numpy())
    for r in w.env_rows:
        sl = slice(r.p_begin, r.p_end)
        assert s[sl].min() >= r.p_begin and s[sl].max() < r.p_end
        k, o = keys[sl], s[sl]
        assert np.all((k[1:] > k[:-1]) | ((k[1:] == k[:-1]) & (o[1:] > o[:-1])))
    # the records moved whole, the material index and the caller's index with them
    assert torch.equal(w.t["p_state"][0], state0[:, src.long()])
    assert torch.equal(w.t["p_mat"], mat0[src.long()])
    assert torch.equal(w._perm_t, perm0[src.long()])
    assert torch.equal(w._inv_perm_t[w._perm_t], torch.arange(N, device=w.device))
    after = w.particles(0)
    assert all(torch.equal(after[k], before[k]) for k in before)
    assert torch.equal(w.t["p_mat"][w._inv_perm_t], mat_before)
    runs_before = float((np.diff(host_keys(w, state0[0, :, :3].cpu().numpy())) == 0).mean())
    runs_after = float((np.diff(keys) == 0).mean())
    print("same-cell neighbours", runs_before, "->", runs_after)
    assert runs_after > runs_before


def test_rebin_permute_round_trip(cuda_lib):
    w = World(two_envs(), n_frames=2, dt=DT)
    N = w.n_particles
    src = torch.empty(N, dtype=torch.int32, device=w.device)
    g = torch.Generator(device=w.device).manual_seed(1)
    w.t["p_state"][0, 0, :, :3] += 0.01 * torch.randn((N, 3), device=w.device, generator=g)  # move across cells
    w.rebin(0, src)
    adj = torch.randn(w.t["p_adj"][1].shape, device=w.device, generator=g)
    w.t["p_adj"][1].copy_(adj)
    mat, perm, inv = w.t["p_mat"].clone(), w._perm_t.clone(), w._inv_perm_t.clone()
    w.rebin_permute(src, inverse=False, adj_buf=1)
    torch.cuda.synchronize()
    assert torch.equal(w.t["p_adj"][1], adj[:, src.long()])
    assert torch.equal(w.t["p_mat"], mat[src.long()])
    w.rebin_permute(src, inverse=True, adj_buf=1)
    torch.cuda.synchronize()
    assert torch.equal(w.t["p_adj"][1], adj)
    assert torch.equal(w.t["p_mat"], mat) and torch.equal(w._perm_t, perm) and torch.equal(w._inv_perm_t, inv)
    assert not torch.equal(src.long(), torch.arange(N, device=w.device))


T_STEPS, SUB = 4, 5


def rollout(rebin_every):
    env = SS.pad_over_box(n=32, model=S.MODEL_VON_MISES, yield_stress=5.0)
    sp = env.sensors[0]
    terms = ((0, int(sp.layer.max()), 1e-4 * np.random.default_rng(21).standard_normal(sp.verts.shape)),)
    w = World([env], n_frames=PoseTrajectory.frames_needed(T_STEPS, SUB, 1), dt=DT, grad_clip=0.0)
    tr = PoseTrajectory(w, T_STEPS, 1, terms, rebin_every=rebin_every)
    a = np.zeros((T_STEPS, 1, 6))
    a[:, 0, 1] = -0.3
    a[:, 0, 0] = 0.2  # slide: particles change cells
    acts = torch.as_tensor(a, dtype=torch.float64, device=w.device)
    loss = float(tr.forward(acts).item())
    g = tr.backward().cpu().numpy()
    torch.cuda.synchronize()
    assert w.error_word() == 0
    adj = {k: v.cpu().numpy() for k, v in w.particle_adjoint(0).items()}
    return w, tr, loss, g, adj, tr.material_grad().cpu().numpy()


def test_rebinned_rollout_matches_plain(cuda_lib):
    w0, _, L0, g0, a0, m0 = rollout(0)
    w1, tr1, L1, g1, a1, m1 = rollout(1)
    moved = [int((tr1.ck_src[s].long() != torch.arange(w1.n_particles, device=w1.device)).sum())
             for s in range(1, T_STEPS)]
    errs = {"loss": abs(L1 - L0) / abs(L0), "actions": SS.rel_err(g1, g0), "mat": SS.rel_err(m1, m0)}
    errs.update({f"adj_{k}": SS.rel_err(a1[k], a0[k]) for k in a0})
    print("re-binned slots per checkpoint", moved, "errors", errs)
    assert moved[0] > 0  # the construction's block-Morton order becomes the block-row order of the nodes
    assert errs["loss"] < 1e-5
    assert max(v for k, v in errs.items() if k != "loss") < 1e-3, errs
    # the rollout's start order again at the end of the sweep
    assert torch.equal(w1._perm_t, torch.as_tensor(w1.perm, device=w1.device))
