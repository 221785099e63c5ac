"""The rollout's checkpoint/recompute schedule on the host (Trajectory, tasks/grasp_plastic.py:594-648
with memory_to_cache / memory_from_cache, object_model/mpm_elastic.py:300-320): a stand-in world on the
CPU runs a small nonlinear system on the same state tensors, frame layout and parity-buffered adjoints
as the CUDA world, so that any state the schedule fails to save, restore or recompute changes the
gradient.  Full tape, one checkpoint per step, and checkpoints every k steps with a ragged last
segment, for odd and even substep counts, all give torch autograd's gradient of the same rollout.
Also the split of a probed adjoint run into fused runs and staged frames (World.substeps_bwd)."""
import types

import numpy as np
import pytest
import torch

from difftactile_gb300.trajectory import Trajectory
from difftactile_gb300.world import World

NP, NV, NR = 3, 2, 2                       # particles, sensor vertices, rope particles
STATE = ("p_state", "v_pos", "v_vel", "v_vpos", "r_state")
ADJ = ("p_adj", "v_adj_pos", "v_adj_vel", "v_adj_vpos", "r_adj")
SHAPES = ((6, NP, 4), (NV, 4), (NV, 4), (NV, 4), (2, NR, 4))
NZ = sum(int(np.prod(s)) for s in SHAPES)  # flattened state size
NC = 3                                     # controls per step
H = 0.05


class System:
    """z' = z + H tanh(W z) + H B c: every state tensor feeds every other one."""

    def __init__(self, seed=0):
        g = torch.Generator().manual_seed(seed)
        self.W = (torch.randn(NZ, NZ, generator=g, dtype=torch.float64) * (1.5 / NZ ** 0.5))
        self.B = torch.randn(NZ, NC, generator=g, dtype=torch.float64)
        self.z0 = torch.randn(NZ, generator=g, dtype=torch.float64)
        self.q = torch.randn(NZ, generator=g, dtype=torch.float64)

    def step(self, z, c):
        return z + H * torch.tanh(self.W.to(z) @ z) + H * (self.B.to(z) @ c)

    def loss(self, z):
        return (self.q.to(z) * z).sum() + 0.5 * (z * z).sum()


class FakeLib:
    """The two loss entry points the trajectory calls (marker loss and its adjoint), on the fake world."""

    def __init__(self, world):
        self.w = world
        self.traj = None

    def dt_marker_loss(self, wp, s, f, layer, tg, loss, stream):
        self.traj.loss.fill_(float(self.w.sys.loss(self.w.z(f).double())))
        return 0

    def dt_marker_loss_bwd(self, wp, s, f, layer, tg, loss_bar, stream):
        z = self.w.z(f).double()
        self.w.set_adj(f & 1, loss_bar * (self.w.sys.q + z))
        return 0


class FakeWorld:
    """The CUDA world's host-visible contract for a rollout: frames of state tensors, substep(f) writes
    frame f + 1 from frame f and the control velocities of frame f, substeps_bwd(hi, lo) maps the adjoint
    of frame f + 1 (buffer (f + 1) & 1) to that of frame f (buffer f & 1) using the state of frame f, and
    accumulates the control adjoint per frame."""

    device = "cpu"
    probe = None
    stream_override = None
    wp = stream = None

    def __init__(self, n_frames, sys):
        self.n_frames, self.sys = n_frames, sys
        self.n_particles, self.n_verts, self.n_rope_particles = NP, NV, NR
        self.sensor_rows = [types.SimpleNamespace(nv=NV)]
        self.t = {k: torch.zeros((n_frames,) + s) for k, s in zip(STATE, SHAPES)}
        self.t.update({k: torch.zeros((2,) + s) for k, s in zip(ADJ, SHAPES)})
        # slot j holds particle p_mat[j] (the CUDA world's material index plays this part: it follows its
        # particle through a re-binning); the system runs in particle order, whatever the slot order
        self.t["p_mat"] = torch.arange(NP, dtype=torch.int32)
        self.rebins = 0
        self.cv = torch.zeros((n_frames, NC))
        self.adj_cv = torch.zeros((n_frames, NC))
        self.lib = FakeLib(self)
        self.calls = []
        self.taped = [False] * n_frames

    def _canon(self, k, x):
        """particle-order view of a slot-ordered particle tensor [6, NP, 4]"""
        return x[:, torch.argsort(self.t["p_mat"].long())] if k in ("p_state", "p_adj") else x

    def _slots(self, k, x):
        return x[:, self.t["p_mat"].long()] if k in ("p_state", "p_adj") else x

    def z(self, f):
        return torch.cat([self._canon(k, self.t[k][f]).reshape(-1) for k in STATE])

    def set_z(self, f, z):
        o = 0
        for k in STATE:
            n = self.t[k][f].numel()
            self.t[k][f].copy_(self._slots(k, z[o:o + n].reshape(self.t[k][f].shape)))
            o += n

    def adj(self, b):
        return torch.cat([self._canon(k, self.t[k][b]).reshape(-1) for k in ADJ])

    def set_adj(self, b, a):
        o = 0
        for k in ADJ:
            n = self.t[k][b].numel()
            self.t[k][b].copy_(self._slots(k, a[o:o + n].reshape(self.t[k][b].shape)))
            o += n

    def rebin(self, frame, src):
        """World.rebin's contract: src[j] = the old slot of new slot j (here: slots sorted by the first
        coordinate); frame's records and the slot -> particle map follow it, nothing else does."""
        src.copy_(torch.argsort(self.t["p_state"][frame, 0, :, 0], stable=True).to(torch.int32))
        s = src.long()
        self.rebins += int(not torch.equal(s, torch.arange(NP)))
        self.t["p_state"][frame].copy_(self.t["p_state"][frame][:, s])
        self.t["p_mat"].copy_(self.t["p_mat"][s])

    def rebin_permute(self, src, inverse, adj_buf=-1):
        s = src.long()

        def perm(x):  # x indexed by slot along dim 0
            if not inverse:
                return x[s]
            out = torch.empty_like(x)
            out[s] = x
            return out

        self.t["p_mat"].copy_(perm(self.t["p_mat"]))
        if adj_buf >= 0:
            self.t["p_adj"][adj_buf].copy_(perm(self.t["p_adj"][adj_buf].transpose(0, 1)).transpose(0, 1))

    tape_on = True

    def step_begin(self):
        self.calls.append("begin")

    def set_tape(self, on):
        self.tape_on = bool(on)

    def substep(self, f):
        assert 0 <= f < self.n_frames - 1
        self.taped[f] = self.tape_on  # whether the substep's tape (read by its adjoint) was written
        self.set_z(f + 1, self.sys.step(self.z(f).double(), self.cv[f].double()))

    def substeps_bwd(self, f_hi, f_lo):
        assert 0 <= f_lo < f_hi < self.n_frames
        W = self.sys.W
        for f in reversed(range(f_lo, f_hi)):
            assert self.taped[f], f"adjoint of frame {f} whose forward substep wrote no tape"
            a = self.adj((f + 1) & 1).double()
            th = torch.tanh(W @ self.z(f).double())
            self.adj_cv[f] += (H * (self.sys.B.T @ a)).float()
            self.set_adj(f & 1, a + H * (W.T @ ((1 - th * th) * a)))

    def copy_frame(self, src, dst):
        self.set_z(dst, self.z(src))

    def adj_clear(self):
        for k in ADJ:
            self.t[k].zero_()
        self.adj_cv.zero_()


class LinearTrajectory(Trajectory):
    """Controls = 2 x actions, held over each step's substeps."""

    def controls(self, actions):
        return 2.0 * actions

    def _apply(self, t, f0):
        self.w.cv[f0:f0 + self.S] = self.ctrl32[t]

    def _apply_bwd(self, t, f0):
        self.ctrl_bar[t] += self.w.adj_cv[f0:f0 + self.S].sum(0)
        self.w.adj_cv[f0:f0 + self.S] = 0


def autograd_reference(sys, actions, S):
    a = actions.clone().requires_grad_(True)
    z = sys.z0.clone().requires_grad_(True)
    zz = z
    for t in range(a.shape[0]):
        for _ in range(S):
            zz = sys.step(zz, 2.0 * a[t])
    L = sys.loss(zz)
    ga, gz = torch.autograd.grad(L, (a, z))
    return float(L.detach()), ga, gz


@pytest.mark.parametrize("T,S,k", [(5, 3, 0), (5, 4, 0), (5, 3, 1), (5, 4, 1), (7, 3, 3), (7, 2, 3), (6, 1, 2),
                                   (4, 3, 4), (4, 5, 9)])
def test_schedule_gives_the_rollouts_gradient(T, S, k):
    sys = System(seed=T * 100 + S * 10 + k)
    actions = torch.randn(T, NC, generator=torch.Generator().manual_seed(7), dtype=torch.float64)
    w = FakeWorld(Trajectory.frames_needed(T, S, k), sys)
    w.set_z(0, sys.z0.float())
    tr = LinearTrajectory(w, T, ckpt_every=k, loss_terms=[(0, 0, np.zeros((NV, 3)))])
    w.lib.traj = tr
    assert (tr.S, tr.full) == (S, k == 0)
    L = float(tr.forward(actions))
    g = tr.backward()
    L_ref, g_ref, gz_ref = autograd_reference(sys, actions, S)
    assert abs(L - L_ref) <= 1e-4 * abs(L_ref)
    assert float((g - g_ref).norm() / g_ref.norm()) < 1e-4
    gz = w.adj(0).double()                          # initial-state adjoint in frame 0's buffer
    assert float((gz - gz_ref).norm() / gz_ref.norm()) < 1e-4
    # a second sweep of the same forward, and one after adjoint_at stopped mid-rollout (both re-run the
    # steps over the world's frames: the final frame the loss adjoint starts from is kept for them)
    assert float((tr.backward() - g_ref).norm() / g_ref.norm()) < 1e-4
    tr.adjoint_at(T - 1, S - 1)
    tr.adjoint_at(T // 2, 0)
    assert float((tr.backward() - g_ref).norm() / g_ref.norm()) < 1e-4
    # a second rollout from the same start repeats the first (checkpoints are rewritten, not appended)
    w.set_z(0, sys.z0.float())
    assert abs(float(tr.forward(actions)) - L) <= 1e-6 * abs(L)
    assert float((tr.backward() - g).abs().max()) <= 1e-6 * float(g.abs().max())


@pytest.mark.parametrize("T,S,k,r", [(6, 3, 1, 1), (6, 4, 1, 2), (7, 3, 2, 1), (7, 2, 3, 1), (9, 1, 2, 2)])
def test_rebinning_schedule_gives_the_rollouts_gradient(T, S, k, r):
    """Checkpointed rollouts that re-sort the particle slots at checkpoints (rebin_every = r) give
    autograd's action and initial-state gradients: every re-binning the backward sweep crosses is
    undone on the adjoint it carries and on the slot -> particle map; the slot order at the end of the
    sweep is the rollout's start order again.  Also after adjoint_at left the world mid-rollout."""
    sys = System(seed=T * 100 + S * 10 + k + r)
    actions = torch.randn(T, NC, generator=torch.Generator().manual_seed(7), dtype=torch.float64)
    w = FakeWorld(Trajectory.frames_needed(T, S, k), sys)
    w.set_z(0, sys.z0.float())
    tr = LinearTrajectory(w, T, ckpt_every=k, loss_terms=[(0, 0, np.zeros((NV, 3)))], rebin_every=r)
    w.lib.traj = tr
    L = float(tr.forward(actions))
    assert w.rebins > 0
    g = tr.backward()
    L_ref, g_ref, gz_ref = autograd_reference(sys, actions, S)
    assert abs(L - L_ref) <= 1e-4 * abs(L_ref)
    assert float((g - g_ref).norm() / g_ref.norm()) < 1e-4
    assert float((w.adj(0).double() - gz_ref).norm() / gz_ref.norm()) < 1e-4
    assert torch.equal(w.t["p_mat"], torch.arange(NP, dtype=torch.int32))
    # inspect an adjoint mid-rollout, then a full backward again from the same forward
    w.set_z(0, sys.z0.float())
    tr.forward(actions)
    tr.adjoint_at(T // 2, 0)
    assert float((tr.backward() - g_ref).norm() / g_ref.norm()) < 1e-4
    assert torch.equal(w.t["p_mat"], torch.arange(NP, dtype=torch.int32))


def test_rebinning_needs_checkpoints():
    sys = System()
    with pytest.raises(ValueError, match="rebin_every"):
        LinearTrajectory(FakeWorld(Trajectory.frames_needed(4, 3, 0), sys), 4, ckpt_every=0, rebin_every=1)


def test_checkpoint_storage_per_mode():
    sys = System()
    w = FakeWorld(Trajectory.frames_needed(7, 3, 3), sys)
    tr = LinearTrajectory(w, 7, ckpt_every=3)
    assert tr.n_ck == 3 and tr.ck_p.shape[0] == 3 and tr.seg_p.shape[0] == 3
    w1 = FakeWorld(Trajectory.frames_needed(7, 3, 1), sys)
    tr1 = LinearTrajectory(w1, 7, ckpt_every=1)
    assert tr1.n_ck == 7 and not hasattr(tr1, "seg_p")
    wf = FakeWorld(Trajectory.frames_needed(7, 3, 0), sys)
    trf = LinearTrajectory(wf, 7, ckpt_every=0)
    assert trf.n_ck == 0 and trf.f_end == 21 and not hasattr(trf, "ck_p")
    with pytest.raises(ValueError, match="not a multiple"):
        LinearTrajectory(FakeWorld(20, sys), 7, ckpt_every=0)


@pytest.mark.parametrize("f_hi,f_lo,every", [(20, 0, 1), (20, 0, 5), (21, 3, 4), (7, 6, 3), (9, 0, 25), (50, 0, 25)])
def test_probed_adjoint_runs_cover_each_frame_once(f_hi, f_lo, every):
    w = World.__new__(World)
    calls = []
    w._substeps_bwd = lambda hi, lo: calls.append(("run", hi, lo))
    w._staged = lambda name, f, n, kind: calls.append(("stage", f, n))
    w.set_probe("bwd", 2, every=every)
    w.substeps_bwd(f_hi, f_lo)
    frames = []
    for c in calls:
        if c[0] == "run":
            assert c[1] > c[2]
            frames += list(reversed(range(c[2], c[1])))
        else:
            assert c[2] == 4                        # the four backward stages
            frames.append(c[1])
    assert frames == list(reversed(range(f_lo, f_hi)))
    assert [c[1] for c in calls if c[0] == "stage"] == [f for f in reversed(range(f_lo, f_hi)) if f % every == 0]
    w.set_probe(None)
    calls.clear()
    w.substeps_bwd(f_hi, f_lo)
    assert calls == [("run", f_hi, f_lo)]            # unprobed: one fused run


def test_actions_of_another_horizon_are_refused_before_any_step():
    sys = System()
    w = FakeWorld(Trajectory.frames_needed(4, 3, 1), sys)
    tr = LinearTrajectory(w, 4, ckpt_every=1)
    with pytest.raises(ValueError, match="control steps"):
        tr.forward(torch.zeros(3, NC, dtype=torch.float64))
    assert float(w.cv.abs().max()) == 0.0 and w.calls == []
