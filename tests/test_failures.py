"""Failure detection without a GPU fault: bad arguments come back as status codes (and as DtError
from the Python binding) before any launch; device-side problems (non-finite state, a particle that
left the grid's safe band, a grid tape that ran out of reserved blocks) set bits of the world's
error word, are skipped or clamped instead of trapping, and the device stays usable afterwards.
Faults are injected on the host only (a NaN in the input state, an undersized tape, an out-of-range
frame).  Repeating a substep from the same state gives the same result to atomic-ordering noise."""
import ctypes

import numpy as np
import pytest
import torch

from difftactile_gb300 import _native as N
from tests import small_scenes as SS

DT = 1e-4


def test_argument_errors_are_status_codes_without_a_device():
    lib = N.load()  # loads without a GPU; every call below returns at its argument check
    w = N.DtWorld()
    w.n_frames = 3
    wp = ctypes.byref(w)
    assert lib.dt_substep_fwd(wp, 2, None) == -1          # frame f + 1 out of range
    assert lib.dt_substep_fwd(wp, -1, None) == -1
    assert lib.dt_substep_fwd(None, 0, None) == -1        # no world
    assert lib.dt_substep_bwd(wp, 5, None) == -1
    assert lib.dt_substeps_bwd(wp, 1, 1, None) == -1      # empty range
    assert lib.dt_copy_frame(wp, 0, 3, None) == -1
    assert lib.dt_pose_control_vel_all(wp, None, 1.0, 0, 1, None) == -1
    assert lib.dt_pose_control_vel_bwd_all(wp, None, 1.0, None, 0, 1, None) == -1
    buf = ctypes.c_int(0)
    assert lib.dt_rebin(wp, 0, None, None, None, None) == -1                  # no material index / permutation
    assert lib.dt_rebin(wp, 3, ctypes.byref(buf), ctypes.byref(buf), ctypes.byref(buf), None) == -1  # frame
    assert lib.dt_rebin(None, 0, ctypes.byref(buf), ctypes.byref(buf), ctypes.byref(buf), None) == -1
    assert lib.dt_rebin_permute(wp, 2, 0, ctypes.byref(buf), ctypes.byref(buf), ctypes.byref(buf), None) == -1
    assert lib.dt_rebin_permute(wp, 0, 1, ctypes.byref(buf), ctypes.byref(buf), ctypes.byref(buf), None) == -1
    assert lib.dt_rebin_scratch_bytes(None) == 0
    with pytest.raises(N.DtError, match="DT_ERR_ARG"):
        N.check(lib.dt_substep_fwd(wp, 7, None), "dt_substep_fwd")


def test_world_on_host_memory_is_refused():
    from difftactile_gb300.world import World
    with pytest.raises(ValueError, match="CUDA device"):
        World([SS.pad_over_box()], n_frames=3, dt=DT, device="cpu")


@pytest.mark.gpu
def test_out_of_range_frame_raises_before_launch(cuda_lib):
    from difftactile_gb300.world import World
    w = World([SS.pad_over_box()], n_frames=3, dt=DT)
    with pytest.raises(N.DtError, match="DT_ERR_ARG"):
        w.substep(2)
    with pytest.raises(N.DtError, match="DT_ERR_ARG"):
        w.copy_frame(0, 9)
    torch.cuda.synchronize()
    assert w.error_word() == 0


@pytest.mark.gpu
def test_nan_state_is_flagged_and_the_device_stays_usable(cuda_lib):
    from difftactile_gb300.world import World
    env = SS.pad_over_box()
    w = World([env], n_frames=4, dt=DT)
    x0 = w.t["p_state"][0].clone()
    v = np.zeros((env.n_particles, 3), np.float32)
    v[env.n_particles // 2] = np.nan
    w.set_particles(0, v=v)
    w.step_begin()
    for f in range(3):
        w.substep(f)
    torch.cuda.synchronize()
    err = w.error_word()
    assert err & 4, err                                 # non-finite value
    # recovery: same world, clean state
    w.clear_error()
    w.t["p_state"][0].copy_(x0)
    w.step_begin()
    for f in range(3):
        w.substep(f)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    assert torch.isfinite(w.particles(3)["x"]).all()


@pytest.mark.gpu
def test_undersized_grid_tape_is_flagged_not_overrun(cuda_lib):
    from difftactile_gb300.world import World
    env = SS.pad_over_box()
    w = World([env], n_frames=2, dt=DT, tape_blocks=2)
    w.step_begin()
    w.substep(0)
    torch.cuda.synchronize()
    assert w.error_word() & 2                           # grid tape capacity exceeded
    assert int(w.t["tape_bcount"][0]) > 2               # the frame had more active blocks than reserved
    w.clear_error()
    big = World([env], n_frames=2, dt=DT)
    big.step_begin()
    big.substep(0)
    torch.cuda.synchronize()
    assert big.error_word() == 0


@pytest.mark.gpu
def test_rope_iterations_beyond_the_workspace_are_flagged_not_overrun(cuda_lib):
    """A rope of six pass pairs whose adjoint workspace is declared for only two (max_rope_iters = 2):
    the adjoint of that rope is skipped and DT_DEVERR_ROPE_ITERS set, nothing is written past the
    workspace, and with the workspace declared again the same world's adjoint runs clean."""
    from difftactile_gb300.world import World
    env = SS.rope_under_pad()
    env = env.replace(ropes=[env.ropes[0].replace(iters=6)])
    w = World([env], n_frames=2, dt=DT, grad_clip=0.0)
    assert w.t["r_work"] is not None and w.w.max_rope_iters == 6
    guard = w.t["r_work"].clone()
    w.step_begin()
    w.substep(0)
    w.adj_clear()
    w.t["r_adj"][1].fill_(1.0)
    w.w.max_rope_iters = 2
    w.substep_bwd(0)
    torch.cuda.synchronize()
    assert w.error_word() & 8                            # the rope's passes exceed the declared workspace
    assert torch.equal(w.t["r_work"][4:], guard[4:])     # nothing written beyond 2 x 2 pass inputs
    w.clear_error()
    w.w.max_rope_iters = 6
    w.adj_clear()
    w.t["r_adj"][1].fill_(1.0)
    w.substep_bwd(0)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    assert torch.isfinite(w.t["r_adj"][0]).all() and float(w.t["r_adj"][0].abs().sum()) > 0


@pytest.mark.gpu
def test_repeated_substep_is_reproducible(cuda_lib):
    from difftactile_gb300.world import World
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    out = []
    for _ in range(2):
        w = World([env], n_frames=3, dt=DT)
        for s, c in enumerate(cv):
            w.set_control_velocity(s, c)
        w.step_begin()
        w.substep(0)
        w.substep(1)
        torch.cuda.synchronize()
        assert w.error_word() == 0
        out.append({k: t.double().cpu().numpy() for k, t in w.particles(2).items()})
    for k in ("x", "v", "C", "F"):
        assert SS.rel_err(out[1][k], out[0][k]) < 1e-5, k
