"""dt_substep_fwd_noalloc: the forward substep for callers that cannot allocate device memory (their
buffers belong to another allocator, e.g. a framework's caching allocator or an arena reserved at
start-up under a fixed memory budget).  Its scratch lives in a static device array inside the
library; this test passes a descriptor whose scratch pointers are NULL and checks, over two calls in a
row, that the result equals the allocating entry point's (dt_substep_fwd) within the parity
tolerances of the forward tests.  Collected last so that a failure here stops a run only after every
other test has run."""
import ctypes

import numpy as np
import pytest
import torch

from difftactile_gb300 import _native as N
from difftactile_gb300.world import World
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4
SCRATCH = ("g_acc", "g_vout", "blk_flag", "tape_blist", "tape_bcount", "tape_acc", "tape_vout", "tape_cidx",
           "tri_cent", "g_adj_vout", "g_adj_acc")


def _world(env, cv):
    w = World([env], n_frames=3, dt=DT)
    w.set_control_velocity(0, cv)
    w.step_begin()
    return w


def test_noalloc_substep_matches_allocating_entry_point(cuda_lib):
    env = SS.pad_over_box()
    cv = SS.control_velocity(env.sensors[0])
    ref = _world(env, cv)
    ref.substep(0)
    ref.substep(1)

    w = _world(env, cv)
    bare = N.DtWorld.from_buffer_copy(w.w)  # same inputs/outputs, no scratch
    for name in SCRATCH:
        setattr(bare, name, None)
    stream = torch.cuda.current_stream().cuda_stream
    for f in (0, 1):  # two calls in a row share (and must re-clear) the static scratch
        rc = w.lib.dt_substep_fwd_noalloc(ctypes.byref(bare), f, stream)
        assert rc == 0, N.ERRORS.get(rc, rc)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    for f in (1, 2):
        a, b = ref.particles(f), w.particles(f)
        for k in ("x", "F"):
            assert SS.rel_err(b[k].cpu().numpy(), a[k].cpu().numpy()) < 1e-5, (f, k)
        for k in ("v", "C"):
            assert SS.rel_err(b[k].cpu().numpy(), a[k].cpu().numpy()) < 1e-4, (f, k)
        for name in ("v_pos", "v_vel"):
            assert SS.rel_err(w.sensor_frame(name, f, 0).cpu().numpy(),
                              ref.sensor_frame(name, f, 0).cpu().numpy()) < 1e-4, (f, name)


def test_noalloc_rejects_grids_beyond_its_capacity(cuda_lib):
    env = SS.elastic_cube(n=72, side_cells=4)  # 72^3 nodes > 64^3
    w = World([env], n_frames=2, dt=DT)
    rc = w.lib.dt_substep_fwd_noalloc(w.wp, 0, torch.cuda.current_stream().cuda_stream)
    assert rc == -3  # DT_ERR_CAPACITY
    torch.cuda.synchronize()
    assert np.allclose(w.particles(1)["x"].cpu().numpy(), 0.0)  # nothing ran


def test_noalloc_substep_with_a_rope(cuda_lib):
    """The rope's frames are shifted with the particle and FEM frames."""
    env = SS.rope_under_pad()
    cv = SS.control_velocity(env.sensors[0], scale=0.02, down=-0.05)
    ref = _world(env, cv)
    ref.substep(0)
    ref.substep(1)
    w = _world(env, cv)
    bare = N.DtWorld.from_buffer_copy(w.w)
    for name in SCRATCH:
        setattr(bare, name, None)
    stream = torch.cuda.current_stream().cuda_stream
    for f in (0, 1):
        rc = w.lib.dt_substep_fwd_noalloc(ctypes.byref(bare), f, stream)
        assert rc == 0, N.ERRORS.get(rc, rc)
    torch.cuda.synchronize()
    assert w.error_word() == 0
    for f in (1, 2):
        a, b = ref.rope_state(f, 0), w.rope_state(f, 0)
        assert SS.rel_err(b["pos"].cpu().numpy(), a["pos"].cpu().numpy()) < 1e-6, f
        assert SS.rel_err(b["vel"].cpu().numpy(), a["vel"].cpu().numpy()) < 1e-4, f
