"""Readouts on the GPU through the C ABI: summed contact force (compute_contact_force,
grasp_plastic.py:218-229) and the fisheye marker readout (extract_markers, fem_sensor.py:161-187),
forward against the oracle restatement, adjoints against float64 central finite differences.
Tolerances: forward 1e-5 (markers) / 1e-4 (force sums of atomically accumulated forces) relative;
directional derivatives 2e-3 relative."""
import numpy as np
import pytest
import torch

from difftactile_gb300.markers import MarkerModel
from difftactile_gb300.world import World
from oracle import markers as OM
from oracle import oracle as O
from tests import small_scenes as SS

pytestmark = pytest.mark.gpu
DT = 1e-4


def test_contact_force_sum_matches_oracle(cuda_lib):
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp) for sp in env.sensors]
    w = World([env], n_frames=3, dt=DT)
    w.set_control_velocity(0, cv[0])
    w.step_begin()
    for f in range(2):
        w.substep(f)
    out = torch.zeros(4, device=w.device)
    N_ = w.lib
    assert N_.dt_contact_force(w.wp, 0, 1, out.data_ptr(), w.stream) == 0
    o = O.Oracle(env, DT)
    st = o.initial_state()
    st, _ = o.substep(st, cv=cv, cv1=cv)
    _, dbg = o.substep(st, cv=cv, cv1=cv)
    ref = OM.contact_force_sum(dbg["ext"][0], env.sensors[0].tris)
    assert np.abs(ref).max() > 0
    assert SS.rel_err(out[:3].cpu().numpy(), ref) < 1e-4


def test_contact_force_adjoint_vs_finite_differences(cuda_lib):
    env = SS.pad_over_box()
    cv = [SS.control_velocity(sp).astype(np.float64) for sp in env.sensors]
    gb = np.array([0.3, -1.0, 0.7])
    w = World([env], n_frames=2, dt=DT, grad_clip=0.0)
    w.set_control_velocity(0, cv[0])
    w.step_begin()
    w.substep(0)
    w.adj_clear()
    g_t = torch.as_tensor(gb, dtype=torch.float32, device=w.device)
    assert w.lib.dt_contact_force_bwd(w.wp, 0, g_t.data_ptr(), w.stream) == 0
    w.substep_bwd(0)
    torch.cuda.synchronize()
    ga = {k: v.double().cpu().numpy() for k, v in w.particle_adjoint(0).items()}
    gpos = w.t["v_adj_pos"][0, w.vslice(0), :3].double().cpu().numpy()
    o = O.Oracle(env, DT, np.float64)
    st0 = o.initial_state()

    def L(st):
        _, dbg = o.substep(st, cv=cv, cv1=cv)
        return float(gb @ OM.contact_force_sum(dbg["ext"][0], env.sensors[0].tris))

    rng = np.random.default_rng(2)
    for trial in range(3):
        dx = 2e-4 * rng.standard_normal(st0["x"].shape)
        dp = 2e-4 * rng.standard_normal(st0["pos"][0].shape)
        pred = float((ga["x"] * dx).sum() + (gpos * dp).sum())
        eps = 1e-3

        def sh(sg):
            st = dict(st0)
            st["x"] = st0["x"] + sg * eps * dx
            st["pos"] = [st0["pos"][0] + sg * eps * dp]
            return L(st)

        fd = (sh(1) - sh(-1)) / (2 * eps)
        assert abs(pred - fd) <= 2e-3 * abs(fd) + 1e-9, (trial, pred, fd)


def test_markers_forward_and_adjoint(cuda_lib):
    env = SS.dome_over_box()
    cv = [SS.control_velocity(sp, scale=0.02, down=-0.05) for sp in env.sensors]
    w = World([env], n_frames=3, dt=DT)
    w.set_control_velocity(0, cv[0])
    w.step_begin()
    for f in range(2):
        w.substep(f)
    mm = MarkerModel(w, 0)
    sp = env.sensors[0]
    Ti = np.linalg.inv(sp.trans_world)
    pred, virt = mm.readout(2)
    pos = w.sensor_frame("v_pos", 2, 0).double().cpu().numpy()
    vpos = w.sensor_frame("v_vpos", 2, 0).double().cpu().numpy()
    rp, rv = OM.extract_markers(pos, vpos, mm.surf, mm.idx, mm.wts, Ti, mm.cam)
    assert SS.rel_err(pred.cpu().numpy(), rp) < 1e-5
    assert SS.rel_err(virt.cpu().numpy(), rv) < 1e-5
    # adjoint
    rng = np.random.default_rng(5)
    pb, vb = rng.standard_normal(rp.shape), rng.standard_normal(rv.shape)
    w.adj_clear()
    Mb = mm.readout_bwd(2, pb, vb).double().cpu().numpy()
    torch.cuda.synchronize()
    gpos = w.t["v_adj_pos"][0, w.vslice(0), :3].double().cpu().numpy()
    gvp = w.t["v_adj_vpos"][0, w.vslice(0), :3].double().cpu().numpy()

    def L(p, vp, M):
        a, b = OM.extract_markers(p, vp, mm.surf, mm.idx, mm.wts, M, mm.cam)
        return float((pb * a).sum() + (vb * b).sum())

    for trial in range(3):
        d1, d2 = 1e-3 * rng.standard_normal(pos.shape), 1e-3 * rng.standard_normal(vpos.shape)
        dM = np.zeros((4, 4))
        dM[:3] = 1e-3 * rng.standard_normal((3, 4))
        pred_d = float((gpos * d1).sum() + (gvp * d2).sum() + (Mb * dM[:3]).sum())
        eps = 1e-3
        fd = (L(pos + eps * d1, vpos + eps * d2, Ti + eps * dM) - L(pos - eps * d1, vpos - eps * d2, Ti - eps * dM)) / (
            2 * eps)
        assert abs(pred_d - fd) <= 2e-3 * abs(fd), (trial, pred_d, fd)
