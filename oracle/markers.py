"""ORACLE (test infrastructure only): float64 numpy restatement of the marker readout
(extract_markers, difftactile/sensor_model/fem_sensor.py:161-187) with the fisheye projection
project_3d_2d (difftactile/sensor_model/fisheye_model.py:12-30), and the summed contact force
(compute_contact_force, difftactile/tasks/grasp_plastic.py:218-229).  Pinned against the
reference's own code: the numpy projection (tests/golden/fisheye_ref.npz, tests/golden/
make_fisheye.py), the marker set-up and readout (tests/golden/markers_ref.npz: init_cam_model and
extract_markers run on a numpy stand-in for Taichi by tests/golden/make_markers.py) and the force
sum (tests/golden/substep_ref.npz, compute_contact_force); also by analytic known answers in
tests/test_oracle_readout.py."""
from __future__ import annotations

import numpy as np


def project_3d_2d(a, cam):
    """[n,3] camera points -> [n,2] pixels, project_3d_2d with its clamp and 1e-8 / 1e-10 guards."""
    a = np.array(a, np.float64).reshape(-1, 3)
    a[:, 2] += cam["plane"]
    an = np.sqrt((a * a).sum(1) + 1e-10)
    cos = np.clip(a[:, 2] / an, -1.0, 1.0)
    theta = np.arccos(cos)
    omega = np.arctan2(a[:, 1], a[:, 0] + 1e-8) + np.pi
    r = cam["m"] * cam["f"] * theta
    return np.stack([r * np.cos(omega) + cam["cx"], r * np.sin(omega) + cam["cy"]], 1)


def extract_markers(pos, vpos, surf, idx, wts, inv_trans, cam):
    """pos, vpos [V,3] (sensor-local vertex order), surf [S], idx/wts [M,K], inv_trans [3,4] or
    [4,4] -> (pred [M,2], virt [M,2])."""
    Mi = np.asarray(inv_trans, np.float64)[:3, :]

    def proj(x):
        h = np.concatenate([np.asarray(x, np.float64), np.ones((len(x), 1))], 1)
        ip = h @ Mi.T
        return project_3d_2d(ip[:, [0, 2, 1]], cam)

    lp = proj(np.asarray(pos)[surf])
    lv = proj(np.asarray(vpos)[surf])
    w = np.asarray(wts, np.float64)
    pred = (w[:, :, None] * lp[idx]).sum(1)
    virt = (w[:, :, None] * lv[idx]).sum(1)
    return pred, virt


def contact_force_sum(ext, tris):
    """Sum over triangles of 1/6 of the force on each vertex: ext [V,3], tris [T,3] -> [3]."""
    ext = np.asarray(ext, np.float64)
    t = np.asarray(tris)
    return (ext[t[:, 0]] / 6 + ext[t[:, 1]] / 6 + ext[t[:, 2]] / 6).sum(0)
