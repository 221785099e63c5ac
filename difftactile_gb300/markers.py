"""Tactile marker readout: the marker model of a sensor and the device readout calls.

Set-up (host, once) follows init_cam_model, fem_sensor.py:130-159: the sensor's outermost layer of
nodes in its own frame is viewed by the fisheye camera (x, z, y), projected to pixels
(project_points_to_pix, fisheye_model.py:32-51), and every marker is interpolated from its k = 5
nearest projected nodes with inverse-distance weights.  The reference detects the marker pixels in
an image with OpenCV; here the marker set is given (default: a regular grid of 8 x 17 = 136 markers
over the projected surface), which is the only input that step produces.

Per frame (device) the CUDA readout (dt_markers) projects the current and virtual surface positions
and interpolates them (extract_markers, fem_sensor.py:161-187); dt_markers_bwd is its adjoint.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N

# project_3d_2d defaults (fisheye_model.py:12)
DEFAULT_CAM = {"f": 8.627e-04, "m": 173913.04, "cx": 3.320e02, "cy": 2.400e02, "plane": 2.0 * 0.01}


def project_points_to_pix(a: np.ndarray, cam=DEFAULT_CAM) -> np.ndarray:
    """Host projection used for the set-up (fisheye_model.py:32-51): [n,3] camera points -> [n,2]."""
    a = np.array(a, np.float64)
    a[:, 2] += cam["plane"]
    cos = a[:, 2] / np.linalg.norm(a, axis=1)
    theta = np.arccos(np.clip(cos, -1.0, 1.0))
    omega = np.arctan2(a[:, 1], a[:, 0]) + np.pi
    r = cam["m"] * cam["f"] * theta
    return np.stack([r * np.cos(omega) + cam["cx"], r * np.sin(omega) + cam["cy"]], 1)


def idw_weights(markers: np.ndarray, points: np.ndarray, k: int = 5):
    """k nearest points of every marker and their normalised inverse-distance weights."""
    idx = np.zeros((len(markers), k), np.int32)
    wts = np.zeros((len(markers), k), np.float64)
    for i, m in enumerate(markers):
        off = np.linalg.norm(m[None, :] - points, axis=1)
        nn = np.argpartition(off, k)[:k] if len(points) > k else np.arange(len(points))
        inv = 1.0 / np.maximum(off[nn], 1e-12)
        idx[i, : len(nn)] = nn
        wts[i, : len(nn)] = inv / inv.sum()
    return idx, wts


class MarkerModel:
    """Markers of sensor ``s`` of a World (see the module docstring)."""

    def __init__(self, world, s: int, markers_2d: np.ndarray | None = None, k: int = 5, cam=None,
                 grid=(8, 17)):
        self.w = world
        self.s = int(s)
        self.cam = dict(DEFAULT_CAM if cam is None else cam)
        sp = world.sensor_specs[s]
        layer = np.asarray(sp.layer)
        self.surf = np.where(layer == layer.max())[0].astype(np.int32)
        T = np.eye(4) if sp.trans_world is None else np.asarray(sp.trans_world, np.float64)
        Ti = np.linalg.inv(T)
        local = (Ti[:3, :3] @ np.asarray(sp.verts, np.float64)[self.surf].T).T + Ti[:3, 3]
        self.cam_points = project_points_to_pix(local[:, [0, 2, 1]], self.cam)
        if markers_2d is None:
            lo, hi = self.cam_points.min(0), self.cam_points.max(0)
            pad = 0.1 * (hi - lo)
            gx = np.linspace(lo[0] + pad[0], hi[0] - pad[0], grid[1])
            gy = np.linspace(lo[1] + pad[1], hi[1] - pad[1], grid[0])
            markers_2d = np.stack(np.meshgrid(gx, gy, indexing="xy"), -1).reshape(-1, 2)
        self.markers_2d = np.asarray(markers_2d, np.float64)
        self.k = int(k)
        idx, wts = idw_weights(self.markers_2d, self.cam_points, self.k)
        self.idx, self.wts = idx, wts
        dev = world.device
        self.M = len(self.markers_2d)
        self.d_surf = torch.as_tensor(self.surf, dtype=torch.int32, device=dev)
        self.d_idx = torch.as_tensor(idx.reshape(-1), dtype=torch.int32, device=dev)
        self.d_wts = torch.as_tensor(wts.reshape(-1), dtype=torch.float32, device=dev)
        self.inv_trans0 = torch.as_tensor(Ti[:3, :].reshape(-1), dtype=torch.float32, device=dev)
        self.fisheye = N.DtFisheye(*(float(self.cam[k_]) for k_ in ("f", "m", "cx", "cy", "plane")))

    def _inv(self, inv_trans):
        if inv_trans is None:
            return self.inv_trans0
        t = torch.as_tensor(inv_trans, dtype=torch.float32, device=self.w.device)
        return (t[:3, :] if t.dim() == 2 else t.reshape(3, 4)).contiguous().reshape(-1)

    def readout(self, f: int, inv_trans=None):
        """(predicted, virtual) marker pixels [M,2] of frame f; inv_trans: world-to-sensor 4x4 or its
        rows 0..2 (default: the rest pose)."""
        w = self.w
        pred = torch.empty((self.M, 2), dtype=torch.float32, device=w.device)
        virt = torch.empty_like(pred)
        Mi = self._inv(inv_trans)
        N.check(w.lib.dt_markers(w.wp, self.s, int(f), self.d_surf.data_ptr(), self.d_idx.data_ptr(),
                                 self.d_wts.data_ptr(), self.k, self.M, Mi.data_ptr(), self.fisheye,
                                 pred.data_ptr(), virt.data_ptr(), w.stream), "markers")
        return pred, virt

    def readout_bwd(self, f: int, pred_b=None, virt_b=None, inv_trans=None) -> torch.Tensor:
        """Adds the adjoints of frame f's surface positions (world adjoint buffer f & 1); returns
        d/d inv_trans rows 0..2 [3,4]."""
        w = self.w
        Mi = self._inv(inv_trans)
        Mb = torch.zeros(12, dtype=torch.float32, device=w.device)
        pb = None if pred_b is None else torch.as_tensor(pred_b, dtype=torch.float32, device=w.device).contiguous()
        vb = None if virt_b is None else torch.as_tensor(virt_b, dtype=torch.float32, device=w.device).contiguous()
        N.check(w.lib.dt_markers_bwd(w.wp, self.s, int(f), self.d_surf.data_ptr(), self.d_idx.data_ptr(),
                                     self.d_wts.data_ptr(), self.k, self.M, Mi.data_ptr(), self.fisheye,
                                     None if pb is None else pb.data_ptr(), None if vb is None else vb.data_ptr(),
                                     Mb.data_ptr(), w.stream), "markers bwd")
        return Mb.reshape(3, 4)
