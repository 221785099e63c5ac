"""Rigid shape matching of an object's rigid part (MPMObj compute_COM / compute_H / compute_H_svd /
compute_R, multi_obj.py:309-340) and the rotation-angle readout of the box-opening task
(compute_angle, box_open.py:401-406).  H comes from the device (dt_rigid_match); its 3x3 SVD,
R = V U^T and the angle run in float64 torch with autograd, and d loss / d H goes back to the
particles through dt_rigid_match_bwd.

torch.linalg.svd returns non-negative singular values, the reference's ti.svd det U = det V = +1; the
two give the same R = V U^T whenever det H > 0, which holds for the small rotations between two
substeps."""
from __future__ import annotations

import torch

from . import _native as N


class RigidMatch:
    def __init__(self, world, e: int = 0, mat: int = 0):
        self.w, self.e, self.mat = world, int(e), int(mat)
        self.out = torch.zeros(20, device=world.device)
        self.scratch = torch.zeros(8, device=world.device)

    def H(self, f: int):
        """(c0, c1, H) between frames f and f+1 (device tensors)."""
        w = self.w
        N.check(w.lib.dt_rigid_match(w.wp, self.e, self.mat, int(f), self.out.data_ptr(), w.stream), "rigid match")
        return self.out[0:3], self.out[4:7], self.out[8:17].reshape(3, 3)

    @staticmethod
    def rotation(H: torch.Tensor) -> torch.Tensor:
        """R = V U^T from H = U S V^T (compute_H_svd + compute_R)."""
        U, S, Vh = torch.linalg.svd(H)
        return Vh.transpose(-1, -2) @ U.transpose(-1, -2)

    @staticmethod
    def angle(R: torch.Tensor) -> torch.Tensor:
        """Rotation about z of one substep (compute_angle's atan2(R[1,0], R[1,1]))."""
        return torch.atan2(R[..., 1, 0], R[..., 1, 1])

    def backward(self, f: int, H_bar: torch.Tensor, part: int):
        """Add the particle adjoint of H_bar: part 0 to frame f, part 1 to frame f + 1 (each while
        that frame's adjoint buffer is current in the backward sweep).  H(f) must have run."""
        w = self.w
        hb = torch.as_tensor(H_bar, dtype=torch.float32, device=w.device).reshape(9).contiguous()
        N.check(w.lib.dt_rigid_match_bwd(w.wp, self.e, self.mat, int(f), int(part), self.out.data_ptr(),
                                         hb.data_ptr(), self.scratch.data_ptr(), w.stream), "rigid match bwd")
