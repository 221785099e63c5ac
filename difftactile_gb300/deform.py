"""Shape-target loss of an environment's object (Deform_Loss, tasks/deform_loss.py:8-146) on the
device: target density -> target distance field (dt_target_sdf), per-frame mass grid
(dt_grid_mass), density + distance-weighted mass loss (dt_deform_loss) and its particle adjoint
(dt_deform_loss_bwd).  Grids are held in the World's block layout; ``to_block`` / ``to_dense``
convert from / to dense (i, j, k) arrays."""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N


class DeformLoss:
    def __init__(self, world, e: int = 0, sdf_weight: float = 1.0, density_weight: float = 1.0):
        self.w = world
        self.e = int(e)
        row = world.env_rows[self.e]
        self.n = tuple(int(v) for v in row.n)
        nb = tuple(int(v) for v in row.nb)
        i, j, k = np.meshgrid(*[np.arange(v) for v in self.n], indexing="ij")
        idx = row.node_off + 64 * (((i >> 2) * nb[1] + (j >> 2)) * nb[2] + (k >> 2)) + 16 * (i & 3) + 4 * (j & 3) + (k & 3)
        dev = world.device
        self.idx = torch.as_tensor(idx.reshape(-1), dtype=torch.long, device=dev)
        NN = world.n_nodes
        self.m = torch.zeros(NN, device=dev)
        self.target = torch.zeros(NN, device=dev)
        self.sdf = torch.zeros(NN, device=dev)
        self.loss = torch.zeros(1, device=dev)
        self.sdf_weight, self.density_weight = float(sdf_weight), float(density_weight)
        self.target_iou = None

    # ---- layout ----
    def to_block(self, dense) -> torch.Tensor:
        out = torch.zeros(self.w.n_nodes, device=self.w.device)
        out[self.idx] = torch.as_tensor(np.asarray(dense) if not torch.is_tensor(dense) else dense,
                                        dtype=torch.float32, device=self.w.device).reshape(-1)
        return out

    def to_dense(self, block: torch.Tensor) -> torch.Tensor:
        return block[self.idx].reshape(self.n)

    # ---- Deform_Loss methods ----
    def set_weights(self, sdf: float, density: float):
        self.sdf_weight, self.density_weight = float(sdf), float(density)

    def initialize(self, target, passes: int | None = None):
        """load_target_density + update_target: target density grid [n0, n1, n2] -> distance field
        (2 max(n) propagation passes by default, as the reference's 2 n_grid)."""
        w = self.w
        self.target = self.to_block(target)
        scratch = torch.zeros((2, w.n_nodes, 4), device=w.device)
        p = 2 * max(self.n) if passes is None else int(passes)
        N.check(w.lib.dt_target_sdf(w.wp, self.e, self.target.data_ptr(), self.sdf.data_ptr(), scratch.data_ptr(), p,
                                    w.stream), "target sdf")
        self.target_iou = self.iou(self.target)

    def grid_mass(self, f: int) -> torch.Tensor:
        """compute_grid_m_kernel(f): mass grid of frame f (block layout)."""
        w = self.w
        self.m.zero_()
        N.check(w.lib.dt_grid_mass(w.wp, self.e, int(f), self.m.data_ptr(), w.stream), "grid mass")
        return self.m

    def compute_loss(self, f: int) -> torch.Tensor:
        """compute_loss_kernel(f): density + sdf loss of frame f (device scalar)."""
        w = self.w
        self.grid_mass(f)
        self.loss.zero_()
        N.check(w.lib.dt_deform_loss(w.wp, self.e, self.m.data_ptr(), self.target.data_ptr(), self.sdf.data_ptr(),
                                     self.density_weight, self.sdf_weight, self.loss.data_ptr(), w.stream), "deform loss")
        return self.loss

    def compute_loss_grad(self, f: int, loss_bar: float = 1.0):
        """compute_loss_kernel_grad(f): adds d loss / d x of frame f to the world's particle adjoint
        (buffer f & 1); compute_loss(f) must have run (its mass grid is reused)."""
        w = self.w
        N.check(w.lib.dt_deform_loss_bwd(w.wp, self.e, int(f), self.m.data_ptr(), self.target.data_ptr(),
                                         self.sdf.data_ptr(), self.density_weight, self.sdf_weight, float(loss_bar),
                                         w.stream), "deform loss bwd")

    def iou(self, m: torch.Tensor | None = None) -> float:
        """Soft IoU of a mass grid with the target (deform_loss.py:128-142)."""
        a = (self.m if m is None else m)[self.idx].double()
        b = self.target[self.idx].double()
        ma, mb = a.max(), b.max()
        inter = (a * b).sum() / ma / mb
        union = a.sum() / ma + b.sum() / mb
        return float(inter / (union - inter))
