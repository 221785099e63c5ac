"""Device-resident world: flat, offset-indexed layout of many environments + the C-ABI calls.

All buffers are torch tensors on one CUDA device (torch is used for allocation and streams only);
every compute step is a call into libdifftactile_gb300.so through ctypes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from .scene import EnvSpec, SensorSpec

F32 = torch.float32
I32 = torch.int32


def _morton_key(cell: np.ndarray) -> np.ndarray:
    """Block-major key of a cell: 4x4x4 block id (Morton-interleaved) then the cell in the block."""
    c = cell.astype(np.int64)
    b = c >> 2
    key = np.zeros(len(c), np.int64)
    for bit in range(10):
        for d in range(3):
            key |= ((b[:, d] >> bit) & 1) << (3 * bit + (2 - d) + 6)
    key |= ((c[:, 0] & 3) << 4) | ((c[:, 1] & 3) << 2) | (c[:, 2] & 3)
    return key


def _kd_groups(pts: np.ndarray, group: int = 32) -> np.ndarray:
    """Order of ``pts`` in which consecutive runs of ``group`` points are spatially compact:
    recursive median splits along the widest axis, the left part a multiple of ``group``."""
    out: list[np.ndarray] = []

    def split(idx):
        n = len(idx)
        if n <= group:
            out.append(idx)
            return
        p = pts[idx]
        ax = int(np.argmax(p.max(0) - p.min(0)))
        left = group * ((n + 2 * group - 1) // (2 * group))
        o = np.argsort(p[:, ax], kind="stable")
        split(idx[o[:left]])
        split(idx[o[left:]])

    if len(pts):
        split(np.arange(len(pts)))
    return np.concatenate(out) if out else np.zeros(0, np.int64)


class World:
    """Flat device layout of ``envs`` (list of EnvSpec) with ``n_frames`` frames per step."""

    def __init__(self, envs: list[EnvSpec], n_frames: int, dt: float, device="cuda", tape_blocks: int | None = None,
                 grad_clip: float = 1000.0, svd_sweeps: int = 4, sort_particles: bool = True,
                 svd_grad_mode: int = 0, scatter_mode: int = 2, svd_tape: bool = True, p_block: int = 128,
                 scatter_depth: int = 0, contact_lanes: int = 8, p_per_thread: int = 1, overlap_ropes: bool = True,
                 scatter_depth_adj: int = 0):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError(f"World buffers must live on a CUDA device (the kernels take device pointers), "
                             f"got {self.device}")
        self.lib = N.load()
        self.specs = envs
        self.n_frames = int(n_frames)
        self.dt = float(dt)
        dev = self.device

        # ---------------- particles ----------------
        perm, p_env, p_mat, env_rows, mats, mat_off = [], [], [], [], [], 0
        node_off = blk_off = p_off = 0
        sensors: list[tuple[int, SensorSpec]] = []
        blk_env = []
        for e, s in enumerate(envs):
            n = s.n_particles
            nb = [(g + 3) // 4 for g in s.n_grid]
            if sort_particles and n:
                cell = np.floor(s.x.astype(np.float64) / s.dx - 0.5).clip(0, max(s.n_grid) - 1).astype(np.int64)
                order = np.argsort(_morton_key(cell), kind="stable")
            else:
                order = np.arange(n)
            perm.append(order + p_off)
            p_env.append(np.full(n, e, np.int32))
            mid = np.zeros(n, np.int32) if s.mat is None else np.asarray(s.mat, np.int32)
            p_mat.append(mid[order] + mat_off)
            mats.extend(s.materials)
            row = N.DtEnv()
            row.p_begin, row.p_end = p_off, p_off + n
            row.node_off, row.blk_off = node_off, blk_off
            row.nb[:] = nb
            row.n[:] = list(s.n_grid)
            row.bound, row.bc = s.bound, s.bc
            row.s_begin = len(sensors)
            for sp in s.sensors:
                sensors.append((e, sp))
            row.s_end = len(sensors)
            if row.s_end - row.s_begin > 4:
                raise ValueError("at most 4 sensors per environment")
            dx = float(s.dx)
            inv_dx = 1.0 / dx
            row.dx, row.inv_dx = dx, inv_dx
            row.p_mass = s.p_mass
            row.stress_k = -self.dt * s.volume * 4 * inv_dx * inv_dx
            row.eps = s.eps
            row.g2p_k = 4 * inv_dx
            row.dt_g[:] = [self.dt * g for g in s.gravity]
            row.kn, row.kd, row.kt, row.mu_t = s.kn, s.kd, s.kt, s.mu_t
            env_rows.append(row)
            nblk = nb[0] * nb[1] * nb[2]
            blk_env.append(np.full(nblk, e, np.int32))
            node_off += 64 * nblk
            blk_off += nblk
            p_off += n
            mat_off += len(s.materials)
        self.n_envs = len(envs)
        self.n_particles = p_off
        self.n_nodes, self.n_blocks = node_off, blk_off
        # construction order: sorted slot -> user index (the device copies below follow later re-binning)
        self.perm = np.concatenate(perm) if perm else np.zeros(0, np.int64)
        self.inv_perm = np.empty_like(self.perm)
        self.inv_perm[self.perm] = np.arange(len(self.perm))
        self._perm_t = torch.as_tensor(self.perm, device=dev)  # current slot -> user index (follows rebin)
        self._inv_perm_t = torch.as_tensor(self.inv_perm, device=dev)
        self._slot_t = torch.arange(len(self.perm), device=dev)
        self._rb_scratch = None
        self.env_rows = env_rows

        # ---------------- sensors ----------------
        v_off = t_off = f_off = 0
        verts, tets, tris, layer, v_sensor, t_sensor, Bs, srows = [], [], [], [], [], [], [], []
        tri_perm = []
        for si, (e, sp) in enumerate(sensors):
            nv, nt, nf = len(sp.verts), len(sp.tets), len(sp.tris)
            verts.append(sp.verts.astype(np.float32))
            tets.append(sp.tets.astype(np.int32) + v_off)
            tris.append(np.concatenate([sp.tris.astype(np.int32) + v_off, np.full((nf, 1), si, np.int32)], 1))
            # contact-search order: groups of 32 consecutive positions are compact patches of the
            # rest surface (ties in the search still resolve on the original index)
            cen = sp.verts[sp.tris].mean(1).astype(np.float64) if nf else np.zeros((0, 3))
            tri_perm.append(_kd_groups(cen).astype(np.int32) + f_off)
            layer.append(sp.layer.astype(np.int32))
            v_sensor.append(np.full(nv, si, np.int32))
            t_sensor.append(np.full(nt, si, np.int32))
            B = sp.rest_inverse()
            Bp = np.zeros((nt, 3, 4), np.float32)
            Bp[:, :, :3] = B
            Bs.append(Bp.reshape(nt, 12))
            r = N.DtSensor()
            r.v_off, r.nv, r.t_off, r.nt, r.f_off, r.nf = v_off, nv, t_off, nt, f_off, nf
            r.env, r.carry = e, sp.carry
            mu, lam = sp.lame()
            r.dt_over_m = self.dt / sp.mass
            r.mu, r.lam = mu, lam
            r.alpha = float(np.float32(1) + np.float32(0.75) * np.float32(mu) / np.float32(lam))
            r.out_dir[:] = [float(c) for c in sp.out_dir]
            r.model = int(getattr(sp, "model", 0))
            srows.append(r)
            v_off, t_off, f_off = v_off + nv, t_off + nt, f_off + nf
        self.sensor_specs = [sp for _, sp in sensors]
        self.sensor_env = [e for e, _ in sensors]
        self.sensor_rows = srows
        self.n_sensors = len(sensors)
        self.n_verts, self.n_tets, self.n_tris = v_off, t_off, f_off

        cat = lambda xs, shape, dt_: (np.concatenate(xs, 0) if xs else np.zeros(shape, dt_))  # noqa: E731
        self.rest_verts = cat(verts, (0, 3), np.float32)

        # ---------------- PBD ropes (flat over all envs, 64 particles per contact CTA) ----------------
        rope_rows, r_x, r_v, self.rope_specs = [], [], [], []
        r_off = r_blk = 0
        for e, s in enumerate(envs):
            for rp in getattr(s, "ropes", []):
                row = N.DtRope()
                row.p_off, row.n, row.env, row.blk_off = r_off, rp.n, e, r_blk
                row.mass, row.inv_m, row.rad = rp.mass, 1.0 / rp.mass, rp.rad
                row.rest, row.bend = rp.rest, rp.bend
                cs, cb = rp.compliance
                row.alpha_s, row.alpha_b = cs / self.dt ** 2, cb / self.dt ** 2
                row.relax_s, row.relax_b = rp.stretch_relax, rp.bend_relax
                row.table_h, row.friction = rp.table_h, rp.friction
                row.dt_g[:] = [self.dt * g for g in rp.gravity]
                x0 = rp.init_positions()
                row.pin[:] = [float(c) for c in x0[0]]
                row.kn, row.kd, row.kt, row.mu_t = rp.kn, rp.kd, rp.kt, rp.mu_t
                row.iters = max(int(getattr(rp, "iters", 1)), 1)
                rope_rows.append(row)
                r_x.append(x0)
                r_v.append(np.zeros((rp.n, 3), np.float32) if rp.v is None else np.asarray(rp.v, np.float32))
                self.rope_specs.append(rp)
                r_off += rp.n
                r_blk += (rp.n + 63) // 64
        self.rope_rows = rope_rows
        self.n_ropes, self.n_rope_particles = len(rope_rows), r_off
        self.t = {}
        t = self.t

        def dtensor(a, dtype):
            return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

        def zeros(shape, dtype=F32):
            return torch.zeros(shape, dtype=dtype, device=dev)

        def struct_tensor(rows, cls):
            buf = bytearray(C.sizeof(cls) * max(len(rows), 1))
            for i, r_ in enumerate(rows):
                C.memmove(C.addressof(C.c_char.from_buffer(buf, i * C.sizeof(cls))), C.addressof(r_), C.sizeof(cls))
            return torch.frombuffer(buf, dtype=torch.uint8).to(dev)

        mat_rows = []
        for m in mats:
            r = N.DtMaterial()
            mu, lam = m.mu_lam
            r.mu, r.lam, r.yield_stress, r.model = mu, lam, m.yield_stress, m.model
            mat_rows.append(r)
        self.materials = list(mats)
        self._mat_rows = mat_rows
        self.n_materials = len(mats)
        t["envs"] = struct_tensor(env_rows, N.DtEnv)
        t["sensors"] = struct_tensor(srows, N.DtSensor)
        t["materials"] = struct_tensor(mat_rows, N.DtMaterial)
        t["p_env"] = dtensor(cat(p_env, (0,), np.int32), I32)
        t["p_mat"] = dtensor(cat(p_mat, (0,), np.int32), I32)
        t["blk_env"] = dtensor(cat(blk_env, (0,), np.int32), I32)
        t["tets"] = dtensor(cat(tets, (0, 4), np.int32), I32)
        t["tet_B"] = dtensor(cat(Bs, (0, 12), np.float32), F32)
        t["tet_sensor"] = dtensor(cat(t_sensor, (0,), np.int32), I32)
        t["tris"] = dtensor(cat(tris, (0, 4), np.int32), I32)
        t["tri_perm"] = dtensor(cat(tri_perm, (0,), np.int32), I32)
        t["v_layer"] = dtensor(cat(layer, (0,), np.int32), I32)
        t["v_sensor"] = dtensor(cat(v_sensor, (0,), np.int32), I32)

        Fn, Np, V, NN, NB = self.n_frames, self.n_particles, self.n_verts, self.n_nodes, self.n_blocks
        self.tape_blocks = int(tape_blocks if tape_blocks is not None else NB)
        TB = self.tape_blocks
        t["p_state"] = zeros((Fn, 6, Np, 4))
        t["p_adj"] = zeros((2, 6, Np, 4))
        t["g_acc"] = zeros((NN, 4))
        t["g_vout"] = zeros((NN, 4))
        t["g_adj_vout"] = zeros((NN, 4))
        t["g_adj_acc"] = zeros((NN, 4))
        t["blk_flag"] = zeros((NB,), I32)
        t["tape_blist"] = zeros((Fn, NB), I32)
        t["tape_bcount"] = zeros((Fn,), I32)
        t["tape_acc"] = zeros((Fn, TB * 64, 4))
        t["tape_vout"] = zeros((Fn, TB * 64, 4))
        t["tape_cidx"] = zeros((Fn, TB * 64, 4), I32)
        for k in ("v_pos", "v_vel", "v_velmid", "v_ext", "v_vpos", "v_cv"):
            t[k] = zeros((Fn, V, 4))
        t["tri_cent"] = zeros((self.n_tris, 4))
        for k in ("v_adj_pos", "v_adj_vel", "v_adj_vpos"):
            t[k] = zeros((2, V, 4))
        t["v_adj_velmid"] = zeros((V, 4))
        t["v_adj_ext"] = zeros((V, 4))
        t["v_adj_cv"] = zeros((Fn, V, 4))
        t["mat_adj"] = zeros((max(self.n_materials, 1), 4))
        t["err"] = zeros((4,), I32)
        NR = self.n_rope_particles
        t["ropes"] = struct_tensor(rope_rows, N.DtRope)
        t["r_state"] = zeros((Fn, 2, NR, 4))
        t["r_ext"] = zeros((Fn, NR, 4))
        t["r_cidx"] = zeros((Fn, NR, 4), I32)
        t["r_adj"] = zeros((2, 2, NR, 4))
        t["r_extb"] = zeros((NR, 4))
        max_iters = max([r.iters for r in rope_rows], default=1)
        # the adjoint of more than one pass pair recomputes every pass's input positions into here
        t["r_work"] = zeros((2 * max_iters, NR, 4)) if (max_iters > 1 and NR) else None
        # the forward's SVD per frame, so that the adjoint need not recompute it (96 B per particle-frame)
        t["p_svd"] = zeros((Fn, 6, Np, 4)) if (svd_tape and Np) else None
        # the linear corotated tets' SVD, likewise (read by the tet adjoint)
        lin = any(int(getattr(sp, "model", 0)) == 1 for sp in self.sensor_specs)
        t["t_svd"] = zeros((Fn, 6, self.n_tets, 4)) if (svd_tape and lin and self.n_tets) else None

        w = N.DtWorld()
        for name in N.WORLD_PTR_FIELDS:
            setattr(w, name, t[name].data_ptr() if t[name].numel() else None)
        w.n_envs, w.n_particles, w.n_sensors, w.n_materials = self.n_envs, Np, self.n_sensors, self.n_materials
        w.n_verts, w.n_tets, w.n_tris = V, self.n_tets, self.n_tris
        w.n_nodes, w.n_blocks, w.n_frames, w.tape_blocks = NN, NB, Fn, TB
        w.dt, w.grad_clip, w.svd_sweeps = self.dt, float(grad_clip), int(svd_sweeps)
        w.svd_grad_mode = int(svd_grad_mode)
        w.max_sensor_tris = max([r.nf for r in srows], default=0)
        w.scatter_mode = int(scatter_mode)
        w.p_block = int(p_block)
        w.scatter_depth = int(scatter_depth)
        w.contact_lanes = int(contact_lanes)
        w.p_per_thread = int(p_per_thread)
        w.scatter_depth_adj = int(scatter_depth_adj)
        for name in N.ROPE_PTR_FIELDS:
            setattr(w, name, t[name].data_ptr() if (self.n_ropes and t[name].numel()) else None)
        w.n_ropes, w.n_rope_particles = self.n_ropes, NR
        w.rope_blocks = r_blk
        w.max_rope_n = max([r.n for r in rope_rows], default=0)
        w.r_work = t["r_work"].data_ptr() if t["r_work"] is not None else None
        w.max_rope_iters = max_iters if t["r_work"] is not None else 1
        w.p_svd = t["p_svd"].data_ptr() if t["p_svd"] is not None else None
        w.t_svd = t["t_svd"].data_ptr() if t["t_svd"] is not None else None
        # ropes: the solver (one CTA per rope) and its adjoint run on a second stream beside the MPM
        # stages (dt_world.aux_stream); the events are created by recording them once
        self._aux = None
        if self.n_ropes and overlap_ropes:
            self._aux = torch.cuda.Stream(device=dev)
            self._aux_ev = [torch.cuda.Event(), torch.cuda.Event()]
            for ev in self._aux_ev:
                ev.record(torch.cuda.current_stream(dev))
            w.aux_stream = self._aux.cuda_stream
            w.aux_events[0], w.aux_events[1] = self._aux_ev[0].cuda_event, self._aux_ev[1].cuda_event
        self.w = w
        self.wp = C.pointer(w)

        # write generations: every call that rewrites a frame's state or tape (or the material table)
        # bumps its counter, so that a differentiable segment can check in its backward that the frames
        # its forward left are still the ones it computed (writes through the tensors in ``t`` are not
        # tracked)
        self.frame_gen = np.zeros(self.n_frames, np.int64)
        self.material_gen = 0

        # FEM rest state in frame 0
        if V:
            vp = torch.zeros((V, 4), dtype=F32, device=dev)
            vp[:, :3] = torch.as_tensor(self.rest_verts, device=dev)
            t["v_pos"][0] = vp
            t["v_vpos"][0] = vp
        # initial particle state (user order), F = I
        xs = np.concatenate([s.x for s in envs], 0) if envs else np.zeros((0, 3), np.float32)
        vs = np.concatenate([(np.zeros_like(s.x) if s.v is None else np.broadcast_to(s.v, s.x.shape)) for s in envs], 0) \
            if envs else np.zeros((0, 3), np.float32)
        self.set_particles(0, x=xs, v=vs, C=np.zeros((Np, 3, 3), np.float32),
                           F=np.broadcast_to(np.eye(3, dtype=np.float32), (Np, 3, 3)))
        for r in range(self.n_ropes):
            self.set_rope_state(0, r, pos=r_x[r], vel=r_v[r], trav=np.zeros(self.rope_rows[r].n, np.float32))

    # ------------------------------------------------------------------------------------------
    # launches go to ``stream_override`` when set (e.g. a capture stream), else torch's current stream
    stream_override = None

    @property
    def stream(self):
        if self.stream_override is not None:
            return self.stream_override
        return torch.cuda.current_stream(self.device).cuda_stream

    def pin_stream(self, handle=None):
        """Fix the stream handle used by every launch (None: follow torch's current stream)."""
        self.stream_override = handle

    def call(self, name, *args):
        N.check(getattr(self.lib, name)(self.wp, *args, self.stream), name)

    # ---- rope state: pos [n,3], vel [n,3], travel_info [n] of rope r at frame f ----
    def rslice(self, r):
        row = self.rope_rows[r]
        return slice(row.p_off, row.p_off + row.n)

    def rope_state(self, f, r):
        sl = self.rslice(r)
        st = self.t["r_state"][f]
        return {"pos": st[0, sl, :3], "vel": st[1, sl, :3], "trav": st[0, sl, 3]}

    def touch(self, frames=None):
        """Mark frames (default: all) as rewritten (see frame_gen)."""
        if frames is None:
            self.frame_gen += 1
        else:
            self.frame_gen[frames] += 1

    def set_material(self, m, mu=None, lam=None, yield_stress=None, E=None, nu=None):
        """Change material m's parameters in the device table (in place: recorded graphs see it).  Lame
        parameters directly (``mu``, ``lam``) or from ``E``, ``nu`` (mpm_elastic.py:70-71)."""
        from .scene import Material, lame
        old = self.materials[m]
        if E is not None or nu is not None:
            E_ = old.E if E is None else float(E)
            nu_ = old.nu if nu is None else float(nu)
            new = Material(E_, nu_, old.yield_stress, old.model)
            mu, lam = lame(E_, nu_)
        else:
            mu = old.mu_lam[0] if mu is None else float(mu)
            lam = old.mu_lam[1] if lam is None else float(lam)
            new = Material(old.E, old.nu, old.yield_stress, old.model, mu=mu, lam=lam)
        if yield_stress is not None:
            new.yield_stress = float(yield_stress)
        row = self._mat_rows[m]
        row.mu, row.lam, row.yield_stress = mu, lam, new.yield_stress
        self.materials[m] = new
        buf = bytearray(C.sizeof(N.DtMaterial) * len(self._mat_rows))
        for i, r_ in enumerate(self._mat_rows):
            C.memmove(C.addressof(C.c_char.from_buffer(buf, i * C.sizeof(N.DtMaterial))), C.addressof(r_),
                      C.sizeof(N.DtMaterial))
        self.t["materials"].copy_(torch.frombuffer(buf, dtype=torch.uint8))
        self.material_gen += 1

    def lame_table(self) -> torch.Tensor:
        """[n_materials, 2] (mu, lambda) of the device table, float64 on the world's device."""
        return torch.tensor([m.mu_lam for m in self.materials], dtype=torch.float64, device=self.device)

    def material_adjoint(self) -> torch.Tensor:
        """[n_materials, 2] (d/dmu, d/dlambda) accumulated by the backward substeps since the last
        adj_clear, float64."""
        return self.t["mat_adj"][: self.n_materials, :2].double().clone()

    def set_rope_state(self, f, r, pos=None, vel=None, trav=None):
        st = self.rope_state(f, r)
        for k, a in (("pos", pos), ("vel", vel), ("trav", trav)):
            if a is not None:
                st[k].copy_(torch.as_tensor(np.asarray(a, np.float32) if not torch.is_tensor(a) else a,
                                            dtype=F32, device=self.device).reshape(st[k].shape))
        self.touch(f)

    def rope_adjoint(self, f, r):
        """Adjoint of rope r's frame f, held in buffer f & 1 during a backward sweep."""
        sl = self.rslice(r)
        a = self.t["r_adj"][f & 1]
        return {"pos": a[0, sl, :3], "vel": a[1, sl, :3], "trav": a[0, sl, 3]}

    def set_rope_adjoint(self, f, r, pos=None, vel=None, trav=None):
        a = self.rope_adjoint(f, r)
        for k, v in (("pos", pos), ("vel", vel), ("trav", trav)):
            if v is not None:
                a[k].copy_(torch.as_tensor(np.asarray(v, np.float32) if not torch.is_tensor(v) else v,
                                           dtype=F32, device=self.device).reshape(a[k].shape))

    # ---- particle state in user order ----
    def set_particles(self, frame, x=None, v=None, C=None, F=None):
        rec = self.t["p_state"][frame].permute(1, 0, 2).reshape(self.n_particles, 24)  # view? no: permute copy
        rec = rec.clone()
        put = lambda a: torch.as_tensor(np.array(a, np.float32) if not torch.is_tensor(a) else a,  # noqa: E731
                                        dtype=F32, device=self.device)
        if x is not None:
            rec[:, 0:3] = put(x).reshape(-1, 3)[self._perm_t]
        if v is not None:
            rec[:, 3:6] = put(v).reshape(-1, 3)[self._perm_t]
        if C is not None:
            rec[:, 6:15] = put(C).reshape(-1, 9)[self._perm_t]
        if F is not None:
            rec[:, 15:24] = put(F).reshape(-1, 9)[self._perm_t]
        self.t["p_state"][frame].copy_(rec.reshape(self.n_particles, 6, 4).permute(1, 0, 2))
        self.touch(frame)

    def particles(self, frame):
        """dict of torch tensors x [N,3], v [N,3], C [N,3,3], F [N,3,3] of ``frame`` in user order."""
        rec = self.t["p_state"][frame].permute(1, 0, 2).reshape(self.n_particles, 24)[self._inv_perm_t]
        return {"x": rec[:, 0:3], "v": rec[:, 3:6], "C": rec[:, 6:15].reshape(-1, 3, 3),
                "F": rec[:, 15:24].reshape(-1, 3, 3)}

    def yield_flags(self, frame):
        """Per particle (user order) whether the von Mises return map yielded in the forward substep
        ``frame`` -> ``frame`` + 1, as recorded on the SVD tape (the branch the adjoint differentiates);
        needs the SVD tape."""
        if self.t["p_svd"] is None:
            raise RuntimeError("the yield flags are recorded on the SVD tape (World(svd_tape=True))")
        return self.t["p_svd"][frame, 5, :, 1][self._inv_perm_t] > 0.5

    def particle_adjoint(self, frame):
        rec = self.t["p_adj"][frame & 1].permute(1, 0, 2).reshape(self.n_particles, 24)[self._inv_perm_t]
        return {"x": rec[:, 0:3], "v": rec[:, 3:6], "C": rec[:, 6:15].reshape(-1, 3, 3),
                "F": rec[:, 15:24].reshape(-1, 3, 3)}

    def set_particle_adjoint(self, frame, x=None, v=None, C=None, F=None):
        rec = torch.zeros((self.n_particles, 24), dtype=F32, device=self.device)
        for a, sl in ((x, slice(0, 3)), (v, slice(3, 6)), (C, slice(6, 15)), (F, slice(15, 24))):
            if a is not None:
                rec[:, sl] = torch.as_tensor(a, dtype=F32, device=self.device).reshape(self.n_particles, -1)[self._perm_t]
        self.t["p_adj"][frame & 1].copy_(rec.reshape(self.n_particles, 6, 4).permute(1, 0, 2))

    # ---- sensor state ----
    def vslice(self, s):
        r = self.sensor_rows[s]
        return slice(r.v_off, r.v_off + r.nv)

    def sensor_frame(self, name, frame, s):
        return self.t[name][frame, self.vslice(s), :3]

    def set_control_velocity(self, s, cv, frames=None):
        """cv: [V,3] (all frames) or [n_frames, V, 3]."""
        cv = torch.as_tensor(cv, dtype=F32, device=self.device)
        sl = self.vslice(s)
        if cv.dim() == 2:
            self.t["v_cv"][:, sl, :3] = cv
        else:
            self.t["v_cv"][:, sl, :3] = cv

    # ---- grid tape readback (tests, debugging): dense (i,j,k) arrays of frame f for env e ----
    def dense_grid(self, f, e=0):
        row = self.env_rows[e]
        n0, n1, n2 = row.n
        nb = list(row.nb)
        cnt = int(self.t["tape_bcount"][f].item())
        cnt = min(cnt, self.tape_blocks)
        bl = self.t["tape_blist"][f, :cnt].long()
        acc = self.t["tape_acc"][f].view(-1, 64, 4)[:cnt]
        vo = self.t["tape_vout"][f].view(-1, 64, 4)[:cnt]
        ci = self.t["tape_cidx"][f].view(-1, 64, 4)[:cnt]
        sel = (bl >= row.blk_off) & (bl < row.blk_off + nb[0] * nb[1] * nb[2])
        bl, acc, vo, ci = bl[sel] - row.blk_off, acc[sel], vo[sel], ci[sel]
        bk = bl % nb[2]
        bj = (bl // nb[2]) % nb[1]
        bi = bl // (nb[1] * nb[2])
        l = torch.arange(64, device=self.device)
        I = (4 * bi[:, None] + (l >> 4)[None]).reshape(-1)
        J = (4 * bj[:, None] + ((l >> 2) & 3)[None]).reshape(-1)
        K = (4 * bk[:, None] + (l & 3)[None]).reshape(-1)
        shape = (4 * nb[0], 4 * nb[1], 4 * nb[2])
        m = torch.zeros(shape, device=self.device)
        mv = torch.zeros(shape + (3,), device=self.device)
        v = torch.zeros(shape + (3,), device=self.device)
        cidx = torch.full(shape + (4,), -1, dtype=I32, device=self.device)
        m[I, J, K] = acc[..., 3].reshape(-1)
        mv[I, J, K] = acc[..., :3].reshape(-1, 3)
        v[I, J, K] = vo[..., :3].reshape(-1, 3)
        cidx[I, J, K] = ci.reshape(-1, 4)
        return {"m": m[:n0, :n1, :n2], "mv": mv[:n0, :n1, :n2], "v_out": v[:n0, :n1, :n2],
                "cidx": cidx[:n0, :n1, :n2]}

    def error_word(self) -> int:
        return int(self.t["err"][0].item())

    def clear_error(self):
        self.t["err"].zero_()

    # ---- C-ABI wrappers ----
    def step_begin(self):
        self.touch()  # clears every frame's tape counters
        self.call("dt_step_begin")

    # ``probe = ("fwd" | "bwd", stage)`` times that launch of every ``probe_every``-th substep with
    # CUDA events on the launching stream (the sampled substeps run as separate stage launches).
    # Pairs recorded from the host accumulate in ``probe_events``; pairs recorded during CUDA-graph
    # capture are graph nodes (external events) in ``probe_graph_events``, re-recorded by every replay.
    probe = None
    probe_every = 1
    probe_events = ()
    probe_graph_events = ()

    def _probed(self, kind, f):
        return self.probe is not None and self.probe[0] == kind and f % self.probe_every == 0

    def _staged(self, name, f, n_stages, kind):
        for s in range(n_stages):
            timed = self.probe[0] == kind and self.probe[1] == s
            if timed:
                graph = torch.cuda.is_current_stream_capturing()
                e0 = torch.cuda.Event(enable_timing=True, external=graph)
                e1 = torch.cuda.Event(enable_timing=True, external=graph)
                e0.record()
            self.call(name, int(f), s)
            if timed:
                e1.record()
                (self.probe_graph_events if graph else self.probe_events).append((e0, e1))

    def set_tape(self, on: bool):
        """Whether the forward substeps write the grid and SVD tapes that a backward substep of the same
        frame reads (dt_world.skip_tape); off for a forward pass whose frames are recomputed before any
        backward reads them."""
        self.w.skip_tape = 0 if on else 1

    def substep(self, f):
        if self._probed("fwd", f):
            self._staged("dt_substep_fwd_stage", f, 3, "fwd")
        else:
            self.call("dt_substep_fwd", int(f))
        self.touch([f, f + 1])  # frame f's grid tape, frame f + 1's state

    def substep_bwd(self, f):
        if self._probed("bwd", f):
            self._staged("dt_substep_bwd_stage", f, 4, "bwd")
        else:
            self.call("dt_substep_bwd", int(f))

    def _substeps_bwd(self, f_hi, f_lo):
        N.check(self.lib.dt_substeps_bwd(self.wp, int(f_hi), int(f_lo), self.stream), "dt_substeps_bwd")

    def substeps_bwd(self, f_hi, f_lo):
        """Adjoint substeps f_hi - 1 down to f_lo (dt_substeps_bwd: restores fused into stage 3)."""
        if self.probe is None or self.probe[0] != "bwd":
            self._substeps_bwd(f_hi, f_lo)
            return
        hi = f_hi  # fused runs between the probed frames, which run as their four stage launches
        for f in reversed(range(f_lo, f_hi)):
            if f % self.probe_every == 0:
                if hi > f + 1:
                    self._substeps_bwd(hi, f + 1)
                self._staged("dt_substep_bwd_stage", f, 4, "bwd")
                hi = f
        if hi > f_lo:
            self._substeps_bwd(hi, f_lo)

    def set_probe(self, kind=None, stage=None, every=1):
        self.probe = None if kind is None else (kind, int(stage))
        self.probe_every = max(int(every), 1)
        self.probe_events = []
        self.probe_graph_events = []

    def probe_ms(self):
        """Mean duration (ms) of the probed launches: those recorded from the host so far and those
        recorded in graphs (as of their latest replay).  Synchronises."""
        torch.cuda.synchronize()
        ts = [a.elapsed_time(b) for a, b in self.probe_events + self.probe_graph_events]
        return (sum(ts) / len(ts)) if ts else float("nan"), len(ts)

    def stage_breakdown(self, frame: int, reps: int = 10, warmup: int = 2) -> dict:
        """Median CUDA-event time (ms) of each launch of one forward + backward substep, replayed on
        the state of ``frame`` (which must be valid): {("fwd", 0..2) | ("bwd", 0..3): ms}.  Frame + 1,
        the tape counters and the grid tape of ``frame`` and the adjoint buffers are overwritten."""
        if not 0 <= frame < self.n_frames - 1:
            raise ValueError(f"frame {frame} outside [0, {self.n_frames - 1})")
        keys = [("fwd", s) for s in range(3)] + [("bwd", s) for s in range(4)]
        times = {k: [] for k in keys}
        self.adj_clear()
        for it in range(warmup + reps):
            self.step_begin()
            ev = []
            for kind, s in keys:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                self.call("dt_substep_fwd_stage" if kind == "fwd" else "dt_substep_bwd_stage", int(frame), s)
                e1.record()
                ev.append((e0, e1))
            torch.cuda.synchronize()
            if it >= warmup:
                for k, (e0, e1) in zip(keys, ev):
                    times[k].append(e0.elapsed_time(e1))
        return {k: float(np.median(v)) for k, v in times.items()}

    def copy_frame(self, src, dst):
        self.call("dt_copy_frame", int(src), int(dst))
        self.touch(dst)

    # ---- particle re-binning (dt_rebin): the slot order follows the cells again ----
    def _rebin_scratch(self) -> torch.Tensor:
        if self._rb_scratch is None:
            n = int(self.lib.dt_rebin_scratch_bytes(self.wp))
            self._rb_scratch = torch.empty(max(n, 256), dtype=torch.uint8, device=self.device)
        return self._rb_scratch

    def _perm_follow(self, s: torch.Tensor, inverse: bool):
        """slot -> user index (and its inverse) after the slots were permuted by s (new j <- old s[j])."""
        if inverse:
            tmp = torch.empty_like(self._perm_t)
            tmp[s] = self._perm_t
            self._perm_t.copy_(tmp)
        else:
            self._perm_t.copy_(self._perm_t[s])
        self._inv_perm_t[self._perm_t] = self._slot_t

    def rebin(self, frame: int, src: torch.Tensor):
        """Sort the particles of ``frame`` by cell: ``src`` ([n_particles] int32, on the device) receives
        the permutation (new slot j <- old slot src[j]); the frame's records, the material index and the
        slot <-> caller-index maps follow it.  Other frames, the tapes and the adjoints keep the old
        order: re-bin a frame the next substeps start from."""
        if src.dtype != I32 or src.numel() != self.n_particles or not src.is_contiguous():
            raise ValueError("src must be a contiguous int32 tensor of n_particles entries")
        self.call("dt_rebin", int(frame), self.t["p_mat"].data_ptr(), src.data_ptr(),
                  self._rebin_scratch().data_ptr())
        self._perm_follow(src.long(), False)
        self.touch()

    def rebin_permute(self, src: torch.Tensor, inverse: bool, adj_buf: int = -1):
        """Apply a rebin's permutation (``inverse``: undo it) to the material index, the slot maps and,
        for ``adj_buf`` 0 or 1, to that particle adjoint buffer."""
        self.call("dt_rebin_permute", int(adj_buf), int(bool(inverse)), self.t["p_mat"].data_ptr(), src.data_ptr(),
                  self._rebin_scratch().data_ptr())
        self._perm_follow(src.long(), bool(inverse))
        self.touch()

    def adj_clear(self):
        self.call("dt_adj_clear")

    def com(self, f):
        out = torch.empty((self.n_envs, 4), dtype=F32, device=self.device)
        N.check(self.lib.dt_com(self.wp, int(f), out.data_ptr(), self.stream), "dt_com")
        return out[:, :3]
