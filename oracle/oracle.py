"""ORACLE (test infrastructure only): ctypes wrapper of the CPU restatement in oracle.cpp.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arms use this
module, to check the CUDA path's results against it.  Parity status: the forward substep is pinned
against golden substeps of the reference's own methods run on a numpy stand-in for Taichi
(tests/golden/make_substep.py, tests/test_golden_substep.py: MPM, FEM sensors, contact and rope
within 2e-15); the adjoints by analytic known-answer tests and finite differences.

Arrays are numpy in the reference layout: x, v [N,3]; C, F [N,3,3]; per sensor pos/vel/vpos/cv
[V,3]; dense grids [n0,n1,n2(,3)].
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class OrcSensor(C.Structure):
    _fields_ = [("nv", C.c_int), ("nt", C.c_int), ("nf", C.c_int), ("tets", C.c_void_p), ("tris", C.c_void_p),
                ("layer", C.c_void_p), ("B", C.c_void_p), ("mass", C.c_double), ("mu", C.c_double),
                ("lam", C.c_double), ("out_dir", C.c_double * 3), ("carry", C.c_int), ("model", C.c_int)]


class OrcRope(C.Structure):
    _fields_ = [("n", C.c_int), ("iters", C.c_int), ("mass", C.c_double), ("rad", C.c_double),
                ("rest", C.c_double), ("bend", C.c_double), ("alpha_s", C.c_double), ("alpha_b", C.c_double),
                ("relax_s", C.c_double), ("relax_b", C.c_double), ("table_h", C.c_double), ("friction", C.c_double),
                ("grav", C.c_double * 3), ("pin", C.c_double * 3),
                ("kn", C.c_double), ("kd", C.c_double), ("kt", C.c_double), ("mu_t", C.c_double)]


class OrcRopeIO(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("pos", "vel", "trav", "pos1", "vel1", "trav1", "ext", "cidx", "posb1",
                                          "velb1", "travb1", "posb", "velb", "travb")]


class OrcScene(C.Structure):
    _fields_ = [("n_particles", C.c_int), ("n", C.c_int * 3), ("bound", C.c_int), ("bc", C.c_int),
                ("dx", C.c_double), ("inv_dx", C.c_double), ("p_vol", C.c_double), ("p_mass", C.c_double),
                ("dt", C.c_double), ("eps", C.c_double), ("grav", C.c_double * 3),
                ("kn", C.c_double), ("kd", C.c_double), ("kt", C.c_double), ("mu_t", C.c_double),
                ("n_materials", C.c_int), ("n_sensors", C.c_int),
                ("mat_mu", C.c_void_p), ("mat_lam", C.c_void_p), ("mat_yield", C.c_void_p), ("mat_model", C.c_void_p),
                ("p_mat", C.c_void_p), ("sensors", C.c_void_p), ("svd_sweeps", C.c_int), ("n_threads", C.c_int),
                ("grad_clip", C.c_double), ("n_ropes", C.c_int), ("pad2_", C.c_int), ("ropes", C.c_void_p),
                ("rope_io", C.c_void_p), ("yield_branch", C.c_void_p)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P, I = C.c_void_p, C.c_int
        for name in ("orc_substep_f32", "orc_substep_f64"):
            fn = getattr(L, name)
            fn.restype = I
            fn.argtypes = [P] * 23
        for name in ("orc_svd3_f32", "orc_svd3_f64"):
            fn = getattr(L, name)
            fn.restype = None
            fn.argtypes = [I, P, P, P, P, I]
        L.orc_svd_grad_f64.restype = None
        L.orc_svd_grad_f64.argtypes = [I] + [P] * 7 + [I, P]
        L.orc_find_closest_f32.restype = None
        L.orc_find_closest_f32.argtypes = [P, P, I, P, P]
        for name in ("orc_substep_bwd_f32", "orc_substep_bwd_f64"):
            fn = getattr(L, name)
            fn.restype = I
            fn.argtypes = [P] * 27 + [I]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None else None


def _ptr_array(arrs):
    return (C.c_void_p * max(len(arrs), 1))(*[a.ctypes.data for a in arrs])


class Oracle:
    """CPU restatement of one environment's substep (float32 or float64)."""

    def __init__(self, env, dt, dtype=np.float32, svd_sweeps=None, n_threads=1, grad_clip=1000.0, yield_branch=None):
        """``yield_branch``: optional [n_particles] branch of the von Mises return map per particle (-1
        decided by the yield test, 0 elastic, 1 yielding), to evaluate the substep on the branch another
        implementation took where the yield test's outcome depends on rounding."""
        self.env = env
        self.dtype = np.dtype(dtype)
        self.dt = float(dt)
        self.keep = []
        sc = OrcScene()
        sc.n_particles = env.n_particles
        sc.n[:] = list(env.n_grid)
        sc.bound, sc.bc = env.bound, env.bc
        sc.dx = float(env.dx)
        sc.inv_dx = 1.0 / float(env.dx)
        sc.p_vol = float(env.volume)
        sc.p_mass = float(env.p_mass)
        sc.dt = self.dt
        sc.eps = float(env.eps)
        sc.grav[:] = list(env.gravity)
        sc.kn, sc.kd, sc.kt, sc.mu_t = env.kn, env.kd, env.kt, env.mu_t
        mu = np.array([m.mu_lam[0] for m in env.materials], np.float64)
        lam = np.array([m.mu_lam[1] for m in env.materials], np.float64)
        ys = np.array([m.yield_stress for m in env.materials], np.float64)
        mdl = np.array([m.model for m in env.materials], np.int32)
        pm = np.zeros(env.n_particles, np.int32) if env.mat is None else np.ascontiguousarray(env.mat, np.int32)
        self.keep += [mu, lam, ys, mdl, pm]
        sc.n_materials = len(env.materials)
        sc.mat_mu, sc.mat_lam, sc.mat_yield, sc.mat_model, sc.p_mat = map(_ptr, (mu, lam, ys, mdl, pm))
        sens = (OrcSensor * max(len(env.sensors), 1))()
        for i, sp in enumerate(env.sensors):
            tets = np.ascontiguousarray(sp.tets, np.int32)
            tris = np.ascontiguousarray(sp.tris, np.int32)
            layer = np.ascontiguousarray(sp.layer, np.int32)
            B = np.ascontiguousarray(sp.rest_inverse().astype(np.float64).reshape(-1, 9))
            self.keep += [tets, tris, layer, B]
            s = sens[i]
            s.nv, s.nt, s.nf = len(sp.verts), len(tets), len(tris)
            s.tets, s.tris, s.layer, s.B = map(_ptr, (tets, tris, layer, B))
            m_, l_ = sp.lame()
            s.mass, s.mu, s.lam = float(sp.mass), float(m_), float(l_)
            s.out_dir[:] = [float(c) for c in sp.out_dir]
            s.carry = int(sp.carry)
            s.model = int(getattr(sp, "model", 0))
        self.keep.append(sens)
        sc.n_sensors = len(env.sensors)
        sc.sensors = C.cast(sens, C.c_void_p)
        sc.svd_sweeps = svd_sweeps if svd_sweeps is not None else (4 if self.dtype == np.float32 else 12)
        sc.n_threads = n_threads
        sc.grad_clip = grad_clip
        ropes = list(getattr(env, "ropes", []))
        rr = (OrcRope * max(len(ropes), 1))()
        for i, rp in enumerate(ropes):
            r = rr[i]
            r.n = rp.n
            r.iters = int(getattr(rp, "iters", 1))
            r.mass, r.rad, r.rest, r.bend = rp.mass, rp.rad, rp.rest, rp.bend
            cs, cb = rp.compliance
            r.alpha_s, r.alpha_b = cs / self.dt ** 2, cb / self.dt ** 2
            r.relax_s, r.relax_b = rp.stretch_relax, rp.bend_relax
            r.table_h, r.friction = rp.table_h, rp.friction
            r.grav[:] = list(rp.gravity)
            r.pin[:] = [float(c) for c in rp.init_positions()[0]]
            r.kn, r.kd, r.kt, r.mu_t = rp.kn, rp.kd, rp.kt, rp.mu_t
        self.rope_io = (OrcRopeIO * max(len(ropes), 1))()
        self.keep += [rr, self.rope_io]
        sc.n_ropes = len(ropes)
        sc.ropes = C.cast(rr, C.c_void_p)
        sc.rope_io = C.cast(self.rope_io, C.c_void_p)
        self.ropes = ropes
        if yield_branch is not None:
            yb = np.ascontiguousarray(yield_branch, np.int8)
            if yb.shape != (env.n_particles,):
                raise ValueError(f"yield_branch: {yb.shape}, expected ({env.n_particles},)")
            self.keep.append(yb)
            sc.yield_branch = _ptr(yb)
        self.sc = sc
        self.fn = lib().orc_substep_f32 if self.dtype == np.float32 else lib().orc_substep_f64
        self.fn.restype = C.c_int

    def initial_state(self):
        e = self.env
        T = self.dtype
        N = e.n_particles
        st = {"x": np.array(e.x, T), "v": np.zeros((N, 3), T) if e.v is None else np.array(np.broadcast_to(e.v, (N, 3)), T),
              "C": np.zeros((N, 3, 3), T), "F": np.array(np.broadcast_to(np.eye(3), (N, 3, 3)), T)}
        st["pos"] = [np.array(sp.verts, T) for sp in e.sensors]
        st["vel"] = [np.zeros((len(sp.verts), 3), T) for sp in e.sensors]
        st["vpos"] = [np.array(sp.verts, T) for sp in e.sensors]
        st["rpos"] = [np.array(rp.init_positions(), T) for rp in self.ropes]
        st["rvel"] = [np.zeros((rp.n, 3), T) if rp.v is None else np.array(rp.v, T) for rp in self.ropes]
        st["rtrav"] = [np.zeros(rp.n, T) for rp in self.ropes]
        return st

    def _rope_io(self, st, c, adj1=None):
        """Fill the per-rope io structs; returns the arrays (kept alive by the caller)."""
        T = self.dtype
        NS = len(self.env.sensors)
        arrs = []
        for i, rp in enumerate(self.ropes):
            a = {"pos": c(st["rpos"][i]), "vel": c(st["rvel"][i]), "trav": c(st["rtrav"][i]),
                 "pos1": np.zeros((rp.n, 3), T), "vel1": np.zeros((rp.n, 3), T), "trav1": np.zeros(rp.n, T),
                 "ext": np.zeros((rp.n, 3), T), "cidx": np.full((rp.n, max(NS, 1)), -1, np.int32)}
            if adj1 is not None:
                a["posb1"] = c(adj1.get("rpos", [np.zeros((rp.n, 3))] * len(self.ropes))[i])
                a["velb1"] = c(adj1.get("rvel", [np.zeros((rp.n, 3))] * len(self.ropes))[i])
                a["travb1"] = c(adj1.get("rtrav", [np.zeros(rp.n)] * len(self.ropes))[i])
                a["posb"], a["velb"], a["travb"] = np.zeros((rp.n, 3), T), np.zeros((rp.n, 3), T), np.zeros(rp.n, T)
            io = self.rope_io[i]
            for k, v in a.items():
                setattr(io, k, v.ctypes.data)
            arrs.append(a)
        return arrs

    def substep(self, st, cv=None, cv1=None):
        """One substep.  ``cv``/``cv1``: per-sensor control velocities of frames f and f+1 (default 0).
        Returns (new state, debug dict)."""
        T = self.dtype
        e = self.env
        n0, n1, n2 = e.n_grid
        N = e.n_particles
        NS = len(e.sensors)
        c = lambda a: np.ascontiguousarray(a, T)  # noqa: E731
        x, v, Cm, F = c(st["x"]), c(st["v"]), c(st["C"]), c(st["F"])
        out = {"x": np.zeros((N, 3), T), "v": np.zeros((N, 3), T), "C": np.zeros((N, 3, 3), T),
               "F": np.zeros((N, 3, 3), T)}
        pos = [c(a).copy() for a in st.get("pos", [])]
        vel = [c(a).copy() for a in st.get("vel", [])]  # updated in place by the elastic forces
        vpos = [c(a) for a in st.get("vpos", [])]
        zeros_v = [np.zeros((len(sp.verts), 3), T) for sp in e.sensors]
        cv = [c(a) for a in cv] if cv is not None else zeros_v
        cv1 = [c(a) for a in cv1] if cv1 is not None else cv
        pos1 = [np.zeros_like(a) for a in pos]
        vel1 = [np.zeros_like(a) for a in pos]
        vpos1 = [np.zeros_like(a) for a in pos]
        ext = [np.zeros_like(a) for a in pos]
        gm = np.zeros((n0, n1, n2), T)
        gvi = np.zeros((n0, n1, n2, 3), T)
        gvo = np.zeros((n0, n1, n2, 3), T)
        gf = np.zeros((n0, n1, n2, 3), T)
        cidx = np.full((n0, n1, n2, max(NS, 1)), -1, np.int32)
        rio = self._rope_io(st, c)
        err = self.fn(C.byref(self.sc), _ptr(x), _ptr(v), _ptr(Cm), _ptr(F), _ptr(out["x"]), _ptr(out["v"]),
                      _ptr(out["C"]), _ptr(out["F"]), _ptr_array(pos), _ptr_array(vel), _ptr_array(vpos),
                      _ptr_array(cv), _ptr_array(cv1), _ptr_array(pos1), _ptr_array(vel1), _ptr_array(vpos1),
                      _ptr_array(ext), _ptr(gm), _ptr(gvi), _ptr(gvo), _ptr(gf), _ptr(cidx))
        out["pos"], out["vel"], out["vpos"] = pos1, vel1, vpos1
        out["rpos"] = [a["pos1"] for a in rio]
        out["rvel"] = [a["vel1"] for a in rio]
        out["rtrav"] = [a["trav1"] for a in rio]
        dbg = {"grid_m": gm, "grid_v_in": gvi, "grid_v_out": gvo, "grid_f": gf, "cidx": cidx, "vel_mid": vel,
               "ext": ext, "err": err, "rope_ext": [a["ext"] for a in rio], "rope_cidx": [a["cidx"] for a in rio]}
        return out, dbg

    def substep_bwd(self, st, adj1, cv=None, cv1=None, svd_grad_mode=0):
        """Adjoint of one substep (recomputes the forward internally).  ``adj1``: adjoint of frame
        f+1 with keys x, v, C, F (and per-sensor lists pos, vel, vpos).  Returns the adjoint of frame
        f (same keys) plus per-sensor control-velocity adjoints cv (frame f), cv1 (frame f+1) and the
        material adjoint mat [n_materials, 2] (d/dmu, d/dlambda)."""
        T = self.dtype
        e = self.env
        N = e.n_particles
        NS = len(e.sensors)
        c = lambda a: np.ascontiguousarray(a, T)  # noqa: E731
        x, v, Cm, F = c(st["x"]), c(st["v"]), c(st["C"]), c(st["F"])
        zeros_v = [np.zeros((len(sp.verts), 3), T) for sp in e.sensors]
        pos = [c(a) for a in st.get("pos", [])]
        vel = [c(a) for a in st.get("vel", [])]
        vpos = [c(a) for a in st.get("vpos", [])]
        cv = [c(a) for a in cv] if cv is not None else zeros_v
        cv1 = [c(a) for a in cv1] if cv1 is not None else cv
        a1 = {k: c(adj1[k]) for k in ("x", "v", "C", "F")}
        for k in ("pos", "vel", "vpos"):
            a1[k] = [c(a) for a in adj1.get(k, zeros_v)]
        out = {"x": np.zeros((N, 3), T), "v": np.zeros((N, 3), T), "C": np.zeros((N, 3, 3), T),
               "F": np.zeros((N, 3, 3), T)}
        for k in ("pos", "vel", "vpos", "cv", "cv1"):
            out[k] = [np.zeros_like(z) for z in zeros_v]
        out["mat"] = np.zeros((len(e.materials), 2), T)
        rio = self._rope_io(st, c, adj1)
        fn = lib().orc_substep_bwd_f32 if T == np.float32 else lib().orc_substep_bwd_f64
        fn(C.byref(self.sc), _ptr(x), _ptr(v), _ptr(Cm), _ptr(F), _ptr_array(pos), _ptr_array(vel), _ptr_array(vpos),
           _ptr_array(cv), _ptr_array(cv1), _ptr(a1["x"]), _ptr(a1["v"]), _ptr(a1["C"]), _ptr(a1["F"]),
           _ptr_array(a1["pos"]), _ptr_array(a1["vel"]), _ptr_array(a1["vpos"]), _ptr(out["x"]), _ptr(out["v"]),
           _ptr(out["C"]), _ptr(out["F"]), _ptr_array(out["pos"]), _ptr_array(out["vel"]), _ptr_array(out["vpos"]),
           _ptr_array(out["cv"]), _ptr_array(out["cv1"]), _ptr(out["mat"]), svd_grad_mode)
        out["rpos"] = [a["posb"] for a in rio]
        out["rvel"] = [a["velb"] for a in rio]
        out["rtrav"] = [a["travb"] for a in rio]
        return out


def svd3(A, dtype=np.float32, sweeps=None):
    """Standalone 3x3 SVD of the oracle: A [n,3,3] -> U [n,3,3], s [n,3], V [n,3,3]."""
    T = np.dtype(dtype)
    A = np.ascontiguousarray(A, T).reshape(-1, 3, 3)
    n = len(A)
    U, s, V = np.zeros_like(A), np.zeros((n, 3), T), np.zeros_like(A)
    fn = lib().orc_svd3_f32 if T == np.float32 else lib().orc_svd3_f64
    fn(C.c_int(n), _ptr(A), _ptr(U), _ptr(s), _ptr(V), C.c_int(sweeps if sweeps else (4 if T == np.float32 else 12)))
    return U, s, V


def svd_grad(U, s, V, Ub, sb, Vb, Rb, mode=0):
    """Standalone SVD adjoint of the oracle in float64 (svd_grad, mpm_elastic.py:145-173): the adjoint
    of F = U diag(s) V^T from the adjoints of U, s, V and of R = U V^T.  All [n,3,3] / [n,3]."""
    a = [np.ascontiguousarray(x, np.float64).reshape(-1, 3, 3) for x in (U, V, Ub, Vb, Rb)]
    ss = [np.ascontiguousarray(x, np.float64).reshape(-1, 3) for x in (s, sb)]
    Fb = np.zeros_like(a[0])
    lib().orc_svd_grad_f64(C.c_int(len(Fb)), _ptr(a[0]), _ptr(ss[0]), _ptr(a[1]), _ptr(a[2]), _ptr(ss[1]),
                           _ptr(a[3]), _ptr(a[4]), C.c_int(mode), _ptr(Fb))
    return Fb


def find_closest(sensor, pos, queries):
    """Standalone argmin of find_closest (fem_sensor.py:344-359) in float32."""
    s = OrcSensor()
    tris = np.ascontiguousarray(sensor.tris, np.int32)
    s.nv, s.nf = len(pos), len(tris)
    s.tris = _ptr(tris)
    pos = np.ascontiguousarray(pos, np.float32)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
    out = np.zeros(len(q), np.int32)
    lib().orc_find_closest_f32(C.byref(s), _ptr(pos), C.c_int(len(q)), _ptr(q), _ptr(out))
    return out
