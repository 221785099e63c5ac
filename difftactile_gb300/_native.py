"""ctypes binding of the C ABI declared in include/difftactile_gb300.h.

The CUDA library is the only compute path: importing this module without the built library
raises, and there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB


class DtEnv(C.Structure):
    _fields_ = [
        ("p_begin", C.c_int), ("p_end", C.c_int), ("node_off", C.c_int), ("blk_off", C.c_int),
        ("nb", C.c_int * 3), ("n", C.c_int * 3), ("bound", C.c_int), ("bc", C.c_int),
        ("s_begin", C.c_int), ("s_end", C.c_int),
        ("dx", C.c_float), ("inv_dx", C.c_float), ("p_mass", C.c_float), ("stress_k", C.c_float),
        ("eps", C.c_float), ("g2p_k", C.c_float), ("dt_g", C.c_float * 3),
        ("kn", C.c_float), ("kd", C.c_float), ("kt", C.c_float), ("mu_t", C.c_float), ("pad_", C.c_float),
    ]


class DtSensor(C.Structure):
    _fields_ = [
        ("v_off", C.c_int), ("nv", C.c_int), ("t_off", C.c_int), ("nt", C.c_int),
        ("f_off", C.c_int), ("nf", C.c_int), ("env", C.c_int), ("carry", C.c_int),
        ("dt_over_m", C.c_float), ("mu", C.c_float), ("lam", C.c_float), ("alpha", C.c_float),
        ("out_dir", C.c_float * 3), ("model", C.c_int),
    ]


class DtRope(C.Structure):
    _fields_ = [("p_off", C.c_int), ("n", C.c_int), ("env", C.c_int), ("blk_off", C.c_int),
                ("mass", C.c_float), ("inv_m", C.c_float), ("rad", C.c_float), ("rest", C.c_float),
                ("bend", C.c_float), ("alpha_s", C.c_float), ("alpha_b", C.c_float), ("relax_s", C.c_float),
                ("relax_b", C.c_float), ("table_h", C.c_float), ("friction", C.c_float), ("dt_g", C.c_float * 3),
                ("pin", C.c_float * 3), ("kn", C.c_float), ("kd", C.c_float), ("kt", C.c_float), ("mu_t", C.c_float),
                ("iters", C.c_int)]


class DtFisheye(C.Structure):
    _fields_ = [("f", C.c_float), ("m", C.c_float), ("cx", C.c_float), ("cy", C.c_float), ("plane", C.c_float)]


class DtMaterial(C.Structure):
    _fields_ = [("mu", C.c_float), ("lam", C.c_float), ("yield_stress", C.c_float), ("model", C.c_int)]


_P = C.c_void_p
WORLD_PTR_FIELDS = [
    "envs", "sensors", "materials", "p_env", "p_mat", "blk_env", "tets", "tet_B", "tet_sensor", "tris",
    "tri_perm", "v_layer", "v_sensor",
    "p_state", "p_adj",
    "g_acc", "g_vout", "g_adj_vout", "g_adj_acc", "blk_flag",
    "tape_blist", "tape_bcount", "tape_acc", "tape_vout", "tape_cidx",
    "v_pos", "v_vel", "v_velmid", "v_ext", "v_vpos", "v_cv", "tri_cent",
    "v_adj_pos", "v_adj_vel", "v_adj_vpos", "v_adj_velmid", "v_adj_ext", "v_adj_cv", "mat_adj",
    "err",
]
ROPE_PTR_FIELDS = ["ropes", "r_state", "r_ext", "r_cidx", "r_adj", "r_extb"]
ROPE_INT_FIELDS = ["n_ropes", "n_rope_particles", "rope_blocks", "max_rope_n"]
WORLD_INT_FIELDS = [
    "n_envs", "n_particles", "n_sensors", "n_materials", "n_verts", "n_tets", "n_tris",
    "n_nodes", "n_blocks", "n_frames", "tape_blocks",
]


class DtWorld(C.Structure):
    _fields_ = ([(n, _P) for n in WORLD_PTR_FIELDS] + [(n, C.c_int) for n in WORLD_INT_FIELDS]
                + [("dt", C.c_float), ("grad_clip", C.c_float), ("svd_sweeps", C.c_int),
                   ("svd_grad_mode", C.c_int), ("max_sensor_tris", C.c_int), ("scatter_mode", C.c_int)]
                + [(n, _P) for n in ROPE_PTR_FIELDS] + [(n, C.c_int) for n in ROPE_INT_FIELDS]
                + [("p_svd", _P), ("p_block", C.c_int), ("scatter_depth", C.c_int), ("contact_lanes", C.c_int),
                   ("skip_tape", C.c_int), ("r_work", _P), ("max_rope_iters", C.c_int), ("p_per_thread", C.c_int)]
                + [("aux_stream", _P), ("aux_events", _P * 2), ("t_svd", _P)]
                + [("scatter_depth_adj", C.c_int)])


# entry points: name -> (restype, argtypes)
_W = C.POINTER(DtWorld)
SIGNATURES = {
    "dt_abi_version": (C.c_int, []),
    "dt_sizeof_world": (C.c_size_t, []),
    "dt_sizeof_env": (C.c_size_t, []),
    "dt_sizeof_sensor": (C.c_size_t, []),
    "dt_sizeof_material": (C.c_size_t, []),
    "dt_sizeof_rope": (C.c_size_t, []),
    "dt_set_pdl": (C.c_int, [C.c_int]),
    "dt_get_pdl": (C.c_int, []),
    "dt_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "dt_step_begin": (C.c_int, [_W, _P]),
    "dt_substep_fwd": (C.c_int, [_W, C.c_int, _P]),
    "dt_substep_fwd_stage": (C.c_int, [_W, C.c_int, C.c_int, _P]),
    "dt_substep_fwd_noalloc": (C.c_int, [_W, C.c_int, _P]),
    "dt_rebin_scratch_bytes": (C.c_size_t, [_W]),
    "dt_rebin": (C.c_int, [_W, C.c_int, _P, _P, _P, _P]),
    "dt_rebin_permute": (C.c_int, [_W, C.c_int, C.c_int, _P, _P, _P, _P]),
    "dt_p2g": (C.c_int, [_W, C.c_int, _P]),
    "dt_fem_update": (C.c_int, [_W, C.c_int, _P]),
    "dt_grid_op": (C.c_int, [_W, C.c_int, _P]),
    "dt_g2p": (C.c_int, [_W, C.c_int, _P]),
    "dt_fem_update2": (C.c_int, [_W, C.c_int, _P]),
    "dt_rope_update": (C.c_int, [_W, C.c_int, _P]),
    "dt_rope_update_bwd": (C.c_int, [_W, C.c_int, _P]),
    "dt_copy_frame": (C.c_int, [_W, C.c_int, C.c_int, _P]),
    "dt_substep_bwd": (C.c_int, [_W, C.c_int, _P]),
    "dt_substep_bwd_stage": (C.c_int, [_W, C.c_int, C.c_int, _P]),
    "dt_substeps_bwd": (C.c_int, [_W, C.c_int, C.c_int, _P]),
    "dt_adj_clear": (C.c_int, [_W, _P]),
    "dt_com": (C.c_int, [_W, C.c_int, _P, _P]),
    "dt_com_bwd": (C.c_int, [_W, C.c_int, _P, _P]),
    "dt_pose_control_vel": (C.c_int, [_W, C.c_int, _P, C.c_float, C.c_int, C.c_int, _P]),
    "dt_pose_control_vel_all": (C.c_int, [_W, _P, C.c_float, C.c_int, C.c_int, _P]),
    "dt_pose_control_vel_bwd": (C.c_int, [_W, C.c_int, _P, C.c_float, _P, C.c_int, C.c_int, _P]),
    "dt_pose_control_vel_bwd_all": (C.c_int, [_W, _P, C.c_float, _P, C.c_int, C.c_int, _P]),
    "dt_affine_control_vel": (C.c_int, [_W, C.c_int, _P, _P, C.c_int, C.c_int, _P]),
    "dt_affine_control_vel_bwd": (C.c_int, [_W, C.c_int, _P, C.c_int, C.c_int, _P, _P]),
    "dt_grid_mass": (C.c_int, [_W, C.c_int, C.c_int, _P, _P]),
    "dt_deform_loss": (C.c_int, [_W, C.c_int, _P, _P, _P, C.c_float, C.c_float, _P, _P]),
    "dt_deform_loss_bwd": (C.c_int, [_W, C.c_int, C.c_int, _P, _P, _P, C.c_float, C.c_float, C.c_float, _P]),
    "dt_target_sdf": (C.c_int, [_W, C.c_int, _P, _P, _P, C.c_int, _P]),
    "dt_rigid_match": (C.c_int, [_W, C.c_int, C.c_int, C.c_int, _P, _P]),
    "dt_rigid_match_bwd": (C.c_int, [_W, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P]),
    "dt_contact_force": (C.c_int, [_W, C.c_int, C.c_int, _P, _P]),
    "dt_contact_force_bwd": (C.c_int, [_W, C.c_int, _P, _P]),
    "dt_markers": (C.c_int, [_W, C.c_int, C.c_int, _P, _P, _P, C.c_int, C.c_int, _P, DtFisheye, _P, _P, _P]),
    "dt_markers_bwd": (C.c_int, [_W, C.c_int, C.c_int, _P, _P, _P, C.c_int, C.c_int, _P, DtFisheye, _P, _P, _P,
                                 _P]),
    "dt_marker_loss": (C.c_int, [_W, C.c_int, C.c_int, C.c_int, _P, _P, _P]),
    "dt_marker_loss_bwd": (C.c_int, [_W, C.c_int, C.c_int, C.c_int, _P, C.c_float, _P]),
}

ERRORS = {0: "DT_OK", -1: "DT_ERR_ARG", -2: "DT_ERR_LAUNCH", -3: "DT_ERR_CAPACITY"}
DEVERR = {1: "particle left the grid's safe band", 2: "grid tape capacity exceeded", 4: "non-finite value",
          8: "rope iterations beyond the adjoint workspace"}


class DtError(RuntimeError):
    pass


_lib = None


def load(path: str | None = None):
    """Load the CUDA library (built by ``difftactile_gb300.build.build()``); raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("DIFFTACTILE_GB300_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(
            f"difftactile_gb300 CUDA library not found at {path}; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    import torch  # noqa: F401  (loads the CUDA runtime the library links against)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    for name, cls in (("world", DtWorld), ("env", DtEnv), ("sensor", DtSensor), ("material", DtMaterial),
                      ("rope", DtRope)):
        n = getattr(lib, f"dt_sizeof_{name}")()
        if n != C.sizeof(cls):
            raise ImportError(f"ABI mismatch: sizeof(dt_{name}) = {n} in the library, {C.sizeof(cls)} in ctypes")
    if lib.dt_abi_version() != 8:
        raise ImportError("ABI version mismatch")
    _lib = lib
    return lib


def last_error() -> tuple[int, str]:
    """(cudaError_t code, "name: description") behind the last DT_ERR_LAUNCH on this thread; clears it."""
    buf = C.create_string_buffer(256)
    code = load().dt_last_error(buf, len(buf))
    return code, buf.value.decode(errors="replace")


def check(rc: int, what: str):
    if rc != 0:
        detail = ""
        if rc == -2 and _lib is not None:
            code, msg = last_error()
            detail = f" ({msg})" if code else ""
        raise DtError(f"{what} failed: {ERRORS.get(rc, rc)}{detail}")
