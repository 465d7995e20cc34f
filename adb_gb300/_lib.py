"""ctypes binding of libabd_gb300.so (the C ABI declared in include/abd_gb300.h).

The library is the only compute path: importing this module raises if it is missing
(build it with ``python -c "import __graft_entry__ as g; g.build()"`` or
``python adb_gb300/build.py``); there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libabd_gb300.so")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)

STATUS = {0: "ABD_OK", 1: "ABD_ERR_NAN", 2: "ABD_ERR_LS_STALL", 3: "ABD_ERR_PAIR_OVERFLOW", 4: "ABD_ERR_TOI_TINY",
          5: "ABD_ERR_NOT_SPD", 6: "ABD_ERR_PCG_NOCONV", 7: "ABD_ERR_CUDA", 8: "ABD_ERR_INVALID", 9: "ABD_ERR_IO",
          10: "ABD_ERR_SAME_DIRECTION"}


class AbdConfig(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dt", "kappa", "dhat", "ortho_kappa", "ground_offset", "mu", "evh", "eps_x", "backoff", "c1", "tol",
        "max_uk", "gravity_y", "ls_grad_tol", "pcg_rel_tol")] + [(n, C.c_int) for n in (
            "max_iter", "ground", "pt", "ee", "psd", "line_search", "upper_bound", "vg_fric", "pt_fric", "ee_fric",
            "clip", "pcg_max_iter", "iaabb", "full_ccd")] + [(n, C.c_double) for n in (
                "safe_factor", "sh_min_xyz", "sh_dx")] + [(n, C.c_int) for n in (
                    "sh_xyz_bits", "sh_fix_edge_trajectory")] + [("dq_tol", C.c_double), ("damping", C.c_int),
                                                                 ("damp_alpha", C.c_double), ("damp_beta", C.c_double),
                                                                 ("pcg_refine", C.c_int), ("pcg_refine_tol", C.c_double),
                                                                 ("solver", C.c_int), ("max_iter_frame", C.c_int),
                                                                 ("autotune", C.c_int), ("tri_direct", C.c_int)]


class AbdSceneDesc(C.Structure):
    _fields_ = [("n_bodies", C.c_int), ("q0", _D), ("dqdt", _D), ("mass", _D), ("Ic", _D), ("vert_off", _I),
                ("rest_vertices", _D), ("edge_off", _I), ("edges", _I), ("face_off", _I), ("faces", _I),
                ("scene_id", _I)]


class AbdFrameStats(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("frames", "newton_iters", "ls_trials", "pcg_iters", "n_pt", "n_ee", "n_vg",
                                       "n_overlaps", "status", "pad")] + [("kernel_launches", C.c_longlong)] + [
        (n, C.c_double) for n in ("toi_min", "alpha_min", "t_ipc_ms", "t_solver_ms", "t_ccd_ms", "t_ls_ms",
                                  "bytes_moved", "device_ms")]

    def as_dict(self):
        return {f[0]: getattr(self, f[0]) for f in self._fields_ if f[0] != "pad"}


class AbdError(RuntimeError):
    pass


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libabd_gb300.so is not built (%s); run adb_gb300/build.py" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        L.abd_create.argtypes = [C.POINTER(AbdSceneDesc), C.POINTER(AbdConfig), C.POINTER(H)]
        L.abd_create_from_files.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(H)]
        L.abd_step.argtypes = [H, C.c_double, C.c_int, C.POINTER(AbdFrameStats)]
        L.abd_get_state.argtypes = [H, _D, _D]
        L.abd_trace_save.argtypes = [H, C.c_char_p, C.c_int, C.c_int]
        L.abd_trace_load.argtypes = [H, C.c_char_p, C.c_int]
        L.abd_set_trace.argtypes = [H, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_char_p]
        L.abd_get_trace.argtypes = [H, _I, _I, _I, C.c_char_p, C.c_int]
        L.abd_trace_files.argtypes = [H, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p)]
        L.abd_run.argtypes = [H, C.c_int, C.POINTER(AbdFrameStats)]
        L.abd_set_state.argtypes = [H, _D, _D]
        L.abd_get_counts.argtypes = [H, _I, _I, _I, _I]
        L.abd_get_iter.argtypes = [H]
        L.abd_set_iter.argtypes = [H, C.c_int]
        L.abd_set_friction.argtypes = [H, C.c_double]
        L.abd_get_friction.argtypes = [H, C.POINTER(C.c_double)]
        L.abd_adjoint_frame.argtypes = [H, _D, _D, _D, _D, _D, _D, C.POINTER(C.c_double)]
        L.abd_adjoint_stats.argtypes = [H, _I, _D]
        L.abd_autotune_info.argtypes = [H, _I, _D]
        L.abd_get_scene_count.argtypes = [H]
        L.abd_get_scene_stats.argtypes = [H, _I, _I, _I, _I]
        L.abd_last_error.restype = C.c_char_p
        L.abd_last_error.argtypes = [H]
        L.abd_destroy.argtypes = [H]
        L.abd_cull.argtypes = [H, C.c_int, _D, _D, _I, _D]
        L.abd_get_pairs.argtypes = [H, _I, _I, _I, _I, _I]
        L.abd_newton_system.argtypes = [H, _D, _D, _D, _I, _I, _D, C.c_int]
        L.abd_newton_dq.argtypes = [H, _D, _D, _I]
        L.abd_energy.argtypes = [H, _D, _D, _D, _I, _D, _D, _D, _D, _D, _D]
        L.abd_ipc_hess_pt_batch.argtypes = [C.c_int, _D, _I, _D, C.c_double, C.c_double, C.c_int, _D, _D]
        L.abd_ipc_hess_ee_batch.argtypes = [C.c_int, _D, _I, _D, C.c_double, C.c_double, C.c_double, C.c_int, _D,
                                            _D, _D]
        L.abd_pt_collision_time_batch.argtypes = [C.c_int, _D, _D]
        L.abd_ee_collision_time_batch.argtypes = [C.c_int, _D, _D]
        L.abd_pt_distance_batch.argtypes = [C.c_int, _D, _I, _D]
        L.abd_ee_distance_batch.argtypes = [C.c_int, _D, _I, _D]
        L.abd_profile.argtypes = [H, C.c_int]
        L.abd_kernel_times.argtypes = [H, C.c_int, C.c_char_p, _D, C.POINTER(C.c_longlong)]
        L.abd_kernel_work.argtypes = [H, C.c_int, C.c_char_p, _D, C.POINTER(C.c_longlong), _D, _D]
        L.abd_pt_min_toi_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.abd_noalloc_last_error.restype = C.c_char_p
        L.abd_noalloc_last_error.argtypes = []
        L.abd_measure_fp64_gflops.restype = C.c_double
        L.abd_measure_fp64_gflops.argtypes = []
        _lib = L
    return _lib


# Every symbol include/abd_gb300.h declares (checked by the CPU test suite).
EXPORTED = ["abd_create", "abd_create_from_files", "abd_step", "abd_get_state", "abd_set_state", "abd_trace_save", "abd_trace_load", "abd_set_trace", "abd_get_trace", "abd_trace_files", "abd_run", "abd_get_counts",
            "abd_get_iter", "abd_set_iter", "abd_get_scene_count", "abd_get_scene_stats", "abd_set_friction", "abd_get_friction", "abd_adjoint_frame", "abd_adjoint_stats", "abd_autotune_info", "abd_last_error", "abd_destroy", "abd_profile", "abd_kernel_times", "abd_kernel_work", "abd_cull", "abd_get_pairs",
            "abd_newton_system", "abd_newton_dq", "abd_energy", "abd_ipc_hess_pt_batch", "abd_ipc_hess_ee_batch",
            "abd_pt_collision_time_batch", "abd_ee_collision_time_batch", "abd_pt_distance_batch",
            "abd_ee_distance_batch", "abd_pt_min_toi_noalloc", "abd_noalloc_last_error", "abd_measure_fp64_gflops"]


def dptr(a):
    return a.ctypes.data_as(_D)


def iptr(a):
    return a.ctypes.data_as(_I)


def check(rc: int, h=None, what: str = ""):
    if rc != 0:
        msg = lib().abd_last_error(h).decode(errors="replace") if h is not None else ""
        raise AbdError("%s failed: %s %s" % (what, STATUS.get(rc, rc), msg))
