"""ctypes bindings of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the product package never does. The shared library is built by
``make -C oracle`` (see oracle/Makefile).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libabd_oracle.so")
REF_CUBIC_PATH = os.path.join(HERE, "_ref", "libref_cubic.so")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class OracleConfig(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "dt", "kappa", "dhat", "ortho_kappa", "ground_offset", "mu", "evh", "eps_x", "backoff", "c1", "tol",
        "max_uk", "dq_tol", "gravity_y", "ls_grad_tol")] + [(n, C.c_int) for n in (
            "max_iter", "ground", "pt", "ee", "psd", "line_search", "upper_bound", "vg_fric", "pt_fric",
            "ee_fric", "clip", "n_threads")] + [(n, C.c_double) for n in ("safe_factor", "sh_min_xyz", "sh_dx")] + [
        (n, C.c_int) for n in ("iaabb", "full_ccd", "sh_bits", "sh_fix_edge", "damp")] + [
        (n, C.c_double) for n in ("damp_alpha", "damp_beta")] + [("max_iter_frame", C.c_int)]


class OracleStats(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("newton_iters", "ls_trials", "n_pt", "n_ee", "n_vg", "status")] + [
        (n, C.c_double) for n in ("toi_min", "alpha_min", "t_ipc", "t_solver", "t_ccd", "t_ls")]


_lib = None


def build() -> None:
    import subprocess
    subprocess.check_call(["make", "-s", "-C", HERE, "libabd_oracle.so"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int, _D, _D, _D, _D, _I, _D, _I, _I, _I, _I, C.POINTER(OracleConfig)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int, C.POINTER(OracleStats)]
        L.orc_get_state.argtypes = [C.c_void_p, _D, _D]
        L.orc_set_state.argtypes = [C.c_void_p, _D, _D]
        L.orc_get_iter.argtypes = [C.c_void_p]
        L.orc_set_iter.argtypes = [C.c_void_p, C.c_int]
        L.orc_cull.restype = C.c_double
        L.orc_cull.argtypes = [C.c_void_p, C.c_int, _D, _D, _I]
        L.orc_get_pairs.argtypes = [C.c_void_p, _I, _I, _I, _I, _I]
        L.orc_newton_system.argtypes = [C.c_void_p, _D, _D, _D, _I, _D, C.c_int]
        L.orc_newton_dq.argtypes = [C.c_void_p, _D, _D]
        L.orc_energy_terms.argtypes = [C.c_void_p, _D, _D, _D, _I, _D, _D, _D, _D, _D, _D]
        L.orc_energy.restype = C.c_double
        L.orc_energy.argtypes = [C.c_void_p, _D]
        L.orc_stats_last.argtypes = [C.c_void_p, C.POINTER(OracleStats)]
        L.orc_pt_type.argtypes = [_D]
        L.orc_pt_dist.restype = C.c_double
        L.orc_pt_dist.argtypes = [_D, C.c_int]
        L.orc_ee_type.argtypes = [_D]
        L.orc_ee_dist.restype = C.c_double
        L.orc_ee_dist.argtypes = [_D, C.c_int]
        L.orc_ipc_hess_pt.argtypes = [_D, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _D, _D]
        L.orc_ipc_hess_ee.restype = C.c_double
        L.orc_ipc_hess_ee.argtypes = [_D, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _D, _D]
        L.orc_barrier.restype = C.c_double
        L.orc_barrier.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_pt_collision_time.restype = C.c_double
        L.orc_pt_collision_time.argtypes = [_D]
        L.orc_ee_collision_time.restype = C.c_double
        L.orc_ee_collision_time.argtypes = [_D]
        L.orc_cubic_roots.argtypes = [_D, C.c_double, C.c_double, _D]
        L.orc_det_polynomial.argtypes = [_D, _D, _D]
        L.orc_friction.argtypes = [_D, C.c_double, _D, C.c_double, C.c_double, C.c_double, _D, _D]
        L.orc_f0.restype = C.c_double
        L.orc_f0.argtypes = [C.c_double, C.c_double]
        L.orc_pt_frame.argtypes = [_D, C.c_int, _D]
        L.orc_ee_frame.argtypes = [_D, C.c_int, _D]
        assert L.orc_sizeof_config() == C.sizeof(OracleConfig)
        assert L.orc_sizeof_stats() == C.sizeof(OracleStats)
        _lib = L
    return _lib


def _d(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _i(a: np.ndarray):
    return a.ctypes.data_as(_I)


def make_config(cfg, n_threads: int = 0) -> OracleConfig:
    c = OracleConfig()
    c.dt, c.kappa, c.dhat, c.ortho_kappa = cfg.dt, cfg.kappa, cfg.dhat, cfg.ortho_kappa
    c.ground_offset, c.mu, c.evh, c.eps_x = cfg.ground_offset, cfg.mu, cfg.evh, cfg.eps_x
    c.backoff, c.c1, c.tol, c.max_uk, c.dq_tol = cfg.backoff, cfg.c1, cfg.tol, cfg.max_uk, cfg.dq_tol
    c.gravity_y, c.ls_grad_tol = cfg.gravity_y, cfg.ls_grad_tol
    c.max_iter = min(int(cfg.max_iter), 2 ** 31 - 1)
    c.max_iter_frame = int(getattr(cfg, "max_iter_frame", 0))
    c.ground, c.pt, c.ee, c.psd = int(cfg.ground), int(cfg.pt), int(cfg.ee), int(cfg.psd)
    c.line_search, c.upper_bound = int(cfg.line_search), int(cfg.upper_bound)
    c.vg_fric, c.pt_fric, c.ee_fric = int(cfg.vg_friction), int(cfg.pt_friction), int(cfg.ee_friction)
    c.clip, c.n_threads = int(cfg.clip), int(n_threads)
    c.safe_factor, c.sh_min_xyz, c.sh_dx = cfg.safe_factor, cfg.sh_min_xyz, cfg.sh_dx
    c.iaabb, c.full_ccd, c.sh_bits, c.sh_fix_edge = int(cfg.iaabb), int(cfg.full_ccd), int(cfg.sh_bits), int(
        cfg.sh_fix_edge_trajectory)
    c.damp, c.damp_alpha, c.damp_beta = int(cfg.damping), cfg.damp_alpha, cfg.damp_beta
    return c


class OracleSim:
    """The restated reference step (ABD::implicit_euler) on the CPU."""

    def __init__(self, scene, cfg, n_threads: int = 0):
        L = lib()
        self._keep = [np.ascontiguousarray(x) for x in (
            scene.q0.astype(np.float64), scene.dqdt.astype(np.float64), scene.mass.astype(np.float64),
            scene.Ic.astype(np.float64), scene.vert_off.astype(np.int32), scene.rest.astype(np.float64),
            scene.edge_off.astype(np.int32), scene.edges.astype(np.int32), scene.face_off.astype(np.int32),
            scene.faces.astype(np.int32))]
        k = self._keep
        self.cfg = make_config(cfg, n_threads)
        self.nb = scene.n_bodies
        self.h = L.orc_create(self.nb, _d(k[0]), _d(k[1]), _d(k[2]), _d(k[3]), _i(k[4]), _d(k[5]), _i(k[6]),
                              _i(k[7]), _i(k[8]), _i(k[9]), C.byref(self.cfg))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def step(self, n_frames: int = 1) -> OracleStats:
        st = OracleStats()
        rc = lib().orc_step(self.h, n_frames, C.byref(st))
        st.status = rc
        return st

    def state(self):
        q0 = np.zeros((self.nb, 12))
        qd = np.zeros((self.nb, 12))
        lib().orc_get_state(self.h, _d(q0), _d(qd))
        return q0, qd

    def set_state(self, q0: np.ndarray, qdot: Optional[np.ndarray] = None):
        q0 = np.ascontiguousarray(q0, np.float64)
        qd = None if qdot is None else np.ascontiguousarray(qdot, np.float64)
        lib().orc_set_state(self.h, _d(q0), None if qd is None else _d(qd))

    @property
    def iter(self) -> int:
        return lib().orc_get_iter(self.h)

    @iter.setter
    def iter(self, v: int):
        lib().orc_set_iter(self.h, int(v))

    def cull(self, vtn: int, q: np.ndarray, dq: Optional[np.ndarray] = None):
        """Returns (pt (n,4), pt_type (n,), ee (m,4), ee_type (m,), vg (k,2)) for vtn 1/2
        or the TOI for vtn 3."""
        q = np.ascontiguousarray(q, np.float64)
        dqa = None if dq is None else np.ascontiguousarray(dq, np.float64)
        cnt = np.zeros(4, np.int32)
        t = lib().orc_cull(self.h, vtn, _d(q), None if dqa is None else _d(dqa), _i(cnt))
        if vtn == 3:
            return t
        return self.pairs(cnt)

    def pairs(self, cnt=None):
        if cnt is None:
            raise ValueError("counts required")
        npt, nee, nvg = int(cnt[0]), int(cnt[1]), int(cnt[2])
        pt = np.zeros((npt, 4), np.int32)
        ptt = np.zeros(npt, np.int32)
        ee = np.zeros((nee, 4), np.int32)
        eet = np.zeros(nee, np.int32)
        vg = np.zeros((nvg, 2), np.int32)
        lib().orc_get_pairs(self.h, _i(pt), _i(ptt), _i(ee), _i(eet), _i(vg))
        return pt, ptt, ee, eet, vg

    def newton_system(self, q: np.ndarray):
        """(grad (nb*12,), diag (nb,12,12), off_keys (n,2), off_vals (n,12,12))."""
        L = lib()
        q = np.ascontiguousarray(q, np.float64)
        grad = np.zeros(self.nb * 12)
        diag = np.zeros((self.nb, 12, 12))
        n = L.orc_newton_system(self.h, _d(q), _d(grad), _d(diag), None, None, 0)
        keys = np.zeros((max(n, 1), 2), np.int32)
        vals = np.zeros((max(n, 1), 12, 12))
        n = L.orc_newton_system(self.h, _d(q), _d(grad), _d(diag), _i(keys), _d(vals), n)
        return grad, diag, keys[:n], vals[:n]

    def newton_dq(self, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, np.float64)
        dq = np.zeros(self.nb * 12)
        rc = lib().orc_newton_dq(self.h, _d(q), _d(dq))
        if rc:
            raise RuntimeError("oracle solve failed: status %d" % rc)
        return dq

    def energy_terms(self, q: np.ndarray, dq: np.ndarray) -> dict:
        """Line-search energy at q + dq with the friction lagged at q (orc_energy_terms)."""
        q = np.ascontiguousarray(q, np.float64)
        dq = np.ascontiguousarray(dq, np.float64)
        cnt = np.zeros(6, np.int32)
        terms = np.zeros(5)
        lib().orc_energy_terms(self.h, _d(q), _d(dq), _d(terms), _i(cnt), None, None, None, None, None, None)
        arr = [np.zeros(max(int(n), 1)) for n in cnt]
        lib().orc_energy_terms(self.h, _d(q), _d(dq), _d(terms), _i(cnt), *[_d(a) for a in arr])
        names = ("e_pt", "e_ee", "e_vg", "f_pt", "f_ee", "f_vg")
        out = {k: a[:int(n)] for k, a, n in zip(names, arr, cnt)}
        out["terms"] = terms
        out["counts"] = cnt
        return out

    def energy(self, q: np.ndarray) -> float:
        q = np.ascontiguousarray(q, np.float64)
        return lib().orc_energy(self.h, _d(q))


# ----- per-primitive helpers -----

def pt_type(x: np.ndarray) -> int:
    return lib().orc_pt_type(_d(np.ascontiguousarray(x, np.float64)))


def pt_dist(x: np.ndarray, ty: int) -> float:
    return lib().orc_pt_dist(_d(np.ascontiguousarray(x, np.float64)), int(ty))


def ee_type(x: np.ndarray) -> int:
    return lib().orc_ee_type(_d(np.ascontiguousarray(x, np.float64)))


def ee_dist(x: np.ndarray, ty: int) -> float:
    return lib().orc_ee_dist(_d(np.ascontiguousarray(x, np.float64)), int(ty))


def ipc_hess_pt(x, ty, d, dhat, kappa, psd=True):
    H = np.zeros((12, 12))
    g = np.zeros(12)
    lib().orc_ipc_hess_pt(_d(np.ascontiguousarray(x, np.float64)), int(ty), float(d), dhat, kappa, int(psd),
                          _d(H), _d(g))
    return H, g


def ipc_hess_ee(x, ty, d, dhat, kappa, eps_x, psd=True):
    H = np.zeros((12, 12))
    g = np.zeros(12)
    m = lib().orc_ipc_hess_ee(_d(np.ascontiguousarray(x, np.float64)), int(ty), float(d), dhat, kappa, eps_x,
                              int(psd), _d(H), _d(g))
    return H, g, m


def barrier(d, dhat, kappa, which=0) -> float:
    return lib().orc_barrier(float(d), dhat, kappa, int(which))


def pt_collision_time(x24: np.ndarray) -> float:
    return lib().orc_pt_collision_time(_d(np.ascontiguousarray(x24, np.float64)))


def ee_collision_time(x24: np.ndarray) -> float:
    return lib().orc_ee_collision_time(_d(np.ascontiguousarray(x24, np.float64)))


def cubic_roots(c, x0=0.0, x1=1.0):
    r = np.zeros(3)
    n = lib().orc_cubic_roots(_d(np.ascontiguousarray(c, np.float64)), x0, x1, _d(r))
    return r[:n]


def det_polynomial(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    out = np.zeros(4)
    lib().orc_det_polynomial(_d(np.ascontiguousarray(a, np.float64)), _d(np.ascontiguousarray(b, np.float64)),
                             _d(out))
    return out


def friction(uk, lam, Tk, mu, epsv, max_uk=0.0):
    g = np.zeros(12)
    H = np.zeros((12, 12))
    lib().orc_friction(_d(np.ascontiguousarray(uk, np.float64)), float(lam), _d(np.ascontiguousarray(Tk, np.float64)),
                       mu, epsv, max_uk, _d(g), _d(H))
    return g, H


def f0(x, epsv) -> float:
    return lib().orc_f0(float(x), float(epsv))


def pt_frame(x, ty):
    T = np.zeros((2, 12))
    lib().orc_pt_frame(_d(np.ascontiguousarray(x, np.float64)), int(ty), _d(T))
    return T


def ee_frame(x, ty):
    T = np.zeros((2, 12))
    lib().orc_ee_frame(_d(np.ascontiguousarray(x, np.float64)), int(ty), _d(T))
    return T


def ref_cubic_roots(c, x0=0.0, x1=1.0):
    """The reference's own cubic root finder, compiled from its sources (only where the
    reference tree is present; returns None otherwise)."""
    if not os.path.exists(REF_CUBIC_PATH):
        return None
    L = C.CDLL(REF_CUBIC_PATH)
    L.ref_cubic_roots.argtypes = [_D, C.c_double, C.c_double, _D]
    r = np.zeros(3)
    n = L.ref_cubic_roots(_d(np.ascontiguousarray(c, np.float64)), x0, x1, _d(r))
    return r[:n]
