"""The step entry point: a drop-in for the reference's `ABD` driver.

``ABD(scene, config)`` mirrors ``ABD(cubes, globals)`` (model/abd.h:13-14) and
``ABD.implicit_euler(dt)`` mirrors ``ABD::implicit_euler(dt)`` (model/abd.cpp:30-140):
one frame of implicit Euler with IPC contact, friction, CCD and line search, computed
on the GPU through libabd_gb300.so. State layout per body: q = [p, a1, a2, a3].
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .scene import Config, Scene


def make_abd_config(cfg: Config) -> L.AbdConfig:
    c = L.AbdConfig()
    c.dt, c.kappa, c.dhat, c.ortho_kappa = cfg.dt, cfg.kappa, cfg.dhat, cfg.ortho_kappa
    c.ground_offset, c.mu, c.evh, c.eps_x = cfg.ground_offset, cfg.mu, cfg.evh, cfg.eps_x
    c.backoff, c.c1, c.tol, c.max_uk = cfg.backoff, cfg.c1, cfg.tol, cfg.max_uk
    c.gravity_y, c.ls_grad_tol, c.pcg_rel_tol = cfg.gravity_y, cfg.ls_grad_tol, cfg.pcg_rel_tol
    c.max_iter = min(int(cfg.max_iter), 2 ** 31 - 1)
    c.ground, c.pt, c.ee, c.psd = int(cfg.ground), int(cfg.pt), int(cfg.ee), int(cfg.psd)
    c.line_search, c.upper_bound = int(cfg.line_search), int(cfg.upper_bound)
    c.vg_fric, c.pt_fric, c.ee_fric = int(cfg.vg_friction), int(cfg.pt_friction), int(cfg.ee_friction)
    c.clip, c.pcg_max_iter = int(cfg.clip), int(cfg.pcg_max_iter)
    c.iaabb, c.full_ccd, c.safe_factor = int(cfg.iaabb), int(cfg.full_ccd), cfg.safe_factor
    c.sh_min_xyz, c.sh_dx, c.sh_xyz_bits = cfg.sh_min_xyz, cfg.sh_dx, int(cfg.sh_bits)
    c.sh_fix_edge_trajectory, c.dq_tol = int(cfg.sh_fix_edge_trajectory), cfg.dq_tol
    c.damping, c.damp_alpha, c.damp_beta = int(cfg.damping), cfg.damp_alpha, cfg.damp_beta
    c.pcg_refine, c.pcg_refine_tol = int(cfg.pcg_refine), cfg.pcg_refine_tol
    if cfg.solver not in ("sparse", "dense"):
        raise ValueError('solver must be "sparse" or "dense"')
    c.solver = 1 if cfg.solver == "dense" else 0
    c.max_iter_frame = int(cfg.max_iter_frame)
    c.autotune = int(cfg.autotune)
    c.tri_direct = int(cfg.tri_direct)
    return c


class ABD:
    """GPU affine-body contact step for one (possibly batched) scene."""

    def __init__(self, scene: Optional[Scene] = None, config: Optional[Config] = None, *, _handle=None, _nb=None):
        self._h = None
        if _handle is not None:
            self._h = _handle
            self.nb = _nb
            self.config = config
            return
        lib = L.lib()
        self.config = config or Config()
        self.nb = scene.n_bodies
        keep = [np.ascontiguousarray(x) for x in (
            scene.q0.astype(np.float64), scene.dqdt.astype(np.float64), scene.mass.astype(np.float64),
            scene.Ic.astype(np.float64), scene.vert_off.astype(np.int32), scene.rest.astype(np.float64),
            scene.edge_off.astype(np.int32), scene.edges.astype(np.int32), scene.face_off.astype(np.int32),
            scene.faces.astype(np.int32))]
        sid = None if scene.scene_id is None else np.ascontiguousarray(scene.scene_id, np.int32)
        d = L.AbdSceneDesc(self.nb, L.dptr(keep[0]), L.dptr(keep[1]), L.dptr(keep[2]), L.dptr(keep[3]),
                           L.iptr(keep[4]), L.dptr(keep[5]), L.iptr(keep[6]), L.iptr(keep[7]), L.iptr(keep[8]),
                           L.iptr(keep[9]), None if sid is None else L.iptr(sid))
        self._cfg = make_abd_config(self.config)
        h = C.c_void_p()
        L.check(lib.abd_create(C.byref(d), C.byref(self._cfg), C.byref(h)), None, "abd_create")
        self._h = h

    @classmethod
    def from_files(cls, config_json: str, scene_json: str) -> "ABD":
        """Reads a reference config.json and scene JSON (the C++ front end parses them)."""
        lib = L.lib()
        h = C.c_void_p()
        L.check(lib.abd_create_from_files(config_json.encode(), scene_json.encode(), C.byref(h)), None,
                "abd_create_from_files")
        nb = C.c_int()
        lib.abd_get_counts(h, C.byref(nb), None, None, None)
        return cls(_handle=h, _nb=nb.value)

    def close(self):
        if self._h is not None:
            L.lib().abd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- the reference's entry point -------------------------------------------------
    def implicit_euler(self, dt: Optional[float] = None) -> L.AbdFrameStats:
        return self.step(1, dt)

    def step(self, n_frames: int = 1, dt: Optional[float] = None, raise_on_error: bool = True) -> L.AbdFrameStats:
        st = L.AbdFrameStats()
        rc = L.lib().abd_step(self._h, float(dt or 0.0), int(n_frames), C.byref(st))
        if raise_on_error and rc not in (0, 6):
            L.check(rc, self._h, "abd_step")
        return st

    # --- state ------------------------------------------------------------------------
    def state(self):
        q0 = np.zeros((self.nb, 12))
        qd = np.zeros((self.nb, 12))
        L.check(L.lib().abd_get_state(self._h, L.dptr(q0), L.dptr(qd)), self._h, "abd_get_state")
        return q0, qd

    def set_state(self, q0: np.ndarray, qdot: Optional[np.ndarray] = None):
        q0 = np.ascontiguousarray(q0, np.float64)
        qd = None if qdot is None else np.ascontiguousarray(qdot, np.float64)
        L.check(L.lib().abd_set_state(self._h, L.dptr(q0), None if qd is None else L.dptr(qd)), self._h,
                "abd_set_state")

    # --- traces and the viewer loop (C++ front end) -------------------------------------
    def trace_save(self, folder: str, ts: int, init: bool = False):
        """Writes the state as frame file <folder>/<ts> (the reference's player_save)."""
        L.check(L.lib().abd_trace_save(self._h, folder.encode(), int(ts), int(init)), self._h, "abd_trace_save")

    def trace_load(self, folder: str, ts: int):
        """Loads frame file <folder>/<ts> into the state (the reference's player_load)."""
        L.check(L.lib().abd_trace_load(self._h, folder.encode(), int(ts)), self._h, "abd_trace_load")

    def set_trace(self, folder: Optional[str] = None, ts: int = 0, starting_ts: int = -1, ending_ts: int = 0):
        L.check(L.lib().abd_set_trace(self._h, folder.encode() if folder else None, int(ts), int(starting_ts),
                                      int(ending_ts), None, None), self._h, "abd_set_trace")

    @property
    def trace(self) -> dict:
        """Trace settings: folder, frame counter ts, starting_ts, ending_ts."""
        ts, st, en = C.c_int(), C.c_int(), C.c_int()
        buf = C.create_string_buffer(4096)
        L.check(L.lib().abd_get_trace(self._h, C.byref(ts), C.byref(st), C.byref(en), buf, 4096), self._h,
                "abd_get_trace")
        return {"folder": buf.value.decode(), "ts": ts.value, "starting_ts": st.value, "ending_ts": en.value}

    def run(self, record: bool = False) -> L.AbdFrameStats:
        """The reference's viewer loop without rendering: frames until ts reaches ending_ts,
        each new state saved as a frame file when recording."""
        st = L.AbdFrameStats()
        rc = L.lib().abd_run(self._h, int(record), C.byref(st))
        if rc not in (0, 6):
            L.check(rc, self._h, "abd_run")
        return st

    @property
    def iter(self) -> int:
        return L.lib().abd_get_iter(self._h)

    @iter.setter
    def iter(self, v: int):
        L.lib().abd_set_iter(self._h, int(v))

    def set_friction(self, mu: float):
        L.check(L.lib().abd_set_friction(self._h, float(mu)), self._h, "abd_set_friction")

    @property
    def friction(self) -> float:
        """The handle's current friction coefficient (config "mu" or the last set_friction)."""
        mu = C.c_double(0.0)
        L.check(L.lib().abd_get_friction(self._h, C.byref(mu)), self._h, "abd_get_friction")
        return mu.value

    def adjoint_frame(self, q_t: np.ndarray, v_t: np.ndarray, q_next: np.ndarray, gq_next: np.ndarray):
        """(dL/dq_t, dL/dv_t, dL/dmu) of one converged frame from dL/dq_{t+1}."""
        a = [np.ascontiguousarray(x, np.float64) for x in (q_t, v_t, q_next, gq_next)]
        gq, gv = np.zeros((self.nb, 12)), np.zeros((self.nb, 12))
        gm = C.c_double(0.0)
        rc = L.lib().abd_adjoint_frame(self._h, *[L.dptr(x) for x in a], L.dptr(gq), L.dptr(gv), C.byref(gm))
        if rc not in (0, 6):
            L.check(rc, self._h, "abd_adjoint_frame")
        return gq, gv, gm.value

    def autotune_info(self) -> dict:
        """Narrow-phase variants the autotuner chose (box-phase steps; 0 = not tuned yet)
        and the times it measured, for the pair cull and the CCD."""
        steps = np.zeros(2, np.int32)
        ms = np.zeros(6)
        L.check(L.lib().abd_autotune_info(self._h, L.iptr(steps), L.dptr(ms)), self._h, "abd_autotune_info")
        return {"pair_cull": {"step": int(steps[0]), "variant_ms": [round(float(x), 4) for x in ms[:3]]},
                "ccd": {"step": int(steps[1]), "variant_ms": [round(float(x), 4) for x in ms[3:]]}}

    def adjoint_stats(self):
        """(GMRES iterations, final relative residual) of the last adjoint_frame."""
        it, res = C.c_int(), C.c_double()
        L.check(L.lib().abd_adjoint_stats(self._h, C.byref(it), C.byref(res)), self._h, "abd_adjoint_stats")
        return it.value, res.value

    # --- per-kernel device timing -----------------------------------------------------
    @property
    def n_scenes(self) -> int:
        return L.lib().abd_get_scene_count(self._h)

    def scene_stats(self) -> dict:
        """Per-scene Newton iterations, line-search trials and PCG iterations of the last
        step call, and each scene's cumulative Newton counter (batched mode)."""
        ns = self.n_scenes
        out = {k: np.zeros(ns, dtype=np.int32) for k in ("newton_iters", "ls_trials", "pcg_iters", "iter")}
        L.check(L.lib().abd_get_scene_stats(self._h, L.iptr(out["newton_iters"]), L.iptr(out["ls_trials"]),
                                            L.iptr(out["pcg_iters"]), L.iptr(out["iter"])), self._h,
                "abd_get_scene_stats")
        return out

    def profile(self, enable: bool = True):
        L.check(L.lib().abd_profile(self._h, int(enable)), self._h, "abd_profile")

    def kernel_times(self):
        """{kernel class: dict(ms, launches, units, bytes)} since the last profile() call."""
        n = 64
        names = C.create_string_buffer(32 * n)
        ms, units, byts = np.zeros(n), np.zeros(n), np.zeros(n)
        cnt = np.zeros(n, np.int64)
        k = L.lib().abd_kernel_work(self._h, n, names, L.dptr(ms), cnt.ctypes.data_as(C.POINTER(C.c_longlong)),
                                    L.dptr(units), L.dptr(byts))
        out = {}
        for i in range(k):
            nm = names.raw[32 * i: 32 * i + 32].split(b"\0")[0].decode()
            out[nm] = {"ms": float(ms[i]), "launches": int(cnt[i]), "units": float(units[i]),
                       "bytes": float(byts[i])}
        return out

    # --- stage access (parity tests, profiling) ------------------------------------
    def cull(self, vtn: int, q: np.ndarray, dq: Optional[np.ndarray] = None):
        q = np.ascontiguousarray(q, np.float64)
        dqa = None if dq is None else np.ascontiguousarray(dq, np.float64)
        cnt = np.zeros(4, np.int32)
        toi = C.c_double(1.0)
        L.check(L.lib().abd_cull(self._h, int(vtn), L.dptr(q), None if dqa is None else L.dptr(dqa), L.iptr(cnt),
                                 C.byref(toi)), self._h, "abd_cull")
        if vtn == 3:
            return toi.value
        npt, nee, nvg = int(cnt[0]), int(cnt[1]), int(cnt[2])
        pt = np.zeros((npt, 4), np.int32)
        ptt = np.zeros(npt, np.int32)
        ee = np.zeros((nee, 4), np.int32)
        eet = np.zeros(nee, np.int32)
        vg = np.zeros((nvg, 2), np.int32)
        L.check(L.lib().abd_get_pairs(self._h, L.iptr(pt), L.iptr(ptt), L.iptr(ee), L.iptr(eet), L.iptr(vg)),
                self._h, "abd_get_pairs")
        return pt, ptt, ee, eet, vg

    def newton_system(self, q: np.ndarray):
        q = np.ascontiguousarray(q, np.float64)
        grad = np.zeros(self.nb * 12)
        diag = np.zeros((self.nb, 12, 12))
        n = C.c_int()
        lib = L.lib()
        L.check(lib.abd_newton_system(self._h, L.dptr(q), L.dptr(grad), L.dptr(diag), C.byref(n), None, None, 0),
                self._h, "abd_newton_system")
        k = max(n.value, 1)
        keys = np.zeros((k, 2), np.int32)
        vals = np.zeros((k, 12, 12))
        L.check(lib.abd_newton_system(self._h, L.dptr(q), L.dptr(grad), L.dptr(diag), C.byref(n), L.iptr(keys),
                                      L.dptr(vals), k), self._h, "abd_newton_system")
        return grad, diag, keys[:n.value], vals[:n.value]

    def energy(self, q: np.ndarray, dq: np.ndarray) -> dict:
        """Line-search energy at q + dq with the friction lagged at q (the first trial of the
        reference's line search at alpha = 1, abd_energy): per-scene `terms` (inertia +
        orthogonality, PT, EE and ground barrier, friction, the line-search total), pair
        `counts`, per-pair barrier energies (e_pt, e_ee, e_vg) of the set at q + dq and
        friction energies (f_pt, f_ee, f_vg) of the lagged set."""
        lib = L.lib()
        q = np.ascontiguousarray(q, np.float64)
        dq = np.ascontiguousarray(dq, np.float64)
        cnt = np.zeros(6, np.int32)
        L.check(lib.abd_energy(self._h, L.dptr(q), L.dptr(dq), None, L.iptr(cnt), None, None, None, None, None,
                               None), self._h, "abd_energy")
        terms = np.zeros((self.n_scenes, 6))
        arr = [np.zeros(max(int(n), 1)) for n in cnt]
        L.check(lib.abd_energy(self._h, L.dptr(q), L.dptr(dq), L.dptr(terms), L.iptr(cnt), *[L.dptr(a) for a in arr]),
                self._h, "abd_energy")
        out = {k: a[:int(n)] for k, a, n in zip(("e_pt", "e_ee", "e_vg", "f_pt", "f_ee", "f_vg"), arr, cnt)}
        out["terms"] = terms
        out["counts"] = cnt
        return out

    def newton_dq(self, q: np.ndarray):
        q = np.ascontiguousarray(q, np.float64)
        dq = np.zeros(self.nb * 12)
        its = C.c_int()
        rc = L.lib().abd_newton_dq(self._h, L.dptr(q), L.dptr(dq), C.byref(its))
        if rc not in (0, 6):
            L.check(rc, self._h, "abd_newton_dq")
        return dq, its.value


def measure_fp64_gflops() -> float:
    return float(L.lib().abd_measure_fp64_gflops())
