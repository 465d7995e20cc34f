"""GPU counterpart of the reference's python module ``abdtk`` (python/bindings.cpp:42-83).

Same functions and enums: ``ipc_hess_pt_12x12``, ``ipc_hess_ee_12x12``,
``pt_collision_time``, ``ee_collision_time``, ``PointTriangleDistanceType`` and
``EdgeEdgeDistanceType``, plus batched forms over numpy arrays. The barrier parameters
default to the values the reference module runs with (d_hat 1e-4 and kappa 1e-3 from
model/barrier.cpp:7, eps_x 1e-3 and psd on from model/settings.h:6-59).
"""
from __future__ import annotations

import enum

import numpy as np

from . import _lib as L


class PointTriangleDistanceType(enum.IntEnum):
    P_T0 = 0
    P_T1 = 1
    P_T2 = 2
    P_E0 = 3
    P_E1 = 4
    P_E2 = 5
    P_T = 6
    AUTO = 7


class EdgeEdgeDistanceType(enum.IntEnum):
    EA0_EB0 = 0
    EA0_EB1 = 1
    EA1_EB0 = 2
    EA1_EB1 = 3
    EA_EB0 = 4
    EA_EB1 = 5
    EA0_EB = 6
    EA1_EB = 7
    EA_EB = 8
    AUTO = 9


PARAMS = {"dhat": 1e-4, "kappa": 1e-3, "eps_x": 1e-3, "psd": True}


def set_params(dhat=None, kappa=None, eps_x=None, psd=None):
    for k, v in (("dhat", dhat), ("kappa", kappa), ("eps_x", eps_x), ("psd", psd)):
        if v is not None:
            PARAMS[k] = v


def _types(t, n, auto):
    t = np.broadcast_to(np.asarray(t, np.int32), (n,)).copy()
    t[t == auto] = -1
    return np.ascontiguousarray(t)


def ipc_hess_pt_batch(x, pt_type=PointTriangleDistanceType.AUTO, dist=None):
    """x: (n, 4, 3) point, t0, t1, t2 -> (H (n,12,12), g (n,12))."""
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 12))
    n = x.shape[0]
    t = _types(pt_type, n, int(PointTriangleDistanceType.AUTO))
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(0.0 if dist is None else dist, np.float64), (n,)))
    if dist is None:
        t[:] = -1
    H = np.zeros((n, 12, 12))
    g = np.zeros((n, 12))
    L.check(L.lib().abd_ipc_hess_pt_batch(n, L.dptr(x), L.iptr(t), L.dptr(d), PARAMS["dhat"], PARAMS["kappa"],
                                          int(PARAMS["psd"]), L.dptr(H), L.dptr(g)), None, "abd_ipc_hess_pt_batch")
    return H, g


def ipc_hess_ee_batch(x, ee_type=EdgeEdgeDistanceType.AUTO, dist=None):
    """x: (n, 4, 3) ea0, ea1, eb0, eb1 -> (H, g, mollifier)."""
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 12))
    n = x.shape[0]
    t = _types(ee_type, n, int(EdgeEdgeDistanceType.AUTO))
    d = np.ascontiguousarray(np.broadcast_to(np.asarray(0.0 if dist is None else dist, np.float64), (n,)))
    if dist is None:
        t[:] = -1
    H = np.zeros((n, 12, 12))
    g = np.zeros((n, 12))
    m = np.zeros(n)
    L.check(L.lib().abd_ipc_hess_ee_batch(n, L.dptr(x), L.iptr(t), L.dptr(d), PARAMS["dhat"], PARAMS["kappa"],
                                          PARAMS["eps_x"], int(PARAMS["psd"]), L.dptr(H), L.dptr(g), L.dptr(m)),
            None, "abd_ipc_hess_ee_batch")
    return H, g, m


def ipc_hess_pt_12x12(pt, ij, pt_type, dist):
    """(core_ipc.cpp:21-46) pt: 4 points; ij: body/primitive indices (unused)."""
    H, g = ipc_hess_pt_batch(np.asarray(pt, np.float64)[None], int(pt_type), np.array([dist]))
    return H[0], g[0]


def ipc_hess_ee_12x12(ee, ij, ee_type, dist):
    """(core_ipc.cpp:47-83) ee: 4 points; returns (H, g, mollifier)."""
    H, g, m = ipc_hess_ee_batch(np.asarray(ee, np.float64)[None], int(ee_type), np.array([dist]))
    return H[0], g[0], float(m[0])


def pt_collision_time_batch(x):
    """x: (n, 8, 3): p, t0, t1, t2 at time 0, then at time 1."""
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 24))
    out = np.zeros(x.shape[0])
    L.check(L.lib().abd_pt_collision_time_batch(x.shape[0], L.dptr(x), L.dptr(out)), None, "pt_collision_time")
    return out


def ee_collision_time_batch(x):
    """x: (n, 8, 3): ei0, ei1, ej0, ej1 at time 0, then at time 1."""
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 24))
    out = np.zeros(x.shape[0])
    L.check(L.lib().abd_ee_collision_time_batch(x.shape[0], L.dptr(x), L.dptr(out)), None, "ee_collision_time")
    return out


def pt_collision_time(p0_t0, t0_t0, t1_t0, t2_t0, p0_t1, t0_t1, t1_t1, t2_t1) -> float:
    return float(pt_collision_time_batch(np.array([p0_t0, t0_t0, t1_t0, t2_t0, p0_t1, t0_t1, t1_t1, t2_t1]))[0])


def ee_collision_time(ei0_t0, ei1_t0, ej0_t0, ej1_t0, ei0_t1, ei1_t1, ej0_t1, ej1_t1) -> float:
    return float(ee_collision_time_batch(np.array([ei0_t0, ei1_t0, ej0_t0, ej1_t0, ei0_t1, ei1_t1, ej0_t1, ej1_t1]))[0])


def pt_distance_batch(x):
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 12))
    t = np.zeros(x.shape[0], np.int32)
    d = np.zeros(x.shape[0])
    L.check(L.lib().abd_pt_distance_batch(x.shape[0], L.dptr(x), L.iptr(t), L.dptr(d)), None, "pt_distance")
    return t, d


def ee_distance_batch(x):
    x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 12))
    t = np.zeros(x.shape[0], np.int32)
    d = np.zeros(x.shape[0])
    L.check(L.lib().abd_ee_distance_batch(x.shape[0], L.dptr(x), L.iptr(t), L.dptr(d)), None, "ee_distance")
    return t, d
