"""CPU oracle pinned against the reference's own golden vectors and known-answer tests.

- cubic roots: bit-exact against the reference's own cy::CubicRoots (fixture made by
  tests/golden/make_golden.py from the reference-compiled checker; plus a live check
  where oracle/_ref is built);
- det_polynomial: Sample-Test1/test.cpp:33-60 (1e-6);
- constructed point-triangle TOIs: Sample-Test1/test.cpp:9-31 (1e-6);
- barrier and friction derivatives against central finite differences:
  iAABB/test.cpp:460-554 (1e-3 there; tighter here);
- iAABB pair sets equal the brute-force all-pairs sets: iAABB/test.cpp:341-435;
- iAABB trajectory TOI equals the brute-force minimum: iAABB/test.cpp:437-458.
"""
import os

import numpy as np
import pytest

from adb_gb300 import scene as S

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_cubic_roots_match_reference_golden(oracle_lib):
    O = oracle_lib
    z = np.load(os.path.join(GOLD, "cubic_roots.npz"))
    bad = 0
    for c, n, r in zip(z["coefs"], z["nroots"], z["roots"]):
        got = O.cubic_roots(c)
        if len(got) != n or not np.array_equal(got, r[:n]):
            bad += 1
    assert bad == 0


def test_cubic_roots_live_reference(oracle_lib):
    O = oracle_lib
    if O.ref_cubic_roots(np.array([1.0, -3.0, 0.5, 1.0])) is None:
        pytest.skip("reference-compiled checker not built here")
    rng = np.random.default_rng(99)
    for _ in range(5000):
        c = rng.normal(size=4) * rng.choice([1e-3, 1.0, 1e3], size=4)
        a, b = O.cubic_roots(c), O.ref_cubic_roots(c)
        assert len(a) == len(b) and np.array_equal(a, b), c


def test_det_polynomial_golden(oracle_lib):
    O = oracle_lib
    z = np.load(os.path.join(GOLD, "det_poly.npz"))
    for a, b, w, d0, d1, dw in zip(z["a"], z["b"], z["w"], z["det0"], z["det1"], z["detw"]):
        p = O.det_polynomial(a, b)
        ev = lambda t: p[0] + t * (p[1] + t * (p[2] + t * p[3]))
        assert abs(ev(0.0) - d0) < 1e-6 and abs(ev(1.0) - d1) < 1e-6 and abs(ev(w) - dw) < 1e-6


def test_pt_toi_known_answer(oracle_lib):
    O = oracle_lib
    z = np.load(os.path.join(GOLD, "pt_toi_known.npz"))
    for p0, tri, p1, toi in zip(z["p0"], z["tri"], z["p1"], z["toi"]):
        x = np.concatenate([p0, tri.ravel(), p1, tri.ravel()])
        assert abs(O.pt_collision_time(x) - toi) < 1e-6


def _fd_grad_hess(E, x, h=1e-7):
    n = len(x)
    g = np.array([(E(x + h * e) - E(x - h * e)) / (2 * h) for e in np.eye(n)])
    H = np.zeros((n, n))
    for i, ei in enumerate(np.eye(n)):
        for j, ej in enumerate(np.eye(n)):
            H[i, j] = (E(x + h * ei + h * ej) - E(x + h * ei - h * ej) - E(x - h * ei + h * ej)
                       + E(x - h * ei - h * ej)) / (4 * h * h)
    return g, H


@pytest.mark.parametrize("kind", ["pt", "ee"])
def test_barrier_derivatives_fd(oracle_lib, kind):
    O = oracle_lib
    rng = np.random.default_rng(5 if kind == "pt" else 6)
    for _ in range(30):
        x = rng.normal(size=12) * 0.05
        if kind == "pt":
            ty = O.pt_type(x); d = O.pt_dist(x, ty)
            dist = lambda y: O.pt_dist(y, O.pt_type(y))
            H, g = O.ipc_hess_pt(x, ty, d, 2 * d, 1.0, psd=False)
            E = lambda y: O.barrier(dist(y), 2 * d, 1.0)
        else:
            ty = O.ee_type(x); d = O.ee_dist(x, ty)
            H, g, _ = O.ipc_hess_ee(x, ty, d, 2 * d, 1.0, 1e-3, psd=False)

            def E(y):
                u, v = y[3:6] - y[0:3], y[9:12] - y[6:9]
                eps = 1e-3 * (u @ u) * (v @ v)
                xx = np.cross(u, v) @ np.cross(u, v)
                m = (-xx / eps + 2) * xx / eps if xx < eps else 1.0
                return O.barrier(O.ee_dist(y, O.ee_type(y)), 2 * d, 1.0) * m
        gf, Hf = _fd_grad_hess(E, x)
        assert np.abs(gf - g).max() <= 1e-4 * np.abs(g).max()
        assert np.abs(Hf - H).max() <= 1e-3 * np.abs(H).max()


def test_psd_projection_properties(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(8)
    for _ in range(20):
        x = rng.normal(size=12) * 0.05
        ty = O.pt_type(x); d = O.pt_dist(x, ty)
        Hn, _ = O.ipc_hess_pt(x, ty, d, 2 * d, 1.0, psd=False)
        Hp, _ = O.ipc_hess_pt(x, ty, d, 2 * d, 1.0, psd=True)
        w, V = np.linalg.eigh(Hn)
        ref = (V * np.maximum(w, 0)) @ V.T
        assert np.abs(Hp - ref).max() <= 1e-9 * np.abs(ref).max()
        assert np.linalg.eigvalsh(Hp).min() >= -1e-9 * np.abs(Hp).max()


def test_friction_derivatives_fd(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(12)
    epsv = 1e-5
    for trial in range(20):
        x = rng.normal(size=12) * 0.05
        ty = O.pt_type(x)
        T = O.pt_frame(x, ty)          # 2 x 12
        lam, mu = 0.7, 0.3
        du = rng.normal(size=12) * (epsv * (0.3 if trial % 2 else 30.0))
        uk = T @ du
        g, H = O.friction(uk, lam, T.T.copy(), mu, epsv)
        E = lambda y: mu * lam * O.f0(np.linalg.norm(T @ y), epsv)
        gf = np.array([(E(du + 1e-9 * e) - E(du - 1e-9 * e)) / 2e-9 for e in np.eye(12)])
        assert np.abs(gf - g).max() <= 1e-4 * max(np.abs(g).max(), 1e-12)


def _rand_cubes(n, seed, extent):
    rng = np.random.default_rng(seed)
    sb = S.SceneBuilder()
    cube = S.cube_mesh()
    for _ in range(n):
        a, b, c = rng.random(3) * 2 * np.pi
        sb.add(cube, rng.uniform(-extent, extent, 3), S.rotation_zyx(a, b, c))
    return sb.build()


def _brute_pairs(O, sc, q, dhat):
    """All-pairs sets: vertex box (+-sqrt dhat) vs face box, then d < dhat; edge pairs
    with I < J likewise (the brute-force reference of iAABB/test.cpp:341-435)."""
    ds = np.sqrt(dhat)
    X = []
    for b in range(sc.n_bodies):
        r = sc.rest[sc.vert_off[b]:sc.vert_off[b + 1]]
        A = q[b, 3:].reshape(3, 3).T
        X.append(r @ A.T + q[b, :3])
    pt, ee = [], []
    nb = sc.n_bodies
    for I in range(nb):
        for J in range(nb):
            if I == J:
                continue
            F = sc.faces[sc.face_off[J]:sc.face_off[J + 1]]
            for v, p in enumerate(X[I]):
                for f, tri in enumerate(F):
                    T = X[J][tri]
                    if np.any(p + ds < T.min(0)) or np.any(p - ds > T.max(0)):
                        continue
                    x = np.concatenate([p, T.ravel()])
                    ty = O.pt_type(x)
                    if O.pt_dist(x, ty) < dhat:
                        pt.append((I, v, J, f))
            if J > I:
                Ei = sc.edges[sc.edge_off[I]:sc.edge_off[I + 1]]
                Ej = sc.edges[sc.edge_off[J]:sc.edge_off[J + 1]]
                for a, ea in enumerate(Ei):
                    A = X[I][ea]
                    for bidx, eb in enumerate(Ej):
                        B = X[J][eb]
                        if np.any(A.max(0) + ds < B.min(0)) or np.any(A.min(0) - ds > B.max(0)):
                            continue
                        x = np.concatenate([A.ravel(), B.ravel()])
                        if O.ee_dist(x, O.ee_type(x)) < dhat:
                            ee.append((I, a, J, bidx))
    return sorted(pt), sorted(ee)


def test_iaabb_pair_sets_equal_brute_force(oracle_lib):
    O = oracle_lib
    sc = _rand_cubes(24, 3, 1.6)
    cfg = S.Config(dhat=1e-2)
    sim = O.OracleSim(sc, cfg)
    pt, _, ee, _, _ = sim.cull(1, sc.q0)
    bpt, bee = _brute_pairs(O, sc, sc.q0, cfg.dhat)
    assert len(bpt) + len(bee) > 0
    assert sorted(map(tuple, pt.tolist())) == bpt
    assert sorted(map(tuple, ee.tolist())) == bee


def test_iaabb_toi_equals_brute_force(oracle_lib):
    O = oracle_lib
    sc = _rand_cubes(16, 4, 1.5)
    cfg = S.Config(dhat=1e-4)
    sim = O.OracleSim(sc, cfg)
    rng = np.random.default_rng(4)
    dq = rng.normal(size=(sc.n_bodies, 12)) * 0.05
    toi = sim.cull(3, sc.q0, dq)
    # brute force over every vertex-face and edge-edge pair with overlapping trajectory boxes
    nb = sc.n_bodies
    X0, X1 = [], []
    for b in range(nb):
        r = sc.rest[sc.vert_off[b]:sc.vert_off[b + 1]]
        for store, qq in ((X0, sc.q0[b]), (X1, sc.q0[b] + dq[b])):
            A = qq[3:].reshape(3, 3).T
            store.append(r @ A.T + qq[:3])
    best = 1.0
    for I in range(nb):
        for J in range(nb):
            if I == J:
                continue
            F = sc.faces[sc.face_off[J]:sc.face_off[J + 1]]
            for v in range(len(X0[I])):
                for tri in F:
                    x = np.concatenate([X0[I][v], X0[J][tri].ravel(), X1[I][v], X1[J][tri].ravel()])
                    best = min(best, O.pt_collision_time(x))
            if J > I:
                for ea in sc.edges[sc.edge_off[I]:sc.edge_off[I + 1]]:
                    for eb in sc.edges[sc.edge_off[J]:sc.edge_off[J + 1]]:
                        x = np.concatenate([X0[I][ea].ravel(), X0[J][eb].ravel(), X1[I][ea].ravel(),
                                            X1[J][eb].ravel()])
                        best = min(best, O.ee_collision_time(x))
    gtoi = 1.0
    ground = min([1.0] + [(a + 0.5) / ((a + 0.5) - (b + 0.5)) for Xa, Xb in zip(X0, X1)
                          for a, b in zip(Xa[:, 1], Xb[:, 1]) if b + 0.5 < 0])
    assert toi == min(best, ground, gtoi)


def test_oracle_cube_stack_runs(oracle_lib):
    O = oracle_lib
    sc = S.cube_stack(10, seed=0)
    cfg = S.workload_config("cubes")
    sim = O.OracleSim(sc, cfg)
    st = sim.step(40)
    assert st.status == 0
    q0, _ = sim.state()
    # every body stays above the ground plane and the stack keeps its order
    assert np.all(q0[:, 1] > -0.5)
    assert np.all(np.diff(q0[:, 1]) > 0.9)


def test_energy_terms_restate_the_line_search_energy(oracle_lib):
    """orc_energy_terms at dq = 0: inertia + barrier terms add up to the line search's
    E_barrier_plus_inert at q (orc_energy), and the per-pair values add up to the terms."""
    O = oracle_lib
    sc, cfg = S.cube_stack(4, gap=0.0005, seed=3), S.workload_config("cubes")
    o = O.OracleSim(sc, cfg)
    q = sc.q0.copy()
    out = o.energy_terms(q, np.zeros_like(q))
    t = out["terms"]
    assert out["counts"][2] > 0 or out["counts"][0] > 0
    assert abs(t[:4].sum() - o.energy(q)) <= 1e-12 * abs(t[:4].sum())
    f = out["f_pt"].sum() + out["f_ee"].sum() + out["f_vg"].sum()
    assert abs(f - t[4]) <= 1e-12 * max(abs(t[4]), 1e-300)
    assert abs(out["e_pt"].sum() - t[1]) <= 1e-12 * max(abs(t[1]), 1e-300)
    assert abs(out["e_vg"].sum() - t[3]) <= 1e-12 * max(abs(t[3]), 1e-300)
