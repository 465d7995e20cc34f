"""GPU path (libabd_gb300.so, called through the C ABI) against the CPU oracle.

Bar: pair sets and distance types bit-exact; TOIs bit-exact; per-pair gradient and
Hessian within 1e-9 relative; Newton systems and Newton steps within 1e-9 relative;
per-frame states from the same start state within 1e-9 relative (relative to the largest
state entry). Per-pair and per-scene energies are checked in test_gpu_energy.py.

A frame of the reference step can amplify rounding-level differences: on a frame with
dozens of Newton iterations and line-search steps of a few 1e-3, the oracle itself moves
by ~1e-9 when its start state is perturbed by 1e-16 relative. No implementation with a
different rounding (another summation order, FMA, a different solver) can agree with it
below that level. So a frame that misses 1e-9 passes only if the oracle's own measured
sensitivity on that frame is above 1e-10 and the GPU error is within SENS_FACTOR of it;
every other frame must meet 1e-9."""
import os

import numpy as np
import pytest

from adb_gb300 import abdtk
from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu

REL = 1e-9
SENS_FACTOR = 10.0   # GPU error allowed on an ill-conditioned frame, in units of the oracle's own sensitivity


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def O(gpu_lib, oracle_lib):
    return oracle_lib


def ABD(scene, cfg):
    from adb_gb300.abd import ABD as _ABD
    return _ABD(scene, cfg)


def rand_cubes(n, seed, extent):
    rng = np.random.default_rng(seed)
    sb = S.SceneBuilder()
    for _ in range(n):
        a, b, c = rng.random(3) * 2 * np.pi
        sb.add(S.cube_mesh(), rng.uniform(-extent, extent, 3), S.rotation_zyx(a, b, c))
    return sb.build()


def assert_sets_equal(g, o):
    for name, a, b in zip(("pt", "pt_type", "ee", "ee_type", "vg"), g, o):
        assert a.shape == b.shape and np.array_equal(a, b), name


def test_cull_bit_exact_random_cubes(O):
    sc = rand_cubes(30, 1, 1.8)
    cfg = S.Config(dhat=1e-2)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    g, o = gpu.cull(1, sc.q0), orc.cull(1, sc.q0)
    assert len(o[0]) + len(o[2]) > 50
    assert_sets_equal(g, o)
    rng = np.random.default_rng(2)
    dq = rng.normal(size=sc.q0.shape) * 0.02
    assert_sets_equal(gpu.cull(2, sc.q0, dq), orc.cull(2, sc.q0, dq))
    assert gpu.cull(3, sc.q0, dq) == orc.cull(3, sc.q0, dq)


def test_cull_bit_exact_along_cube_stack_run(O):
    sc = S.cube_stack(10, seed=0)
    cfg = S.workload_config("cubes")
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    rng = np.random.default_rng(3)
    n_checked = 0
    for f in range(48):
        orc.step(1)
        if f % 6 == 5:
            q0, _ = orc.state()
            g, o = gpu.cull(1, q0), orc.cull(1, q0)
            assert_sets_equal(g, o)
            n_checked += len(o[2]) + len(o[4])
            dq = rng.normal(size=q0.shape) * 1e-2
            assert gpu.cull(3, q0, dq) == orc.cull(3, q0, dq)
    assert n_checked > 0


def test_cull_bit_exact_sphere_pile(O):
    sc = S.sphere_pile(4, 4, 2, subdiv=2, seed=1)
    cfg = S.workload_config("pile")
    orc = O.OracleSim(sc, cfg)
    orc.step(25)
    q0, _ = orc.state()
    gpu = ABD(sc, cfg)
    g, o = gpu.cull(1, q0), orc.cull(1, q0)
    assert len(o[0]) > 0 and len(o[2]) > 0
    assert_sets_equal(g, o)


def test_cull_bit_exact_dense_overlap(O):
    # two near-coincident spheres: a single overlap with more pairs than the narrow phase
    # keeps in shared memory (2048), so the recomputing write pass produces it
    sc = S.sphere_pile(2, 1, 1, subdiv=2, jitter=0.0, vel_sigma=0.0, seed=3)
    q = sc.q0.copy()
    q[1, :3] = q[0, :3] + np.array([0.004, 0.003, -0.002])
    cfg = S.workload_config("pile")
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    g, o = gpu.cull(1, q), orc.cull(1, q)
    assert len(o[0]) + len(o[2]) > 2048
    assert_sets_equal(g, o)


def test_distance_types_and_tois_bit_exact(O):
    rng = np.random.default_rng(4)
    X = rng.normal(size=(3000, 4, 3)) * 0.02
    t, d = abdtk.pt_distance_batch(X)
    assert np.array_equal(t, [O.pt_type(x.ravel()) for x in X])
    assert np.array_equal(d, [O.pt_dist(x.ravel(), k) for x, k in zip(X, t)])
    t, d = abdtk.ee_distance_batch(X)
    assert np.array_equal(t, [O.ee_type(x.ravel()) for x in X])
    assert np.array_equal(d, [O.ee_dist(x.ravel(), k) for x, k in zip(X, t)])
    Y = rng.random((3000, 8, 3))
    assert np.array_equal(abdtk.pt_collision_time_batch(Y), [O.pt_collision_time(y.ravel()) for y in Y])
    assert np.array_equal(abdtk.ee_collision_time_batch(Y), [O.ee_collision_time(y.ravel()) for y in Y])


def test_known_answer_toi_on_gpu():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "pt_toi_known.npz"))
    x = np.concatenate([z["p0"][:, None], z["tri"], z["p1"][:, None], z["tri"]], axis=1)
    toi = abdtk.pt_collision_time_batch(x)
    assert np.abs(toi - z["toi"]).max() < 1e-6


# kappa 1e-120 and 1e40 put the reduced matrices outside FP32 range, so the projection
# starts its Jacobi from the identity instead of from FP32 eigenvectors
@pytest.mark.parametrize("kappa", [0.5, 1e-120, 1e40])
@pytest.mark.parametrize("kind", ["pt", "ee"])
def test_pair_hessians_match_oracle(O, kind, kappa):
    rng = np.random.default_rng(5)
    X = rng.normal(size=(400, 4, 3)) * 0.02
    if kind == "pt":
        t, d = abdtk.pt_distance_batch(X)
    else:
        t, d = abdtk.ee_distance_batch(X)
        X[:50, 3] = X[:50, 2] + (X[:50, 1] - X[:50, 0]) * 1.3 + 1e-4 * rng.normal(size=(50, 3))
        t, d = abdtk.ee_distance_batch(X)
    dhat = float(d.max()) * 2
    abdtk.set_params(dhat=dhat, kappa=kappa, eps_x=1e-3, psd=True)
    try:
        if kind == "pt":
            H, g = abdtk.ipc_hess_pt_batch(X, t, d)
        else:
            H, g, m = abdtk.ipc_hess_ee_batch(X, t, d)
    finally:
        abdtk.set_params(dhat=1e-4, kappa=1e-3)
    worst = 0.0
    for i in range(len(X)):
        if kind == "pt":
            Ho, go = O.ipc_hess_pt(X[i].ravel(), t[i], d[i], dhat, kappa)
        else:
            Ho, go, mo = O.ipc_hess_ee(X[i].ravel(), t[i], d[i], dhat, kappa, 1e-3)
            assert abs(m[i] - mo) <= 1e-12
        assert rel(H[i], Ho) <= REL and rel(g[i], go) <= REL
        worst = max(worst, rel(H[i], Ho))
    print("%s kappa %g: worst Hessian relative error %.2e" % (kind, kappa, worst))


def test_newton_system_matches_oracle(O):
    sc = S.cube_stack(6, seed=2)
    cfg = S.workload_config("cubes")
    orc = O.OracleSim(sc, cfg)
    orc.step(30)
    q0, qd = orc.state()
    gpu = ABD(sc, cfg)
    gpu.set_state(q0, qd)
    rng = np.random.default_rng(6)
    q = q0.copy()
    q[:, :3] += rng.normal(size=(q0.shape[0], 3)) * 1e-4   # translations only: keeps the system SPD
    gg, gd, gk, gv = gpu.newton_system(q)
    og, od, ok, ov = orc_system(O, sc, cfg, q0, qd, q)
    assert np.array_equal(gk, ok)
    assert rel(gg, og) <= REL and rel(gd, od) <= REL
    if len(ov):
        assert rel(gv, ov) <= REL
    gdq, its = gpu.newton_dq(q)
    assert rel(gdq, orc_dq(O, sc, cfg, q0, qd, q)) <= REL


def test_newton_steps_match_direct_solve_on_pile_frames(O):
    """The block-Jacobi PCG step against the oracle's direct block-sparse Cholesky (the
    reference factorizes, abd.cpp:229-303) on ten contact-rich frames of a small pile."""
    sc = S.sphere_pile(3, 3, 2, subdiv=1, seed=2)
    cfg = S.workload_config("pile")
    orc = O.OracleSim(sc, cfg)
    orc.step(20)
    gpu = ABD(sc, cfg)
    for _ in range(10):
        orc.step(1)
        q0, qd = orc.state()
        gpu.set_state(q0, qd)
        gdq, its = gpu.newton_dq(q0)
        assert its > 0
        assert rel(gdq, orc_dq(O, sc, cfg, q0, qd, q0)) <= REL


def orc_system(O, sc, cfg, q0, qd, q):
    o = O.OracleSim(sc, cfg)
    o.set_state(q0, qd)
    return o.newton_system(q)


def orc_dq(O, sc, cfg, q0, qd, q):
    o = O.OracleSim(sc, cfg)
    o.set_state(q0, qd)
    return o.newton_dq(q)


def run_pair(O, sc, cfg, frames, start=None, gpu=None):
    """Steps both implementations frame by frame; before every frame the GPU state is
    reset to the oracle's, so each comparison is one frame from the same start state.
    Returns the per-frame relative state differences and each frame's start (q0, qdot,
    Newton counter). Newton and line-search counts (the discrete decisions of the step)
    must match on every frame."""
    gpu = gpu or ABD(sc, cfg)
    orc = O.OracleSim(sc, cfg, n_threads=os.cpu_count() or 1)
    if start is not None:
        orc.set_state(start[0], start[1])
        orc.iter = start[2]
    errs, starts = [], []
    for _ in range(frames):
        q0, qd = orc.state()
        starts.append((q0, qd, orc.iter))
        gpu.set_state(q0, qd)
        gpu.iter = orc.iter
        sg = gpu.implicit_euler()
        so = orc.step(1)
        assert sg.status in (0, 6) and so.status == 0
        assert (sg.newton_iters, sg.ls_trials) == (so.newton_iters, so.ls_trials)
        qg, vg = gpu.state()
        qo, vo = orc.state()
        errs.append(rel(qg, qo))
        assert gpu.iter == orc.iter
    return np.array(errs), starts


def oracle_sensitivity(O, sc, cfg, start, n=4, eps=1e-16, seed=0):
    """Largest relative change of the oracle's frame when its start positions are
    perturbed by eps relative (n seeded perturbations): the reproducibility floor of the
    reference step on that frame."""
    q0, qd, it = start

    def frame(q):
        o = O.OracleSim(sc, cfg, n_threads=os.cpu_count() or 1)
        o.set_state(q, qd)
        o.iter = it
        o.step(1)
        return o.state()[0]

    base = frame(q0)
    rng = np.random.default_rng(seed)
    return max(rel(frame(q0 * (1 + eps * rng.normal(size=q0.shape))), base) for _ in range(n))


def assert_frames(O, sc, cfg, errs, starts):
    """Every frame within REL, or, on a frame where the oracle's own sensitivity to
    rounding-level perturbations is above REL / 10, within SENS_FACTOR of it."""
    for k, e in enumerate(errs):
        if e <= REL:
            continue
        s = oracle_sensitivity(O, sc, cfg, starts[k])
        print("frame %d: GPU vs oracle %.2e, oracle sensitivity %.2e" % (k, e, s))
        assert s > REL / 10 and e <= SENS_FACTOR * s, (k, e, s)


def test_frames_match_oracle_cube_stack(O):
    errs, _ = run_pair(O, S.cube_stack(10, seed=0), S.workload_config("cubes"), 60)
    assert errs.max() <= REL


def test_frames_match_oracle_cube_stack_500_frames(O):
    """The 10-cube stack of the plain-method workload over all of its 500 frames."""
    sc, cfg = S.cube_stack(10, seed=0), S.workload_config("cubes")
    errs, starts = run_pair(O, sc, cfg, 500)
    assert_frames(O, sc, cfg, errs, starts)


def test_frames_match_oracle_small_pile(O):
    sc, cfg = S.sphere_pile(3, 3, 2, subdiv=1, seed=2), S.workload_config("pile")
    errs, starts = run_pair(O, sc, cfg, 30)
    assert np.quantile(errs, 0.9) <= REL
    assert_frames(O, sc, cfg, errs, starts)


def test_frames_match_oracle_chain_with_static_link(O):
    cfg = S.workload_config("chain")
    sc = S.torus_chain(6, nu=24, nv=12, seed=3)
    gpu = ABD(sc, cfg)
    gpu.step(60)   # links swing into contact (first edge-edge pairs near frame 48)
    q0, qd = gpu.state()
    errs, starts = run_pair(O, sc, cfg, 30, start=(q0, qd, gpu.iter), gpu=gpu)
    assert_frames(O, sc, cfg, errs, starts)


def test_frames_match_oracle_full_chain(O):
    """The 200-link chain of 48 x 24 tori at full size: the GPU steps it into contact,
    then three frames are compared with the oracle from the same start states."""
    sc, cfg = S.torus_chain(seed=0), S.workload_config("chain")
    gpu = ABD(sc, cfg)
    gpu.step(60)
    q0, qd = gpu.state()
    errs, starts = run_pair(O, sc, cfg, 3, start=(q0, qd, gpu.iter), gpu=gpu)
    assert_frames(O, sc, cfg, errs, starts)


PILE_CKPT = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "adb_gb300", "data",
                         "pile_ckpt.npz")


@pytest.fixture(scope="module")
def full_pile(O):
    z = np.load(PILE_CKPT)
    return S.sphere_pile(seed=0), S.workload_config("pile"), z["q0"], z["qdot"]


def test_cull_bit_exact_full_pile(O, full_pile):
    """The 1024-icosphere pile at its contact-rich checkpoint: pair sets, types and order
    at q (vtn 1) and at q + dq (vtn 2), and the trajectory TOI (vtn 3), all exact."""
    sc, cfg, q0, qd = full_pile
    gpu = ABD(sc, cfg)
    orc = O.OracleSim(sc, cfg, n_threads=os.cpu_count() or 1)
    g, o = gpu.cull(1, q0), orc.cull(1, q0)
    assert len(o[0]) > 10000 and len(o[2]) > 10000
    assert_sets_equal(g, o)
    rng = np.random.default_rng(11)
    dq = np.zeros_like(q0)
    dq[:, :3] = rng.normal(size=(len(q0), 3)) * 2e-3
    dq[:, 3:] = rng.normal(size=(len(q0), 9)) * 2e-4
    assert_sets_equal(gpu.cull(2, q0, dq), orc.cull(2, q0, dq))
    assert gpu.cull(3, q0, dq) == orc.cull(3, q0, dq)


def test_frame_matches_oracle_full_pile(O, full_pile):
    """One whole frame of the 1024-icosphere pile from its checkpoint."""
    sc, cfg, q0, qd = full_pile
    errs, starts = run_pair(O, sc, cfg, 1, start=(q0, qd, 0))
    print("full pile frame: rel %.3e" % errs[0])
    assert errs[0] <= REL
