"""Config switches of the step against the oracle: damping (damping_sparse,
mutils.cpp:106-115), the same-direction stop (abd.cpp:180-190) and the dense solver
("solver": "dense", abd.cpp:233-264)."""
import dataclasses

import numpy as np
import pytest

from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O(gpu_lib, oracle_lib):
    return oracle_lib


def ABD(scene, cfg):
    from adb_gb300.abd import ABD as _ABD
    return _ABD(scene, cfg)


def test_damping_frames_match_oracle(O):
    sc = S.cube_stack(6, seed=3)
    cfg = dataclasses.replace(S.workload_config("cubes"), damping=True, damp_alpha=0.05, damp_beta=0.025)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    worst = 0.0
    for _ in range(20):
        sg, so = gpu.step(1), orc.step(1)
        assert (sg.newton_iters, sg.ls_trials) == (so.newton_iters, so.ls_trials)
        qg, _ = gpu.state()
        qo, qdo = orc.state()
        worst = max(worst, float(np.abs(qg - qo).max() / np.abs(qo).max()))
        gpu.set_state(qo, qdo)
    assert worst <= 1e-9


def test_same_direction_stop_matches_oracle(O):
    sb = S.SceneBuilder()
    sb.add(S.cube_mesh(), (0.0, 3.0, 0.0), S.rotation_zyx(0.2, 0.1, 0.3), p_dot=(0.5, 0.0, 0.0))
    sc = sb.build()
    cfg = dataclasses.replace(S.workload_config("cubes"), dq_tol=1.5)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    stop_g = stop_o = None
    for f in range(10):
        so = orc.step(1)
        if stop_o is None and so.status == 10:
            stop_o = f
        sg = gpu.step(1, raise_on_error=False)
        if stop_g is None and sg.status == 10:
            stop_g = f
        if stop_o is not None or stop_g is not None:
            break
    assert stop_o is not None and stop_g == stop_o


def test_dense_solver_frames_match_oracle(O):
    """"solver": "dense": each Newton step by a dense Cholesky of the scene's matrix (the
    reference's big_hess.ldlt()); frames against the oracle's direct solve from the same
    start states, at the per-frame bar of the sparse path."""
    from test_gpu_parity import assert_frames, run_pair
    for sc, name, frames in ((S.cube_stack(10, seed=0), "cubes", 60),
                             (S.sphere_pile(3, 3, 2, subdiv=1, seed=2), "pile", 30)):
        cfg = dataclasses.replace(S.workload_config(name), solver="dense")
        errs, starts = run_pair(O, sc, cfg, frames)
        assert np.quantile(errs, 0.9) <= 1e-9
        assert_frames(O, sc, cfg, errs, starts)


def test_dense_and_sparse_steps_agree(O):
    """Newton steps of the dense Cholesky and of the PCG on the same contact-rich systems
    (a 27-sphere pile: 324 unknowns, six 64 x 64 tiles per side)."""
    sc = S.sphere_pile(3, 3, 3, subdiv=1, seed=4)
    cfg = S.workload_config("pile")
    orc = O.OracleSim(sc, cfg)
    orc.step(30)
    q0, qd = orc.state()
    sp = ABD(sc, cfg)
    de = ABD(sc, dataclasses.replace(cfg, solver="dense"))
    for g in (sp, de):
        g.set_state(q0, qd)
    a, _ = sp.newton_dq(q0)
    b, its = de.newton_dq(q0)
    assert its == 0
    o = O.OracleSim(sc, cfg)
    o.set_state(q0, qd)
    ref = o.newton_dq(q0).reshape(a.shape)
    scale = np.abs(ref).max()
    assert np.abs(b - ref).max() <= 1e-9 * scale
    assert np.abs(a - b).max() <= 1e-9 * scale


def test_dense_solver_batched_equals_looped(O):
    """Dense solves of a batch run scene by scene: a batched handle reproduces each scene
    stepped alone bit for bit."""
    sc = S.batched_scenes(n_scenes=5, seed=2, hi=10)
    cfg = dataclasses.replace(S.workload_config("batched"), solver="dense")
    bat = ABD(sc, cfg)
    bat.step(40)
    bq, bqd = bat.state()
    for b0, b1 in sc.scene_ranges():
        h = ABD(sc.body_range(b0, b1), cfg)
        h.step(40)
        q, qd = h.state()
        assert np.array_equal(q, bq[b0:b1]) and np.array_equal(qd, bqd[b0:b1])
