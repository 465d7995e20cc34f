"""Batched mode: independent scenes stepped in one handle give, scene by scene, exactly
what each scene gives when stepped alone (same pair sets, same Newton and line-search
decisions, same states bit for bit), because every scene keeps its own Newton loop, CCD
bound, line search and CG scalars and every reduction runs in a scene-relative order."""
import numpy as np
import pytest

from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu


def ABD(scene, cfg):
    from adb_gb300.abd import ABD as _ABD
    return _ABD(scene, cfg)


def small_batch(seed=3, n=6):
    return S.batched_scenes(n_scenes=n, seed=seed, lo=2, hi=6, spacing=4.0)


@pytest.mark.parametrize("frames", [6])
def test_batched_equals_looped_bitwise(gpu_lib, frames):
    sc = small_batch()
    cfg = S.workload_config("batched")
    ranges = sc.scene_ranges()
    assert len(ranges) == 6
    bat = ABD(sc, cfg)
    assert bat.n_scenes == 6
    newton = np.zeros(len(ranges), dtype=np.int64)
    ls = np.zeros(len(ranges), dtype=np.int64)
    for _ in range(frames):
        bat.step(1)
        st = bat.scene_stats()
        newton += st["newton_iters"]
        ls += st["ls_trials"]
    bq, bqd = bat.state()
    iters = bat.scene_stats()["iter"]
    for k, (b0, b1) in enumerate(ranges):
        one = ABD(sc.body_range(b0, b1), cfg)
        n_k = ls_k = 0
        for _ in range(frames):
            s1 = one.step(1)
            n_k += s1.newton_iters
            ls_k += s1.ls_trials
        q, qd = one.state()
        assert (n_k, ls_k) == (newton[k], ls[k]), "scene %d Newton/line-search counts" % k
        assert one.iter == iters[k]
        assert np.array_equal(q, bq[b0:b1]), "scene %d q0" % k
        assert np.array_equal(qd, bqd[b0:b1]), "scene %d qdot" % k
    # the run must have had contacts and more than one Newton iteration somewhere
    assert newton.max() > frames


def test_batched_scenes_finish_independently(gpu_lib):
    """A scene at rest converges in fewer iterations than a falling, colliding one, and
    its state is not touched while the other keeps iterating."""
    sb = S.SceneBuilder()
    cube = S.cube_mesh()
    g = S.GROUND_SHIFT
    # scene 0: one cube resting just above the ground with no velocity
    sb.add(cube, (0.0, 0.5 + 0.05 + g, 0.0), np.eye(3), scene_id=0)
    # scene 1: two cubes, the upper one thrown down onto the lower one
    sb.add(cube, (10.0, 0.5 + 0.05 + g, 0.0), np.eye(3), scene_id=1)
    sb.add(cube, (10.0, 1.6 + 0.05 + g, 0.0), S.rotation_zyx(0.3, 0.2, 0.1), p_dot=(0.0, -3.0, 0.0), scene_id=1)
    sc = sb.build()
    cfg = S.workload_config("batched")
    bat = ABD(sc, cfg)
    for _ in range(4):
        bat.step(1)
    st = bat.scene_stats()
    q, qd = bat.state()
    for k, (b0, b1) in enumerate(sc.scene_ranges()):
        one = ABD(sc.body_range(b0, b1), cfg)
        one.step(4)
        q1, qd1 = one.state()
        assert np.array_equal(q1, q[b0:b1]) and np.array_equal(qd1, qd[b0:b1])
    assert st["newton_iters"][0] <= st["newton_iters"][1]


def test_non_contiguous_scene_ids_rejected(gpu_lib):
    from adb_gb300 import _lib as L
    sb = S.SceneBuilder()
    cube = S.cube_mesh()
    for k, sid in enumerate((0, 1, 0)):
        sb.add(cube, (3.0 * k, 1.0, 0.0), np.eye(3), scene_id=sid)
    sc = sb.build()
    with pytest.raises(L.AbdError):
        ABD(sc, S.workload_config("batched"))


def test_many_groups_equal_single_scenes_bitwise(gpu_lib):
    """More body groups than one cooperative wave holds (the PCG then loops over groups,
    each CTA serving several) against the same scenes stepped alone (one group per CTA):
    the two solver layouts give the same iterates bit for bit."""
    sc = S.batched_scenes(n_scenes=200, seed=5, lo=2, hi=3, spacing=4.0)
    cfg = S.workload_config("batched")
    ranges = sc.scene_ranges()
    bat = ABD(sc, cfg)
    bat.step(4)
    bq, bqd = bat.state()
    newton = bat.scene_stats()["newton_iters"]
    for k in (0, 57, 123, 199):
        b0, b1 = ranges[k]
        one = ABD(sc.body_range(b0, b1), cfg)
        one.step(4)
        q, qd = one.state()
        assert np.array_equal(q, bq[b0:b1]) and np.array_equal(qd, bqd[b0:b1]), "scene %d" % k
    assert newton.max() >= 1
