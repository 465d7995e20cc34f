"""The oracle's restatement of the spatial-hash broad phase (spatial_hashing.cpp,
col_set.cpp) and of step_size_upper_bound (upper_bound.cpp), checked against the oracle's
iAABB brute force: both cull the set {pairs of different bodies with squared distance
< dhat * safe_factor^2}, so with safe_factor 1 the sets agree; the hashed trajectory bound
agrees with the iAABB trajectory pass once edge trajectories are registered by both ends
(the reference registers them by their start only, which can only miss collisions)."""
import dataclasses

import numpy as np
import pytest

from adb_gb300 import scene as S


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def rand_cubes(n, seed, extent):
    rng = np.random.default_rng(seed)
    sb = S.SceneBuilder()
    for _ in range(n):
        a, b, c = rng.random(3) * 2 * np.pi
        sb.add(S.cube_mesh(), rng.uniform(-extent, extent, 3), S.rotation_zyx(a, b, c))
    return sb.build()


def sim(O, sc, cfg, **kw):
    return O.OracleSim(sc, dataclasses.replace(cfg, **kw))


def sorted_set(res):
    pt, ptt, ee, eet, vg = res
    a = sorted(map(tuple, np.column_stack([pt, ptt]).tolist()))
    b = sorted(map(tuple, np.column_stack([ee, eet]).tolist()))
    c = sorted(map(tuple, vg.tolist()))
    return a, b, c


@pytest.mark.parametrize("bits,dx", [(6, 0.8), (7, 0.12), (2, 0.3)])
def test_hash_set_equals_iaabb_set(O, bits, dx):
    sc = rand_cubes(40, 5, 2.0)
    cfg = S.Config(dhat=1e-2, sh_bits=bits, sh_dx=dx, sh_min_xyz=-5.0)
    ref = sim(O, sc, cfg, iaabb=3).cull(1, sc.q0)
    sh = sim(O, sc, cfg, iaabb=2).cull(1, sc.q0)
    assert len(ref[0]) + len(ref[2]) > 50
    assert sorted_set(sh) == sorted_set(ref)
    rng = np.random.default_rng(1)
    dq = rng.normal(size=sc.q0.shape) * 0.02
    assert sorted_set(sim(O, sc, cfg, iaabb=2).cull(2, sc.q0, dq)) == sorted_set(
        sim(O, sc, cfg, iaabb=3).cull(2, sc.q0, dq))


def test_hash_set_is_canonically_ordered(O):
    """Pairs come grouped by body pair (I < J), vertex-on-I before vertex-on-J, each by
    (primitive, primitive), the layout the overlap-based assembly consumes."""
    sc = rand_cubes(30, 2, 1.8)
    cfg = S.Config(dhat=1e-2, iaabb=2)
    pt, ptt, ee, eet, vg = sim(O, sc, cfg).cull(1, sc.q0)
    lo, hi = np.minimum(pt[:, 0], pt[:, 2]), np.maximum(pt[:, 0], pt[:, 2])
    key = np.lexsort((pt[:, 3], pt[:, 1], (pt[:, 0] > pt[:, 2]).astype(int), hi, lo))
    assert np.array_equal(key, np.arange(len(pt)))
    assert np.all(ee[:, 0] < ee[:, 2])
    key = np.lexsort((ee[:, 3], ee[:, 1], ee[:, 2], ee[:, 0]))
    assert np.array_equal(key, np.arange(len(ee)))


def test_safe_factor_scales_the_threshold(O):
    sc = rand_cubes(30, 3, 1.8)
    cfg = S.Config(dhat=1e-2, iaabb=2)
    a = sorted_set(sim(O, sc, cfg, safe_factor=1.0).cull(1, sc.q0))
    b = sorted_set(sim(O, sc, cfg, safe_factor=1.5).cull(1, sc.q0))
    assert set(a[0]) <= set(b[0]) and set(a[1]) <= set(b[1]) and len(b[0]) + len(b[1]) > len(a[0]) + len(a[1])


def test_hashed_step_bound(O):
    sc = rand_cubes(40, 7, 2.0)
    cfg = S.Config(dhat=1e-2, sh_min_xyz=-5.0)
    rng = np.random.default_rng(4)
    n_hit = 0
    for k in range(6):
        dq = rng.normal(size=sc.q0.shape) * 0.15
        t_ref = sim(O, sc, cfg, iaabb=3).cull(3, sc.q0, dq)
        t_fix = sim(O, sc, cfg, iaabb=0, full_ccd=True, sh_fix_edge_trajectory=True).cull(3, sc.q0, dq)
        t_bug = sim(O, sc, cfg, iaabb=0, full_ccd=True).cull(3, sc.q0, dq)
        assert t_fix == t_ref
        assert t_bug >= t_ref
        n_hit += t_ref < 1.0
    assert n_hit >= 3


def test_norm1_step_bound(O):
    sc = rand_cubes(20, 8, 1.5)
    cfg = S.Config(dhat=1e-2, iaabb=0, full_ccd=False, safe_factor=1.0, ground=False)
    rng = np.random.default_rng(5)
    dq = rng.normal(size=sc.q0.shape) * 0.05
    o = sim(O, sc, cfg)
    o.cull(1, sc.q0)
    t = o.cull(3, sc.q0, dq)
    n1 = np.abs(dq).sum(axis=1).max()
    assert 0 < t <= min(1.0, np.sqrt(cfg.dhat) / 2 / n1) + 0.0


def test_hash_frames_match_iaabb_frames(O):
    """Whole frames with the spatial-hash culling and hashed step bound (edges registered
    by both ends) against the iAABB configuration: same pair sets at every cull, so the
    states agree to rounding."""
    sc = S.cube_stack(6, seed=1)
    cfg = S.workload_config("cubes")
    a = sim(O, sc, cfg, iaabb=3)
    b = sim(O, sc, cfg, iaabb=0, sh_fix_edge_trajectory=True, sh_min_xyz=-5.0, sh_dx=0.3, sh_bits=6)
    for _ in range(30):
        sa, sb = a.step(1), b.step(1)
        assert (sa.newton_iters, sa.ls_trials) == (sb.newton_iters, sb.ls_trials)
    qa, qda = a.state()
    qb, qdb = b.state()
    assert np.abs(qa - qb).max() <= 1e-12 * np.abs(qa).max()
