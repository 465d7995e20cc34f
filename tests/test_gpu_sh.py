"""Spatial-hash broad phase on the GPU (iaabb even; step_size_upper_bound for iaabb <= 1)
against the oracle's restatement: pair sets, their order and distance types bit-exact,
step bounds bit-exact, frames within 1e-9 relative."""
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


def rand_cubes(n, seed, extent, lift=0.0):
    rng = np.random.default_rng(seed)
    sb = S.SceneBuilder()
    for _ in range(n):
        a, b, c = rng.random(3) * 2 * np.pi
        p = rng.uniform(-extent, extent, 3)
        p[1] += lift
        sb.add(S.cube_mesh(), p, S.rotation_zyx(a, b, c))
    return sb.build()


def assert_sets_equal(g, o):
    for name, a, b in zip(("pt", "pt_type", "ee", "ee_type", "vg"), g, o):
        assert a.shape == b.shape and np.array_equal(a, b), name


@pytest.mark.parametrize("bits,dx", [(6, 0.8), (7, 0.12), (2, 0.3)])
def test_hash_cull_bit_exact(O, bits, dx):
    sc = rand_cubes(40, 5, 2.0)
    cfg = S.Config(dhat=1e-2, iaabb=2, sh_bits=bits, sh_dx=dx, sh_min_xyz=-5.0)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    g, o = gpu.cull(1, sc.q0), orc.cull(1, sc.q0)
    assert len(o[0]) + len(o[2]) > 50
    assert_sets_equal(g, o)
    rng = np.random.default_rng(1)
    dq = rng.normal(size=sc.q0.shape) * 0.02
    assert_sets_equal(gpu.cull(2, sc.q0, dq), orc.cull(2, sc.q0, dq))


@pytest.mark.parametrize("fix", [False, True])
def test_hashed_step_bound_bit_exact(O, fix):
    sc = rand_cubes(40, 7, 2.0, lift=3.0)
    cfg = S.Config(dhat=1e-2, iaabb=0, full_ccd=True, sh_fix_edge_trajectory=fix, sh_min_xyz=-5.0, sh_dx=0.4)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    rng = np.random.default_rng(4)
    hits = 0
    for _ in range(5):
        dq = rng.normal(size=sc.q0.shape) * 0.15
        tg, to = gpu.cull(3, sc.q0, dq), orc.cull(3, sc.q0, dq)
        assert tg == to
        hits += to < 1.0
    assert hits >= 2


def test_norm1_step_bound_bit_exact(O):
    sc = rand_cubes(30, 8, 1.6, lift=3.0)
    cfg = S.Config(dhat=1e-2, iaabb=0, full_ccd=False, safe_factor=1.0)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    rng = np.random.default_rng(5)
    for k in range(4):
        dq = rng.normal(size=sc.q0.shape) * (0.01 if k % 2 else 0.2)
        gpu.cull(1, sc.q0)
        orc.cull(1, sc.q0)
        assert gpu.cull(3, sc.q0, dq) == orc.cull(3, sc.q0, dq)


@pytest.mark.parametrize("iaabb", [0, 2])
def test_hash_frames_match_oracle(O, iaabb):
    sc = S.cube_stack(8, seed=2)
    cfg = dataclasses.replace(S.workload_config("cubes"), iaabb=iaabb, sh_min_xyz=-5.0, sh_dx=0.3)
    gpu, orc = ABD(sc, cfg), O.OracleSim(sc, cfg)
    worst = 0.0
    for _ in range(25):
        sg, so = gpu.step(1), orc.step(1)
        assert (sg.newton_iters, sg.ls_trials) == (so.newton_iters, so.ls_trials)
        qg, _ = gpu.state()
        qo, qdo = orc.state()
        worst = max(worst, float(np.abs(qg - qo).max() / np.abs(qo).max()))
        gpu.set_state(qo, qdo)
    assert worst <= 1e-9
