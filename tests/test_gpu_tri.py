"""Direct solve of block-tridiagonal scenes (tri.cu): a scene whose contacts only join
consecutive bodies (a chain, a stack) is solved by a block Cholesky of each run of linked
bodies instead of the block-Jacobi PCG. Its Newton steps are compared with the oracle's
direct block-sparse Cholesky (the reference factorizes, model/abd.cpp:229-303), and a
batch that mixes such scenes with a pile (PCG) must still reproduce every scene stepped
alone bit for bit. Frames of the chain and the cube stack against the oracle run through
this path in test_gpu_parity.py."""
import dataclasses

import numpy as np
import pytest

from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu
REL = 1e-9


@pytest.fixture(scope="module")
def O(gpu_lib, oracle_lib):
    return oracle_lib


def ABD(scene, cfg):
    from adb_gb300.abd import ABD as _ABD
    return _ABD(scene, cfg)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def orc_dq(O, sc, cfg, q0, qd, q):
    o = O.OracleSim(sc, cfg)
    o.set_state(q0, qd)
    return o.newton_dq(q)


def coupled_state(sc, cfg, first, last, blocks):
    """The first frame start in [first, last) whose Newton system couples at least
    `blocks` body pairs."""
    sim = ABD(sc, cfg)
    sim.step(first)
    for _ in range(first, last):
        q0, qd = sim.state()
        sim.cull(1, q0)
        keys = sim.newton_system(q0)[2]
        if len(keys) >= blocks:
            return q0, qd, keys
        sim.step(1)
    raise AssertionError("no frame with %d coupled body pairs" % blocks)


def test_tri_direct_steps_match_oracle_direct_solve(O):
    """A 6-link chain swung into contact and a 10-cube stack that has landed, its cubes
    resting on one another (a run of at least six linked bodies)."""
    cases = [("chain", S.torus_chain(6, nu=24, nv=12, seed=3), S.workload_config("chain"), 40, 200, 1),
             ("stack", S.cube_stack(10, seed=0), S.workload_config("cubes"), 5, 200, 6)]
    for name, sc, cfg, first, last, blocks in cases:
        q0, qd, keys = coupled_state(sc, cfg, first, last, blocks)
        assert np.all(np.abs(keys[:, 0] - keys[:, 1]) == 1), name
        sim = ABD(sc, cfg)
        sim.set_state(q0, qd)
        ref = orc_dq(O, sc, cfg, q0, qd, q0)
        dq, its = sim.newton_dq(q0)
        assert its == 0, name          # no CG iteration: the direct path solved it
        pcg = ABD(sc, dataclasses.replace(cfg, tri_direct=False))
        pcg.set_state(q0, qd)
        dq_p, its_p = pcg.newton_dq(q0)
        assert its_p > 0, name
        e, e_p = rel(dq, ref), rel(dq_p, ref)
        print("%s: %d coupling blocks; direct %.2e, PCG %.2e (%d iterations) from the oracle" % (
            name, len(keys), e, e_p, its_p))
        assert e <= 1e-11 and e_p <= REL, name


def shifted(sc, dx):
    sc = sc.copy()
    sc.q0[:, 0] += dx
    return sc


def test_mixed_batch_equals_looped_bitwise(gpu_lib):
    """A pile (CG) and two stacks (direct) in one handle: every scene's states and Newton,
    line-search and CG counts equal those of the scene stepped alone."""
    parts = [S.sphere_pile(3, 3, 2, subdiv=1, seed=2), shifted(S.cube_stack(6, seed=1), 8.0),
             shifted(S.cube_stack(4, seed=4), 12.0)]
    sc = parts[0]
    for p in parts[1:]:
        sc = S.concat_scenes(sc, p)
    sc.scene_id = np.concatenate([np.full(p.n_bodies, k, np.int32) for k, p in enumerate(parts)])
    cfg = S.workload_config("batched")
    frames = 30
    bat = ABD(sc, cfg)
    counts = np.zeros((len(parts), 3), np.int64)
    for _ in range(frames):
        bat.step(1)
        st = bat.scene_stats()
        counts[:, 0] += st["newton_iters"]
        counts[:, 1] += st["ls_trials"]
        counts[:, 2] += st["pcg_iters"]
    bq, bqd = bat.state()
    assert counts[0, 2] > 0 and counts[1, 2] == 0 and counts[2, 2] == 0
    for k, (b0, b1) in enumerate(sc.scene_ranges()):
        one = ABD(sc.body_range(b0, b1), cfg)
        c = np.zeros(3, np.int64)
        for _ in range(frames):
            s1 = one.step(1)
            c += (s1.newton_iters, s1.ls_trials, s1.pcg_iters)
        q, qd = one.state()
        assert np.array_equal(c, counts[k]), k
        assert np.array_equal(q, bq[b0:b1]) and np.array_equal(qd, bqd[b0:b1]), k
    assert counts[:, 0].min() > frames   # every scene met contacts
