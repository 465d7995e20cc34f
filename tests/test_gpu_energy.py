"""Energies of the GPU step (abd_energy, through the C ABI) against the oracle's
restatement of the reference's line-search energies (energy.cpp:19-86 E_barrier_plus_inert,
:195-258 E_fric, :261-270 E_ground).

Each case is the first line-search trial of a Newton iteration at alpha = 1: friction
lagged at q, barrier and inertia at q + dq, dq a Newton step of the oracle. Bar: the same
pair lists; every per-pair barrier and friction energy within 1e-9 relative; every
per-scene term and the line-search total within 1e-9 relative."""
import numpy as np
import pytest

from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu

REL = 1e-9


@pytest.fixture(scope="module")
def O(gpu_lib, oracle_lib):
    return oracle_lib


def pair_rel(g, o):
    """Largest per-pair relative difference (pairs with zero energy must match exactly)."""
    if len(o) == 0:
        return 0.0
    den = np.abs(o)
    err = np.abs(g - o)
    zero = den == 0
    assert np.all(err[zero] == 0.0)
    return float((err[~zero] / den[~zero]).max()) if (~zero).any() else 0.0


def compare(O, sc, cfg, q0, qd, dq):
    from adb_gb300.abd import ABD
    gpu = ABD(sc, cfg)
    gpu.set_state(q0, qd)
    orc = O.OracleSim(sc, cfg)
    orc.set_state(q0, qd)
    g = gpu.energy(q0, dq)
    o = orc.energy_terms(q0, dq)
    assert np.array_equal(g["counts"], o["counts"])
    for k in ("e_pt", "e_ee", "e_vg", "f_pt", "f_ee", "f_vg"):
        assert pair_rel(g[k], o[k]) <= REL, k
    assert_terms(g["terms"][0], o["terms"])
    gpu.close()
    return g, o


def assert_terms(gt, ot):
    """Scene terms within REL of the scene's energy scale: a Newton step that lands on the
    inertial target leaves an inertia term of ~1e-26 that only rounding decides, so each
    term is measured against the largest of itself and the scene total."""
    scale = max(np.abs(ot).sum(), 1e-300)
    for i in range(5):
        assert abs(gt[i] - ot[i]) <= REL * max(abs(ot[i]), scale), (i, gt[i], ot[i])
    assert abs(gt[5] - ot.sum()) <= REL * scale


def newton_dq(O, sc, cfg, q0, qd, scale):
    o = O.OracleSim(sc, cfg)
    o.set_state(q0, qd)
    return o.newton_dq(q0).reshape(q0.shape) * scale


def test_energies_match_oracle_small_pile(O):
    sc, cfg = S.sphere_pile(3, 3, 2, subdiv=1, seed=2), S.workload_config("pile")
    orc = O.OracleSim(sc, cfg)
    n_pairs = 0
    for f in range(28):
        orc.step(1)
        if f % 4 == 3:
            q0, qd = orc.state()
            for scale in (0.0, 0.5, 1.0):
                g, o = compare(O, sc, cfg, q0, qd, newton_dq(O, sc, cfg, q0, qd, scale))
                n_pairs += int(g["counts"].sum())
                if scale == 0.0:  # no step: the set at q + dq is the lagged one
                    assert np.array_equal(g["counts"][:3], g["counts"][3:])
    assert n_pairs > 1000


def test_energies_match_oracle_cube_stack_with_friction(O):
    sc, cfg = S.cube_stack(10, seed=0), S.workload_config("cubes")
    orc = O.OracleSim(sc, cfg)
    orc.step(40)
    q0, qd = orc.state()
    g, o = compare(O, sc, cfg, q0, qd, newton_dq(O, sc, cfg, q0, qd, 1.0))
    assert g["counts"][2] > 0 and g["terms"][0][4] > 0.0


def test_energies_match_oracle_chain(O):
    from adb_gb300.abd import ABD
    sc, cfg = S.torus_chain(6, nu=24, nv=12, seed=3), S.workload_config("chain")
    gpu = ABD(sc, cfg)
    gpu.step(78)   # links in contact
    q0, qd = gpu.state()
    gpu.close()
    g, o = compare(O, sc, cfg, q0, qd, newton_dq(O, sc, cfg, q0, qd, 1.0))
    assert g["counts"][1] > 0


def test_energies_per_scene_in_a_batch(O):
    """Per-scene terms of a batched handle equal those of each scene alone (oracle)."""
    from adb_gb300.abd import ABD
    sc = S.batched_scenes(n_scenes=6, seed=4, hi=12)
    cfg = S.workload_config("batched")
    bat = ABD(sc, cfg)
    bat.step(45)
    q0, qd = bat.state()
    dq = np.zeros_like(q0)
    for b0, b1 in sc.scene_ranges():
        sub = sc.body_range(b0, b1)
        dq[b0:b1] = newton_dq(O, sub, cfg, q0[b0:b1], qd[b0:b1], 1.0)
    bat.set_state(q0, qd)
    g = bat.energy(q0, dq)
    for k, (b0, b1) in enumerate(sc.scene_ranges()):
        o = O.OracleSim(sc.body_range(b0, b1), cfg)
        o.set_state(q0[b0:b1], qd[b0:b1])
        assert_terms(g["terms"][k], o.energy_terms(q0[b0:b1], dq[b0:b1])["terms"])
