"""Config switches of the step against the oracle: damping (damping_sparse,
mutils.cpp:106-115) and the same-direction stop (abd.cpp:180-190)."""
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
