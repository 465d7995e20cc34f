"""C ABI behaviour on the GPU: file front end, status codes and bounded loops.
Failures are made on the host (invalid arguments, a NaN state, an iteration cap);
nothing here faults or hangs the GPU."""
import ctypes as C
import json

import numpy as np
import pytest

from adb_gb300 import _lib as L
from adb_gb300 import scene as S

pytestmark = pytest.mark.gpu


def test_create_from_files_matches_array_path(gpu_lib, tmp_path):
    from adb_gb300.abd import ABD
    S.write_obj(str(tmp_path / "ico.obj"), S.icosphere_mesh(1))
    entries = [{"omega": [0, 0, 0], "p": [0, 0.2, 0], "p_dot": [0, 0, 0], "euler": [0, 30, 0]},
               {"obj": "ico.obj", "omega": [0.5, 0, 0], "p": [0.1, 1.4, 0], "p_dot": [0, -1, 0], "theta": 10,
                "mass": 400}]
    S.scene_to_json(entries, str(tmp_path / "scene.json"))
    cfg = S.workload_config("cubes")
    with open(tmp_path / "config.json", "w") as f:
        json.dump(S.config_to_json(cfg), f)
    a = ABD.from_files(str(tmp_path / "config.json"), str(tmp_path / "scene.json"))
    b = ABD(S.load_scene(str(tmp_path / "scene.json")), S.load_config(str(tmp_path / "config.json")))
    qa, _ = a.state()
    qb, _ = b.state()
    assert np.array_equal(qa, qb)
    for _ in range(3):
        a.implicit_euler()
        b.implicit_euler()
    qa, va = a.state()
    qb, vb = b.state()
    assert np.abs(qa - qb).max() <= 1e-12 * np.abs(qb).max()


def test_invalid_arguments_return_status(gpu_lib):
    h = C.c_void_p()
    assert gpu_lib.abd_create(None, None, C.byref(h)) == 8
    assert gpu_lib.abd_create_from_files(b"/nonexistent/config.json", b"/nonexistent/scene.json", C.byref(h)) == 9
    assert gpu_lib.abd_step(None, 0.0, 1, None) == 8


def test_nan_state_reports_status(gpu_lib):
    from adb_gb300.abd import ABD
    sc = S.cube_stack(2, seed=0)
    sim = ABD(sc, S.workload_config("cubes"))
    q, qd = sim.state()
    qd[0, 1] = np.nan
    sim.set_state(q, qd)
    st = sim.step(1, raise_on_error=False)
    assert st.status == 1  # ABD_ERR_NAN


def test_pcg_iteration_cap_reports_and_continues(gpu_lib):
    from adb_gb300.abd import ABD
    cfg = S.workload_config("cubes")
    cfg.pcg_max_iter = 1
    cfg.tri_direct = False   # a stack is block-tridiagonal: keep it on the CG
    sim = ABD(S.cube_stack(4, gap=0.01, seed=2), cfg)
    st = sim.step(3, raise_on_error=False)
    assert st.frames == 3
    assert st.status in (0, 6)


def test_stats_and_profile(gpu_lib):
    from adb_gb300.abd import ABD
    sim = ABD(S.cube_stack(4, gap=0.01, seed=3), S.workload_config("cubes"))
    sim.profile(True)
    st = sim.step(2)
    kt = sim.kernel_times()
    sim.profile(False)
    assert st.kernel_launches > 0 and st.device_ms > 0
    assert kt["pair_terms"]["launches"] >= 0 and kt["pcg"]["launches"] == st.newton_iters
    assert sum(v["launches"] for v in kt.values()) == st.kernel_launches
