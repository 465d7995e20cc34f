"""Traces and the viewer loop through the C++ front end (abd_create_from_files,
abd_run, abd_trace_save / abd_trace_load): frame files in the reference's binary layout
(player_save / player_load, model/mutils.cpp:257-276, 293-329), "starting_ts" resume
(view/control.cpp:84-90) and the ending_ts stop of the viewer loop
(view/model_view.cpp:282-295)."""
import json
import os

import numpy as np
import pytest

from adb_gb300 import scene as S
from adb_gb300 import trace as T

pytestmark = pytest.mark.gpu


def write_case(tmp_path, starting_ts, ending_ts, folder):
    entries = []
    rng = np.random.default_rng(5)
    for k in range(4):
        entries.append({"omega": [0.0, float(rng.normal()), 0.0], "p": [0.0, 0.05 + 1.1 * k, 0.0],
                        "p_dot": [0.0, 0.0, 0.0], "euler": [0.0, float(rng.uniform(0, 90)), 0.0]})
    S.scene_to_json(entries, str(tmp_path / "scene.json"))
    cfg = S.config_to_json(S.workload_config("cubes"))
    cfg.update({"trace_folder": str(folder), "starting_ts": starting_ts, "ending_ts": ending_ts, "player": False})
    with open(tmp_path / "config.json", "w") as f:
        json.dump(cfg, f)
    return str(tmp_path / "config.json"), str(tmp_path / "scene.json")


def test_record_resume_and_oracle_parity(gpu_lib, oracle_lib, tmp_path):
    from adb_gb300.abd import ABD
    folder = tmp_path / "trace"
    cj, sj = write_case(tmp_path, -1, 12, folder)
    a = ABD.from_files(cj, sj)
    assert a.trace == {"folder": str(folder), "ts": 0, "starting_ts": -1, "ending_ts": 12}
    st = a.run(record=True)
    assert st.frames == 12 and a.trace["ts"] == 12
    # frame files 1..12 (the counter advances inside the step), plus the copied config and scene
    names = sorted(os.listdir(folder))
    assert names == sorted([str(k) for k in range(1, 13)] + ["config.json", "scene.json"])
    qa, va = a.state()
    q12, v12 = T.player_load(str(folder), 12, a.nb)
    assert np.array_equal(q12, qa) and np.array_equal(v12, va)
    # the oracle steps the same scene through the same 12 frames
    sc, cfg = S.load_scene(sj), S.load_config(cj)
    orc = oracle_lib.OracleSim(sc, cfg)
    for k in range(1, 13):
        orc.step(1)
        qo, _ = orc.state()
        qk, _ = T.player_load(str(folder), k, a.nb)
        assert np.abs(qk - qo).max() <= 1e-9 * np.abs(qo).max(), k
    # resume from frame 6 of the trace: the state is the file's, the counter starts there,
    # and the loop reproduces frames 7..12 bit for bit
    cj2, sj2 = write_case(tmp_path, 6, 12, folder)
    b = ABD.from_files(cj2, sj2)
    q6, v6 = T.player_load(str(folder), 6, b.nb)
    qb, vb = b.state()
    assert np.array_equal(qb, q6) and np.array_equal(vb, v6)
    assert b.trace["ts"] == 6 and b.trace["starting_ts"] == 6
    ref = {k: T.player_load(str(folder), k, b.nb) for k in range(7, 13)}
    b.run(record=True)
    for k in range(7, 13):
        qk, vk = T.player_load(str(folder), k, b.nb)
        assert np.array_equal(qk, ref[k][0]) and np.array_equal(vk, ref[k][1]), k


def test_trace_files_written_by_python_load_exactly(gpu_lib, tmp_path):
    from adb_gb300.abd import ABD
    sc = S.cube_stack(3, seed=1)
    sim = ABD(sc, S.workload_config("cubes"))
    rng = np.random.default_rng(2)
    q, v = rng.normal(size=(3, 12)), rng.normal(size=(3, 12))
    T.player_save(str(tmp_path / "t"), 4, q, v, init=True)
    sim.trace_load(str(tmp_path / "t"), 4)
    q1, v1 = sim.state()
    assert np.array_equal(q1, q) and np.array_equal(v1, v)
    sim.trace_save(str(tmp_path / "t"), 5)
    with open(tmp_path / "t" / "4", "rb") as f4, open(tmp_path / "t" / "5", "rb") as f5:
        assert f4.read() == f5.read()


def test_missing_trace_frame_is_an_io_error(gpu_lib, tmp_path):
    from adb_gb300 import _lib as L
    from adb_gb300.abd import ABD
    cj, sj = write_case(tmp_path, 3, 10, tmp_path / "nothing_here")
    with pytest.raises(L.AbdError, match="ABD_ERR_IO"):
        ABD.from_files(cj, sj)
    sim = ABD.from_files(*write_case(tmp_path, -1, 0, tmp_path / "x"))
    assert L.lib().abd_run(sim._h, 0, None) == 8   # no ending_ts: the loop would not end
