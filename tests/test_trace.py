"""Trace files in the reference's binary layout (model/mutils.cpp:257-329)."""
import numpy as np

from adb_gb300 import trace


def test_player_save_load_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    q0, qd = rng.normal(size=(5, 12)), rng.normal(size=(5, 12))
    cfg = tmp_path / "config.json"
    cfg.write_text("{}")
    p = trace.player_save(str(tmp_path / "trace"), 0, q0, qd, init=True, config_json=str(cfg))
    raw = open(p, "rb").read()
    assert len(raw) == 5 * 24 * 8
    # body 0: q0[0] (p) first, then a1, a2, a3, then dqdt
    assert np.frombuffer(raw[:24], "<f8").tolist() == q0[0, :3].tolist()
    assert np.frombuffer(raw[96:120], "<f8").tolist() == qd[0, :3].tolist()
    a, b = trace.player_load(str(tmp_path / "trace"), 0, 5)
    assert np.array_equal(a, q0) and np.array_equal(b, qd)
    assert (tmp_path / "trace" / "config.json").exists()
