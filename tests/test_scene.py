"""Scene/config front end: reference schema, meshes and generators (CPU only)."""
import json
import os

import numpy as np

from adb_gb300 import scene as S


def test_cube_mesh_matches_reference_layout():
    m = S.cube_mesh()
    assert m.vertices.shape == (8, 3) and m.faces.shape == (12, 3) and m.edges.shape == (12, 2)
    # edges run along x, then y, then z (cube.h:45-56)
    d = np.abs(m.vertices[m.edges[:, 1]] - m.vertices[m.edges[:, 0]])
    assert np.all(np.argmax(d, axis=1) == np.repeat([0, 1, 2], 4))
    assert abs(m.volume - 1.0) < 1e-12


def test_mesh_counts():
    ico3 = S.icosphere_mesh(3)
    assert (len(ico3.vertices), len(ico3.faces), len(ico3.edges)) == (642, 1280, 1920)
    ico2 = S.icosphere_mesh(2)
    assert (len(ico2.vertices), len(ico2.faces), len(ico2.edges)) == (162, 320, 480)
    tor = S.torus_mesh()
    assert (len(tor.vertices), len(tor.faces), len(tor.edges)) == (1152, 2304, 3456)
    # float-representable rest vertices
    assert np.array_equal(ico3.vertices, ico3.vertices.astype(np.float32).astype(np.float64))


def test_config_parse(tmp_path):
    d = {"dt": 0.005, "max_iter": 50, "gravity": True, "line_search": True, "ee": True, "pt": True, "ground": False,
         "uppper_bound": True, "mu": 0.2, "backoff": 0.8, "eps_x": 1e-3, "psd": True, "iaabb": 3, "evh": 1e-3,
         "vg_friction": True, "pt_friction": True, "ee_friction": False, "kappa": 1e-4,
         "params_double": {"tol": 1e-4, "c1": 1e-4, "max_uk": 0.0}, "params_int": {"clip": 0}}
    p = tmp_path / "config.json"
    p.write_text(json.dumps(d))
    c = S.load_config(str(p))
    assert c.dt == 0.005 and c.max_iter == 50 and not c.ground and c.mu == 0.2 and c.tol == 1e-4
    assert not c.ee_friction and c.dhat == 1e-4 and c.ground_offset == 0.5 and c.gravity_y == -9.8
    back = S.config_to_json(c)
    assert back["uppper_bound"] and back["params_double"]["tol"] == 1e-4


def test_config_library_keys_roundtrip(tmp_path):
    """Keys with no reference counterpart survive the JSON front end both ways."""
    c = S.workload_config("chain")
    c.tri_direct, c.autotune, c.solver = False, False, "dense"
    p = tmp_path / "config.json"
    p.write_text(json.dumps(S.config_to_json(c)))
    b = S.load_config(str(p))
    assert (b.tri_direct, b.autotune, b.solver, b.max_iter_frame) == (False, False, "dense", 100)
    assert S.load_config(str(p)).pcg_rel_tol == c.pcg_rel_tol
    d = json.loads(p.read_text())
    del d["tri_direct"]
    p.write_text(json.dumps(d))
    assert S.load_config(str(p)).tri_direct   # default on


def test_scene_json_roundtrip(tmp_path):
    S.write_obj(str(tmp_path / "ico.obj"), S.icosphere_mesh(1))
    entries = [
        {"omega": [0, 0, 0], "p": [0, 0.6, 0], "p_dot": [0, 0, 0], "euler": [0, 30, 0]},
        {"obj": "ico.obj", "omega": [1, 2, 3], "p": [0, 2, 0], "p_dot": [0, -1, 0], "theta": 45, "mass": 500},
        {"omega": [0, 0, 0], "p": [3, 0, 0], "p_dot": [0, 0, 0], "theta": 0, "mass": -1},
    ]
    S.scene_to_json(entries, str(tmp_path / "scene.json"))
    sc = S.load_scene(str(tmp_path / "scene.json"))
    assert sc.n_bodies == 3
    assert sc.mass[1] == 500 and abs(sc.Ic[1] - 500 / 12) < 1e-12 and sc.mass[2] < 0
    assert abs(sc.Ic[0] - 1000 / 12) < 1e-12
    A0 = sc.q0[0, 3:].reshape(3, 3).T
    assert np.allclose(A0, S.rotation_zyx(0, np.pi / 6, 0))
    # omega -> dA/dt = [w]x (spinning_cube.cpp:100-101)
    W = sc.dqdt[1, 3:].reshape(3, 3).T
    assert np.allclose(W, np.array([[0, -3, 2], [3, 0, -1], [-2, 1, 0]]))


def test_generators_shapes():
    c0 = S.cube_stack(10)
    assert c0.n_bodies == 10 and c0.n_vertices == 80
    assert np.all(np.diff(c0.q0[:, 1]) > 1.0)
    ch = S.torus_chain(4)
    assert ch.mass[0] < 0 and np.all(ch.mass[1:] > 0)
    b = S.batched_scenes(6, seed=1)
    assert len(set(b.scene_id.tolist())) == 6
    assert np.all(np.diff(b.scene_id) >= 0)


def test_scene_ranges_and_body_range():
    sc = S.batched_scenes(n_scenes=5, seed=2, lo=2, hi=6)
    ranges = sc.scene_ranges()
    assert len(ranges) == 5 and ranges[0][0] == 0 and ranges[-1][1] == sc.n_bodies
    assert all(a < b for a, b in ranges) and all(ranges[i][1] == ranges[i + 1][0] for i in range(4))
    b0, b1 = ranges[2]
    sub = sc.body_range(b0, b1)
    assert sub.n_bodies == b1 - b0 and sub.scene_id is None
    assert np.array_equal(sub.q0, sc.q0[b0:b1])
    assert np.array_equal(sub.rest, sc.rest[sc.vert_off[b0]:sc.vert_off[b1]])
    assert sub.vert_off[0] == 0 and sub.vert_off[-1] == sub.rest.shape[0]
    assert sub.faces.max() < (sub.vert_off[1:] - sub.vert_off[:-1]).max()
