"""Frame traces in the reference's binary format.

`player_save` (model/mutils.cpp:293-329) writes one file per frame, `<folder>/<ts>`,
holding for each body its q0 (4 x vec3: p, a1, a2, a3) then its dqdt (4 x vec3) as raw
little-endian doubles; `player_load` (model/mutils.cpp:257-276) reads them back and the
viewer resumes from `"starting_ts"` (view/control.cpp:84-90). `dump_states`
(model/mutils.cpp:278-292) writes q then dq under the same layout.
"""
from __future__ import annotations

import os
import shutil
from typing import Optional, Tuple

import numpy as np


def frame_path(folder: str, ts: int) -> str:
    return os.path.join(folder, str(int(ts)))


def player_save(folder: str, ts: int, q0: np.ndarray, qdot: np.ndarray, init: bool = False,
                config_json: Optional[str] = None, scene_json: Optional[str] = None) -> str:
    """Writes frame `ts`. With init=True the folder is recreated and the config and scene
    files are copied into it, as the reference does on its first frame."""
    if init:
        if os.path.exists(folder):
            shutil.rmtree(folder)
        os.makedirs(folder)
        for f in (config_json, scene_json):
            if f:
                shutil.copy(f, folder)
    os.makedirs(folder, exist_ok=True)
    q0 = np.asarray(q0, np.float64).reshape(-1, 12)
    qd = np.asarray(qdot, np.float64).reshape(-1, 12)
    buf = np.concatenate([q0, qd], axis=1).astype("<f8")
    p = frame_path(folder, ts)
    with open(p, "wb") as f:
        f.write(buf.tobytes())
    return p


def player_load(folder: str, ts: int, n_bodies: int) -> Tuple[np.ndarray, np.ndarray]:
    with open(frame_path(folder, ts), "rb") as f:
        raw = np.frombuffer(f.read(), dtype="<f8")
    if raw.size != 24 * n_bodies:
        raise ValueError("trace frame %s holds %d doubles, expected %d" % (frame_path(folder, ts), raw.size,
                                                                            24 * n_bodies))
    a = raw.reshape(n_bodies, 24)
    return a[:, :12].copy(), a[:, 12:].copy()


def dump_states(path: str, q: np.ndarray, dq: np.ndarray) -> None:
    buf = np.concatenate([np.asarray(q, np.float64).reshape(-1, 12), np.asarray(dq, np.float64).reshape(-1, 12)],
                         axis=1).astype("<f8")
    with open(path, "wb") as f:
        f.write(buf.tobytes())


def record(sim, folder: str, frames: int, start_ts: int = 0, config_json=None, scene_json=None) -> None:
    """Steps `sim` (ABD) for `frames` frames, saving each frame like the reference's
    viewer loop (view/model_view.cpp:284-295)."""
    for k in range(frames):
        sim.implicit_euler()
        q0, qd = sim.state()
        player_save(folder, start_ts + k, q0, qd, init=(k == 0 and start_ts == 0), config_json=config_json,
                    scene_json=scene_json)


def resume(sim, folder: str, ts: int) -> None:
    """Loads frame `ts` into `sim` (the reference's "starting_ts" resume)."""
    q0, qd = player_load(folder, ts, sim.nb)
    sim.set_state(q0, qd)
