"""Writes the contact-rich starting state of the pile benchmark.

Runs the 1024-body icosphere pile (adb_gb300.scene.sphere_pile(seed=0), the "pile"
workload parameters) from rest for FRAMES frames with the GPU step and stores the
per-body state (q0, qdot: 12 doubles each, the reference's trace layout) with the frame
index. Usage: python adb_gb300/data/make_checkpoint.py [frames] [out.npz]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main():
    frames = int(sys.argv[1]) if len(sys.argv) > 1 else 40
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                              "pile_ckpt.npz")
    import __graft_entry__ as G
    G.build()
    from adb_gb300 import scene as S
    from adb_gb300.abd import ABD
    sc = S.sphere_pile(seed=0)
    sim = ABD(sc, S.workload_config("pile"))
    for f in range(frames):
        st = sim.step(1)
        print("frame", f, "status", st.status, "newton", st.newton_iters, "ls", st.ls_trials, "pcg", st.pcg_iters,
              "pairs", st.n_pt, st.n_ee, st.n_vg, "device_ms %.1f" % st.device_ms, flush=True)
    q0, qd = sim.state()
    np.savez_compressed(out, q0=q0, qdot=qd, frame=frames, iter=sim.iter)
    print("wrote", out)


if __name__ == "__main__":
    main()
