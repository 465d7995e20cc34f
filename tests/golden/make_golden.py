"""Generates the golden fixtures of the oracle tests (run in a container that has the
reference tree; the outputs are committed next to this script).

- cubic_roots.npz: coefficients and the roots returned by the reference's own cubic
  root finder (cyCodeBase/cyPolynomial.h `cy::CubicRoots`, compiled from the reference
  sources by oracle/Makefile into oracle/_ref/libref_cubic.so) on [0, 1].
- pt_toi_known.npz: point-triangle trajectories with a constructed time of impact, the
  reference's known-answer test Sample-Test1/test.cpp:9-31 (explicit PCG64 seed).
- det_poly.npz: det_polynomial inputs with the determinants at t in {0, 1, w}
  (Sample-Test1/test.cpp:33-60), computed with numpy.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cubic_cases(rng, n):
    cs = []
    for i in range(n):
        c = rng.normal(size=4)
        k = i % 6
        if k == 1:
            c[3] *= 1e-6          # nearly quadratic
        elif k == 2:
            r = rng.random(3)     # three roots in [0, 1]
            c = np.array([-r[0] * r[1] * r[2], r[0] * r[1] + r[1] * r[2] + r[0] * r[2], -(r.sum()), 1.0])
        elif k == 3:
            r = rng.random()      # double root in [0, 1]
            s = rng.random() * 2 - 0.5
            c = np.array([-r * r * s, r * r + 2 * r * s, -(2 * r + s), 1.0])
        elif k == 4:
            c[0] = 0.0            # root at 0
        cs.append(c)
    return np.array(cs)


def main():
    from oracle import oracle as O
    rng = np.random.default_rng(20240601)
    coefs = cubic_cases(rng, 3000)
    if O.ref_cubic_roots(coefs[0]) is None:
        raise SystemExit("oracle/_ref/libref_cubic.so missing: build with `make -C oracle` where the reference exists")
    nr = np.zeros(len(coefs), np.int32)
    roots = np.full((len(coefs), 3), np.nan)
    for i, c in enumerate(coefs):
        r = O.ref_cubic_roots(c)
        nr[i] = len(r)
        roots[i, :len(r)] = r
    np.savez_compressed(os.path.join(HERE, "cubic_roots.npz"), coefs=coefs, nroots=nr, roots=roots)

    rng = np.random.default_rng(7)
    n = 1000
    toi = rng.random(n)
    pts = rng.random((n, 4, 3))
    p1 = pts[:, 2] / toi[:, None] - pts[:, 0] * ((1 - toi) / toi)[:, None]
    np.savez_compressed(os.path.join(HERE, "pt_toi_known.npz"), p0=pts[:, 0], tri=pts[:, 1:], p1=p1, toi=toi)

    rng = np.random.default_rng(11)
    a = rng.random((80, 3, 3))
    b = rng.random((80, 3, 3))
    w = rng.random(80)
    det0 = np.linalg.det(b)
    det1 = np.linalg.det(a + b)
    detw = np.linalg.det(a * w[:, None, None] + b)
    np.savez_compressed(os.path.join(HERE, "det_poly.npz"), a=a, b=b, w=w, det0=det0, det1=det1, detw=detw)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
