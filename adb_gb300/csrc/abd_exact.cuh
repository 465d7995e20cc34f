// Exact-order FP64 geometry of the contact path: vertex projection, AABBs, distance
// types and distances, the coplanarity cubic of the CCD and its root finder.
//
// The pair sets, their distance types and the time of impact must be bit-identical
// to the CPU restatement of the reference. Every operation below is therefore spelled
// out in a fixed order with non-contracting IEEE intrinsics (__dmul_rn / __dadd_rn /
// __ddiv_rn / __dsqrt_rn never fuse into FMA), so the device produces exactly the
// IEEE-754 results of the same expression sequence evaluated without contraction.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace abd {

#ifdef __CUDA_ARCH__
#define XM(a, b) __dmul_rn((a), (b))
#define XA(a, b) __dadd_rn((a), (b))
#define XS(a, b) __dsub_rn((a), (b))
#define XD(a, b) __ddiv_rn((a), (b))
#define XSQRT(a) __dsqrt_rn(a)
#else
#define XM(a, b) ((a) * (b))
#define XA(a, b) ((a) + (b))
#define XS(a, b) ((a) - (b))
#define XD(a, b) ((a) / (b))
#define XSQRT(a) sqrt(a)
#endif
#define HD __host__ __device__ __forceinline__

struct d3 {
  double x, y, z;
};
HD d3 mk(double x, double y, double z) { return d3{x, y, z}; }
HD d3 add(d3 a, d3 b) { return mk(XA(a.x, b.x), XA(a.y, b.y), XA(a.z, b.z)); }
HD d3 sub(d3 a, d3 b) { return mk(XS(a.x, b.x), XS(a.y, b.y), XS(a.z, b.z)); }
HD d3 scl(double s, d3 a) { return mk(XM(s, a.x), XM(s, a.y), XM(s, a.z)); }
HD d3 dvs(d3 a, double s) { return mk(XD(a.x, s), XD(a.y, s), XD(a.z, s)); }
HD double dot(d3 a, d3 b) { return XA(XA(XM(a.x, b.x), XM(a.y, b.y)), XM(a.z, b.z)); }
HD d3 cross(d3 a, d3 b) {
  return mk(XS(XM(a.y, b.z), XM(a.z, b.y)), XS(XM(a.z, b.x), XM(a.x, b.z)), XS(XM(a.x, b.y), XM(a.y, b.x)));
}
HD double sqn(d3 a) { return dot(a, a); }
HD double nrm(d3 a) { return XSQRT(sqn(a)); }
HD double dmin(double a, double b) { return b < a ? b : a; }
HD double dmax(double a, double b) { return a < b ? b : a; }
HD d3 vmin(d3 a, d3 b) { return mk(dmin(a.x, b.x), dmin(a.y, b.y), dmin(a.z, b.z)); }
HD d3 vmax(d3 a, d3 b) { return mk(dmax(a.x, b.x), dmax(a.y, b.y), dmax(a.z, b.z)); }
HD double comp(d3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

struct box {
  d3 lo, hi;
};
HD bool overlaps(const box& a, const box& b) {
  return a.lo.x <= b.hi.x && a.hi.x >= b.lo.x && a.lo.y <= b.hi.y && a.hi.y >= b.lo.y && a.lo.z <= b.hi.z &&
         a.hi.z >= b.lo.z;
}
HD bool intersection(const box& a, const box& b, box& o) {
  o.lo = vmax(a.lo, b.lo);
  o.hi = vmin(a.hi, b.hi);
  return o.lo.x <= o.hi.x && o.lo.y <= o.hi.y && o.lo.z <= o.hi.z;
}
HD box merge(const box& a, const box& b) { return box{vmin(a.lo, b.lo), vmax(a.hi, b.hi)}; }
HD box box2(d3 a, d3 b) { return box{vmin(a, b), vmax(a, b)}; }
HD box box3(d3 a, d3 b, d3 c) { return box{vmin(vmin(a, b), c), vmax(vmax(a, b), c)}; }
HD box box4(d3 a, d3 b, d3 c, d3 d) { return box{vmin(vmin(vmin(a, b), c), d), vmax(vmax(vmax(a, b), c), d)}; }
HD box inflate(const box& b, double r) {
  return box{mk(XS(b.lo.x, r), XS(b.lo.y, r), XS(b.lo.z, r)), mk(XA(b.hi.x, r), XA(b.hi.y, r), XA(b.hi.z, r))};
}

// x = A xbar + p, row r: ((a1_r x0 + a2_r x1) + a3_r x2) + p_r  (q = [p, a1, a2, a3]).
HD d3 project(const double* q, double x0, double x1, double x2) {
  double o[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) o[r] = XA(XA(XA(XM(q[3 + r], x0), XM(q[6 + r], x1)), XM(q[9 + r], x2)), q[r]);
  return mk(o[0], o[1], o[2]);
}

// Transformed AABB of a rest box (the 8 corners mapped by A, then translated).
HD box affine_box(const box& r, const double* q) {
  d3 lo = mk(0, 0, 0), hi = mk(0, 0, 0);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    int i = (c >> 2) & 1, j = (c >> 1) & 1, k = c & 1;
    double c0 = i ? r.hi.x : r.lo.x, c1 = j ? r.hi.y : r.lo.y, c2 = k ? r.hi.z : r.lo.z;
    double p[3];
#pragma unroll
    for (int row = 0; row < 3; ++row) p[row] = XA(XA(XM(q[3 + row], c0), XM(q[6 + row], c1)), XM(q[9 + row], c2));
    d3 pv = mk(p[0], p[1], p[2]);
    if (c == 0) {
      lo = pv;
      hi = pv;
    } else {
      lo = vmin(lo, pv);
      hi = vmax(hi, pv);
    }
  }
  d3 t = mk(q[0], q[1], q[2]);
  return box{add(lo, t), add(hi, t)};
}

// ---------------------------------------------------------------------------------
// Distance types (ipc-toolkit enum order).
enum { P_T0 = 0, P_T1, P_T2, P_E0, P_E1, P_E2, P_T };
enum { EA0_EB0 = 0, EA0_EB1, EA1_EB0, EA1_EB1, EA_EB0, EA_EB1, EA0_EB, EA1_EB, EA_EB };

// [a b; b c] x = r by diagonally pivoted LDL^T.
HD void solve2_ldlt(double a, double b, double c, double r0, double r1, double& x0, double& x1) {
  bool swp = fabs(c) > fabs(a);
  double m00 = swp ? c : a, m11 = swp ? a : c, m10 = b;
  double y0 = swp ? r1 : r0, y1 = swp ? r0 : r1;
  double l = (m00 != 0.0) ? XD(m10, m00) : m10;
  double d0 = m00;
  double d1 = XS(m11, XM(l, XM(m00, l)));
  y1 = XS(y1, XM(l, y0));
  const double tiny = 2.2250738585072014e-308;
  y0 = (fabs(d0) > tiny) ? XD(y0, d0) : 0.0;
  y1 = (fabs(d1) > tiny) ? XD(y1, d1) : 0.0;
  y0 = XS(y0, XM(l, y1));
  x0 = swp ? y1 : y0;
  x1 = swp ? y0 : y1;
}

HD int pt_type(d3 p, d3 t0, d3 t1, d3 t2) {
  d3 n = cross(sub(t1, t0), sub(t2, t0));
  double s[3], h[3];
  d3 o[3] = {t0, t1, t2};
  d3 e[3] = {t1, t2, t0};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    d3 b0 = sub(e[k], o[k]);
    d3 b1 = cross(b0, n);
    d3 r = sub(p, o[k]);
    solve2_ldlt(dot(b0, b0), dot(b0, b1), dot(b1, b1), dot(b0, r), dot(b1, r), s[k], h[k]);
    if (s[k] > 0.0 && s[k] < 1.0 && h[k] >= 0.0) return P_E0 + k;
  }
  if (s[0] <= 0.0 && s[2] >= 1.0) return P_T0;
  if (s[1] <= 0.0 && s[0] >= 1.0) return P_T1;
  if (s[2] <= 0.0 && s[1] >= 1.0) return P_T2;
  return P_T;
}

HD double pp_dist(d3 a, d3 b) { return sqn(sub(b, a)); }
HD double pl_dist(d3 p, d3 e0, d3 e1) { return XD(sqn(cross(sub(e0, p), sub(e1, p))), sqn(sub(e1, e0))); }
HD double plane_dist(d3 p, d3 t0, d3 t1, d3 t2) {
  d3 n = cross(sub(t1, t0), sub(t2, t0));
  double s = dot(sub(p, t0), n);
  return XD(XM(s, s), sqn(n));
}
HD double ll_dist(d3 a0, d3 a1, d3 b0, d3 b1) {
  d3 n = cross(sub(a1, a0), sub(b1, b0));
  double s = dot(sub(b0, a0), n);
  return XD(XM(s, s), sqn(n));
}
HD double pt_dist(d3 p, d3 t0, d3 t1, d3 t2, int ty) {
  switch (ty) {
    case P_T0: return pp_dist(p, t0);
    case P_T1: return pp_dist(p, t1);
    case P_T2: return pp_dist(p, t2);
    case P_E0: return pl_dist(p, t0, t1);
    case P_E1: return pl_dist(p, t1, t2);
    case P_E2: return pl_dist(p, t2, t0);
    default: return plane_dist(p, t0, t1, t2);
  }
}

HD int ee_parallel_type(d3 a0, d3 a1, d3 b0, d3 b1) {
  d3 ea = sub(a1, a0);
  double l2 = sqn(ea);
  double alpha = XD(dot(sub(b0, a0), ea), l2);
  double beta = XD(dot(sub(b1, a0), ea), l2);
  int eac, ebc;
  if (alpha < 0) {
    eac = (0 <= beta && beta <= 1) ? 2 : 0;
    ebc = (beta <= alpha) ? 0 : (beta <= 1 ? 1 : 2);
  } else if (alpha > 1) {
    eac = (0 <= beta && beta <= 1) ? 2 : 1;
    ebc = (beta >= alpha) ? 0 : (0 <= beta ? 1 : 2);
  } else {
    eac = 2;
    ebc = 0;
  }
  return ebc < 2 ? ((eac << 1) | ebc) : (6 + eac);
}

HD int ee_type(d3 a0, d3 a1, d3 b0, d3 b1) {
  d3 u = sub(a1, a0), v = sub(b1, b0), w = sub(a0, b0);
  double a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w), e = dot(v, w);
  double D = XS(XM(a, c), XM(b, b));
  if (a == 0.0 && c == 0.0) return EA0_EB0;
  if (a == 0.0) return EA0_EB;
  if (c == 0.0) return EA_EB0;
  double ac = XM(a, c);
  double tol = XM(1.0e-20, (ac > 1.0 ? ac : 1.0));
  if (sqn(cross(u, v)) < tol) return ee_parallel_type(a0, a1, b0, b1);
  int def = EA_EB;
  double sN = XS(XM(b, e), XM(c, d)), tN, tD;
  if (sN <= 0.0) {
    tN = e;
    tD = c;
    def = EA0_EB;
  } else if (sN >= D) {
    tN = XA(e, b);
    tD = c;
    def = EA1_EB;
  } else {
    tN = XS(XM(a, e), XM(b, d));
    tD = D;
  }
  if (tN <= 0.0) {
    if (-d <= 0.0) return EA0_EB0;
    if (-d >= a) return EA1_EB0;
    return EA_EB0;
  } else if (tN >= tD) {
    if (XA(-d, b) <= 0.0) return EA0_EB1;
    if (XA(-d, b) >= a) return EA1_EB1;
    return EA_EB1;
  }
  return def;
}

HD double ee_dist(d3 a0, d3 a1, d3 b0, d3 b1, int ty) {
  switch (ty) {
    case EA0_EB0: return pp_dist(a0, b0);
    case EA0_EB1: return pp_dist(a0, b1);
    case EA1_EB0: return pp_dist(a1, b0);
    case EA1_EB1: return pp_dist(a1, b1);
    case EA_EB0: return pl_dist(b0, a0, a1);
    case EA_EB1: return pl_dist(b1, a0, a1);
    case EA0_EB: return pl_dist(a0, b0, b1);
    case EA1_EB: return pl_dist(a1, b0, b1);
    default: return ll_dist(a0, a1, b0, b1);
  }
}

// ---------------------------------------------------------------------------------
// Cubic roots in [x0, x1] by Yuksel's isolate-then-Newton method (HPG 2022), as the
// reference uses it (cyCodeBase/cyPolynomial.h:787 with xError 6e-7). The bracketed
// refinement loop that the published method leaves unbounded is capped here; the cap
// (1000 safeguarded steps) is far above the few dozen the method needs.
HD double poly3(const double* c, double x) {
  double r = c[3];
  r = XA(XM(r, x), c[2]);
  r = XA(XM(r, x), c[1]);
  r = XA(XM(r, x), c[0]);
  return r;
}
HD double poly2(const double* c, double x) {
  double r = c[2];
  r = XA(XM(r, x), c[1]);
  r = XA(XM(r, x), c[0]);
  return r;
}
HD bool diff_sign(double a, double b) { return (a < 0) != (b < 0); }
HD double sgn_mul(double v, double s) { return XM(v, (s < 0 ? -1.0 : 1.0)); }
HD double mn_(double a, double b) { return a <= b ? a : b; }
HD double mx_(double a, double b) { return a >= b ? a : b; }

HD double cubic_bracketed(const double* c, const double* dc, double x0, double x1, double y0, double xe) {
  double ep2 = XM(2.0, xe);
  double xr = XD(XA(x0, x1), 2.0);
  if (XS(x1, x0) <= ep2) return xr;
  double xr0 = xr;
  for (int it = 0; it < 16; ++it) {
    double xn = XS(xr, XD(poly3(c, xr), poly2(dc, xr)));
    xn = mn_(x1, mx_(x0, xn));
    if (fabs(XS(xr, xn)) <= xe) return xn;
    xr = xn;
  }
  if (!isfinite(xr)) xr = xr0;
  double yr = poly3(c, xr);
  double xb0 = x0, xb1 = x1;
  for (int guard = 0; guard < 1000; ++guard) {
    bool side = diff_sign(y0, yr);
    if (side) xb1 = xr;
    else xb0 = xr;
    double dy = poly2(dc, xr);
    double dx = XD(yr, dy);
    double xn = XS(xr, dx);
    if (xn > xb0 && xn < xb1) {
      double step = fabs(XS(xr, xn));
      xr = xn;
      if (step > xe) yr = poly3(c, xr);
      else break;
    } else {
      xr = XD(XA(xb0, xb1), 2.0);
      if (xr == xb0 || xr == xb1 || XS(xb1, xb0) <= ep2) break;
      yr = poly3(c, xr);
    }
  }
  return xr;
}

HD int quadratic_roots(double* roots, const double* q, double x0, double x1) {
  double c = q[0], b = q[1], a = q[2];
  double delta = XS(XM(b, b), XM(XM(4.0, a), c));
  if (delta > 0) {
    double d = XSQRT(delta);
    double qq = XM(-0.5, XA(b, sgn_mul(d, b)));
    double rv0 = XD(qq, a), rv1 = XD(c, qq);
    double r0 = mn_(rv0, rv1), r1 = mx_(rv0, rv1);
    int r0i = (r0 >= x0) & (r0 <= x1);
    int r1i = (r1 >= x0) & (r1 <= x1);
    roots[0] = r0;
    roots[r0i] = r1;
    return r0i + r1i;
  } else if (delta < 0) {
    return 0;
  }
  double r0 = XD(XM(-0.5, b), a);
  roots[0] = r0;
  return (r0 >= x0) & (r0 <= x1);
}

HD void deflate3(const double* c, double r, double* o) {
  o[2] = c[3];
  o[1] = XA(c[2], XM(r, o[2]));
  o[0] = XA(c[1], XM(r, o[1]));
}

HD int cubic_roots(double* roots, const double* c, double x0, double x1, double xe = 6e-7) {
  double y0 = poly3(c, x0), y1 = poly3(c, x1);
  double a = XM(c[3], 3.0), b2 = c[2], cc = c[1];
  double dc[3] = {cc, XM(2.0, b2), a};
  double delta = XS(XM(b2, b2), XM(a, cc));
  if (delta > 0) {
    double d2 = XSQRT(delta);
    double q = -XA(b2, sgn_mul(d2, b2));
    double rv0 = XD(q, a), rv1 = XD(cc, q);
    double xa = mn_(rv0, rv1), xb = mx_(rv0, rv1);
    if (diff_sign(y0, y1)) {
      if (xa >= x1 || xb <= x0 || (xa <= x0 && xb >= x1)) {
        roots[0] = cubic_bracketed(c, dc, x0, x1, y0, xe);
        return 1;
      }
    } else {
      if ((xa >= x1 || xb <= x0) || (xa <= x0 && xb >= x1)) return 0;
    }
    if (xa > x0) {
      double ya = poly3(c, xa);
      if (diff_sign(y0, ya)) {
        roots[0] = cubic_bracketed(c, dc, x0, xa, y0, xe);
        if (diff_sign(ya, y1) || (xb < x1 && diff_sign(ya, poly3(c, xb)))) {
          double dp[3];
          deflate3(c, roots[0], dp);
          return quadratic_roots(roots + 1, dp, xa, x1) + 1;
        }
        return 1;
      }
      if (xb < x1) {
        double yb = poly3(c, xb);
        if (diff_sign(ya, yb)) {
          roots[0] = cubic_bracketed(c, dc, xa, xb, ya, xe);
          if (diff_sign(yb, y1)) {
            double dp[3];
            deflate3(c, roots[0], dp);
            return quadratic_roots(roots + 1, dp, xb, x1) + 1;
          }
          return 1;
        }
        if (diff_sign(yb, y1)) {
          roots[0] = cubic_bracketed(c, dc, xb, x1, yb, xe);
          return 1;
        }
      } else {
        if (diff_sign(ya, y1)) {
          roots[0] = cubic_bracketed(c, dc, xa, x1, ya, xe);
          return 1;
        }
      }
    } else {
      double yb = poly3(c, xb);
      if (diff_sign(y0, yb)) {
        roots[0] = cubic_bracketed(c, dc, x0, xb, y0, xe);
        if (diff_sign(yb, y1)) {
          double dp[3];
          deflate3(c, roots[0], dp);
          return quadratic_roots(roots + 1, dp, xb, x1) + 1;
        }
        return 1;
      }
      if (diff_sign(yb, y1)) {
        roots[0] = cubic_bracketed(c, dc, xb, x1, yb, xe);
        return 1;
      }
    }
    return 0;
  }
  if (diff_sign(y0, y1)) {
    roots[0] = cubic_bracketed(c, dc, x0, x1, y0, xe);
    return 1;
  }
  return 0;
}

// Coplanarity cubic det[p1-p0, p2-p0, p3-p0](t) accumulated as the alternating sum of
// four 3x3 determinant polynomials (the expansion of the reference's det_polynomial).
HD void cubic_binomial(const double* a, const double* b, double* p) {
  p[0] = XA(p[0], XM(XM(b[0], b[1]), b[2]));
  p[1] = XA(p[1], XA(XA(XM(XM(a[0], b[1]), b[2]), XM(XM(b[0], b[1]), a[2])), XM(XM(b[0], a[1]), b[2])));
  p[2] = XA(p[2], XA(XA(XM(XM(a[0], a[1]), b[2]), XM(XM(b[0], a[1]), a[2])), XM(XM(a[0], b[1]), a[2])));
  p[3] = XA(p[3], XM(XM(a[0], a[1]), a[2]));
}
// a, b: 3x3 with column k = point k.
HD void det_polynomial(const d3* a, const d3* b, double* out) {
  double pos[4] = {0, 0, 0, 0}, neg[4] = {0, 0, 0, 0};
  // (row, col) triples: + (00,11,22) (01,12,20) (02,10,21); - (00,12,21) (01,10,22) (02,11,20)
  const int T[6][6] = {{0, 0, 1, 1, 2, 2}, {0, 1, 1, 2, 2, 0}, {0, 2, 1, 0, 2, 1},
                       {0, 0, 1, 2, 2, 1}, {0, 1, 1, 0, 2, 2}, {0, 2, 1, 1, 2, 0}};
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    double aa[3], bb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      aa[k] = comp(a[T[t][2 * k + 1]], T[t][2 * k]);
      bb[k] = comp(b[T[t][2 * k + 1]], T[t][2 * k]);
    }
    cubic_binomial(aa, bb, t < 3 ? pos : neg);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) out[i] = XS(pos[i], neg[i]);
}

HD int coplanar_roots(const d3* p0, const d3* p1, double* roots) {
  const int sel[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  double d[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    d3 a[3], b[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      b[j] = p0[sel[k][j]];
      a[j] = sub(p1[sel[k][j]], b[j]);
    }
    det_polynomial(a, b, d[k]);
  }
  double t[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) t[i] = XS(XA(XS(d[0][i], d[1][i]), d[2][i]), d[3][i]);
  return cubic_roots(roots, t, 0.0, 1.0);
}

HD double area(d3 a, d3 b, d3 c) { return nrm(cross(sub(c, a), sub(b, a))); }
HD bool inside(d3 t0, d3 t1, d3 t2, d3 v) {
  double a1 = area(t1, t0, t2);
  double a2 = XA(XA(area(t0, t1, v), area(t1, t2, v)), area(t2, t0, v));
  return a2 <= XA(a1, 1e-8);
}
HD d3 lerp(d3 p1, d3 p0, double t) {
  double s = XS(1.0, t);
  return mk(XA(XM(t, p1.x), XM(s, p0.x)), XA(XM(t, p1.y), XM(s, p0.y)), XA(XM(t, p1.z), XM(s, p0.z)));
}
HD bool verify_root_pt(d3 v_, d3 t0, d3 t1, d3 t2) {
  d3 n = cross(sub(t0, t1), sub(t0, t2));
  n = dvs(n, XSQRT(dot(n, n)));
  double d = dot(n, sub(v_, t0));
  d3 v = sub(v_, scl(d, n));
  return inside(t0, t1, t2, v);
}
HD bool ee_cross_test(d3 i0, d3 i1, d3 j0, d3 j1) {
  d3 vei = sub(i1, i0), vej0 = sub(j0, i0), vej1 = sub(j1, i0);
  return dot(cross(vei, vej0), cross(vei, vej1)) < 0.0;
}
HD bool verify_root_ee(d3 i0, d3 i1, d3 j0, d3 j1) { return ee_cross_test(i0, i1, j0, j1) && ee_cross_test(j0, j1, i0, i1); }

// First verified root of the point-triangle coplanarity cubic (1.0 if none).
HD double pt_collision_time(d3 p0, const d3* f0, d3 p1, const d3* f1) {
  d3 a[4] = {p0, f0[0], f0[1], f0[2]}, b[4] = {p1, f1[0], f1[1], f1[2]};
  double roots[3];
  int found = coplanar_roots(a, b, roots);
  bool ok = false;
  double root = 1.0;
  for (int i = 0; i < found && !ok; ++i) {
    root = roots[i];
    ok = verify_root_pt(lerp(p1, p0, root), lerp(f1[0], f0[0], root), lerp(f1[1], f0[1], root),
                        lerp(f1[2], f0[2], root));
  }
  return (found && ok) ? root : 1.0;
}
HD double ee_collision_time(const d3* ei0, const d3* ej0, const d3* ei1, const d3* ej1) {
  d3 a[4] = {ei0[0], ei0[1], ej0[0], ej0[1]}, b[4] = {ei1[0], ei1[1], ej1[0], ej1[1]};
  double roots[3];
  int found = coplanar_roots(a, b, roots);
  bool ok = false;
  double root = 1.0;
  for (int i = 0; i < found && !ok; ++i) {
    root = roots[i];
    ok = verify_root_ee(lerp(ei1[0], ei0[0], root), lerp(ei1[1], ei0[1], root), lerp(ej1[0], ej0[0], root),
                        lerp(ej1[1], ej0[1], root));
  }
  return (found && ok) ? root : 1.0;
}

}  // namespace abd
