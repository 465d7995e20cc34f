// CPU oracle — test infrastructure only. Nothing in the product links, imports or
// executes this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// use it as the checker.
//
// Small fixed-size linear algebra and the per-primitive geometry of the reference's
// contact path, restated in plain C++ (no Eigen). Every operation is written out in a
// fixed evaluation order and the file is compiled with -ffp-contract=off, so the
// functions whose results must agree bit for bit with the GPU path (vertex projection,
// AABBs, distance types and distances, the CCD polynomial and its root finder) produce
// the same IEEE-754 results as the CUDA kernels, which spell out the same order with
// non-contracting intrinsics.
#pragma once
#include <cmath>
#include <cstring>
#include <algorithm>

namespace orc {

struct V3 {
  double x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(double a, double b, double c) : x(a), y(b), z(c) {}
  double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(const V3& a, double s) { return V3(a.x / s, a.y / s, a.z / s); }
// (a0 b0 + a1 b1) + a2 b2
inline double dot(const V3& a, const V3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double sqnorm(const V3& a) { return dot(a, a); }
inline double norm(const V3& a) { return std::sqrt(sqnorm(a)); }
inline V3 normalized(const V3& a) { return a / norm(a); }
inline V3 vmin(const V3& a, const V3& b) { return V3(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)); }
inline V3 vmax(const V3& a, const V3& b) { return V3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)); }

// Dense small matrices, row-major.
template <int R, int C>
struct Mat {
  double a[R * C];
  Mat() { std::memset(a, 0, sizeof(a)); }
  double& operator()(int i, int j) { return a[i * C + j]; }
  double operator()(int i, int j) const { return a[i * C + j]; }
};
using M12 = Mat<12, 12>;
using V12 = Mat<12, 1>;

template <int R, int K, int C>
inline Mat<R, C> matmul(const Mat<R, K>& A, const Mat<K, C>& B) {
  Mat<R, C> out;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      double s = 0;
      for (int k = 0; k < K; ++k) s += A(i, k) * B(k, j);
      out(i, j) = s;
    }
  return out;
}
template <int R, int C>
inline Mat<C, R> transpose(const Mat<R, C>& A) {
  Mat<C, R> out;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) out(j, i) = A(i, j);
  return out;
}

// Axis-aligned box (bounds3 / lu of the reference: model/bounds3.h).
struct Box {
  V3 lo, hi;
};
// bounds3.h:52-59 `intersects`: closed-interval overlap on every axis.
inline bool intersects(const Box& a, const Box& b) {
  return a.lo.x <= b.hi.x && a.hi.x >= b.lo.x && a.lo.y <= b.hi.y && a.hi.y >= b.lo.y &&
         a.lo.z <= b.hi.z && a.hi.z >= b.lo.z;
}
// bounds3.h:61-69 `intersection`
inline bool intersection(const Box& a, const Box& b, Box& out) {
  out.lo = vmax(a.lo, b.lo);
  out.hi = vmin(a.hi, b.hi);
  return out.lo.x <= out.hi.x && out.lo.y <= out.hi.y && out.lo.z <= out.hi.z;
}
inline Box merge(const Box& a, const Box& b) { return Box{vmin(a.lo, b.lo), vmax(a.hi, b.hi)}; }
inline Box box_of(const V3& p0, const V3& p1) { return Box{vmin(p0, p1), vmax(p0, p1)}; }
inline Box box_of(const V3& p0, const V3& p1, const V3& p2) {
  return Box{vmin(vmin(p0, p1), p2), vmax(vmax(p0, p1), p2)};
}
inline Box box_of4(const V3& p0, const V3& p1, const V3& p2, const V3& p3) {
  return Box{vmin(vmin(vmin(p0, p1), p2), p3), vmax(vmax(vmax(p0, p1), p2), p3)};
}
inline Box inflate(const Box& b, double r) {
  return Box{V3(b.lo.x - r, b.lo.y - r, b.lo.z - r), V3(b.hi.x + r, b.hi.y + r, b.hi.z + r)};
}

// ---------------------------------------------------------------------------------
// Distance types (ipc-toolkit v1.2.1 enum order; python/bindings.cpp:53-76).
enum PTType { P_T0 = 0, P_T1, P_T2, P_E0, P_E1, P_E2, P_T };
enum EEType { EA0_EB0 = 0, EA0_EB1, EA1_EB0, EA1_EB1, EA_EB0, EA_EB1, EA0_EB, EA1_EB, EA_EB };

// Solves the symmetric 2x2 system [a b; b c] x = r with a diagonally pivoted LDL^T
// factorisation (the method Eigen's LDLT applies), in a fixed operation order.
inline void solve2_ldlt(double a, double b, double c, double r0, double r1, double& x0, double& x1) {
  bool swap = std::fabs(c) > std::fabs(a);
  double m00 = swap ? c : a, m11 = swap ? a : c, m10 = b;
  double y0 = swap ? r1 : r0, y1 = swap ? r0 : r1;
  double l = (m00 != 0.0) ? m10 / m00 : m10;
  double d0 = m00;
  double d1 = m11 - l * (m00 * l);
  y1 = y1 - l * y0;
  const double tiny = 2.2250738585072014e-308;
  y0 = (std::fabs(d0) > tiny) ? y0 / d0 : 0.0;
  y1 = (std::fabs(d1) > tiny) ? y1 / d1 : 0.0;
  y0 = y0 - l * y1;
  x0 = swap ? y1 : y0;
  x1 = swap ? y0 : y1;
}

// Point-triangle distance-type classification (ipc-toolkit v1.2.1
// distance/distance_type.cpp, called at model/geometry.cpp:108).
inline PTType pt_type(const V3& p, const V3& t0, const V3& t1, const V3& t2) {
  V3 n = cross(t1 - t0, t2 - t0);
  double s[3], h[3];
  const V3* o[3] = {&t0, &t1, &t2};
  const V3* e[3] = {&t1, &t2, &t0};
  for (int k = 0; k < 3; ++k) {
    V3 b0 = *e[k] - *o[k];
    V3 b1 = cross(b0, n);
    V3 r = p - *o[k];
    solve2_ldlt(dot(b0, b0), dot(b0, b1), dot(b1, b1), dot(b0, r), dot(b1, r), s[k], h[k]);
    if (s[k] > 0.0 && s[k] < 1.0 && h[k] >= 0.0) return PTType(P_E0 + k);
  }
  if (s[0] <= 0.0 && s[2] >= 1.0) return P_T0;
  if (s[1] <= 0.0 && s[0] >= 1.0) return P_T1;
  if (s[2] <= 0.0 && s[1] >= 1.0) return P_T2;
  return P_T;
}

inline double pp_dist(const V3& a, const V3& b) { return sqnorm(b - a); }
// |(e0 - p) x (e1 - p)|^2 / |e1 - e0|^2
inline double pl_dist(const V3& p, const V3& e0, const V3& e1) {
  return sqnorm(cross(e0 - p, e1 - p)) / sqnorm(e1 - e0);
}
inline double plane_dist(const V3& p, const V3& t0, const V3& t1, const V3& t2) {
  V3 n = cross(t1 - t0, t2 - t0);
  double s = dot(p - t0, n);
  return s * s / sqnorm(n);
}
inline double ll_dist(const V3& a0, const V3& a1, const V3& b0, const V3& b1) {
  V3 n = cross(a1 - a0, b1 - b0);
  double s = dot(b0 - a0, n);
  return s * s / sqnorm(n);
}
inline double pt_dist(const V3& p, const V3& t0, const V3& t1, const V3& t2, PTType ty) {
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

// Parallel-edge classification (ipc-toolkit v1.2.1 edge_edge_parallel_distance_type).
inline EEType ee_parallel_type(const V3& a0, const V3& a1, const V3& b0, const V3& b1) {
  V3 ea = a1 - a0;
  double l2 = sqnorm(ea);
  double alpha = dot(b0 - a0, ea) / l2;
  double beta = dot(b1 - a0, ea) / l2;
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
  return EEType(ebc < 2 ? ((eac << 1) | ebc) : (6 + eac));
}

// Edge-edge distance-type classification (ipc-toolkit v1.2.1, called at
// model/thread_local_culling.cpp:375 and model/abd.cpp:353).
inline EEType ee_type(const V3& a0, const V3& a1, const V3& b0, const V3& b1) {
  V3 u = a1 - a0, v = b1 - b0, w = a0 - b0;
  double a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w), e = dot(v, w);
  double D = a * c - b * b;
  if (a == 0.0 && c == 0.0) return EA0_EB0;
  if (a == 0.0) return EA0_EB;
  if (c == 0.0) return EA_EB0;
  double ac = a * c;
  double tol = 1.0e-20 * (ac > 1.0 ? ac : 1.0);
  if (sqnorm(cross(u, v)) < tol) return ee_parallel_type(a0, a1, b0, b1);
  EEType def = EA_EB;
  double sN = b * e - c * d, tN, tD;
  if (sN <= 0.0) {
    tN = e; tD = c; def = EA0_EB;
  } else if (sN >= D) {
    tN = e + b; tD = c; def = EA1_EB;
  } else {
    tN = a * e - b * d; tD = D;
  }
  if (tN <= 0.0) {
    if (-d <= 0.0) return EA0_EB0;
    if (-d >= a) return EA1_EB0;
    return EA_EB0;
  } else if (tN >= tD) {
    if (-d + b <= 0.0) return EA0_EB1;
    if (-d + b >= a) return EA1_EB1;
    return EA_EB1;
  }
  return def;
}

inline double ee_dist(const V3& a0, const V3& a1, const V3& b0, const V3& b1, EEType ty) {
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
// Cubic roots in [x0, x1] by C. Yuksel's isolate-then-Newton method ("High-Performance
// Polynomial Root Finding for Graphics", HPG 2022), as the reference calls it through
// cyCodeBase/cyPolynomial.h:787 (`cy::CubicRoots`, xError 6e-7 from :169,
// boundError=false). Restated here in its published steps; the operation order follows
// the published method so that the reference header, compiled from its own source,
// returns bit-identical roots (checked by the oracle tests).
inline double poly3(const double c[4], double x) {
  double r = c[3];
  r = r * x + c[2];
  r = r * x + c[1];
  r = r * x + c[0];
  return r;
}
inline double poly2(const double c[3], double x) {
  double r = c[2];
  r = r * x + c[1];
  r = r * x + c[0];
  return r;
}
inline bool diff_sign(double a, double b) { return (a < 0) != (b < 0); }
inline double sgn_mul(double v, double s) { return v * (s < 0 ? -1.0 : 1.0); }
inline double mn(double a, double b) { return a <= b ? a : b; }
inline double mx(double a, double b) { return a >= b ? a : b; }

// Single root bracketed in [x0, x1] (y0, y1 of different sign): Newton from the
// midpoint clamped to the bracket, then safeguarded Newton/bisection.
inline double cubic_bracketed(const double c[4], const double dc[3], double x0, double x1, double y0,
                              double y1, double xe) {
  (void)y1;
  double ep2 = 2 * xe;
  double xr = (x0 + x1) / 2;
  if (x1 - x0 <= ep2) return xr;
  double xr0 = xr;
  for (int it = 0; it < 16; ++it) {
    double xn = xr - poly3(c, xr) / poly2(dc, xr);
    xn = mn(x1, mx(x0, xn));
    if (std::fabs(xr - xn) <= xe) return xn;
    xr = xn;
  }
  if (!std::isfinite(xr)) xr = xr0;
  double yr = poly3(c, xr);
  double xb0 = x0, xb1 = x1;
  for (int guard = 0; guard < 100000; ++guard) {
    bool side = diff_sign(y0, yr);
    if (side) xb1 = xr; else xb0 = xr;
    double dy = poly2(dc, xr);
    double dx = yr / dy;
    double xn = xr - dx;
    if (xn > xb0 && xn < xb1) {
      double step = std::fabs(xr - xn);
      xr = xn;
      if (step > xe) yr = poly3(c, xr);
      else break;
    } else {
      xr = (xb0 + xb1) / 2;
      if (xr == xb0 || xr == xb1 || xb1 - xb0 <= ep2) break;
      yr = poly3(c, xr);
    }
  }
  return xr;
}

inline int quadratic_roots(double roots[2], const double q[3], double x0, double x1) {
  double c = q[0], b = q[1], a = q[2];
  double delta = b * b - 4 * a * c;
  if (delta > 0) {
    double d = std::sqrt(delta);
    double qq = -0.5 * (b + sgn_mul(d, b));
    double rv0 = qq / a, rv1 = c / qq;
    double r0 = mn(rv0, rv1), r1 = mx(rv0, rv1);
    int r0i = (r0 >= x0) & (r0 <= x1);
    int r1i = (r1 >= x0) & (r1 <= x1);
    roots[0] = r0;
    roots[r0i] = r1;
    return r0i + r1i;
  } else if (delta < 0) {
    return 0;
  }
  double r0 = -0.5 * b / a;
  roots[0] = r0;
  return (r0 >= x0) & (r0 <= x1);
}

inline int cubic_roots(double roots[3], const double c[4], double x0, double x1, double xe = 6e-7) {
  double y0 = poly3(c, x0), y1 = poly3(c, x1);
  double a = c[3] * 3, b2 = c[2], cc = c[1];
  double dc[3] = {cc, 2 * b2, a};
  double delta = b2 * b2 - a * cc;
  auto deflate = [&](double r, double out[3]) {
    out[2] = c[3];
    out[1] = c[2] + r * out[2];
    out[0] = c[1] + r * out[1];
  };
  if (delta > 0) {
    double d2 = std::sqrt(delta);
    double q = -(b2 + sgn_mul(d2, b2));
    double rv0 = q / a, rv1 = cc / q;
    double xa = mn(rv0, rv1), xb = mx(rv0, rv1);
    if (diff_sign(y0, y1)) {
      if (xa >= x1 || xb <= x0 || (xa <= x0 && xb >= x1)) {
        roots[0] = cubic_bracketed(c, dc, x0, x1, y0, y1, xe);
        return 1;
      }
    } else {
      if ((xa >= x1 || xb <= x0) || (xa <= x0 && xb >= x1)) return 0;
    }
    if (xa > x0) {
      double ya = poly3(c, xa);
      if (diff_sign(y0, ya)) {
        roots[0] = cubic_bracketed(c, dc, x0, xa, y0, ya, xe);
        if (diff_sign(ya, y1) || (xb < x1 && diff_sign(ya, poly3(c, xb)))) {
          double dp[3];
          deflate(roots[0], dp);
          return quadratic_roots(roots + 1, dp, xa, x1) + 1;
        }
        return 1;
      }
      if (xb < x1) {
        double yb = poly3(c, xb);
        if (diff_sign(ya, yb)) {
          roots[0] = cubic_bracketed(c, dc, xa, xb, ya, yb, xe);
          if (diff_sign(yb, y1)) {
            double dp[3];
            deflate(roots[0], dp);
            return quadratic_roots(roots + 1, dp, xb, x1) + 1;
          }
          return 1;
        }
        if (diff_sign(yb, y1)) {
          roots[0] = cubic_bracketed(c, dc, xb, x1, yb, y1, xe);
          return 1;
        }
      } else {
        if (diff_sign(ya, y1)) {
          roots[0] = cubic_bracketed(c, dc, xa, x1, ya, y1, xe);
          return 1;
        }
      }
    } else {
      double yb = poly3(c, xb);
      if (diff_sign(y0, yb)) {
        roots[0] = cubic_bracketed(c, dc, x0, xb, y0, yb, xe);
        if (diff_sign(yb, y1)) {
          double dp[3];
          deflate(roots[0], dp);
          return quadratic_roots(roots + 1, dp, xb, x1) + 1;
        }
        return 1;
      }
      if (diff_sign(yb, y1)) {
        roots[0] = cubic_bracketed(c, dc, xb, x1, yb, y1, xe);
        return 1;
      }
    }
    return 0;
  }
  if (diff_sign(y0, y1)) {
    roots[0] = cubic_bracketed(c, dc, x0, x1, y0, y1, xe);
    return 1;
  }
  return 0;
}

// ---------------------------------------------------------------------------------
// Coplanarity cubic (model/collision.cpp:107-178). a, b: column-major 3x3 given as
// columns; c(r, k) = column k, row r.
struct M3c {
  V3 col[3];
  double operator()(int r, int k) const { return col[k][r]; }
};
inline void cubic_binomial(const double a[3], const double b[3], double p[4]) {
  p[0] += b[0] * b[1] * b[2];
  p[1] += a[0] * b[1] * b[2] + b[0] * b[1] * a[2] + b[0] * a[1] * b[2];
  p[2] += a[0] * a[1] * b[2] + b[0] * a[1] * a[2] + a[0] * b[1] * a[2];
  p[3] += a[0] * a[1] * a[2];
}
inline void det_polynomial(const M3c& a, const M3c& b, double out[4]) {
  double pos[4] = {0, 0, 0, 0}, neg[4] = {0, 0, 0, 0};
  double t[2][3];
  auto run = [&](int r0, int c0, int r1, int c1, int r2, int c2, double* acc) {
    double aa[3] = {a(r0, c0), a(r1, c1), a(r2, c2)};
    double bb[3] = {b(r0, c0), b(r1, c1), b(r2, c2)};
    (void)t;
    cubic_binomial(aa, bb, acc);
  };
  run(0, 0, 1, 1, 2, 2, pos);
  run(0, 1, 1, 2, 2, 0, pos);
  run(0, 2, 1, 0, 2, 1, pos);
  run(0, 0, 1, 2, 2, 1, neg);
  run(0, 1, 1, 0, 2, 2, neg);
  run(0, 2, 1, 1, 2, 0, neg);
  for (int i = 0; i < 4; ++i) out[i] = pos[i] - neg[i];
}

// collision.cpp:222-257
inline int coplanar_roots(const V3 p0[4], const V3 p1[4], double roots[3]) {
  M3c b[4], a[4];
  const int sel[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  for (int k = 0; k < 4; ++k)
    for (int j = 0; j < 3; ++j) {
      b[k].col[j] = p0[sel[k][j]];
      a[k].col[j] = p1[sel[k][j]] - b[k].col[j];
    }
  double d[4][4];
  for (int k = 0; k < 4; ++k) det_polynomial(a[k], b[k], d[k]);
  double t[4];
  for (int i = 0; i < 4; ++i) t[i] = ((d[0][i] - d[1][i]) + d[2][i]) - d[3][i];
  return cubic_roots(roots, t, 0.0, 1.0);
}

inline double area(const V3& a, const V3& b, const V3& c) { return norm(cross(c - a, b - a)); }
// geometry.cpp:153-157
inline bool inside(const V3& t0, const V3& t1, const V3& t2, const V3& v) {
  double a1 = area(t1, t0, t2);
  double a2 = area(t0, t1, v) + area(t1, t2, v) + area(t2, t0, v);
  return a2 <= a1 + 1e-8;
}
inline V3 lerp(const V3& p1, const V3& p0, double t) { return t * p1 + (1 - t) * p0; }

// collision.cpp:179-186
inline bool verify_root_pt(const V3& v_, const V3& t0, const V3& t1, const V3& t2) {
  V3 n = cross(t0 - t1, t0 - t2);
  n = n / std::sqrt(dot(n, n));
  double d = dot(n, v_ - t0);
  V3 v = v_ - d * n;
  return inside(t0, t1, t2, v);
}
// collision.cpp:188-200
inline bool ee_cross_test(const V3& i0, const V3& i1, const V3& j0, const V3& j1) {
  V3 vei = i1 - i0, vej0 = j0 - i0, vej1 = j1 - i0;
  return dot(cross(vei, vej0), cross(vei, vej1)) < 0.0;
}
inline bool verify_root_ee(const V3& i0, const V3& i1, const V3& j0, const V3& j1) {
  return ee_cross_test(i0, i1, j0, j1) && ee_cross_test(j0, j1, i0, i1);
}

// collision.cpp:259-277: first verified root of the point-triangle coplanarity cubic.
inline double pt_collision_time(const V3& p0, const V3 f0[3], const V3& p1, const V3 f1[3]) {
  V3 a[4] = {p0, f0[0], f0[1], f0[2]}, b[4] = {p1, f1[0], f1[1], f1[2]};
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
// collision.cpp:279-297
inline double ee_collision_time(const V3 ei0[2], const V3 ej0[2], const V3 ei1[2], const V3 ej1[2]) {
  V3 a[4] = {ei0[0], ei0[1], ej0[0], ej0[1]}, b[4] = {ei1[0], ei1[1], ej1[0], ej1[1]};
  double roots[3];
  int found = coplanar_roots(a, b, roots);
  bool ok = false;
  double root = 1.0;
  for (int i = 0; i < found && !ok; ++i) {
    root = roots[i];
    ok = verify_root_ee(lerp(ei1[0], ei0[0], root), lerp(ei1[1], ei0[1], root),
                        lerp(ej1[0], ej0[0], root), lerp(ej1[1], ej0[1], root));
  }
  return (found && ok) ? root : 1.0;
}

}  // namespace orc
