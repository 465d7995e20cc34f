// Derivatives of the point-triangle / edge-edge friction force with respect to the
// configuration through its tangent frame and its multiplier, for the adjoint of a
// converged frame.
//
// The reference recomputes, at every Newton iterate, each pair's closest-point weights
// gamma and tangent basis P_k (Tk = P_k^T Gamma, model/pt_ipc.cpp:22-107,
// model/ee_ipc.cpp:21-118) and its multiplier lambda = -b'(d) 2 sqrt(d) (pt_ipc.cpp:105),
// and adds the friction force mu lambda f1(|u|)/|u| Tk^T u with u = Tk (x - x0)
// (model/friction.cpp:15-47). At the converged state x* the optimality condition
// therefore carries Tk(x*) and lambda(x*): its Jacobian is the friction Hessian with the
// frame held fixed (assembled with the barrier terms) plus the terms from d Tk / dx and
// d lambda / dx. The latter are computed here by forward-mode differentiation: the force
// is restated for a dual-number scalar, and one evaluation per vertex coordinate, with
// the tangent seeded on the positions the frame and multiplier read (x - x0 held at its
// value), gives one column of that extra Jacobian. The formulas are those of
// frame_pt / frame_ee (abd_ipc.cuh), pt_dist / ee_dist (abd_exact.cuh) and
// friction_2x2, written once for a dual-number scalar.
#pragma once
#include "abd_ipc.cuh"

namespace abd {
namespace fadj {

struct Dual {
  double v, d;
};
DEV Dual dc(double v) { return Dual{v, 0.0}; }
DEV Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
DEV Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
DEV Dual operator-(Dual a) { return Dual{-a.v, -a.d}; }
DEV Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + a.v * b.d}; }
DEV Dual operator/(Dual a, Dual b) { return Dual{a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
DEV Dual operator*(double s, Dual a) { return Dual{s * a.v, s * a.d}; }
DEV Dual dsqrt(Dual a) {
  const double r = sqrt(a.v);
  return Dual{r, r > 0.0 ? a.d / (2.0 * r) : 0.0};
}
DEV Dual dlog(Dual a) { return Dual{log(a.v), a.d / a.v}; }
DEV Dual dclamp01(Dual a) { return a.v < 0.0 ? dc(0.0) : (a.v > 1.0 ? dc(1.0) : a); }

struct V3 {
  Dual x, y, z;
};
DEV V3 vsub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
DEV V3 vadd(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
DEV V3 vscl(Dual s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
DEV Dual vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DEV V3 vcross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
DEV V3 vnormalized(V3 a) { return vscl(dc(1.0) / dsqrt(vdot(a, a)), a); }
DEV V3 vconst(double x, double y, double z) { return V3{dc(x), dc(y), dc(z)}; }

// [a b; b c] x = r (the closest-point normal equations; the forward pass solves the same
// system by a pivoted LDL^T, equal up to rounding)
DEV void solve2(Dual a, Dual b, Dual c, Dual r0, Dual r1, Dual& x0, Dual& x1) {
  const Dual det = a * c - b * b;
  x0 = (c * r0 - b * r1) / det;
  x1 = (a * r1 - b * r0) / det;
}

struct Frame {
  V3 c0, c1;
  Dual gam[4];
};

DEV void pp_basis(V3 p0, V3 p1, Frame& f) {
  V3 d = vsub(p1, p0);
  V3 cx = vcross(vconst(1, 0, 0), d), cy = vcross(vconst(0, 1, 0), d);
  if (vdot(cx, cx).v > vdot(cy, cy).v) {
    f.c0 = vnormalized(cx);
    f.c1 = vnormalized(vcross(d, cx));
  } else {
    f.c0 = vnormalized(cy);
    f.c1 = vnormalized(vcross(d, cy));
  }
}
DEV void pe_basis(V3 p, V3 e0, V3 e1, Frame& f) {
  V3 e = vsub(e1, e0);
  f.c0 = vnormalized(e);
  f.c1 = vnormalized(vcross(e, vsub(p, e0)));
}
DEV Dual pe_closest(V3 p, V3 e0, V3 e1) {
  V3 e = vsub(e1, e0);
  return vdot(vsub(p, e0), e) / vdot(e, e);
}

DEV void frame_pt(const V3* X, int ty, Frame& f) {
  Dual l0, l1;
  {
    V3 b0 = vsub(X[2], X[1]), b1 = vsub(X[3], X[1]), r = vsub(X[0], X[1]);
    solve2(vdot(b0, b0), vdot(b0, b1), vdot(b1, b1), vdot(b0, r), vdot(b1, r), l0, l1);
  }
  Dual tl[3] = {dc(1.0) - l0 - l1, l0, l1};
  {
    V3 e0 = vsub(X[2], X[1]);
    V3 n = vcross(e0, vsub(X[3], X[1]));
    f.c0 = vnormalized(e0);
    f.c1 = vnormalized(vcross(n, e0));
  }
  switch (ty) {
    case P_T0: pp_basis(X[0], X[1], f); tl[0] = dc(1); tl[1] = dc(0); tl[2] = dc(0); break;
    case P_T1: pp_basis(X[0], X[2], f); tl[0] = dc(0); tl[1] = dc(1); tl[2] = dc(0); break;
    case P_T2: pp_basis(X[0], X[3], f); tl[0] = dc(0); tl[1] = dc(0); tl[2] = dc(1); break;
    case P_E0: { Dual e = pe_closest(X[0], X[1], X[2]); tl[0] = dc(1) - e; tl[1] = e; tl[2] = dc(0); pe_basis(X[0], X[1], X[2], f); break; }
    case P_E1: { Dual e = pe_closest(X[0], X[2], X[3]); tl[0] = dc(0); tl[1] = dc(1) - e; tl[2] = e; pe_basis(X[0], X[2], X[3], f); break; }
    case P_E2: { Dual e = pe_closest(X[0], X[3], X[1]); tl[0] = e; tl[1] = dc(0); tl[2] = dc(1) - e; pe_basis(X[0], X[3], X[1], f); break; }
    default: break;
  }
  f.gam[0] = dc(-1.0);
  f.gam[1] = tl[0];
  f.gam[2] = tl[1];
  f.gam[3] = tl[2];
}

DEV void frame_ee(const V3* X, int ty, Frame& f) {
  Dual s, t;
  {
    V3 w = vsub(X[0], X[2]), ea = vsub(X[1], X[0]), eb = vsub(X[3], X[2]);
    solve2(vdot(ea, ea), -vdot(eb, ea), vdot(eb, eb), -vdot(w, ea), vdot(w, eb), s, t);
  }
  {
    V3 ea = vsub(X[1], X[0]);
    V3 n = vcross(ea, vsub(X[3], X[2]));
    f.c0 = vnormalized(ea);
    f.c1 = vnormalized(vcross(n, ea));
  }
  switch (ty) {
    case EA0_EB0: pp_basis(X[0], X[2], f); s = dc(0); t = dc(0); break;
    case EA0_EB1: pp_basis(X[0], X[3], f); s = dc(0); t = dc(1); break;
    case EA1_EB0: pp_basis(X[1], X[2], f); s = dc(1); t = dc(0); break;
    case EA1_EB1: pp_basis(X[1], X[3], f); s = dc(1); t = dc(1); break;
    case EA_EB0: s = pe_closest(X[2], X[0], X[1]); t = dc(0); pe_basis(X[2], X[0], X[1], f); break;
    case EA_EB1: s = pe_closest(X[3], X[0], X[1]); t = dc(1); pe_basis(X[3], X[0], X[1], f); break;
    case EA0_EB: s = dc(0); t = pe_closest(X[0], X[2], X[3]); pe_basis(X[0], X[2], X[3], f); break;
    case EA1_EB: s = dc(1); t = pe_closest(X[1], X[2], X[3]); pe_basis(X[1], X[2], X[3], f); break;
    default: break;
  }
  s = dclamp01(s);
  t = dclamp01(t);
  f.gam[0] = -(dc(1) - s);
  f.gam[1] = -s;
  f.gam[2] = dc(1) - t;
  f.gam[3] = t;
}

DEV Dual pp_dist(V3 a, V3 b) {
  V3 d = vsub(b, a);
  return vdot(d, d);
}
DEV Dual pl_dist(V3 p, V3 e0, V3 e1) {
  V3 c = vcross(vsub(e0, p), vsub(e1, p)), e = vsub(e1, e0);
  return vdot(c, c) / vdot(e, e);
}
DEV Dual plane_dist(V3 p, V3 t0, V3 t1, V3 t2) {
  V3 n = vcross(vsub(t1, t0), vsub(t2, t0));
  Dual s = vdot(vsub(p, t0), n);
  return s * s / vdot(n, n);
}
DEV Dual ll_dist(V3 a0, V3 a1, V3 b0, V3 b1) {
  V3 n = vcross(vsub(a1, a0), vsub(b1, b0));
  Dual s = vdot(vsub(b0, a0), n);
  return s * s / vdot(n, n);
}
DEV Dual pair_dist(int kind, int ty, const V3* X) {
  if (kind == 0) {
    switch (ty) {
      case P_T0: return pp_dist(X[0], X[1]);
      case P_T1: return pp_dist(X[0], X[2]);
      case P_T2: return pp_dist(X[0], X[3]);
      case P_E0: return pl_dist(X[0], X[1], X[2]);
      case P_E1: return pl_dist(X[0], X[2], X[3]);
      case P_E2: return pl_dist(X[0], X[3], X[1]);
      default: return plane_dist(X[0], X[1], X[2], X[3]);
    }
  }
  switch (ty) {
    case EA0_EB0: return pp_dist(X[0], X[2]);
    case EA0_EB1: return pp_dist(X[0], X[3]);
    case EA1_EB0: return pp_dist(X[1], X[2]);
    case EA1_EB1: return pp_dist(X[1], X[3]);
    case EA_EB0: return pl_dist(X[2], X[0], X[1]);
    case EA_EB1: return pl_dist(X[3], X[0], X[1]);
    case EA0_EB: return pl_dist(X[0], X[2], X[3]);
    case EA1_EB: return pl_dist(X[1], X[2], X[3]);
    default: return ll_dist(X[0], X[1], X[2], X[3]);
  }
}

// b'(d) of the barrier (barrier.cpp:11-28)
DEV Dual barrier_b1(Dual x, double dhat, double kappa) {
  if (x.v >= dhat) return dc(0.0);
  return -(kappa / (dhat * dhat)) * ((x - dc(dhat)) * (2.0 * dlog(x / dc(dhat)) + (x - dc(dhat)) / x));
}

// Friction force on the pair's four vertices (g[i] = gamma_i F) with the frame and the
// multiplier evaluated at X and the tangent displacement at du = x - x0.
DEV void friction_force(int kind, int ty, const V3* X, const d3* du, double dhat, double kappa, double mu,
                        double epsv, V3* g) {
  Frame fr;
  if (kind == 0) frame_pt(X, ty, fr);
  else frame_ee(X, ty, fr);
  const Dual d = pair_dist(kind, ty, X);
  const Dual lam = -(2.0 * (barrier_b1(d, dhat, kappa) * dsqrt(d)));
  Dual u0 = dc(0.0), u1 = dc(0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    V3 dv = vconst(du[i].x, du[i].y, du[i].z);
    u0 = u0 + fr.gam[i] * vdot(fr.c0, dv);
    u1 = u1 + fr.gam[i] * vdot(fr.c1, dv);
  }
  const Dual uk = dsqrt(u0 * u0 + u1 * u1);
  // f1(x) / x (friction.cpp:24, ipc-toolkit f1_SF_over_x)
  const Dual f1x = uk.v >= epsv ? dc(1.0) / uk : (dc(2.0 * epsv) - uk) / dc(epsv * epsv);
  const Dual gs = mu * (lam * f1x);
  const V3 F = vadd(vscl(gs * u0, fr.c0), vscl(gs * u1, fr.c1));
#pragma unroll
  for (int i = 0; i < 4; ++i) g[i] = vscl(fr.gam[i], F);
}

// Column k (vertex k / 3, coordinate k % 3) of the force's Jacobian through its frame and
// multiplier: d g / d x_k with x - x0 held fixed.
DEV void frame_jacobian_column(int kind, int ty, const d3* X, const d3* du, double dhat, double kappa, double mu,
                               double epsv, int k, double* col) {
  V3 Xd[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    Xd[i] = vconst(X[i].x, X[i].y, X[i].z);
    if (i == k / 3) {
      const int r = k % 3;
      if (r == 0) Xd[i].x.d = 1.0;
      else if (r == 1) Xd[i].y.d = 1.0;
      else Xd[i].z.d = 1.0;
    }
  }
  V3 g[4];
  friction_force(kind, ty, Xd, du, dhat, kappa, mu, epsv, g);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    col[3 * i] = g[i].x.d;
    col[3 * i + 1] = g[i].y.d;
    col[3 * i + 2] = g[i].z.d;
  }
}

}  // namespace fadj
}  // namespace abd
