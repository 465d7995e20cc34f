// CPU oracle — test infrastructure only (see oracle_math.h header).
//
// Per-pair IPC terms restated from the reference and from the published IPC
// formulation of ipc-toolkit v1.2.1 (the reference fetches it at configure time,
// CMakeLists.txt:24-31; it is not vendored). Everything here is explicit 12x12
// vertex-space algebra: distance gradients/Hessians, the log barrier, the EE
// mollifier, a cyclic-Jacobi eigen projection to PSD, lagged friction and the chain
// rule onto the 12 affine DOFs of each body.
#pragma once
#include "oracle_math.h"

namespace orc {

struct BarrierParams {
  double dhat, kappa;
};

// model/barrier.cpp:11-28 (b, b'' and b' on the squared distance).
inline double barrier(double d, const BarrierParams& p) {
  if (d >= p.dhat) return 0.0;
  return p.kappa * -(d - p.dhat) * (d - p.dhat) * std::log(d / p.dhat) / (p.dhat * p.dhat);
}
inline double barrier_d2(double d, const BarrierParams& p) {
  if (d >= p.dhat) return 0.0;
  double dh = p.dhat;
  return -p.kappa * (2 * std::log(d / dh) + (d - dh) / d + (d - dh) * (2 / d + dh / d / d)) / (dh * dh);
}
inline double barrier_d1(double x, const BarrierParams& p) {
  if (x >= p.dhat) return 0.0;
  double dh = p.dhat;
  return -(x - dh) * p.kappa * (2 * std::log(x / dh) + (x - dh) / x) / (dh * dh);
}

// ---------------------------------------------------------------------------------
// Distance derivatives. Each distance type is the squared norm of
//   w(x, beta) = sum_i c_i(beta) x_i     (c affine in the m closest-point parameters)
// minimised over beta. With phi = |w|^2 and beta* the interior minimiser,
//   grad d = phi_x,   hess d = phi_xx - phi_xb phi_bb^{-1} phi_bx      (Schur complement)
// where phi_xx = 2 (c c^T (x) I3), phi_bb = 2 W^T W (W_k = dw/dbeta_k) and
// phi_x beta_k (point i) = 2 (c_i W_k + a_ik w), a_k = dc/dbeta_k.
struct DistStencil {
  int np;            // number of points involved (<= 4)
  int idx[4];        // which of the 4 pair points
  double c[4];       // coefficients c_i at the optimum
  int m;             // number of free parameters
  double a[2][4];    // dc/dbeta_k
};

// Builds gradient (12) and Hessian (12x12) of a squared distance from its stencil.
inline void stencil_derivs(const V3 X[4], const DistStencil& s, V12& g, M12& H) {
  V3 w;
  for (int i = 0; i < s.np; ++i) w = w + s.c[i] * X[s.idx[i]];
  V3 W[2];
  for (int k = 0; k < s.m; ++k)
    for (int i = 0; i < s.np; ++i) W[k] = W[k] + s.a[k][i] * X[s.idx[i]];
  g = V12();
  H = M12();
  for (int i = 0; i < s.np; ++i)
    for (int r = 0; r < 3; ++r) g(3 * s.idx[i] + r, 0) = 2 * s.c[i] * w[r];
  for (int i = 0; i < s.np; ++i)
    for (int j = 0; j < s.np; ++j)
      for (int r = 0; r < 3; ++r) H(3 * s.idx[i] + r, 3 * s.idx[j] + r) += 2 * s.c[i] * s.c[j];
  if (s.m == 0) return;
  // Phi (12 x m), G = 2 W^T W
  double Phi[12][2] = {};
  for (int k = 0; k < s.m; ++k)
    for (int i = 0; i < s.np; ++i)
      for (int r = 0; r < 3; ++r) Phi[3 * s.idx[i] + r][k] = 2 * (s.c[i] * W[k][r] + s.a[k][i] * w[r]);
  double G[2][2];
  for (int k = 0; k < s.m; ++k)
    for (int l = 0; l < s.m; ++l) G[k][l] = 2 * dot(W[k], W[l]);
  double Gi[2][2];
  if (s.m == 1) {
    Gi[0][0] = 1.0 / G[0][0];
  } else {
    double det = G[0][0] * G[1][1] - G[0][1] * G[1][0];
    Gi[0][0] = G[1][1] / det;
    Gi[1][1] = G[0][0] / det;
    Gi[0][1] = -G[0][1] / det;
    Gi[1][0] = -G[1][0] / det;
  }
  for (int p = 0; p < 12; ++p)
    for (int q = 0; q < 12; ++q) {
      double acc = 0;
      for (int k = 0; k < s.m; ++k)
        for (int l = 0; l < s.m; ++l) acc += Phi[p][k] * Gi[k][l] * Phi[q][l];
      H(p, q) -= acc;
    }
}

// Point-edge stencil: point P, segment (E0, E1); parameter s along the segment.
inline void pe_stencil(const V3 X[4], int P, int E0, int E1, DistStencil& s) {
  V3 e = X[E1] - X[E0];
  double t = dot(X[P] - X[E0], e) / sqnorm(e);
  s.np = 3;
  s.idx[0] = P; s.idx[1] = E0; s.idx[2] = E1;
  s.c[0] = 1; s.c[1] = -(1 - t); s.c[2] = -t;
  s.m = 1;
  s.a[0][0] = 0; s.a[0][1] = 1; s.a[0][2] = -1;
}
inline void pp_stencil(int P, int Q, DistStencil& s) {
  s.np = 2;
  s.idx[0] = P; s.idx[1] = Q;
  s.c[0] = 1; s.c[1] = -1;
  s.m = 0;
}

inline void pt_stencil(const V3 X[4], PTType ty, DistStencil& s) {
  switch (ty) {
    case P_T0: pp_stencil(0, 1, s); return;
    case P_T1: pp_stencil(0, 2, s); return;
    case P_T2: pp_stencil(0, 3, s); return;
    case P_E0: pe_stencil(X, 0, 1, 2, s); return;
    case P_E1: pe_stencil(X, 0, 2, 3, s); return;
    case P_E2: pe_stencil(X, 0, 3, 1, s); return;
    default: {
      V3 e1 = X[2] - X[1], e2 = X[3] - X[1], r = X[0] - X[1];
      double b1, b2;
      double g11 = dot(e1, e1), g12 = dot(e1, e2), g22 = dot(e2, e2);
      double det = g11 * g22 - g12 * g12;
      double r1 = dot(e1, r), r2 = dot(e2, r);
      b1 = (g22 * r1 - g12 * r2) / det;
      b2 = (g11 * r2 - g12 * r1) / det;
      s.np = 4;
      for (int i = 0; i < 4; ++i) s.idx[i] = i;
      s.c[0] = 1; s.c[1] = -(1 - b1 - b2); s.c[2] = -b1; s.c[3] = -b2;
      s.m = 2;
      double a0[4] = {0, 1, -1, 0}, a1[4] = {0, 1, 0, -1};
      for (int i = 0; i < 4; ++i) { s.a[0][i] = a0[i]; s.a[1][i] = a1[i]; }
    }
  }
}

inline void ee_stencil(const V3 X[4], EEType ty, DistStencil& s) {
  switch (ty) {
    case EA0_EB0: pp_stencil(0, 2, s); return;
    case EA0_EB1: pp_stencil(0, 3, s); return;
    case EA1_EB0: pp_stencil(1, 2, s); return;
    case EA1_EB1: pp_stencil(1, 3, s); return;
    case EA_EB0: pe_stencil(X, 2, 0, 1, s); return;
    case EA_EB1: pe_stencil(X, 3, 0, 1, s); return;
    case EA0_EB: pe_stencil(X, 0, 2, 3, s); return;
    case EA1_EB: pe_stencil(X, 1, 2, 3, s); return;
    default: {
      V3 u = X[1] - X[0], v = X[3] - X[2], w0 = X[0] - X[2];
      double a = dot(u, u), b = dot(u, v), c = dot(v, v), d = dot(u, w0), e = dot(v, w0);
      double D = a * c - b * b;
      double sp = (b * e - c * d) / D, tp = (a * e - b * d) / D;
      s.np = 4;
      for (int i = 0; i < 4; ++i) s.idx[i] = i;
      s.c[0] = 1 - sp; s.c[1] = sp; s.c[2] = -(1 - tp); s.c[3] = -tp;
      s.m = 2;
      double a0[4] = {-1, 1, 0, 0}, a1[4] = {0, 0, 1, -1};
      for (int i = 0; i < 4; ++i) { s.a[0][i] = a0[i]; s.a[1][i] = a1[i]; }
    }
  }
}

// ---------------------------------------------------------------------------------
// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major, in place:
// A becomes diagonal, V accumulates the rotations).
template <int N>
inline void jacobi_eig(double A[N][N], double V[N][N]) {
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        tot += A[i][j] * A[i][j];
        if (i != j) off += A[i][j] * A[i][j];
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < N - 1; ++p)
      for (int q = p + 1; q < N; ++q) {
        double apq = A[p][q];
        if (apq == 0.0) continue;
        double theta = (A[q][q] - A[p][p]) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < N; ++k) {
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < N; ++k) {
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < N; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
        A[p][q] = A[q][p] = 0.0;
      }
  }
}

// model/psd.h:5-33: nearest PSD matrix (negative eigenvalues clamped); returned
// unchanged when already PSD.
template <int N>
inline void project_psd(Mat<N, N>& M) {
  double A[N][N], V[N][N];
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) A[i][j] = 0.5 * (M(i, j) + M(j, i));
  jacobi_eig<N>(A, V);
  double lam[N];
  bool neg = false;
  for (int i = 0; i < N; ++i) {
    lam[i] = A[i][i];
    if (lam[i] < 0.0) neg = true;
  }
  if (!neg) return;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double s = 0;
      for (int k = 0; k < N; ++k)
        if (lam[k] > 0) s += V[i][k] * lam[k] * V[j][k];
      M(i, j) = s;
    }
}

// ---------------------------------------------------------------------------------
// Edge-edge mollifier (ipc-toolkit v1.2.1 edge_edge_mollifier*) on x = |ea x eb|^2.
inline void ee_mollifier(const V3 X[4], double eps_x, double& m, V12& gm, M12& Hm) {
  V3 u = X[1] - X[0], v = X[3] - X[2];
  double x = sqnorm(cross(u, v));
  gm = V12();
  Hm = M12();
  if (!(x < eps_x)) {
    m = 1.0;
    return;
  }
  double xe = x / eps_x;
  m = (-xe + 2.0) * xe;
  double m1 = 2.0 * (1.0 - xe) / eps_x;
  double m2 = -2.0 / (eps_x * eps_x);
  double uu = dot(u, u), vv = dot(v, v), uv = dot(u, v);
  V3 gu = 2.0 * (vv * u - uv * v), gv = 2.0 * (uu * v - uv * u);
  // dx/dpoints: ea0 = -gu, ea1 = gu, eb0 = -gv, eb1 = gv
  V12 gx;
  for (int r = 0; r < 3; ++r) {
    gx(r, 0) = -gu[r]; gx(3 + r, 0) = gu[r]; gx(6 + r, 0) = -gv[r]; gx(9 + r, 0) = gv[r];
  }
  // second derivatives in (u, v)
  double Huu[3][3] = {}, Hvv[3][3] = {}, Huv[3][3] = {};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double dij = (i == j) ? 1.0 : 0.0;
      Huu[i][j] = 2.0 * (vv * dij - v[i] * v[j]);
      Hvv[i][j] = 2.0 * (uu * dij - u[i] * u[j]);
      Huv[i][j] = 2.0 * (2.0 * u[i] * v[j] - v[i] * u[j] - uv * dij);
    }
  const double Da[4] = {-1, 1, 0, 0}, Db[4] = {0, 0, -1, 1};
  M12 Hx;
  for (int I = 0; I < 4; ++I)
    for (int J = 0; J < 4; ++J)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          Hx(3 * I + i, 3 * J + j) = Da[I] * Da[J] * Huu[i][j] + Db[I] * Db[J] * Hvv[i][j] +
                                     Da[I] * Db[J] * Huv[i][j] + Db[I] * Da[J] * Huv[j][i];
  for (int p = 0; p < 12; ++p) {
    gm(p, 0) = m1 * gx(p, 0);
    for (int q = 0; q < 12; ++q) Hm(p, q) = m2 * gx(p, 0) * gx(q, 0) + m1 * Hx(p, q);
  }
}

// ---------------------------------------------------------------------------------
// Smoothed friction (ipc-toolkit v1.2.1 friction/smooth_friction_mollifier).
inline double f0_SF(double x, double epsv) {
  if (std::fabs(x) >= epsv) return x;
  return x * x * (-x / (3 * epsv) + 1) / epsv + epsv / 3;
}
inline double f1_SF_over_x(double x, double epsv) {
  if (std::fabs(x) >= epsv) return 1 / x;
  return (-x + 2 * epsv) / (epsv * epsv);
}

struct FrictionParams {
  double mu, epsv, max_uk;
};

// model/friction.cpp:15-47. Tk is 12x2 (vertex or body space); adds into g, H.
template <int N>
inline void friction(const double uk2[2], double lam, const Mat<N, 2>& Tk, Mat<N, 1>& g, Mat<N, N>& H,
                     const FrictionParams& fp) {
  double uk = std::sqrt(uk2[0] * uk2[0] + uk2[1] * uk2[1]);
  double f1 = f1_SF_over_x(uk, fp.epsv);
  double s = fp.mu * lam * f1;
  for (int i = 0; i < N; ++i) g(i, 0) += s * (Tk(i, 0) * uk2[0] + Tk(i, 1) * uk2[1]);
  double M[2][2];
  if (uk >= fp.epsv) {
    double ut[2] = {-uk2[1], uk2[0]};
    double sc = fp.mu * lam * f1 / (uk * uk);
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) M[a][b] = sc * ut[a] * ut[b];
  } else if (uk <= fp.max_uk) {
    double sc = fp.mu * lam * f1;
    M[0][0] = sc; M[1][1] = sc; M[0][1] = M[1][0] = 0;
  } else {
    double f2 = -1.0 / (fp.epsv * fp.epsv);
    Mat<2, 2> m2;
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) m2(a, b) = f2 / uk * uk2[a] * uk2[b];
    m2(0, 0) += f1;
    m2(1, 1) += f1;
    for (int a = 0; a < 4; ++a) m2.a[a] *= fp.mu * lam;
    project_psd<2>(m2);
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) M[a][b] = m2(a, b);
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double acc = 0;
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) acc += Tk(i, a) * M[a][b] * Tk(j, b);
      H(i, j) += acc;
    }
}

// ---------------------------------------------------------------------------------
// Closest points and tangent bases (ipc-toolkit v1.2.1 friction/closest_point.cpp and
// friction/tangent_basis.cpp) used by model/pt_ipc.cpp:22-107, model/ee_ipc.cpp:21-118.
struct Basis32 {
  V3 c0, c1;
};
inline Basis32 pp_basis(const V3& p0, const V3& p1) {
  V3 d = p1 - p0;
  V3 cx = cross(V3(1, 0, 0), d), cy = cross(V3(0, 1, 0), d);
  Basis32 b;
  if (sqnorm(cx) > sqnorm(cy)) {
    b.c0 = normalized(cx);
    b.c1 = normalized(cross(d, cx));
  } else {
    b.c0 = normalized(cy);
    b.c1 = normalized(cross(d, cy));
  }
  return b;
}
inline Basis32 pe_basis(const V3& p, const V3& e0, const V3& e1) {
  V3 e = e1 - e0;
  Basis32 b;
  b.c0 = normalized(e);
  b.c1 = normalized(cross(e, p - e0));
  return b;
}
inline Basis32 pt_basis(const V3& p, const V3& t0, const V3& t1, const V3& t2) {
  (void)p;
  V3 e0 = t1 - t0;
  V3 n = cross(e0, t2 - t0);
  Basis32 b;
  b.c0 = normalized(e0);
  b.c1 = normalized(cross(n, e0));
  return b;
}
inline Basis32 ee_basis(const V3& a0, const V3& a1, const V3& b0, const V3& b1) {
  V3 ea = a1 - a0;
  V3 n = cross(ea, b1 - b0);
  Basis32 b;
  b.c0 = normalized(ea);
  b.c1 = normalized(cross(n, ea));
  return b;
}
inline double pe_closest(const V3& p, const V3& e0, const V3& e1) {
  V3 e = e1 - e0;
  return dot(p - e0, e) / sqnorm(e);
}
inline void pt_closest(const V3& p, const V3& t0, const V3& t1, const V3& t2, double& l0, double& l1) {
  V3 b0 = t1 - t0, b1 = t2 - t0, r = p - t0;
  solve2_ldlt(dot(b0, b0), dot(b0, b1), dot(b1, b1), dot(b0, r), dot(b1, r), l0, l1);
}
inline void ee_closest(const V3& a0, const V3& a1, const V3& b0, const V3& b1, double& s, double& t) {
  V3 w = a0 - b0, ea = a1 - a0, eb = b1 - b0;
  solve2_ldlt(sqnorm(ea), -dot(eb, ea), sqnorm(eb), -dot(w, ea), dot(w, eb), s, t);
}

// Friction frame of a PT pair (pt_ipc.cpp:22-107): Tk (2x12 vertex space) and the
// barycentric weights gamma of the relative tangential displacement.
inline void pt_frame(const V3 X[4], PTType ty, Mat<2, 12>& TkT) {
  double l0, l1;
  pt_closest(X[0], X[1], X[2], X[3], l0, l1);
  double tl[3] = {1 - l0 - l1, l0, l1};
  Basis32 P = pt_basis(X[0], X[1], X[2], X[3]);
  switch (ty) {
    case P_T0: P = pp_basis(X[0], X[1]); tl[0] = 1; tl[1] = 0; tl[2] = 0; break;
    case P_T1: P = pp_basis(X[0], X[2]); tl[0] = 0; tl[1] = 1; tl[2] = 0; break;
    case P_T2: P = pp_basis(X[0], X[3]); tl[0] = 0; tl[1] = 0; tl[2] = 1; break;
    case P_E0: { double e = pe_closest(X[0], X[1], X[2]); tl[0] = 1 - e; tl[1] = e; tl[2] = 0; P = pe_basis(X[0], X[1], X[2]); break; }
    case P_E1: { double e = pe_closest(X[0], X[2], X[3]); tl[0] = 0; tl[1] = 1 - e; tl[2] = e; P = pe_basis(X[0], X[2], X[3]); break; }
    case P_E2: { double e = pe_closest(X[0], X[3], X[1]); tl[0] = e; tl[1] = 0; tl[2] = 1 - e; P = pe_basis(X[0], X[3], X[1]); break; }
    default: break;
  }
  double gam[4] = {-1.0, tl[0], tl[1], tl[2]};
  TkT = Mat<2, 12>();
  for (int i = 0; i < 4; ++i)
    for (int r = 0; r < 3; ++r) {
      TkT(0, 3 * i + r) = P.c0[r] * gam[i];
      TkT(1, 3 * i + r) = P.c1[r] * gam[i];
    }
}

inline void ee_frame(const V3 X[4], EEType ty, Mat<2, 12>& TkT) {
  double s, t;
  ee_closest(X[0], X[1], X[2], X[3], s, t);
  Basis32 P = ee_basis(X[0], X[1], X[2], X[3]);
  switch (ty) {
    case EA0_EB0: P = pp_basis(X[0], X[2]); s = 0; t = 0; break;
    case EA0_EB1: P = pp_basis(X[0], X[3]); s = 0; t = 1; break;
    case EA1_EB0: P = pp_basis(X[1], X[2]); s = 1; t = 0; break;
    case EA1_EB1: P = pp_basis(X[1], X[3]); s = 1; t = 1; break;
    case EA_EB0: s = pe_closest(X[2], X[0], X[1]); t = 0; P = pe_basis(X[2], X[0], X[1]); break;
    case EA_EB1: s = pe_closest(X[3], X[0], X[1]); t = 1; P = pe_basis(X[3], X[0], X[1]); break;
    case EA0_EB: s = 0; t = pe_closest(X[0], X[2], X[3]); P = pe_basis(X[0], X[2], X[3]); break;
    case EA1_EB: s = 1; t = pe_closest(X[1], X[2], X[3]); P = pe_basis(X[1], X[2], X[3]); break;
    default: break;
  }
  s = std::max(std::min(1.0, s), 0.0);
  t = std::max(std::min(1.0, t), 0.0);
  double gam[4] = {-(1 - s), -s, 1 - t, t};
  TkT = Mat<2, 12>();
  for (int i = 0; i < 4; ++i)
    for (int r = 0; r < 3; ++r) {
      TkT(0, 3 * i + r) = P.c0[r] * gam[i];
      TkT(1, 3 * i + r) = P.c1[r] * gam[i];
    }
}

// ---------------------------------------------------------------------------------
// Vertex-space barrier Hessian/gradient of one pair (model/core_ipc.cpp:21-83).
inline void ipc_hess_pt(const V3 X[4], PTType ty, double d, const BarrierParams& bp, bool psd, M12& H,
                        V12& g) {
  DistStencil s;
  pt_stencil(X, ty, s);
  V12 gd;
  M12 Hd;
  stencil_derivs(X, s, gd, Hd);
  double B1 = barrier_d1(d, bp), B2 = barrier_d2(d, bp);
  for (int p = 0; p < 12; ++p) {
    g(p, 0) = gd(p, 0) * B1;
    for (int q = 0; q < 12; ++q) H(p, q) = Hd(p, q) * B1 + gd(p, 0) * gd(q, 0) * B2;
  }
  if (psd) project_psd<12>(H);
}

inline double ipc_hess_ee(const V3 X[4], EEType ty, double d, const BarrierParams& bp, double eps_x_param,
                          bool psd, M12& H, V12& g) {
  double eps_x = eps_x_param * sqnorm(X[0] - X[1]) * sqnorm(X[2] - X[3]);
  double m;
  V12 gm;
  M12 Hm;
  ee_mollifier(X, eps_x, m, gm, Hm);
  DistStencil s;
  ee_stencil(X, ty, s);
  V12 gd;
  M12 Hd;
  stencil_derivs(X, s, gd, Hd);
  double B1 = barrier_d1(d, bp), B2 = barrier_d2(d, bp), B = barrier(d, bp);
  for (int p = 0; p < 12; ++p) {
    g(p, 0) = m * gd(p, 0) * B1 + gm(p, 0) * B;
    for (int q = 0; q < 12; ++q)
      H(p, q) = Hm(p, q) * B + B1 * (gm(p, 0) * gd(q, 0) + gd(p, 0) * gm(q, 0)) +
                m * (B2 * gd(p, 0) * gd(q, 0) + B1 * Hd(p, q));
  }
  if (psd) project_psd<12>(H);
  return m;
}

}  // namespace orc
