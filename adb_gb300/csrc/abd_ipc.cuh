// Per-pair IPC terms on the device: barrier energy, gradient and PSD-projected Hessian
// of one point-triangle or edge-edge pair, lagged friction, and the chain rule onto the
// 12 affine DOFs of the two bodies.
//
// The reference forms the 12x12 vertex-space Hessian H = b'' g g^T + b' hess(d) (plus
// the edge-edge mollifier terms), projects it to PSD with a full eigen-decomposition
// (model/psd.h:5-33, called from model/core_ipc.cpp:40,79), adds friction
// (model/friction.cpp:15-47) and multiplies by the Jacobians of x = A xbar + p
// (model/pt_ipc.cpp:153-169, model/ee_ipc.cpp:180-196).
//
// Here the same quantities are built without ever forming H in vertex space. Every
// squared distance d(x) is invariant under a common translation of the four points,
// so H lives in the 9-dimensional translation-free subspace spanned by Q (x) I3 with
//   Q = [(1,-1,0,0)/sqrt2, (0,0,1,-1)/sqrt2, (1,1,-1,-1)/2]  (orthonormal, _|_ (1,1,1,1)).
// H is assembled directly as the 9x9 matrix S = (Q (x) I)^T H (Q (x) I) from its
// rank-structured pieces, S is eigen-projected (cyclic Jacobi), friction is added in
// the same coordinates (the friction stencil also sums to zero), and the body blocks are
// Y_A S Y_B^T with Y_b[k][a] = sum_{i on body b} xbar~_i[k] Q[i][a]. Because Q is
// orthonormal, projecting S is exactly projecting H (same eigenvalues, eigenvectors
// mapped by Q (x) I), so the result equals the reference's up to rounding.
#pragma once
#include "abd_exact.cuh"

namespace abd {

#define DEV __device__ __forceinline__

struct BarrierP {
  double dhat, kappa;
};

DEV double barrier_b(double d, const BarrierP& p) {
  if (d >= p.dhat) return 0.0;
  return p.kappa * -(d - p.dhat) * (d - p.dhat) * log(d / p.dhat) / (p.dhat * p.dhat);
}
DEV double barrier_b2(double d, const BarrierP& p) {
  if (d >= p.dhat) return 0.0;
  double dh = p.dhat;
  return -p.kappa * (2 * log(d / dh) + (d - dh) / d + (d - dh) * (2 / d + dh / d / d)) / (dh * dh);
}
DEV double barrier_b1(double x, const BarrierP& p) {
  if (x >= p.dhat) return 0.0;
  double dh = p.dhat;
  return -(x - dh) * p.kappa * (2 * log(x / dh) + (x - dh) / x) / (dh * dh);
}

DEV double f0_SF(double x, double epsv) {
  if (fabs(x) >= epsv) return x;
  return x * x * (-x / (3 * epsv) + 1) / epsv + epsv / 3;
}
DEV double f1_SF_over_x(double x, double epsv) {
  if (fabs(x) >= epsv) return 1 / x;
  return (-x + 2 * epsv) / (epsv * epsv);
}

// Squared-distance stencil: d = |w|^2, w = sum_i c_i x_i at the optimal closest-point
// parameters; a_k = dc/dbeta_k for the m free parameters.
struct Stencil {
  double c[4];
  double a[2][4];
  int m;
};

DEV d3 fd3(double x, double y, double z) { return d3{x, y, z}; }
DEV d3 fadd(d3 a, d3 b) { return fd3(a.x + b.x, a.y + b.y, a.z + b.z); }
DEV d3 fsub(d3 a, d3 b) { return fd3(a.x - b.x, a.y - b.y, a.z - b.z); }
DEV d3 fscl(double s, d3 a) { return fd3(s * a.x, s * a.y, s * a.z); }
DEV double fdot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
DEV d3 fcross(d3 a, d3 b) { return fd3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
DEV d3 fnormalized(d3 a) { return fscl(1.0 / sqrt(fdot(a, a)), a); }
DEV double c3(d3 a, int r) { return r == 0 ? a.x : (r == 1 ? a.y : a.z); }

DEV void st_clear(Stencil& s) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    s.c[i] = 0;
    s.a[0][i] = 0;
    s.a[1][i] = 0;
  }
  s.m = 0;
}
DEV void st_pp(int P, int Q_, Stencil& s) {
  st_clear(s);
  s.c[P] = 1;
  s.c[Q_] = -1;
}
DEV void st_pe(const d3* X, int P, int E0, int E1, Stencil& s) {
  st_clear(s);
  d3 e = fsub(X[E1], X[E0]);
  double t = fdot(fsub(X[P], X[E0]), e) / fdot(e, e);
  s.c[P] = 1;
  s.c[E0] = -(1 - t);
  s.c[E1] = -t;
  s.m = 1;
  s.a[0][E0] = 1;
  s.a[0][E1] = -1;
}
DEV void st_pt(const d3* X, int ty, Stencil& s) {
  switch (ty) {
    case P_T0: st_pp(0, 1, s); return;
    case P_T1: st_pp(0, 2, s); return;
    case P_T2: st_pp(0, 3, s); return;
    case P_E0: st_pe(X, 0, 1, 2, s); return;
    case P_E1: st_pe(X, 0, 2, 3, s); return;
    case P_E2: st_pe(X, 0, 3, 1, s); return;
    default: {
      st_clear(s);
      d3 e1 = fsub(X[2], X[1]), e2 = fsub(X[3], X[1]), r = fsub(X[0], X[1]);
      double g11 = fdot(e1, e1), g12 = fdot(e1, e2), g22 = fdot(e2, e2);
      double det = g11 * g22 - g12 * g12;
      double r1 = fdot(e1, r), r2 = fdot(e2, r);
      double b1 = (g22 * r1 - g12 * r2) / det, b2 = (g11 * r2 - g12 * r1) / det;
      s.c[0] = 1;
      s.c[1] = -(1 - b1 - b2);
      s.c[2] = -b1;
      s.c[3] = -b2;
      s.m = 2;
      s.a[0][1] = 1; s.a[0][2] = -1;
      s.a[1][1] = 1; s.a[1][3] = -1;
    }
  }
}
DEV void st_ee(const d3* X, int ty, Stencil& s) {
  switch (ty) {
    case EA0_EB0: st_pp(0, 2, s); return;
    case EA0_EB1: st_pp(0, 3, s); return;
    case EA1_EB0: st_pp(1, 2, s); return;
    case EA1_EB1: st_pp(1, 3, s); return;
    case EA_EB0: st_pe(X, 2, 0, 1, s); return;
    case EA_EB1: st_pe(X, 3, 0, 1, s); return;
    case EA0_EB: st_pe(X, 0, 2, 3, s); return;
    case EA1_EB: st_pe(X, 1, 2, 3, s); return;
    default: {
      st_clear(s);
      d3 u = fsub(X[1], X[0]), v = fsub(X[3], X[2]), w0 = fsub(X[0], X[2]);
      double a = fdot(u, u), b = fdot(u, v), c = fdot(v, v), d = fdot(u, w0), e = fdot(v, w0);
      double D = a * c - b * b;
      double sp = (b * e - c * d) / D, tp = (a * e - b * d) / D;
      s.c[0] = 1 - sp;
      s.c[1] = sp;
      s.c[2] = -(1 - tp);
      s.c[3] = -tp;
      s.m = 2;
      s.a[0][0] = -1; s.a[0][1] = 1;
      s.a[1][2] = 1; s.a[1][3] = -1;
    }
  }
}

// Q^T u for a 4-vector u.
DEV void qt4(const double* u, double* o) {
  const double r2 = 0.70710678118654752440;
  o[0] = (u[0] - u[1]) * r2;
  o[1] = (u[2] - u[3]) * r2;
  o[2] = 0.5 * ((u[0] + u[1]) - (u[2] + u[3]));
}
DEV double Qe(int i, int a) {
  const double r2 = 0.70710678118654752440;
  if (a == 0) return i == 0 ? r2 : (i == 1 ? -r2 : 0.0);
  if (a == 1) return i == 2 ? r2 : (i == 3 ? -r2 : 0.0);
  return i < 2 ? 0.5 : -0.5;
}

// Symmetric eigen-projection of an n x n matrix in place (cyclic Jacobi, n <= 9).
template <int N>
DEV void psd_project(double (&S)[N][N]) {
  double A[N][N], V[N][N];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) {
      A[i][j] = 0.5 * (S[i][j] + S[j][i]);
      V[i][j] = (i == j) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        double v = A[i][j] * A[i][j];
        tot += v;
        if (i != j) off += v;
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < N - 1; ++p)
      for (int q = p + 1; q < N; ++q) {
        double apq = A[p][q];
        if (apq == 0.0) continue;
        double theta = (A[q][q] - A[p][p]) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        double c = 1 / sqrt(t * t + 1), s = t * c;
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
        A[p][q] = 0.0;
        A[q][p] = 0.0;
      }
  }
  bool neg = false;
  double lam[N];
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
      S[i][j] = s;
    }
}

// The 9x9 projection of mollified edge-edge pairs, out of line: the rare path stays out of
// the register allocation of the kernels that contain it.
static __device__ __noinline__ void psd_project9(double (&S)[9][9]) { psd_project<9>(S); }

// Eigenvector estimate of a small symmetric matrix for psd_project_small: cyclic Jacobi
// in FP32 on a copy scaled to max |s_ij| = 1, until the off-diagonal mass is ~1e-6 of the
// total (FP32 rounding level), then the columns re-orthonormalised in FP64 by modified
// Gram-Schmidt. FP32 arithmetic runs at 64x the FP64 rate on this part, so the sweeps that
// bring a dense matrix close to diagonal cost little; the FP64 sweeps that follow start
// from off-diagonals ~1e-7 of the norm and, converging quadratically, stop after about
// two. Each column's norm^2 = 1 + e with |e| ~ 1e-7 is normalised by the Taylor series
// (1 + e)^(-1/2) = 1 - e/2 + 3e^2/8 - 5e^3/16 (remainder < 35 e^4 / 128). Returns false
// (Q untouched) for a zero, non-finite or out-of-FP32-range matrix, or a column whose
// norm is not within 1e-5 of 1; the caller then starts from the identity.
template <int N>
DEV bool jacobi_f32_start(const double (&S)[N][N], double (&Q)[N][N]) {
  float a[N][N], v[N][N];
  float mx = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      a[i][j] = __double2float_rn(S[i][j]);
      mx = fmaxf(mx, fabsf(a[i][j]));
    }
  if (!(mx > 1e-30f && mx < 1e30f)) return false;
  const float sc = 1.f / mx;
#pragma unroll
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int j = i; j < N; ++j) a[i][j] *= sc;
#pragma unroll
    for (int j = 0; j < N; ++j) v[i][j] = (i == j) ? 1.f : 0.f;
  }
  for (int sweep = 0; sweep < 8; ++sweep) {
    float off = 0.f, dg = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      dg += a[i][i] * a[i][i];
#pragma unroll
      for (int j = i + 1; j < N; ++j) off += a[i][j] * a[i][j];
    }
    if (off == 0.f || 2.f * off <= 1e-12f * (dg + 2.f * off)) break;
#pragma unroll
    for (int p = 0; p < N - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < N; ++q) {
        float apq = a[p][q];
        float h = 0.5f * (a[q][q] - a[p][p]);
        float den = apq != 0.f ? fabsf(h) + sqrtf(h * h + apq * apq) : 0.f;
        if (den > 0.f) {
          float t = __fdividef(h >= 0.f ? apq : -apq, den);
          float c = rsqrtf(1.f + t * t), s = t * c;
          a[p][p] -= t * apq;
          a[q][q] += t * apq;
#pragma unroll
          for (int k = 0; k < N; ++k) {
            if (k == p || k == q) continue;
            float akp = k < p ? a[k][p] : a[p][k];
            float akq = k < q ? a[k][q] : a[q][k];
            float np_ = c * akp - s * akq, nq = s * akp + c * akq;
            if (k < p) a[k][p] = np_;
            else a[p][k] = np_;
            if (k < q) a[k][q] = nq;
            else a[q][k] = nq;
          }
#pragma unroll
          for (int k = 0; k < N; ++k) {
            float vkp = v[k][p], vkq = v[k][q];
            v[k][p] = c * vkp - s * vkq;
            v[k][q] = s * vkp + c * vkq;
          }
        }
        a[p][q] = 0.f;
      }
  }
  double U[N][N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) u[i] = (double)v[i][k];
#pragma unroll
    for (int j = 0; j < k; ++j) {
      double d = 0;
#pragma unroll
      for (int i = 0; i < N; ++i) d += U[i][j] * u[i];
#pragma unroll
      for (int i = 0; i < N; ++i) u[i] -= d * U[i][j];
    }
    double e = -1.0;
#pragma unroll
    for (int i = 0; i < N; ++i) e += u[i] * u[i];
    if (!(fabs(e) <= 1e-5)) return false;
    double r = 1.0 + e * (-0.5 + e * (0.375 - 0.3125 * e));
#pragma unroll
    for (int i = 0; i < N; ++i) U[i][k] = u[i] * r;
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) Q[i][j] = U[i][j];
  return true;
}

// Eigen-projection of a small symmetric matrix held in registers (fully unrolled
// cyclic Jacobi on the upper triangle; N <= 5). Returns whether any eigenvalue was
// negative (then S holds the projection), leaving S untouched otherwise.
// The sweeps run on A = Q^T S Q, Q the orthonormal FP32-Jacobi estimate of the
// eigenvectors (jacobi_f32_start; the identity when it declines), accumulating the
// rotations onto Q, until the off-diagonal mass is 1e-32 of the total, as a Jacobi from
// the identity would. A rotation annihilating a_pq has t = tan(theta) = sgn(h) a_pq /
// (|h| + r), h = (a_qq - a_pp) / 2, r = sqrt(h^2 + a_pq^2). With g = 1 / r,
// c^2 = 1 / (1 + t^2) = (|h| + r) / (2 r), so t = sgn(h) a_pq g / (2 c^2) and
// s = t c = sgn(h) a_pq g / (2 c): two reciprocal square roots per rotation (g and 1 / c),
// no division. The 2x2 block is updated in closed form (a_pp -= t a_pq, a_qq += t a_pq,
// a_pq = 0), and only the entries of one triangle. Where h^2 + a_pq^2 is below the
// normal range the rotation takes t = a_pq / (|h| + r) by division instead. The
// projection V max(L, 0) V^T is formed on the upper triangle and mirrored.
template <int N>
DEV bool psd_project_small(double (&S)[N][N]) {
  double A[N][N], V[N][N];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  if (jacobi_f32_start<N>(S, V)) {
#pragma unroll
    for (int q = 0; q < N; ++q) {
      double t[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        double acc = 0;
#pragma unroll
        for (int k = 0; k < N; ++k) acc += (i <= k ? S[i][k] : S[k][i]) * V[k][q];
        t[i] = acc;
      }
#pragma unroll
      for (int p = 0; p <= q; ++p) {
        double acc = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) acc += V[i][p] * t[i];
        A[p][q] = acc;
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = i; j < N; ++j) A[i][j] = S[i][j];
  }
  for (int sweep = 0; sweep < 20; ++sweep) {
    double off = 0, dg = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      dg += A[i][i] * A[i][i];
#pragma unroll
      for (int j = i + 1; j < N; ++j) off += A[i][j] * A[i][j];
    }
    if (off == 0.0 || 2 * off <= 1e-32 * (dg + 2 * off)) break;
#pragma unroll
    for (int p = 0; p < N - 1; ++p)
#pragma unroll
      for (int q = p + 1; q < N; ++q) {
        double apq = A[p][q];
        if (apq != 0.0) {
          double h = 0.5 * (A[q][q] - A[p][p]);
          double sa = h >= 0 ? apq : -apq;
          double r2 = fma(h, h, apq * apq);
          double t, c, s;
          if (r2 >= 1e-300) {
            double g = rsqrt(r2);
            double c2 = 0.5 * fma(r2, g, fabs(h)) * g;
            double ic = rsqrt(c2);
            double sg = 0.5 * sa * g * ic;
            c = c2 * ic;
            s = sg;
            t = sg * ic;
          } else {
            double den = fabs(h) + sqrt(r2);
            t = den > 0.0 ? sa / den : 0.0;
            c = rsqrt(1.0 + t * t);
            s = t * c;
          }
          A[p][p] -= t * apq;
          A[q][q] += t * apq;
#pragma unroll
          for (int k = 0; k < N; ++k) {
            if (k == p || k == q) continue;
            double akp = k < p ? A[k][p] : A[p][k];
            double akq = k < q ? A[k][q] : A[q][k];
            double np_ = c * akp - s * akq, nq = s * akp + c * akq;
            if (k < p) A[k][p] = np_;
            else A[p][k] = np_;
            if (k < q) A[k][q] = nq;
            else A[q][k] = nq;
          }
#pragma unroll
          for (int k = 0; k < N; ++k) {
            double vkp = V[k][p], vkq = V[k][q];
            V[k][p] = c * vkp - s * vkq;
            V[k][q] = s * vkp + c * vkq;
          }
        }
        A[p][q] = 0.0;
      }
  }
  bool neg = false;
  double lam[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    lam[i] = A[i][i];
    neg |= lam[i] < 0.0;
  }
  if (!neg) return false;
#pragma unroll
  for (int k = 0; k < N; ++k) lam[k] = lam[k] > 0.0 ? lam[k] : 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      double acc = 0;
#pragma unroll
      for (int k = 0; k < N; ++k) acc += (V[i][k] * lam[k]) * V[j][k];
      S[i][j] = acc;
      S[j][i] = acc;
    }
  return true;
}

// Destinations of a reduced 9x9 Hessian S (symmetric; producers give the entries with
// p <= q): a local array (both triangles written) or the upper triangle of a per-pair
// record in global memory (structure of arrays, entry k of pair i at base[k * stride + i]).
DEV int s9_index(int p, int q) { return p * 9 - (p * (p - 1)) / 2 + (q - p); }  // p <= q, 0..44
DEV void s9_put(double (&S)[9][9], int p, int q, double v) {
  S[p][q] = v;
  S[q][p] = v;
}
struct S9Rec {
  double* base;
  size_t stride;
};
DEV void s9_put(const S9Rec& o, int p, int q, double v) { o.base[(size_t)s9_index(p, q) * o.stride] = v; }

// Reduced projection of a non-mollified pair: H lives in the span of
// { c (x) e_x, c (x) e_y, c (x) e_z, a_k' (x) w } (a_k' = the parameter directions
// orthonormalised against c; at most 3 + m <= 5 columns), where
//   S_r = [[2 b' |c|^2 I + 4 b'' |c|^2 w w^T, 0], [0, 0]] - b' Phi_r G^-1 Phi_r^T.
// S_r is projected (analytically for m = 0) and written back in the 9-dim Q (x) I basis.
template <int M, class Out>
DEV void reduced_project(const Stencil& st, d3 w, const d3* W, const double (&Gi)[2][2], double B1, double B2,
                         bool psd, Out& S9) {
  constexpr int N = 3 + M;
  double cn2 = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) cn2 += st.c[i] * st.c[i];
  double cn = sqrt(cn2);
  double ch[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) ch[i] = st.c[i] / cn;
  double wn = sqrt(fdot(w, w));
  d3 wh = fscl(1.0 / wn, w);
  // orthonormal parameter directions a_hat (R^4, _|_ c)
  double ah[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
  double ca[2] = {0, 0};   // c_hat . a_k
  double aa[2][2] = {{0, 0}, {0, 0}};  // a_hat_l . a_k
#pragma unroll
  for (int k = 0; k < M; ++k) {
    double t[4];
    double d = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) d += ch[i] * st.a[k][i];
    ca[k] = d;
#pragma unroll
    for (int i = 0; i < 4; ++i) t[i] = st.a[k][i] - d * ch[i];
#pragma unroll
    for (int l = 0; l < k; ++l) {
      double e = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) e += ah[l][i] * t[i];
#pragma unroll
      for (int i = 0; i < 4; ++i) t[i] -= e * ah[l][i];
    }
    double tn = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) tn += t[i] * t[i];
    tn = 1.0 / sqrt(tn);
#pragma unroll
    for (int i = 0; i < 4; ++i) ah[k][i] = t[i] * tn;
  }
#pragma unroll
  for (int l = 0; l < M; ++l)
#pragma unroll
    for (int k = 0; k < M; ++k) {
      double e = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) e += ah[l][i] * st.a[k][i];
      aa[l][k] = e;
    }
  double Sr[N][N];
  double wv[3] = {w.x, w.y, w.z};
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) Sr[i][j] = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Sr[i][j] = (i == j ? 2 * B1 * cn2 : 0.0) + 4 * B2 * cn2 * wv[i] * wv[j];
  if (M > 0) {
    double Phi[N][M > 0 ? M : 1];
#pragma unroll
    for (int k = 0; k < M; ++k) {
      double Wk[3] = {W[k].x, W[k].y, W[k].z};
#pragma unroll
      for (int j = 0; j < 3; ++j) Phi[j][k] = 2 * (cn * Wk[j] + ca[k] * wv[j]);
#pragma unroll
      for (int l = 0; l < M; ++l) Phi[3 + l][k] = 2 * aa[l][k] * wn;
    }
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        double acc = 0;
#pragma unroll
        for (int k = 0; k < M; ++k)
#pragma unroll
          for (int l = 0; l < M; ++l) acc += Phi[i][k] * Gi[k][l] * Phi[j][l];
        Sr[i][j] -= B1 * acc;
      }
  }
  if (psd) {
    if (M == 0) {
      // eigenpairs: w_hat with 2b'|c|^2 + 4b''|c|^2 |w|^2, the two normals with 2b'|c|^2
      double lw = 2 * B1 * cn2 + 4 * B2 * cn2 * wn * wn, ln = 2 * B1 * cn2;
      if (lw < 0.0 || ln < 0.0) {
        double whv[3] = {wh.x, wh.y, wh.z};
        double lwp = lw > 0 ? lw : 0.0, lnp = ln > 0 ? ln : 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) Sr[i][j] = lnp * (i == j ? 1.0 : 0.0) + (lwp - lnp) * whv[i] * whv[j];
      }
    } else {
      psd_project_small<N>(Sr);
    }
  }
  // back to the 9-dim basis: column alpha of the reduced basis has Q-coordinates
  // (Q^T u_alpha) (x) v_alpha, i.e. (Q^T c_hat) (x) e_r for alpha = r < 3 and
  // (Q^T a_hat_l) (x) w_hat for alpha = 3 + l. With cq = Q^T c_hat, aq_l = Q^T a_hat_l:
  //   S9[3a+r][3b+s] = cq_a cq_b Sr[r][s] + cq_a w_s al[b][r] + cq_b w_r al[a][s]
  //                    + w_r w_s be[a][b],
  //   al[a][r] = sum_l aq_l[a] Sr[r][3+l],  be[a][b] = sum_{l,l'} aq_l[a] Sr[3+l][3+l'] aq_l'[b].
  double cq[3];
  qt4(ch, cq);
  const double whv[3] = {wh.x, wh.y, wh.z};
  double aq[2][3] = {{0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int l = 0; l < M; ++l) qt4(ah[l], aq[l]);
  double al[3][3], be[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double acc = 0;
#pragma unroll
      for (int l = 0; l < M; ++l) acc += aq[l][a] * Sr[r][3 + l];
      al[a][r] = acc;
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      double acc = 0;
#pragma unroll
      for (int l = 0; l < M; ++l)
#pragma unroll
        for (int l2 = 0; l2 < M; ++l2) acc += aq[l][a] * Sr[3 + l][3 + l2] * aq[l2][b];
      be[a][b] = acc;
    }
  }
#pragma unroll
  for (int p = 0; p < 9; ++p)
#pragma unroll
    for (int q = p; q < 9; ++q) {
      const int a = p / 3, r = p % 3, b = q / 3, s = q % 3;
      double v = cq[a] * cq[b] * (r <= s ? Sr[r][s] : Sr[s][r]);
      if (M > 0) v += cq[a] * whv[s] * al[b][r] + cq[b] * whv[r] * al[a][s] + whv[r] * whv[s] * be[a][b];
      s9_put(S9, p, q, v);
    }
}

// Friction stencil of a pair: tangent basis (c0, c1), relative-displacement weights
// gamma (model/pt_ipc.cpp:22-107, model/ee_ipc.cpp:21-118).
struct FrictionFrame {
  d3 c0, c1;
  double gam[4];
};

DEV void pp_basis(d3 p0, d3 p1, FrictionFrame& f) {
  d3 d = fsub(p1, p0);
  d3 cx = fcross(fd3(1, 0, 0), d), cy = fcross(fd3(0, 1, 0), d);
  if (fdot(cx, cx) > fdot(cy, cy)) {
    f.c0 = fnormalized(cx);
    f.c1 = fnormalized(fcross(d, cx));
  } else {
    f.c0 = fnormalized(cy);
    f.c1 = fnormalized(fcross(d, cy));
  }
}
DEV void pe_basis(d3 p, d3 e0, d3 e1, FrictionFrame& f) {
  d3 e = fsub(e1, e0);
  f.c0 = fnormalized(e);
  f.c1 = fnormalized(fcross(e, fsub(p, e0)));
}
DEV double pe_closest(d3 p, d3 e0, d3 e1) {
  d3 e = fsub(e1, e0);
  return fdot(fsub(p, e0), e) / fdot(e, e);
}
DEV void frame_pt(const d3* X, int ty, FrictionFrame& f) {
  double l0, l1;
  {
    d3 b0 = fsub(X[2], X[1]), b1 = fsub(X[3], X[1]), r = fsub(X[0], X[1]);
    solve2_ldlt(fdot(b0, b0), fdot(b0, b1), fdot(b1, b1), fdot(b0, r), fdot(b1, r), l0, l1);
  }
  double tl[3] = {1 - l0 - l1, l0, l1};
  {
    d3 e0 = fsub(X[2], X[1]);
    d3 n = fcross(e0, fsub(X[3], X[1]));
    f.c0 = fnormalized(e0);
    f.c1 = fnormalized(fcross(n, e0));
  }
  switch (ty) {
    case P_T0: pp_basis(X[0], X[1], f); tl[0] = 1; tl[1] = 0; tl[2] = 0; break;
    case P_T1: pp_basis(X[0], X[2], f); tl[0] = 0; tl[1] = 1; tl[2] = 0; break;
    case P_T2: pp_basis(X[0], X[3], f); tl[0] = 0; tl[1] = 0; tl[2] = 1; break;
    case P_E0: { double e = pe_closest(X[0], X[1], X[2]); tl[0] = 1 - e; tl[1] = e; tl[2] = 0; pe_basis(X[0], X[1], X[2], f); break; }
    case P_E1: { double e = pe_closest(X[0], X[2], X[3]); tl[0] = 0; tl[1] = 1 - e; tl[2] = e; pe_basis(X[0], X[2], X[3], f); break; }
    case P_E2: { double e = pe_closest(X[0], X[3], X[1]); tl[0] = e; tl[1] = 0; tl[2] = 1 - e; pe_basis(X[0], X[3], X[1], f); break; }
    default: break;
  }
  f.gam[0] = -1.0;
  f.gam[1] = tl[0];
  f.gam[2] = tl[1];
  f.gam[3] = tl[2];
}
DEV void frame_ee(const d3* X, int ty, FrictionFrame& f) {
  double s, t;
  {
    d3 w = fsub(X[0], X[2]), ea = fsub(X[1], X[0]), eb = fsub(X[3], X[2]);
    solve2_ldlt(fdot(ea, ea), -fdot(eb, ea), fdot(eb, eb), -fdot(w, ea), fdot(w, eb), s, t);
  }
  {
    d3 ea = fsub(X[1], X[0]);
    d3 n = fcross(ea, fsub(X[3], X[2]));
    f.c0 = fnormalized(ea);
    f.c1 = fnormalized(fcross(n, ea));
  }
  switch (ty) {
    case EA0_EB0: pp_basis(X[0], X[2], f); s = 0; t = 0; break;
    case EA0_EB1: pp_basis(X[0], X[3], f); s = 0; t = 1; break;
    case EA1_EB0: pp_basis(X[1], X[2], f); s = 1; t = 0; break;
    case EA1_EB1: pp_basis(X[1], X[3], f); s = 1; t = 1; break;
    case EA_EB0: s = pe_closest(X[2], X[0], X[1]); t = 0; pe_basis(X[2], X[0], X[1], f); break;
    case EA_EB1: s = pe_closest(X[3], X[0], X[1]); t = 1; pe_basis(X[3], X[0], X[1], f); break;
    case EA0_EB: s = 0; t = pe_closest(X[0], X[2], X[3]); pe_basis(X[0], X[2], X[3], f); break;
    case EA1_EB: s = 1; t = pe_closest(X[1], X[2], X[3]); pe_basis(X[1], X[2], X[3], f); break;
    default: break;
  }
  s = fmax(fmin(1.0, s), 0.0);
  t = fmax(fmin(1.0, t), 0.0);
  f.gam[0] = -(1 - s);
  f.gam[1] = -s;
  f.gam[2] = 1 - t;
  f.gam[3] = t;
}

struct FrictionP {
  double mu, epsv, max_uk;
};

// 2x2 friction Hessian factor M and gradient scale (friction.cpp:15-47):
// g += gamma (x) (mu lam f1 P uk), H += (gamma gamma^T) (x) (P M P^T).
DEV void friction_2x2(const double* uk2, double lam, const FrictionP& fp, double& gscale, double M[2][2]) {
  double uk = sqrt(uk2[0] * uk2[0] + uk2[1] * uk2[1]);
  double f1 = f1_SF_over_x(uk, fp.epsv);
  gscale = fp.mu * lam * f1;
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
    double m00 = f2 / uk * uk2[0] * uk2[0] + f1, m11 = f2 / uk * uk2[1] * uk2[1] + f1, m01 = f2 / uk * uk2[0] * uk2[1];
    double s = fp.mu * lam;
    m00 *= s; m11 *= s; m01 *= s;
    // closed-form 2x2 eigen-projection
    double tr = 0.5 * (m00 + m11), df = 0.5 * (m00 - m11);
    double rad = sqrt(df * df + m01 * m01);
    double l0 = tr - rad, l1 = tr + rad;
    if (l0 >= 0.0) {
      M[0][0] = m00; M[1][1] = m11; M[0][1] = M[1][0] = m01;
    } else {
      // eigenvector of l1
      double vx, vy;
      if (rad == 0.0) { vx = 1; vy = 0; }
      else if (df >= 0) { vx = df + rad; vy = m01; }
      else { vx = m01; vy = rad - df; }
      double n = sqrt(vx * vx + vy * vy);
      vx /= n; vy /= n;
      double l = l1 > 0 ? l1 : 0.0;
      M[0][0] = l * vx * vx; M[1][1] = l * vy * vy; M[0][1] = M[1][0] = l * vx * vy;
    }
  }
}

// Everything a mollified edge-edge pair's 9x9 reduced Hessian is built from: the
// distance's first and second derivatives (gd, Phi, Gi, ch), the barrier derivatives,
// the mollifier m(x) with its derivatives and x's gradient gx, and the two edge vectors
// (x's Hessian follows from them).
struct MollData {
  double gd[9], gx[9], Phi[2][9];
  double ch[3], Gi[2][2];
  double mol, B, B1, B2, m1, m2;
  double u[3], v[3], uu, vv, uv;
  int m;
};

// Entry (p, q) of x = |u x v|^2's Hessian in the reduced coordinates (u = 2 x_0..2,
// v = x_3..5 directions, zero for 6..8).
DEV double moll_hx(const MollData& md, int p, int q) {
  if (p >= 6 || q >= 6) return 0.0;
  const int i = p % 3, j = q % 3;
  const double dij = (i == j) ? 1.0 : 0.0;
  if (p < 3 && q < 3) return 2.0 * (2.0 * (md.vv * dij - md.v[i] * md.v[j]));
  if (p >= 3 && q >= 3) return 2.0 * (2.0 * (md.uu * dij - md.u[i] * md.u[j]));
  if (p < 3) return 2.0 * (2.0 * (2.0 * md.u[i] * md.v[j] - md.v[i] * md.u[j] - md.uv * dij));
  return 2.0 * (2.0 * (2.0 * md.u[j] * md.v[i] - md.v[j] * md.u[i] - md.uv * dij));
}

// Entry (p, q) of a mollified pair's reduced Hessian (before projection):
// m (b'' grad d grad d^T + b' hess d) + b (m'' grad x grad x^T + m' hess x)
// + b' m' (grad x grad d^T + grad d grad x^T).
DEV double moll_entry(const MollData& md, int p, int q) {
  const int a = p / 3, r = p % 3, b = q / 3, s = q % 3;
  double hd = (r == s ? 2 * md.ch[a] * md.ch[b] : 0.0);
  for (int k = 0; k < md.m; ++k)
    for (int l = 0; l < md.m; ++l) hd -= md.Phi[k][p] * md.Gi[k][l] * md.Phi[l][q];
  double h = md.mol * (md.B2 * md.gd[p] * md.gd[q] + md.B1 * hd);
  double gmp = md.m1 * md.gx[p], gmq = md.m1 * md.gx[q];
  h += (md.m2 * md.gx[p] * md.gx[q] + md.m1 * moll_hx(md, p, q)) * md.B + md.B1 * (gmp * md.gd[q] + md.gd[p] * gmq);
  return h;
}

// Shared set-up of pair_reduced: stencil, closest-point derivatives and, for edge-edge
// pairs inside the mollifier's range, the mollifier data. Returns whether the pair is
// mollified; for the others the outputs needed by reduced_project are set.
DEV bool pair_setup(int kind, int ty, const d3* X, double d, const BarrierP& bp, double eps_x_param, Stencil& st,
                    d3& w, d3 (&W)[2], double (&Gi)[2][2], MollData& md, d3& gu, d3& gv) {
  if (kind == 0) st_pt(X, ty, st);
  else st_ee(X, ty, st);
  w = fd3(0, 0, 0);
  W[0] = fd3(0, 0, 0);
  W[1] = fd3(0, 0, 0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    w = fadd(w, fscl(st.c[i], X[i]));
    W[0] = fadd(W[0], fscl(st.a[0][i], X[i]));
    W[1] = fadd(W[1], fscl(st.a[1][i], X[i]));
  }
  Gi[0][0] = Gi[0][1] = Gi[1][0] = Gi[1][1] = 0.0;
  if (st.m == 1) {
    Gi[0][0] = 1.0 / (2 * fdot(W[0], W[0]));
  } else if (st.m == 2) {
    double g00 = 2 * fdot(W[0], W[0]), g01 = 2 * fdot(W[0], W[1]), g11 = 2 * fdot(W[1], W[1]);
    double det = g00 * g11 - g01 * g01;
    Gi[0][0] = g11 / det;
    Gi[1][1] = g00 / det;
    Gi[0][1] = Gi[1][0] = -g01 / det;
  }
  md.B1 = barrier_b1(d, bp);
  md.B2 = barrier_b2(d, bp);
  md.mol = 1.0;
  md.B = md.m1 = md.m2 = 0.0;
  gu = gv = fd3(0, 0, 0);
  if (kind != 1) return false;
  d3 u = fsub(X[1], X[0]), v = fsub(X[3], X[2]);
  double eps_x = eps_x_param * fdot(fsub(X[0], X[1]), fsub(X[0], X[1])) * fdot(fsub(X[2], X[3]), fsub(X[2], X[3]));
  d3 cr = fcross(u, v);
  double x = fdot(cr, cr);
  if (!(x < eps_x)) return false;
  double xe = x / eps_x;
  md.mol = (-xe + 2.0) * xe;
  md.m1 = 2.0 * (1.0 - xe) / eps_x;
  md.m2 = -2.0 / (eps_x * eps_x);
  md.B = barrier_b(d, bp);
  md.uu = fdot(u, u);
  md.vv = fdot(v, v);
  md.uv = fdot(u, v);
  gu = fsub(fscl(2.0 * md.vv, u), fscl(2.0 * md.uv, v));
  gv = fsub(fscl(2.0 * md.uu, v), fscl(2.0 * md.uv, u));
  md.u[0] = u.x; md.u[1] = u.y; md.u[2] = u.z;
  md.v[0] = v.x; md.v[1] = v.y; md.v[2] = v.z;
  const double sq2 = 1.41421356237309504880;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    md.gx[r] = -sq2 * c3(gu, r);
    md.gx[3 + r] = -sq2 * c3(gv, r);
    md.gx[6 + r] = 0.0;
  }
  double ah[2][3];
  qt4(st.c, md.ch);
  qt4(st.a[0], ah[0]);
  qt4(st.a[1], ah[1]);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      md.gd[3 * a + r] = 2 * md.ch[a] * c3(w, r);
      md.Phi[0][3 * a + r] = 2 * (md.ch[a] * c3(W[0], r) + ah[0][a] * c3(w, r));
      md.Phi[1][3 * a + r] = 2 * (md.ch[a] * c3(W[1], r) + ah[1][a] * c3(w, r));
    }
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int l = 0; l < 2; ++l) md.Gi[k][l] = Gi[k][l];
  md.m = st.m;
  return true;
}

// Vertex-space gradient of a pair: m b' grad d + b grad m.
DEV void pair_gradient(const Stencil& st, d3 w, const MollData& md, d3 gu, d3 gv, d3* g) {
#pragma unroll
  for (int i = 0; i < 4; ++i) g[i] = fscl(md.mol * md.B1 * 2 * st.c[i], w);
  if (md.m1 != 0.0 || md.B != 0.0) {
    g[0] = fsub(g[0], fscl(md.B * md.m1, gu));
    g[1] = fadd(g[1], fscl(md.B * md.m1, gu));
    g[2] = fsub(g[2], fscl(md.B * md.m1, gv));
    g[3] = fadd(g[3], fscl(md.B * md.m1, gv));
  }
}

// Reduced 9x9 Hessian S of a pair. Returns the vertex-space gradient g[4] (3-vectors).
// kind 0: point-triangle, 1: edge-edge (mollified when the edges are near parallel).
template <class Out>
DEV void pair_reduced(int kind, int ty, const d3* X, double d, const BarrierP& bp, double eps_x_param, bool psd,
                      Out& S, d3* g) {
  Stencil st;
  d3 w, W[2], gu, gv;
  double Gi[2][2];
  MollData md;
  const bool mollified = pair_setup(kind, ty, X, d, bp, eps_x_param, st, w, W, Gi, md, gu, gv);
  if (!mollified) {
    if (st.m == 0) reduced_project<0>(st, w, W, Gi, md.B1, md.B2, psd, S);
    else if (st.m == 1) reduced_project<1>(st, w, W, Gi, md.B1, md.B2, psd, S);
    else reduced_project<2>(st, w, W, Gi, md.B1, md.B2, psd, S);
#pragma unroll
    for (int i = 0; i < 4; ++i) g[i] = fscl(md.B1 * 2 * st.c[i], w);
    return;
  }
  double Sm[9][9];
  for (int p = 0; p < 9; ++p)
    for (int q = 0; q < 9; ++q) Sm[p][q] = moll_entry(md, p, q);
  if (psd) psd_project9(Sm);
  for (int p = 0; p < 9; ++p)
    for (int q = p; q < 9; ++q) s9_put(S, p, q, Sm[p][q]);
  pair_gradient(st, w, md, gu, gv, g);
}

// Friction of a pair: adds its force to the vertex gradient and returns its reduced
// Hessian in factored form, S9[3a+r][3b+s] += gh[a] gh[b] N[r][s] (gh = Q^T gamma,
// N = P M P^T with the tangent basis P and the 2x2 friction Hessian M); N6 holds the
// upper triangle of N row by row.
DEV void pair_friction(const FrictionFrame& fr, const double* uk, double lam, const FrictionP& fp, d3* g,
                       double (&gh)[3], double (&N6)[6]) {
  double gs, M[2][2];
  friction_2x2(uk, lam, fp, gs, M);
  d3 F = fadd(fscl(gs * uk[0], fr.c0), fscl(gs * uk[1], fr.c1));
#pragma unroll
  for (int i = 0; i < 4; ++i) g[i] = fadd(g[i], fscl(fr.gam[i], F));
  int k = 0;
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int s = r; s < 3; ++s) {
      double p0r = c3(fr.c0, r), p1r = c3(fr.c1, r), p0s = c3(fr.c0, s), p1s = c3(fr.c1, s);
      N6[k++] = p0r * (M[0][0] * p0s + M[0][1] * p1s) + p1r * (M[1][0] * p0s + M[1][1] * p1s);
    }
  qt4(fr.gam, gh);
}

}  // namespace abd
