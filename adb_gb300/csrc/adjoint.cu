// Device parts of the adjoint of a converged frame that the Newton system does not
// already hold: the Jacobian of each point-triangle / edge-edge friction force through
// its tangent frame and multiplier (abd_fric_adj.cuh), its transposed product in body
// coordinates, and the vector kernels of the GMRES solve. Every reduction runs in a
// fixed order.
#include "abd_engine.h"
#include "abd_fric_adj.cuh"

namespace abd {
namespace {

inline int nblk_a(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ d3 ldXa(const double* X, int nv, int v) { return mk(X[v], X[nv + v], X[2 * nv + v]); }

__device__ __forceinline__ void pair_vids(const Geo& g, int kind, const int* tup, int p, int (&vid)[4], int& A,
                                          int& B) {
  A = tup[4 * p];
  B = tup[4 * p + 2];
  const int a = tup[4 * p + 1], b = tup[4 * p + 3];
  if (kind == 0) {
    vid[0] = g.v_off[A] + a;
    const int f = g.f_off[B] + b;
    vid[1] = g.fv[3 * f];
    vid[2] = g.fv[3 * f + 1];
    vid[3] = g.fv[3 * f + 2];
  } else {
    const int ea = g.e_off[A] + a, eb = g.e_off[B] + b;
    vid[0] = g.ev[2 * ea];
    vid[1] = g.ev[2 * ea + 1];
    vid[2] = g.ev[2 * eb];
    vid[3] = g.ev[2 * eb + 1];
  }
}

// Per pair: the 12 x 12 vertex-space Jacobian of its friction force through the frame
// and multiplier, row-major (J[12 r + c] = d g_r / d x_c); 0 for inactive pairs.
__global__ void k_fric_frame_jac(Geo g, Params P, int kind, int n, const int* tup, const int8_t* tys, double* J) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  double* Jp = J + 144 * (size_t)p;
  int vid[4], A, B;
  pair_vids(g, kind, tup, p, vid, A, B);
  d3 X[4], du[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    X[i] = ldXa(g.X, g.nv, vid[i]);
    du[i] = fsub(X[i], ldXa(g.X0, g.nv, vid[i]));
  }
  const int ty = tys[p];
  const double d = kind == 0 ? pt_dist(X[0], X[1], X[2], X[3], ty) : ee_dist(X[0], X[1], X[2], X[3], ty);
  const bool on = d < P.dhat && P.mu > 0.0 && (kind == 0 ? (P.pt && P.pt_fric) : (P.ee && P.ee_fric));
  for (int c = 0; c < 12; ++c) {
    double col[12];
    if (on) {
      fadj::frame_jacobian_column(kind, ty, X, du, P.dhat, P.kappa, P.mu, P.epsv, c, col);
    } else {
#pragma unroll
      for (int r = 0; r < 12; ++r) col[r] = 0.0;
    }
#pragma unroll
    for (int r = 0; r < 12; ++r) Jp[12 * r + c] = col[r];
  }
}

// Per pair: y = J^T (Jx w) in vertex space, returned in body space as the pair's
// contributions to its two bodies (12 each: p, a1, a2, a3 rows of Jx^T y). Vertices of
// static bodies do not move: their entries of Jx w are 0, and so are their bodies' rows.
__global__ void k_fric_frame_apply(Geo g, int kind, int n, const int* tup, const double* J, const double* w,
                                   double* contrib) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int vid[4], A, B;
  pair_vids(g, kind, tup, p, vid, A, B);
  const int na = kind == 0 ? 1 : 2;
  double xb[4][4], v[12];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = i < na ? A : B;
    xb[i][0] = 1.0;
    xb[i][1] = g.rest[3 * vid[i]];
    xb[i][2] = g.rest[3 * vid[i] + 1];
    xb[i][3] = g.rest[3 * vid[i] + 2];
    const bool moves = g.mass[b] > 0.0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < 4; ++k) s += xb[i][k] * w[12 * b + 3 * k + r];
      v[3 * i + r] = moves ? s : 0.0;
    }
  }
  const double* Jp = J + 144 * (size_t)p;
  double y[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) {
    double s = 0.0;
    for (int r = 0; r < 12; ++r) s += Jp[12 * r + c] * v[r];
    y[c] = s;
  }
  double* out = contrib + 24 * (size_t)p;
#pragma unroll
  for (int k = 0; k < 24; ++k) out[k] = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    double* o = out + (i < na ? 0 : 12);
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int r = 0; r < 3; ++r) o[3 * k + r] += xb[i][k] * y[3 * i + r];
  }
}

// Per body (one thread per body DOF row): the sum of its pairs' contributions, over its
// overlaps in row order and each overlap's PT then EE pairs in pair order.
__global__ void k_fric_frame_gather(int nb, const double* mass, const int* row_ptr, const int* upidx,
                                    const int* pt_seg, const int* ee_seg, const int* pt, const int* ee,
                                    const double* cpt, const double* cee, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = t / 12, k = t - 12 * b;
  if (b >= nb) return;
  double s = 0.0;
  if (mass[b] > 0.0) {
    for (int e = row_ptr[b]; e < row_ptr[b + 1]; ++e) {
      const int u = upidx[e];
      if (u < 0) continue;
      for (int p = pt_seg[u]; p < pt_seg[u + 1]; ++p) s += cpt[24 * (size_t)p + (pt[4 * p] == b ? 0 : 12) + k];
      for (int p = ee_seg[u]; p < ee_seg[u + 1]; ++p) s += cee[24 * (size_t)p + (ee[4 * p] == b ? 0 : 12) + k];
    }
  }
  out[t] = s;
}

// Dot product by one CTA: thread t adds entries t, t + 1024, ... in order, then a fixed
// tree over the threads.
__global__ void __launch_bounds__(1024) k_dot(int n, const double* a, const double* b, double* out) {
  __shared__ double sh[1024];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) s += a[i] * b[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 512; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// y = a x + b y
__global__ void k_axpby(int n, double a, const double* x, double b, double* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i] + b * y[i];
}

}  // namespace

void fric_frame_jacobians(const Geo& g, const Params& P, PairSet& S, NewtonBufs& B, cudaStream_t s) {
  B.fj_pt.ensure(144 * (size_t)S.npt + 1);
  B.fj_ee.ensure(144 * (size_t)S.nee + 1);
  if (S.npt)
    KLAUNCH(K_PAIR_TERMS, s, k_fric_frame_jac<<<nblk_a(S.npt, 64), 64, 0, s>>>(g, P, 0, S.npt, S.pt.p, S.pt_ty.p,
                                                                               B.fj_pt.p));
  if (S.nee)
    KLAUNCH(K_PAIR_TERMS, s, k_fric_frame_jac<<<nblk_a(S.nee, 64), 64, 0, s>>>(g, P, 1, S.nee, S.ee.p, S.ee_ty.p,
                                                                               B.fj_ee.p));
}

void fric_frame_apply_t(const Geo& g, PairSet& S, NewtonBufs& B, const double* w, double* out, cudaStream_t s) {
  B.fc_pt.ensure(24 * (size_t)S.npt + 1);
  B.fc_ee.ensure(24 * (size_t)S.nee + 1);
  if (S.npt)
    KLAUNCH(K_VEC, s, k_fric_frame_apply<<<nblk_a(S.npt, 128), 128, 0, s>>>(g, 0, S.npt, S.pt.p, B.fj_pt.p, w,
                                                                            B.fc_pt.p));
  if (S.nee)
    KLAUNCH(K_VEC, s, k_fric_frame_apply<<<nblk_a(S.nee, 128), 128, 0, s>>>(g, 1, S.nee, S.ee.p, B.fj_ee.p, w,
                                                                            B.fc_ee.p));
  KLAUNCH(K_VEC, s, k_fric_frame_gather<<<nblk_a(12ll * g.nb, 128), 128, 0, s>>>(
                        g.nb, g.mass, S.row_ptr.p, S.upidx.p, B.pt_seg.p, B.ee_seg.p, S.pt.p, S.ee.p, B.fc_pt.p,
                        B.fc_ee.p, out));
}

double dev_dot(int n, const double* a, const double* b, NewtonBufs& B, cudaStream_t s) {
  B.e_out.ensure(1);
  if (!B.h_dot) CK(cudaMallocHost(&B.h_dot, sizeof(double)));
  KLAUNCH(K_DOTS, s, k_dot<<<1, 1024, 0, s>>>(n, a, b, B.e_out.p));
  CK(cudaMemcpyAsync(B.h_dot, B.e_out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return *B.h_dot;
}

void dev_axpby(int n, double a, const double* x, double b, double* y, cudaStream_t s) {
  if (n > 0) KLAUNCH(K_VEC, s, k_axpby<<<nblk_a(n, 256), 256, 0, s>>>(n, a, x, b, y));
}

}  // namespace abd
