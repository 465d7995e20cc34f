// Newton system of one iteration on the GPU and its solve:
//  - per-pair IPC terms (ABD::ipc, model/abd.cpp:305-405) into per-pair block records,
//  - deterministic per-overlap reduction of the records (the reference scatters them
//    under per-column OpenMP locks, model/assemble_matrices.cpp:28-59),
//  - per-body inertia + orthogonality + vertex-ground terms and the diagonal blocks
//    (model/mutils.cpp:53-76, model/vg_ipc.cpp:12-30, abd.cpp:249-260),
//  - block-Jacobi preconditioned CG over the 12x12 block-sparse matrix (the reference
//    factorizes with Pardiso LLT, abd.cpp:229-303),
//  - the line-search energies (model/energy.cpp:19-86, 195-258).
// All reductions use a fixed order, so results are bitwise reproducible run to run.
#include <cooperative_groups.h>

#include "abd_engine.h"
#include "abd_ipc.cuh"

namespace cg = cooperative_groups;

namespace abd {

namespace {

__device__ __forceinline__ d3 ldX(const double* X, int nv, int v) { return mk(X[v], X[nv + v], X[2 * nv + v]); }
inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// ---------------------------------------------------------------------------------
// Per-pair terms. kind 0: PT (point on body A, triangle on body B); 1: EE.
__global__ void __launch_bounds__(128) k_pair_terms(Geo g, Params P, int kind, int n, const int* tup,
                                                    const int* pov, const int* ovI, double* C, double* lag) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int A = tup[4 * p], a = tup[4 * p + 1], B = tup[4 * p + 2], b = tup[4 * p + 3];
  int vid[4];
  int na;
  if (kind == 0) {
    vid[0] = g.v_off[A] + a;
    int f = g.f_off[B] + b;
    vid[1] = g.fv[3 * f];
    vid[2] = g.fv[3 * f + 1];
    vid[3] = g.fv[3 * f + 2];
    na = 1;
  } else {
    int ea = g.e_off[A] + a, eb = g.e_off[B] + b;
    vid[0] = g.ev[2 * ea];
    vid[1] = g.ev[2 * ea + 1];
    vid[2] = g.ev[2 * eb];
    vid[3] = g.ev[2 * eb + 1];
    na = 2;
  }
  d3 X[4], X0[4];
  double xt[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    X[i] = ldX(g.X, g.nv, vid[i]);
    X0[i] = ldX(g.X0, g.nv, vid[i]);
    xt[i][0] = 1.0;
    xt[i][1] = g.rest[3 * vid[i]];
    xt[i][2] = g.rest[3 * vid[i] + 1];
    xt[i][3] = g.rest[3 * vid[i] + 2];
  }
  int ty;
  double d;
  if (kind == 0) {
    ty = pt_type(X[0], X[1], X[2], X[3]);
    d = pt_dist(X[0], X[1], X[2], X[3], ty);
  } else {
    ty = ee_type(X[0], X[1], X[2], X[3]);
    d = ee_dist(X[0], X[1], X[2], X[3], ty);
  }
  double S[9][9];
  d3 gv[4];
  FrictionFrame fr;
  double lam = 0.0;
  bool active = d < P.dhat;
  if (active) {
    BarrierP bp{P.dhat, P.kappa};
    if (kind == 0) frame_pt(X, ty, fr);
    else frame_ee(X, ty, fr);
    double uk[2] = {0.0, 0.0};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      d3 du = fsub(X[i], X0[i]);
      uk[0] += fr.gam[i] * fdot(fr.c0, du);
      uk[1] += fr.gam[i] * fdot(fr.c1, du);
    }
    lam = -barrier_b1(d, bp) * 2 * sqrt(d);
    pair_reduced(kind, ty, X, d, bp, P.eps_x, P.psd != 0, S, gv);
    bool fric = (kind == 0) ? P.pt_fric : P.ee_fric;
    if (fric) pair_friction(fr, uk, lam, FrictionP{P.mu, P.epsv, P.max_uk}, S, gv);
  } else {
    fr.c0 = fd3(0, 0, 0);
    fr.c1 = fd3(0, 0, 0);
    for (int i = 0; i < 4; ++i) fr.gam[i] = 0;
  }
  // lagged friction record
  lag[0 * n + p] = fr.c0.x; lag[1 * n + p] = fr.c0.y; lag[2 * n + p] = fr.c0.z;
  lag[3 * n + p] = fr.c1.x; lag[4 * n + p] = fr.c1.y; lag[5 * n + p] = fr.c1.z;
  for (int i = 0; i < 4; ++i) lag[(6 + i) * n + p] = fr.gam[i];
  lag[10 * n + p] = lam;

  int I = ovI[pov[p]];
  bool a_is_I = (A == I);
  bool a_dyn = g.mass[A] > 0.0, b_dyn = g.mass[B] > 0.0;
  double* dI = C;
  double* dJ = C + 144 * (size_t)n;
  double* off = C + 288 * (size_t)n;
  double* gI = C + 432 * (size_t)n;
  double* gJ = C + 444 * (size_t)n;
  double* dA = a_is_I ? dI : dJ;
  double* dB = a_is_I ? dJ : dI;
  double* gA = a_is_I ? gI : gJ;
  double* gB = a_is_I ? gJ : gI;
  if (!active) {
    for (int e = 0; e < 144; ++e) {
      dI[(size_t)e * n + p] = 0.0;
      dJ[(size_t)e * n + p] = 0.0;
      off[(size_t)e * n + p] = 0.0;
    }
    for (int e = 0; e < 12; ++e) {
      gI[(size_t)e * n + p] = 0.0;
      gJ[(size_t)e * n + p] = 0.0;
    }
    return;
  }
  // Y matrices of the chain rule
  double YA[4][3], YB[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int aa = 0; aa < 3; ++aa) {
      double sa = 0, sb = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        double v = xt[i][k] * Qe(i, aa);
        if (i < na) sa += v;
        else sb += v;
      }
      YA[k][aa] = sa;
      YB[k][aa] = sb;
    }
  for (int r = 0; r < 3; ++r)
    for (int s = 0; s < 3; ++s) {
      double M[3][3];
#pragma unroll
      for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) M[aa][bb] = S[3 * aa + r][3 * bb + s];
      double TA[4][3], TB[4][3];
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
          TA[k][bb] = YA[k][0] * M[0][bb] + YA[k][1] * M[1][bb] + YA[k][2] * M[2][bb];
          TB[k][bb] = YB[k][0] * M[0][bb] + YB[k][1] * M[1][bb] + YB[k][2] * M[2][bb];
        }
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          double aa_ = TA[k][0] * YA[l][0] + TA[k][1] * YA[l][1] + TA[k][2] * YA[l][2];
          double bb_ = TB[k][0] * YB[l][0] + TB[k][1] * YB[l][1] + TB[k][2] * YB[l][2];
          double ab_ = TA[k][0] * YB[l][0] + TA[k][1] * YB[l][1] + TA[k][2] * YB[l][2];
          int e = (3 * k + r) * 12 + (3 * l + s);
          int et = (3 * l + s) * 12 + (3 * k + r);
          dA[(size_t)e * n + p] = a_dyn ? aa_ : 0.0;
          dB[(size_t)e * n + p] = b_dyn ? bb_ : 0.0;
          // block (A, B) -> stored as block (I, J)
          off[(size_t)(a_is_I ? e : et) * n + p] = (a_dyn && b_dyn) ? ab_ : 0.0;
        }
    }
  // body gradients
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double sa = 0, sb = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        double v = xt[i][k] * c3(gv[i], r);
        if (i < na) sa += v;
        else sb += v;
      }
      gA[(size_t)(3 * k + r) * n + p] = a_dyn ? sa : 0.0;
      gB[(size_t)(3 * k + r) * n + p] = b_dyn ? sb : 0.0;
    }
}

// First pair of each overlap (pairs are ordered by overlap).
__global__ void k_seg(int nov, int n, const int* pov, int* seg) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u > nov) return;
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (pov[mid] < u) lo = mid + 1;
    else hi = mid;
  }
  seg[u] = lo;
}

// Per-overlap sums of the pair records: 8 warps, each owns components c = w + 8k;
// lanes stride over the overlap's pairs; fixed shuffle tree.
__global__ void __launch_bounds__(256) k_ov_reduce(int nov, const int* pt_seg, const int* ee_seg, const double* ptC,
                                                   int npt, const double* eeC, int nee, double* ovr, int* has) {
  int u = blockIdx.x;
  if (u >= nov) return;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int p0 = pt_seg[u], p1 = pt_seg[u + 1], e0 = ee_seg[u], e1 = ee_seg[u + 1];
  if (threadIdx.x == 0) has[u] = (p1 > p0) || (e1 > e0);
  for (int c = w; c < CONTRIB; c += 8) {
    double s = 0.0;
    for (int p = p0 + lane; p < p1; p += 32) s += ptC[(size_t)c * npt + p];
    for (int p = e0 + lane; p < e1; p += 32) s += eeC[(size_t)c * nee + p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) ovr[(size_t)u * CONTRIB + c] = s;
  }
}

// Per-body diagonal block and gradient: one CTA per body, threads 0..143 own the
// Hessian entries, 144..155 the gradient entries.
__global__ void __launch_bounds__(160) k_body_system(Geo g, Params P, const int* row_ptr, const int* col,
                                                     const int* upidx, const double* ovr, const int* has,
                                                     const int* vg, const int* vg_seg, double* vg_lam, double* D,
                                                     double* grad) {
  int b = blockIdx.x;
  int t = threadIdx.x;
  if (t >= 156) return;
  bool is_h = t < 144;
  int i = is_h ? t / 12 : t - 144;
  int j = is_h ? t % 12 : 0;
  int k = i / 3, r = i % 3, l = j / 3, s = j % 3;
  double m = g.mass[b];
  const double* q = g.q + 12 * b;
  double dt = P.dt;
  double val = 0.0;
  if (m < 0.0) {
    // static body: identity block, zero gradient (mutils.cpp:55-56, 70)
    if (is_h) D[144 * b + t] = (i == j) ? 1.0 : 0.0;
    else grad[12 * b + i] = 0.0;
    if (t == 0)
      for (int kk = vg_seg[b]; kk < vg_seg[b + 1]; ++kk) {
        int v = g.v_off[b] + vg[2 * kk + 1];
        double _d = g.X[g.nv + v] + P.ground_offset;
        double dd = _d * _d;
        vg_lam[kk] = dd < P.dhat ? -barrier_b1(dd, BarrierP{P.dhat, P.kappa}) * 2 * _d : 0.0;
      }
    return;
  }
  double mi = (i < 3) ? m : g.Ic[b];
  double kap = 4.0 * P.ortho_kappa;
  if (is_h) {
    val = (i == j) ? mi : 0.0;
    if (k >= 1 && l >= 1) {
      d3 ak = mk(q[3 * k], q[3 * k + 1], q[3 * k + 2]);
      double h;
      if (k == l) {
        h = 2 * c3(ak, r) * c3(ak, s) + (r == s ? (fdot(ak, ak) - 1) : 0.0);
        for (int kk = 1; kk < 4; ++kk)
          if (kk != k) h += q[3 * kk + r] * q[3 * kk + s];
      } else {
        d3 al = mk(q[3 * l], q[3 * l + 1], q[3 * l + 2]);
        h = (r == s ? fdot(al, ak) : 0.0) + c3(al, r) * c3(ak, s);
      }
      val += h * kap * dt * dt;
    }
  } else {
    double og = 0.0;
    if (k >= 1) {
      d3 ak = mk(q[3 * k], q[3 * k + 1], q[3 * k + 2]);
      for (int jj = 1; jj < 4; ++jj) {
        d3 aj = mk(q[3 * jj], q[3 * jj + 1], q[3 * jj + 2]);
        og += (fdot(ak, aj) - (jj == k ? 1.0 : 0.0)) * c3(aj, r);
      }
      og *= kap;
    }
    double qt = g.q0[12 * b + i] + dt * g.dqdt[12 * b + i];
    if (i == 1) qt += dt * dt * P.gravity_y;
    val = dt * dt * og + mi * (q[i] - qt);
  }
  // vertex-ground terms (barrier.cpp:31-69, friction with basis (e_x, e_z))
  BarrierP bp{P.dhat, P.kappa};
  for (int kk = vg_seg[b]; kk < vg_seg[b + 1]; ++kk) {
    int v = g.v_off[b] + vg[2 * kk + 1];
    double py = g.X[g.nv + v];
    double _d = py + P.ground_offset;
    double dd = _d * _d;
    if (!(dd < P.dhat)) {
      if (t == 0) vg_lam[kk] = 0.0;
      continue;
    }
    double b1 = barrier_b1(dd, bp), b2 = barrier_b2(dd, bp);
    double lamv = -b1 * 2 * _d;
    if (t == 0) vg_lam[kk] = lamv;
    double xt[4] = {1.0, g.rest[3 * v], g.rest[3 * v + 1], g.rest[3 * v + 2]};
    double uk[2] = {g.X[v] - g.X0[v], g.X[2 * g.nv + v] - g.X0[2 * g.nv + v]};
    double gs = 0.0, M[2][2] = {{0, 0}, {0, 0}};
    if (P.vg_fric) friction_2x2(uk, lamv, FrictionP{P.mu, P.epsv, P.max_uk}, gs, M);
    if (is_h) {
      double N = 0.0;
      if (r == 1 && s == 1) N = b2 * (2 * _d) * (2 * _d);
      int rr = (r == 0) ? 0 : (r == 2 ? 1 : -1), ss = (s == 0) ? 0 : (s == 2 ? 1 : -1);
      if (rr >= 0 && ss >= 0) N += M[rr][ss];
      val += xt[k] * xt[l] * N;
    } else {
      double F = 0.0;
      if (r == 1) F = b1 * 2 * _d;
      if (r == 0) F += gs * uk[0];
      if (r == 2) F += gs * uk[1];
      val += xt[k] * F;
    }
  }
  // contact partial sums of the overlaps this body takes part in
  for (int e = row_ptr[b]; e < row_ptr[b + 1]; ++e) {
    int u = upidx[e];
    if (u < 0 || !has[u]) continue;
    const double* rec = ovr + (size_t)u * CONTRIB;
    bool isI = col[e] > b;
    if (is_h) val += rec[(isI ? 0 : 144) + t];
    else val += rec[(isI ? 432 : 444) + i];
  }
  if (is_h) D[144 * b + t] = val;
  else grad[12 * b + i] = val;
}

// Inverse of each SPD diagonal block via Cholesky (block-Jacobi preconditioner).
__global__ void k_block_inverse(int nb, const double* D, double* Dinv, int* status) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  double L[12][12];
  for (int i = 0; i < 12; ++i)
    for (int j = 0; j < 12; ++j) L[i][j] = 0.5 * (D[144 * b + 12 * i + j] + D[144 * b + 12 * j + i]);
  for (int j = 0; j < 12; ++j) {
    double s = L[j][j];
    for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
    if (!(s > 0)) {
      atomicExch(status, (int)ABD_ERR_NOT_SPD);
      s = 1e-300;
    }
    double l = sqrt(s);
    L[j][j] = l;
    for (int i = j + 1; i < 12; ++i) {
      double t = L[i][j];
      for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
      L[i][j] = t / l;
    }
  }
  // inverse of L (lower), then Dinv = L^-T L^-1
  double Li[12][12];
  for (int i = 0; i < 12; ++i)
    for (int j = 0; j < 12; ++j) Li[i][j] = 0.0;
  for (int c = 0; c < 12; ++c) {
    for (int i = 0; i < 12; ++i) {
      double t = (i == c) ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) t -= L[i][k] * Li[k][c];
      Li[i][c] = t / L[i][i];
    }
  }
  for (int i = 0; i < 12; ++i)
    for (int j = 0; j < 12; ++j) {
      double s = 0;
      for (int k = (i > j ? i : j); k < 12; ++k) s += Li[k][i] * Li[k][j];
      Dinv[144 * b + 12 * i + j] = s;
    }
}

// ---------------------------------------------------------------------------------
// Block-Jacobi PCG, one cooperative launch; slots (body, row) in groups of 16 lanes so
// the 12 rows of a body always sit in one warp.
struct PcgArgs {
  int nb;
  const int *row_ptr, *col, *upidx, *has;
  const double *ovr, *D, *Dinv, *b;
  double *x, *r, *z, *p, *q, *partial, *dq;
  double tol2;
  int maxit;
  int* out;  // [0] status, [1] iterations
};

__device__ __forceinline__ double row_spmv(const PcgArgs& a, int body, int row, const double* v) {
  double s = 0.0;
  const double* Db = a.D + 144 * body + 12 * row;
  const double* vb = v + 12 * body;
#pragma unroll
  for (int c = 0; c < 12; ++c) s += Db[c] * vb[c];
  for (int e = a.row_ptr[body]; e < a.row_ptr[body + 1]; ++e) {
    int u = a.upidx[e];
    if (u < 0 || !a.has[u]) continue;
    int cb = a.col[e];
    const double* B = a.ovr + (size_t)u * CONTRIB + 288;
    const double* vc = v + 12 * cb;
    if (cb > body) {
#pragma unroll
      for (int c = 0; c < 12; ++c) s += B[12 * row + c] * vc[c];
    } else {
#pragma unroll
      for (int c = 0; c < 12; ++c) s += B[12 * c + row] * vc[c];
    }
  }
  return s;
}

__device__ __forceinline__ void block_sum2(double& a, double& b, double* sh) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    sh[2 * w] = a;
    sh[2 * w + 1] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0, sb = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      sa += sh[2 * i];
      sb += sh[2 * i + 1];
    }
    a = sa;
    b = sb;
  }
}

// Sums the per-block partials of one slot in a fixed order; result broadcast to the block.
__device__ __forceinline__ void grid_sum2(const double* part, double& a, double& b, double* sh) {
  if (threadIdx.x < 32) {
    int lane = threadIdx.x;
    double sa = 0, sb = 0;
    for (int i = lane; i < (int)gridDim.x; i += 32) {
      sa += part[2 * i];
      sb += part[2 * i + 1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sa += __shfl_xor_sync(0xffffffffu, sa, o);
      sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    if (lane == 0) {
      sh[64] = sa;
      sh[65] = sb;
    }
  }
  __syncthreads();
  a = sh[64];
  b = sh[65];
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_pcg(PcgArgs a) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double sh[80];
  const int nslot = a.nb * 16;
  const int nthr = gridDim.x * blockDim.x;
  const int nloop = (nslot + nthr - 1) / nthr;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double* P0 = a.partial;                       // slot 0: (rz, bb)
  double* P1 = a.partial + 2 * gridDim.x;       // slot 1: (pq, -)
  double* P2 = a.partial + 4 * gridDim.x;       // slot 2: (rr, rz)
  // init: x = 0, r = b, z = M^-1 b, p = z
  double l0 = 0, l1 = 0;
  for (int it = 0; it < nloop; ++it) {
    int s = tid + it * nthr;
    int body = s >> 4, row = s & 15;
    if (s < nslot && row < 12) {
      int idx = 12 * body + row;
      double bv = a.b[idx];
      a.x[idx] = 0.0;
      a.r[idx] = bv;
      const double* Mi = a.Dinv + 144 * body + 12 * row;
      double zv = 0;
#pragma unroll
      for (int c = 0; c < 12; ++c) zv += Mi[c] * a.b[12 * body + c];
      a.z[idx] = zv;
      a.p[idx] = zv;
      l0 += bv * zv;
      l1 += bv * bv;
    }
  }
  block_sum2(l0, l1, sh);
  if (threadIdx.x == 0) {
    P0[2 * blockIdx.x] = l0;
    P0[2 * blockIdx.x + 1] = l1;
  }
  grid.sync();
  double rz, bb;
  grid_sum2(P0, rz, bb, sh);
  int iters = 0;
  bool conv = (bb == 0.0);
  for (int k = 0; k < a.maxit && !conv; ++k) {
    double lp = 0, dummy = 0;
    for (int it = 0; it < nloop; ++it) {
      int s = tid + it * nthr;
      int body = s >> 4, row = s & 15;
      if (s < nslot && row < 12) {
        int idx = 12 * body + row;
        double qv = row_spmv(a, body, row, a.p);
        a.q[idx] = qv;
        lp += a.p[idx] * qv;
      }
    }
    block_sum2(lp, dummy, sh);
    if (threadIdx.x == 0) {
      P1[2 * blockIdx.x] = lp;
      P1[2 * blockIdx.x + 1] = 0.0;
    }
    grid.sync();
    double pq;
    grid_sum2(P1, pq, dummy, sh);
    double alpha = rz / pq;
    double lrr = 0, lrz = 0;
    for (int it = 0; it < nloop; ++it) {
      int s = tid + it * nthr;
      int body = s >> 4, row = s & 15;
      bool act = s < nslot && row < 12;
      int idx = 12 * body + row;
      if (act) {
        a.x[idx] += alpha * a.p[idx];
        a.r[idx] -= alpha * a.q[idx];
      }
      __syncwarp();
      if (act) {
        const double* Mi = a.Dinv + 144 * body + 12 * row;
        double zv = 0;
#pragma unroll
        for (int c = 0; c < 12; ++c) zv += Mi[c] * a.r[12 * body + c];
        a.z[idx] = zv;
        double rv = a.r[idx];
        lrr += rv * rv;
        lrz += rv * zv;
      }
    }
    block_sum2(lrr, lrz, sh);
    if (threadIdx.x == 0) {
      P2[2 * blockIdx.x] = lrr;
      P2[2 * blockIdx.x + 1] = lrz;
    }
    grid.sync();
    double rr, rzn;
    grid_sum2(P2, rr, rzn, sh);
    iters = k + 1;
    if (!(rr > a.tol2 * bb)) {
      conv = true;
      break;
    }
    double beta = rzn / rz;
    rz = rzn;
    for (int it = 0; it < nloop; ++it) {
      int s = tid + it * nthr;
      int body = s >> 4, row = s & 15;
      if (s < nslot && row < 12) {
        int idx = 12 * body + row;
        a.p[idx] = a.z[idx] + beta * a.p[idx];
      }
    }
    grid.sync();
  }
  // dq = -x
  for (int it = 0; it < nloop; ++it) {
    int s = tid + it * nthr;
    int body = s >> 4, row = s & 15;
    if (s < nslot && row < 12) a.dq[12 * body + row] = -a.x[12 * body + row];
  }
  if (tid == 0) {
    a.out[1] = iters;
    if (!conv) a.out[0] = ABD_ERR_PCG_NOCONV;
  }
}

// ---------------------------------------------------------------------------------
// Line-search energies over a virtual index range; per-CTA partials, fixed-order sum.
struct EnergyArgs {
  int nb, npt, nee, nvg, lpt, lee, lvg;
  double alpha;
  int with_bi;
  const int *pt, *ee, *vg, *lpt_t, *lee_t, *lvg_t;
  const double *lpt_lag, *lee_lag, *lvg_lam;
  double* partial;
};

__device__ double inertia_energy(const Geo& g, const Params& P, int b, double alpha) {
  double m = g.mass[b];
  if (m < 0.0) return 0.0;
  double q[12];
  for (int i = 0; i < 12; ++i) q[i] = XA(g.q[12 * b + i], XM(g.dq[12 * b + i], alpha));
  double E = 0.0;
  for (int i = 1; i < 4; ++i)
    for (int j = 1; j < 4; ++j) {
      double e = q[3 * i] * q[3 * j] + q[3 * i + 1] * q[3 * j + 1] + q[3 * i + 2] * q[3 * j + 2] - (i == j ? 1.0 : 0.0);
      E += e * e;
    }
  E *= P.ortho_kappa;
  double dt = P.dt, pp = 0, rr = 0;
  for (int i = 0; i < 12; ++i) {
    double qt = g.q0[12 * b + i] + dt * g.dqdt[12 * b + i];
    if (i == 1) qt += dt * dt * P.gravity_y;
    double dd = q[i] - qt;
    if (i < 3) pp += dd * dd;
    else rr += dd * dd;
  }
  return E * dt * dt + 0.5 * (pp * m + rr * g.Ic[b]);
}

__device__ __forceinline__ void pair_vids(const Geo& g, int kind, const int* tup, int p, int* vid) {
  int A = tup[4 * p], a = tup[4 * p + 1], B = tup[4 * p + 2], b = tup[4 * p + 3];
  if (kind == 0) {
    vid[0] = g.v_off[A] + a;
    int f = g.f_off[B] + b;
    vid[1] = g.fv[3 * f]; vid[2] = g.fv[3 * f + 1]; vid[3] = g.fv[3 * f + 2];
  } else {
    int ea = g.e_off[A] + a, eb = g.e_off[B] + b;
    vid[0] = g.ev[2 * ea]; vid[1] = g.ev[2 * ea + 1]; vid[2] = g.ev[2 * eb]; vid[3] = g.ev[2 * eb + 1];
  }
}

__global__ void __launch_bounds__(256) k_energy(Geo g, Params P, EnergyArgs a) {
  __shared__ double sh[80];
  long long total = (long long)(a.with_bi ? a.nb + a.npt + a.nee + a.nvg : 0) + a.lpt + a.lee + a.lvg;
  double acc = 0.0;
  BarrierP bp{P.dhat, P.kappa};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    long long i = t;
    if (a.with_bi) {
      if (i < a.nb) { acc += inertia_energy(g, P, (int)i, a.alpha); continue; }
      i -= a.nb;
      if (i < a.npt) {
        if (P.pt) {
          int vid[4];
          pair_vids(g, 0, a.pt, (int)i, vid);
          d3 X0 = ldX(g.X, g.nv, vid[0]), X1 = ldX(g.X, g.nv, vid[1]), X2 = ldX(g.X, g.nv, vid[2]),
             X3 = ldX(g.X, g.nv, vid[3]);
          int ty = pt_type(X0, X1, X2, X3);
          acc += barrier_b(pt_dist(X0, X1, X2, X3, ty), bp);
        }
        continue;
      }
      i -= a.npt;
      if (i < a.nee) {
        if (P.ee) {
          int vid[4];
          pair_vids(g, 1, a.ee, (int)i, vid);
          d3 X0 = ldX(g.X, g.nv, vid[0]), X1 = ldX(g.X, g.nv, vid[1]), X2 = ldX(g.X, g.nv, vid[2]),
             X3 = ldX(g.X, g.nv, vid[3]);
          d3 u = fsub(X1, X0), v = fsub(X3, X2);
          double eps_x = fdot(fsub(X0, X1), fsub(X0, X1)) * fdot(fsub(X2, X3), fsub(X2, X3)) * P.eps_x;
          d3 cr = fcross(u, v);
          double x = fdot(cr, cr);
          double m = 1.0;
          if (x < eps_x) {
            double xe = x / eps_x;
            m = (-xe + 2.0) * xe;
          }
          int ty = ee_type(X0, X1, X2, X3);
          acc += barrier_b(ee_dist(X0, X1, X2, X3, ty), bp) * m;
        }
        continue;
      }
      i -= a.nee;
      if (i < a.nvg) {
        if (P.ground) {
          int b = a.vg[2 * i], v = g.v_off[b] + a.vg[2 * i + 1];
          double d = XA(g.X[g.nv + v], P.ground_offset);
          d = XM(d, d);
          if (d < P.dhat) acc += barrier_b(d, bp);
        }
        continue;
      }
      i -= a.nvg;
    }
    // lagged friction
    if (i < a.lpt || (i >= a.lpt && i < a.lpt + a.lee)) {
      int kind = (i < a.lpt) ? 0 : 1;
      int n = kind ? a.lee : a.lpt;
      int p = (int)(kind ? i - a.lpt : i);
      bool on = kind ? (P.ee && P.ee_fric) : (P.pt && P.pt_fric);
      if (!on) continue;
      const double* L = kind ? a.lee_lag : a.lpt_lag;
      int vid[4];
      pair_vids(g, kind, kind ? a.lee_t : a.lpt_t, p, vid);
      d3 c0 = fd3(L[0 * n + p], L[1 * n + p], L[2 * n + p]), c1 = fd3(L[3 * n + p], L[4 * n + p], L[5 * n + p]);
      double u0 = 0, u1 = 0;
      for (int k = 0; k < 4; ++k) {
        d3 du = fsub(ldX(g.X, g.nv, vid[k]), ldX(g.X0, g.nv, vid[k]));
        double gm = L[(6 + k) * n + p];
        u0 += gm * fdot(c0, du);
        u1 += gm * fdot(c1, du);
      }
      acc += P.mu * L[10 * n + p] * f0_SF(sqrt(u0 * u0 + u1 * u1), P.epsv);
      continue;
    }
    i -= a.lpt + a.lee;
    if (i < a.lvg) {
      if (!(P.ground && P.vg_fric)) continue;
      int b = a.lvg_t[2 * i], v = g.v_off[b] + a.lvg_t[2 * i + 1];
      double dx = g.X[v] - g.X0[v], dz = g.X[2 * g.nv + v] - g.X0[2 * g.nv + v];
      acc += P.mu * a.lvg_lam[i] * f0_SF(sqrt(dx * dx + dz * dz), P.epsv);
    }
  }
  double dummy = 0;
  block_sum2(acc, dummy, sh);
  if (threadIdx.x == 0) a.partial[blockIdx.x] = acc;
}

__global__ void k_final_sum(const double* part, int n, double* out) {
  __shared__ double sh[32];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
    *out = t;
  }
}

__global__ void k_dots(int n, const double* a, const double* b, double* part) {
  __shared__ double sh[80];
  double s0 = 0, s1 = 0, s2 = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    s0 += a[i] * b[i];
    s1 += b[i] * b[i];
    s2 += a[i] * a[i];
  }
  double t = s2;
  block_sum2(s0, s1, sh);
  __syncthreads();
  double d = 0;
  block_sum2(t, d, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = s0;
    part[3 * blockIdx.x + 1] = s1;
    part[3 * blockIdx.x + 2] = t;
  }
}
__global__ void k_dots_final(const double* part, int nblocks, double* out) {
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0;
    for (int i = 0; i < nblocks; ++i) {
      a += part[3 * i];
      b += part[3 * i + 1];
      c += part[3 * i + 2];
    }
    out[0] = a;
    out[1] = b;
    out[2] = c;
  }
}

__global__ void k_scale(double* v, int n, double s) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = XM(v[i], s);
}
__global__ void k_q_update(double* q, const double* dq, int n, double alpha) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = XA(q[i], XM(dq[i], alpha));
}
__global__ void k_frame_end(double* q, double* q0, double* dqdt, int n, double dt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    dqdt[i] = XD(XS(q[i], q0[i]), dt);
    q0[i] = q[i];
  }
}
__global__ void k_copy(double* d, const double* s, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = s[i];
}

}  // namespace

void assemble(const Geo& g, const Params& P, PairSet& S, NewtonBufs& B, cudaStream_t s) {
  int nb = g.nb, npt = S.npt, nee = S.nee, nov = S.nov;
  B.pt_c.ensure((size_t)CONTRIB * npt + 1);
  B.ee_c.ensure((size_t)CONTRIB * nee + 1);
  S.pt_lag.ensure(11 * (size_t)npt + 1);
  S.ee_lag.ensure(11 * (size_t)nee + 1);
  S.vg_lam.ensure((size_t)S.nvg + 1);
  B.pt_seg.ensure(nov + 2);
  B.ee_seg.ensure(nov + 2);
  B.ovr.ensure((size_t)CONTRIB * nov + 1);
  B.has.ensure(nov + 1);
  B.D.ensure(144 * (size_t)nb);
  B.Dinv.ensure(144 * (size_t)nb);
  B.grad.ensure(12 * (size_t)nb);
  // pair terms: tuple 20 B + 4 world and 4 rest positions 192 B + lagged friction 200 B
  prof_work(K_PAIR_TERMS, (double)npt + nee, 412.0 * ((double)npt + nee));
  prof_work(K_OV_REDUCE, nov, 2.0 * 1152 * nov);
  prof_work(K_BODY_SYSTEM, nb, 2.0 * 1152 * nb + 2 * 96.0 * nb);
  if (npt) {
    KLAUNCH(K_PAIR_TERMS, s, k_pair_terms<<<nblk(npt, 128), 128, 0, s>>>(g, P, 0, npt, S.pt.p, S.pt_ov.p, S.ovI.p, B.pt_c.p, S.pt_lag.p));
  }
  if (nee) {
    KLAUNCH(K_PAIR_TERMS, s, k_pair_terms<<<nblk(nee, 128), 128, 0, s>>>(g, P, 1, nee, S.ee.p, S.ee_ov.p, S.ovI.p, B.ee_c.p, S.ee_lag.p));
  }
  if (nov) {
    KLAUNCH(K_SEG, s, k_seg<<<nblk(nov + 1, 256), 256, 0, s>>>(nov, npt, S.pt_ov.p, B.pt_seg.p));
    KLAUNCH(K_SEG, s, k_seg<<<nblk(nov + 1, 256), 256, 0, s>>>(nov, nee, S.ee_ov.p, B.ee_seg.p));
    KLAUNCH(K_OV_REDUCE, s, k_ov_reduce<<<nov, 256, 0, s>>>(nov, B.pt_seg.p, B.ee_seg.p, B.pt_c.p, npt, B.ee_c.p, nee, B.ovr.p, B.has.p));
  }
  KLAUNCH(K_BODY_SYSTEM, s, k_body_system<<<nb, 160, 0, s>>>(g, P, S.row_ptr.p, S.col.p, S.upidx.p, B.ovr.p, B.has.p, S.vg.p, S.vg_seg.p,
                                   S.vg_lam.p, B.D.p, B.grad.p));
}

int pcg_solve(const Geo& g, PairSet& S, NewtonBufs& B, double rel_tol, int max_iter, double* dq, cudaStream_t s,
              int* status) {
  int nb = g.nb;
  B.status.ensure(4);
  if (!B.h_int) CK(cudaMallocHost(&B.h_int, 16 * sizeof(int)));
  CK(cudaMemsetAsync(B.status.p, 0, 4 * sizeof(int), s));
  KLAUNCH(K_BLOCK_INVERSE, s, k_block_inverse<<<nblk(nb, 64), 64, 0, s>>>(nb, B.D.p, B.Dinv.p, B.status.p));
  B.x.ensure(12 * (size_t)nb);
  B.r.ensure(12 * (size_t)nb);
  B.z.ensure(12 * (size_t)nb);
  B.p.ensure(12 * (size_t)nb);
  B.qv.ensure(12 * (size_t)nb);
  static int max_blocks = 0;
  if (!max_blocks) {
    int dev, sms, per;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg, 256, 0));
    max_blocks = sms * (per > 0 ? per : 1);
  }
  int want = nblk((long long)nb * 16, 256);
  int grid = want < max_blocks ? want : max_blocks;
  if (grid < 1) grid = 1;
  B.partial.ensure(6 * (size_t)grid + 8);
  PcgArgs a;
  a.nb = nb;
  a.row_ptr = S.row_ptr.p;
  a.col = S.col.p;
  a.upidx = S.upidx.p;
  a.has = B.has.p;
  a.ovr = B.ovr.p;
  a.D = B.D.p;
  a.Dinv = B.Dinv.p;
  a.b = B.grad.p;
  a.x = B.x.p;
  a.r = B.r.p;
  a.z = B.z.p;
  a.p = B.p.p;
  a.q = B.qv.p;
  a.partial = B.partial.p;
  a.dq = dq;
  a.tol2 = rel_tol * rel_tol;
  a.maxit = max_iter;
  a.out = B.status.p;
  void* args[] = {&a};
  KLAUNCH(K_PCG, s, CK(cudaLaunchCooperativeKernel((void*)k_pcg, dim3(grid), dim3(256), args, 0, s)));
  CK(cudaMemcpyAsync(B.h_int, B.status.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *status = B.h_int[0];
  // per iteration: the block matrix once (1152 B per block) and ~6 vector streams
  prof_work(K_PCG, B.h_int[1], B.h_int[1] * (1152.0 * (nb + 2.0 * S.nov) + 6 * 96.0 * nb) + 1152.0 * nb);
  return B.h_int[1];
}

double energy(const Geo& g, const Params& P, double alpha, PairSet& Snew, PairSet& Slag, bool with_bi,
              NewtonBufs& B, cudaStream_t s) {
  EnergyArgs a;
  a.nb = g.nb;
  a.npt = Snew.npt;
  a.nee = Snew.nee;
  a.nvg = Snew.nvg;
  a.lpt = Slag.npt;
  a.lee = Slag.nee;
  a.lvg = Slag.nvg;
  a.alpha = alpha;
  a.with_bi = with_bi ? 1 : 0;
  a.pt = Snew.pt.p;
  a.ee = Snew.ee.p;
  a.vg = Snew.vg.p;
  a.lpt_t = Slag.pt.p;
  a.lee_t = Slag.ee.p;
  a.lvg_t = Slag.vg.p;
  a.lpt_lag = Slag.pt_lag.p;
  a.lee_lag = Slag.ee_lag.p;
  a.lvg_lam = Slag.vg_lam.p;
  const int G = 512;
  B.red.ensure(G + 8);
  a.partial = B.red.p;
  if (!B.h_red) CK(cudaMallocHost(&B.h_red, 16 * sizeof(double)));
  prof_work(K_ENERGY, (double)a.npt + a.nee + a.lpt + a.lee,
            136.0 * ((double)a.npt + a.nee + a.lpt + a.lee) + 96.0 * g.nb);
  KLAUNCH(K_ENERGY, s, k_energy<<<G, 256, 0, s>>>(g, P, a));
  KLAUNCH(K_ENERGY, s, k_final_sum<<<1, 256, 0, s>>>(B.red.p, G, B.red.p + G));
  CK(cudaMemcpyAsync(B.h_red, B.red.p + G, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return B.h_red[0];
}

void dots(int n, const double* dq, const double* grad, NewtonBufs& B, double* out, cudaStream_t s) {
  const int G = 64;
  B.red.ensure(3 * G + 8);
  if (!B.h_red) CK(cudaMallocHost(&B.h_red, 16 * sizeof(double)));
  KLAUNCH(K_DOTS, s, k_dots<<<G, 256, 0, s>>>(n, dq, grad, B.red.p));
  KLAUNCH(K_DOTS, s, k_dots_final<<<1, 32, 0, s>>>(B.red.p, G, B.red.p + 3 * G));
  CK(cudaMemcpyAsync(B.h_red, B.red.p + 3 * G, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  out[0] = B.h_red[0];
  out[1] = B.h_red[1];
  out[2] = B.h_red[2];
}

void launch_scale(double* v, int n, double sc, cudaStream_t st) {
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_scale<<<nblk(n, 256), 256, 0, st>>>(v, n, sc));
}
void launch_q_update(double* q, const double* dq, int n, double alpha, cudaStream_t st) {
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_q_update<<<nblk(n, 256), 256, 0, st>>>(q, dq, n, alpha));
}
void launch_frame_end(double* q, double* q0, double* dqdt, int n, double dt, cudaStream_t st) {
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_frame_end<<<nblk(n, 256), 256, 0, st>>>(q, q0, dqdt, n, dt));
}
void launch_copy(double* d, const double* s_, int n, cudaStream_t st) {
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_copy<<<nblk(n, 256), 256, 0, st>>>(d, s_, n));
}

}  // namespace abd
