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
// Pairs are processed grouped by distance type (PT: 0-6, EE: 0-8), so that a warp runs
// one branch of the type-dependent code (stencil, friction frame) and one projection
// size (the stencil's parameter count m = 0, 1, 2 follows from the type). Mollified
// edge-edge pairs (near-parallel edges, the full 9x9 projection) form a class of their
// own, so their long projections occupy a few warps instead of slowing many.
constexpr int NCLS = 10;
constexpr int CLS_T = 256;

__device__ __forceinline__ int pair_class(const Geo& g, const Params& P, int kind, const int* tup, const int8_t* ty,
                                          int p);

// Pairs per class in each block of CLS_T pairs: cnt[class * nblk + block].
__global__ void k_class_count(Geo g, Params P, int kind, int n, const int* tup, const int8_t* ty, int* cnt) {
  __shared__ int sc[NCLS];
  if (threadIdx.x < NCLS) sc[threadIdx.x] = 0;
  __syncthreads();
  int p = blockIdx.x * CLS_T + threadIdx.x;
  if (p < n) atomicAdd(&sc[pair_class(g, P, kind, tup, ty, p)], 1);
  __syncthreads();
  if (threadIdx.x < NCLS) cnt[threadIdx.x * gridDim.x + blockIdx.x] = sc[threadIdx.x];
}

// Stable partition of the pairs by class (offsets from the scan of k_class_count).
__global__ void k_class_scatter(Geo g, Params P, int kind, int n, const int* tup, const int8_t* ty, const int* off,
                                int* perm) {
  __shared__ int wc[NCLS][CLS_T / 32];
  const int p = blockIdx.x * CLS_T + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = p < n ? pair_class(g, P, kind, tup, ty, p) : -1;
  unsigned mine = 0;
#pragma unroll
  for (int k = 0; k < NCLS; ++k) {
    unsigned m = __ballot_sync(0xffffffffu, c == k);
    if (c == k) mine = m;
    if (lane == 0) wc[k][w] = __popc(m);
  }
  __syncthreads();
  if (c >= 0) {
    int r = off[c * gridDim.x + blockIdx.x] + __popc(mine & ((1u << lane) - 1u));
    for (int i = 0; i < w; ++i) r += wc[c][i];
    perm[r] = p;
  }
}

// Per-pair record between the two pair-term kernels (structure of arrays, stride = pairs):
// the reduced Hessian's upper triangle (45), the vertex gradient (12), the friction
// factors gh (3) and N (6, upper triangle) and an activity flag (1).
enum { REC_S = 0, REC_G = 45, REC_GH = 57, REC_N = 60, REC_ACT = 66, REC = 67 };

__device__ __forceinline__ void pair_vertices(const Geo& g, int kind, const int* tup, int p, int (&vid)[4], int& na,
                                              int& A, int& B) {
  A = tup[4 * p];
  B = tup[4 * p + 2];
  const int a = tup[4 * p + 1], b = tup[4 * p + 3];
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
}

// Class of a pair for the grouping above: 0 for an edge-edge pair inside the
// mollifier's range (the test of pair_reduced; first, so that their long projections
// start with the first CTAs and overlap the rest), else 1 + its distance type.
__device__ __forceinline__ int pair_class(const Geo& g, const Params& P, int kind, const int* tup, const int8_t* ty,
                                          int p) {
  int t = ty[p];
  t = 1 + (t < 0 ? 0 : (t > NCLS - 2 ? NCLS - 2 : t));
  if (kind == 1) {
    int vid[4], na, A, B;
    pair_vertices(g, kind, tup, p, vid, na, A, B);
    d3 x0 = ldX(g.X, g.nv, vid[0]), x1 = ldX(g.X, g.nv, vid[1]);
    d3 x2 = ldX(g.X, g.nv, vid[2]), x3 = ldX(g.X, g.nv, vid[3]);
    d3 u = fsub(x1, x0), v = fsub(x3, x2);
    double eps_x = P.eps_x * fdot(u, u) * fdot(v, v);
    d3 cr = fcross(u, v);
    if (fdot(cr, cr) < eps_x) t = 0;
  }
  return t;
}

// Per-pair terms, part 1 (kind 0: PT, point on body A, triangle on body B; 1: EE): the
// barrier's reduced Hessian and gradient, the lagged friction frame and the friction
// terms, written to the pair's record. Threads take pairs in stencil-class order (perm).
__global__ void __launch_bounds__(128) k_pair_hess(Geo g, Params P, int kind, int n, const int* tup,
                                                   const int8_t* tys, const int* perm, const int* n_moll, double* R,
                                                   double* lag) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n || (n_moll && t < *n_moll)) return;  // mollified pairs: k_pair_moll
  const int p = perm[t];
  int vid[4], na, A, B;
  pair_vertices(g, kind, tup, p, vid, na, A, B);
  if (!scene_on(g, A)) return;  // scene not iterating: its blocks are not used
  d3 X[4], X0[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    X[i] = ldX(g.X, g.nv, vid[i]);
    X0[i] = ldX(g.X0, g.nv, vid[i]);
  }
  // the distance type the cull classified at this same configuration
  const int ty = tys[p];
  const double d = kind == 0 ? pt_dist(X[0], X[1], X[2], X[3], ty) : ee_dist(X[0], X[1], X[2], X[3], ty);
  const size_t N = n;
  d3 gv[4];
  FrictionFrame fr;
  double lam = 0.0;
  const bool active = d < P.dhat;
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
    S9Rec rec{R + REC_S * N + p, N};
    pair_reduced(kind, ty, X, d, bp, P.eps_x, P.psd != 0, rec, gv);
    if (!(P.terms & TERM_BARRIER)) {
      for (int k = 0; k < 45; ++k) R[(REC_S + k) * N + p] = 0.0;
      for (int i = 0; i < 4; ++i) gv[i] = fd3(0, 0, 0);
    }
    double gh[3] = {0, 0, 0}, N6[6] = {0, 0, 0, 0, 0, 0};
    bool fric = ((kind == 0) ? P.pt_fric : P.ee_fric) && (P.terms & TERM_FRICTION);
    if (fric) pair_friction(fr, uk, lam, FrictionP{P.mu, P.epsv, P.max_uk}, gv, gh, N6);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      R[(REC_G + 3 * i) * N + p] = gv[i].x;
      R[(REC_G + 3 * i + 1) * N + p] = gv[i].y;
      R[(REC_G + 3 * i + 2) * N + p] = gv[i].z;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) R[(REC_GH + k) * N + p] = gh[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) R[(REC_N + k) * N + p] = N6[k];
  } else {
    fr.c0 = fd3(0, 0, 0);
    fr.c1 = fd3(0, 0, 0);
    for (int i = 0; i < 4; ++i) fr.gam[i] = 0;
  }
  R[REC_ACT * N + p] = active ? 1.0 : 0.0;
  // lagged friction record
  lag[0 * N + p] = fr.c0.x; lag[1 * N + p] = fr.c0.y; lag[2 * N + p] = fr.c0.z;
  lag[3 * N + p] = fr.c1.x; lag[4 * N + p] = fr.c1.y; lag[5 * N + p] = fr.c1.z;
  for (int i = 0; i < 4; ++i) lag[(6 + i) * N + p] = fr.gam[i];
  lag[10 * N + p] = lam;
}

// Per-pair terms, part 1 for mollified edge-edge pairs (the first *n_moll entries of
// perm): one warp per pair. Their 9x9 reduced Hessian has no low-rank structure, so it is
// built entry by entry across the lanes and projected by a cyclic Jacobi in shared
// memory whose rotations update the 9 rows in parallel (one lane each); a thread-serial
// 9x9 Jacobi in local memory kept a few warps busy long after the rest of the launch.
constexpr int MOLL_W = 4;  // warps (pairs) per CTA
__global__ void __launch_bounds__(32 * MOLL_W) k_pair_moll(Geo g, Params P, int n, const int* tup,
                                                           const int8_t* tys, const int* perm, const int* n_moll,
                                                           double* R, double* lag) {
  __shared__ double sA[MOLL_W][9][9], sV[MOLL_W][9][9];
  __shared__ MollData smd[MOLL_W];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int nm = *n_moll;
  double(&A)[9][9] = sA[wi];
  double(&V)[9][9] = sV[wi];
  for (int t = blockIdx.x * MOLL_W + wi; t < nm && t < n; t += gridDim.x * MOLL_W) {
    const int p = perm[t];
    int vid[4], na, Ab, Bb;
    pair_vertices(g, 1, tup, p, vid, na, Ab, Bb);
    if (!scene_on(g, Ab)) continue;
    d3 X[4], X0[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      X[i] = ldX(g.X, g.nv, vid[i]);
      X0[i] = ldX(g.X0, g.nv, vid[i]);
    }
    const int ty = tys[p];
    const double d = ee_dist(X[0], X[1], X[2], X[3], ty);
    const size_t N = n;
    const bool active = d < P.dhat;
    FrictionFrame fr;
    double lam = 0.0;
    if (active) {
      BarrierP bp{P.dhat, P.kappa};
      frame_ee(X, ty, fr);
      double uk[2] = {0.0, 0.0};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        d3 du = fsub(X[i], X0[i]);
        uk[0] += fr.gam[i] * fdot(fr.c0, du);
        uk[1] += fr.gam[i] * fdot(fr.c1, du);
      }
      lam = -barrier_b1(d, bp) * 2 * sqrt(d);
      Stencil st;
      d3 w, W[2], gu, gv;
      double Gi[2][2];
      MollData md;
      const bool moll = pair_setup(1, ty, X, d, bp, P.eps_x, st, w, W, Gi, md, gu, gv);
      if (lane == 0) smd[wi] = md;
      __syncwarp();
      // entries of S (upper triangle mirrored), lane e takes e, e + 32, e + 64
      double orig[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int e = lane + 32 * j;
        orig[j] = 0.0;
        if (e < 81) {
          const int pp = e / 9, qq = e % 9;
          double h;
          if (moll) {
            h = moll_entry(smd[wi], pp <= qq ? pp : qq, pp <= qq ? qq : pp);
          } else {  // not mollified at this configuration after all: reduced form
            h = 0.0;
          }
          A[pp][qq] = h;
          V[pp][qq] = pp == qq ? 1.0 : 0.0;
          orig[j] = h;
        }
      }
      __syncwarp();
      if (!moll) {
        // the class test saw a mollified pair but pair_setup does not: the thread path
        if (lane == 0) {
          S9Rec rec{R + REC_S * N + p, N};
          d3 gtmp[4];
          pair_reduced(1, ty, X, d, bp, P.eps_x, P.psd != 0, rec, gtmp);
        }
      } else {
        bool neg = false;
        if (P.psd) {
          for (int sweep = 0; sweep < 30; ++sweep) {
            double off = 0, tot = 0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const int e = lane + 32 * j;
              if (e < 81) {
                const double v = A[e / 9][e % 9];
                tot += v * v;
                if (e / 9 != e % 9) off += v * v;
              }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
              off += __shfl_xor_sync(0xffffffffu, off, o);
              tot += __shfl_xor_sync(0xffffffffu, tot, o);
            }
            if (off <= 1e-32 * tot || off == 0.0) break;
            for (int pp = 0; pp < 8; ++pp)
              for (int qq = pp + 1; qq < 9; ++qq) {
                const double apq = A[pp][qq];
                if (apq == 0.0) continue;
                const double app = A[pp][pp], aqq = A[qq][qq];
                const double gq = 100.0 * fabs(apq);
                if (sweep > 2 && fabs(app) + gq == fabs(app) && fabs(aqq) + gq == fabs(aqq)) {
                  __syncwarp();
                  if (lane == 0) A[pp][qq] = A[qq][pp] = 0.0;
                  __syncwarp();
                  continue;
                }
                // rotation parameters from two reciprocal square roots (g = 1 / r,
                // c^2 = (|h| + r) / (2 r), t = sgn(h) a g / (2 c^2), s = sgn(h) a g / (2 c)),
                // as in psd_project_small; by division below the normal range
                const double h = 0.5 * (aqq - app);
                const double sa = h >= 0 ? apq : -apq;
                const double r2 = fma(h, h, apq * apq);
                double tt, c, sn;
                if (r2 >= 1e-300) {
                  const double g = rsqrt(r2);
                  const double c2 = 0.5 * fma(r2, g, fabs(h)) * g;
                  const double ic = rsqrt(c2);
                  sn = 0.5 * sa * g * ic;
                  c = c2 * ic;
                  tt = sn * ic;
                } else {
                  const double den = fabs(h) + sqrt(r2);
                  tt = den > 0.0 ? sa / den : 0.0;
                  c = rsqrt(1.0 + tt * tt);
                  sn = tt * c;
                }
                __syncwarp();
                if (lane < 9 && lane != pp && lane != qq) {
                  const double akp = A[lane][pp], akq = A[lane][qq];
                  const double np_ = c * akp - sn * akq, nq = sn * akp + c * akq;
                  A[lane][pp] = np_;
                  A[pp][lane] = np_;
                  A[lane][qq] = nq;
                  A[qq][lane] = nq;
                }
                if (lane < 9) {
                  const double vkp = V[lane][pp], vkq = V[lane][qq];
                  V[lane][pp] = c * vkp - sn * vkq;
                  V[lane][qq] = sn * vkp + c * vkq;
                }
                if (lane == 0) {
                  A[pp][pp] = app - tt * apq;
                  A[qq][qq] = aqq + tt * apq;
                  A[pp][qq] = A[qq][pp] = 0.0;
                }
                __syncwarp();
              }
          }
#pragma unroll
          for (int i = 0; i < 9; ++i) neg |= A[i][i] < 0.0;
        }
        // S+ = V max(lam, 0) V^T (or S itself when no eigenvalue is negative), upper triangle
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int e = lane + 32 * j;
          if (e < 81) {
            const int pp = e / 9, qq = e % 9;
            if (pp <= qq) {
              double v = orig[j];
              if (neg) {
                v = 0.0;
                for (int k = 0; k < 9; ++k) {
                  const double lk = A[k][k];
                  if (lk > 0) v += V[pp][k] * lk * V[qq][k];
                }
              }
              R[(REC_S + s9_index(pp, qq)) * N + p] = v;
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) {
        d3 gvv[4];
        pair_gradient(st, w, md, gu, gv, gvv);
        if (!(P.terms & TERM_BARRIER)) {
          for (int k = 0; k < 45; ++k) R[(REC_S + k) * N + p] = 0.0;
          for (int i = 0; i < 4; ++i) gvv[i] = fd3(0, 0, 0);
        }
        double gh[3] = {0, 0, 0}, N6[6] = {0, 0, 0, 0, 0, 0};
        if (P.ee_fric && (P.terms & TERM_FRICTION)) pair_friction(fr, uk, lam, FrictionP{P.mu, P.epsv, P.max_uk}, gvv, gh, N6);
        for (int i = 0; i < 4; ++i) {
          R[(REC_G + 3 * i) * N + p] = gvv[i].x;
          R[(REC_G + 3 * i + 1) * N + p] = gvv[i].y;
          R[(REC_G + 3 * i + 2) * N + p] = gvv[i].z;
        }
        for (int k = 0; k < 3; ++k) R[(REC_GH + k) * N + p] = gh[k];
        for (int k = 0; k < 6; ++k) R[(REC_N + k) * N + p] = N6[k];
      }
    } else {
      fr.c0 = fd3(0, 0, 0);
      fr.c1 = fd3(0, 0, 0);
      for (int i = 0; i < 4; ++i) fr.gam[i] = 0;
    }
    if (lane == 0) {
      R[REC_ACT * N + p] = active ? 1.0 : 0.0;
      lag[0 * N + p] = fr.c0.x; lag[1 * N + p] = fr.c0.y; lag[2 * N + p] = fr.c0.z;
      lag[3 * N + p] = fr.c1.x; lag[4 * N + p] = fr.c1.y; lag[5 * N + p] = fr.c1.z;
      for (int i = 0; i < 4; ++i) lag[(6 + i) * N + p] = fr.gam[i];
      lag[10 * N + p] = lam;
    }
    __syncwarp();
  }
}

// Per-pair body-space record (structure of arrays, stride = pairs): the two diagonal
// blocks as upper triangles (78 entries each, row-major over row <= col), the
// off-diagonal block (144, row-major, block (I, J)) and the two gradients (12 each).
enum { PC_DJ = 78, PC_OFF = 156, PC_GI = 300, PC_GJ = 312, PAIRC = 324 };
__host__ __device__ constexpr int sym12(int i, int j) { return i * 12 - (i * (i - 1)) / 2 + (j - i); }  // i <= j
// upper-triangle index of entry (row, col) = e / 12, e % 12 of a symmetric 12 x 12 block
struct Sym12Table {
  unsigned char v[144];
  constexpr Sym12Table() : v() {
    for (int e = 0; e < 144; ++e) {
      const int i = e / 12, j = e % 12;
      v[e] = (unsigned char)(i <= j ? sym12(i, j) : sym12(j, i));
    }
  }
};
__constant__ Sym12Table c_sym12 = Sym12Table();

// Per-pair terms, part 2: the chain rule onto the 12 affine DOFs of the two bodies,
// d_A = Y_A S Y_A^T, d_B = Y_B S Y_B^T, off = Y_A S Y_B^T with Y_b[k][a] = sum over the
// pair's vertices i on body b of xbar~_i[k] Q[i][a], and the body gradients.
// S is symmetric, so for r < s one 3x3 slice M = S[3a+r][3b+s] gives the (r, s) and
// (s, r) entries of all three blocks (d_A, d_B mirrored; off via M^T), and for r = s
// only k <= l is formed for d_A and d_B.
// Q's column 1 vanishes on vertices 0 and 1 and its column 0 on vertices 2 and 3, so
// Y_A's column 1 is zero for both kinds (body A holds vertex 0, and 1 for edge-edge) and
// Y_B's column 0 is zero for edge-edge pairs: those terms are left out (KIND 0:
// point-triangle, 1: edge-edge).
template <int KIND>
__global__ void __launch_bounds__(128) k_pair_chain(Geo g, int n, const int* tup, const int* pov,
                                                    const int* ovI, const double* R, double* C) {
  constexpr int kind = KIND;
  constexpr int na = KIND ? 2 : 1;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int vid[4], na_, A, B;
  pair_vertices(g, kind, tup, p, vid, na_, A, B);
  if (!scene_on(g, A)) return;
  const size_t N = n;
  const int I = ovI[pov[p]];
  const bool a_is_I = (A == I);
  const bool a_dyn = g.mass[A] > 0.0, b_dyn = g.mass[B] > 0.0;
  double* dI = C;
  double* dJ = C + PC_DJ * N;
  double* off = C + PC_OFF * N;
  double* gI = C + PC_GI * N;
  double* gJ = C + PC_GJ * N;
  double* dA = a_is_I ? dI : dJ;
  double* dB = a_is_I ? dJ : dI;
  double* gA = a_is_I ? gI : gJ;
  double* gB = a_is_I ? gJ : gI;
  if (R[REC_ACT * N + p] == 0.0) {
    for (int e = 0; e < 78; ++e) {
      dI[e * N + p] = 0.0;
      dJ[e * N + p] = 0.0;
    }
    for (int e = 0; e < 144; ++e) off[e * N + p] = 0.0;
    for (int e = 0; e < 12; ++e) {
      gI[e * N + p] = 0.0;
      gJ[e * N + p] = 0.0;
    }
    return;
  }
  double xt[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    xt[i][0] = 1.0;
    xt[i][1] = g.rest[3 * vid[i]];
    xt[i][2] = g.rest[3 * vid[i] + 1];
    xt[i][3] = g.rest[3 * vid[i] + 2];
  }
  // nonzero columns of Y_A and Y_B
  auto a_nz = [](int c) { return c != 1; };
  auto b_nz = [](int c) { return KIND == 0 || c != 0; };
  // Y matrices of the chain rule
  double YA[4][3], YB[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int aa = 0; aa < 3; ++aa) {
      double sa = 0, sb = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (Qe(i, aa) == 0.0) continue;  // a compile-time zero of Q
        double v = xt[i][k] * Qe(i, aa);
        if (i < na) sa += v;
        else sb += v;
      }
      YA[k][aa] = sa;
      YB[k][aa] = sb;
    }
  double gh[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) gh[k] = R[(REC_GH + k) * N + p];
  const bool off_on = a_dyn && b_dyn;
  // one (r, s) slice at a time keeps the live state to Y, T and M
#pragma unroll 1
  for (int nidx = 0; nidx < 6; ++nidx) {
    const int r = nidx < 3 ? 0 : (nidx < 5 ? 1 : 2);
    const int s = nidx < 3 ? nidx : (nidx < 5 ? nidx - 2 : 2);
    {
      const double Nrs = R[(REC_N + nidx) * N + p];
      double M[3][3];
#pragma unroll
      for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
          const int pp = 3 * aa + r, qq = 3 * bb + s;
          const int e = pp <= qq ? s9_index(pp, qq) : s9_index(qq, pp);
          M[aa][bb] = R[(REC_S + e) * N + p] + gh[aa] * gh[bb] * Nrs;
        }
      double TA[4][3], TB[4][3];
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
          double ta = 0.0, tb = 0.0;
          bool fa = true, fb = true;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            if (a_nz(c)) {
              ta = fa ? YA[k][c] * M[c][bb] : ta + YA[k][c] * M[c][bb];
              fa = false;
            }
            if (b_nz(c)) {
              tb = fb ? YB[k][c] * M[c][bb] : tb + YB[k][c] * M[c][bb];
              fb = false;
            }
          }
          TA[k][bb] = ta;
          TB[k][bb] = tb;
        }
      // u . v over the columns where Y (of `side`: 0 A, 1 B) is nonzero
      auto dotY = [&](const double (&u)[3], const double (&v)[3], int side) {
        double acc = 0.0;
        bool first = true;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (side == 0 ? !a_nz(c) : !b_nz(c)) continue;
          acc = first ? u[c] * v[c] : acc + u[c] * v[c];
          first = false;
        }
        return acc;
      };
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          const int e = (3 * k + r) * 12 + (3 * l + s);
          const int et = (3 * l + s) * 12 + (3 * k + r);
          if (r < s || k <= l) {
            double aa_ = dotY(TA[k], YA[l], 0);
            double bb_ = dotY(TB[k], YB[l], 1);
            const int ui = c_sym12.v[e];  // the same entry for the whole warp
            dA[ui * N + p] = a_dyn ? aa_ : 0.0;
            dB[ui * N + p] = b_dyn ? bb_ : 0.0;
          }
          // (A row (k, r), B column (l, s)), stored as block (I, J)
          double ab_ = dotY(TA[k], YB[l], 1);
          off[(a_is_I ? e : et) * N + p] = off_on ? ab_ : 0.0;
          if (r < s) {
            // (A row (k, s), B column (l, r)) = Y_A[k] M^T Y_B[l]^T
            const int e2 = (3 * k + s) * 12 + (3 * l + r);
            const int et2 = (3 * l + r) * 12 + (3 * k + s);
            double ba_ = dotY(TB[l], YA[k], 0);
            off[(a_is_I ? e2 : et2) * N + p] = off_on ? ba_ : 0.0;
          }
        }
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
        double v = xt[i][k] * R[(REC_G + 3 * i + r) * N + p];
        if (i < na) sa += v;
        else sb += v;
      }
      gA[(3 * k + r) * N + p] = a_dyn ? sa : 0.0;
      gB[(3 * k + r) * N + p] = b_dyn ? sb : 0.0;
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

// Per-overlap sums of the pair records: one CTA per overlap, one thread per record entry
// (CONTRIB of them, one pass with 512 threads), each adding the overlap's pairs in order.
__global__ void __launch_bounds__(512) k_ov_reduce(int nov, const int* pt_seg, const int* ee_seg, const double* ptC,
                                                   int npt, const double* eeC, int nee, double* ovr, int* has,
                                                   double off_scale) {
  int u = blockIdx.x;
  if (u >= nov) return;
  int p0 = pt_seg[u], p1 = pt_seg[u + 1], e0 = ee_seg[u], e1 = ee_seg[u + 1];
  if (threadIdx.x == 0) has[u] = (p1 > p0) || (e1 > e0);
  if (p1 == p0 && e1 == e0) return;  // no pairs: the record is never read (has[u] = 0)
  // one thread per record entry, summing the overlap's pairs in order (each thread streams
  // its own component row; no FP64 shuffle tree, which costs more than the sums on GB300)
  for (int c = threadIdx.x; c < PAIRC; c += blockDim.x) {
    double s = 0.0;
    const double* pr = ptC + (size_t)c * npt;
    const double* er = eeC + (size_t)c * nee;
    int p = p0;
    for (; p + 3 < p1; p += 4) {
      const double a0 = pr[p], a1 = pr[p + 1], a2 = pr[p + 2], a3 = pr[p + 3];
      s += a0;
      s += a1;
      s += a2;
      s += a3;
    }
    for (; p < p1; ++p) s += pr[p];
    int e = e0;
    for (; e + 3 < e1; e += 4) {
      const double a0 = er[e], a1 = er[e + 1], a2 = er[e + 2], a3 = er[e + 3];
      s += a0;
      s += a1;
      s += a2;
      s += a3;
    }
    for (; e < e1; ++e) s += er[e];
    // into the overlap record (CONTRIB layout: dI, dJ, off as full 12 x 12 blocks, gI,
    // gJ); a diagonal-block entry fills both of its mirrored positions; the off-diagonal
    // block takes the damping scale (1 + beta), like every matrix entry
    double* o = ovr + (size_t)u * CONTRIB;
    if (c < PC_OFF) {
      const int blk = c < PC_DJ ? 0 : 144, t = c < PC_DJ ? c : c - PC_DJ;
      int i = 0;
      while (sym12(i, 11) < t) ++i;
      const int j = i + (t - sym12(i, i));
      o[blk + 12 * i + j] = s;
      o[blk + 12 * j + i] = s;
    } else if (c < PC_GI) {
      o[288 + (c - PC_OFF)] = s * off_scale;
    } else {
      o[432 + (c - PC_GI)] = s;
    }
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
  const bool ent = t < 156;  // threads 156..159 only help with the vertex-ground pairs
  bool is_h = t < 144;
  int i = is_h ? t / 12 : t - 144;
  int j = is_h ? t % 12 : 0;
  int k = i / 3, r = i % 3, l = j / 3, s = j % 3;
  double m = g.mass[b];
  const double* q = g.q + 12 * b;
  double dt = P.dt;
  double val = 0.0;
  if (m < 0.0 || !scene_on(g, b)) {
    // static body: identity block, zero gradient (mutils.cpp:55-56, 70); bodies of scenes
    // that are not iterating get the same (their step is zero)
    if (!ent) return;
    if (is_h) {
      double v = (i == j) ? 1.0 : 0.0;
      // damping_sparse scales every body's block (mutils.cpp:106-115)
      if (P.damp) v = v * (1 + P.damp_beta) + ((i == j) ? (i < 3 ? m : g.Ic[b]) * (P.damp_alpha - P.damp_beta) : 0.0);
      D[144 * b + t] = v;
    } else {
      grad[12 * b + i] = 0.0;
    }
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
  if (!ent || !(P.terms & TERM_INERTIA)) {
    // no inertia / orthogonality terms (adjoint of the friction terms alone)
  } else if (is_h) {
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
  const bool vg_bar = (P.terms & TERM_BARRIER) != 0, vg_fr = (P.terms & TERM_FRICTION) && P.vg_fric;
  // vertex-ground terms (barrier.cpp:31-69, friction with basis (e_x, e_z)). The scalars
  // of each pair (barrier derivatives, friction factors) are computed once, by one thread
  // per pair, into shared memory; then every entry thread adds the pairs in order.
  constexpr int VGC = 160;
  __shared__ double s_n11[VGC], s_f1[VGC], s_g0[VGC], s_g2[VGC], s_M[VGC][4], s_xt[VGC][3];
  __shared__ int s_on[VGC];
  BarrierP bp{P.dhat, P.kappa};
  const int kb = vg_seg[b], ke = vg_seg[b + 1];
  for (int c0 = kb; c0 < ke; c0 += VGC) {
    const int cn = ke - c0 < VGC ? ke - c0 : VGC;
    __syncthreads();
    if (t < cn) {
      const int kk = c0 + t;
      int v = g.v_off[b] + vg[2 * kk + 1];
      double py = g.X[g.nv + v];
      double _d = py + P.ground_offset;
      double dd = _d * _d;
      const bool on = dd < P.dhat;
      s_on[t] = on;
      if (!on) {
        vg_lam[kk] = 0.0;
      } else {
        double b1 = barrier_b1(dd, bp), b2 = barrier_b2(dd, bp);
        double lamv = -b1 * 2 * _d;
        vg_lam[kk] = lamv;
        double uk[2] = {g.X[v] - g.X0[v], g.X[2 * g.nv + v] - g.X0[2 * g.nv + v]};
        double gs = 0.0, M[2][2] = {{0, 0}, {0, 0}};
        if (vg_fr) friction_2x2(uk, lamv, FrictionP{P.mu, P.epsv, P.max_uk}, gs, M);
        // the reference drops b' d'' = 2 b' from the ground Hessian (barrier.cpp:62-69);
        // the exact Hessian (adjoint systems) keeps it
        s_n11[t] = vg_bar ? b2 * (2 * _d) * (2 * _d) + (P.exact ? 2 * b1 : 0.0) : 0.0;
        s_f1[t] = vg_bar ? b1 * 2 * _d : 0.0;
        s_g0[t] = gs * uk[0];
        s_g2[t] = gs * uk[1];
        s_M[t][0] = M[0][0];
        s_M[t][1] = M[0][1];
        s_M[t][2] = M[1][0];
        s_M[t][3] = M[1][1];
        s_xt[t][0] = g.rest[3 * v];
        s_xt[t][1] = g.rest[3 * v + 1];
        s_xt[t][2] = g.rest[3 * v + 2];
      }
    }
    __syncthreads();
    if (ent)
      for (int q = 0; q < cn; ++q) {
        if (!s_on[q]) continue;
        const double xk = k == 0 ? 1.0 : s_xt[q][k - 1];
        if (is_h) {
          double N = 0.0;
          if (r == 1 && s == 1) N = s_n11[q];
          int rr = (r == 0) ? 0 : (r == 2 ? 1 : -1), ss = (s == 0) ? 0 : (s == 2 ? 1 : -1);
          if (rr >= 0 && ss >= 0) N += s_M[q][2 * rr + ss];
          const double xl = l == 0 ? 1.0 : s_xt[q][l - 1];
          val += xk * xl * N;
        } else {
          double F = 0.0;
          if (r == 1) F = s_f1[q];
          if (r == 0) F += s_g0[q];
          if (r == 2) F += s_g2[q];
          val += xk * F;
        }
      }
  }
  if (!ent) return;
  // contact partial sums of the overlaps this body takes part in
  for (int e = row_ptr[b]; e < row_ptr[b + 1]; ++e) {
    int u = upidx[e];
    if (u < 0 || !has[u]) continue;
    const double* rec = ovr + (size_t)u * CONTRIB;
    bool isI = col[e] > b;
    if (is_h) val += rec[(isI ? 0 : 144) + t];
    else val += rec[(isI ? 432 : 444) + i];
  }
  if (is_h) {
    // damping_sparse (mutils.cpp:106-115): H (1 + beta) + diag(m, Ic) (alpha - beta)
    if (P.damp) val = val * (1 + P.damp_beta) + ((i == j) ? mi * (P.damp_alpha - P.damp_beta) : 0.0);
    D[144 * b + t] = val;
  } else {
    grad[12 * b + i] = val;
  }
}

// Inverse of each SPD diagonal block via Cholesky (block-Jacobi preconditioner).
// Inverse of each SPD diagonal block via Cholesky (block-Jacobi preconditioner), one warp
// per block: lane i holds row i; the factor and its inverse pass through shared memory
// between the column steps. The operations and their order are those of a serial
// Cholesky and forward substitution.
constexpr int BINV_W = 4;  // warps (blocks) per CTA
__global__ void __launch_bounds__(32 * BINV_W) k_block_inverse(int nb, const double* D, double* Dinv, int* status) {
  __shared__ double sL[BINV_W][12][12], sLi[BINV_W][12][12];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * BINV_W + wi;
  if (b >= nb) return;  // whole warps leave together
  double(&L)[12][12] = sL[wi];
  double(&Li)[12][12] = sLi[wi];
  const bool rowl = lane < 12;
  if (rowl)
    for (int j = 0; j < 12; ++j) L[lane][j] = 0.5 * (D[144 * b + 12 * lane + j] + D[144 * b + 12 * j + lane]);
  __syncwarp();
  for (int j = 0; j < 12; ++j) {
    // diagonal entry by lane j, then the column below it by lanes i > j
    if (lane == j) {
      double s = L[j][j];
      for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
      if (!(s > 0)) {
        atomicExch(status, (int)ABD_ERR_NOT_SPD);
        s = 1e-300;
      }
      L[j][j] = sqrt(s);
    }
    __syncwarp();
    if (rowl && lane > j) {
      double t = L[lane][j];
      for (int k = 0; k < j; ++k) t -= L[lane][k] * L[j][k];
      L[lane][j] = t / L[j][j];
    }
    __syncwarp();
  }
  // column c of L^-1 by lane c (forward substitution)
  if (rowl) {
    const int c = lane;
    for (int i = 0; i < 12; ++i) {
      double t = (i == c) ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) t -= L[i][k] * Li[k][c];
      Li[i][c] = (i < c) ? 0.0 : t / L[i][i];
    }
  }
  __syncwarp();
  // Dinv = L^-T L^-1, row i by lane i
  if (rowl) {
    const int i = lane;
    for (int j = 0; j < 12; ++j) {
      double s = 0;
      for (int k = (i > j ? i : j); k < 12; ++k) s += Li[k][i] * Li[k][j];
      Dinv[144 * b + 12 * i + j] = s;
    }
  }
}

// ---------------------------------------------------------------------------------
// Block-Jacobi PCG, one cooperative launch.
//
// The system is first copied into row-block form (k_pcg_rows): for each body its diagonal
// block, then every off-diagonal block that holds a contribution, each stored row-major
// for that body's rows, so a row of the product reads 96 contiguous bytes per block and
// empty overlaps cost nothing. A body's product is split over NPART groups of 16 lanes
// (lane = row, rows 12..15 idle) that take every NPART-th block of the row list; the
// partial rows are added in part order in shared memory.
//
// Bodies are handled in groups of up to GB consecutive bodies of one scene, cut from each
// scene's first body (a scene of n bodies has ceil(n / GB) groups); a CTA takes one group
// at a time, so every CTA works on one scene.
//
// One iteration is two grid-wide phases:
//   A_k: stopping test and beta from the previous r.r and r.z; p_k = z + beta p_{k-1}
//        applied to every neighbour read (p kept in two buffers by iteration parity, so no
//        barrier is needed between the update and the product); q = H p_k; p.q.
//   B_k: alpha = r.z / p.q; x += alpha p, r -= alpha q, z = M^-1 r; r.r, r.z.
//
// Every scene of a batch runs its own CG (its own alpha, beta and stopping test), so a
// scene solved in a batch gets exactly the iterates it gets when solved alone. Dot
// products are reduced per body (16-lane shuffle tree), per group (its bodies in order),
// then per scene over the scene's groups (thread t takes groups gbeg + t, gbeg + t + NT,
// ..., then a fixed tree); groups are cut relative to the scene's first body, so none of
// this depends on where the scene sits in a batch. Every CTA working on a scene computes
// the scene's sums itself; the CTA holding the scene's first group publishes the scalars
// carried to the next iteration, in buffers alternating by iteration parity.
constexpr int NPART = 4;                 // 16-lane groups per body in the product
constexpr int BODY_SLOTS = 16 * NPART;   // threads per body
constexpr int GB = 8;                    // bodies per group
constexpr int PCG_NT = GB * BODY_SLOTS;  // threads per CTA
constexpr int PCG_CACHE = 16;            // loop steps whose scene scalars a CTA keeps on chip

struct PcgArgs {
  int nb, ns, ngrp;
  const int *row_ptr, *rcol, *rn;       // row-block lists: slot body + row_ptr[body], rn blocks
  const double *Hrow, *Dinv, *b;
  const int *grp_body, *grp_n, *grp_scene;  // group -> first body, bodies, scene
  const int *sc_gbeg, *sc_gend;             // scene -> its groups
  const int* sc_on;                     // ns: 0 -> the scene is not solved (dq = 0)
  double *x, *r, *z, *q, *dq;
  double* pbuf;                         // 2 x 12 nb: search direction by iteration parity
  double *gpA, *gpB;                    // 2 per group: partial sums
  double *sc_rz;                        // 2 ns (parity)
  double *sc_bb;                        // ns
  int *sc_conv;                         // 2 ns (parity)
  int *sc_iters;                        // ns
  int *n_active;                        // 3 (iteration mod 3)
  double tol2;
  int maxit;
  int* out;  // [0] status, [1] iterations (max over scenes)
};

// Assembled system as stored by the assembly (diagonal blocks D, off-diagonal blocks in
// the per-overlap records), for products outside the PCG.
struct SysView {
  const int *row_ptr, *col, *upidx, *has;
  const double *ovr, *D;
};

__device__ __forceinline__ double row_spmv(const SysView& a, int body, int row, const double* v) {
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

// One warp per body: the diagonal block, then the off-diagonal blocks with a
// contribution in overlap-list order, transposed where the body is the record's J side.
// kept[0] accumulates the blocks kept (for the algorithmic byte count).
__global__ void k_pcg_rows(int nb, const int* row_ptr, const int* col, const int* upidx, const int* has,
                           const double* ovr, const double* D, double* Hrow, int* rcol, int* rn, int* kept) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nb) return;
  const int body = warp;
  const int base = body + row_ptr[body];
  for (int t = lane; t < 144; t += 32) Hrow[(size_t)base * 144 + t] = D[(size_t)body * 144 + t];
  if (lane == 0) rcol[base] = body;
  int n = 1;
  const unsigned below = (1u << lane) - 1u;
  const int e1 = row_ptr[body + 1];
  for (int e0 = row_ptr[body]; e0 < e1; e0 += 32) {
    int e = e0 + lane;
    int u = -1, cb = 0;
    if (e < e1) {
      u = upidx[e];
      cb = col[e];
      if (u >= 0 && !has[u]) u = -1;
    }
    unsigned m = __ballot_sync(0xffffffffu, u >= 0);
    if (u >= 0) rcol[base + n + __popc(m & below)] = cb;
    while (m) {
      int l = __ffs(m) - 1;
      m &= m - 1;
      int uu = __shfl_sync(0xffffffffu, u, l);
      int cc = __shfl_sync(0xffffffffu, cb, l);
      const double* B = ovr + (size_t)uu * CONTRIB + 288;
      double* dst = Hrow + (size_t)(base + n) * 144;
      for (int t = lane; t < 144; t += 32) {
        int rr = t / 12, c = t - 12 * rr;
        dst[t] = cc > body ? B[t] : B[12 * c + rr];
      }
      ++n;
    }
  }
  if (lane == 0) {
    rn[body] = n;
    atomicAdd(kept, n);
  }
}

// Sum of v[2k + comp] over the groups k in [beg, end) of a scene, by one warp: lane l
// adds k = beg + l, beg + l + 32, ... in order, then a butterfly over the lanes; every
// lane gets the total. (GB300 runs FP64 at 2 FMA per clock per SM, so a CTA-wide tree
// over all warps costs far more than one warp doing it.)
__device__ __forceinline__ double warp_scene_sum(const double* v, int comp, int beg, int end) {
  double s = 0.0;
  int k = beg + (int)(threadIdx.x & 31);
  // four loads in flight before the adds (same order of additions)
  for (; k + 96 < end; k += 128) {
    const double a = v[2 * k + comp], b = v[2 * (k + 32) + comp], c = v[2 * (k + 64) + comp],
                 d = v[2 * (k + 96) + comp];
    s += a;
    s += b;
    s += c;
    s += d;
  }
  for (; k < end; k += 32) s += v[2 * k + comp];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// Block-wide sums of a and b (shuffle tree, then the warps in order); thread 0 gets them.
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

// Sum over the 16 lanes of a body's slot group (rows 12..15 contribute 0).
__device__ __forceinline__ double body_sum16(double v) {
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Group partials from the per-row phase (threads 0 .. 16 GB - 1, two bodies per warp):
// c0, c1 hold each body's sums on its 16 lanes; the warp adds its two bodies, thread 0
// adds the warps in order and writes gp[2 g] (no write for g < 0). Ends with a CTA
// barrier; called by every thread of the CTA.
__device__ __forceinline__ void group_partial(double c0, double c1, double* s_w, double* gp, int g) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x < 16 * GB) {
    c0 += __shfl_down_sync(0xffffffffu, c0, 16);
    c1 += __shfl_down_sync(0xffffffffu, c1, 16);
    if (lane == 0) {
      s_w[2 * w] = c0;
      s_w[2 * w + 1] = c1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && g >= 0) {
    double t0 = s_w[0], t1 = s_w[1];
#pragma unroll
    for (int i = 1; i < GB / 2; ++i) {
      t0 += s_w[2 * i];
      t1 += s_w[2 * i + 1];
    }
    gp[2 * g] = t0;
    gp[2 * g + 1] = t1;
  }
  __syncthreads();
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

// p_k entry: z + beta p_{k-1} (one expression for a body's own entry and for every read
// of it as a neighbour, so all readers see one value)
__device__ __forceinline__ double dir(double z, double beta, double p) { return __fma_rn(beta, p, z); }

__global__ void __launch_bounds__(PCG_NT) k_pcg(PcgArgs a) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double s_part[PCG_NT];
  __shared__ double s_w[GB];                              // warp partials of group_partial
  __shared__ __align__(16) double s_v[PCG_NT / 16][12];  // direction entries of the block being read
  __shared__ double s_sum[2];
  __shared__ double s_val;   // alpha or beta of this CTA's scene
  __shared__ int s_flag;     // 1: this CTA's scene does no work in this phase
  // the scalars this CTA computed for the scene of loop step it < PCG_CACHE (the global
  // copies, written by the scene's owner CTA, serve the later steps)
  __shared__ double s_c_rz[PCG_CACHE], s_c_bb[PCG_CACHE];
  __shared__ int s_c_conv[PCG_CACHE];
  const int nloop = (a.ngrp + gridDim.x - 1) / gridDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // product phase: 64 threads per body (NPART groups of 16 lanes, lane = row)
  const int part = (threadIdx.x >> 4) & (NPART - 1), prow = threadIdx.x & 15;
  const int plb = threadIdx.x / BODY_SLOTS;
  const int hg = threadIdx.x >> 4;
  // per-row phases: threads 0 .. 16 GB - 1, body vlb = t / 16, row = t % 16
  const bool vthr = threadIdx.x < 16 * GB;
  const int vlb = threadIdx.x >> 4, row = threadIdx.x & 15;

  // group handled in loop step `it`: g (or -1), its scene, first body, bodies
  auto group = [&](int it, int& g, int& sc, int& b0, int& nbody) {
    g = blockIdx.x + it * gridDim.x;
    if (g >= a.ngrp) {
      g = -1;
      sc = -1;
      b0 = 0;
      nbody = 0;
      return;
    }
    sc = a.grp_scene[g];
    nbody = a.grp_n[g];
    b0 = a.grp_body[g];
  };

  // ---- init: x = 0, r = b, z = M^-1 b, p_{-1} = 0 (zero for scenes not solved) ----
  for (int it = 0; it < nloop; ++it) {
    int g, sc, b0, nbody;
    group(it, g, sc, b0, nbody);
    double c0 = 0.0, c1 = 0.0;
    if (vthr && g >= 0 && vlb < nbody && row < 12) {
      const int body = b0 + vlb, idx = 12 * body + row;
      bool on = a.sc_on[sc] != 0;
      double bv = on ? a.b[idx] : 0.0;
      double zv = 0.0;
      if (on) {
        const double* Mi = a.Dinv + 144 * body + 12 * row;
#pragma unroll
        for (int c = 0; c < 12; ++c) zv += Mi[c] * a.b[12 * body + c];
      }
      a.x[idx] = 0.0;
      a.r[idx] = bv;
      a.z[idx] = zv;
      a.pbuf[idx] = 0.0;
      a.pbuf[12 * a.nb + idx] = 0.0;
      c0 = bv * bv;
      c1 = bv * zv;
    }
    if (vthr) {
      c0 = body_sum16(c0);
      c1 = body_sum16(c1);
    }
    group_partial(c0, c1, s_w, a.gpB, g);
  }
  if (tid == 0) {
    a.n_active[0] = 0;
    a.n_active[1] = 0;
    a.n_active[2] = 0;
  }
  grid.sync();
  int k = 0;
  for (;; ++k) {
    const int par = k & 1;
    const double* p_old = a.pbuf + (par ^ 1) * 12 * a.nb;  // p_{k-1}
    double* p_new = a.pbuf + par * 12 * a.nb;               // p_k
    double* rz_cur = a.sc_rz + par * a.ns;
    const double* rz_prev = a.sc_rz + (par ^ 1) * a.ns;
    int* conv_cur = a.sc_conv + par * a.ns;
    const int* conv_prev = a.sc_conv + (par ^ 1) * a.ns;
    if (tid == 0) a.n_active[(k + 1) % 3] = 0;
    // ---- A_k: stopping test, beta, q = H p_k, p.q ----
    for (int it = 0; it < nloop; ++it) {
      int g, sc, b0, nbody;
      group(it, g, sc, b0, nbody);
      if (g >= 0) {
        // scalars of the scene (thread 0 loads them while warps 0 and 1 reduce r.r, r.z)
        int was_conv = 0, on = 1;
        double bb = 0.0, rzp = 1.0;
        if (threadIdx.x == 0) {
          if (it < PCG_CACHE) {  // this CTA's own values from the previous iteration
            was_conv = k > 0 ? s_c_conv[it] : 0;
            on = k > 0 ? 1 : a.sc_on[sc];
            if (k > 0) {
              bb = s_c_bb[it];
              rzp = s_c_rz[it];
            }
          } else {
            was_conv = k > 0 ? conv_prev[sc] : 0;
            on = a.sc_on[sc];
            if (k > 0) {
              bb = a.sc_bb[sc];
              rzp = rz_prev[sc];
            }
          }
        }
        if (warp < 2) {
          double v = warp_scene_sum(a.gpB, warp, a.sc_gbeg[sc], a.sc_gend[sc]);
          if (lane == 0) s_sum[warp] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          const bool owner = g == a.sc_gbeg[sc];
          const double rr = s_sum[0], rz = s_sum[1];
          if (was_conv) {
            if (owner) conv_cur[sc] = 1;
            s_flag = 1;
          } else {
            bool conv;
            if (k == 0) {
              conv = !on || rr == 0.0;
              if (owner) a.sc_bb[sc] = rr;
              if (it < PCG_CACHE) s_c_bb[it] = rr;
            } else {
              conv = !(rr > a.tol2 * bb);
            }
            s_val = k == 0 ? 0.0 : rz / rzp;
            s_flag = conv || k == a.maxit;
            if (it < PCG_CACHE) {
              s_c_conv[it] = conv ? 1 : 0;
              s_c_rz[it] = rz;
            }
            if (owner) {
              rz_cur[sc] = rz;
              conv_cur[sc] = conv ? 1 : 0;
              if (conv) {
                a.sc_iters[sc] = k;
              } else if (k == a.maxit) {
                a.sc_iters[sc] = k;
                a.out[0] = ABD_ERR_PCG_NOCONV;
              } else {
                atomicAdd(&a.n_active[k % 3], 1);
              }
            }
          }
        }
      }
      __syncthreads();
      const bool act = g >= 0 && !s_flag;
      const double beta = act ? s_val : 0.0;
      double acc = 0.0;
      if (act && plb < nbody) {
        // the two 16-lane halves of a warp are different parts and may run different
        // trip counts: each half synchronises only itself
        const unsigned half = 0xffffu << (threadIdx.x & 16);
        const int body = b0 + plb;
        const int base = body + a.row_ptr[body], n = a.rn[body];
        for (int j = part; j < n; j += NPART) {
          const int cb = a.rcol[base + j];
          if (prow < 12) s_v[hg][prow] = dir(a.z[12 * cb + prow], beta, p_old[12 * cb + prow]);
          __syncwarp(half);
          if (prow < 12) {
            const double2* H = reinterpret_cast<const double2*>(a.Hrow + (size_t)(base + j) * 144 + 12 * prow);
            const double2* v = reinterpret_cast<const double2*>(s_v[hg]);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              double2 h = H[c], vv = v[c];
              acc += h.x * vv.x;
              acc += h.y * vv.y;
            }
          }
          __syncwarp(half);
        }
      }
      s_part[threadIdx.x] = acc;
      __syncthreads();
      if (act) {
        double c0 = 0.0;
        if (vthr && vlb < nbody && row < 12) {
          const double* sp = s_part + vlb * BODY_SLOTS + row;
          double qv = sp[0];
#pragma unroll
          for (int pp = 1; pp < NPART; ++pp) qv += sp[16 * pp];
          const int idx = 12 * (b0 + vlb) + row;
          double pv = dir(a.z[idx], beta, p_old[idx]);
          p_new[idx] = pv;
          a.q[idx] = qv;
          c0 = pv * qv;
        }
        if (vthr) c0 = body_sum16(c0);
        group_partial(c0, 0.0, s_w, a.gpA, g);
      }
      __syncthreads();
    }
    if (k == a.maxit) break;
    grid.sync();
    if (ld_volatile(&a.n_active[k % 3]) == 0) break;
    // ---- B_k: alpha; x += alpha p, r -= alpha q, z = M^-1 r; r.r, r.z ----
    for (int it = 0; it < nloop; ++it) {
      int g, sc, b0, nbody;
      group(it, g, sc, b0, nbody);
      const bool act = g >= 0 && !(it < PCG_CACHE ? s_c_conv[it] : conv_cur[sc]);
      if (act && warp == 0) {
        const double rz = lane == 0 ? (it < PCG_CACHE ? s_c_rz[it] : rz_cur[sc]) : 0.0;
        const double pq = warp_scene_sum(a.gpA, 0, a.sc_gbeg[sc], a.sc_gend[sc]);
        if (lane == 0) s_val = rz / pq;
      }
      __syncthreads();
      if (act) {
        double c0 = 0.0, c1 = 0.0;
        const bool mine = vthr && vlb < nbody && row < 12;
        const int body = b0 + vlb, idx = 12 * body + row;
        if (mine) {
          const double alpha = s_val;
          a.x[idx] += alpha * p_new[idx];
          a.r[idx] -= alpha * a.q[idx];
        }
        __syncwarp();
        if (mine) {
          const double* Mi = a.Dinv + 144 * body + 12 * row;
          double zv = 0;
#pragma unroll
          for (int c = 0; c < 12; ++c) zv += Mi[c] * a.r[12 * body + c];
          a.z[idx] = zv;
          double rv = a.r[idx];
          c0 = rv * rv;
          c1 = rv * zv;
        }
        if (vthr) {
          c0 = body_sum16(c0);
          c1 = body_sum16(c1);
        }
        group_partial(c0, c1, s_w, a.gpB, g);
      }
      __syncthreads();
    }
    grid.sync();
  }
  // dq = -x (each entry written by the thread that owns it)
  for (int it = 0; it < nloop; ++it) {
    int g, sc, b0, nbody;
    group(it, g, sc, b0, nbody);
    if (vthr && g >= 0 && vlb < nbody && row < 12) {
      const int idx = 12 * (b0 + vlb) + row;
      a.dq[idx] = -a.x[idx];
    }
  }
  if (tid == 0) a.out[1] = k;
}

// The same solve when every CTA holds exactly one body group (grid = groups, the common
// case up to 152 groups per cooperative launch): each thread keeps its row's x, r, z, p
// and q, its row of the block-Jacobi inverse and its first two row blocks of the product
// in registers for the whole solve, and z = M^-1 r takes the body's r from its 16-lane
// half by shuffles. Only the neighbour reads of z and p and the group partials go through
// memory. The arithmetic is that of k_pcg, operation for operation, so both give the same
// iterates bit for bit.
constexpr int PCG1_NC = 2;  // row blocks per part kept in registers
__global__ void __launch_bounds__(PCG_NT) k_pcg1(PcgArgs a) {
  cg::grid_group grid = cg::this_grid();
  __shared__ double s_part[PCG_NT];
  __shared__ double s_w[GB];
  __shared__ __align__(16) double s_v[PCG_NT / 16][12];
  __shared__ double s_sum[2];
  __shared__ double s_val;
  __shared__ double s_beta, s_rzp;  // beta from warp 1's r.z sum; the previous r.z
  __shared__ int s_flag;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int part = (threadIdx.x >> 4) & (NPART - 1), prow = threadIdx.x & 15;
  const int plb = threadIdx.x / BODY_SLOTS;
  const int hg = threadIdx.x >> 4;
  const bool vthr = threadIdx.x < 16 * GB;
  const int vlb = threadIdx.x >> 4, row = threadIdx.x & 15;
  const int g = blockIdx.x;
  const int sc = a.grp_scene[g], nbody = a.grp_n[g], b0 = a.grp_body[g];
  const bool owner = g == a.sc_gbeg[sc];
  // product-phase state
  const bool pact = plb < nbody;
  const int pbody = b0 + plb;
  const int pbase = pact ? pbody + a.row_ptr[pbody] : 0, pn = pact ? a.rn[pbody] : 0;
  int rc[PCG1_NC];
  double hr[PCG1_NC][12];
#pragma unroll
  for (int jj = 0; jj < PCG1_NC; ++jj) {
    const int j = part + NPART * jj;
    rc[jj] = j < pn ? a.rcol[pbase + j] : 0;
#pragma unroll
    for (int c = 0; c < 12; ++c) hr[jj][c] = (j < pn && prow < 12) ? a.Hrow[(size_t)(pbase + j) * 144 + 12 * prow + c] : 0.0;
  }
  // per-row state
  const bool mine = vthr && vlb < nbody && row < 12;
  const int vbody = b0 + vlb, idx = 12 * vbody + row;
  double Dr[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) Dr[c] = mine ? a.Dinv[144 * vbody + 12 * row + c] : 0.0;
  double x_r = 0.0, r_r = 0.0, z_r = 0.0, pold_r = 0.0, q_r = 0.0, pv_r = 0.0;
  // thread 0: the scene's carried scalars
  int conv_r = 0;
  double bb_r = 0.0, rz_r = 1.0;

  // ---- init ----
  {
    double c0 = 0.0, c1 = 0.0;
    if (mine) {
      const bool on = a.sc_on[sc] != 0;
      const double bv = on ? a.b[idx] : 0.0;
      double zv = 0.0;
      if (on) {
#pragma unroll
        for (int c = 0; c < 12; ++c) zv += Dr[c] * a.b[12 * vbody + c];
      }
      r_r = bv;
      z_r = zv;
      a.z[idx] = zv;
      a.pbuf[idx] = 0.0;
      a.pbuf[12 * a.nb + idx] = 0.0;
      c0 = bv * bv;
      c1 = bv * zv;
    }
    if (vthr) {
      c0 = body_sum16(c0);
      c1 = body_sum16(c1);
    }
    group_partial(c0, c1, s_w, a.gpB, g);
  }
  if (tid == 0) {
    a.n_active[0] = 0;
    a.n_active[1] = 0;
    a.n_active[2] = 0;
  }
  grid.sync();
  int k = 0;
  for (;; ++k) {
    const int par = k & 1;
    const double* p_old = a.pbuf + (par ^ 1) * 12 * a.nb;
    double* p_new = a.pbuf + par * 12 * a.nb;
    if (tid == 0) a.n_active[(k + 1) % 3] = 0;
    // ---- A_k ----
    if (warp < 2) {
      double v = warp_scene_sum(a.gpB, warp, a.sc_gbeg[sc], a.sc_gend[sc]);
      if (lane == 0) {
        s_sum[warp] = v;
        // beta = r.z / previous r.z, divided here beside warp 0's sum instead of after it
        if (warp == 1 && k > 0) s_beta = v / s_rzp;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const double rr = s_sum[0], rz = s_sum[1];
      int* conv_cur = a.sc_conv + par * a.ns;
      if (k > 0 && conv_r) {
        if (owner) conv_cur[sc] = 1;
        s_flag = 1;
      } else {
        bool conv;
        if (k == 0) {
          conv = !a.sc_on[sc] || rr == 0.0;
          if (owner) a.sc_bb[sc] = rr;
          bb_r = rr;
        } else {
          conv = !(rr > a.tol2 * bb_r);
        }
        s_val = k == 0 ? 0.0 : s_beta;
        s_flag = conv || k == a.maxit;
        conv_r = conv ? 1 : 0;
        rz_r = rz;
        s_rzp = rz;
        if (owner) {
          a.sc_rz[par * a.ns + sc] = rz;
          conv_cur[sc] = conv ? 1 : 0;
          if (conv) {
            a.sc_iters[sc] = k;
          } else if (k == a.maxit) {
            a.sc_iters[sc] = k;
            a.out[0] = ABD_ERR_PCG_NOCONV;
          } else {
            atomicAdd(&a.n_active[k % 3], 1);
          }
        }
      }
    }
    __syncthreads();
    const bool act = !s_flag;
    const double beta = act ? s_val : 0.0;
    double acc = 0.0;
    if (act && pact) {
      const unsigned half = 0xffffu << (threadIdx.x & 16);
      // the neighbour entries of both register blocks are loaded before either is used
      double zn[PCG1_NC], pn_[PCG1_NC];
#pragma unroll
      for (int jj = 0; jj < PCG1_NC; ++jj) {
        const bool ld = part + NPART * jj < pn && prow < 12;
        zn[jj] = ld ? a.z[12 * rc[jj] + prow] : 0.0;
        pn_[jj] = ld ? p_old[12 * rc[jj] + prow] : 0.0;
      }
#pragma unroll
      for (int jj = 0; jj < PCG1_NC; ++jj) {
        const int j = part + NPART * jj;
        if (j < pn) {
          if (prow < 12) s_v[hg][prow] = dir(zn[jj], beta, pn_[jj]);
          __syncwarp(half);
          if (prow < 12) {
            const double2* v = reinterpret_cast<const double2*>(s_v[hg]);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              double2 vv = v[c];
              acc += hr[jj][2 * c] * vv.x;
              acc += hr[jj][2 * c + 1] * vv.y;
            }
          }
          __syncwarp(half);
        }
      }
      for (int j = part + NPART * PCG1_NC; j < pn; j += NPART) {
        const int cb = a.rcol[pbase + j];
        if (prow < 12) s_v[hg][prow] = dir(a.z[12 * cb + prow], beta, p_old[12 * cb + prow]);
        __syncwarp(half);
        if (prow < 12) {
          const double2* H = reinterpret_cast<const double2*>(a.Hrow + (size_t)(pbase + j) * 144 + 12 * prow);
          const double2* v = reinterpret_cast<const double2*>(s_v[hg]);
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            double2 h = H[c], vv = v[c];
            acc += h.x * vv.x;
            acc += h.y * vv.y;
          }
        }
        __syncwarp(half);
      }
    }
    s_part[threadIdx.x] = acc;
    __syncthreads();
    if (act) {
      double c0 = 0.0;
      if (mine) {
        const double* sp = s_part + vlb * BODY_SLOTS + row;
        double qv = sp[0];
#pragma unroll
        for (int pp = 1; pp < NPART; ++pp) qv += sp[16 * pp];
        const double pv = dir(z_r, beta, pold_r);
        p_new[idx] = pv;
        pv_r = pv;
        q_r = qv;
        c0 = pv * qv;
      }
      if (vthr) c0 = body_sum16(c0);
      group_partial(c0, 0.0, s_w, a.gpA, g);
    }
    __syncthreads();
    if (k == a.maxit) break;
    grid.sync();
    // the count of scenes still iterating and the p.q partials are loaded together
    const int nact = ld_volatile(&a.n_active[k % 3]);
    double pq = 0.0;
    if (!s_flag && warp == 0) pq = warp_scene_sum(a.gpA, 0, a.sc_gbeg[sc], a.sc_gend[sc]);
    if (nact == 0) break;
    // ---- B_k (s_flag still holds whether the scene stopped in A_k: its CG ends there) ----
    if (!s_flag) {
      if (threadIdx.x == 0) s_val = rz_r / pq;
      __syncthreads();
      double c0 = 0.0, c1 = 0.0;
      if (mine) {
        const double alpha = s_val;
        x_r += alpha * pv_r;
        r_r -= alpha * q_r;
      }
      if (vthr) {
        double zv = 0;
#pragma unroll
        for (int c = 0; c < 12; ++c) zv += Dr[c] * __shfl_sync(0xffffffffu, r_r, (lane & 16) + c);
        if (mine) {
          z_r = zv;
          a.z[idx] = zv;
          pold_r = pv_r;
          c0 = r_r * r_r;
          c1 = r_r * zv;
        }
        c0 = body_sum16(c0);
        c1 = body_sum16(c1);
      }
      group_partial(c0, c1, s_w, a.gpB, g);
    }
    __syncthreads();
    grid.sync();
  }
  if (mine) {
    a.x[idx] = x_r;
    a.dq[idx] = -x_r;
  }
  if (tid == 0) a.out[1] = k;
}

// ---------------------------------------------------------------------------------
// Line-search energies, one total per scene. A scene's terms form one virtual index
// range (its bodies, PT, EE and VG pairs of the trial set, then the PT, EE and VG pairs
// of the lagged set); the range is cut into chunks of ECHUNK terms counted from the
// scene's own start, each chunk is summed by one block in a fixed order, and the chunk
// sums of a scene are added in chunk order. The total of a scene therefore does not
// depend on where the scene sits in a batch.
constexpr int ECHUNK = 512;
enum { SEG_PT, SEG_EE, SEG_VG, SEG_LPT, SEG_LEE, SEG_LVG, NSEG };

struct EnergyArgs {
  int nb, ns, npt, nee, nvg, lpt, lee, lvg;
  double alpha;  // used when the geometry carries no per-scene step
  int with_bi;
  const int *pt, *ee, *vg, *lpt_t, *lee_t, *lvg_t;
  const int8_t *pt_ty, *ee_ty;  // distance types classified by the cull at this configuration
  const double *lpt_lag, *lee_lag, *lvg_lam;
  const int* off;        // NSEG * (ns + 1): first element of each scene in each list
  const int* chunk_off;  // ns + 1
  double* partial;       // one per chunk
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

// One term: seg -1 = body (inertia + orthogonality), else an index into the list `seg`.
__device__ double energy_term(const Geo& g, const Params& P, const EnergyArgs& a, int seg, int i) {
  BarrierP bp{P.dhat, P.kappa};
  if (seg < 0) {
    double alpha = g.alpha_s ? g.alpha_s[g.bscene[i]] : a.alpha;
    return inertia_energy(g, P, i, alpha);
  }
  if (seg == SEG_PT) {
    if (!P.pt) return 0.0;
    int vid[4];
    pair_vids(g, 0, a.pt, i, vid);
    d3 X0 = ldX(g.X, g.nv, vid[0]), X1 = ldX(g.X, g.nv, vid[1]), X2 = ldX(g.X, g.nv, vid[2]),
       X3 = ldX(g.X, g.nv, vid[3]);
    return barrier_b(pt_dist(X0, X1, X2, X3, a.pt_ty[i]), bp);
  }
  if (seg == SEG_EE) {
    if (!P.ee) return 0.0;
    int vid[4];
    pair_vids(g, 1, a.ee, i, vid);
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
    return barrier_b(ee_dist(X0, X1, X2, X3, a.ee_ty[i]), bp) * m;
  }
  if (seg == SEG_VG) {
    if (!P.ground) return 0.0;
    int b = a.vg[2 * i], v = g.v_off[b] + a.vg[2 * i + 1];
    double d = XA(g.X[g.nv + v], P.ground_offset);
    d = XM(d, d);
    return d < P.dhat ? barrier_b(d, bp) : 0.0;
  }
  if (seg == SEG_LPT || seg == SEG_LEE) {
    int kind = seg == SEG_LEE ? 1 : 0;
    int n = kind ? a.lee : a.lpt;
    bool on = kind ? (P.ee && P.ee_fric) : (P.pt && P.pt_fric);
    if (!on) return 0.0;
    const double* L = kind ? a.lee_lag : a.lpt_lag;
    int vid[4];
    pair_vids(g, kind, kind ? a.lee_t : a.lpt_t, i, vid);
    d3 c0 = fd3(L[0 * n + i], L[1 * n + i], L[2 * n + i]), c1 = fd3(L[3 * n + i], L[4 * n + i], L[5 * n + i]);
    double u0 = 0, u1 = 0;
    for (int k = 0; k < 4; ++k) {
      d3 du = fsub(ldX(g.X, g.nv, vid[k]), ldX(g.X0, g.nv, vid[k]));
      double gm = L[(6 + k) * n + i];
      u0 += gm * fdot(c0, du);
      u1 += gm * fdot(c1, du);
    }
    return P.mu * L[10 * n + i] * f0_SF(sqrt(u0 * u0 + u1 * u1), P.epsv);
  }
  // SEG_LVG
  if (!(P.ground && P.vg_fric)) return 0.0;
  int b = a.lvg_t[2 * i], v = g.v_off[b] + a.lvg_t[2 * i + 1];
  double dx = g.X[v] - g.X0[v], dz = g.X[2 * g.nv + v] - g.X0[2 * g.nv + v];
  return P.mu * a.lvg_lam[i] * f0_SF(sqrt(dx * dx + dz * dz), P.epsv);
}

// First element of list `tup` (stride ints per element, body id first) whose body lies in
// scene >= s; the lists are ordered by scene.
__device__ __forceinline__ int scene_lower_bound(const int* bscene, const int* tup, int stride, int n, int s) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (bscene[tup[stride * mid]] < s) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Per-scene list offsets and chunk counts (thread per scene, plus one for the ends).
// First element of each scene in each list (one thread per list and scene bound; the
// lists are ordered by scene), then each scene's chunk count.
__global__ void k_scene_offsets(Geo g, EnergyArgs a, int* off) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= NSEG * (a.ns + 1)) return;
  const int k = t / (a.ns + 1), s = t - k * (a.ns + 1);
  const int* lists[NSEG] = {a.pt, a.ee, a.vg, a.lpt_t, a.lee_t, a.lvg_t};
  const int stride[NSEG] = {4, 4, 2, 4, 4, 2};
  const int n[NSEG] = {a.npt, a.nee, a.nvg, a.lpt, a.lee, a.lvg};
  off[t] = (s == a.ns) ? n[k] : scene_lower_bound(g.bscene, lists[k], stride[k], n[k], s);
}
__global__ void k_scene_chunks(Geo g, EnergyArgs a, const int* off, int* chunk_cnt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.ns) return;
  long long total = a.with_bi ? g.sc_end[s] - g.sc_beg[s] : 0;
  for (int k = 0; k < NSEG; ++k) {
    if (k < SEG_LPT && !a.with_bi) continue;
    total += off[k * (a.ns + 1) + s + 1] - off[k * (a.ns + 1) + s];
  }
  long long c = (total + ECHUNK - 1) / ECHUNK;
  chunk_cnt[s] = c > 0 ? (int)c : 1;
}

__global__ void __launch_bounds__(256) k_energy(Geo g, Params P, EnergyArgs a) {
  __shared__ double sh[80];
  const int nchunk = a.chunk_off[a.ns];
  for (int c = blockIdx.x; c < nchunk; c += gridDim.x) {
    // scene of chunk c: last s with chunk_off[s] <= c
    int lo = 0, hi = a.ns - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (a.chunk_off[mid] <= c) lo = mid;
      else hi = mid - 1;
    }
    const int s = lo;
    const int S1 = a.ns + 1;
    if (g.sc_act && !g.sc_act[s]) {  // scene not processed: its total is not used
      if (threadIdx.x == 0) a.partial[c] = 0.0;
      continue;
    }
    int len[1 + NSEG], beg[1 + NSEG];
    len[0] = a.with_bi ? g.sc_end[s] - g.sc_beg[s] : 0;
    beg[0] = g.sc_beg[s];
    for (int k = 0; k < NSEG; ++k) {
      beg[k + 1] = a.off[k * S1 + s];
      len[k + 1] = (k < SEG_LPT && !a.with_bi) ? 0 : a.off[k * S1 + s + 1] - beg[k + 1];
    }
    long long total = 0;
    for (int k = 0; k <= NSEG; ++k) total += len[k];
    long long e0 = (long long)(c - a.chunk_off[s]) * ECHUNK;
    long long e1 = e0 + ECHUNK < total ? e0 + ECHUNK : total;
    double acc = 0.0;
    for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      long long i = e;
      int k = 0;
      while (i >= len[k]) {
        i -= len[k];
        ++k;
      }
      acc += energy_term(g, P, a, k - 1, beg[k] + (int)i);
    }
    double dummy = 0;
    block_sum2(acc, dummy, sh);
    if (threadIdx.x == 0) a.partial[c] = acc;
    __syncthreads();
  }
}

// Every term of one list on its own (the values k_energy sums): out[i] = term i of
// segment seg (-1: bodies).
__global__ void k_energy_each(Geo g, Params P, EnergyArgs a, int seg, int n, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = energy_term(g, P, a, seg, i);
}

// Scene totals of the chunk partials: one warp per scene, lane l adding chunks l, l + 32,
// ... in order, then a fixed shuffle tree (a serial sum by one thread was a chain of
// hundreds of dependent FP64 adds).
__global__ void k_scene_energy(int ns, const int* chunk_off, const double* part, double* out) {
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= ns) return;
  double t = 0.0;
  for (int c = chunk_off[s] + lane; c < chunk_off[s + 1]; c += 32) t += part[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[s] = t;
}

// Per scene: dq.grad, |grad|^2, |dq|^2 (one block per scene; thread t takes the scene's
// bodies t, t + 256, ..., each body's 12 entries in order).
__global__ void __launch_bounds__(256) k_scene_dots(const int* sc_beg, const int* sc_end, const double* a,
                                                   const double* b, double* out) {
  __shared__ double sh[80];
  int s = blockIdx.x;
  double s0 = 0, s1 = 0, s2 = 0;
  for (int k = sc_beg[s] + (int)threadIdx.x; k < sc_end[s]; k += blockDim.x) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int i = 12 * k; i < 12 * k + 12; ++i) {
      t0 += a[i] * b[i];
      t1 += b[i] * b[i];
      t2 += a[i] * a[i];
    }
    s0 += t0;
    s1 += t1;
    s2 += t2;
  }
  block_sum2(s0, s1, sh);
  __syncthreads();
  double d = 0;
  block_sum2(s2, d, sh);
  if (threadIdx.x == 0) {
    out[3 * s] = s0;
    out[3 * s + 1] = s1;
    out[3 * s + 2] = s2;
  }
}

// Per scene: a.b, |b|^2, |a - b|^2 (same layout and order as k_scene_dots).
__global__ void __launch_bounds__(256) k_scene_diff(const int* sc_beg, const int* sc_end, const double* a,
                                                   const double* b, double* out) {
  __shared__ double sh[80];
  int s = blockIdx.x;
  double s0 = 0, s1 = 0, s2 = 0;
  for (int k = sc_beg[s] + (int)threadIdx.x; k < sc_end[s]; k += blockDim.x) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int i = 12 * k; i < 12 * k + 12; ++i) {
      double d = a[i] - b[i];
      t0 += a[i] * b[i];
      t1 += b[i] * b[i];
      t2 += d * d;
    }
    s0 += t0;
    s1 += t1;
    s2 += t2;
  }
  block_sum2(s0, s1, sh);
  __syncthreads();
  double d = 0;
  block_sum2(s2, d, sh);
  if (threadIdx.x == 0) {
    out[3 * s] = s0;
    out[3 * s + 1] = s1;
    out[3 * s + 2] = s2;
  }
}

// dst = src on the bodies of scenes with on[scene] != 0
__global__ void k_copy_scene(double* dst, const double* src, int n, const int* bscene, const int* on) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && on[bscene[i / 12]]) dst[i] = src[i];
}

// Transpose of the ground-friction multiplier coupling (adjoint systems): the lagged
// multiplier lam(y) = -2 b'(d) (y + off) of each vertex-ground pair moves with the
// vertex height at the solution, which adds C = (r_f / lam) (dlam/dy J_y)^T to the
// Jacobian of the gradient. out = C^T w, one thread per body.
__global__ void k_vg_lag_adj(Geo g, Params P, const int* vg, const int* vg_seg, const double* w, double* out) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nb) return;
  double acc[4] = {0, 0, 0, 0};
  const double* wb = w + 12 * b;
  if (g.mass[b] > 0.0 && P.ground && P.vg_fric) {
    BarrierP bp{P.dhat, P.kappa};
    for (int kk = vg_seg[b]; kk < vg_seg[b + 1]; ++kk) {
      int v = g.v_off[b] + vg[2 * kk + 1];
      double _d = g.X[g.nv + v] + P.ground_offset;
      double dd = _d * _d;
      if (!(dd < P.dhat)) continue;
      double b1 = barrier_b1(dd, bp), b2 = barrier_b2(dd, bp);
      double lam = -b1 * 2 * _d;
      if (lam == 0.0) continue;
      double dlam = -2.0 * (2.0 * b2 * dd + b1);
      double uk[2] = {g.X[v] - g.X0[v], g.X[2 * g.nv + v] - g.X0[2 * g.nv + v]};
      double gs = 0.0, M[2][2];
      friction_2x2(uk, lam, FrictionP{P.mu, P.epsv, P.max_uk}, gs, M);
      double xt[4] = {1.0, g.rest[3 * v], g.rest[3 * v + 1], g.rest[3 * v + 2]};
      double wx = 0.0, wz = 0.0;
      for (int k = 0; k < 4; ++k) {
        wx += xt[k] * wb[3 * k];
        wz += xt[k] * wb[3 * k + 2];
      }
      double c = dlam * (gs / lam) * (uk[0] * wx + uk[1] * wz);
      for (int k = 0; k < 4; ++k) acc[k] += xt[k] * c;
    }
  }
  for (int k = 0; k < 4; ++k) {
    out[12 * b + 3 * k] = 0.0;
    out[12 * b + 3 * k + 1] = acc[k];
    out[12 * b + 3 * k + 2] = 0.0;
  }
}

// y = H x over the assembled block-sparse matrix (diagonal blocks D, off-diagonal blocks
// in the per-overlap records), one thread per (body, row) slot.
__global__ void k_spmv(int nb, const int* row_ptr, const int* col, const int* upidx, const int* has,
                       const double* ovr, const double* D, const double* x, double* y) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  int body = s >> 4, row = s & 15;
  if (body >= nb || row >= 12) return;
  SysView a{row_ptr, col, upidx, has, ovr, D};
  y[12 * body + row] = row_spmv(a, body, row, x);
}

// True residual r = b - H x of the row-block system the PCG iterates on (one thread per
// body row, the row's blocks in list order); bodies of scenes that are not solved get 0.
__global__ void k_true_residual(int nb, const int* row_ptr, const int* rcol, const int* rn, const double* Hrow,
                                const int* bscene, const int* sc_on, const double* b, const double* x, double* r) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int body = t / 12, row = t - 12 * body;
  if (body >= nb) return;
  if (!sc_on[bscene[body]]) {
    r[t] = 0.0;
    return;
  }
  const int base = body + row_ptr[body], n = rn[body];
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    const double* H = Hrow + (size_t)(base + j) * 144 + 12 * row;
    const double* v = x + 12 * rcol[base + j];
#pragma unroll
    for (int c = 0; c < 12; ++c) acc = __fma_rn(H[c], v[c], acc);
  }
  r[t] = __dsub_rn(b[t], acc);
}

// Iteration counts of a refinement solve added to the running totals: acc[0] += the
// solve's count (its longest scene), acc[2 + k] += scene k's.
__global__ void k_iter_add(int ns, const int* its, const int* sc_its, int* acc) {
  if (threadIdx.x == 0) acc[0] += its[0];
  for (int k = threadIdx.x; k < ns; k += blockDim.x) acc[2 + k] += sc_its[k];
}

// x += d, dq = -x (a refinement step of the Newton solve)
__global__ void k_refine_add(int n, double* x, const double* d, double* dq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = __dadd_rn(x[i], d[i]);
  x[i] = v;
  dq[i] = -v;
}

// v *= f[scene of body]
__global__ void k_scale_scene(double* v, int n, const int* bscene, const double* f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = XM(v[i], f[bscene[i / 12]]);
}
// q += alpha[scene of body] dq
__global__ void k_q_update_scene(double* q, const double* dq, int n, const int* bscene, const double* alpha) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = XA(q[i], XM(dq[i], alpha[bscene[i / 12]]));
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
  B.pt_c.ensure((size_t)PAIRC * npt + 1);
  B.ee_c.ensure((size_t)PAIRC * nee + 1);
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
  for (int kind = 0; kind < 2; ++kind) {
    int n = kind ? nee : npt;
    if (!n) continue;
    int nb_c = nblk(n, CLS_T);
    B.cls_cnt.ensure(NCLS * (size_t)nb_c);
    B.cls_off.ensure(NCLS * (size_t)nb_c);
    B.perm.ensure(n);
    const int8_t* ty = kind ? S.ee_ty.p : S.pt_ty.p;
    const int* tup = kind ? S.ee.p : S.pt.p;
    KLAUNCH(K_SEG, s, k_class_count<<<nb_c, CLS_T, 0, s>>>(g, P, kind, n, tup, ty, B.cls_cnt.p));
    scan_exclusive_int(B.cls_cnt.p, B.cls_off.p, NCLS * nb_c, nullptr, s, B.cls_tmp);
    KLAUNCH(K_SEG, s, k_class_scatter<<<nb_c, CLS_T, 0, s>>>(g, P, kind, n, tup, ty, B.cls_off.p, B.perm.p));
    B.prec.ensure(REC * (size_t)n);
    // class 0 (mollified edge-edge pairs) comes first in perm; its size is the offset of
    // class 1
    const int* n_moll = kind ? B.cls_off.p + nb_c : nullptr;
    if (kind) {
      // the few mollified pairs take one warp each for a long serial projection: run
      // them on a side stream, overlapped with the main kernel
      if (!B.side) {
        CK(cudaStreamCreateWithFlags(&B.side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&B.ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&B.ev_join, cudaEventDisableTiming));
      }
      CK(cudaEventRecord(B.ev_fork, s));
      CK(cudaStreamWaitEvent(B.side, B.ev_fork, 0));
      KLAUNCH(K_PAIR_TERMS, B.side, k_pair_moll<<<64, 32 * MOLL_W, 0, B.side>>>(g, P, n, tup, ty, B.perm.p, n_moll,
                                                                              B.prec.p, S.ee_lag.p));
      CK(cudaEventRecord(B.ev_join, B.side));
    }
    KLAUNCH(K_PAIR_TERMS, s, k_pair_hess<<<nblk(n, 128), 128, 0, s>>>(g, P, kind, n, tup, ty, B.perm.p, n_moll,
                                                                    B.prec.p, kind ? S.ee_lag.p : S.pt_lag.p));
    if (kind) CK(cudaStreamWaitEvent(s, B.ev_join, 0));
    if (kind)
      KLAUNCH(K_PAIR_TERMS, s, k_pair_chain<1><<<nblk(n, 128), 128, 0, s>>>(g, n, tup, S.ee_ov.p, S.ovI.p, B.prec.p,
                                                                            B.ee_c.p));
    else
      KLAUNCH(K_PAIR_TERMS, s, k_pair_chain<0><<<nblk(n, 128), 128, 0, s>>>(g, n, tup, S.pt_ov.p, S.ovI.p, B.prec.p,
                                                                            B.pt_c.p));
  }
  if (nov) {
    KLAUNCH(K_SEG, s, k_seg<<<nblk(nov + 1, 256), 256, 0, s>>>(nov, npt, S.pt_ov.p, B.pt_seg.p));
    KLAUNCH(K_SEG, s, k_seg<<<nblk(nov + 1, 256), 256, 0, s>>>(nov, nee, S.ee_ov.p, B.ee_seg.p));
    KLAUNCH(K_OV_REDUCE, s, k_ov_reduce<<<nov, 512, 0, s>>>(nov, B.pt_seg.p, B.ee_seg.p, B.pt_c.p, npt, B.ee_c.p, nee, B.ovr.p, B.has.p,
                                                                P.damp ? 1 + P.damp_beta : 1.0));
  }
  KLAUNCH(K_BODY_SYSTEM, s, k_body_system<<<nb, 160, 0, s>>>(g, P, S.row_ptr.p, S.col.p, S.upidx.p, B.ovr.p, B.has.p, S.vg.p, S.vg_seg.p,
                                   S.vg_lam.p, B.D.p, B.grad.p));
}

int pcg_solve(const Geo& g, PairSet& S, NewtonBufs& B, const SolveOpts& o, const int* sc_on,
              const std::vector<char>& on, double* dq, cudaStream_t s, int* status, int* scene_iters) {
  const double rel_tol = o.rel_tol, refine_tol = o.refine_tol;
  const int max_iter = o.max_iter, refine = o.refine;
  int nb = g.nb, ns = g.ns;
  B.status.ensure(4);
  if (!B.h_int) CK(cudaMallocHost(&B.h_int, 16 * sizeof(int)));
  CK(cudaMemsetAsync(B.status.p, 0, 4 * sizeof(int), s));
  KLAUNCH(K_BLOCK_INVERSE, s, k_block_inverse<<<nblk(nb, BINV_W), 32 * BINV_W, 0, s>>>(nb, B.D.p, B.Dinv.p,
                                                                                        B.status.p));
  B.x.ensure(12 * (size_t)nb);
  B.r.ensure(12 * (size_t)nb);
  B.z.ensure(12 * (size_t)nb);
  B.p.ensure(24 * (size_t)nb);
  B.qv.ensure(12 * (size_t)nb);
  B.Hrow.ensure(144 * ((size_t)nb + S.nnz));
  B.rcol.ensure((size_t)nb + S.nnz);
  B.rn.ensure(nb);
  if (B.ngrp <= 0) {  // pcg_groups was not called for these scenes
    *status = ABD_ERR_INVALID;
    return 0;
  }
  B.gpA.ensure(2 * (size_t)B.ngrp);
  B.gpB.ensure(2 * (size_t)B.ngrp);
  B.sc_rz.ensure(2 * (size_t)ns);
  B.sc_bb.ensure(ns);
  B.sc_conv.ensure(2 * (size_t)ns);
  B.sc_iters.ensure(ns);
  B.n_active.ensure(3);
  // solve setup (counted with the preconditioner): row-block copy of the system
  KLAUNCH(K_BLOCK_INVERSE, s, k_pcg_rows<<<nblk((long long)nb * 32, 256), 256, 0, s>>>(nb, S.row_ptr.p, S.col.p,
                                                                                        S.upidx.p, B.has.p, B.ovr.p,
                                                                                        B.D.p, B.Hrow.p, B.rcol.p,
                                                                                        B.rn.p, B.status.p + 2));
  if (o.dense) {
    dense_solve(g, S, B, on, dq, s);
    CK(cudaMemcpyAsync(B.h_int, B.status.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *status = B.h_int[0];
    if (scene_iters)
      for (int k = 0; k < ns; ++k) scene_iters[k] = 0;
    prof_work(K_BLOCK_INVERSE, 1, 2 * 1152.0 * B.h_int[2]);
    return 0;
  }
  // block-tridiagonal scenes are solved directly (tri.cu); the CG takes the others
  int n_pcg = 1, n_tri = 0;
  const int* pcg_mask = sc_on;
  if (o.tri) {
    tri_classify(g, S, B, 1, sc_on, s, &n_pcg, &n_tri);
    if (n_tri > 0) pcg_mask = B.pcg_on.p;
  }
  const bool run_pcg = n_tri == 0 || n_pcg > 0;
  static int max_blocks = 0, max_blocks1 = 0;
  if (!max_blocks) {
    int dev, sms, per, per1;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pcg, PCG_NT, 0));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, k_pcg1, PCG_NT, 0));
    max_blocks = sms * (per > 0 ? per : 1);
    max_blocks1 = sms * per1;
  }
  // one group per CTA when the groups fit one cooperative wave, else groups in loop steps
  const bool one = B.ngrp <= max_blocks1;
  int grid = one ? B.ngrp : (B.ngrp < max_blocks ? B.ngrp : max_blocks);
  if (grid < 1) grid = 1;
  PcgArgs a;
  a.nb = nb;
  a.ns = ns;
  a.ngrp = B.ngrp;
  a.row_ptr = S.row_ptr.p;
  a.rcol = B.rcol.p;
  a.rn = B.rn.p;
  a.Hrow = B.Hrow.p;
  a.Dinv = B.Dinv.p;
  a.b = B.grad.p;
  a.grp_body = B.grp_body.p;
  a.grp_n = B.grp_n.p;
  a.grp_scene = B.grp_scene.p;
  a.sc_gbeg = B.sc_gbeg.p;
  a.sc_gend = B.sc_gend.p;
  a.sc_on = pcg_mask;
  a.x = B.x.p;
  a.r = B.r.p;
  a.z = B.z.p;
  a.pbuf = B.p.p;
  a.q = B.qv.p;
  a.dq = dq;
  a.gpA = B.gpA.p;
  a.gpB = B.gpB.p;
  a.sc_rz = B.sc_rz.p;
  a.sc_bb = B.sc_bb.p;
  a.sc_conv = B.sc_conv.p;
  a.sc_iters = B.sc_iters.p;
  a.n_active = B.n_active.p;
  a.tol2 = rel_tol * rel_tol;
  a.maxit = max_iter < 0 ? 0 : max_iter;
  a.out = B.status.p;
  void* args[] = {&a};
  const void* kern = one ? (void*)k_pcg1 : (void*)k_pcg;
  if (run_pcg) KLAUNCH(K_PCG, s, CK(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(PCG_NT), args, 0, s)));
  const int nrows = 12 * nb;
  if (run_pcg && refine > 0) {
    // Iterative refinement: the PCG's recurrence residual drifts from b - H x as the
    // iterates converge, so the solution is corrected with the true residual computed
    // from the same row-block matrix, each correction solved by the same PCG to
    // refine_tol relative to its residual. The first iteration count is read with the
    // corrections' (one host read at the end).
    B.xr.ensure(nrows);
    B.rt.ensure(nrows);
    B.it_ref.ensure(2 * (size_t)ns + 2);
    B.h_ref.resize(2 * (size_t)ns + 2);
    CK(cudaMemcpyAsync(B.xr.p, B.x.p, nrows * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(B.it_ref.p, B.status.p + 1, sizeof(int), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(B.it_ref.p + 2, B.sc_iters.p, ns * sizeof(int), cudaMemcpyDeviceToDevice, s));
    PcgArgs c = a;
    c.b = B.rt.p;
    c.tol2 = refine_tol * refine_tol;
    B.dqc.ensure(nrows);
    c.dq = B.dqc.p;  // the correction's -d (unused)
    void* cargs[] = {&c};
    for (int k = 0; k < refine; ++k) {
      KLAUNCH(K_PCG, s, k_true_residual<<<nblk(nrows, 256), 256, 0, s>>>(nb, S.row_ptr.p, B.rcol.p, B.rn.p,
                                                                         B.Hrow.p, g.bscene, pcg_mask, B.grad.p,
                                                                         B.xr.p, B.rt.p));
      KLAUNCH(K_PCG, s, CK(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(PCG_NT), cargs, 0, s)));
      KLAUNCH(K_VEC, s, k_refine_add<<<nblk(nrows, 256), 256, 0, s>>>(nrows, B.xr.p, B.x.p, dq));
      KLAUNCH(K_VEC, s, k_iter_add<<<1, 32, 0, s>>>(ns, B.status.p + 1, B.sc_iters.p, B.it_ref.p));
    }
    CK(cudaMemcpyAsync(B.x.p, B.xr.p, nrows * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  if (n_tri > 0) tri_solve(g, S, B, sc_on, dq, s);
  CK(cudaMemcpyAsync(B.h_int, B.status.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
  if (run_pcg && refine > 0) {
    CK(cudaMemcpyAsync(B.h_ref.data(), B.it_ref.p, (2 + (size_t)ns) * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    B.h_int[1] = B.h_ref[0];
    if (scene_iters)
      for (int k = 0; k < ns; ++k) scene_iters[k] = B.h_ref[2 + k];
  } else if (run_pcg) {
    if (scene_iters) CK(cudaMemcpyAsync(scene_iters, B.sc_iters.p, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  } else {
    CK(cudaStreamSynchronize(s));
    B.h_int[1] = 0;
    if (scene_iters)
      for (int k = 0; k < ns; ++k) scene_iters[k] = 0;
  }
  *status = B.h_int[0];
  // per iteration: the kept blocks once (1152 B each) and ~6 vector streams
  prof_work(K_PCG, B.h_int[1], B.h_int[1] * (1152.0 * B.h_int[2] + 6 * 96.0 * nb) + 1152.0 * nb);
  prof_work(K_BLOCK_INVERSE, 1, 2 * 1152.0 * B.h_int[2]);
  return B.h_int[1];
}

void pcg_groups(const std::vector<int>& sc_beg, const std::vector<int>& sc_end, NewtonBufs& B, cudaStream_t s) {
  std::vector<int> gb, gn, gs, sgb, sge;
  for (size_t k = 0; k < sc_beg.size(); ++k) {
    sgb.push_back((int)gb.size());
    for (int b = sc_beg[k]; b < sc_end[k]; b += GB) {
      gb.push_back(b);
      gn.push_back(sc_end[k] - b < GB ? sc_end[k] - b : GB);
      gs.push_back((int)k);
    }
    sge.push_back((int)gb.size());
  }
  B.ngrp = (int)gb.size();
  B.h_sc_beg = sc_beg;
  B.h_sc_end = sc_end;
  DBuf<int>* dst[] = {&B.grp_body, &B.grp_n, &B.grp_scene, &B.sc_gbeg, &B.sc_gend};
  std::vector<int>* src[] = {&gb, &gn, &gs, &sgb, &sge};
  for (int i = 0; i < 5; ++i) {
    dst[i]->ensure(src[i]->size() + 1);
    if (!src[i]->empty())
      CK(cudaMemcpyAsync(dst[i]->p, src[i]->data(), src[i]->size() * sizeof(int), cudaMemcpyHostToDevice, s));
  }
  CK(cudaStreamSynchronize(s));
}

static EnergyArgs energy_args(const Geo& g, double alpha, PairSet& Snew, PairSet& Slag, bool with_bi) {
  EnergyArgs a;
  a.nb = g.nb;
  a.ns = g.ns;
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
  a.pt_ty = Snew.pt_ty.p;
  a.ee_ty = Snew.ee_ty.p;
  a.vg = Snew.vg.p;
  a.lpt_t = Slag.pt.p;
  a.lee_t = Slag.ee.p;
  a.lvg_t = Slag.vg.p;
  a.lpt_lag = Slag.pt_lag.p;
  a.lee_lag = Slag.ee_lag.p;
  a.lvg_lam = Slag.vg_lam.p;
  a.off = nullptr;
  a.chunk_off = nullptr;
  a.partial = nullptr;
  return a;
}

void energy_terms(const Geo& g, const Params& P, double alpha, PairSet& Snew, PairSet& Slag, double* out,
                  cudaStream_t s) {
  EnergyArgs a = energy_args(g, alpha, Snew, Slag, true);
  const int n[1 + NSEG] = {g.nb, a.npt, a.nee, a.nvg, a.lpt, a.lee, a.lvg};
  size_t o = 0;
  for (int k = 0; k <= NSEG; ++k) {
    if (n[k] > 0)
      KLAUNCH(K_ENERGY, s, k_energy_each<<<nblk(n[k], 128), 128, 0, s>>>(g, P, a, k - 1, n[k], out + o));
    o += n[k];
  }
}

void energy(const Geo& g, const Params& P, double alpha, PairSet& Snew, PairSet& Slag, bool with_bi, NewtonBufs& B,
            cudaStream_t s, double* out) {
  EnergyArgs a = energy_args(g, alpha, Snew, Slag, with_bi);
  const int ns = g.ns;
  B.e_off.ensure((size_t)NSEG * (ns + 1));
  B.e_chunk_cnt.ensure(ns + 1);
  B.e_chunk_off.ensure(ns + 1);
  B.e_out.ensure(ns);
  a.off = B.e_off.p;
  a.chunk_off = B.e_chunk_off.p;
  KLAUNCH(K_ENERGY, s, k_scene_offsets<<<nblk((long long)NSEG * (ns + 1), 128), 128, 0, s>>>(g, a, B.e_off.p));
  KLAUNCH(K_ENERGY, s, k_scene_chunks<<<nblk(ns, 128), 128, 0, s>>>(g, a, B.e_off.p, B.e_chunk_cnt.p));
  scan_exclusive_int(B.e_chunk_cnt.p, B.e_chunk_off.p, ns, B.e_chunk_off.p + ns, s, B.e_scan_tmp);
  // chunk count bound: every scene has at least one chunk, plus one per ECHUNK terms
  long long terms = (long long)(with_bi ? g.nb + a.npt + a.nee + a.nvg : 0) + a.lpt + a.lee + a.lvg;
  size_t max_chunks = (size_t)ns + (size_t)(terms / ECHUNK) + 1;
  B.red.ensure(max_chunks + 8);
  a.partial = B.red.p;
  const int G = 608;
  prof_work(K_ENERGY, (double)a.npt + a.nee + a.lpt + a.lee,
            136.0 * ((double)a.npt + a.nee + a.lpt + a.lee) + 96.0 * g.nb);
  KLAUNCH(K_ENERGY, s, k_energy<<<G, 256, 0, s>>>(g, P, a));
  KLAUNCH(K_ENERGY, s, k_scene_energy<<<nblk(32ll * ns, 128), 128, 0, s>>>(ns, B.e_chunk_off.p, B.red.p, B.e_out.p));
  CK(cudaMemcpyAsync(out, B.e_out.p, ns * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
}

void dots(const Geo& g, const double* dq, const double* grad, NewtonBufs& B, double* out, cudaStream_t s) {
  B.e_out.ensure(3 * (size_t)g.ns);
  KLAUNCH(K_DOTS, s, k_scene_dots<<<g.ns, 256, 0, s>>>(g.sc_beg, g.sc_end, dq, grad, B.e_out.p));
  CK(cudaMemcpyAsync(out, B.e_out.p, 3 * (size_t)g.ns * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
}

void scene_diff(const Geo& g, const double* a, const double* b, NewtonBufs& B, double* out, cudaStream_t s) {
  B.e_out.ensure(3 * (size_t)g.ns);
  KLAUNCH(K_DOTS, s, k_scene_diff<<<g.ns, 256, 0, s>>>(g.sc_beg, g.sc_end, a, b, B.e_out.p));
  CK(cudaMemcpyAsync(out, B.e_out.p, 3 * (size_t)g.ns * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
}

void launch_copy_scene(const Geo& g, double* dst, const double* src, const int* on, cudaStream_t st) {
  int n = 12 * g.nb;
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_copy_scene<<<nblk(n, 256), 256, 0, st>>>(dst, src, n, g.bscene, on));
}

void spmv(const Geo& g, const PairSet& S, NewtonBufs& B, const double* x, double* y, cudaStream_t st) {
  KLAUNCH(K_PCG, st, k_spmv<<<nblk((long long)g.nb * 16, 256), 256, 0, st>>>(g.nb, S.row_ptr.p, S.col.p, S.upidx.p,
                                                                            B.has.p, B.ovr.p, B.D.p, x, y));
}

void spmv_blocks(const Geo& g, const PairSet& S, const int* has, const double* ovr, const double* D, const double* x,
                 double* y, cudaStream_t st) {
  KLAUNCH(K_PCG, st, k_spmv<<<nblk((long long)g.nb * 16, 256), 256, 0, st>>>(g.nb, S.row_ptr.p, S.col.p, S.upidx.p,
                                                                            has, ovr, D, x, y));
}

void vg_lag_adjoint(const Geo& g, const Params& P, const PairSet& S, const double* w, double* out, cudaStream_t st) {
  KLAUNCH(K_BODY_SYSTEM, st, k_vg_lag_adj<<<nblk(g.nb, 128), 128, 0, st>>>(g, P, S.vg.p, S.vg_seg.p, w, out));
}

void launch_scale_scene(const Geo& g, double* v, const double* f, cudaStream_t st) {
  int n = 12 * g.nb;
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_scale_scene<<<nblk(n, 256), 256, 0, st>>>(v, n, g.bscene, f));
}
void launch_q_update_scene(const Geo& g, double* q, const double* dq, const double* alpha, cudaStream_t st) {
  int n = 12 * g.nb;
  if (n <= 0) return;
  KLAUNCH(K_VEC, st, k_q_update_scene<<<nblk(n, 256), 256, 0, st>>>(q, dq, n, g.bscene, alpha));
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
