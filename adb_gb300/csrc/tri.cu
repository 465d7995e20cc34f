// Direct solve of block-tridiagonal scenes (chains, stacks): the Newton matrix of a scene
// whose contacts only join consecutive bodies is block-tridiagonal in body order. The
// reference solves every Newton system with a sparse direct factorization (Pardiso LLT,
// model/abd.cpp:233-264), which on such a matrix is a block Cholesky along the bodies;
// here each run of linked bodies (a maximal sequence i, i+1, ... with a contact block
// between each neighbour pair) is factorized and solved by one CTA:
//
//   S_0 = D_0,  S_k = D_k - W_{k-1}^T W_{k-1},  S_k = L_k L_k^T,  W_k = L_k^-1 U_k
//   (U_k = H[k][k+1]);  y_k = L_k^-1 (b_k - W_{k-1}^T y_{k-1});
//   x_last = L_last^-T y_last,  x_k = L_k^-T (y_k - W_k x_{k+1}).
//
// Runs are independent, so a chain broken into segments by missing contacts solves in
// parallel; a body without neighbours is a run of one. The preconditioned CG keeps the
// other scenes. Every sum runs in a fixed order, and a run's arithmetic depends only on
// its own blocks, so a scene gets the same solution in a batch as alone.
#include "abd_engine.h"

namespace abd {
namespace {

constexpr int TNT = 160;  // threads per run: 144 for the 12 x 12 entries, lanes for the rest

inline int nblk_t(long long n, int t) { return (int)((n + t - 1) / t); }

// Flags of the block structure from the row-block copy of the system (k_pcg_rows: per body
// its diagonal block, then the neighbour blocks that hold a contribution): link[i] = 1 when
// body i has a block with body i + 1; a scene with any block between bodies further apart
// is marked in bad[scene].
__global__ void k_tri_mark(int nb, const int* row_ptr, const int* rcol, const int* rn, const int* bscene, int* link,
                           int* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb) return;
  const int base = i + row_ptr[i], n = rn[i];
  int l = 0;
  bool far = false;
  for (int j = 1; j < n; ++j) {
    const int c = rcol[base + j];
    if (c == i + 1) l = 1;
    else if (c != i - 1) far = true;
  }
  link[i] = l;
  if (far) atomicOr(&bad[bscene[i]], 1);
}

// Per scene: solved directly (tri_on) or by the CG (pcg_on); cnt[0] / cnt[1] count them.
__global__ void k_tri_masks(int ns, int enable, const int* sc_on, const int* bad, int* tri_on, int* pcg_on, int* cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int on = sc_on[k] != 0;
  const int t = enable && on && !bad[k];
  tri_on[k] = t;
  pcg_on[k] = on && !t;
  if (t) atomicAdd(&cnt[1], 1);
  if (on && !t) atomicAdd(&cnt[0], 1);
}

struct TriArgs {
  const int *row_ptr, *rcol, *rn;
  const double* Hrow;
  const int *bscene, *sc_on, *tri_on, *link;
  const double* b;
  double *Li, *W, *y;  // per body: inverse of the factor's diagonal block, coupling block, forward solution
  double *x, *dq;
  int* status;
};

// Pivot of a right-looking Cholesky: r = 1 / sqrt(a), L_kk = a r. A non-positive pivot
// sets ABD_ERR_NOT_SPD and is replaced by 1e-300, as the block-Jacobi preconditioner does.
__device__ __forceinline__ void tri_pivot(double a, double* r, double* lkk, int* status) {
  if (!(a > 0)) {
    atomicExch(status, (int)ABD_ERR_NOT_SPD);
    a = 1e-300;
  }
  const double q = rsqrt(a);
  *r = q;
  *lkk = a * q;
}

// One CTA per body; the CTA of the first body of each run in a directly solved scene
// factorizes and solves the run. Bodies of scenes that take no step get x = 0, dq = -0
// (what the CG writes for them).
//
// A link's 12 x 12 work is spread over 144 threads (thread (i, j) = (t / 12, t % 12)),
// because on this part a dependent FP64 instruction of one warp waits ~64 cycles: the
// Cholesky factor is right-looking, one barrier per column (the column scaled and the
// trailing triangle updated in the same phase; the thread that updates the next pivot takes
// its reciprocal square root), and row c of L^-1, which needs L's column c, is formed one
// phase later by the threads of columns <= c, which the factorization no longer uses. The
// next link's diagonal block and right-hand side are loaded while this one factorizes.
__global__ void __launch_bounds__(TNT) k_tri_solve(TriArgs a) {
  __shared__ double sA[12][13], sL[12][13], sT[12][13], sLi[12][13], sW[12][13], sU[12][13];
  __shared__ double sy[12], st[12], sx[12], sv[12], sR[12];
  __shared__ int s_u;
  const int b0 = blockIdx.x, t = threadIdx.x;
  const int sc = a.bscene[b0];
  if (!a.sc_on[sc]) {
    if (t < 12) {
      a.x[12 * b0 + t] = 0.0;
      a.dq[12 * b0 + t] = -0.0;
    }
    return;
  }
  if (!a.tri_on[sc]) return;
  if (b0 > 0 && a.bscene[b0 - 1] == sc && a.link[b0 - 1]) return;  // not the first body of its run
  const bool act = t < 144;
  const int ei = t / 12, ej = t - 12 * (t / 12);
  int k = b0;
  int base = k + a.row_ptr[k];
  // this link's diagonal entries (i, j), (j, i) and right-hand side entry
  double d_ij = act ? a.Hrow[(size_t)base * 144 + 12 * ei + ej] : 0.0;
  double d_ji = act ? a.Hrow[(size_t)base * 144 + 12 * ej + ei] : 0.0;
  double b_t = t < 12 ? a.b[12 * k + t] : 0.0;
  for (;;) {
    if (t == 0) {
      // the coupling block to body k + 1 in k's row list (rows of k, columns of k + 1)
      int u = -1;
      if (a.link[k]) {
        const int n = a.rn[k];
        for (int j = 1; j < n; ++j)
          if (a.rcol[base + j] == k + 1) u = base + j;
      }
      s_u = u;
    }
    // S_k = sym(D_k) - W_{k-1}^T W_{k-1}; right-hand side b_k - W_{k-1}^T y_{k-1}
    if (act) {
      double v = 0.5 * (d_ij + d_ji);
      if (k > b0) {
#pragma unroll
        for (int m = 0; m < 12; ++m) v -= sW[m][ei] * sW[m][ej];
      }
      sA[ei][ej] = v;
      sT[ei][ej] = ei == ej ? 1.0 : 0.0;
      if (t == 0) tri_pivot(v, &sR[0], &sL[0][0], a.status);
    }
    if (t < 12) {
      double v = b_t;
      if (k > b0) {
#pragma unroll
        for (int m = 0; m < 12; ++m) v -= sW[m][t] * sy[m];
      }
      st[t] = v;
    }
    __syncthreads();
    const int u = s_u;
    if (act && u >= 0) {
      sU[ei][ej] = a.Hrow[(size_t)u * 144 + t];
      // the next link's block and right-hand side, in flight during the factorization
      base = (k + 1) + a.row_ptr[k + 1];
      d_ij = a.Hrow[(size_t)base * 144 + 12 * ei + ej];
      d_ji = a.Hrow[(size_t)base * 144 + 12 * ej + ei];
      if (t < 12) b_t = a.b[12 * (k + 1) + t];
    }
    // S = L L^T column by column (threads of columns >= c); row c - 1 of L^-1 beside it
    // (threads of columns <= c - 1). T holds I minus the finished rows' contributions.
    for (int c = 0; c <= 12; ++c) {
      if (act && c < 12 && ej >= c && ei >= ej) {
        const double r = sR[c];
        if (ej == c) {
          if (ei > c) sL[ei][c] = sA[ei][c] * r;
        } else {
          const double v = sA[ei][ej] - (sA[ei][c] * r) * (sA[ej][c] * r);
          sA[ei][ej] = v;
          if (ei == ej && ej == c + 1) tri_pivot(v, &sR[c + 1], &sL[c + 1][c + 1], a.status);
        }
      }
      if (act && c >= 1 && ej <= c - 1 && ei >= c - 1) {
        const int rw = c - 1;
        const double l = sT[rw][ej] * sR[rw];
        if (ei == rw) sLi[rw][ej] = l;
        else sT[ei][ej] -= sL[ei][rw] * l;
      }
      __syncthreads();
    }
    // y_k = L^-1 rhs, W_k = L^-1 U_k (L^-1 lower triangular)
    if (t < 12) {
      double v = 0.0;
      for (int m = 0; m <= t; ++m) v += sLi[t][m] * st[m];
      sy[t] = v;
      a.y[12 * k + t] = v;
    }
    if (act) {
      a.Li[(size_t)144 * k + t] = ej <= ei ? sLi[ei][ej] : 0.0;
      if (u >= 0) {
        double v = 0.0;
        for (int m = 0; m <= ei; ++m) v += sLi[ei][m] * sU[m][ej];
        sW[ei][ej] = v;
        a.W[(size_t)144 * k + t] = v;
      }
    }
    __syncthreads();
    if (u < 0) break;
    ++k;
  }
  // back substitution from the last body of the run
  for (int kk = k; kk >= b0; --kk) {
    if (t < 12) {
      double v = a.y[12 * kk + t];
      if (kk < k) {
        const double* W = a.W + (size_t)144 * kk;
#pragma unroll
        for (int m = 0; m < 12; ++m) v -= W[12 * t + m] * sx[m];
      }
      sv[t] = v;
    }
    __syncthreads();
    if (t < 12) {
      const double* Li = a.Li + (size_t)144 * kk;
      double v = 0.0;
      for (int m = t; m < 12; ++m) v += Li[12 * m + t] * sv[m];
      a.x[12 * kk + t] = v;
      a.dq[12 * kk + t] = -v;
      sx[t] = v;
    }
    __syncthreads();
  }
}

}  // namespace

void tri_classify(const Geo& g, PairSet& S, NewtonBufs& B, int enable, const int* sc_on, cudaStream_t s,
                  int* n_pcg, int* n_tri) {
  const int nb = g.nb, ns = g.ns;
  B.tri_bad.ensure(ns);
  B.tri_on.ensure(ns);
  B.pcg_on.ensure(ns);
  B.tri_cnt.ensure(2);
  B.tri_link.ensure(nb);
  CK(cudaMemsetAsync(B.tri_bad.p, 0, ns * sizeof(int), s));
  CK(cudaMemsetAsync(B.tri_cnt.p, 0, 2 * sizeof(int), s));
  KLAUNCH(K_BLOCK_INVERSE, s, k_tri_mark<<<nblk_t(nb, 256), 256, 0, s>>>(nb, S.row_ptr.p, B.rcol.p, B.rn.p, g.bscene,
                                                                       B.tri_link.p, B.tri_bad.p));
  KLAUNCH(K_BLOCK_INVERSE, s, k_tri_masks<<<nblk_t(ns, 256), 256, 0, s>>>(ns, enable, sc_on, B.tri_bad.p, B.tri_on.p,
                                                                        B.pcg_on.p, B.tri_cnt.p));
  CK(cudaMemcpyAsync(B.h_int + 8, B.tri_cnt.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *n_pcg = B.h_int[8];
  *n_tri = B.h_int[9];
}

void tri_solve(const Geo& g, PairSet& S, NewtonBufs& B, const int* sc_on, double* dq, cudaStream_t s) {
  const int nb = g.nb;
  B.tri_Li.ensure(144 * (size_t)nb);
  B.tri_W.ensure(144 * (size_t)nb);
  B.tri_y.ensure(12 * (size_t)nb);
  TriArgs a{S.row_ptr.p, B.rcol.p, B.rn.p, B.Hrow.p, g.bscene, sc_on, B.tri_on.p, B.tri_link.p, B.grad.p,
            B.tri_Li.p, B.tri_W.p, B.tri_y.p, B.x.p, dq, B.status.p};
  KLAUNCH(K_PCG, s, k_tri_solve<<<nb, TNT, 0, s>>>(a));
  // per body: its diagonal and coupling blocks read, the factor's blocks written and read
  // back (4 x 1152 B), the right-hand side, y and x
  prof_work(K_PCG, 1, 6.0 * 1152.0 * nb);
}

}  // namespace abd
