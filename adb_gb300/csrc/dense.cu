// Dense direct solve of the Newton system, one scene at a time: the reference's
// "solver": "dense" (view/control.cpp:29-30), which solves dq = -big_hess.ldlt().solve(r)
// on the assembled 12 n x 12 n matrix (model/abd.cpp:233-264). The system is SPD after
// the PSD projection, so a Cholesky factorization without pivoting solves it.
//
// The scene's matrix is filled from the row-block copy of the system that the PCG
// setup builds (k_pcg_rows: every body's diagonal block and its kept neighbour blocks,
// row-major for its rows), padded to a multiple of the 64 x 64 tile with identity rows,
// factorized by a blocked right-looking Cholesky in one cooperative launch (per tile
// column: the diagonal tile on one CTA, the panel below it, then the trailing lower
// triangle of tiles, each phase ended by a grid barrier), and solved by blocked forward
// and back substitution in a second cooperative launch. Every sum runs in a fixed order,
// so results are reproducible bit for bit.
#include <cooperative_groups.h>

#include "abd_engine.h"

namespace cg = cooperative_groups;

namespace abd {
namespace {

constexpr int DT = 64;          // tile size
constexpr int DLD = DT + 1;     // shared-memory leading dimension (no bank conflicts on columns)
constexpr int DNT = 256;        // threads per CTA
constexpr size_t DSMEM = 2 * DT * DLD * sizeof(double);

inline int nblk_d(long long n, int t) { return (int)((n + t - 1) / t); }

__global__ void k_dense_zero(double* A, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    A[i] = 0.0;
}

// One warp per body of the scene [b0, b1): its row blocks into the dense matrix
// (leading dimension N). Every neighbour of a body lies in its scene.
__global__ void k_dense_fill(int b0, int b1, int N, const int* row_ptr, const int* rcol, const int* rn,
                             const double* Hrow, double* A) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int b = b0 + warp;
  if (b >= b1) return;
  const int base = b + row_ptr[b], n = rn[b];
  for (int j = 0; j < n; ++j) {
    const int c = rcol[base + j];
    const double* H = Hrow + (size_t)(base + j) * 144;
    for (int t = lane; t < 144; t += 32) {
      const int r = t / 12, col = t - 12 * r;
      A[(size_t)(12 * (b - b0) + r) * N + 12 * (c - b0) + col] = H[t];
    }
  }
}

// Identity on the padding rows; right-hand side y = b of the scene (0 when the scene is
// not solved, and on the padding).
__global__ void k_dense_rhs(int n, int N, int on, const double* b, double* A, double* y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (i >= n) A[(size_t)i * N + i] = 1.0;
  y[i] = (i < n && on) ? b[i] : 0.0;
}

// x = y on the scene's rows, dq = -x
__global__ void k_dense_out(int n, const double* y, double* x, double* dq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = y[i];
  dq[i] = -y[i];
}

struct DenseArgs {
  double* A;  // N x N row-major; the lower triangle becomes L
  double* y;  // N: right-hand side, then the solution
  int N, nt;  // size, tiles per side
  int* status;
};

__device__ __forceinline__ void load_tile(const double* A, int N, int ti, int tj, double* S) {
  const double* src = A + (size_t)ti * DT * N + (size_t)tj * DT;
  for (int t = threadIdx.x; t < DT * DT; t += blockDim.x) {
    const int r = t / DT, c = t - DT * r;
    S[r * DLD + c] = src[(size_t)r * N + c];
  }
}
__device__ __forceinline__ void store_tile(double* A, int N, int ti, int tj, const double* S) {
  double* dst = A + (size_t)ti * DT * N + (size_t)tj * DT;
  for (int t = threadIdx.x; t < DT * DT; t += blockDim.x) {
    const int r = t / DT, c = t - DT * r;
    dst[(size_t)r * N + c] = S[r * DLD + c];
  }
}

// (i, j) with 0 <= j <= i from the index t of the lower triangle in row order
__device__ __forceinline__ void tri_index(int t, int& i, int& j) {
  int r = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while ((r + 1) * (r + 2) / 2 <= t) ++r;
  while (r * (r + 1) / 2 > t) --r;
  i = r;
  j = t - r * (r + 1) / 2;
}

__global__ void __launch_bounds__(DNT) k_dense_chol(DenseArgs a) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double sm[];
  double* S0 = sm;
  double* S1 = sm + DT * DLD;
  const int N = a.N, nt = a.nt;
  for (int kb = 0; kb < nt; ++kb) {
    // 1. the diagonal tile, unblocked, on CTA 0
    if (blockIdx.x == 0) {
      load_tile(a.A, N, kb, kb, S0);
      __syncthreads();
      for (int k = 0; k < DT; ++k) {
        if (threadIdx.x == 0) {
          double d = S0[k * DLD + k];
          if (!(d > 0.0)) {  // not positive definite: flagged, the factor continues on 1
            a.status[0] = ABD_ERR_NOT_SPD;
            d = 1.0;
          }
          S0[k * DLD + k] = sqrt(d);
        }
        __syncthreads();
        const double lkk = S0[k * DLD + k];
        for (int i = k + 1 + threadIdx.x; i < DT; i += blockDim.x) S0[i * DLD + k] = S0[i * DLD + k] / lkk;
        __syncthreads();
        const int m = DT - k - 1, tot = m * (m + 1) / 2;
        for (int t = threadIdx.x; t < tot; t += blockDim.x) {
          int ii, jj;
          tri_index(t, ii, jj);
          const int i = k + 1 + ii, j = k + 1 + jj;
          S0[i * DLD + j] = __fma_rn(-S0[i * DLD + k], S0[j * DLD + k], S0[i * DLD + j]);
        }
        __syncthreads();
      }
      store_tile(a.A, N, kb, kb, S0);
    }
    grid.sync();
    // 2. the panel: L_ik = A_ik L_kk^-T for the tiles below the diagonal (thread per row)
    if (kb + 1 < nt) {
      bool loaded = false;
      for (int i = kb + 1 + blockIdx.x; i < nt; i += gridDim.x) {
        if (!loaded) {
          load_tile(a.A, N, kb, kb, S0);
          loaded = true;
        }
        load_tile(a.A, N, i, kb, S1);
        __syncthreads();
        if (threadIdx.x < DT) {
          const int r = threadIdx.x;
          for (int c = 0; c < DT; ++c) {
            double v = S1[r * DLD + c];
            for (int m = 0; m < c; ++m) v = __fma_rn(-S1[r * DLD + m], S0[c * DLD + m], v);
            S1[r * DLD + c] = v / S0[c * DLD + c];
          }
        }
        __syncthreads();
        store_tile(a.A, N, i, kb, S1);
        __syncthreads();
      }
    }
    grid.sync();
    // 3. the trailing lower triangle of tiles: A_ij -= L_ik L_jk^T, each thread a 4 x 4
    //    block of the 64 x 64 tile
    {
      const int m = nt - kb - 1, tot = m * (m + 1) / 2;
      const int ty = threadIdx.x / 16, tx = threadIdx.x - 16 * ty;
      for (int t = blockIdx.x; t < tot; t += gridDim.x) {
        int ii, jj;
        tri_index(t, ii, jj);
        const int i = kb + 1 + ii, j = kb + 1 + jj;
        load_tile(a.A, N, i, kb, S0);
        load_tile(a.A, N, j, kb, S1);
        __syncthreads();
        double acc[4][4] = {};
        for (int k = 0; k < DT; ++k) {
          double u[4], v[4];
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            u[p] = S0[(4 * ty + p) * DLD + k];
            v[p] = S1[(4 * tx + p) * DLD + k];
          }
#pragma unroll
          for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[p][q] = __fma_rn(u[p], v[q], acc[p][q]);
        }
        double* C = a.A + (size_t)i * DT * N + (size_t)j * DT;
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            double* e = C + (size_t)(4 * ty + p) * N + 4 * tx + q;
            *e = *e - acc[p][q];
          }
        __syncthreads();
      }
    }
    grid.sync();
  }
}

// L L^T x = y in place on y: blocked forward then back substitution.
__global__ void __launch_bounds__(DNT) k_dense_trsv(DenseArgs a) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double sm[];
  double* S0 = sm;
  double* v = sm + DT * DLD;  // DT values
  const int N = a.N, nt = a.nt;
  // forward: L y' = y
  for (int kb = 0; kb < nt; ++kb) {
    if (blockIdx.x == 0) {
      load_tile(a.A, N, kb, kb, S0);
      for (int t = threadIdx.x; t < DT; t += blockDim.x) v[t] = a.y[kb * DT + t];
      __syncthreads();
      for (int k = 0; k < DT; ++k) {
        if (threadIdx.x == 0) v[k] = v[k] / S0[k * DLD + k];
        __syncthreads();
        for (int i = k + 1 + threadIdx.x; i < DT; i += blockDim.x) v[i] = __fma_rn(-S0[i * DLD + k], v[k], v[i]);
        __syncthreads();
      }
      for (int t = threadIdx.x; t < DT; t += blockDim.x) a.y[kb * DT + t] = v[t];
    }
    grid.sync();
    for (int i = kb + 1 + blockIdx.x; i < nt; i += gridDim.x) {
      if (threadIdx.x < DT) {
        const int r = threadIdx.x;
        const double* L = a.A + (size_t)(i * DT + r) * N + (size_t)kb * DT;
        double s = 0.0;
        for (int c = 0; c < DT; ++c) s = __fma_rn(L[c], a.y[kb * DT + c], s);
        a.y[i * DT + r] -= s;
      }
    }
    grid.sync();
  }
  // back: L^T x = y'
  for (int kb = nt - 1; kb >= 0; --kb) {
    if (blockIdx.x == 0) {
      load_tile(a.A, N, kb, kb, S0);
      for (int t = threadIdx.x; t < DT; t += blockDim.x) v[t] = a.y[kb * DT + t];
      __syncthreads();
      for (int k = DT - 1; k >= 0; --k) {
        if (threadIdx.x == 0) v[k] = v[k] / S0[k * DLD + k];
        __syncthreads();
        for (int i = threadIdx.x; i < k; i += blockDim.x) v[i] = __fma_rn(-S0[k * DLD + i], v[k], v[i]);
        __syncthreads();
      }
      for (int t = threadIdx.x; t < DT; t += blockDim.x) a.y[kb * DT + t] = v[t];
    }
    grid.sync();
    for (int i = blockIdx.x; i < kb; i += gridDim.x) {
      if (threadIdx.x < DT) {
        const int r = threadIdx.x;  // row r of tile i: y_i[r] -= sum_c L_{kb,i}[c][r] x_kb[c]
        const double* L = a.A + (size_t)kb * DT * N + (size_t)i * DT + r;
        double s = 0.0;
        for (int c = 0; c < DT; ++c) s = __fma_rn(L[(size_t)c * N], a.y[kb * DT + c], s);
        a.y[i * DT + r] -= s;
      }
    }
    grid.sync();
  }
}

}  // namespace

void dense_solve(const Geo& g, PairSet& S, NewtonBufs& B, const std::vector<char>& on, double* dq, cudaStream_t s) {
  static int max_coop = 0;
  if (!max_coop) {
    int dev, sms, per1, per2;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaFuncSetAttribute(k_dense_chol, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DSMEM));
    CK(cudaFuncSetAttribute(k_dense_trsv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DSMEM));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, k_dense_chol, DNT, DSMEM));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_dense_trsv, DNT, DSMEM));
    max_coop = sms * (per1 < per2 ? per1 : per2);
    if (max_coop < 1) max_coop = 1;
  }
  size_t maxN = 0;
  for (size_t k = 0; k < B.h_sc_beg.size(); ++k) {
    size_t n = 12 * (size_t)(B.h_sc_end[k] - B.h_sc_beg[k]);
    size_t N = (n + DT - 1) / DT * DT;
    maxN = N > maxN ? N : maxN;
  }
  B.dense_A.ensure(maxN * maxN);
  B.dense_y.ensure(maxN);
  for (size_t k = 0; k < B.h_sc_beg.size(); ++k) {
    const int b0 = B.h_sc_beg[k], b1 = B.h_sc_end[k];
    const int n = 12 * (b1 - b0), N = (n + DT - 1) / DT * DT, nt = N / DT;
    if (!on[k]) {
      // a scene that is not iterating takes no step; its off-diagonal blocks are stale
      // (its pair terms were skipped), so its matrix is not factorized
      KLAUNCH(K_VEC, s, k_dense_zero<<<nblk_d(n, 256), 256, 0, s>>>(B.x.p + 12 * (size_t)b0, n));
      KLAUNCH(K_VEC, s, k_dense_zero<<<nblk_d(n, 256), 256, 0, s>>>(dq + 12 * (size_t)b0, n));
      continue;
    }
    const int zgrid = nblk_d((long long)N * N, 256) < 1216 ? nblk_d((long long)N * N, 256) : 1216;
    KLAUNCH(K_PCG, s, k_dense_zero<<<zgrid, 256, 0, s>>>(B.dense_A.p, (long long)N * N));
    KLAUNCH(K_PCG, s, k_dense_fill<<<nblk_d(32ll * (b1 - b0), 256), 256, 0, s>>>(b0, b1, N, S.row_ptr.p, B.rcol.p,
                                                                                B.rn.p, B.Hrow.p, B.dense_A.p));
    KLAUNCH(K_PCG, s, k_dense_rhs<<<nblk_d(N, 256), 256, 0, s>>>(n, N, 1, B.grad.p + 12 * (size_t)b0, B.dense_A.p,
                                                                 B.dense_y.p));
    DenseArgs a{B.dense_A.p, B.dense_y.p, N, nt, B.status.p};
    const int work = nt * (nt + 1) / 2;
    int grid = work < max_coop ? work : max_coop;
    if (grid < 1) grid = 1;
    void* args[] = {&a};
    KLAUNCH(K_PCG, s, CK(cudaLaunchCooperativeKernel((void*)k_dense_chol, dim3(grid), dim3(DNT), args, DSMEM, s)));
    int gs = nt < max_coop ? nt : max_coop;
    KLAUNCH(K_PCG, s, CK(cudaLaunchCooperativeKernel((void*)k_dense_trsv, dim3(gs), dim3(DNT), args, DSMEM, s)));
    KLAUNCH(K_VEC, s, k_dense_out<<<nblk_d(n, 256), 256, 0, s>>>(n, B.dense_y.p, B.x.p + 12 * (size_t)b0,
                                                                 dq + 12 * (size_t)b0));
    // matrix fill, factor and both substitutions: (N^3 / 3 + 2 N^2) flops; bytes: the
    // matrix written, read by the factor, and read twice by the solves
    prof_work(K_PCG, 1, 4.0 * 8.0 * (double)N * N);
  }
}

}  // namespace abd
