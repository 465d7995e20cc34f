// Batched per-primitive entry points mirroring the reference's python module `abdtk`
// (python/bindings.cpp:42-83: ipc_hess_pt_12x12, ipc_hess_ee_12x12, pt_collision_time,
// ee_collision_time), evaluated on the GPU with the same device code as the step, and
// the FP64 throughput probe used as the roofline denominator of FP64-bound kernels.
#include <vector>

#include "abd_engine.h"
#include "abd_ipc.cuh"

namespace abd {
namespace {

__device__ __forceinline__ d3 ld12(const double* x, int i) { return mk(x[3 * i], x[3 * i + 1], x[3 * i + 2]); }

__global__ void k_distance(int kind, int n, const double* x, int* type, double* dist) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = x + 12 * i;
  d3 a = ld12(p, 0), b = ld12(p, 1), c = ld12(p, 2), d = ld12(p, 3);
  int ty = kind == 0 ? pt_type(a, b, c, d) : ee_type(a, b, c, d);
  type[i] = ty;
  dist[i] = kind == 0 ? pt_dist(a, b, c, d, ty) : ee_dist(a, b, c, d, ty);
}

// Vertex-space Hessian H = (Q (x) I) S (Q (x) I)^T and gradient of one pair.
__global__ void k_hess(int kind, int n, const double* x, const int* type, const double* dist, double dhat,
                       double kappa, double eps_x, int psd, double* H, double* g, double* moll) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = x + 12 * i;
  d3 X[4] = {ld12(p, 0), ld12(p, 1), ld12(p, 2), ld12(p, 3)};
  int ty = type ? type[i] : -1;
  if (ty < 0) ty = kind == 0 ? pt_type(X[0], X[1], X[2], X[3]) : ee_type(X[0], X[1], X[2], X[3]);
  double d = (dist && type && type[i] >= 0) ? dist[i]
                                            : (kind == 0 ? pt_dist(X[0], X[1], X[2], X[3], ty) : ee_dist(X[0], X[1], X[2], X[3], ty));
  double S[9][9];
  d3 gv[4];
  pair_reduced(kind, ty, X, d, BarrierP{dhat, kappa}, eps_x, psd != 0, S, gv);
  for (int a = 0; a < 12; ++a)
    for (int b = 0; b < 12; ++b) {
      int ia = a / 3, ra = a % 3, ib = b / 3, rb = b % 3;
      double s = 0;
      for (int qa = 0; qa < 3; ++qa)
        for (int qb = 0; qb < 3; ++qb) s += Qe(ia, qa) * S[3 * qa + ra][3 * qb + rb] * Qe(ib, qb);
      H[144 * (size_t)i + 12 * a + b] = s;
    }
  for (int k = 0; k < 4; ++k) {
    g[12 * (size_t)i + 3 * k] = gv[k].x;
    g[12 * (size_t)i + 3 * k + 1] = gv[k].y;
    g[12 * (size_t)i + 3 * k + 2] = gv[k].z;
  }
  if (moll) {
    double m = 1.0;
    if (kind == 1) {
      d3 u = fsub(X[1], X[0]), v = fsub(X[3], X[2]);
      double ex = eps_x * fdot(u, u) * fdot(v, v);
      d3 cr = fcross(u, v);
      double xx = fdot(cr, cr);
      if (xx < ex) {
        double xe = xx / ex;
        m = (-xe + 2.0) * xe;
      }
    }
    moll[i] = m;
  }
}

__global__ void k_toi(int kind, int n, const double* x, double* toi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = x + 24 * i;
  d3 a[4] = {ld12(p, 0), ld12(p, 1), ld12(p, 2), ld12(p, 3)};
  d3 b[4] = {ld12(p, 4), ld12(p, 5), ld12(p, 6), ld12(p, 7)};
  if (kind == 0) {
    toi[i] = pt_collision_time(a[0], a + 1, b[0], b + 1);
  } else {
    d3 ei0[2] = {a[0], a[1]}, ej0[2] = {a[2], a[3]}, ei1[2] = {b[0], b[1]}, ej1[2] = {b[2], b[3]};
    toi[i] = ee_collision_time(ei0, ej0, ei1, ej1);
  }
}

// Independent FMA chains; result stored per thread so nothing is optimised away.
__global__ void k_fma64(double* out, int iters, double a, double b) {
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double x0 = tid * 1e-7, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[tid] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
struct DevArr {
  T* p = nullptr;
  explicit DevArr(size_t n) { CK(cudaMalloc(&p, (n ? n : 1) * sizeof(T))); }
  ~DevArr() {
    if (p) cudaFree(p);
  }
};

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

std::string g_prim_err;

template <typename F>
int guard(F&& f) {
  try {
    f();
    return ABD_OK;
  } catch (const CudaError& e) {
    g_prim_err = std::string(e.where) + ": " + cudaGetErrorString(e.code);
    return ABD_ERR_CUDA;
  }
}

int hess_batch(int kind, int n, const double* x, const int* type, const double* dist, double dhat, double kappa,
               double eps_x, int psd, double* H, double* g, double* moll) {
  if (n < 0 || !x || !H || !g) return ABD_ERR_INVALID;
  if (n == 0) return ABD_OK;
  return guard([&]() {
    DevArr<double> dx(12 * (size_t)n), dd(n), dH(144 * (size_t)n), dg(12 * (size_t)n), dm(n);
    DevArr<int> dt(n);
    CK(cudaMemcpy(dx.p, x, 12 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    if (type) CK(cudaMemcpy(dt.p, type, n * sizeof(int), cudaMemcpyHostToDevice));
    if (dist) CK(cudaMemcpy(dd.p, dist, n * sizeof(double), cudaMemcpyHostToDevice));
    k_hess<<<nblk(n, 64), 64>>>(kind, n, dx.p, type ? dt.p : nullptr, dist ? dd.p : nullptr, dhat, kappa, eps_x, psd,
                                dH.p, dg.p, moll ? dm.p : nullptr);
    CK(cudaGetLastError());
    CK(cudaMemcpy(H, dH.p, 144 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(g, dg.p, 12 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    if (moll) CK(cudaMemcpy(moll, dm.p, n * sizeof(double), cudaMemcpyDeviceToHost));
  });
}

int toi_batch(int kind, int n, const double* x, double* toi) {
  if (n < 0 || !x || !toi) return ABD_ERR_INVALID;
  if (n == 0) return ABD_OK;
  return guard([&]() {
    DevArr<double> dx(24 * (size_t)n), dt(n);
    CK(cudaMemcpy(dx.p, x, 24 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    k_toi<<<nblk(n, 128), 128>>>(kind, n, dx.p, dt.p);
    CK(cudaGetLastError());
    CK(cudaMemcpy(toi, dt.p, n * sizeof(double), cudaMemcpyDeviceToHost));
  });
}

int dist_batch(int kind, int n, const double* x, int* type, double* dist) {
  if (n < 0 || !x || !type || !dist) return ABD_ERR_INVALID;
  if (n == 0) return ABD_OK;
  return guard([&]() {
    DevArr<double> dx(12 * (size_t)n), dd(n);
    DevArr<int> dt(n);
    CK(cudaMemcpy(dx.p, x, 12 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    k_distance<<<nblk(n, 128), 128>>>(kind, n, dx.p, dt.p, dd.p);
    CK(cudaGetLastError());
    CK(cudaMemcpy(type, dt.p, n * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dist, dd.p, n * sizeof(double), cudaMemcpyDeviceToHost));
  });
}

}  // namespace

double measure_fp64_gflops() {
  int dev, sms;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int blocks = sms * 8, threads = 256, n = blocks * threads, iters = 2048;
  DevArr<double> out(n);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    CK(cudaEventRecord(e0));
    k_fma64<<<blocks, threads>>>(out.p, iters, 0.999999, 1e-9);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 2.0 * 8.0 * iters * (double)n / (best * 1e-3) / 1e9;
}

}  // namespace abd

extern "C" {

int abd_ipc_hess_pt_batch(int n, const double* x, const int* type, const double* dist, double dhat, double kappa,
                          int psd, double* H, double* g) {
  return abd::hess_batch(0, n, x, type, dist, dhat, kappa, 0.0, psd, H, g, nullptr);
}
int abd_ipc_hess_ee_batch(int n, const double* x, const int* type, const double* dist, double dhat, double kappa,
                          double eps_x, int psd, double* H, double* g, double* mollifier) {
  return abd::hess_batch(1, n, x, type, dist, dhat, kappa, eps_x, psd, H, g, mollifier);
}
int abd_pt_collision_time_batch(int n, const double* x, double* toi) { return abd::toi_batch(0, n, x, toi); }
int abd_ee_collision_time_batch(int n, const double* x, double* toi) { return abd::toi_batch(1, n, x, toi); }
int abd_pt_distance_batch(int n, const double* x, int* type, double* dist) {
  return abd::dist_batch(0, n, x, type, dist);
}
int abd_ee_distance_batch(int n, const double* x, int* type, double* dist) {
  return abd::dist_batch(1, n, x, type, dist);
}
double abd_measure_fp64_gflops(void) {
  try {
    return abd::measure_fp64_gflops();
  } catch (...) {
    return -1.0;
  }
}

}  // extern "C"
