// Allocation-free variant of the batched point-triangle time-of-impact entry point.
//
// Some callers cannot allocate device memory at the point where they need this
// function: code that runs while a stream is being captured into a CUDA graph (a
// cudaMalloc there breaks or invalidates the capture), and host applications whose
// device memory is owned entirely by their own pool allocator or by a framework that
// forbids driver allocations in its hot loop. For them, abd_pt_min_toi_noalloc takes the
// caller's device buffers for inputs and outputs and keeps its only scratch -- the
// per-block minima of the reduction -- in a fixed array in this library's device
// memory, so the call never allocates.
//
// The scratch array below is a device symbol: every GPU that loads the library holds it
// until the process exits. Host code must not pass its name to a kernel (on the host it
// is only a stand-in, not a device address); its device address is looked up once per
// device with cudaGetSymbolAddress and cached. The cache assumes one CUDA context per
// device for the life of the process: after cudaDeviceReset (or any teardown that
// re-creates the primary context) the cached address is stale, so a process that resets
// a device must not call this entry point again. Every call shares the array: calls that
// overlap on the GPU (different streams, or different host threads on one device) race
// on it and must be serialised by the caller. The error message is kept per host thread,
// so concurrent failing calls never write to one string.
#include <mutex>
#include <string>

#include "abd_engine.h"
#include "abd_exact.cuh"

namespace abd {
namespace {

constexpr int NOALLOC_THREADS = 128;
constexpr int NOALLOC_MAX_BLOCKS = ABD_NOALLOC_MAX_N / NOALLOC_THREADS;

// Per-block minima of the time-of-impact reduction (256 kB).
static __device__ __align__(256) double g_noalloc_partial[NOALLOC_MAX_BLOCKS];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kMaxDevices] = {};
thread_local std::string g_noalloc_err;  // last error of the calling host thread

__device__ __forceinline__ d3 ld(const double* x, int i) { return mk(x[3 * i], x[3 * i + 1], x[3 * i + 2]); }

// One thread per trajectory (same device function as the batched entry point), then a
// fixed-order block minimum into the block's scratch slot. Every slot the second pass
// reads is written in the same call, so the scratch needs no clearing.
__global__ void __launch_bounds__(NOALLOC_THREADS) k_toi_blockmin(int n, const double* x, double* toi,
                                                                 double* partial) {
  __shared__ double sh[NOALLOC_THREADS / 32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double t = 1.0;
  if (i < n) {
    const double* p = x + 24 * (size_t)i;
    d3 a[4] = {ld(p, 0), ld(p, 1), ld(p, 2), ld(p, 3)};
    d3 b[4] = {ld(p, 4), ld(p, 5), ld(p, 6), ld(p, 7)};
    t = pt_collision_time(a[0], a + 1, b[0], b + 1);
    toi[i] = t;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t = dmin(t, __shfl_xor_sync(0xffffffffu, t, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = sh[0];
    for (int w = 1; w < NOALLOC_THREADS / 32; ++w) m = dmin(m, sh[w]);
    partial[blockIdx.x] = m;
  }
}

__global__ void k_min_partials(int nblocks, const double* partial, double* out) {
  __shared__ double sh[32];
  double m = 1.0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) m = dmin(m, partial[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = dmin(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = sh[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = dmin(r, sh[w]);
    *out = r;
  }
}

// Device address of the scratch array on the current device (looked up on the first
// call per device; that first call must not happen inside a stream capture).
int scratch_on_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    g_noalloc_err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return ABD_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    g_noalloc_err = "device index out of range";
    return ABD_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_partial);
    if (e != cudaSuccess || !p) {
      g_noalloc_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return ABD_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return ABD_OK;
}

}  // namespace
}  // namespace abd

extern "C" {

int abd_pt_min_toi_noalloc(int n, const double* d_x, double* d_toi, double* d_min, void* stream) {
  using namespace abd;
  if (n < 1 || !d_x || !d_toi || !d_min) {
    g_noalloc_err = "abd_pt_min_toi_noalloc: n must be >= 1 and all buffers non-null";
    return ABD_ERR_INVALID;
  }
  if (n > ABD_NOALLOC_MAX_N) {
    g_noalloc_err = "abd_pt_min_toi_noalloc: n exceeds ABD_NOALLOC_MAX_N (" + std::to_string(ABD_NOALLOC_MAX_N) +
                    "); split the batch";
    return ABD_ERR_INVALID;
  }
  double* partial = nullptr;
  int rc = scratch_on_current_device(&partial);
  if (rc != ABD_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int blocks = (n + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
  k_toi_blockmin<<<blocks, NOALLOC_THREADS, 0, s>>>(n, d_x, d_toi, partial);
  k_min_partials<<<1, 256, 0, s>>>(blocks, partial, d_min);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_noalloc_err = std::string("launch: ") + cudaGetErrorString(e);
    return ABD_ERR_CUDA;
  }
  return ABD_OK;
}

const char* abd_noalloc_last_error(void) { return abd::g_noalloc_err.c_str(); }

}  // extern "C"
