// Deterministic device exclusive scans (int and int64) used by the ordered compactions
// of the culling stages: block-local scans, a recursive scan of the block totals, and
// an add pass. The result does not depend on scheduling. The grand total is written by
// the tile scan (one tile) or by the add pass (several), not by a launch of its own:
// a scan of up to 2048 entries is one launch.
#include "abd_engine.h"

namespace abd {

namespace {
constexpr int SCAN_T = 512;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_T * SCAN_ITEMS;

template <typename T>
__device__ T block_excl_scan(T v, T* sh, T& total) {
  // warp inclusive scan
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    T s = (lane < (SCAN_T / 32)) ? sh[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (SCAN_T / 32)) sh[lane] = s;
  }
  __syncthreads();
  T wp = (w > 0) ? sh[w - 1] : T(0);
  total = sh[SCAN_T / 32 - 1];
  __syncthreads();
  return wp + x - v;
}

template <typename T>
__global__ void k_scan_tiles(const T* in, T* out, int n, T* tile_sums, T* grand) {
  __shared__ T sh[32];
  int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T loc = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int i = base + k;
    v[k] = (i < n) ? in[i] : T(0);
    loc += v[k];
  }
  T total;
  T pre = block_excl_scan<T>(loc, sh, total);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int i = base + k;
    if (i < n) out[i] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) {
    tile_sums[blockIdx.x] = total;
    if (grand && gridDim.x == 1) *grand = total;
  }
}

template <typename T>
__global__ void k_scan_add(T* out, int n, const T* tile_off, const T* in, T* grand) {
  int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  T add = tile_off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int i = base + k;
    if (i < n) {
      const T v = out[i] + add;
      out[i] = v;
      if (grand && i == n - 1) *grand = v + in[i];
    }
  }
}

// Scans of up to SCAN_ONE entries in one CTA (one launch instead of three): each thread
// sums a contiguous run of ONE_ITEMS entries, the CTA scans the run sums, and each thread
// writes its run from its offset.
constexpr int ONE_T = 1024;
constexpr int ONE_ITEMS = 16;
constexpr int SCAN_ONE = ONE_T * ONE_ITEMS;
template <typename T>
__global__ void __launch_bounds__(ONE_T) k_scan_one(const T* in, T* out, int n, T* grand) {
  __shared__ T sh[32];
  const int base = threadIdx.x * ONE_ITEMS;
  T v[ONE_ITEMS];
  T loc = 0;
#pragma unroll
  for (int k = 0; k < ONE_ITEMS; ++k) {
    const int i = base + k;
    v[k] = (i < n) ? in[i] : T(0);
    loc += v[k];
  }
  // CTA exclusive scan of the run sums (warp scans, then the warp totals)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = loc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    T t = sh[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    sh[lane] = t;
  }
  __syncthreads();
  T pre = (w > 0 ? sh[w - 1] : T(0)) + x - loc;
#pragma unroll
  for (int k = 0; k < ONE_ITEMS; ++k) {
    const int i = base + k;
    if (i < n) out[i] = pre;
    pre += v[k];
  }
  if (grand && threadIdx.x == 0) *grand = sh[31];
}

// Exclusive scan of in[0, n) into out; *grand (if not null) receives the total.
template <typename T>
void scan_rec(const T* in, T* out, int n, cudaStream_t s, T* tmp, size_t tmp_cap, T* grand) {
  if (n <= 0) return;
  int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles > 1 && n <= SCAN_ONE) {
    KLAUNCH(K_SCAN, s, (k_scan_one<T><<<1, ONE_T, 0, s>>>(in, out, n, grand)));
    return;
  }
  T* sums = tmp;
  T* sums_off = tmp + tiles;
  if ((size_t)(2 * tiles) > tmp_cap) throw CudaError{cudaErrorMemoryAllocation, "scan scratch"};
  KLAUNCH(K_SCAN, s, (k_scan_tiles<T><<<tiles, SCAN_T, 0, s>>>(in, out, n, sums, grand)));
  if (tiles > 1) {
    scan_rec<T>(sums, sums_off, tiles, s, tmp + 2 * tiles, tmp_cap - 2 * tiles, nullptr);
    KLAUNCH(K_SCAN, s, (k_scan_add<T><<<tiles, SCAN_T, 0, s>>>(out, n, sums_off, in, grand)));
  }
}

template <typename T>
size_t scan_scratch(int n) {
  size_t tot = 0;
  while (n > 1) {
    int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    tot += 2 * (size_t)tiles;
    n = tiles;
  }
  return tot + 4;
}
}  // namespace

void scan_exclusive_int(const int* in, int* out, int n, int* d_total, cudaStream_t s, DBuf<int>& tmp) {
  tmp.ensure(scan_scratch<int>(n) + 8);
  scan_rec<int>(in, out, n, s, tmp.p, tmp.cap, d_total);
  if (d_total && n <= 0) CK(cudaMemsetAsync(d_total, 0, sizeof(int), s));
}

void scan_exclusive_ll(const long long* in, long long* out, int n, long long* d_total, cudaStream_t s,
                       DBuf<long long>& tmp) {
  tmp.ensure(scan_scratch<long long>(n) + 8);
  scan_rec<long long>(in, out, n, s, tmp.p, tmp.cap, d_total);
  if (d_total && n <= 0) CK(cudaMemsetAsync(d_total, 0, sizeof(long long), s));
}

}  // namespace abd
