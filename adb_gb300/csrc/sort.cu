// Deterministic in-place sort of 64-bit keys (bitonic network): tiles of 2048 keys are
// sorted and merged in shared memory, merge steps wider than a tile run as global
// compare-exchange passes. Used by the spatial-hash broad phase to order bucket entries
// and pair keys; the result depends only on the keys.
#include "abd_engine.h"

namespace abd {

namespace {

constexpr int BT = 1024;          // threads per block
constexpr int BTILE = 2 * BT;     // keys per shared-memory tile

__device__ __forceinline__ void cmp_swap(unsigned long long& a, unsigned long long& b, bool up) {
  if ((a > b) == up) {
    unsigned long long t = a;
    a = b;
    b = t;
  }
}

// Full sort of each tile (sizes 2 .. BTILE) with the direction of global element index.
__global__ void __launch_bounds__(BT) k_bitonic_tile(unsigned long long* a) {
  __shared__ unsigned long long s[BTILE];
  const size_t base = (size_t)blockIdx.x * BTILE;
  s[threadIdx.x] = a[base + threadIdx.x];
  s[threadIdx.x + BT] = a[base + threadIdx.x + BT];
  __syncthreads();
  for (int k = 2; k <= BTILE; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      int i = 2 * threadIdx.x - (threadIdx.x & (j - 1));
      size_t gi = base + i;
      cmp_swap(s[i], s[i + j], (gi & (size_t)k) == 0);
      __syncthreads();
    }
  a[base + threadIdx.x] = s[threadIdx.x];
  a[base + threadIdx.x + BT] = s[threadIdx.x + BT];
}

// Merge steps j = BTILE/2 .. 1 of stage k (k > BTILE) inside each tile.
__global__ void __launch_bounds__(BT) k_bitonic_tile_merge(unsigned long long* a, size_t k) {
  __shared__ unsigned long long s[BTILE];
  const size_t base = (size_t)blockIdx.x * BTILE;
  s[threadIdx.x] = a[base + threadIdx.x];
  s[threadIdx.x + BT] = a[base + threadIdx.x + BT];
  __syncthreads();
  const bool up = ((base & k) == 0);  // a tile never straddles a k-block boundary
  for (int j = BTILE >> 1; j > 0; j >>= 1) {
    int i = 2 * threadIdx.x - (threadIdx.x & (j - 1));
    cmp_swap(s[i], s[i + j], up);
    __syncthreads();
  }
  a[base + threadIdx.x] = s[threadIdx.x];
  a[base + threadIdx.x + BT] = s[threadIdx.x + BT];
}

// One global compare-exchange step (partner distance j >= BTILE) of stage k.
__global__ void k_bitonic_global(unsigned long long* a, size_t n2, size_t j, size_t k) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n2 / 2) return;
  size_t i = 2 * t - (t & (j - 1));
  size_t l = i + j;
  unsigned long long x = a[i], y = a[l];
  bool up = (i & k) == 0;
  if ((x > y) == up) {
    a[i] = y;
    a[l] = x;
  }
}

__global__ void k_pad_keys(unsigned long long* a, size_t n, size_t n2) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x + n;
  if (i < n2) a[i] = ~0ull;
}

}  // namespace

size_t sort_padded_size(size_t n) {
  size_t n2 = BTILE;
  while (n2 < n) n2 <<= 1;
  return n2;
}

void sort_u64(unsigned long long* a, size_t n, size_t cap, cudaStream_t s) {
  if (n <= 1) return;
  size_t n2 = sort_padded_size(n);
  if (cap < n2) throw CudaError{cudaErrorInvalidValue, "sort_u64: buffer smaller than the padded size"};
  if (n2 > n) KLAUNCH(K_SORT, s, k_pad_keys<<<(unsigned)((n2 - n + 255) / 256), 256, 0, s>>>(a, n, n2));
  unsigned tiles = (unsigned)(n2 / BTILE);
  KLAUNCH(K_SORT, s, k_bitonic_tile<<<tiles, BT, 0, s>>>(a));
  for (size_t k = 2 * BTILE; k <= n2; k <<= 1) {
    for (size_t j = k >> 1; j >= (size_t)BTILE; j >>= 1)
      KLAUNCH(K_SORT, s, k_bitonic_global<<<(unsigned)((n2 / 2 + 255) / 256), 256, 0, s>>>(a, n2, j, k));
    KLAUNCH(K_SORT, s, k_bitonic_tile_merge<<<tiles, BT, 0, s>>>(a, k));
  }
}

}  // namespace abd
