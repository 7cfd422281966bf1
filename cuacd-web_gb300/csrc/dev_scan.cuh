// dev_scan.cuh — device-wide exclusive scan of uint32 or uint4 values, in
// three launches (tile sums, tile starts in one block, the tiles rescanned
// from their starts); out has n + 1 entries, out[n] = the total.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cuacd {
namespace scan {

#define SCAN_FULL 0xffffffffu

__device__ __forceinline__ uint32_t vadd(uint32_t a, uint32_t b) { return a + b; }
__device__ __forceinline__ uint4 vadd(uint4 a, uint4 b) { return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ uint32_t vsub(uint32_t a, uint32_t b) { return a - b; }
__device__ __forceinline__ uint4 vsub(uint4 a, uint4 b) { return make_uint4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <typename T>
__device__ __forceinline__ T vzero();
template <>
__device__ __forceinline__ uint32_t vzero<uint32_t>() { return 0u; }
template <>
__device__ __forceinline__ uint4 vzero<uint4>() { return make_uint4(0, 0, 0, 0); }
__device__ __forceinline__ uint32_t vshfl_up(uint32_t v, int d) { return __shfl_up_sync(SCAN_FULL, v, d); }
__device__ __forceinline__ uint4 vshfl_up(uint4 v, int d) {
  return make_uint4(__shfl_up_sync(SCAN_FULL, v.x, d), __shfl_up_sync(SCAN_FULL, v.y, d),
                    __shfl_up_sync(SCAN_FULL, v.z, d), __shfl_up_sync(SCAN_FULL, v.w, d));
}

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// inclusive scan of one value per thread over the block (blockDim.x a
// multiple of 32, at most 1024); *total = the block's sum
template <typename T>
__device__ T block_inclusive(T v, T* warpSums, T* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int d = 1; d < 32; d <<= 1) {
    T u = vshfl_up(v, d);
    if (lane >= d) v = vadd(v, u);
  }
  if (lane == 31) warpSums[wid] = v;
  __syncthreads();
  if (wid == 0) {
    T s = lane < nw ? warpSums[lane] : vzero<T>();
    for (int d = 1; d < 32; d <<= 1) {
      T u = vshfl_up(s, d);
      if (lane >= d) s = vadd(s, u);
    }
    warpSums[lane] = s;
  }
  __syncthreads();
  if (wid > 0) v = vadd(v, warpSums[wid - 1]);
  *total = warpSums[nw - 1];
  __syncthreads();
  return v;
}

template <typename T>
__global__ void k_scan_tiles(const T* __restrict__ in, uint32_t n, T* __restrict__ tileSums) {
  __shared__ T ws[32];
  const uint32_t base = blockIdx.x * SCAN_TILE;
  T s = vzero<T>();
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const uint32_t i = base + threadIdx.x * SCAN_ITEMS + k;
    if (i < n) s = vadd(s, in[i]);
  }
  T total;
  block_inclusive(s, ws, &total);
  if (threadIdx.x == 0) tileSums[blockIdx.x] = total;
}

// tile sums to exclusive tile starts, in place (one block); total at [nTiles]
template <typename T>
__global__ void k_scan_tile_starts(T* __restrict__ tileSums, uint32_t nTiles) {
  __shared__ T ws[32];
  T carry = vzero<T>();
  for (uint32_t c = 0; c < nTiles; c += blockDim.x) {
    const uint32_t i = c + threadIdx.x;
    const T v = i < nTiles ? tileSums[i] : vzero<T>();
    T total;
    const T inc = block_inclusive(v, ws, &total);
    if (i < nTiles) tileSums[i] = vadd(carry, vsub(inc, v));
    carry = vadd(carry, total);
    __syncthreads();
  }
  if (threadIdx.x == 0) tileSums[nTiles] = carry;
}

template <typename T>
__global__ void k_scan_apply(const T* __restrict__ in, uint32_t n, const T* __restrict__ tileStarts, uint32_t nTiles,
                             T* __restrict__ out) {
  __shared__ T ws[32];
  const uint32_t base = blockIdx.x * SCAN_TILE;
  T loc[SCAN_ITEMS];
  T s = vzero<T>();
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const uint32_t i = base + threadIdx.x * SCAN_ITEMS + k;
    loc[k] = i < n ? in[i] : vzero<T>();
    s = vadd(s, loc[k]);
  }
  T total;
  const T inc = block_inclusive(s, ws, &total);
  T cur = vadd(tileStarts[blockIdx.x], vsub(inc, s));
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const uint32_t i = base + threadIdx.x * SCAN_ITEMS + k;
    if (i < n) out[i] = cur;
    cur = vadd(cur, loc[k]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = tileStarts[nTiles];
}

// tiles needed for n values (tileSums must hold tiles + 1 entries)
inline uint32_t tiles_for(uint32_t n) { return n == 0 ? 1u : (n + SCAN_TILE - 1) / SCAN_TILE; }

// exclusive scan of n values of in into out (n + 1 entries) on stream s
template <typename T>
inline void exclusive(const T* in, uint32_t n, T* out, T* tileSums, cudaStream_t s) {
  const uint32_t nt = tiles_for(n);
  k_scan_tiles<T><<<nt, SCAN_THREADS, 0, s>>>(in, n, tileSums);
  k_scan_tile_starts<T><<<1, 1024, 0, s>>>(tileSums, nt);
  k_scan_apply<T><<<nt, SCAN_THREADS, 0, s>>>(in, n, tileSums, nt, out);
}

}  // namespace scan
}  // namespace cuacd
