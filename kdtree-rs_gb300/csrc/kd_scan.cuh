// kd_scan.cuh -- exclusive prefix sum of a u32 array on the device (per-tile
// block scans, a scan of the tile sums, a fix-up pass): the counting sorts that
// order query batches by landing leaf.  Included inside namespace
// kd { namespace { ... } } by each translation unit that sorts queries.
#pragma once

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ uint32_t block_scan_excl(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  const uint32_t off = warp ? warp_sums[warp - 1] : 0;
  *total = warp_sums[SCAN_THREADS / 32 - 1];
  __syncthreads();
  return off + x - v;
}

// Exclusive scan of a[0, n) in place: per-tile scan, tile sums, offsets.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(uint32_t* a, uint64_t n, uint32_t* tile_sums) {
  const uint64_t base = blockIdx.x * static_cast<uint64_t>(SCAN_TILE) + threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    v[j] = (base + j < n) ? a[base + j] : 0;
    s += v[j];
  }
  uint32_t total;
  uint32_t run = block_scan_excl(s, &total);
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    if (base + j < n) a[base + j] = run;
    run += v[j];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(uint32_t* sums, uint64_t n_tiles) {
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint64_t b = 0; b < n_tiles; b += SCAN_THREADS) {
    uint64_t i = b + threadIdx.x;
    uint32_t v = i < n_tiles ? sums[i] : 0, total;
    uint32_t ex = block_scan_excl(v, &total);
    const uint32_t c = carry;
    if (i < n_tiles) sums[i] = c + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry = c + total;
    __syncthreads();
  }
}

__global__ void k_scan_add(uint32_t* a, uint64_t n, const uint32_t* tile_sums) {
  const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i < n) a[i] += tile_sums[i / SCAN_TILE];
}
