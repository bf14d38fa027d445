// kd_common.cuh -- device data layout and exact FP64 helpers shared by the
// build and query kernels of the GB300 kd-tree engine.
//
// Every FP64 operation whose result must equal the reference's goes through an
// explicit round-to-nearest intrinsic (__dadd_rn / __dsub_rn / __dmul_rn): those
// are never contracted into FMAs, matching rustc, which never contracts.  The
// translation units are additionally compiled with -fmad=false.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/kdtree_gb300.h"

namespace kd {

// ---------------------------------------------------------------------------
// Device tree layout (HBM).
//
// Node: 16 bytes, preorder, left child = id + 1 (src/tree.rs:1-4, 11-27).
//   inner: split = split_value, right = right child id,
//          meta = split_dim | KD_NODE_BOX_ORDER (order_by_box flag)
//   leaf:  split bits = start | (uint64_t)end << 32, meta = KD_NODE_LEAF
// ---------------------------------------------------------------------------
constexpr uint32_t KD_NODE_LEAF = 0x80000000u;
constexpr uint32_t KD_NODE_BOX_ORDER = 0x40000000u;
constexpr uint32_t KD_NODE_DIM_MASK = 0x3fffffffu;

struct __align__(16) DNode {
  double split;
  uint32_t right;
  uint32_t meta;
};
static_assert(sizeof(DNode) == 16, "node must stay 16 bytes");

// Largest depth a preorder tree with u32 node ids can reach, plus one.
constexpr int KD_MAX_DEPTH = 34;

// Metric kinds (src/metric.rs:37-42) and scan strategies (src/kernel.rs:244-270).
enum MetricKind : int { M_L1 = 0, M_L2 = 1, M_LINF = 2, M_LP = 3 };
enum Strategy : int { S_PACKED = 0, S_FOLDED = 1, S_STREAMED = 2 };

constexpr int LANES = 8;  // src/simd.rs:6

// f64::total_cmp as an unsigned key (finite values; -0 < +0).
__host__ __device__ __forceinline__ uint64_t total_key_bits(uint64_t b) {
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ uint64_t from_total_key_bits(uint64_t k) {
  return (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
}
__device__ __forceinline__ uint64_t total_key(double v) {
  return total_key_bits(static_cast<uint64_t>(__double_as_longlong(v)));
}
__device__ __forceinline__ double from_total_key(uint64_t k) {
  return __longlong_as_double(static_cast<long long>(from_total_key_bits(k)));
}

// Exact FP64 primitives (never contracted).
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Non-negative doubles (and +inf) order like their bit patterns; every reduced
// distance, bound and cutoff the query compares is normalised to that domain.
__device__ __forceinline__ uint64_t dbits(double v) {
  return static_cast<uint64_t>(__double_as_longlong(v));
}
__device__ __forceinline__ double bitsd(uint64_t b) {
  return __longlong_as_double(static_cast<long long>(b));
}

}  // namespace kd
