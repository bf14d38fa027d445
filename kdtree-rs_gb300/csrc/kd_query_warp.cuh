// kd_query_warp.cuh -- exact k-NN with one warp per query (eps = 0, k <= 64,
// L1 / L2 / L-inf, compile-time widths 2, 3, 8, 16).  Included by
// kd_query_packet.cu.
//
// Where a query scans thousands of leaf rows (clustered data in 8 or 16
// dimensions: the reference's own descent reads 3.8k rows per query at d = 8
// and 14.5k at d = 16 on a 64-cluster mixture), the packet traversal's warp
// walks the union of 32 queries' leaves.  Here the 32 lanes work on ONE query:
// every leaf's rows are split across the lanes (row r + lane), every box's
// dimensions too (lane i takes dimension i), and the k best (exact FP64 reduced
// distance bits, original index) live one or two per lane, sorted, lane j
// holding the j-th (and the (32 + j)-th).  The traversal is best-first at each
// node (the child with the smaller box bound first) and prunes a subtree whose
// rigorous FP32 lower bound exceeds the FP32 upper enclosure of the exact bound
// min(k-th best, cutoff).
//
// Candidate points pass the same rigorous FP32 filter as the packet traversal
// (PointFilter), get their exact FP64 distance in the reference's summation
// order, and enter the list by (distance, index) -- BestK's order
// (query.rs:461-481).  The result is therefore the k smallest (exact distance,
// index) among the points within max_distance, as for the packet traversal.
#pragma once

constexpr int WARP_STACK = 2 * KD_MAX_DEPTH;
constexpr uint32_t FULL_MASK = 0xffffffffu;
constexpr uint64_t EMPTY_KEY = ~0ull;

template <int D>
struct Log2Ceil {
  static constexpr int value = D <= 1 ? 0 : 1 + Log2Ceil<(D + 1) / 2>::value;
};
template <>
struct Log2Ceil<1> {
  static constexpr int value = 0;
};

// Lower bound of the exact box distance: lane i < D takes dimension i; the
// terms are combined with downward-rounded folds (any order gives a lower
// bound) and the result broadcast from lane 0.
template <int M, int D>
__device__ __forceinline__ float warp_box_lb(const float* b32, float my_qlo, float my_qhi, uint32_t lane) {
  float o = 0.f;
  if (lane < static_cast<uint32_t>(D)) {
    o = fmaxf(__fsub_rd(b32[lane], my_qhi), __fsub_rd(my_qlo, b32[D + lane]));
    o = o > 0.f ? o : 0.f;
    o = red_lb<M>(o);
  }
#pragma unroll
  for (int s = Log2Ceil<D>::value - 1; s >= 0; --s) o = fold_lb<M>(o, __shfl_xor_sync(FULL_MASK, o, 1 << s));
  o = __shfl_sync(FULL_MASK, o, 0);
  return __fmul_rd(o, LB_SHRINK);
}

__device__ __forceinline__ uint64_t shfl_u64(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(FULL_MASK, static_cast<uint32_t>(v), src);
  const uint32_t hi = __shfl_sync(FULL_MASK, static_cast<uint32_t>(v >> 32), src);
  return (static_cast<uint64_t>(hi) << 32) | lo;
}
__device__ __forceinline__ uint64_t shfl_up_u64(uint64_t v) {
  const uint32_t lo = __shfl_up_sync(FULL_MASK, static_cast<uint32_t>(v), 1);
  const uint32_t hi = __shfl_up_sync(FULL_MASK, static_cast<uint32_t>(v >> 32), 1);
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

// The warp's sorted k best, KS slots per lane (k <= 32 KS): rank r lives in
// lane r % 32, slot r / 32 (key = exact distance bits, id = original index);
// EMPTY_KEY sorts after everything.
template <int KS>
struct WarpList {
  uint64_t key[KS];
  uint32_t id[KS];
  uint32_t k;
  uint32_t lane;
  uint64_t cut_bits;
  uint64_t bound_bits;  // min(k-th key, cutoff)
  float bound32;        // an FP32 upper enclosure of it

  __device__ __forceinline__ void init(uint32_t k_, double cutoff, uint32_t lane_) {
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      key[s] = EMPTY_KEY;
      id[s] = NO_ID;
    }
    k = k_;
    lane = lane_;
    cut_bits = dbits(cutoff);
    refresh();
  }
  __device__ __forceinline__ void refresh() {
    const uint32_t r = k - 1;
    uint64_t kth = shfl_u64(key[0], static_cast<int>(r & 31));
    if (KS > 1) {
      const uint64_t k1 = shfl_u64(key[KS - 1], static_cast<int>(r & 31));
      if (r >= 32) kth = k1;
    }
    bound_bits = kth < cut_bits ? kth : cut_bits;
    bound32 = mag_up32(bound_bits);
  }
  // Insert candidate (cb, cid) if it is among the k smallest; warp-uniform.
  __device__ __forceinline__ void insert(uint64_t cb, uint32_t cid) {
    uint32_t pos = 0;
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const uint32_t r = lane + 32u * s;
      const bool before = r < k && (key[s] < cb || (key[s] == cb && id[s] < cid));
      pos += __popc(__ballot_sync(FULL_MASK, before));
    }
    if (pos >= k) return;  // uniform
    // ranks above pos move up by one: from the lane below, or (lane 0 of
    // slot 1) from lane 31 of slot 0
    uint64_t up_key[KS];
    uint32_t up_id[KS];
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      up_key[s] = shfl_up_u64(key[s]);
      up_id[s] = __shfl_up_sync(FULL_MASK, id[s], 1);
    }
    if (KS > 1) {
      const uint64_t wrap_key = shfl_u64(key[0], 31);
      const uint32_t wrap_id = __shfl_sync(FULL_MASK, id[0], 31);
      if (lane == 0) {
        up_key[KS - 1] = wrap_key;
        up_id[KS - 1] = wrap_id;
      }
    }
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const uint32_t r = lane + 32u * s;
      if (r > pos && r < k) {
        key[s] = up_key[s];
        id[s] = up_id[s];
      } else if (r == pos) {
        key[s] = cb;
        id[s] = cid;
      }
    }
  }
};

template <int M, int D, int KS>
__device__ __forceinline__ void warp_query(const QArgs& a, uint64_t w, uint32_t* stack_n, float* stack_lb) {
  static_assert(D > 0 && M != M_LP, "warp path: compile-time width, metric without pow()");
  const uint32_t lane = threadIdx.x & 31;
  if (w >= a.nq) return;  // uniform per warp
  const uint64_t qi = a.order ? a.order[w] : w;
  QVec<D> q;
  q.g = a.queries + qi * D;
  bool live = true;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    q.v[i] = q.g[i];
    live &= isfinite(q.v[i]);
  }
  if (!live) {  // uniform: every lane read the same query
    if (lane == 0) atomicOr(a.status, 1u);
    return;
  }
  PointFilter<M, D> filt;
  filt.init(q, a.coord_max);
  float my_qlo = 0.f, my_qhi = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i)
    if (lane == static_cast<uint32_t>(i)) rn_enclose(filt.q32[i], &my_qlo, &my_qhi);

  WarpList<KS> best;
  best.init(static_cast<uint32_t>(a.k), a.cutoff, lane);
  float thr = filt.threshold(best.bound32);

  int sp = 0;
  uint32_t node = 0;
  bool have = true;
  while (have) {
    // descend: the child with the smaller bound first, the other one stacked
    DNode nd = a.nodes[node];
    while (!(nd.meta & KD_NODE_LEAF)) {
      const uint32_t l = node + 1, r = nd.right;
      const float lb_l = warp_box_lb<M, D>(a.boxes32 + static_cast<uint64_t>(l) * 2 * D, my_qlo, my_qhi, lane);
      const float lb_r = warp_box_lb<M, D>(a.boxes32 + static_cast<uint64_t>(r) * 2 * D, my_qlo, my_qhi, lane);
      const bool left_first = lb_l <= lb_r;
      const uint32_t nn = left_first ? l : r, fn = left_first ? r : l;
      const float lb_n = left_first ? lb_l : lb_r, lb_f = left_first ? lb_r : lb_l;
      if (!(lb_f > best.bound32)) {
        stack_n[sp] = fn;
        stack_lb[sp] = lb_f;
        ++sp;
      }
      if (lb_n > best.bound32) {
        nd.meta = 0;  // nothing below the near child either: go pop
        break;
      }
      node = nn;
      nd = a.nodes[node];
    }
    if (nd.meta & KD_NODE_LEAF) {
      const uint64_t se = dbits(nd.split);
      const uint32_t start = static_cast<uint32_t>(se), end = static_cast<uint32_t>(se >> 32);
      const uint32_t chunk_end = (D == 8 && M != M_LINF) ? start + (end - start) / 8 * 8 : end;
      for (uint32_t c0 = start; c0 < end; c0 += 32) {
        const uint32_t r = c0 + lane;
        bool cand = false;
        if (r < end) {
          const float s = filt.sum(a.data32 + static_cast<uint64_t>(r) * D);
          cand = !(s > thr);
        }
        uint64_t xb = EMPTY_KEY;
        uint32_t xid = NO_ID;
        if (cand) {
          xb = dbits(exact_dist<M, D>(q, a.data + static_cast<uint64_t>(r) * D, D, S_PACKED, r < chunk_end, 0.0));
          xid = a.indices[r];
          cand = xb <= best.bound_bits;
        }
        uint32_t mask = __ballot_sync(FULL_MASK, cand);
        if (!mask) continue;
        while (mask) {
          const int c = __ffs(mask) - 1;
          mask &= mask - 1;
          const uint64_t cb = shfl_u64(xb, c);
          const uint32_t cid = __shfl_sync(FULL_MASK, xid, c);
          if (cb <= best.bound_bits) best.insert(cb, cid);
          best.refresh();
        }
        thr = filt.threshold(best.bound32);
      }
    }
    // next: the most recently stacked subtree that can still hold a result
    have = false;
    while (sp > 0) {
      --sp;
      if (!(stack_lb[sp] > best.bound32)) {
        node = stack_n[sp];
        have = true;
        break;
      }
    }
  }
#pragma unroll
  for (int s = 0; s < KS; ++s) {
    const uint32_t r = lane + 32u * s;
    if (r < a.k) {
      const bool real = best.key[s] != EMPTY_KEY;
      a.out_d[qi * a.k + r] = real ? restore<M>(bitsd(best.key[s]), 0.0) : bitsd(INF_BITS);
      a.out_i[qi * a.k + r] = real ? static_cast<int64_t>(best.id[s]) : static_cast<int64_t>(a.n_points);
    }
  }
}

// One warp per query; the block's warps keep their stacks in shared memory
// (every lane writes the same entry and reads back what it wrote).
template <int M, int D, int KS>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_warp(QArgs a) {
  __shared__ uint32_t s_node[QUERY_THREADS / 32][WARP_STACK];
  __shared__ float s_lb[QUERY_THREADS / 32][WARP_STACK];
  const uint32_t wid = threadIdx.x >> 5;
  warp_query<M, D, KS>(a, blockIdx.x * static_cast<uint64_t>(QUERY_THREADS / 32) + wid, s_node[wid], s_lb[wid]);
}
