// kd_query_warp.cuh -- exact k-NN with one warp per query, best-first
// (eps = 0, k <= 64, L1 / L2 / L-inf, widths 1..128).  Included after
// kd_warp.cuh.
//
// Where a query scans thousands of leaf rows (clustered data in 8 or 16
// dimensions: the reference's own descent reads 3.8k rows per query at d = 8
// and 14.5k at d = 16 on a 64-cluster mixture; wide data, where the planes
// hardly prune), the packet traversal's warp walks the union of 32 queries'
// leaves.  Here the 32 lanes work on ONE query: every leaf's rows are split
// across the lanes (row r + lane), a node's two children's boxes across the
// lanes (by dimension), and the k best (WarpList: FP32 enclosures of the exact
// FP64 reduced distances, tree row, original index) live one or two per lane,
// sorted.  The traversal is best-first at each node (the child with the smaller
// box bound first) and prunes a subtree whose rigorous FP32 lower bound exceeds
// the FP32 upper enclosure of the exact bound min(k-th best, cutoff).
//
// Candidate points pass a rigorous FP32 filter (PointFilter / PointFilterDyn)
// and enter the list by their exact (distance, index) order -- BestK's
// (query.rs:461-481) -- decided on FP32 enclosures of the exact FP64 distance
// in the reference's summation order (Packed, Folded or Streamed, kernel.rs),
// with the exact value computed only when enclosures overlap (GB300 runs FP64
// at 1/58 of the FP32 rate).  The result is the k smallest (exact distance,
// index) among the points within max_distance; near ties -- where the
// reference's own descent may leave one of them out -- are flagged for a
// reference-order rerun (kd_warp.cuh).
#pragma once

template <int M, int D, int KS>
__device__ __forceinline__ void warp_query(const QArgs& a, uint64_t w, WarpStack* stack, float* sq_w) {
  static_assert(M != M_LP, "warp path: metrics without pow()");
  const uint32_t lane = threadIdx.x & 31;
  if (w >= a.nq) return;  // uniform per warp
  const uint64_t qi = a.order ? a.order[w] : w;
  const uint32_t d = D > 0 ? static_cast<uint32_t>(D) : static_cast<uint32_t>(a.d);
  const double* qg = a.queries + qi * d;
  typename RowFilterOf<M, D>::type filt;
  float my_qlo = 0.f, my_qhi = 0.f;  // compile-time widths: dimension lane % 16
  LaneQ lq;                          // runtime widths: dimensions lane + 32 j
  if constexpr (D > 0) {
    QVec<D> q;
    q.g = qg;
    bool live = true;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      q.v[i] = qg[i];
      live &= isfinite(q.v[i]);
    }
    if (!live) {  // uniform: every lane read the same query
      if (lane == 0) atomicOr(a.status, 1u);
      return;
    }
    filt.init(q, a.coord_max);
    // Every lane holds the same query.  Taking the FP32 copies out of shuffles
    // pins them in registers: left as conversions of the FP64 query, they were
    // recomputed inside the row loop, one FP64-pipe conversion per dimension
    // and row (the FP64 pipe issues one warp instruction per 16 cycles).
#pragma unroll
    for (int i = 0; i < D; ++i) filt.q32[i] = __shfl_sync(FULL_MASK, filt.q32[i], 0);
#pragma unroll
    for (int i = 0; i < D; ++i)
      if ((lane & 15) == static_cast<uint32_t>(i)) rn_enclose(filt.q32[i], &my_qlo, &my_qhi);
  } else {
    bool fin = true;
    for (uint32_t i = lane; i < d; i += 32) fin &= isfinite(qg[i]);
    if (!__all_sync(FULL_MASK, fin)) {
      if (lane == 0) atomicOr(a.status, 1u);
      return;
    }
    filt.init(qg, d, a.w32, a.coord_max, sq_w, lane);
    lane_query_enclosure(qg, d, lane, &lq);
  }
  const float* rows32 = filter_rows<D>(a);
  const uint64_t rstride = filter_stride<D>(a);
  const uint64_t bstride = 2ull * d;
  // Packed d4 / d8 chunk flags (kernel.rs:517-562): L1 / L2 only
  const uint32_t chunk_w = (M != M_LINF && (d == 4 || d == 8)) ? (d == 4 ? 2u : 8u) : 0u;

  WarpList<M, D, KS> best;
  best.init(static_cast<uint32_t>(a.k), a.cutoff, lane, qg, a.data, d, 0.0);
  float thr = filt.threshold(best.bound32), thr2 = filt.threshold(band_of(best.bound32));

  auto children_lb = [&](uint32_t l, uint32_t r, float* lb_l, float* lb_r) {
    if constexpr (D > 0)
      warp_box_lb2<M, D>(a.boxes32 + l * bstride, a.boxes32 + r * bstride, my_qlo, my_qhi, lane, lb_l, lb_r);
    else
      warp_box_lb2_dyn<M>(a.boxes32 + l * bstride, a.boxes32 + r * bstride, d, lane, lq, lb_l, lb_r);
  };

  int sp = 0;
  uint32_t node = 0;
  DNode nd = a.nodes[0];
  bool have = true;
  while (have) {
    // descend: the child with the smaller bound first, the other one stacked;
    // both children's records load with their boxes (one round trip a level)
    while (!(nd.meta & KD_NODE_LEAF)) {
      const uint32_t l = node + 1, r = nd.right;
      const DNode nd_l = a.nodes[l], nd_r = a.nodes[r];
      float lb_l, lb_r;
      children_lb(l, r, &lb_l, &lb_r);
      const bool left_first = lb_l <= lb_r;
      const float lb_n = left_first ? lb_l : lb_r, lb_f = left_first ? lb_r : lb_l;
      if (!(lb_f > best.bound32)) {
        stack->node[sp] = left_first ? r : l;
        stack->lb[sp] = lb_f;
        stack->nd[sp] = left_first ? nd_r : nd_l;
        ++sp;
      } else {
        best.note(lb_f);
      }
      if (lb_n > best.bound32) {
        best.note(lb_n);
        nd.meta = 0;  // nothing below the near child either: go pop
        break;
      }
      node = left_first ? l : r;
      nd = left_first ? nd_l : nd_r;
    }
    if (nd.meta & KD_NODE_LEAF) {
      const uint64_t se = dbits(nd.split);
      const uint32_t start = static_cast<uint32_t>(se), end = static_cast<uint32_t>(se >> 32);
      const uint32_t chunk_end = chunk_w ? start + (end - start) / chunk_w * chunk_w : end;
      for (uint32_t c0 = start; c0 < end; c0 += 32) {
        // lanes past the leaf's end re-read its last row and drop it: no
        // divergent branch around the row sum
        const uint32_t r = c0 + lane;
        const float s = filt.sum(rows32 + static_cast<uint64_t>(min(r, end - 1)) * rstride);
        // s > thr2 proves the point lies beyond the near-tie band above the
        // bound: neither a candidate nor a note.  Most chunks hold only such
        // rows, and skip the enclosures.
        if (!__any_sync(FULL_MASK, r < end && !(s > thr2))) continue;
        float clo, chi;
        filt.enclose(s, &clo, &chi);
        const bool cand = r < end && !(s > thr) && !(clo > best.bound32);
        // dropped inside the near-tie band: noted by its exact value (rare)
        if (r < end && !cand && !(s > thr2) && !(clo > near_window(best.bound32)))
          best.note(mag_dn32(dbits(best.exact_of(r, r < chunk_end))));
        uint32_t mask = __ballot_sync(FULL_MASK, cand);
        if (!mask) continue;
        const uint32_t my_id = cand ? a.indices[r] : NO_ID;
        // several candidates: ranked together when enclosures decide every
        // comparison
        if constexpr (KS == 1) {
          if (__popc(mask) >= WARP_BULK_MIN &&
              best.offer_all(cand, clo, chi, r, my_id, r < chunk_end, mask, &stack->slots))
            mask = 0;
        }
        while (mask) {
          const int c = __ffs(mask) - 1;
          mask &= mask - 1;
          const float cl = __shfl_sync(FULL_MASK, clo, c), ch = __shfl_sync(FULL_MASK, chi, c);
          const uint32_t cid = __shfl_sync(FULL_MASK, my_id, c);
          const uint32_t cr = c0 + static_cast<uint32_t>(c);
          best.offer(cl, ch, cr, cid, cr < chunk_end);
        }
        thr = filt.threshold(best.bound32);
        thr2 = filt.threshold(band_of(best.bound32));
      }
    }
    // next: the most recently stacked subtree that can still hold a result
    have = false;
    while (sp > 0) {
      --sp;
      if (!(stack->lb[sp] > best.bound32)) {
        node = stack->node[sp];
        nd = stack->nd[sp];
        have = true;
        break;
      }
      best.note(stack->lb[sp]);
    }
  }
  const bool near = best.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.n_points, a.rerun_count != nullptr);
  if (near && lane == 0) flag_rerun(a, qi);
}

// One warp per query; the block's warps keep their stacks (and, for runtime
// widths, their FP32 queries) in shared memory.
template <int M, int D, int KS>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_warp(QArgs a) {
  __shared__ WarpStack s_stack[QUERY_THREADS / 32];
  __shared__ __align__(16) float s_q[D > 0 ? 1 : QUERY_THREADS / 32][D > 0 ? 4 : WARP_MAX_D];
  const uint32_t wid = threadIdx.x >> 5;
  warp_query<M, D, KS>(a, blockIdx.x * static_cast<uint64_t>(QUERY_THREADS / 32) + wid, &s_stack[wid],
                       s_q[D > 0 ? 0 : wid]);
}
