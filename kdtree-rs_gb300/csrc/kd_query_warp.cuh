// kd_query_warp.cuh -- exact k-NN with one warp per query (eps = 0, k <= 64,
// L1 / L2 / L-inf, compile-time widths 2, 3, 8, 16).  Included by
// kd_query_packet.cu.
//
// Where a query scans thousands of leaf rows (clustered data in 8 or 16
// dimensions: the reference's own descent reads 3.8k rows per query at d = 8
// and 14.5k at d = 16 on a 64-cluster mixture), the packet traversal's warp
// walks the union of 32 queries' leaves.  Here the 32 lanes work on ONE query:
// every leaf's rows are split across the lanes (row r + lane), a node's two
// children's boxes across the two half-warps (lane i of a half takes dimension
// i), and the k best (FP32 enclosures of the exact FP64 reduced distances, tree
// row, original index) live one or two per lane, sorted, lane j holding the
// j-th (and the (32 + j)-th).  The traversal is best-first at each node (the
// child with the smaller box bound first) and prunes a subtree whose rigorous
// FP32 lower bound exceeds the FP32 upper enclosure of the exact bound
// min(k-th best, cutoff).
//
// Candidate points pass the same rigorous FP32 filter as the packet traversal
// (PointFilter) and enter the list by their exact (distance, index) order --
// BestK's (query.rs:461-481) -- decided on FP32 enclosures of the exact FP64
// distance in the reference's summation order, with the exact value computed
// only when enclosures overlap (GB300 runs FP64 at 1/58 of the FP32 rate).
// The result is therefore the k smallest (exact distance, index) among the
// points within max_distance, as for the packet traversal.
#pragma once

constexpr int WARP_STACK = 2 * KD_MAX_DEPTH;
constexpr uint32_t FULL_MASK = 0xffffffffu;

template <int D>
struct Log2Ceil {
  static constexpr int value = D <= 1 ? 0 : 1 + Log2Ceil<(D + 1) / 2>::value;
};
template <>
struct Log2Ceil<1> {
  static constexpr int value = 0;
};

// Lower bounds of the exact box distances of a node's two children, both at
// once: lanes 0-15 take box bl, lanes 16-31 box br, lane i of a half
// dimension i (my_qlo / my_qhi: the query's enclosure in dimension lane % 16).
// Each term is rounded down and the terms are combined with downward-rounded
// folds (any order gives a lower bound), which stay inside each half (D <= 16).
template <int M, int D>
__device__ __forceinline__ void warp_box_lb2(const float* bl, const float* br, float my_qlo, float my_qhi,
                                             uint32_t lane, float* lb_l, float* lb_r) {
  static_assert(D <= 16, "one 16-lane half per box");
  const uint32_t i = lane & 15;
  const float* b = lane < 16 ? bl : br;
  float o = 0.f;
  if (i < static_cast<uint32_t>(D)) {
    o = fmaxf(__fsub_rd(b[i], my_qhi), __fsub_rd(my_qlo, b[D + i]));
    o = o > 0.f ? o : 0.f;
    o = red_lb<M>(o);
  }
#pragma unroll
  for (int s = Log2Ceil<D>::value - 1; s >= 0; --s) o = fold_lb<M>(o, __shfl_xor_sync(FULL_MASK, o, 1 << s));
  *lb_l = __fmul_rd(__shfl_sync(FULL_MASK, o, 0), LB_SHRINK);
  *lb_r = __fmul_rd(__shfl_sync(FULL_MASK, o, 16), LB_SHRINK);
}

// The warp's sorted k best, KS slots per lane (k <= 32 KS): rank r lives in
// lane r % 32, slot r / 32.  Like the packet traversal's heap, an entry keeps
// an FP32 enclosure [lo, hi] of its exact FP64 distance (a one-point enclosure
// once that is known), its tree row and original index; entries are in exact
// (distance, index) order.  A candidate's rank comes from enclosure
// comparisons; only entries whose enclosure overlaps the candidate's compute
// exact values (one lane each, in parallel), and the candidate's own exact
// value is computed then too.  Empty slots: row ROW_NONE, after everything.
template <int M, int D, int KS>
struct WarpLazyList {
  float lo[KS], hi[KS];
  uint32_t row[KS], id[KS];
  bool chunk[KS];  // the point lies in a full Packed d8 chunk (kernel.rs:540-562)
  uint32_t k, lane;
  uint64_t cut_bits;
  float cut_lo, cut_hi;
  float bound32;  // FP32 upper bound of min(k-th best, cutoff)
  QMem<D> q;
  const double* data;

  __device__ __forceinline__ double exact_of(uint32_t r, bool in_chunk) const {
    return exact_dist<M, D>(q, data + static_cast<uint64_t>(r) * D, D, S_PACKED, in_chunk, 0.0);
  }
  __device__ __forceinline__ void init(uint32_t k_, double cutoff, uint32_t lane_, const double* qg,
                                       const double* data_) {
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      lo[s] = hi[s] = __int_as_float(0x7f800000);
      row[s] = ROW_NONE;
      id[s] = NO_ID;
      chunk[s] = false;
    }
    k = k_;
    lane = lane_;
    cut_bits = dbits(cutoff);
    cut_lo = mag_dn32(cut_bits);
    cut_hi = mag_up32(cut_bits);
    q.g = qg;
    data = data_;
    refresh();
  }
  __device__ __forceinline__ void refresh() {
    const uint32_t r = k - 1;
    float kth = __shfl_sync(FULL_MASK, hi[0], static_cast<int>(r & 31));
    if (KS > 1) {
      const float k1 = __shfl_sync(FULL_MASK, hi[KS - 1], static_cast<int>(r & 31));
      if (r >= 32) kth = k1;
    }
    bound32 = fminf(kth, cut_hi);
  }
  // Offer the candidate at tree row cr (original index cid) whose exact
  // distance lies in [cl, ch]; warp-uniform arguments.
  __device__ __forceinline__ void offer(float cl, float ch, uint32_t cr, uint32_t cid, bool cchunk) {
    if (cl > bound32) return;
    uint64_t cx_bits = 0;
    bool have_x = false;
    if (!(ch <= cut_lo)) {  // the cutoff test, unless clearly inside
      if (cl > cut_hi) return;
      cx_bits = dbits(exact_of(cr, cchunk));
      have_x = true;
      if (cx_bits > cut_bits) return;
    }
    bool before[KS], amb[KS];
    bool any_amb = false;
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const uint32_t r = lane + 32u * s;
      const bool valid = r < k && row[s] != ROW_NONE;
      before[s] = valid && hi[s] < cl;
      amb[s] = valid && !before[s] && !(lo[s] > ch);
      any_amb |= amb[s];
    }
    if (__any_sync(FULL_MASK, any_amb)) {  // too close to call on enclosures
      if (!have_x) cx_bits = dbits(exact_of(cr, cchunk));
#pragma unroll
      for (int s = 0; s < KS; ++s) {
        if (amb[s]) {
          const uint64_t xb = dbits(exact_of(row[s], chunk[s]));
          lo[s] = mag_dn32(xb);
          hi[s] = mag_up32(xb);
          before[s] = xb < cx_bits || (xb == cx_bits && id[s] < cid);
        }
      }
      cl = mag_dn32(cx_bits);
      ch = mag_up32(cx_bits);
    }
    uint32_t pos = 0;
#pragma unroll
    for (int s = 0; s < KS; ++s) pos += __popc(__ballot_sync(FULL_MASK, before[s]));
    if (pos >= k) {
      refresh();  // enclosures may have tightened
      return;
    }
    float up_lo[KS], up_hi[KS];
    uint32_t up_row[KS], up_id[KS];
    bool up_chunk[KS];
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      up_lo[s] = __shfl_up_sync(FULL_MASK, lo[s], 1);
      up_hi[s] = __shfl_up_sync(FULL_MASK, hi[s], 1);
      up_row[s] = __shfl_up_sync(FULL_MASK, row[s], 1);
      up_id[s] = __shfl_up_sync(FULL_MASK, id[s], 1);
      up_chunk[s] = __shfl_up_sync(FULL_MASK, static_cast<int>(chunk[s]), 1);
    }
    if (KS > 1) {
      const float wl = __shfl_sync(FULL_MASK, lo[0], 31), wh = __shfl_sync(FULL_MASK, hi[0], 31);
      const uint32_t wr = __shfl_sync(FULL_MASK, row[0], 31), wi = __shfl_sync(FULL_MASK, id[0], 31);
      const bool wc = __shfl_sync(FULL_MASK, static_cast<int>(chunk[0]), 31);
      if (lane == 0) {
        up_lo[KS - 1] = wl;
        up_hi[KS - 1] = wh;
        up_row[KS - 1] = wr;
        up_id[KS - 1] = wi;
        up_chunk[KS - 1] = wc;
      }
    }
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const uint32_t r = lane + 32u * s;
      if (r > pos && r < k) {
        lo[s] = up_lo[s];
        hi[s] = up_hi[s];
        row[s] = up_row[s];
        id[s] = up_id[s];
        chunk[s] = up_chunk[s];
      } else if (r == pos) {
        lo[s] = cl;
        hi[s] = ch;
        row[s] = cr;
        id[s] = cid;
        chunk[s] = cchunk;
      }
    }
    refresh();
  }
  // write_results (query.rs:421-429, 483-493): lane j writes rank j (and
  // 32 + j); the entries are in exact order already, their exact values are
  // computed once here.
  __device__ __forceinline__ void write(double* od, int64_t* oi, uint64_t n_points) const {
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const uint32_t r = lane + 32u * s;
      if (r < k) {
        const bool real = row[s] != ROW_NONE;
        od[r] = real ? restore<M>(exact_of(row[s], chunk[s]), 0.0) : bitsd(INF_BITS);
        oi[r] = real ? static_cast<int64_t>(id[s]) : static_cast<int64_t>(n_points);
      }
    }
  }
};

// A warp's traversal stack in shared memory: subtree id, the lower bound of
// its box distance and its node record (read with its box when its parent was
// expanded, so a pop costs no global load).  Every lane writes the same entry
// and reads back what it wrote.
struct WarpStack {
  uint32_t node[WARP_STACK];
  float lb[WARP_STACK];
  DNode nd[WARP_STACK];
};

template <int M, int D, int KS>
__device__ __forceinline__ void warp_query(const QArgs& a, uint64_t w, WarpStack* stack) {
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
  // Every lane holds the same query.  Taking the FP32 copies out of shuffles
  // pins them in registers: left as conversions of the FP64 query, they were
  // recomputed inside the row loop, one FP64-pipe conversion per dimension
  // and row (the FP64 pipe issues one warp instruction per 16 cycles).
#pragma unroll
  for (int i = 0; i < D; ++i) filt.q32[i] = __shfl_sync(FULL_MASK, filt.q32[i], 0);
  float my_qlo = 0.f, my_qhi = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i)
    if ((lane & 15) == static_cast<uint32_t>(i)) rn_enclose(filt.q32[i], &my_qlo, &my_qhi);

  WarpLazyList<M, D, KS> best;
  best.init(static_cast<uint32_t>(a.k), a.cutoff, lane, q.g, a.data);
  float thr = filt.threshold(best.bound32);

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
      warp_box_lb2<M, D>(a.boxes32 + static_cast<uint64_t>(l) * 2 * D, a.boxes32 + static_cast<uint64_t>(r) * 2 * D,
                         my_qlo, my_qhi, lane, &lb_l, &lb_r);
      const bool left_first = lb_l <= lb_r;
      const float lb_n = left_first ? lb_l : lb_r, lb_f = left_first ? lb_r : lb_l;
      if (!(lb_f > best.bound32)) {
        stack->node[sp] = left_first ? r : l;
        stack->lb[sp] = lb_f;
        stack->nd[sp] = left_first ? nd_r : nd_l;
        ++sp;
      }
      if (lb_n > best.bound32) {
        nd.meta = 0;  // nothing below the near child either: go pop
        break;
      }
      node = left_first ? l : r;
      nd = left_first ? nd_l : nd_r;
    }
    if (nd.meta & KD_NODE_LEAF) {
      const uint64_t se = dbits(nd.split);
      const uint32_t start = static_cast<uint32_t>(se), end = static_cast<uint32_t>(se >> 32);
      const uint32_t chunk_end = (D == 8 && M != M_LINF) ? start + (end - start) / 8 * 8 : end;
      for (uint32_t c0 = start; c0 < end; c0 += 32) {
        // lanes past the leaf's end re-read its last row and drop it: no
        // divergent branch around the row sum
        const uint32_t r = c0 + lane;
        const float s = filt.sum(a.data32 + static_cast<uint64_t>(min(r, end - 1)) * D);
        float clo, chi;
        filt.enclose(s, &clo, &chi);
        const bool cand = r < end && !(s > thr) && !(clo > best.bound32);
        uint32_t mask = __ballot_sync(FULL_MASK, cand);
        if (!mask) continue;
        const uint32_t my_id = cand ? a.indices[r] : NO_ID;
        while (mask) {
          const int c = __ffs(mask) - 1;
          mask &= mask - 1;
          const float cl = __shfl_sync(FULL_MASK, clo, c), ch = __shfl_sync(FULL_MASK, chi, c);
          const uint32_t cid = __shfl_sync(FULL_MASK, my_id, c);
          const uint32_t cr = c0 + static_cast<uint32_t>(c);
          best.offer(cl, ch, cr, cid, cr < chunk_end);
        }
        thr = filt.threshold(best.bound32);
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
    }
  }
  best.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.n_points);
}

// One warp per query; the block's warps keep their stacks in shared memory.
template <int M, int D, int KS>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_warp(QArgs a) {
  __shared__ WarpStack s_stack[QUERY_THREADS / 32];
  const uint32_t wid = threadIdx.x >> 5;
  warp_query<M, D, KS>(a, blockIdx.x * static_cast<uint64_t>(QUERY_THREADS / 32) + wid, &s_stack[wid]);
}
