// kd_query_ref.cuh -- the reference's own descent with one warp per query
// (any eps, every metric, widths 1..128, k <= 64).  Included after
// kd_warp.cuh.
//
// The warp walks the tree in exactly the reference's order (src/query.rs:
// 223-341): the root only if its seed admits (CellBound::start, query.rs:
// 169-194); at an inner node the near child first with the unchanged cell
// bound, then the far child if the split-plane bound replace_axis(cell,
// axes[dim], reduce(|diff|)) (metric.rs:93-98) and then the far child's box
// distance (kernel.rs:565-616) admit -- `dist * eps_factor <= bound` with the
// bound read after the near child (query.rs:242-244, 275-285); at an
// `order_by_box` node both children's box distances, the smaller first, each
// admitted with the bound of its moment (query.rs:298-327).  Every gate value
// is the reference's FP64 value, computed with its operations in its order, and
// each comparison decides exactly as the reference's does: against FP32
// enclosures of the bound first, against the exact bound when those cannot
// tell.  So the set of scanned leaves -- and the result -- is the reference's,
// eps > 0 included.
//
// The leaf scan is the part spread across the lanes.  Within one leaf the
// reference offers the points in row order, refreshing the bound after each
// accepted offer (kernel.rs:366-385); the list it ends with is the k smallest
// (distance, index) of the list before and the leaf's points within
// max_distance, whatever the order of the offers (a point above the bound of
// its moment has k better ones kept, or lies beyond the cutoff).  Here the
// lanes filter their rows in FP32 and offer the survivors to the warp's list
// (WarpList), which keeps exactly that set, so the list after the leaf -- and
// every later gate -- matches.  For L^p (pow) the lanes compute every row's
// exact FP64 distance.
//
// The kernel serves three callers: queries with eps > 0 or general p (whose
// answers depend on this order), the reference-order path asked for
// explicitly, and the near-tie reruns of the eps = 0 fast paths (count /
// list: the flagged queries, kd_warp.cuh).
#pragma once

struct RefFrame {
  uint32_t node;  // parent node id (F_FAR / F_BOX_*) or split dim (F_RESTORE)
  uint32_t kind;
  double x;       // parent cell_dist, or the saved axis value
  double y;       // the pending child's box distance (F_BOX_*)
};
enum RefFrameKind : uint32_t { RF_FAR = 0, RF_RESTORE = 1, RF_BOX_FAR = 2, RF_BOX_NEAR = 3 };
constexpr int REF_FRAMES = 2 * KD_MAX_DEPTH;

// Shared memory of one warp of the reference-order kernel: its frames, the
// CellBound axes (d doubles, padded to 16 bytes) and the FP32 query (w32
// floats, read as float4: it must start on a 16-byte boundary).
__host__ __device__ constexpr uint64_t ref_axes_offset() { return REF_FRAMES * sizeof(RefFrame); }
__host__ __device__ constexpr uint64_t ref_q32_offset(uint64_t d) { return ref_axes_offset() + (8 * d + 15) / 16 * 16; }
__host__ __device__ constexpr uint64_t ref_warp_smem(uint64_t d, uint64_t w32) {
  return (ref_q32_offset(d) + 4 * w32 + 15) / 16 * 16;
}
static_assert(ref_axes_offset() % 16 == 0, "frames keep the axes 16-byte aligned");

// Lower and upper bounds of one box's exact FP64 distance, compile-time widths
// <= 16 (both half-warps take the same box; lane i of a half dimension i).
template <int M, int D>
__device__ __forceinline__ void warp_box_enc1(const float* b32, float my_qlo, float my_qhi, uint32_t lane,
                                              float* lb_out, float* ub_out) {
  static_assert(D > 0 && D <= 16, "one 16-lane half per box");
  const uint32_t i = lane & 15;
  float lb = 0.f, ub = 0.f;
  if (i < static_cast<uint32_t>(D)) {
    const float lo32 = b32[i], hi32 = b32[D + i];
    const float lo_up = __fadd_ru(lo32, __fmaf_ru(fabsf(lo32), TWO_M23, TINY32));
    const float hi_dn = __fsub_rd(hi32, __fmaf_ru(fabsf(hi32), TWO_M23, TINY32));
    float o_lb = fmaxf(__fsub_rd(lo32, my_qhi), __fsub_rd(my_qlo, hi32));
    o_lb = o_lb > 0.f ? o_lb : 0.f;
    const float o_ub = fmaxf(fmaxf(__fsub_ru(lo_up, my_qlo), __fsub_ru(my_qhi, hi_dn)), 0.f);
    lb = red_lb<M>(o_lb);
    ub = red_ub<M>(o_ub);
  }
#pragma unroll
  for (int s = Log2Ceil<D>::value - 1; s >= 0; --s) {
    lb = fold_lb<M>(lb, __shfl_xor_sync(FULL_MASK, lb, 1 << s));
    ub = fold_ub<M>(ub, __shfl_xor_sync(FULL_MASK, ub, 1 << s));
  }
  // The folds above only span the first 2^ceil(log2 D) lanes of each half;
  // every lane must take the same gate decision, so all take lane 0's sums.
  *lb_out = __fmul_rd(__shfl_sync(FULL_MASK, lb, 0), LB_SHRINK);
  *ub_out = __fmul_ru(__shfl_sync(FULL_MASK, ub, 0), UB_GROW);
}

template <int M, int D, int KS>
__device__ __forceinline__ void ref_query(const QArgs& a, uint64_t qi, RefFrame* fr, double* axes, float* sq_w) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t d = D > 0 ? static_cast<uint32_t>(D) : static_cast<uint32_t>(a.d);
  const double pexp = a.p;
  const double* qg = a.queries + qi * d;
  bool fin = true;
  for (uint32_t i = lane; i < d; i += 32) fin &= isfinite(qg[i]);
  if (!__all_sync(FULL_MASK, fin)) {
    if (lane == 0) atomicOr(a.status, 1u);
    return;
  }
  QVec<D> q;  // FP64 query: registers for compile-time widths (uniform loops only), memory otherwise
  q.g = qg;
  if constexpr (D > 0) {
#pragma unroll
    for (int i = 0; i < D; ++i) q.v[i] = qg[i];
  }
  constexpr bool FILTER = M != M_LP;
  using Filt = std::conditional_t<FILTER, typename RowFilterOf<(FILTER ? M : M_L2), D>::type, int>;
  Filt filt{};
  float my_qlo = 0.f, my_qhi = 0.f;
  LaneQ lq;
  if constexpr (FILTER) {
    if constexpr (D > 0) {
      filt.init(q, a.coord_max);
#pragma unroll
      for (int i = 0; i < D; ++i) filt.q32[i] = __shfl_sync(FULL_MASK, filt.q32[i], 0);
#pragma unroll
      for (int i = 0; i < D; ++i)
        if ((lane & 15) == static_cast<uint32_t>(i)) rn_enclose(filt.q32[i], &my_qlo, &my_qhi);
    } else {
      filt.init(qg, d, a.w32, a.coord_max, sq_w, lane);
      lane_query_enclosure(qg, d, lane, &lq);
    }
  }
  const float* rows32 = filter_rows<D>(a);
  const uint64_t rstride = filter_stride<D>(a);
  const uint64_t bstride = 2ull * d;
  const uint32_t chunk_w = (M != M_LINF && M != M_LP && (d == 4 || d == 8)) ? (d == 4 ? 2u : 8u) : 0u;
  // FP32 enclosure of eps_factor (1 when eps = 0)
  const float ef_lo = mag_dn32(dbits(a.eps_factor)), ef_hi = mag_up32(dbits(a.eps_factor));

  WarpList<M, D, KS> best;
  best.init(static_cast<uint32_t>(a.k), a.cutoff, lane, qg, a.data, d, pexp);
  float thr = 0.f;
  if constexpr (FILTER) thr = filt.threshold(best.bound32);

  // admits_at(dist, bound): dist * eps_factor <= min(k-th best, cutoff)
  // (query.rs:242-244), decided on the bound's enclosure where it can be.
  auto admits = [&](double x) -> bool {
    const double g = a.use_eps ? dmul(x, a.eps_factor) : x;
    const double blo = static_cast<double>(best.bound_lo), bhi = static_cast<double>(best.bound32);
    if (g < blo) return true;
    if (g > bhi) return false;
    return leq_bound(g, best.bound_exact());
  };
  // The far child's box gate: FP32 enclosure first, the exact FP64 box
  // distance when it cannot decide.
  auto box_admits = [&](uint32_t id) -> bool {
    if constexpr (FILTER) {
      float lb, ub;
      if constexpr (D > 0 && D <= 16)
        warp_box_enc1<M, D>(a.boxes32 + id * bstride, my_qlo, my_qhi, lane, &lb, &ub);
      else
        warp_box_enc_dyn<M>(a.boxes32 + id * bstride, d, lane, lq, &lb, &ub);
      const float glb = __fmul_rd(__fmul_rd(lb, ef_lo), LB_SHRINK);
      const float gub = __fmul_ru(__fmul_ru(ub, ef_hi), UB_GROW);
      if (glb > best.bound32) return false;
      if (gub < best.bound_lo) return true;
    }
    return admits(exact_box_dist<M, D>(q, a.boxes + id * bstride, d, pexp));
  };
  auto box_exact = [&](uint32_t id) -> double { return exact_box_dist<M, D>(q, a.boxes + id * bstride, d, pexp); };

  // scan_leaf (query.rs:343-375) with the rows split across the lanes
  auto scan_leaf = [&](uint32_t start, uint32_t end) {
    const uint32_t chunk_end = chunk_w ? start + (end - start) / chunk_w * chunk_w : end;
    for (uint32_t c0 = start; c0 < end; c0 += 32) {
      const uint32_t r = c0 + lane;
      float clo = 0.f, chi = 0.f;
      bool cand;
      if constexpr (FILTER) {
        const float s = filt.sum(rows32 + static_cast<uint64_t>(min(r, end - 1)) * rstride);
        // s > thr proves the point lies beyond the bound: a chunk of such rows
        // skips the enclosures
        if (!__any_sync(FULL_MASK, r < end && !(s > thr))) continue;
        filt.enclose(s, &clo, &chi);
        cand = r < end && !(s > thr) && !(clo > best.bound32);
      } else {
        // L^p: the exact value (pow) of every row
        const uint32_t rr = min(r, end - 1);
        const uint64_t xb = dbits(best.exact_of(rr, false));
        clo = mag_dn32(xb);
        chi = mag_up32(xb);
        cand = r < end && !(clo > best.bound32);
      }
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
      if constexpr (FILTER) thr = filt.threshold(best.bound32);
    }
  };

  // Descent::run (query.rs:223-232): CellBound::start seeds the axes from the
  // root box when the query lies outside it.
  double seed = 0.0;
  const double rb = box_exact(0);
  if (rb != 0.0) {
    for (uint32_t i = lane; i < d; i += 32) axes[i] = reduce<M>(axis_offset(qg[i], a.boxes[i], a.boxes[d + i]), pexp);
    __syncwarp();
    for (uint32_t i = 0; i < d; ++i) seed = (M == M_LINF) ? max_nn(seed, axes[i]) : dadd(seed, axes[i]);
  } else {
    for (uint32_t i = lane; i < d; i += 32) axes[i] = 0.0;
    __syncwarp();
  }
  // Every lane writes the same frames and axis values and reads back its own
  // writes, so the per-warp shared state needs no further synchronisation.
  int sp = 0;
  uint32_t node = 0;
  double cell = seed;
  bool descending = admits(seed);
  for (;;) {
    while (descending) {
      // Descent::descend (query.rs:248-289)
      const DNode nd = a.nodes[node];
      if (nd.meta & KD_NODE_LEAF) {
        const uint64_t se = dbits(nd.split);
        scan_leaf(static_cast<uint32_t>(se), static_cast<uint32_t>(se >> 32));
        descending = false;
        break;
      }
      const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
      const double qd = qg[dim];
      // diff <= 0  <=>  q[dim] <= split (exact for finite doubles)
      const bool left_near = ieee_key(dbits(qd)) <= ieee_key(dbits(nd.split));
      const uint32_t near = left_near ? node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : node + 1;
      if (nd.meta & KD_NODE_BOX_ORDER) {
        // descend_by_box (query.rs:298-327)
        const double near_box = box_exact(near), far_box = box_exact(far);
        if (dbits(near_box) <= dbits(far_box)) {
          fr[sp++] = RefFrame{node, RF_BOX_FAR, cell, far_box};
          if (admits(near_box)) {
            node = near;
            continue;
          }
          descending = false;
          break;
        }
        fr[sp++] = RefFrame{node, RF_BOX_NEAR, cell, near_box};
        if (admits(far_box)) {
          const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), pexp);
          const double old = axes[dim];
          const double far_dist = (M == M_LINF) ? max_nn(cell, far_axis) : dadd(dsub(cell, old), far_axis);
          fr[sp++] = RefFrame{dim, RF_RESTORE, old, 0.0};
          axes[dim] = far_axis;
          node = far;
          cell = far_dist;
          continue;
        }
        descending = false;
        break;
      }
      fr[sp++] = RefFrame{node, RF_FAR, cell, 0.0};
      node = near;  // the near child keeps the parent's cell bound
    }
    // unwind to the next pending far-child decision
    bool resumed = false;
    while (sp > 0 && !resumed) {
      const RefFrame f = fr[--sp];
      if (f.kind == RF_RESTORE) {
        axes[f.node] = f.x;
        continue;
      }
      const DNode nd = a.nodes[f.node];
      const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
      const double qd = qg[dim];
      const bool left_near = ieee_key(dbits(qd)) <= ieee_key(dbits(nd.split));
      const uint32_t near = left_near ? f.node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : f.node + 1;
      if (f.kind == RF_BOX_NEAR) {
        if (admits(f.y)) {
          node = near;
          cell = f.x;
          resumed = true;
        }
        continue;
      }
      if (f.kind == RF_BOX_FAR && !admits(f.y)) continue;
      // far_dist = replace_axis(cell, axes[dim], reduce(|diff|)) (metric.rs:93-98)
      const double old = axes[dim];
      const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), pexp);
      const double far_dist = (M == M_LINF) ? max_nn(f.x, far_axis) : dadd(dsub(f.x, old), far_axis);
      const bool enter = f.kind == RF_BOX_FAR || (admits(far_dist) && box_admits(far));
      if (enter) {
        // enter_far (query.rs:329-341)
        fr[sp++] = RefFrame{dim, RF_RESTORE, old, 0.0};
        axes[dim] = far_axis;
        node = far;
        cell = far_dist;
        resumed = true;
      }
    }
    if (!resumed) break;
    descending = true;
  }
  best.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.n_points, false);
}

// Whether the eps = 0 result already written for query qi is the reference's
// own, decided without its descent.  The reference's bound min(k-th best,
// cutoff) never falls below T = min(k-th exact distance, cutoff) of the exact
// top-k (the k-th best among the points it has seen is at least the k-th
// among all points), and it enters a subtree when every gate on the way admits
// (x <= bound): the root's seed (query.rs:223-232); at an inner node, the far
// child's plane bound replace_axis(cell, axes[dim], reduce(|diff|)) and then
// its box distance (query.rs:270-289); at an order_by_box node, the child's box
// distance (query.rs:298-327); the near child of an inner node has none.  Those
// gate values depend on the path alone.  So when every gate on the path to
// each of the k result points admits at T, the reference reaches all of them,
// and the k smallest of what it sees are they: the same rows in the same
// order.  Only a gate that rounds within an ulp or so of T fails the test.
// Lane j walks the path of result slot j (and j + 32); the CellBound axes its
// path replaces are kept as a per-lane log.
template <int M, int D>
__device__ bool ref_results_stand(const QArgs& a, uint64_t qi) {
  if constexpr (M == M_LP) {
    return false;
  } else {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t d = D > 0 ? static_cast<uint32_t>(D) : static_cast<uint32_t>(a.d);
    const double* qg = a.queries + qi * d;
    QVec<D> q;
    q.g = qg;
    if constexpr (D > 0) {
#pragma unroll
      for (int i = 0; i < D; ++i) q.v[i] = qg[i];
    }
    const uint32_t k = static_cast<uint32_t>(a.k);
    const int64_t* oi = a.out_i + qi * a.k;
    uint32_t row[2] = {0, 0};
    bool real[2];
    uint32_t n_real = 0;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const uint32_t j = lane + 32u * s;
      const int64_t id = j < k ? oi[j] : -1;
      real[s] = id >= 0 && static_cast<uint64_t>(id) < a.n_points;
      if (real[s]) row[s] = a.rows_of[id];
      n_real += __popc(__ballot_sync(FULL_MASK, real[s]));
    }
    // T: the cutoff, or the k-th point's exact distance (its Packed chunk flag
    // needs its leaf: the left child of a node holds the first len / 2 rows)
    uint64_t T = dbits(a.cutoff);
    if (n_real == k && k > 0) {
      const uint32_t j = k - 1;
      uint64_t xb = 0;
      if (lane == (j & 31)) {
        const uint32_t r = row[j >> 5];
        uint32_t node = 0, start = 0, len = static_cast<uint32_t>(a.n_points);
        DNode nd = a.nodes[0];
        while (!(nd.meta & KD_NODE_LEAF)) {
          const uint32_t mid = len / 2;
          if (r < start + mid) {
            node = node + 1;
            len = mid;
          } else {
            node = nd.right;
            start += mid;
            len -= mid;
          }
          nd = a.nodes[node];
        }
        const uint32_t cw = (M != M_LINF && (d == 4 || d == 8)) ? (d == 4 ? 2u : 8u) : 0u;
        const bool in_chunk = cw && r < start + len / cw * cw;
        const int strat = (d <= 8) ? S_PACKED : ((M == M_L1 || M == M_L2) && d <= 16 ? S_FOLDED : S_STREAMED);
        if constexpr (D > 0) {
          QMem<D> qm;
          qm.g = qg;
          xb = dbits(exact_dist<M, D>(qm, a.data + static_cast<uint64_t>(r) * D, D, S_PACKED, in_chunk, 0.0));
        } else {
          xb = dbits(exact_dist<M, 0>(q, a.data + static_cast<uint64_t>(r) * d, d, strat, in_chunk, 0.0));
        }
      }
      xb = __shfl_sync(FULL_MASK, xb, static_cast<int>(j & 31));
      T = xb < T ? xb : T;
    }
    // the root's seed (CellBound::start)
    const double rb = exact_box_dist<M, D>(q, a.boxes, d, 0.0);
    auto seed_axis = [&](uint32_t i) -> double {
      return rb != 0.0 ? reduce<M>(axis_offset(qg[i], a.boxes[i], a.boxes[d + i]), 0.0) : 0.0;
    };
    double seed = 0.0;
    if (rb != 0.0)
      for (uint32_t i = 0; i < d; ++i) seed = (M == M_LINF) ? max_nn(seed, seed_axis(i)) : dadd(seed, seed_axis(i));
    bool ok = leq_bound(seed, T);
    uint32_t log_dim[KD_MAX_DEPTH];
    double log_val[KD_MAX_DEPTH];
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
      if (!ok || !real[s]) continue;
      const uint32_t r = row[s];
      uint32_t node = 0, start = 0, len = static_cast<uint32_t>(a.n_points);
      double cell = seed;
      int n_log = 0;
      for (;;) {
        const DNode nd = a.nodes[node];
        if (nd.meta & KD_NODE_LEAF) break;
        const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
        const double qd = qg[dim];
        const bool left_near = ieee_key(dbits(qd)) <= ieee_key(dbits(nd.split));
        const uint32_t mid = len / 2;
        const bool go_left = r < start + mid;
        const uint32_t child = go_left ? node + 1 : nd.right;
        const bool far = go_left != left_near;
        const double* cbox = a.boxes + static_cast<uint64_t>(child) * 2 * d;
        if (nd.meta & KD_NODE_BOX_ORDER) {
          if (!leq_bound(exact_box_dist<M, D>(q, cbox, d, 0.0), T)) {
            ok = false;
            break;
          }
        }
        if (far) {
          double old = seed_axis(dim);
          for (int t = n_log - 1; t >= 0; --t)
            if (log_dim[t] == dim) {
              old = log_val[t];
              break;
            }
          const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), 0.0);
          const double far_dist = (M == M_LINF) ? max_nn(cell, far_axis) : dadd(dsub(cell, old), far_axis);
          if (!(nd.meta & KD_NODE_BOX_ORDER) &&
              !(leq_bound(far_dist, T) && leq_bound(exact_box_dist<M, D>(q, cbox, d, 0.0), T))) {
            ok = false;
            break;
          }
          if (n_log < KD_MAX_DEPTH) {
            log_dim[n_log] = dim;
            log_val[n_log] = far_axis;
            ++n_log;
          } else {
            ok = false;  // deeper than any tree the build makes
            break;
          }
          cell = far_dist;
        }
        if (go_left) {
          node = node + 1;
          len = mid;
        } else {
          node = nd.right;
          start += mid;
          len -= mid;
        }
      }
    }
    return __all_sync(FULL_MASK, ok);
  }
}

// Warps take queries w = global warp, + total warps, ... < n: positions of
// the batch (a.order when set), or -- with `list` -- the flagged queries of a
// rerun (count on the device): those whose results the path test above
// confirms are left as they are, the rest run in the reference's order.  Dynamic shared memory: ref_warp_smem(d, w32)
// bytes per warp.
template <int M, int D, int KS>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_ref(QArgs a, const uint32_t* count, const uint64_t* list) {
  extern __shared__ __align__(16) unsigned char ref_smem[];
  const uint32_t wid = threadIdx.x >> 5;
  const uint32_t d = D > 0 ? static_cast<uint32_t>(D) : static_cast<uint32_t>(a.d);
  const uint64_t per = ref_warp_smem(d, (D == 0 && M != M_LP) ? a.w32 : 0);
  unsigned char* base = ref_smem + wid * per;
  RefFrame* fr = reinterpret_cast<RefFrame*>(base);
  double* axes = reinterpret_cast<double*>(base + ref_axes_offset());
  float* sq = reinterpret_cast<float*>(base + ref_q32_offset(d));
  const uint64_t n = count ? *count : a.nq;
  const uint64_t warps = static_cast<uint64_t>(gridDim.x) * (QUERY_THREADS / 32);
  for (uint64_t w = blockIdx.x * static_cast<uint64_t>(QUERY_THREADS / 32) + wid; w < n; w += warps) {
    const uint64_t qi = list ? static_cast<uint32_t>(list[w]) : (a.order ? a.order[w] : w);
    if (list) {
      if (ref_results_stand<M, D>(a, qi)) continue;
      if (a.rerun_total && (threadIdx.x & 31) == 0) atomicAdd(a.rerun_total + 1, 1ull);
    }
    ref_query<M, D, KS>(a, qi, fr, axes, sq);
  }
}
