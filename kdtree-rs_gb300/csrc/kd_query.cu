// kd_query.cu -- exact k-NN query on the GPU.
//
// One thread runs one query's depth-first descent with an explicit stack, in
// exactly the reference's order (src/query.rs:223-341): near child first, the
// far child gated by the O(1) split-plane bound and then by the far child's
// tight box, `order_by_box` nodes visiting the child with the smaller box
// distance first.  The pruning bound, the CellBound per-axis offsets and every
// distance are computed with the reference's FP64 operations in the reference's
// order (src/kernel.rs summation orders, src/metric.rs algebra), so each
// decision -- and therefore the result -- is the reference's, ties and eps > 0
// included.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so exact FP64 arithmetic is spent
// only where a decision needs it: every leaf point and every far-child box is
// first bounded from below in FP32 with directed rounding (a rigorous lower
// bound of the exact distance), and only candidates whose lower bound does not
// already exceed the pruning bound are recomputed in FP64 in the reference's
// order.  A rejected point could never have been accepted, so the sequence of
// accepted offers -- and every bound after them -- is unchanged.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "kd_internal.hpp"

namespace kd {

namespace {

#include "kd_query_common.cuh"

// ---------------------------------------------------------------------------
// The k best so far, sorted by (reduced distance, original index): K register
// slots, the first K - k holding (0, 0) placeholders nothing sorts before, the
// rest (+inf, NO_ID) until filled (BestK / Best1, src/query.rs:379-494).
// Distances are compared as the bit patterns of non-negative doubles.
// ---------------------------------------------------------------------------
template <int K>
struct BestList {
  uint64_t dist[K];
  uint32_t id[K];
  __device__ __forceinline__ void reset(uint64_t k) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
      bool pad = static_cast<uint64_t>(j) < K - k;
      dist[j] = pad ? 0ull : INF_BITS;
      id[j] = pad ? 0u : NO_ID;
    }
  }
  __device__ __forceinline__ uint64_t worst() const { return dist[K - 1]; }
  __device__ __forceinline__ static bool lt(uint64_t da, uint32_t ia, uint64_t db, uint32_t ib) {
    return da < db || (da == db && ia < ib);
  }
  __device__ __forceinline__ void consider(uint64_t dd, uint32_t ii) {
    if (!lt(dd, ii, dist[K - 1], id[K - 1])) return;
#pragma unroll
    for (int j = K - 1; j > 0; --j) {
      bool before_prev = lt(dd, ii, dist[j - 1], id[j - 1]);
      bool before_cur = lt(dd, ii, dist[j], id[j]);
      uint64_t nd = before_prev ? dist[j - 1] : (before_cur ? dd : dist[j]);
      uint32_t ni = before_prev ? id[j - 1] : (before_cur ? ii : id[j]);
      dist[j] = nd;
      id[j] = ni;
    }
    if (lt(dd, ii, dist[0], id[0])) {
      dist[0] = dd;
      id[0] = ii;
    }
  }
};

// k > 32: the same sorted list held in the query's own output row (distance
// bits in the distance slots, indices in the index slots), shifted in memory.
template <>
struct BestList<0> {
  uint64_t* dist;
  int64_t* id;
  uint64_t k;
  __device__ __forceinline__ void bind(double* od, int64_t* oi, uint64_t kk) {
    dist = reinterpret_cast<uint64_t*>(od);
    id = oi;
    k = kk;
  }
  __device__ __forceinline__ void reset(uint64_t) {
    for (uint64_t j = 0; j < k; ++j) {
      dist[j] = INF_BITS;
      id[j] = NO_ID;
    }
  }
  __device__ __forceinline__ uint64_t worst() const { return dist[k - 1]; }
  __device__ __forceinline__ static bool lt(uint64_t da, uint32_t ia, uint64_t db, uint32_t ib) {
    return da < db || (da == db && ia < ib);
  }
  __device__ void consider(uint64_t dd, uint32_t ii) {
    if (!lt(dd, ii, dist[k - 1], static_cast<uint32_t>(id[k - 1]))) return;
    uint64_t pos = k - 1;
    while (pos > 0 && lt(dd, ii, dist[pos - 1], static_cast<uint32_t>(id[pos - 1]))) {
      dist[pos] = dist[pos - 1];
      id[pos] = id[pos - 1];
      --pos;
    }
    dist[pos] = dd;
    id[pos] = ii;
  }
};

// Stack frames of the iterative descent.
enum FrameKind : uint32_t { F_FAR = 0, F_RESTORE = 1, F_BOX_FAR = 2, F_BOX_NEAR = 3 };
struct Frame {
  uint32_t node;  // parent node id (F_FAR / F_BOX_*) or split dim (F_RESTORE)
  uint32_t kind;
  double x;       // parent cell_dist, or the saved axis value
  double y;       // the pending child's box distance (F_BOX_*)
};

template <int M, int D, int K>
__global__ void __launch_bounds__(QUERY_THREADS) k_query(QArgs a) {
  const uint64_t tid = blockIdx.x * static_cast<uint64_t>(QUERY_THREADS) + threadIdx.x;
  if (tid >= a.nq) return;
  const uint64_t qi = a.order ? a.order[tid] : tid;
  const uint64_t d = D > 0 ? D : a.d;
  const double pexp = a.p;
  const int strat = (M != M_LP && d <= 8) ? S_PACKED : ((M == M_L1 || M == M_L2) && d <= 16 ? S_FOLDED : S_STREAMED);
  // FP32 interval gates: compile-time widths, metrics without pow(), eps = 0.
  constexpr bool FAST = D > 0 && M != M_LP;
  const bool gates = FAST && !a.use_eps;

  QVec<D> q;
  q.g = a.queries + qi * d;
  bool finite = true;
  if (D > 0) {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      q.v[i] = q.g[i];
      finite &= isfinite(q.v[i]);
    }
  } else {
    for (uint64_t i = 0; i < d; ++i) finite &= isfinite(q.g[i]);
  }
  if (!finite) {
    atomicOr(a.status, 1u);
    return;
  }
  // FP32 enclosures and IEEE keys of the query (compile-time widths only)
  float qlo[D > 0 ? D : 1], qhi[D > 0 ? D : 1];
  uint64_t qkey[D > 0 ? D : 1];
  if (D > 0) {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      rn_enclose(__double2float_rn(q.v[i]), &qlo[i], &qhi[i]);
      qkey[i] = ieee_key(dbits(q.v[i]));
    }
  }
  auto qkey_of = [&](uint32_t j) -> uint64_t {
    if (D > 0) {
      uint64_t v = 0;
#pragma unroll
      for (int i = 0; i < D; ++i) v = (static_cast<uint32_t>(i) == j) ? qkey[i] : v;
      return v;
    }
    return ieee_key(dbits(q.g[j]));
  };

  // CellBound axes (query.rs:156-211)
  double axes_r[D > 0 ? D : 1];
  double* axes_g = a.axes_scratch + (D > 0 ? 0 : qi * d);
  auto axis_get = [&](uint32_t j) -> double {
    if (D > 0) {
      double v = 0.0;
#pragma unroll
      for (int i = 0; i < D; ++i) v = (static_cast<uint32_t>(i) == j) ? axes_r[i] : v;
      return v;
    }
    return axes_g[j];
  };
  auto axis_set = [&](uint32_t j, double v) {
    if (D > 0) {
#pragma unroll
      for (int i = 0; i < D; ++i) axes_r[i] = (static_cast<uint32_t>(i) == j) ? v : axes_r[i];
    } else {
      axes_g[j] = v;
    }
  };
  if (D > 0) {
#pragma unroll
    for (int i = 0; i < D; ++i) axes_r[i] = 0.0;
  } else {
    for (uint64_t i = 0; i < d; ++i) axes_g[i] = 0.0;
  }

  const uint64_t cutoff_bits = dbits(a.cutoff);
  BestList<K> best;
  if constexpr (K == 0) best.bind(a.out_d + qi * a.k, a.out_i + qi * a.k, a.k);
  best.reset(a.k);
  auto bound_bits = [&]() -> uint64_t {
    uint64_t w = best.worst();
    return w < cutoff_bits ? w : cutoff_bits;
  };
  // FP32 enclosure of the current bound, refreshed whenever it changes
  uint64_t bnd = bound_bits();
  float b_hi = __fmul_ru(mag_up32(bnd), UB_GROW);
  float b_lo = __fmul_rd(mag_dn32(bnd), LB_SHRINK);
  auto refresh_bound = [&]() {
    bnd = bound_bits();
    b_hi = __fmul_ru(mag_up32(bnd), UB_GROW);
    b_lo = __fmul_rd(mag_dn32(bnd), LB_SHRINK);
  };
  auto admits_at = [&](double dist, uint64_t bb) -> bool {
    if (a.use_eps) dist = dmul(dist, a.eps_factor);
    return leq_bound(dist, bb);
  };

  // Far-child box gate (query.rs:283): interval bounds first, exact FP64 box
  // distance (kernel.rs:565-616) only when they cannot decide.
  auto box_admits = [&](uint32_t id) -> bool {
    if (gates) {
      const float* b32 = a.boxes32 + static_cast<uint64_t>(id) * 2 * D;
      float lb = 0.f, ub = 0.f;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        // lo in [lo32, lo32 + ulp], hi in [hi32 - ulp, hi32]: outward-rounded copies
        const float lo32 = b32[i], hi32 = b32[D + i];
        const float lo_up = __fadd_ru(lo32, __fmaf_ru(fabsf(lo32), TWO_M23, TINY32));
        const float hi_dn = __fsub_rd(hi32, __fmaf_ru(fabsf(hi32), TWO_M23, TINY32));
        float o_lb = fmaxf(__fsub_rd(lo32, qhi[i]), __fsub_rd(qlo[i], hi32));
        o_lb = o_lb > 0.f ? o_lb : 0.f;
        const float o_ub = fmaxf(fmaxf(__fsub_ru(lo_up, qlo[i]), __fsub_ru(qhi[i], hi_dn)), 0.f);
        lb = fold_lb<M>(lb, red_lb<M>(o_lb));
        ub = fold_ub<M>(ub, red_ub<M>(o_ub));
      }
      if (lb > b_hi) return false;
      if (ub < b_lo) return true;
    }
    double bd = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(id) * 2 * d, d, pexp);
    return admits_at(bd, bnd);
  };

  // scan_leaf + Strategy::scan + LeafSink (query.rs:343-375, kernel.rs:366-562)
  auto scan_leaf = [&](uint32_t start, uint32_t end) {
    const uint32_t len = end - start;
    uint32_t chunk_pts = len;
    if (strat == S_PACKED && M != M_LINF) {
      if (d == 4) chunk_pts = len / 2 * 2;
      else if (d == 8) chunk_pts = len / 8 * 8;
    }
    for (uint32_t j = 0; j < len; ++j) {
      const uint64_t row = static_cast<uint64_t>(start) + j;
      if (FAST) {
        const float* p32 = a.data32 + row * D;
        float lb = 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) {
          float plo, phi;
          rn_enclose(p32[i], &plo, &phi);
          lb = fold_lb<M>(lb, red_lb<M>(absdiff_lb(plo, phi, qlo[i], qhi[i])));
        }
        if (lb > b_hi) continue;  // exact distance > bound: never offered
      }
      double dist = exact_dist<M, D>(q, a.data + row * d, d, strat, j < chunk_pts, pexp);
      if (dbits(dist) <= bnd) {
        best.consider(dbits(dist), a.indices[row]);
        refresh_bound();
      }
    }
  };

  // Descent::run (query.rs:223-232): CellBound::start seeds from the root box.
  double seed = 0.0;
  {
    double rb = exact_box_dist<M, D>(q, a.boxes, d, pexp);
    if (rb != 0.0) {
      for (uint64_t i = 0; i < d; ++i) {
        double ax = reduce<M>(axis_offset(q[i], a.boxes[i], a.boxes[d + i]), pexp);
        axis_set(static_cast<uint32_t>(i), ax);
        seed = (M == M_LINF) ? max_nn(seed, ax) : dadd(seed, ax);
      }
    }
  }

  Frame stack[2 * KD_MAX_DEPTH];
  int sp = 0;
  uint32_t node = 0;
  double cell = seed;
  bool descending = admits_at(seed, bnd);

  for (;;) {
    while (descending) {
      // Descent::descend (query.rs:248-289)
      const DNode nd = a.nodes[node];
      if (nd.meta & KD_NODE_LEAF) {
        uint64_t se = dbits(nd.split);
        scan_leaf(static_cast<uint32_t>(se), static_cast<uint32_t>(se >> 32));
        descending = false;
        break;
      }
      const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
      // diff <= 0  <=>  q[dim] <= split (exact for finite doubles)
      const bool left_near = qkey_of(dim) <= ieee_key(dbits(nd.split));
      const uint32_t near = left_near ? node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : node + 1;
      if (nd.meta & KD_NODE_BOX_ORDER) {
        // descend_by_box (query.rs:298-327)
        double near_box = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(near) * 2 * d, d, pexp);
        double far_box = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(far) * 2 * d, d, pexp);
        if (dbits(near_box) <= dbits(far_box)) {
          stack[sp++] = Frame{node, F_BOX_FAR, cell, far_box};
          if (admits_at(near_box, bnd)) {
            node = near;
            continue;
          }
          descending = false;
          break;
        }
        stack[sp++] = Frame{node, F_BOX_NEAR, cell, near_box};
        if (admits_at(far_box, bnd)) {
          const double far_axis = reduce<M>(fabs(dsub(q[dim], nd.split)), pexp);
          const double old = axis_get(dim);
          const double far_dist = (M == M_LINF) ? max_nn(cell, far_axis) : dadd(dsub(cell, old), far_axis);
          stack[sp++] = Frame{dim, F_RESTORE, old, 0.0};
          axis_set(dim, far_axis);
          node = far;
          cell = far_dist;
          continue;
        }
        descending = false;
        break;
      }
      stack[sp++] = Frame{node, F_FAR, cell, 0.0};
      node = near;  // near child keeps the parent's cell bound
    }
    // unwind to the next pending far-child decision
    bool resumed = false;
    while (sp > 0 && !resumed) {
      const Frame f = stack[--sp];
      if (f.kind == F_RESTORE) {
        axis_set(f.node, f.x);
        continue;
      }
      const DNode nd = a.nodes[f.node];
      const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
      const bool left_near = qkey_of(dim) <= ieee_key(dbits(nd.split));
      const uint32_t near = left_near ? f.node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : f.node + 1;
      if (f.kind == F_BOX_NEAR) {
        if (admits_at(f.y, bnd)) {
          node = near;
          cell = f.x;
          resumed = true;
        }
        continue;
      }
      const double old = axis_get(dim);
      if (f.kind == F_BOX_FAR) {
        if (!admits_at(f.y, bnd)) continue;
      }
      // far_dist = replace_axis(cell, old, reduce(|diff|)) (metric.rs:93-98).
      // c = cell - old is the first FP64 step; the plane gate is first decided
      // on c and an FP32 lower bound of reduce(|diff|).
      const double c = (M == M_LINF) ? f.x : dsub(f.x, old);
      if (gates && f.kind == F_FAR) {
        float slo = rd32(dbits(nd.split)), shi = ru32(dbits(nd.split));
        float qlo_d = 0.f, qhi_d = 0.f;
#pragma unroll
        for (int i = 0; i < (D > 0 ? D : 1); ++i)
          if (static_cast<uint32_t>(i) == dim) {
            qlo_d = qlo[i];
            qhi_d = qhi[i];
          }
        const float fa_lb = __fmul_rd(red_lb<M>(absdiff_lb(qlo_d, qhi_d, slo, shi)), LB_SHRINK);
        float lb;
        if (M == M_LINF) {
          const float c_lb = mag_dn32(dbits(c));
          lb = c_lb > fa_lb ? c_lb : fa_lb;
        } else {
          lb = __fadd_rd(rd32(dbits(c)), fa_lb);
          lb = lb > 0.f ? __fmul_rd(lb, LB_SHRINK) : lb;
        }
        if (lb > b_hi) continue;  // plane bound already above the bound
      }
      const double far_axis = reduce<M>(fabs(dsub(q[dim], nd.split)), pexp);
      const double far_dist = (M == M_LINF) ? max_nn(c, far_axis) : dadd(c, far_axis);
      bool enter = true;
      if (f.kind == F_FAR) enter = admits_at(far_dist, bnd) && box_admits(far);
      if (enter) {
        // enter_far (query.rs:329-341)
        stack[sp++] = Frame{dim, F_RESTORE, old, 0.0};
        axis_set(dim, far_axis);
        node = far;
        cell = far_dist;
        resumed = true;
      }
    }
    if (!resumed) break;
    descending = true;
  }

  // write_results (query.rs:421-429, 483-493)
  double* od = a.out_d + qi * a.k;
  int64_t* oi = a.out_i + qi * a.k;
  if constexpr (K == 0) {
    for (uint64_t j = 0; j < a.k; ++j) {  // convert the in-place list
      if (oi[j] != static_cast<int64_t>(NO_ID)) {
        od[j] = restore<M>(od[j], pexp);
      } else {
        od[j] = __longlong_as_double(0x7ff0000000000000ll);
        oi[j] = static_cast<int64_t>(a.n_points);
      }
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (static_cast<uint64_t>(j) >= K - a.k) {
      const uint64_t o = j - (K - a.k);
      if (best.id[j] != NO_ID) {
        od[o] = restore<M>(bitsd(best.dist[j]), pexp);
        oi[o] = static_cast<int64_t>(best.id[j]);
      } else {
        od[o] = __longlong_as_double(0x7ff0000000000000ll);
        oi[o] = static_cast<int64_t>(a.n_points);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Spatial ordering of a batch: each query's landing leaf (where its descent
// first arrives: left iff q[dim] <= split, query.rs:263-268), then a counting
// sort by that leaf's preorder id.  Queries that share a leaf then share a warp
// and follow nearly the same descent.  The order changes no result.
// ---------------------------------------------------------------------------
__global__ void k_landing_leaf(const DNode* nodes, const double* queries, uint64_t nq, uint64_t d,
                               uint32_t* leaf_of, uint32_t* counts) {
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i >= nq) return;
  const double* q = queries + i * d;
  uint32_t node = 0;
  for (;;) {
    const DNode nd = nodes[node];
    if (nd.meta & KD_NODE_LEAF) break;
    // the order of IEEE keys (integer work; GB300's FP64 pipe is narrow): the
    // same side as q <= split except for signed zeros, which only moves a query
    // between neighbouring leaves of the sort
    node = (ieee_key(dbits(q[nd.meta & KD_NODE_DIM_MASK])) <= ieee_key(dbits(nd.split))) ? node + 1 : nd.right;
  }
  leaf_of[i] = node;
  atomicAdd(&counts[node], 1u);
}

#include "kd_scan.cuh"

__global__ void k_scatter_order(const uint32_t* leaf_of, uint32_t* offsets, uint64_t nq, uint32_t* order) {
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i >= nq) return;
  order[atomicAdd(&offsets[leaf_of[i]], 1u)] = static_cast<uint32_t>(i);
}

// Below this many queries the ordering costs more than it saves.
constexpr uint64_t ORDER_MIN_QUERIES = 4096;


// KD_QUERY_MODE=dfs runs every query through the reference-order descent (the
// eps > 0 kernel) instead of the packet traversal; a diagnostic switch, same results.
bool force_reference_order() {
  static const bool force = [] {
    const char* m = std::getenv("KD_QUERY_MODE");
    return m && std::strcmp(m, "dfs") == 0;
  }();
  return force;
}

// The one-thread reference-order kernel, for what the warp kernels do not
// take (k > 64, widths above 128): its k-best list lives in the query's own
// output row, so any k fits.
template <int M, int D>
int dispatch_k(const QArgs& a, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((a.nq + QUERY_THREADS - 1) / QUERY_THREADS);
  k_query<M, D, 0><<<blocks, QUERY_THREADS, 0, st>>>(a);
  KD_TRY_CUDA(cudaGetLastError());
  return KD_OK;
}

template <int M>
int dispatch_d(const QArgs& a, cudaStream_t st) {
  if (M != M_LP) {
    switch (a.d) {
      case 2: return dispatch_k<M, 2>(a, st);
      case 3: return dispatch_k<M, 3>(a, st);
      case 8: return dispatch_k<M, 8>(a, st);
      default: break;
    }
  }
  return dispatch_k<M, 0>(a, st);
}

// The automatic choice between the two eps = 0 traversals, from measurements on
// GB300 (uniform and clustered data, N = 1M): one warp per query wins at
// d >= 8, for k > 16, for k >= 8 below a few hundred thousand queries, and for
// any k on small batches (the packet traversal's 32-query warps have long
// serial chains, which only a large batch hides); the packet traversal wins for
// small k on big batches.  Widths the packet traversal lacks always take the
// warp.
bool warp_preferred(const QArgs& a) {
  return a.d >= 8 || a.k > 16 || (a.k >= 8 && a.nq < 400000) || a.nq < 32768;
}

// Events around the last query kernel launched by this thread (not while the
// stream is being captured), read by kd_last_query_kernel_ms.
struct KernelClock {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int dev = -1;
  bool valid = false;
};
KernelClock& kernel_clock() {
  thread_local KernelClock c;
  return c;
}

struct KernelTimer {
  cudaStream_t st;
  bool on = false;
  explicit KernelTimer(cudaStream_t s) : st(s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
      cudaGetLastError();
      return;
    }
    KernelClock& c = kernel_clock();
    int dev = 0;
    cudaGetDevice(&dev);
    if (c.dev != dev) {
      if (c.e0) cudaEventDestroy(c.e0);
      if (c.e1) cudaEventDestroy(c.e1);
      c.e0 = c.e1 = nullptr;
      if (cudaEventCreate(&c.e0) != cudaSuccess || cudaEventCreate(&c.e1) != cudaSuccess) {
        cudaGetLastError();
        return;
      }
      c.dev = dev;
    }
    on = cudaEventRecord(c.e0, st) == cudaSuccess;
  }
  ~KernelTimer() {
    KernelClock& c = kernel_clock();
    c.valid = on && cudaEventRecord(c.e1, st) == cudaSuccess;
  }
};

// Launch the query kernels for `a`.  eps = 0 (and not forced to the reference
// order): the packet or warp traversal, then -- when a.rerun_count is set --
// the reference-order rerun of the near ties they flag (that count is zeroed
// here first).  Otherwise the reference-order warp kernel, or for k > 64 or
// widths above 128 the one-thread reference-order kernels.
int run_kernels(const QArgs& a, int metric, cudaStream_t st, int path) {
  KernelTimer timer(st);
  if (!a.reference_order && !force_reference_order() && path != PATH_REFERENCE_ORDER) {
    const bool eps0 = !a.use_eps;
    const bool warp = warp_applicable(a.d, metric, a.k, a.n_points, !eps0);
    const bool packet = packet_applicable(a.d, metric, a.k, a.n_points, !eps0);
    int use = 0;  // 1 warp, 2 packet
    if (path == PATH_WARP) use = warp ? 1 : 0;
    else if (path == PATH_PACKET) use = packet ? 2 : 0;
    else if (warp && (warp_preferred(a) || !packet)) use = 1;
    else if (packet) use = 2;
    if (use) {
      if (a.rerun_count) KD_TRY_CUDA(cudaMemsetAsync(a.rerun_count, 0, sizeof(uint32_t), st));
      const int rc = use == 1 ? launch_warp_query(a, metric, st) : launch_packet_query(a, metric, st);
      if (rc || !a.rerun_count) return rc;
      return launch_rerun(a, metric, st, a.rerun_count, a.rerun_list);
    }
  }
  if (ref_warp_applicable(a.d, a.k, a.n_points)) return launch_ref_query(a, metric, st);
  switch (metric) {
    case M_L1: return dispatch_d<M_L1>(a, st);
    case M_L2: return dispatch_d<M_L2>(a, st);
    case M_LINF: return dispatch_d<M_LINF>(a, st);
    default: return dispatch_d<M_LP>(a, st);
  }
}

}  // namespace

bool writes_whole_rows(const kd_tree* t, const QueryParams& qp) {
  if (qp.path == PATH_REFERENCE_ORDER || qp.path == PATH_TENSOR_CORE || force_reference_order()) return false;
  if (qp.path == PATH_AUTO && tc_applicable(t, qp)) return false;  // may run the tensor-core filter
  const bool use_eps = qp.eps_factor != 1.0;
  if (!warp_applicable(t->ndim, qp.metric, qp.k, t->n_points, use_eps)) return false;
  // The warp kernels (and the near-tie reruns, which rewrite a few rows after
  // the first kernel, in stream order) write rows whole; so do the packet
  // traversal's heaps (k >= 5).
  if (!packet_applicable(t->ndim, qp.metric, qp.k, t->n_points, use_eps)) return true;
  return qp.k >= 5;
}

uint64_t order_scratch_words(const kd_tree* t) {
  return t->n_nodes + (t->n_nodes + SCAN_TILE - 1) / SCAN_TILE;
}

void order_by_landing_leaf(const kd_tree* t, const double* d_queries, uint64_t nq, uint32_t* leaf_of,
                           uint32_t* order, uint32_t* scratch, cudaStream_t st) {
  const uint64_t n_tiles = (t->n_nodes + SCAN_TILE - 1) / SCAN_TILE;
  uint32_t* counts = scratch;
  uint32_t* tile_sums = counts + t->n_nodes;
  cudaMemsetAsync(counts, 0, t->n_nodes * sizeof(uint32_t), st);
  const unsigned qb = static_cast<unsigned>((nq + 255) / 256);
  k_landing_leaf<<<qb, 256, 0, st>>>(t->nodes, d_queries, nq, t->ndim, leaf_of, counts);
  k_scan_tiles<<<static_cast<unsigned>(n_tiles), SCAN_THREADS, 0, st>>>(counts, t->n_nodes, tile_sums);
  k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(tile_sums, n_tiles);
  k_scan_add<<<static_cast<unsigned>((t->n_nodes + 255) / 256), 256, 0, st>>>(counts, t->n_nodes, tile_sums);
  k_scatter_order<<<qb, 256, 0, st>>>(leaf_of, counts, nq, order);
}

// Width 16 (L2, eps = 0) has two exact paths: the tensor-core filter, which
// scores whole point tiles, and the warp-per-query traversal, which wins where
// the tree prunes well.  Which one is faster also depends on the batch size
// (the tensor-core path needs whole 128-query tiles on every SM), so the
// choice is kept per batch-size class: the first automatic query of each class
// on a tree times both on a sample of its batch (the first min(n, 16384)
// queries, written to the caller's outputs -- both paths produce the same
// values) and the tree keeps the faster for every later call of that class.
constexpr uint64_t AUTO_LARGE_BATCH = 32768;

int auto_prefers_tc(kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp, double* d_out_d,
                    int64_t* d_out_i, cudaStream_t st, uint32_t* d_status, bool* tc) {
  std::lock_guard<std::mutex> lock(t->choice_mutex);
  int& choice = t->auto_choice[nq >= AUTO_LARGE_BATCH ? 1 : 0];
  if (choice >= 0) {
    *tc = choice == 1;
    return KD_OK;
  }
  if (qp.no_sync) {  // a stream-ordered call times nothing: the warp traversal until a timed call chose
    *tc = false;
    return KD_OK;
  }
  const uint64_t ns = std::min<uint64_t>(nq, 16384);
  QueryParams pq = qp;
  pq.path = PATH_WARP;
  cudaEvent_t e[3];
  for (cudaEvent_t& x : e) KD_TRY_CUDA(cudaEventCreate(&x));
  int rc = query_tc_on_device(t, d_queries, ns, qp, d_out_d, d_out_i, st, d_status, nullptr);  // warm-up
  if (!rc) rc = cudaEventRecord(e[0], st) == cudaSuccess ? KD_OK : cuda_fail(cudaErrorUnknown, "cudaEventRecord");
  if (!rc) rc = query_tc_on_device(t, d_queries, ns, qp, d_out_d, d_out_i, st, d_status, nullptr);
  if (!rc) cudaEventRecord(e[1], st);
  if (!rc) rc = query_on_device(t, d_queries, ns, pq, d_out_d, d_out_i, st, d_status, nullptr);
  if (!rc) cudaEventRecord(e[2], st);
  float ms_tc = 0.f, ms_pk = 0.f;
  if (!rc) {
    cudaError_t err = cudaEventSynchronize(e[2]);
    if (err != cudaSuccess) rc = cuda_fail(err, "cudaEventSynchronize");
    cudaEventElapsedTime(&ms_tc, e[0], e[1]);
    cudaEventElapsedTime(&ms_pk, e[1], e[2]);
  }
  for (cudaEvent_t x : e) cudaEventDestroy(x);
  if (rc) return rc;
  choice = ms_tc <= ms_pk ? 1 : 0;
  *tc = choice == 1;
  return KD_OK;
}

QArgs query_args(const kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp, double* d_out_d,
                 int64_t* d_out_i, uint32_t* d_status) {
  QArgs a{};
  a.reference_order = qp.path == PATH_REFERENCE_ORDER;
  a.data = t->data;
  a.data32 = t->data32;
  a.data32w = t->data32w;
  a.w32 = t->w32;
  a.indices = t->indices;
  a.rows_of = t->rows_of;
  a.nodes = t->nodes;
  a.boxes = t->boxes;
  a.boxes32 = t->boxes32;
  a.coord_max = t->coord_max32;
  a.queries = d_queries;
  a.out_d = d_out_d;
  a.out_i = d_out_i;
  a.status = d_status;
  a.nq = nq;
  a.d = t->ndim;
  a.k = qp.k;
  a.n_points = t->n_points;
  a.p = qp.p;
  a.cutoff = qp.cutoff;
  a.eps_factor = qp.eps_factor;
  a.use_eps = qp.eps_factor != 1.0;
  return a;
}

namespace {

// Where neither traversal is clearly ahead (widths 2 and 3, eps = 0, batches
// of 32,768 up to 524,287 queries), the first automatic call of each class
// on a tree runs both on its whole batch and the tree keeps the faster for
// later calls of that class; stream-ordered calls time nothing and take the
// rule of warp_preferred.
constexpr uint64_t TRAVERSAL_TIMED_MIN = 32768, TRAVERSAL_TIMED_MAX = 524288, TRAVERSAL_TIMED_SPLIT = 131072;

bool traversal_timed(const kd_tree* t, uint64_t nq, const QueryParams& qp) {
  const bool use_eps = qp.eps_factor != 1.0;
  return !qp.no_sync && !force_reference_order() && (t->ndim == 2 || t->ndim == 3) && nq >= TRAVERSAL_TIMED_MIN &&
         nq < TRAVERSAL_TIMED_MAX && warp_applicable(t->ndim, qp.metric, qp.k, t->n_points, use_eps) &&
         packet_applicable(t->ndim, qp.metric, qp.k, t->n_points, use_eps);
}

// Run the query with the warp traversal, then with the packet traversal (the
// same results), timing each with events; *choice = 1 when the packet
// traversal was faster.  The first run counts no near-tie reruns, so the
// counters count one run.
int time_traversals(QArgs a, int metric, cudaStream_t st, int* choice) {
  cudaEvent_t e[3];
  for (int i = 0; i < 3; ++i) {
    if (cudaEventCreate(&e[i]) != cudaSuccess) {
      for (int j = 0; j < i; ++j) cudaEventDestroy(e[j]);
      return cuda_fail(cudaErrorMemoryAllocation, "cudaEventCreate");
    }
  }
  unsigned long long* total = a.rerun_total;
  a.rerun_total = nullptr;
  int rc = cudaEventRecord(e[0], st) == cudaSuccess ? KD_OK : cuda_fail(cudaErrorUnknown, "cudaEventRecord");
  if (!rc) rc = run_kernels(a, metric, st, PATH_WARP);
  if (!rc) cudaEventRecord(e[1], st);
  a.rerun_total = total;
  if (!rc) rc = run_kernels(a, metric, st, PATH_PACKET);
  if (!rc) cudaEventRecord(e[2], st);
  float ms_warp = 0.f, ms_packet = 0.f;
  if (!rc) {
    const cudaError_t err = cudaEventSynchronize(e[2]);
    if (err != cudaSuccess) rc = cuda_fail(err, "cudaEventSynchronize");
    cudaEventElapsedTime(&ms_warp, e[0], e[1]);
    cudaEventElapsedTime(&ms_packet, e[1], e[2]);
  }
  for (cudaEvent_t x : e) cudaEventDestroy(x);
  if (!rc) *choice = ms_packet < ms_warp ? 1 : 0;
  return rc;
}

// Whether the call can reach the one-thread reference-order kernels with a
// runtime width, which keep each query's CellBound axes in global scratch.
bool uses_axes_scratch(const kd_tree* t, const QueryParams& qp) {
  if (ref_warp_applicable(t->ndim, qp.k, t->n_points)) return false;
  return !(qp.metric != M_LP && (t->ndim == 2 || t->ndim == 3 || t->ndim == 8));
}

}  // namespace

int query_on_device(const kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp,
                    double* d_out_d, int64_t* d_out_i, cudaStream_t st, uint32_t* d_status,
                    unsigned long long* d_survivors) {
  // d >= 16, L2, eps = 0: the tensor-core filter, unless (d = 16, automatic
  // choice) the warp-per-query traversal measured faster on this tree
  const bool tc_allowed = qp.path == PATH_TENSOR_CORE || (qp.path == PATH_AUTO && !force_reference_order());
  if (tc_allowed && tc_applicable(t, qp)) {
    bool tc = true;
    if (qp.path == PATH_AUTO && warp_applicable(t->ndim, qp.metric, qp.k, t->n_points, false)) {
      int rc = auto_prefers_tc(const_cast<kd_tree*>(t), d_queries, nq, qp, d_out_d, d_out_i, st, d_status, &tc);
      if (rc) return rc;
    }
    if (tc) {
      KernelTimer timer(st);
      return query_tc_on_device(const_cast<kd_tree*>(t), d_queries, nq, qp, d_out_d, d_out_i, st, d_status,
                                d_survivors);
    }
  }
  QArgs a = query_args(t, d_queries, nq, qp, d_out_d, d_out_i, d_status);
  void* axes = nullptr;
  if (uses_axes_scratch(t, qp)) {
    cudaError_t e = dev_alloc(&axes, std::max<uint64_t>(1, nq * t->ndim) * sizeof(double), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
    }
    a.axes_scratch = static_cast<double*>(axes);
  }
  // near-tie reruns of the eps = 0 fast paths: a counter and a list
  void* rerun = nullptr;
  if (dev_alloc(&rerun, 16 + nq * sizeof(uint64_t), st) != cudaSuccess) {
    cudaGetLastError();
    if (axes) cudaFreeAsync(axes, st);
    return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
  }
  a.rerun_count = static_cast<uint32_t*>(rerun);
  a.rerun_list = reinterpret_cast<uint64_t*>(static_cast<unsigned char*>(rerun) + 16);
  a.rerun_total = d_survivors ? d_survivors + 1 : nullptr;
  void* sort_mem = nullptr;
  if (nq >= ORDER_MIN_QUERIES && nq < 0xffffffffull) {
    const uint64_t words = 2 * nq + order_scratch_words(t);
    cudaError_t e = dev_alloc(&sort_mem, words * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
      uint32_t* leaf_of = static_cast<uint32_t*>(sort_mem);
      uint32_t* order = leaf_of + nq;
      order_by_landing_leaf(t, d_queries, nq, leaf_of, order, order + nq, st);
      a.order = order;
      a.leaf_of = leaf_of;
    } else {
      cudaGetLastError();  // run unordered: same results, less coherence
      sort_mem = nullptr;
    }
  }
  int rc = KD_OK;
  int path = qp.path;
  if (path == PATH_AUTO && traversal_timed(t, nq, qp)) {
    kd_tree* mt = const_cast<kd_tree*>(t);  // the choice is a cache on the tree
    std::lock_guard<std::mutex> lock(mt->choice_mutex);
    int& choice = mt->auto_traversal[(qp.k > 16 ? 2 : 0) + (nq >= TRAVERSAL_TIMED_SPLIT ? 1 : 0)];
    if (choice < 0) {
      rc = time_traversals(a, qp.metric, st, &choice);  // both write the same results
      path = -1;
    } else {
      path = choice == 1 ? PATH_PACKET : PATH_WARP;
    }
  }
  if (path >= 0) rc = run_kernels(a, qp.metric, st, path);
  if (axes) cudaFreeAsync(axes, st);
  cudaFreeAsync(rerun, st);
  if (sort_mem) cudaFreeAsync(sort_mem, st);
  return rc;
}

uint64_t query_scratch_bytes(uint64_t nq, uint64_t ndim) {
  // the larger use: CellBound axes (nq * ndim doubles) or the rerun list (nq u64)
  return std::max<uint64_t>(1, nq * std::max<uint64_t>(ndim, 1)) * sizeof(double);
}

int query_on_device_scratch(const kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp,
                            double* d_out_d, int64_t* d_out_i, cudaStream_t st, uint32_t* d_status,
                            void* d_scratch, uint32_t* d_rerun_count) {
  QArgs a = query_args(t, d_queries, nq, qp, d_out_d, d_out_i, d_status);
  // The one-thread kernels (the only users of the axes) never flag near ties,
  // and the kernels that flag them never use the axes: one region serves both.
  a.axes_scratch = static_cast<double*>(d_scratch);
  a.rerun_count = d_rerun_count;
  a.rerun_list = static_cast<uint64_t*>(d_scratch);
  return run_kernels(a, qp.metric, st, qp.path);
}

}  // namespace kd

extern "C" double kd_last_query_kernel_ms(void) {
  kd::KernelClock& c = kd::kernel_clock();
  if (!c.valid) return -1.0;
  float ms = 0.f;
  if (cudaEventSynchronize(c.e1) != cudaSuccess || cudaEventElapsedTime(&ms, c.e0, c.e1) != cudaSuccess) {
    cudaGetLastError();
    return -1.0;
  }
  return ms;
}
