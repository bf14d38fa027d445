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

#include "kd_internal.hpp"

namespace kd {

namespace {

constexpr uint32_t NO_ID = 0xffffffffu;
constexpr uint64_t INF_BITS = 0x7ff0000000000000ull;
constexpr int QUERY_THREADS = 128;

struct QArgs {
  const double* data;     // tree order, n * d
  const float* data32;    // FP32 copy
  const uint32_t* indices;
  const DNode* nodes;
  const double* boxes;    // [lo | hi] per node
  const float* boxes32;   // outward-rounded FP32 boxes
  const double* queries;  // nq * d
  double* out_d;          // nq * k
  int64_t* out_i;         // nq * k
  double* axes_scratch;   // nq * d, dynamic-d CellBound (unused for static d)
  uint32_t* status;       // bit 0: non-finite query
  uint64_t nq;
  uint64_t d;
  uint64_t k;
  uint64_t n_points;
  double p;               // LP exponent
  double cutoff;          // reduced max_distance, >= +0
  double eps_factor;
  int use_eps;            // eps_factor != 1
};

// ---------------------------------------------------------------------------
// Metric algebra (src/metric.rs:64-98), exact.
// ---------------------------------------------------------------------------
template <int M>
__device__ __forceinline__ double reduce(double x, double p) {
  if (M == M_L2) return dmul(x, x);
  if (M == M_LP) return pow(x, p);
  return x;
}
template <int M>
__device__ __forceinline__ double restore(double x, double p) {
  if (M == M_L2) return __dsqrt_rn(x);
  if (M == M_LP) return pow(x, 1.0 / p);
  return x;
}
template <int M>
__device__ __forceinline__ double axis_of(double delta) {  // axes_lanes (kernel.rs:22-29)
  return M == M_L2 ? dmul(delta, delta) : fabs(delta);
}
__device__ __forceinline__ double hsum8(const double* v) {  // src/simd.rs:26-30
  return dadd(dadd(dadd(v[0], v[4]), dadd(v[2], v[6])), dadd(dadd(v[1], v[5]), dadd(v[3], v[7])));
}
__device__ __forceinline__ double max_nn(double a, double b) { return b > a ? b : a; }
// axis_offset (src/layout.rs:147-149)
__device__ __forceinline__ double axis_offset(double q, double lo, double hi) {
  double a = dsub(lo, q), b = dsub(q, hi);
  double m = a > b ? a : b;
  return m > 0.0 ? m : 0.0;
}

// Query coordinates: registers for a compile-time width, global otherwise.
template <int D>
struct QVec {
  double v[D > 0 ? D : 1];
  const double* g;
  __device__ __forceinline__ double operator[](uint64_t i) const {
    if (D > 0) return v[i];
    return g[i];
  }
};

// ---------------------------------------------------------------------------
// Exact reduced point distance (src/kernel.rs:163-218, 343-354, 411-562).
// `in_chunk`: the point lies inside a full Packed chunk of its leaf (d4: pairs,
// d8: groups of 8); only then do d4 / d8 use their pairwise orders.
// ---------------------------------------------------------------------------
template <int M, int D>
__device__ __forceinline__ double exact_dist(const QVec<D>& q, const double* p, uint64_t d, int strat, bool in_chunk,
                                             double pexp) {
  if (M == M_LP) {
    double dist = 0.0;
    for (uint64_t i = 0; i < d; ++i) dist = dadd(dist, pow(fabs(dsub(q[i], p[i])), pexp));
    return dist;
  }
  if (M == M_LINF) {
    double dist = 0.0;
    if (D > 0) {
#pragma unroll
      for (int i = 0; i < D; ++i) dist = max_nn(dist, fabs(dsub(q[i], p[i])));
    } else {
      for (uint64_t i = 0; i < d; ++i) dist = max_nn(dist, fabs(dsub(q[i], p[i])));
    }
    return dist;
  }
  if (D > 0) {
    if (D == 4 && in_chunk) {
      double a0 = axis_of<M>(dsub(p[0], q[0])), a1 = axis_of<M>(dsub(p[1], q[1]));
      double a2 = axis_of<M>(dsub(p[2], q[2])), a3 = axis_of<M>(dsub(p[3], q[3]));
      return dadd(dadd(a0, a2), dadd(a1, a3));
    }
    if (D == 8 && in_chunk) {
      double a[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = axis_of<M>(dsub(p[i], q[i]));
      return dadd(dadd(dadd(a[0], a[1]), dadd(a[2], a[3])), dadd(dadd(a[4], a[5]), dadd(a[6], a[7])));
    }
    double dist = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) dist = dadd(dist, axis_of<M>(dsub(q[i], p[i])));
    return dist;
  }
  if (strat == S_PACKED) {
    if (d == 4 && in_chunk) {
      double a0 = axis_of<M>(dsub(p[0], q[0])), a1 = axis_of<M>(dsub(p[1], q[1]));
      double a2 = axis_of<M>(dsub(p[2], q[2])), a3 = axis_of<M>(dsub(p[3], q[3]));
      return dadd(dadd(a0, a2), dadd(a1, a3));
    }
    if (d == 8 && in_chunk) {
      double a[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = axis_of<M>(dsub(p[i], q[i]));
      return dadd(dadd(dadd(a[0], a[1]), dadd(a[2], a[3])), dadd(dadd(a[4], a[5]), dadd(a[6], a[7])));
    }
    double dist = 0.0;
    for (uint64_t i = 0; i < d; ++i) dist = dadd(dist, axis_of<M>(dsub(q[i], p[i])));
    return dist;
  }
  const uint64_t nch = d / LANES;
  double dist = 0.0;
  if (strat == S_FOLDED) {
    double acc[LANES] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint64_t c = 0; c < nch; ++c)
#pragma unroll
      for (int j = 0; j < LANES; ++j) acc[j] = dadd(acc[j], axis_of<M>(dsub(q[c * LANES + j], p[c * LANES + j])));
    dist = nch ? hsum8(acc) : 0.0;
  } else {
    for (uint64_t c = 0; c < nch; ++c) {
      double v[LANES];
#pragma unroll
      for (int j = 0; j < LANES; ++j) v[j] = axis_of<M>(dsub(q[c * LANES + j], p[c * LANES + j]));
      dist = dadd(dist, hsum8(v));
    }
  }
  for (uint64_t i = nch * LANES; i < d; ++i) dist = dadd(dist, axis_of<M>(dsub(q[i], p[i])));
  return dist;
}

// Exact box distance (src/kernel.rs:565-616).
template <int M, int D>
__device__ __forceinline__ double exact_box_dist(const QVec<D>& q, const double* box, uint64_t d, double pexp) {
  const double* lo = box;
  const double* hi = box + d;
  if (M == M_LINF) {
    double worst = 0.0;
    for (uint64_t i = 0; i < d; ++i) worst = max_nn(worst, axis_offset(q[i], lo[i], hi[i]));
    return worst;
  }
  if (M == M_LP) {
    double dist = 0.0;
    for (uint64_t i = 0; i < d; ++i) {
      double off = axis_offset(q[i], lo[i], hi[i]);
      if (off > 0.0) dist = dadd(dist, pow(off, pexp));
    }
    return dist;
  }
  const uint64_t nch = d / LANES;
  double dist = 0.0;
  if (nch) {
    double acc[LANES] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint64_t c = 0; c < nch; ++c)
#pragma unroll
      for (int j = 0; j < LANES; ++j) {
        uint64_t i = c * LANES + j;
        double off = max_nn(max_nn(dsub(lo[i], q[i]), dsub(q[i], hi[i])), 0.0);
        acc[j] = dadd(acc[j], axis_of<M>(off));
      }
    dist = hsum8(acc);
  }
  for (uint64_t i = nch * LANES; i < d; ++i) dist = dadd(dist, reduce<M>(axis_offset(q[i], lo[i], hi[i]), pexp));
  return dist;
}

// ---------------------------------------------------------------------------
// FP32 lower bounds with directed rounding.  data32 = RN(p) and q32 = RN(q)
// satisfy |p - p32| <= 2^-24 |p32| + 2^-150 (likewise q), so per axis
//   |p - q| >= |p32 - q32| - e,   e = 2^-24 (|p32| + |q32|) + 2^-149,
// and every FP32 operation below rounds toward the safe side; non-finite FP32
// values (overflowing inputs) collapse to a zero contribution.  The caller
// rejects only when this bound exceeds an FP32 upper bound of the FP64 pruning
// bound divided by (1 - 2^-40), which covers the FP64 rounding of the exact
// distance (at most d + 2 relative roundings of 2^-53 each).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float axis_lb32(float p32, float q32) {
  float hi = __fsub_ru(p32, q32), lo = __fsub_rd(p32, q32);
  float a = lo > 0.f ? lo : (hi < 0.f ? -hi : 0.f);  // lower bound of |p32 - q32|
  float e = __fadd_ru(__fmul_ru(__fadd_ru(fabsf(p32), fabsf(q32)), 5.9604645e-08f /* 2^-24 */),
                      1.4e-45f /* 2^-149 */);
  float t = __fsub_rd(a, e);
  return t > 0.f ? t : 0.f;  // NaN (inf - inf) also lands on 0
}

template <int M>
__device__ __forceinline__ float acc_lb32(float acc, float t) {
  if (M == M_L2) return __fadd_rd(acc, __fmul_rd(t, t));
  if (M == M_L1) return __fadd_rd(acc, t);
  return acc > t ? acc : t;  // LINF
}

// FP32 upper bound of a non-negative FP64 bound, inflated so that rejecting
// lb32 > ub32 implies exact_fp64 > bound.  +inf stays +inf (never rejects).
__device__ __forceinline__ float bound_ub32(double b) {
  float f = __double2float_ru(b);
  return __fmul_ru(f, 1.0000002f);
}

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
  const uint64_t qi = blockIdx.x * static_cast<uint64_t>(QUERY_THREADS) + threadIdx.x;
  if (qi >= a.nq) return;
  const uint64_t d = D > 0 ? D : a.d;
  const double pexp = a.p;
  const int strat = (M != M_LP && d <= 8) ? S_PACKED : ((M == M_L1 || M == M_L2) && d <= 16 ? S_FOLDED : S_STREAMED);

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
  // FP32 copy of the query for the filters (static widths only)
  float q32[D > 0 ? D : 1];
  if (D > 0) {
#pragma unroll
    for (int i = 0; i < D; ++i) q32[i] = __double2float_rn(q.v[i]);
  }

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
  best.reset(a.k);
  auto bound_bits = [&]() -> uint64_t {
    uint64_t w = best.worst();
    return w < cutoff_bits ? w : cutoff_bits;
  };
  auto admits_at = [&](double dist, uint64_t bnd) -> bool {
    if (a.use_eps) dist = dmul(dist, a.eps_factor);
    return dbits(dist) <= bnd;  // NaN bit patterns sort above +inf: never admitted
  };

  // Box gate: FP32 lower bound first; exact FP64 box distance only if needed.
  auto box_admits = [&](uint32_t id, uint64_t bnd) -> bool {
    if (D > 0 && M != M_LP) {
      const float* b32 = a.boxes32 + static_cast<uint64_t>(id) * 2 * D;
      float lb = 0.f;
#pragma unroll
      for (int i = 0; i < D; ++i) {
        // offset lower bound: max(lo - q, q - hi, 0) with lo / hi rounded outward
        float o1 = __fsub_rd(b32[i], q32[i]);
        float o2 = __fsub_rd(q32[i], b32[D + i]);
        float o = o1 > o2 ? o1 : o2;
        o = o > 0.f ? o : 0.f;
        float e = __fmul_ru(fabsf(q32[i]), 5.9604645e-08f);
        o = __fsub_rd(o, e);
        o = o > 0.f ? o : 0.f;
        lb = acc_lb32<M>(lb, o);
      }
      float ub = bound_ub32(bitsd(bnd));
      if (a.use_eps) ub = __fdiv_ru(ub, __double2float_rd(a.eps_factor));
      if (lb > ub) return false;
    }
    double bd = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(id) * 2 * d, d, pexp);
    return admits_at(bd, bnd);
  };

  // scan_leaf + Strategy::scan + LeafSink (query.rs:343-375, kernel.rs:366-562)
  auto scan_leaf = [&](uint32_t start, uint32_t end) {
    uint64_t bnd = bound_bits();
    const uint32_t len = end - start;
    uint32_t chunk_pts = len;
    if (strat == S_PACKED && M != M_LINF) {
      if (d == 4) chunk_pts = len / 2 * 2;
      else if (d == 8) chunk_pts = len / 8 * 8;
    }
    float ub = bound_ub32(bitsd(bnd));
    for (uint32_t j = 0; j < len; ++j) {
      const uint64_t row = static_cast<uint64_t>(start) + j;
      if (D > 0 && M != M_LP) {
        const float* p32 = a.data32 + row * D;
        float lb = 0.f;
#pragma unroll
        for (int i = 0; i < D; ++i) lb = acc_lb32<M>(lb, axis_lb32(p32[i], q32[i]));
        if (lb > ub) continue;  // exact distance > bound: never offered
      }
      double dist = exact_dist<M, D>(q, a.data + row * d, d, strat, j < chunk_pts, pexp);
      if (dbits(dist) <= bnd) {
        best.consider(dbits(dist), a.indices[row]);
        bnd = bound_bits();
        ub = bound_ub32(bitsd(bnd));
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
  bool descending = admits_at(seed, bound_bits());

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
      const double diff = dsub(q[dim], nd.split);
      const bool left_near = diff <= 0.0;
      const uint32_t near = left_near ? node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : node + 1;
      if (nd.meta & KD_NODE_BOX_ORDER) {
        // descend_by_box (query.rs:298-327)
        double near_box = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(near) * 2 * d, d, pexp);
        double far_box = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(far) * 2 * d, d, pexp);
        if (dbits(near_box) <= dbits(far_box)) {
          stack[sp++] = Frame{node, F_BOX_FAR, cell, far_box};
          if (admits_at(near_box, bound_bits())) {
            node = near;
            continue;
          }
          descending = false;
          break;
        }
        stack[sp++] = Frame{node, F_BOX_NEAR, cell, near_box};
        if (admits_at(far_box, bound_bits())) {
          const double far_axis = reduce<M>(fabs(diff), pexp);
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
      const double diff = dsub(q[dim], nd.split);
      const bool left_near = diff <= 0.0;
      const uint32_t near = left_near ? f.node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : f.node + 1;
      if (f.kind == F_BOX_NEAR) {
        if (admits_at(f.y, bound_bits())) {
          node = near;
          cell = f.x;
          resumed = true;
        }
        continue;
      }
      const uint64_t bnd = bound_bits();
      const double far_axis = reduce<M>(fabs(diff), pexp);
      const double old = axis_get(dim);
      const double far_dist = (M == M_LINF) ? max_nn(f.x, far_axis) : dadd(dsub(f.x, old), far_axis);
      bool enter;
      if (f.kind == F_BOX_FAR)
        enter = admits_at(f.y, bnd);
      else
        enter = admits_at(far_dist, bnd) && box_admits(far, bnd);
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

template <int M, int D, int K>
int launch(const QArgs& a, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((a.nq + QUERY_THREADS - 1) / QUERY_THREADS);
  k_query<M, D, K><<<blocks, QUERY_THREADS, 0, st>>>(a);
  KD_TRY_CUDA(cudaGetLastError());
  return KD_OK;
}

template <int M, int D>
int dispatch_k(const QArgs& a, cudaStream_t st) {
  if (a.k == 1) return launch<M, D, 1>(a, st);
  if (a.k <= 4) return launch<M, D, 4>(a, st);
  if (a.k <= 8) return launch<M, D, 8>(a, st);
  if (a.k <= 16) return launch<M, D, 16>(a, st);
  if (a.k <= 32) return launch<M, D, 32>(a, st);
  return fail(KD_ERR_INVALID_ARGUMENT, "k > 32 is not supported by this query path");
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

}  // namespace

int query_on_device(const kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp,
                    double* d_out_d, int64_t* d_out_i, cudaStream_t st, uint32_t* d_status) {
  QArgs a{};
  a.data = t->data;
  a.data32 = t->data32;
  a.indices = t->indices;
  a.nodes = t->nodes;
  a.boxes = t->boxes;
  a.boxes32 = t->boxes32;
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
  void* axes = nullptr;
  const bool dyn = !(qp.metric != M_LP && (t->ndim == 2 || t->ndim == 3 || t->ndim == 8));
  if (dyn) {
    cudaError_t e = cudaMallocAsync(&axes, std::max<uint64_t>(1, nq * t->ndim) * sizeof(double), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
    }
    a.axes_scratch = static_cast<double*>(axes);
  }
  int rc;
  switch (qp.metric) {
    case M_L1: rc = dispatch_d<M_L1>(a, st); break;
    case M_L2: rc = dispatch_d<M_L2>(a, st); break;
    case M_LINF: rc = dispatch_d<M_LINF>(a, st); break;
    default: rc = dispatch_d<M_LP>(a, st); break;
  }
  if (axes) cudaFreeAsync(axes, st);
  return rc;
}

int query_on_device_scratch(const kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp,
                            double* d_out_d, int64_t* d_out_i, cudaStream_t st, uint32_t* d_status,
                            double* d_axes_scratch) {
  QArgs a{};
  a.data = t->data;
  a.data32 = t->data32;
  a.indices = t->indices;
  a.nodes = t->nodes;
  a.boxes = t->boxes;
  a.boxes32 = t->boxes32;
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
  a.axes_scratch = d_axes_scratch;
  switch (qp.metric) {
    case M_L1: return dispatch_d<M_L1>(a, st);
    case M_L2: return dispatch_d<M_L2>(a, st);
    case M_LINF: return dispatch_d<M_LINF>(a, st);
    default: return dispatch_d<M_LP>(a, st);
  }
}

}  // namespace kd
