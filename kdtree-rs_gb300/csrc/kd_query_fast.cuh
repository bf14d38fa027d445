// kd_query_fast.cuh -- the query kernel for compile-time widths (d in {2, 3, 8})
// and the L1 / L2 / L-inf metrics: the reference's descent with FP64 confined to
// the decisions that need it.  Included by kd_query.cu after its helpers.
//
// Every distance, plane bound and box distance the reference computes in FP64
// is carried here as an FP32 enclosure [lo, hi] of that exact FP64 value (see
// the interval helpers in kd_query.cu).  A comparison whose enclosures do not
// overlap is decided without FP64; an overlapping one computes the exact FP64
// values with the reference's operations and compares those.  Decisions are
// therefore always the reference's, while the common case runs on the FP32 and
// integer pipes:
//  - a leaf point is offered by its enclosure; its exact value is computed only
//    when an ordering or bound decision needs it, and once more for each final
//    result (the k best of every query, all lanes together);
//  - a rejected split-plane gate costs no FP64 (cell bound and axes carry
//    enclosures next to their exact values); entering a far child computes the
//    exact cell bound the reference would have.
#pragma once

// Frames of the fast descent: the cell bound (or saved axis) with its enclosure.
struct FFrame {
  uint32_t node;  // parent node id, or split dim (F_RESTORE)
  uint32_t kind;
  double x;       // parent cell_dist, or the saved axis value
  double y;       // pending child's box distance (F_BOX_*)
  float lo, hi;   // enclosure of x
};

template <int M, int D, int K>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_fast(QArgs a) {
  static_assert(D > 0 && M != M_LP, "fast path: compile-time width, metric without pow()");
  const uint64_t tid = blockIdx.x * static_cast<uint64_t>(QUERY_THREADS) + threadIdx.x;
  if (tid >= a.nq) return;
  const uint64_t qi = a.order ? a.order[tid] : tid;
  const int strat = S_PACKED;  // d <= 8 and metric in {L1, L2, L-inf} (kernel.rs:249-254)
  const bool gates = !a.use_eps;

  QVec<D> q;
  q.g = a.queries + qi * D;
  bool finite = true;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    q.v[i] = q.g[i];
    finite &= isfinite(q.v[i]);
  }
  if (!finite) {
    atomicOr(a.status, 1u);
    return;
  }
  float qlo[D], qhi[D];
#pragma unroll
  for (int i = 0; i < D; ++i) rn_enclose(__double2float_rn(q.v[i]), &qlo[i], &qhi[i]);

  // the k best, as enclosures of their exact distances
  LazyBest<M, D, K> best;
  best.init(a.k, a.cutoff, q.g, a.data, a.indices);
  const float& b_lo = best.b_lo;
  const float& b_hi = best.b_hi;
  auto bound_exact = [&]() -> uint64_t { return best.bound_exact(); };
  auto admits_at = [&](double dist, uint64_t bb) -> bool {
    if (a.use_eps) dist = dmul(dist, a.eps_factor);
    return leq_bound(dist, bb);
  };

  // scan_leaf (query.rs:343-353) with the Packed strategy (kernel.rs:277-292)
  auto scan_leaf = [&](uint32_t start, uint32_t end) {
    const uint32_t len = end - start;
    const uint32_t chunk_pts = (D == 8 && M != M_LINF) ? len / 8 * 8 : len;
    for (uint32_t j = 0; j < len; ++j) {
      const uint32_t row = start + j;
      float clo, chi;
      LazyBest<M, D, K>::point_enclosure(a.data32 + static_cast<uint64_t>(row) * D, qlo, qhi, &clo, &chi);
      if (clo > b_hi) continue;  // exact > bound: the reference does not offer it
      best.offer(clo, chi, row, j < chunk_pts);
    }
  };

  // CellBound axes (query.rs:156-211): exact values with enclosures
  double axes[D];
  float alo[D], ahi[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    axes[i] = 0.0;
    alo[i] = 0.f;
    ahi[i] = 0.f;
  }
  auto sel = [&](const auto* arr, uint32_t j) {
    auto v = arr[0];
#pragma unroll
    for (int i = 1; i < D; ++i) v = (static_cast<uint32_t>(i) == j) ? arr[i] : v;
    return v;
  };
  auto set_axis = [&](uint32_t j, double v, float lo, float hi) {
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const bool m = static_cast<uint32_t>(i) == j;
      axes[i] = m ? v : axes[i];
      alo[i] = m ? lo : alo[i];
      ahi[i] = m ? hi : ahi[i];
    }
  };

  // Descent::run (query.rs:223-232): CellBound::start seeds from the root box.
  double cell = 0.0;
  {
    const double rb = exact_box_dist<M, D>(q, a.boxes, D, 0.0);
    if (rb != 0.0) {
#pragma unroll
      for (int i = 0; i < D; ++i) {
        const double ax = reduce<M>(axis_offset(q[i], a.boxes[i], a.boxes[D + i]), 0.0);
        axes[i] = ax;
        alo[i] = mag_dn32(dbits(ax));
        ahi[i] = mag_up32(dbits(ax));
        cell = (M == M_LINF) ? max_nn(cell, ax) : dadd(cell, ax);
      }
    }
  }
  float cell_lo = rd32(dbits(cell)), cell_hi = ru32(dbits(cell));

  // Far-child box gate (query.rs:283) by enclosures, exact when they overlap.
  auto box_admits = [&](uint32_t id) -> bool {
    if (gates) {
      float lb, ub;
      box_enclosure<M, D>(a.boxes32 + static_cast<uint64_t>(id) * 2 * D, qlo, qhi, &lb, &ub);
      if (lb > b_hi) return false;
      if (ub < b_lo) return true;
    }
    const double bd = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(id) * 2 * D, D, 0.0);
    return admits_at(bd, bound_exact());
  };

  FFrame stack[2 * KD_MAX_DEPTH];
  int sp = 0;
  uint32_t node = 0;
  bool descending = admits_at(cell, bound_exact());

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
      const double qd = sel(q.v, dim);
      const bool left_near = ieee_key(dbits(qd)) <= ieee_key(dbits(nd.split));  // diff <= 0
      const uint32_t near = left_near ? node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : node + 1;
      if (nd.meta & KD_NODE_BOX_ORDER) {
        // descend_by_box (query.rs:298-327), exact
        const double near_box = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(near) * 2 * D, D, 0.0);
        const double far_box = exact_box_dist<M, D>(q, a.boxes + static_cast<uint64_t>(far) * 2 * D, D, 0.0);
        if (dbits(near_box) <= dbits(far_box)) {
          stack[sp++] = FFrame{node, F_BOX_FAR, cell, far_box, cell_lo, cell_hi};
          if (admits_at(near_box, bound_exact())) {
            node = near;
            continue;
          }
          descending = false;
          break;
        }
        stack[sp++] = FFrame{node, F_BOX_NEAR, cell, near_box, cell_lo, cell_hi};
        if (admits_at(far_box, bound_exact())) {
          const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), 0.0);
          const double old = sel(axes, dim);
          const double far_dist = (M == M_LINF) ? max_nn(cell, far_axis) : dadd(dsub(cell, old), far_axis);
          stack[sp++] = FFrame{dim, F_RESTORE, old, 0.0, sel(alo, dim), sel(ahi, dim)};
          set_axis(dim, far_axis, mag_dn32(dbits(far_axis)), mag_up32(dbits(far_axis)));
          node = far;
          cell = far_dist;
          cell_lo = rd32(dbits(far_dist));
          cell_hi = ru32(dbits(far_dist));
          continue;
        }
        descending = false;
        break;
      }
      stack[sp++] = FFrame{node, F_FAR, cell, 0.0, cell_lo, cell_hi};
      node = near;  // near child keeps the parent's cell bound
    }
    // unwind to the next pending far-child decision
    bool resumed = false;
    while (sp > 0 && !resumed) {
      const FFrame f = stack[--sp];
      if (f.kind == F_RESTORE) {
        set_axis(f.node, f.x, f.lo, f.hi);
        continue;
      }
      const DNode nd = a.nodes[f.node];
      const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
      const double qd = sel(q.v, dim);
      const bool left_near = ieee_key(dbits(qd)) <= ieee_key(dbits(nd.split));
      const uint32_t near = left_near ? f.node + 1 : nd.right;
      const uint32_t far = left_near ? nd.right : f.node + 1;
      if (f.kind == F_BOX_NEAR) {
        if (admits_at(f.y, bound_exact())) {
          node = near;
          cell = f.x;
          cell_lo = f.lo;
          cell_hi = f.hi;
          resumed = true;
        }
        continue;
      }
      bool enter;
      if (f.kind == F_BOX_FAR) {
        enter = admits_at(f.y, bound_exact());
      } else if (gates) {
        // plane gate on enclosures: far_dist = (cell - old) + reduce(|q - split|)
        const float slo_ = rd32(dbits(nd.split)), shi_ = ru32(dbits(nd.split));
        const float qlo_d = sel(qlo, dim), qhi_d = sel(qhi, dim);
        // enclosure of reduce(|fl(q - split)|): FP64 rounding of the difference and the square
        const float fa_lo = __fmul_rd(red_lb<M>(absdiff_lb(qlo_d, qhi_d, slo_, shi_)), LB_SHRINK);
        const float fa_hi = __fmul_ru(red_ub<M>(absdiff_ub(qlo_d, qhi_d, slo_, shi_)), UB_GROW);
        float far_lo, far_hi;
        if (M == M_LINF) {
          far_lo = fmaxf(f.lo, fa_lo);
          far_hi = fmaxf(f.hi, fa_hi);
        } else {
          // c = fl(cell - old): real difference of the enclosures, widened by
          // one rounding; then fl(c + far_axis) widened by 2^-20.
          float c_lo = __fsub_rd(f.lo, sel(ahi, dim)), c_hi = __fsub_ru(f.hi, sel(alo, dim));
          const float err = __fmul_ru(fmaxf(fabsf(c_lo), fabsf(c_hi)), 2.220446e-16f /* 2^-52 */);
          c_lo = __fsub_rd(c_lo, err);
          c_hi = __fadd_ru(c_hi, err);
          const float s = __fadd_rd(c_lo, fa_lo), t = __fadd_ru(c_hi, fa_hi);
          far_lo = s >= 0.f ? __fmul_rd(s, LB_SHRINK) : __fmul_rd(s, UB_GROW);
          far_hi = t >= 0.f ? __fmul_ru(t, UB_GROW) : __fmul_ru(t, LB_SHRINK);
        }
        if (far_lo > b_hi) continue;  // the reference prunes the far child
        bool plane_ok = far_hi < b_lo;
        if (!plane_ok) {
          const double old = sel(axes, dim);
          const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), 0.0);
          const double far_dist = (M == M_LINF) ? max_nn(f.x, far_axis) : dadd(dsub(f.x, old), far_axis);
          plane_ok = leq_bound(far_dist, bound_exact());
        }
        enter = plane_ok && box_admits(far);
      } else {
        const double old = sel(axes, dim);
        const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), 0.0);
        const double far_dist = (M == M_LINF) ? max_nn(f.x, far_axis) : dadd(dsub(f.x, old), far_axis);
        const uint64_t bb = bound_exact();
        enter = admits_at(far_dist, bb) && box_admits(far);
      }
      if (enter) {
        // enter_far (query.rs:329-341): the exact cell bound of the far child
        const double old = sel(axes, dim);
        const double far_axis = reduce<M>(fabs(dsub(qd, nd.split)), 0.0);
        const double far_dist = (M == M_LINF) ? max_nn(f.x, far_axis) : dadd(dsub(f.x, old), far_axis);
        stack[sp++] = FFrame{dim, F_RESTORE, old, 0.0, sel(alo, dim), sel(ahi, dim)};
        set_axis(dim, far_axis, mag_dn32(dbits(far_axis)), mag_up32(dbits(far_axis)));
        node = far;
        cell = far_dist;
        cell_lo = rd32(dbits(far_dist));
        cell_hi = ru32(dbits(far_dist));
        resumed = true;
      }
    }
    if (!resumed) break;
    descending = true;
  }

  // write_results (query.rs:421-429, 483-493): exact values of the k best
  best.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.k, a.n_points);
}
