// kd_query_packet.cuh -- exact k-NN by packet traversal (eps = 0, compile-time
// widths, L1 / L2 / L-inf).  Included by kd_query.cu.
//
// The 32 queries of a warp -- neighbours, since the batch is sorted by landing
// leaf -- walk ONE depth-first traversal together: every lane holds the same
// node stack, so control flow is uniform and the stack accesses coalesce.  A
// node is entered when at least one lane's rigorous FP32 lower bound of the
// exact box distance does not exceed that lane's pruning bound; its children are
// visited near side first by majority vote.  At a leaf every lane that needs it
// offers each point to its own k-best list (LazyBest: FP32 enclosures of the
// reference's exact FP64 distances, exact FP64 only when enclosures overlap).
//
// Each lane's result is the k smallest (exact FP64 reduced distance in the
// reference's summation order, original index) among the points within
// max_distance: every pruned subtree's points exceed that lane's bound, and the
// list keeps exactly those k in order whatever the order of the offers.  That is
// the reference's result for eps = 0 (its answer does not depend on the visiting
// order) except where the reference's own FP64 plane bound rounds above a point's
// exact distance that also sits within rounding error of the k-th distance.  With
// eps > 0 the result depends on the visiting order and the reference-order
// descent (k_query_fast) is used instead.
#pragma once

constexpr int PACKET_STACK = 2 * KD_MAX_DEPTH;

template <int M, int D, int K>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_packet(QArgs a) {
  static_assert(D > 0 && M != M_LP, "packet path: compile-time width, metric without pow()");
  const uint64_t tid = blockIdx.x * static_cast<uint64_t>(QUERY_THREADS) + threadIdx.x;
  const bool in_range = tid < a.nq;
  const uint64_t qi = in_range ? (a.order ? a.order[tid] : tid) : 0;
  // Lanes past the batch end (or with a non-finite query) stay in the warp for
  // the ballots but never need a node.
  QVec<D> q;
  q.g = a.queries + qi * D;
  bool live = in_range;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    q.v[i] = in_range ? q.g[i] : 0.0;
    live &= isfinite(q.v[i]);
  }
  if (in_range && !live) atomicOr(a.status, 1u);
  if (!live) {
#pragma unroll
    for (int i = 0; i < D; ++i) q.v[i] = 0.0;
  }
  float qlo[D], qhi[D];
  uint64_t qkey[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    rn_enclose(__double2float_rn(q.v[i]), &qlo[i], &qhi[i]);
    qkey[i] = ieee_key(dbits(q.v[i]));
  }

  LazyBest<M, D, K> best;
  best.init(a.k, a.cutoff, &q, a.data, a.indices);

  uint32_t stack[PACKET_STACK];  // identical in every lane
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const uint32_t node = stack[--sp];
    const float lb = box_lb<M, D>(a.boxes32 + static_cast<uint64_t>(node) * 2 * D, qlo, qhi);
    const bool need = live && !(lb > best.b_hi);
    const uint32_t need_mask = __ballot_sync(0xffffffffu, need);
    if (!need_mask) continue;  // every lane's points there exceed its bound
    const DNode nd = a.nodes[node];
    if (nd.meta & KD_NODE_LEAF) {
      const uint64_t se = dbits(nd.split);
      const uint32_t start = static_cast<uint32_t>(se), end = static_cast<uint32_t>(se >> 32);
      const uint32_t chunk_end = (D == 8 && M != M_LINF) ? start + (end - start) / 8 * 8 : end;
      for (uint32_t r = start; r < end; ++r) {
        float clo, chi;
        LazyBest<M, D, K>::point_enclosure(a.data32 + static_cast<uint64_t>(r) * D, qlo, qhi, &clo, &chi);
        if (need && !(clo > best.b_hi)) best.offer(clo, chi, r, r < chunk_end);
      }
      continue;
    }
    // near child first, by majority of the lanes that need this node
    const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
    uint64_t qk = qkey[0];
#pragma unroll
    for (int i = 1; i < D; ++i) qk = (static_cast<uint32_t>(i) == dim) ? qkey[i] : qk;
    const bool left = qk <= ieee_key(dbits(nd.split));
    const uint32_t left_votes = __popc(__ballot_sync(0xffffffffu, need && left));
    const bool left_first = 2 * left_votes >= static_cast<uint32_t>(__popc(need_mask));
    stack[sp++] = left_first ? nd.right : node + 1;
    stack[sp++] = left_first ? node + 1 : nd.right;
  }
  if (live) best.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.k, a.n_points);
}
