// kd_query_packet.cuh -- exact k-NN by packet traversal (eps = 0, compile-time
// widths, L1 / L2 / L-inf).  Included by kd_query.cu.
//
// The 32 queries of a warp -- neighbours, since the batch is sorted by landing
// leaf -- walk ONE depth-first traversal together: every lane holds the same
// node stack (one copy per warp, in shared memory), so control flow is uniform.  A
// node is entered when at least one lane's rigorous FP32 lower bound of the
// exact box distance does not exceed that lane's pruning bound; its children are
// visited near side first by majority vote.  At a leaf every lane that needs it
// offers each point to its own k-best set (LazySet: FP32 enclosures of the
// reference's exact FP64 distances, exact FP64 only when enclosures overlap).
//
// Each lane's result is the k smallest (exact FP64 reduced distance in the
// reference's summation order, original index) among the points within
// max_distance: every pruned subtree's points exceed that lane's bound, and the
// list keeps exactly those k in order whatever the order of the offers.  That is
// the reference's result for eps = 0 except where one of the reference's own
// FP64 gates rounds above the distance of a point that ties the k-th distance
// or the cutoff; such near ties are detected (kd_warp.cuh) and those queries
// run again in the reference's order.  With eps > 0 the result depends on the
// visiting order and the reference-order kernels are used instead.
#pragma once

constexpr int PACKET_STACK = 2 * KD_MAX_DEPTH;

// Work counters of the measurement build (KD_WORK_COUNTS; kd_work_counts reads
// them): what the warps of this translation unit's packet traversals did.
//   0 warps, 1 live queries, 2 seed-leaf rows (per query), 3 node pops (per
//   warp), 4 nodes entered (per warp), 5 lane-nodes needed (sum over entered
//   nodes of the lanes that need them), 6 leaves scanned (per warp), 7 rows
//   scanned (per warp: every lane evaluates them), 8 lane-rows needed, 9 rows
//   offered or noted after the filter (per query), 10 offers (per query)
//   11..15: SM clock cycles of each phase, summed over warps (lane 0 reads
//   clock64 at the phase boundaries, the warp synchronised there): 11 setup
//   and seed leaf, 12 node steps, 13 leaf filter rounds, 14 offers, 15 sort
//   and write.
// Each thread adds into its own 32-bit counters (registers) and flushes them
// with one atomic each when its queries are done, so the counting does not
// contend on the global counters inside the phases it times.
#ifdef KD_WORK_COUNTS
__device__ unsigned long long g_work[16];
#define KD_WORK(i, v) (kd_acc_[i] += static_cast<uint32_t>(v))
#define KD_PHASE(i)                                          \
  do {                                                       \
    __syncwarp();                                            \
    const long long kd_now_ = clock64();                     \
    if ((threadIdx.x & 31) == 0) KD_WORK(i, kd_now_ - kd_t_); \
    kd_t_ = kd_now_;                                         \
  } while (0)
#define KD_WORK_FLUSH()                                                                    \
  do {                                                                                     \
    _Pragma("unroll") for (int kd_i_ = 0; kd_i_ < 16; ++kd_i_) if (kd_acc_[kd_i_])         \
        atomicAdd(&g_work[kd_i_], static_cast<unsigned long long>(kd_acc_[kd_i_]));         \
  } while (0)
#else
#define KD_WORK(i, v) ((void)0)
#define KD_PHASE(i) ((void)0)
#define KD_WORK_FLUSH() ((void)0)
#endif

// Cheap rigorous point filter.  With a = p32 - q32 (exact reals) and every
// coordinate within E = 2^-24 (|coordinate bound| + |q|) + 2^-148 of its FP32
// copy, the triangle inequality gives |p - q| >= |a| - sqrt(d) E (L2; d E for L1,
// E for L-inf), and the round-to-nearest FP32 sum s over-estimates |a| (squared
// for L2) by at most (d + 3) 2^-24 relative.  So s > T(b) with g the larger of
// 1 + 2^-20 and 1 + (d + 4) 2^-24 (GROW),
//   T(b) = g (sqrt(b) + sqrt(d) E)^2 + d 2^-148   (L2),
//   T(b) = g (b + d E) + d 2^-148                (L1),
//   T(b) = g (b + E) + 2^-148                    (L-inf),
// all rounded up, proves the exact distance exceeds b.  NaN never rejects.
// An FP32 upper bound of sqrt(b) from the hardware reciprocal square root:
// b * rsqrtf(b) is within 3 units in the last place of sqrt(b) (rsqrtf: 2,
// the product: 1/2), so growing it by 2^-19 and rounding up covers it (a
// directed-rounding square root is a long instruction sequence).
__device__ __forceinline__ float sqrt_up(float b) {
  if (!(b > 0.f)) return 0.f;
  if (!(b <= 3.4e38f)) return b;  // +inf (or larger than any finite bound)
  return __fmul_ru(b * rsqrtf(b), 1.0000020f /* 1 + 2^-19 */);
}

template <int M, int D>
struct PointFilter {
  static constexpr float GROW = D + 3 <= 16 ? UB_GROW : 1.0f + (D + 4) * TWO_M24;
  float q32[D];
  float spread;
  __device__ __forceinline__ void init(const QVec<D>& q, float coord_max) {
    float qmax = 0.f;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      q32[i] = __double2float_rn(q.v[i]);
      qmax = fmaxf(qmax, fabsf(q32[i]));
    }
    const float e = __fmaf_ru(__fadd_ru(coord_max, qmax), TWO_M24, 2.9e-45f /* 2^-148 */);
    spread = (M == M_L2) ? __fmul_ru(e, __fsqrt_ru(static_cast<float>(D)))
                         : (M == M_L1 ? __fmul_ru(e, static_cast<float>(D)) : e);
  }
  __device__ __forceinline__ float threshold(float b) const {
    constexpr float abs_slack = D * 2.9e-45f;
    if (M == M_L2) {
      const float r = __fadd_ru(sqrt_up(b), spread);
      return __fadd_ru(__fmul_ru(__fmul_ru(r, r), GROW), abs_slack);
    }
    return __fadd_ru(__fmul_ru(__fadd_ru(b, spread), GROW), abs_slack);
  }
  // Enclosure [clo, chi] of the exact FP64 distance from the same sum s: |a|
  // within 2^-19 of s * rsqrt(s) (rsqrtf: 2 ulp; s: (d + 3) 2^-24), then the
  // spread and the FP64 roundings, as above.
  __device__ __forceinline__ void enclose(float s, float* clo, float* chi) const {
    float lo, hi;
    if (M == M_L2) {
      const float r = s > 0.f ? s * rsqrtf(s) : 0.f;
      if (!(r <= 3.4e38f)) {  // overflow or NaN: no information
        *clo = 0.f;
        *chi = __int_as_float(0x7f800000);
        return;
      }
      lo = fmaxf(__fsub_rd(__fmul_rd(r, 0.99999809f /* 1 - 2^-19 */), spread), 0.f);
      hi = __fadd_ru(__fmul_ru(r, 1.0000020f /* 1 + 2^-19 */), spread);
      lo = __fmul_rd(lo, lo);
      hi = __fmul_ru(hi, hi);
    } else {
      lo = fmaxf(__fsub_rd(__fmul_rd(s, 0.99999809f), spread), 0.f);
      hi = __fadd_ru(__fmul_ru(s, 1.0000020f), spread);
      if (!(s <= 3.4e38f)) hi = __int_as_float(0x7f800000);
    }
    *clo = __fmul_rd(lo, LB_SHRINK);
    *chi = __fmul_ru(hi, UB_GROW);
  }
  // FP32 reduced distance of the row at p32, summed in dimension order.  The
  // FP32 copy starts on an allocation boundary, so rows of a width divisible
  // by 4 (2) are 16 (8) byte aligned and load as vectors: a quarter (half)
  // of the load instructions.  Width 3 reads the copy padded to 4 floats
  // (filter_rows): one 16-byte load.
  __device__ __forceinline__ float sum(const float* p32) const {
    float p[D];
    load(p32, p);
    return reduce_of(p, q32);
  }
  // The FP32 reduced distance of the loaded row p to the FP32 query q, in
  // dimension order: every filter sum of the packet traversal is this one
  // sequence of operations, so two evaluations of a (row, query) agree.
  static __device__ __forceinline__ float reduce_of(const float (&p)[D], const float (&q)[D]) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const float t = __fsub_rn(p[i], q[i]);
      if (M == M_L2) s = __fmaf_rn(t, t, s);
      else if (M == M_L1) s = __fadd_rn(s, fabsf(t));
      else s = fmaxf(s, fabsf(t));
    }
    return s;
  }
  // The row at p32 loaded (widths: as sum)
  static __device__ __forceinline__ void load(const float* p32, float (&p)[D]) {
    if constexpr (D == 3) {
      const float4 v = *reinterpret_cast<const float4*>(p32);
      p[0] = v.x;
      p[1] = v.y;
      p[2] = v.z;
    } else if constexpr (D % 4 == 0) {
#pragma unroll
      for (int c = 0; c < D / 4; ++c) {
        const float4 v = reinterpret_cast<const float4*>(p32)[c];
        p[4 * c] = v.x;
        p[4 * c + 1] = v.y;
        p[4 * c + 2] = v.z;
        p[4 * c + 3] = v.w;
      }
    } else if constexpr (D % 2 == 0) {
#pragma unroll
      for (int c = 0; c < D / 2; ++c) {
        const float2 v = reinterpret_cast<const float2*>(p32)[c];
        p[2 * c] = v.x;
        p[2 * c + 1] = v.y;
      }
    } else {
#pragma unroll
      for (int i = 0; i < D; ++i) p[i] = p32[i];
    }
  }
};

// The band above a bound b inside which a point the filter drops still counts
// for the near-tie test: points with s > threshold(band_of(b)) are farther
// than (1 + 2^-19) b.
__device__ __forceinline__ float band_of(float b) { return __fmul_ru(b, 1.0000020f /* 1 + 2^-19 */); }

// Shared memory of one block: the warps' node stacks and the k-best heaps
// (K >= 8; a dummy word below).
template <int K>
struct PacketSmem {
  static constexpr int HK = K >= 8 ? K : 1;
  uint32_t stack[QUERY_THREADS / 32 * PACKET_STACK];
  float lo[HK * QUERY_THREADS], hi[HK * QUERY_THREADS];
  uint32_t row[HK * QUERY_THREADS];
};

// The 32 lanes of a warp run the sorted batch positions tid (one per lane) of
// the queries described by `a`; every lane of the warp must call it together.
// s_lo / s_hi / s_row: the block's heap arrays, K * QUERY_THREADS words each
// (unused for K < 8); stack: this warp's node stack, PACKET_STACK words.
template <int M, int D, int K>
__device__ __forceinline__ void packet_queries(const QArgs& a, uint64_t tid, float* s_lo, float* s_hi,
                                               uint32_t* s_row, uint32_t* stack) {
  static_assert(D > 0 && M != M_LP, "packet path: compile-time width, metric without pow()");
#ifdef KD_WORK_COUNTS
  uint32_t kd_acc_[16] = {};
  long long kd_t_ = clock64();
#endif
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
#ifdef KD_WORK_COUNTS
  {
    const uint32_t lv = __popc(__ballot_sync(0xffffffffu, live));
    if ((threadIdx.x & 31) == 0) {
      KD_WORK(0, 1);
      KD_WORK(1, lv);
    }
  }
#endif
  if (!live) {
#pragma unroll
    for (int i = 0; i < D; ++i) q.v[i] = 0.0;
  }
  float qlo[D], qhi[D];
  uint64_t qkey[D];  // order keys of the coordinates, for exact side tests against splits
#pragma unroll
  for (int i = 0; i < D; ++i) {
    rn_enclose(__double2float_rn(q.v[i]), &qlo[i], &qhi[i]);
    qkey[i] = ieee_key(dbits(q.v[i]));
  }
  PointFilter<M, D> filt;
  filt.init(q, a.coord_max);
  const float* rows32 = filter_rows<D>(a);
  auto row_sum = [&](uint32_t r) { return filt.sum(rows32 + static_cast<uint64_t>(r) * filter_stride<D>(a)); };

  // k-best set: a shared-memory heap from K = 8 up, register slots below
  std::conditional_t<(K >= 8), LazyHeap<M, D, K>, LazySet<M, D, K>> best;
  if constexpr (K >= 8)
    best.init(a.k, a.cutoff, q.g, a.data, a.indices, s_lo, s_hi, s_row);
  else
    best.init(a.k, a.cutoff, q.g, a.data, a.indices);
  float thr = filt.threshold(best.b_hi), thr2 = filt.threshold(band_of(best.b_hi));

  // Seed: each lane first offers the points of its own landing leaf (the
  // leaf the reference's descent reaches; any leaf would be correct), so
  // its bound is tight before the shared traversal starts; the traversal then
  // skips that leaf for this lane.
  uint32_t own = NO_ID;
  if (live) {
    uint32_t n = 0;
    DNode nd;
    if (a.leaf_of) {  // the batch sort found it already
      n = a.leaf_of[qi];
      nd = a.nodes[n];
    } else {
      nd = a.nodes[0];
      while (!(nd.meta & KD_NODE_LEAF)) {
        const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
        uint64_t kq = qkey[0];
#pragma unroll
        for (int i = 1; i < D; ++i) kq = (static_cast<uint32_t>(i) == dim) ? qkey[i] : kq;
        n = kq <= ieee_key(dbits(nd.split)) ? n + 1 : nd.right;
        nd = a.nodes[n];
      }
    }
    own = n;
    const uint64_t se = dbits(nd.split);
    const uint32_t start = static_cast<uint32_t>(se), end = static_cast<uint32_t>(se >> 32);
    KD_WORK(2, end - start);
    const uint32_t chunk_end = (D == 8 && M != M_LINF) ? start + (end - start) / 8 * 8 : end;
    for (uint32_t r = start; r < end; ++r) {
      const float sr = row_sum(r);
      if (!(sr > thr2)) {
        float clo, chi;
        filt.enclose(sr, &clo, &chi);
        if (!(sr > thr) && !(clo > best.b_hi)) {
          const float before = best.b_hi;
          best.offer(clo, chi, r, r < chunk_end);
          if (best.b_hi != before) {  // the bound stays +inf (or unchanged) until the list fills
            thr = filt.threshold(best.b_hi);
            thr2 = filt.threshold(band_of(best.b_hi));
          }
        } else {
          best.note_point(clo, r, r < chunk_end);
        }
      }
    }
  }

  // Every lane pushes the same ids to the same words and pops what it pushed
  // itself, so no lane depends on another's store.  An entered inner node
  // stacks its far child and continues with the near one.
  int sp = 0;
  uint32_t node = 0;  // the node at hand; the near child follows an entered node without a push
  KD_PHASE(11);
  for (;;) {
    // the record loads with the box: one round trip a pop (it is wasted only
    // when no lane needs the node)
    const DNode nd = a.nodes[node];
    const float lb = box_lb<M, D>(a.boxes32 + static_cast<uint64_t>(node) * 2 * D, qlo, qhi);
    const bool need = live && !(lb > best.b_hi);
    if (live && !need) best.note(lb);
    const uint32_t need_mask = __ballot_sync(0xffffffffu, need);
#ifdef KD_WORK_COUNTS
    if ((threadIdx.x & 31) == 0) {
      KD_WORK(3, 1);
      if (need_mask) {
        KD_WORK(4, 1);
        KD_WORK(5, __popc(need_mask));
      }
    }
#endif
    if (!need_mask) {  // every lane's points there exceed its bound
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    if (nd.meta & KD_NODE_LEAF) {
      const bool take = need && node != own;  // its own leaf was offered already
      const uint32_t take_mask = __ballot_sync(0xffffffffu, take);
      if (!take_mask) {
        if (sp == 0) break;
        node = stack[--sp];
        continue;
      }
      KD_PHASE(12);
      const uint64_t se = dbits(nd.split);
      const uint32_t start = static_cast<uint32_t>(se), end = static_cast<uint32_t>(se >> 32);
      const uint32_t chunk_end = (D == 8 && M != M_LINF) ? start + (end - start) / 8 * 8 : end;
#ifdef KD_WORK_COUNTS
      if ((threadIdx.x & 31) == 0) {
        KD_WORK(6, 1);
        KD_WORK(7, end - start);
        KD_WORK(8, __popc(take_mask) * (end - start));
      }
#endif
      const uint32_t lane = threadIdx.x & 31;
      const uint32_t n_take = __popc(take_mask);
      const uint32_t my_rank = __popc(take_mask & ((1u << lane) - 1));  // among the lanes that take the leaf
      for (uint32_t c0 = start; c0 < end; c0 += 32) {
        // 1. which of these rows can each taker's bound admit (or put in the
        //    near-tie band just above it)?  Lanes take the rows (gs lanes a
        //    taker, 32 / gs takers a round) and get each taker's FP32 query
        //    and band threshold by shuffle: only the takers' rows are summed.
        const uint32_t rows = min(32u, end - c0);
        const uint32_t gs = rows <= 8 ? 8u : (rows <= 16 ? 16u : 32u);
        const uint32_t in_group = lane & (gs - 1), group = lane / gs;
        float p[D];
        PointFilter<M, D>::load(rows32 + static_cast<uint64_t>(c0 + min(in_group, rows - 1)) * filter_stride<D>(a), p);
        uint32_t pending = 0;
        uint32_t rem = take_mask;  // the takers not served yet
        for (uint32_t base = 0; base < n_take; base += 32 / gs) {  // uniform
          const uint32_t j = base + group;
          // this group's taker: the group-th lowest of rem (group < 4)
          uint32_t m = rem;
          if (group >= 1) m &= m - 1;
          if (group >= 2) m &= m - 1;
          if (group >= 3) m &= m - 1;
          const uint32_t src = m ? static_cast<uint32_t>(__ffs(m) - 1) : 0u;
          for (uint32_t i = 0; i < 32 / gs; ++i) rem &= rem - 1;  // uniform
          float q[D];
#pragma unroll
          for (int i = 0; i < D; ++i) q[i] = __shfl_sync(0xffffffffu, filt.q32[i], static_cast<int>(src));
          const float th = __shfl_sync(0xffffffffu, thr2, static_cast<int>(src));
          const float sv = PointFilter<M, D>::reduce_of(p, q);
          const uint32_t bits = __ballot_sync(0xffffffffu, j < n_take && in_group < rows && !(sv > th));
          if (take && my_rank >= base && my_rank < base + 32 / gs) {
            const uint32_t sl = my_rank - base;
            pending = (bits >> (sl * gs)) & (gs == 32 ? 0xffffffffu : ((1u << gs) - 1));
          }
        }
        KD_PHASE(13);
        // 2. offer them, all lanes with a pending point together.  The
        //    filter thresholds follow the bound once the chunk is done: within
        //    it they may lag (a lagging threshold only lets more rows reach
        //    the enclosure test against the present bound).  A pending row's
        //    sum is the one pass 1 compared with this lane's thr2 (the same
        //    operations on the same FP32 values), so it passes thr2 again.
        const float b_chunk = best.b_hi;
        while (__any_sync(0xffffffffu, pending != 0)) {
          if (pending) {
            const uint32_t r = c0 + __ffs(pending) - 1;
            pending &= pending - 1;
            const float sr = row_sum(r);
            KD_WORK(9, 1);
            float clo, chi;
            filt.enclose(sr, &clo, &chi);
            if (!(sr > thr) && !(clo > best.b_hi)) {
              KD_WORK(10, 1);
              best.offer(clo, chi, r, r < chunk_end);
            } else {
              best.note_point(clo, r, r < chunk_end);
            }
          }
        }
        if (best.b_hi != b_chunk) {
          thr = filt.threshold(best.b_hi);
          thr2 = filt.threshold(band_of(best.b_hi));
        }
        KD_PHASE(14);
      }
      if (sp == 0) break;
      node = stack[--sp];
      continue;
    }
    // near child first, by majority of the lanes that need this node
    const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
    uint64_t kq = qkey[0];
#pragma unroll
    for (int i = 1; i < D; ++i) kq = (static_cast<uint32_t>(i) == dim) ? qkey[i] : kq;
    const bool left = kq <= ieee_key(dbits(nd.split));
    const uint32_t left_votes = __popc(__ballot_sync(0xffffffffu, need && left));
    const bool left_first = 2 * left_votes >= static_cast<uint32_t>(__popc(need_mask));
    stack[sp++] = left_first ? nd.right : node + 1;
    node = left_first ? node + 1 : nd.right;
  }
  KD_PHASE(12);
  if constexpr (K >= 8) {
    if (live) best.sort_exact();
    best.write_warp(live, a.out_d + qi * a.k, a.out_i + qi * a.k, a.k, a.n_points);
    if (live && best.near_tie()) flag_rerun(a, qi);
  } else {
    if (live && best.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.k, a.n_points)) flag_rerun(a, qi);
  }
  KD_PHASE(15);
  KD_WORK_FLUSH();
}

template <int M, int D, int K>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_packet(QArgs a) {
  __shared__ PacketSmem<K> sm;
  packet_queries<M, D, K>(a, blockIdx.x * static_cast<uint64_t>(QUERY_THREADS) + threadIdx.x, sm.lo, sm.hi,
                          sm.row, sm.stack + (threadIdx.x >> 5) * PACKET_STACK);
}

// The same with the shared memory supplied at launch (sizeof(PacketSmem<K>)
// bytes): for k-best heaps larger than a static allocation may be (K = 64).
template <int M, int D, int K>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_packet_dyn(QArgs a) {
  extern __shared__ __align__(16) unsigned char packet_dyn[];
  PacketSmem<K>* sm = reinterpret_cast<PacketSmem<K>*>(packet_dyn);
  packet_queries<M, D, K>(a, blockIdx.x * static_cast<uint64_t>(QUERY_THREADS) + threadIdx.x, sm->lo, sm->hi,
                          sm->row, sm->stack + (threadIdx.x >> 5) * PACKET_STACK);
}
