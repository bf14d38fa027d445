// kd_lazy_best.cuh -- the k best candidates of one query held by one thread,
// kept as FP32 enclosures of their exact FP64 reduced distances (BestK /
// Best1, src/query.rs:379-494): LazySet (register slots) and LazyHeap
// (shared-memory max-heap) for the packet traversal's compile-time widths,
// LazySetDyn for the tensor-core filter's runtime widths; plus the FP32 box
// lower bound the packet traversal prunes with.  Included by the query
// translation units after their interval helpers.
//
// Placeholder slots (k < K) are [-inf, -inf]: every candidate sorts after them;
// empty slots are [+inf, +inf] with row ROW_NONE (exact +inf, index after all).
// Each real slot keeps the tree row of its point: the exact value is recomputed
// from the point's coordinates with the reference's operations whenever two
// enclosures overlap -- rarely -- and for the final results.  The original index
// is read from `indices` only for exact ties and for the output.
#pragma once

constexpr uint32_t ROW_NONE = 0xffffffffu;

// Lower bound only (the packet traversal's pruning test).
template <int M, int D>
__device__ __forceinline__ float box_lb(const float* b32, const float* qlo, const float* qhi) {
  // A node's box is 2D floats at node * 2D: 16-byte aligned for even D
  // (float4 loads), 8-byte aligned otherwise (float2 loads).
  float v[2 * D];
  if constexpr (D % 2 == 0) {
#pragma unroll
    for (int c = 0; c < D / 2; ++c) {
      const float4 w = reinterpret_cast<const float4*>(b32)[c];
      v[4 * c] = w.x;
      v[4 * c + 1] = w.y;
      v[4 * c + 2] = w.z;
      v[4 * c + 3] = w.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const float2 w = reinterpret_cast<const float2*>(b32)[c];
      v[2 * c] = w.x;
      v[2 * c + 1] = w.y;
    }
  }
  float lb = 0.f;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    float o = fmaxf(__fsub_rd(v[i], qhi[i]), __fsub_rd(qlo[i], v[D + i]));
    o = o > 0.f ? o : 0.f;
    lb = fold_lb<M>(lb, red_lb<M>(o));
  }
  return __fmul_rd(lb, LB_SHRINK);
}

// ---------------------------------------------------------------------------
// LazySet: the k best of one query (BestK keeps the k smallest by
// (distance, index), query.rs:461-481 -- a set under a strict total order),
// held unsorted: while slots are empty a candidate fills one (the reference
// inserts unconditionally then); afterwards an accepted candidate replaces the
// worst slot, and the k survivors are sorted by their exact (distance, index)
// once, at the end.  Used by the packet traversal, where offers arrive in no
// particular order.  Placeholders (k < K) are [-inf, -inf]; empty slots are
// [+inf, +inf] with row ROW_NONE.
// ---------------------------------------------------------------------------
template <int M, int D, int K>
struct LazySet {
  float lo[K], hi[K];
  uint32_t row[K];
  uint32_t chunk;    // bit j: slot j's point lies in a full Packed d8 chunk
  uint32_t n_empty;  // empty real slots
  int worst;         // an empty slot, else the slot with the largest hi
  float max_lo;      // the k-th exact distance is >= max_lo (when full)
  float second_hi;   // largest hi among the other slots
  float b_lo, b_hi;  // enclosure of the pruning bound min(k-th best, cutoff)
  float cut_lo, cut_hi;
  float runner;      // FP32 lower bound of every point dropped within max_distance (near-tie test)
  uint64_t cut_bits;
  QMem<D> q;
  const double* data;
  const uint32_t* indices;

  __device__ __forceinline__ void init(uint64_t k, double cutoff, const double* qg, const double* data_,
                                       const uint32_t* indices_) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool pad = static_cast<uint64_t>(j) < K - k;
      lo[j] = pad ? __int_as_float(0xff800000) : __int_as_float(0x7f800000);
      hi[j] = lo[j];
      row[j] = ROW_NONE;
    }
    chunk = 0;
    runner = __int_as_float(0x7f800000);
    n_empty = static_cast<uint32_t>(k);
    cut_bits = dbits(cutoff);
    cut_lo = mag_dn32(cut_bits);
    cut_hi = mag_up32(cut_bits);
    q.g = qg;
    data = data_;
    indices = indices_;
    rescan();
  }
  __device__ __forceinline__ bool is_empty(int j) const {
    return row[j] == ROW_NONE && lo[j] > 0.f;  // placeholders have lo = -inf
  }
  // worst, max_lo, second_hi and the bound enclosure after a change
  __device__ __forceinline__ void rescan() {
    float mh = __int_as_float(0xff800000), sh = mh, ml = mh;
    int w = 0, first_empty = -1;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool g = hi[j] > mh || (j == 0);
      sh = g ? mh : fmaxf(sh, hi[j]);
      mh = g ? hi[j] : mh;
      w = g ? j : w;
      ml = fmaxf(ml, lo[j]);
      first_empty = (first_empty < 0 && is_empty(j)) ? j : first_empty;
    }
    if (n_empty) {
      w = first_empty;
      mh = __int_as_float(0x7f800000);
      ml = mh;
    }
    worst = w;
    max_lo = ml;
    second_hi = sh;
    b_lo = fminf(ml, cut_lo);
    b_hi = fminf(mh, cut_hi);
  }
  __device__ __forceinline__ double exact_of(uint32_t r, bool in_chunk) const {
    return exact_dist<M, D>(q, data + static_cast<uint64_t>(r) * D, D, S_PACKED, in_chunk, 0.0);
  }
  __device__ __forceinline__ float slot_lo(int w) const {
    float v = lo[0];
#pragma unroll
    for (int j = 1; j < K; ++j) v = (j == w) ? lo[j] : v;
    return v;
  }
  __device__ __forceinline__ float slot_hi(int w) const {
    float v = hi[0];
#pragma unroll
    for (int j = 1; j < K; ++j) v = (j == w) ? hi[j] : v;
    return v;
  }

  // The worst slot exactly (full list): the largest (exact distance, index)
  // among the slots whose enclosure reaches max_lo -- no other slot can be it.
  __device__ void resolve_worst(double* wx, uint32_t* wid) {
    const float ml = max_lo;
    uint64_t best_bits = 0;
    uint32_t best_id = 0;
    int best_j = -1;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (hi[j] >= ml && row[j] != ROW_NONE) {
        const double x = exact_of(row[j], (chunk >> j) & 1u);
        const uint32_t id = indices[row[j]];
        lo[j] = mag_dn32(dbits(x));  // keep the tighter enclosure
        hi[j] = mag_up32(dbits(x));
        const bool g = best_j < 0 || dbits(x) > best_bits || (dbits(x) == best_bits && id > best_id);
        best_bits = g ? dbits(x) : best_bits;
        best_id = g ? id : best_id;
        best_j = g ? j : best_j;
      }
    }
    rescan();
    worst = best_j;
    *wx = bitsd(best_bits);
    *wid = best_id;
  }

  // exact bound min(k-th best, cutoff) as bits (query.rs:452-459)
  __device__ uint64_t bound_exact() {
    if (n_empty) return cut_bits;  // not full: the k-th best is +inf
    double wx;
    uint32_t wid;
    resolve_worst(&wx, &wid);
    const uint64_t kb = dbits(wx);
    return kb < cut_bits ? kb : cut_bits;
  }

  // Offer the point at tree row r whose exact distance lies in [clo, chi].
  __device__ __forceinline__ void offer(float clo, float chi, uint32_t r, bool in_chunk) {
    double cx = 0.0;
    bool have_x = false;
    if (!(chi <= cut_lo)) {  // the cutoff test, unless clearly inside
      if (clo > cut_hi) return;
      cx = exact_of(r, in_chunk);
      have_x = true;
      if (dbits(cx) > cut_bits) return;
    }
    if (n_empty == 0) {
      const float wlo = slot_lo(worst), whi = slot_hi(worst);
      const bool definite = second_hi < wlo;  // no other enclosure reaches the worst's
      if (definite && clo > whi) {            // after the worst: not kept
        note_point(clo, r, in_chunk);
        return;
      }
      if (chi < max_lo) {  // before the worst, whichever slot it is
        if (!definite) {
          double wx;
          uint32_t wid;
          resolve_worst(&wx, &wid);
        }
      } else {  // too close to call on enclosures
        double wx;
        uint32_t wid;
        resolve_worst(&wx, &wid);
        if (!have_x) cx = exact_of(r, in_chunk);
        const uint32_t cid = indices[r];
        if (!(dbits(cx) < dbits(wx) || (dbits(cx) == dbits(wx) && cid < wid))) {
          note(mag_dn32(dbits(cx)));
          return;
        }
        clo = mag_dn32(dbits(cx));
        chi = mag_up32(dbits(cx));
      }
    } else {
      --n_empty;
    }
    const int w = worst;
    // the worst drops out (when the set was full): its row and lower
    // enclosure, noted against the bound after the replacement
    const bool evict = row_of(w) != ROW_NONE;
    const float ev_lo = slot_lo(w);
    const uint32_t ev_row = row_of(w);
    const bool ev_chunk = (chunk >> w) & 1u;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool m = j == w;
      lo[j] = m ? clo : lo[j];
      hi[j] = m ? chi : hi[j];
      row[j] = m ? r : row[j];
    }
    if (D == 4 || D == 8) chunk = (chunk & ~(1u << w)) | (static_cast<uint32_t>(in_chunk) << w);
    rescan();
    if (evict) note_point(ev_lo, ev_row, ev_chunk);
  }
  __device__ __forceinline__ void note(float x) { runner = fminf(runner, x); }
  // A dropped point (tree row r) whose exact distance is at least lb: noted as
  // near_window (kd_query_common.cuh) describes.
  __device__ __forceinline__ void note_point(float lb, uint32_t r, bool in_chunk) {
    if (lb > near_window(b_hi)) return;
    note(mag_dn32(dbits(exact_of(r, in_chunk))));
  }
  __device__ __forceinline__ uint32_t row_of(int w) const {
    uint32_t r = row[0];
#pragma unroll
    for (int j = 1; j < K; ++j) r = (j == w) ? row[j] : r;
    return r;
  }

  // write_results (query.rs:421-429, 483-493): the exact values sorted by
  // (distance, index); empty slots after every real one.  Returns whether
  // the query is a near tie (kd_warp.cuh: the reference's descent may leave
  // out a point of this set; the caller reruns it in the reference's order).
  __device__ __forceinline__ bool write(double* od, int64_t* oi, uint64_t k, uint64_t n_points) const {
    uint64_t xb[K];
    uint32_t id[K];
    uint64_t dmax = 0;
    bool any = false;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (static_cast<uint64_t>(j) < K - k) {  // placeholder: sorts first
        xb[j] = 0;
        id[j] = 0;
      } else if (row[j] == ROW_NONE) {  // empty: sorts last
        xb[j] = ~0ull;
        id[j] = NO_ID;
      } else {
        const uint64_t x = dbits(exact_of(row[j], (chunk >> j) & 1u));
        dmax = x > dmax ? x : dmax;
        any = true;
        xb[j] = x + 1;
        id[j] = indices[row[j]];
      }
    }
#pragma unroll
    for (int i = 1; i < K; ++i) {
#pragma unroll
      for (int j = i; j > 0; --j) {
        const bool sw = xb[j] < xb[j - 1] || (xb[j] == xb[j - 1] && id[j] < id[j - 1]);
        const uint64_t tx = xb[j];
        const uint32_t ti = id[j];
        xb[j] = sw ? xb[j - 1] : xb[j];
        id[j] = sw ? id[j - 1] : id[j];
        xb[j - 1] = sw ? tx : xb[j - 1];
        id[j - 1] = sw ? ti : id[j - 1];
      }
    }
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (static_cast<uint64_t>(j) >= K - k) {
        const uint64_t o = j - (K - k);
        if (xb[j] != ~0ull) {
          od[o] = restore<M>(bitsd(xb[j] - 1), 0.0);
          oi[o] = static_cast<int64_t>(id[j]);
        } else {
          od[o] = bitsd(INF_BITS);
          oi[o] = static_cast<int64_t>(n_points);
        }
      }
    }
    if (!any) return false;
    const float g = fmaxf(__fmul_ru(mag_up32(dmax), UB_GROW), 1.17549435e-38f);
    return runner <= g || cut_lo <= g;
  }
};

// ---------------------------------------------------------------------------
// LazyHeap: the same k best as LazySet, as a binary max-heap on the upper
// enclosure `hi`, in shared memory (slot j of a thread at [j * QUERY_THREADS]:
// the 32 lanes of a warp touch 32 consecutive words, one per bank, whatever
// slot each lane is at).  Replacing the worst costs one sift-down, log2(k)
// levels, instead of a scan of all K register slots.
//
// The root has the largest hi, so its exact distance is at most hi[0] and the
// k-th best (the largest exact distance kept) is at least lo[0]:
//  - a candidate with clo > hi[0] is after every kept point: rejected;
//  - a candidate with chi < lo[0] is before the worst, and when no other slot
//    reaches lo[0] (both children's hi < lo[0]) the root IS the worst:
//    the candidate replaces it;
//  - otherwise (enclosures too close to call) the exact FP64 values decide, by
//    (distance, original index) as BestK does (query.rs:461-481), and the heap
//    is rebuilt.
// In a full Packed d8 chunk (kernel.rs:540-562) the summation order differs;
// that flag rides in the sign bit of lo (lo >= 0 otherwise).
// ---------------------------------------------------------------------------
template <int M, int D, int K>
struct LazyHeap {
  static constexpr int S = QUERY_THREADS;
  float* lo;
  float* hi;
  uint32_t* row;
  uint32_t n, k;
  float b_hi;  // upper bound of the pruning bound min(k-th best, cutoff)
  float cut_lo, cut_hi;
  float runner;  // FP32 lower bound of every point dropped within max_distance (near-tie test)
  uint64_t cut_bits;
  QMem<D> q;
  const double* data;
  const uint32_t* indices;

  __device__ __forceinline__ void init(uint64_t k_, double cutoff, const double* qg, const double* data_,
                                       const uint32_t* indices_, float* s_lo, float* s_hi, uint32_t* s_row) {
    lo = s_lo + threadIdx.x;
    hi = s_hi + threadIdx.x;
    row = s_row + threadIdx.x;
    n = 0;
    k = static_cast<uint32_t>(k_);
    cut_bits = dbits(cutoff);
    cut_lo = mag_dn32(cut_bits);
    cut_hi = mag_up32(cut_bits);
    q.g = qg;
    data = data_;
    indices = indices_;
    b_hi = cut_hi;
    runner = __int_as_float(0x7f800000);
  }
  __device__ __forceinline__ void note(float x) { runner = fminf(runner, x); }
  // A dropped point (tree row r) whose exact distance is at least lb: noted
  // as near_window (kd_query_common.cuh) describes.
  __device__ __forceinline__ void note_point(float lb, uint32_t r, bool in_chunk) {
    if (lb > near_window(b_hi)) return;
    note(mag_dn32(dbits(exact_of(r, in_chunk))));
  }
  static __device__ __forceinline__ float tag(float l, bool in_chunk) {
    return __uint_as_float(__float_as_uint(l) | (static_cast<uint32_t>(in_chunk) << 31));
  }
  static __device__ __forceinline__ bool chunk_of(float tagged) { return __float_as_uint(tagged) >> 31; }
  __device__ __forceinline__ double exact_of(uint32_t r, bool in_chunk) const {
    return exact_dist<M, D>(q, data + static_cast<uint64_t>(r) * D, D, S_PACKED, in_chunk, 0.0);
  }
  __device__ __forceinline__ void put(uint32_t j, float tl, float h, uint32_t r) {
    lo[j * S] = tl;
    hi[j * S] = h;
    row[j * S] = r;
  }
  __device__ __forceinline__ void sift_up(uint32_t j, float tl, float h, uint32_t r) {
    while (j > 0) {
      const uint32_t p = (j - 1) >> 1;
      const float ph = hi[p * S];
      if (!(ph < h)) break;
      put(j, lo[p * S], ph, row[p * S]);
      j = p;
    }
    put(j, tl, h, r);
  }
  __device__ __forceinline__ void sift_down(uint32_t j, float tl, float h, uint32_t r) {
    for (;;) {
      uint32_t c = 2 * j + 1;
      if (c >= n) break;
      float ch = hi[c * S];
      if (c + 1 < n) {
        const float c2 = hi[(c + 1) * S];
        if (c2 > ch) {
          ++c;
          ch = c2;
        }
      }
      if (!(ch > h)) break;
      put(j, lo[c * S], ch, row[c * S]);
      j = c;
    }
    put(j, tl, h, r);
  }
  __device__ __forceinline__ void refresh() { b_hi = n < k ? cut_hi : fminf(hi[0], cut_hi); }

  // Offer the point at tree row r whose exact distance lies in [clo, chi].
  __device__ __forceinline__ void offer(float clo, float chi, uint32_t r, bool in_chunk) {
    double cx = 0.0;
    bool have_x = false;
    if (!(chi <= cut_lo)) {  // the cutoff test, unless clearly inside
      if (clo > cut_hi) return;
      cx = exact_of(r, in_chunk);
      have_x = true;
      if (dbits(cx) > cut_bits) return;
    }
    if (n < k) {  // not full: the reference keeps every candidate
      ++n;
      sift_up(n - 1, tag(clo, in_chunk), chi, r);
      refresh();
      return;
    }
    const float rh = hi[0];
    if (clo > rh) {
      note_point(clo, r, in_chunk);
      return;
    }
    const float rl = fabsf(lo[0]);
    float sec = __int_as_float(0xff800000);
    if (n > 1) sec = hi[S];
    if (n > 2) sec = fmaxf(sec, hi[2 * S]);
    if (chi < rl && sec < rl) {  // the root drops out
      const uint32_t ev_row = row[0];
      const bool ev_chunk = chunk_of(lo[0]);
      sift_down(0, tag(clo, in_chunk), chi, r);
      refresh();
      note_point(rl, ev_row, ev_chunk);  // against the bound after the eviction
      return;
    }
    offer_exact(r, in_chunk, have_x, cx);
  }

  // Enclosures too close to call: exact values of the candidate and of every
  // slot that can be the worst (hi >= lo[0]); those slots keep their tightened
  // enclosures; the candidate replaces the exact worst if it is before it.
  // Inline although rare: out of line, as a member call, it put the heap
  // object in local memory, so every access to its fields (and, through them,
  // to the shared-memory slots) on the hot path became a local or generic
  // load; as a call on a copy, the call's register convention cost more
  // registers than the inlined code does.
  __device__ __forceinline__ void offer_exact(uint32_t r, bool in_chunk, bool have_x, double cx) {
    if (!have_x) cx = exact_of(r, in_chunk);
    const uint32_t cid = indices[r];
    const float rl = fabsf(lo[0]);
    uint64_t wb = 0;
    uint32_t wid = 0, wj = 0;
    bool any = false;
    for (uint32_t j = 0; j < n; ++j) {
      if (hi[j * S] >= rl) {
        const bool ic = chunk_of(lo[j * S]);
        const uint32_t rj = row[j * S];
        const uint64_t xb = dbits(exact_of(rj, ic));
        lo[j * S] = tag(mag_dn32(xb), ic);
        hi[j * S] = mag_up32(xb);
        const uint32_t id = indices[rj];
        if (!any || xb > wb || (xb == wb && id > wid)) {
          wb = xb;
          wid = id;
          wj = j;
          any = true;
        }
      }
    }
    const uint64_t cb = dbits(cx);
    if (cb < wb || (cb == wb && cid < wid)) {
      note(mag_dn32(wb));  // the worst drops out
      put(wj, tag(mag_dn32(cb), in_chunk), mag_up32(cb), r);
    } else {
      note(mag_dn32(cb));
    }
    for (uint32_t j = n / 2; j-- > 0;) sift_down(j, lo[j * S], hi[j * S], row[j * S]);
    refresh();
  }

  // write_results (query.rs:421-429, 483-493): the exact values sorted by
  // (distance, index), empty slots after every real one.  The slots are
  // rewritten in place -- exact distance bits in lo / hi, original index in
  // row -- and heap-sorted there, so no K-sized register array is needed.
  __device__ __forceinline__ uint64_t key_at(uint32_t j) const {
    return (static_cast<uint64_t>(__float_as_uint(hi[j * S])) << 32) | __float_as_uint(lo[j * S]);
  }
  __device__ __forceinline__ bool after(uint32_t a, uint32_t b) const {  // slot a sorts after slot b
    const uint64_t ka = key_at(a), kb = key_at(b);
    return ka > kb || (ka == kb && row[a * S] > row[b * S]);
  }
  __device__ __forceinline__ void swap_slots(uint32_t a, uint32_t b) {
    const float l = lo[a * S], h = hi[a * S];
    const uint32_t r = row[a * S];
    lo[a * S] = lo[b * S];
    hi[a * S] = hi[b * S];
    row[a * S] = row[b * S];
    lo[b * S] = l;
    hi[b * S] = h;
    row[b * S] = r;
  }
  __device__ __forceinline__ void sift_exact(uint32_t j, uint32_t m) {
    for (;;) {
      uint32_t c = 2 * j + 1;
      if (c >= m) return;
      if (c + 1 < m && after(c + 1, c)) ++c;
      if (!after(c, j)) return;
      swap_slots(j, c);
      j = c;
    }
  }
  // Exact keys in place, heap-sorted ascending (one lane's own column).
  __device__ __forceinline__ void sort_exact() {
    for (uint32_t j = 0; j < n; ++j) {
      const uint32_t rj = row[j * S];
      const uint64_t xb = dbits(exact_of(rj, chunk_of(lo[j * S])));
      lo[j * S] = __uint_as_float(static_cast<uint32_t>(xb));
      hi[j * S] = __uint_as_float(static_cast<uint32_t>(xb >> 32));
      row[j * S] = indices[rj];
    }
    for (uint32_t j = n / 2; j-- > 0;) sift_exact(j, n);
    for (uint32_t m = n; m > 1; --m) {
      swap_slots(0, m - 1);
      sift_exact(0, m - 1);
    }
  }
  // After sort_exact: whether the query is a near tie (kd_warp.cuh: the
  // reference's descent may leave out a point of this set).
  __device__ __forceinline__ bool near_tie() const {
    if (n == 0) return false;
    const float g = fmaxf(__fmul_ru(mag_up32(key_at(n - 1)), UB_GROW), 1.17549435e-38f);
    return runner <= g || cut_lo <= g;
  }
  // The whole warp writes its lanes' results, one query row at a time, lane j
  // storing element j: every row of distances (and of indices) goes out as
  // whole contiguous segments.  Every lane of the warp calls it; `live` says
  // whether this lane has a query whose results to write (sorted already).
  // The warp's (query, slot) pairs are written 32 at a time, pair f = lane +
  // 32 t being slot f % k of lane f / k's query: every lane takes part in each
  // pass (the FP64 square root of L2 is a long instruction sequence on the
  // FP64 pipe) and one store covers 32 / k queries' rows.
  __device__ __forceinline__ void write_warp(bool live, double* od, int64_t* oi, uint64_t k_, uint64_t n_points) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t live_mask = __ballot_sync(0xffffffffu, live);
    __syncwarp();
    const uint32_t col0 = threadIdx.x - lane;  // this warp's first heap column
    const uint32_t kk = static_cast<uint32_t>(k_);
    const uint32_t total = 32 * kk;
    for (uint32_t f0 = 0; f0 < total; f0 += 32) {
      const uint32_t f = f0 + lane;
      const uint32_t r = min(f / kk, 31u), j = f - r * kk;
      double* od_r = reinterpret_cast<double*>(__shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(od), r));
      int64_t* oi_r = reinterpret_cast<int64_t*>(__shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(oi), r));
      const uint32_t n_r = __shfl_sync(0xffffffffu, n, r);
      if (f >= total || !((live_mask >> r) & 1u)) continue;
      if (j < n_r) {
        const uint32_t c = (col0 + r) + j * S;
        const uint64_t key = (static_cast<uint64_t>(__float_as_uint(hi[c - threadIdx.x])) << 32) |
                             __float_as_uint(lo[c - threadIdx.x]);
        od_r[j] = restore<M>(bitsd(key), 0.0);
        oi_r[j] = static_cast<int64_t>(row[c - threadIdx.x]);
      } else {
        od_r[j] = bitsd(INF_BITS);
        oi_r[j] = static_cast<int64_t>(n_points);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Runtime-width variants (the tensor-core filter path, 16 <= d <= 128):
// the exact FP64 value follows the reference's Folded (d <= 16) or Streamed
// (d > 16) L2 order (kernel.rs:343-354, 177-188) from the query in memory.
// ---------------------------------------------------------------------------
struct DynPoint {
  const double* q;     // the query, FP64
  const double* data;  // tree-ordered points, FP64
  uint64_t d;
  int strat;
  __device__ __forceinline__ double exact(uint32_t r) const {
    QVec<0> qv;
    qv.g = q;
    return exact_dist<M_L2, 0>(qv, data + static_cast<uint64_t>(r) * d, d, strat, false, 0.0);
  }
};

template <int K>
struct LazySetDyn {
  float lo[K], hi[K];
  uint32_t row[K];
  uint32_t n_empty;
  int worst;
  float max_lo, second_hi;
  float b_lo, b_hi;
  float cut_lo, cut_hi;
  float runner;  // FP32 lower bound of every point dropped within max_distance (near-tie test)
  uint64_t cut_bits;
  DynPoint pt;
  const uint32_t* indices;

  __device__ __forceinline__ void note(float x) { runner = fminf(runner, x); }
  // A dropped point (tree row r) whose exact distance is at least lb: noted as
  // near_window (kd_query_common.cuh) describes.
  __device__ __forceinline__ void note_point(float lb, uint32_t r) {
    if (lb > near_window(b_hi)) return;
    note(mag_dn32(dbits(pt.exact(r))));
  }
  __device__ __forceinline__ uint32_t row_of(int w) const {
    uint32_t r = row[0];
#pragma unroll
    for (int j = 1; j < K; ++j) r = (j == w) ? row[j] : r;
    return r;
  }
  __device__ __forceinline__ void init(uint64_t k, double cutoff, DynPoint p, const uint32_t* indices_) {
    runner = __int_as_float(0x7f800000);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool pad = static_cast<uint64_t>(j) < K - k;
      lo[j] = pad ? __int_as_float(0xff800000) : __int_as_float(0x7f800000);
      hi[j] = lo[j];
      row[j] = ROW_NONE;
    }
    n_empty = static_cast<uint32_t>(k);
    cut_bits = dbits(cutoff);
    cut_lo = mag_dn32(cut_bits);
    cut_hi = mag_up32(cut_bits);
    pt = p;
    indices = indices_;
    rescan();
  }
  __device__ __forceinline__ bool is_empty(int j) const { return row[j] == ROW_NONE && lo[j] > 0.f; }
  __device__ __forceinline__ void rescan() {
    float mh = __int_as_float(0xff800000), sh = mh, ml = mh;
    int w = 0, first_empty = -1;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool g = hi[j] > mh || (j == 0);
      sh = g ? mh : fmaxf(sh, hi[j]);
      mh = g ? hi[j] : mh;
      w = g ? j : w;
      ml = fmaxf(ml, lo[j]);
      first_empty = (first_empty < 0 && is_empty(j)) ? j : first_empty;
    }
    if (n_empty) {
      w = first_empty;
      mh = __int_as_float(0x7f800000);
      ml = mh;
    }
    worst = w;
    max_lo = ml;
    second_hi = sh;
    b_lo = fminf(ml, cut_lo);
    b_hi = fminf(mh, cut_hi);
  }
  __device__ __forceinline__ float slot_lo(int w) const {
    float v = lo[0];
#pragma unroll
    for (int j = 1; j < K; ++j) v = (j == w) ? lo[j] : v;
    return v;
  }
  __device__ __forceinline__ float slot_hi(int w) const {
    float v = hi[0];
#pragma unroll
    for (int j = 1; j < K; ++j) v = (j == w) ? hi[j] : v;
    return v;
  }
  __device__ void resolve_worst(double* wx, uint32_t* wid) {
    const float ml = max_lo;
    uint64_t best_bits = 0;
    uint32_t best_id = 0;
    int best_j = -1;
#pragma unroll
    for (int j = 0; j < K; ++j) {  // static indices keep the slots in registers
      if (hi[j] >= ml && row[j] != ROW_NONE) {
        const double x = pt.exact(row[j]);
        const uint32_t id = indices[row[j]];
        lo[j] = mag_dn32(dbits(x));
        hi[j] = mag_up32(dbits(x));
        const bool g = best_j < 0 || dbits(x) > best_bits || (dbits(x) == best_bits && id > best_id);
        best_bits = g ? dbits(x) : best_bits;
        best_id = g ? id : best_id;
        best_j = g ? j : best_j;
      }
    }
    rescan();
    worst = best_j;
    *wx = bitsd(best_bits);
    *wid = best_id;
  }
  __device__ void offer(float clo, float chi, uint32_t r) {
    double cx = 0.0;
    bool have_x = false;
    if (!(chi <= cut_lo)) {
      if (clo > cut_hi) return;
      cx = pt.exact(r);
      have_x = true;
      if (dbits(cx) > cut_bits) return;
    }
    if (n_empty == 0) {
      const float wlo = slot_lo(worst), whi = slot_hi(worst);
      const bool definite = second_hi < wlo;
      if (definite && clo > whi) {
        note_point(clo, r);
        return;
      }
      if (chi < max_lo) {
        if (!definite) {
          double wx;
          uint32_t wid;
          resolve_worst(&wx, &wid);
        }
      } else {
        double wx;
        uint32_t wid;
        resolve_worst(&wx, &wid);
        if (!have_x) cx = pt.exact(r);
        const uint32_t cid = indices[r];
        if (!(dbits(cx) < dbits(wx) || (dbits(cx) == dbits(wx) && cid < wid))) {
          note(mag_dn32(dbits(cx)));
          return;
        }
        clo = mag_dn32(dbits(cx));
        chi = mag_up32(dbits(cx));
      }
    } else {
      --n_empty;
    }
    const int w = worst;
    // the worst drops out (when the set was full): noted against the bound
    // after the replacement
    const bool evict = row_of(w) != ROW_NONE;
    const float ev_lo = slot_lo(w);
    const uint32_t ev_row = row_of(w);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const bool m = j == w;
      lo[j] = m ? clo : lo[j];
      hi[j] = m ? chi : hi[j];
      row[j] = m ? r : row[j];
    }
    rescan();
    if (evict) note_point(ev_lo, ev_row);
  }
  // exact values of the k best, sorted by (distance, index), written out;
  // returns whether the query is a near tie (kd_warp.cuh).
  __device__ bool write(double* od, int64_t* oi, uint64_t k, uint64_t n_points) const {
    uint64_t xb[K];
    uint32_t id[K];
    uint64_t dmax = 0;
    bool any = false;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (static_cast<uint64_t>(j) < K - k) {
        xb[j] = 0;
        id[j] = 0;
      } else if (row[j] == ROW_NONE) {
        xb[j] = ~0ull;
        id[j] = NO_ID;
      } else {
        const uint64_t x = dbits(pt.exact(row[j]));
        dmax = x > dmax ? x : dmax;
        any = true;
        xb[j] = x + 1;
        id[j] = indices[row[j]];
      }
    }
    for (int i = 1; i < K; ++i) {
      const uint64_t tx = xb[i];
      const uint32_t ti = id[i];
      int j = i;
      while (j > 0 && (tx < xb[j - 1] || (tx == xb[j - 1] && ti < id[j - 1]))) {
        xb[j] = xb[j - 1];
        id[j] = id[j - 1];
        --j;
      }
      xb[j] = tx;
      id[j] = ti;
    }
    for (int j = 0; j < K; ++j) {
      if (static_cast<uint64_t>(j) >= K - k) {
        const uint64_t o = j - (K - k);
        if (xb[j] != ~0ull) {
          od[o] = __dsqrt_rn(bitsd(xb[j] - 1));
          oi[o] = static_cast<int64_t>(id[j]);
        } else {
          od[o] = bitsd(INF_BITS);
          oi[o] = static_cast<int64_t>(n_points);
        }
      }
    }
    if (!any) return false;
    const float g = fmaxf(__fmul_ru(mag_up32(dmax), UB_GROW), 1.17549435e-38f);
    return runner <= g || cut_lo <= g;
  }
};
