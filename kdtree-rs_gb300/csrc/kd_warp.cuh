// kd_warp.cuh -- building blocks of the warp-per-query kernels (best-first,
// kd_query_warp.cuh; reference order, kd_query_ref.cuh): the warp's k-best
// list, FP32 row filters for every width, box bounds split across the lanes.
// Included inside namespace kd { namespace { ... } } after kd_query_common.cuh,
// kd_lazy_best.cuh and kd_query_packet.cuh.
//
// Widths.  D > 0 is a compile-time width (1, 2, 3, 4, 8, 16): the query's FP32
// copy lives in registers and rows are read from the tree's FP32 copy
// (`data32`, d floats a row).  D = 0 is any width up to WARP_MAX_D: the FP32
// query lives in shared memory and rows are read from `data32w`, the FP32
// copy padded to w32 floats (a multiple of 4, zeros after the last
// coordinate), so every row loads as whole float4 vectors.
//
// Near ties.  A kernel that does not follow the reference's visiting order
// (the best-first traversal here, the packet traversal, the tensor-core filter)
// returns the exact top-k: the k smallest (FP64 distance in the reference's
// summation order, index) within max_distance.  The reference's descent can
// leave out a point of that set: its gates -- the root seed, the split-plane
// bound and the box distance (src/query.rs:169-194, 248-327) -- are rounded
// lower bounds that can come out a few ulps above the distance of a point
// inside the subtree, as the leaf scan computes it.  That needs the pruned
// point p to satisfy dist(p) <= bound_t < gate <= dist(p) (1 + e), with
// e < 2^-40 (at most 2 x 34 plane updates and d + 2 roundings of 2^-53),
// where bound_t is the bound at that moment, at least the final k-th
// distance D.  Either bound_t is the cutoff, and then the cutoff lies in
// [D / (1 + e), D (1 + e)); or k points within bound_t were already kept and p
// is another, so the (k + 1)-th smallest distance within the cutoff is below
// D (1 + e).  A fast kernel therefore keeps `runner`, an FP32 lower bound of
// every point it dropped (rejected, evicted, or in a pruned subtree) -- a
// lower bound of the (k + 1)-th distance -- and flags the query when runner
// or the cutoff is within 2^-20 of D: only then can the reference's answer
// differ, and flagged queries are run again in the reference's order
// (kd_query_ref.cuh).  Points the filters drop without an enclosure are
// farther than (1 + 2^-19) times the bound of that moment.
#pragma once

constexpr uint32_t FULL_MASK = 0xffffffffu;
constexpr int WARP_STACK = 2 * KD_MAX_DEPTH;
// Candidates in one leaf chunk from which the warp traversal ranks them
// together (WarpList::offer_all) instead of offering them one at a time
// (a batch of 256 trees of widths 2, 3 and 8, k in {1, 4, 32}, on GB300:
// 83.7 M q/s from 2, 83.5 from 3, 83.2 from 4, 82.2 from 8).
constexpr int WARP_BULK_MIN = 2;
constexpr uint32_t WARP_MAX_D = static_cast<uint32_t>(WARP_MAX_WIDTH);  // widest query (4 dimensions a lane)

template <int D>
struct Log2Ceil {
  static constexpr int value = D <= 1 ? 0 : 1 + Log2Ceil<(D + 1) / 2>::value;
};
template <>
struct Log2Ceil<1> {
  static constexpr int value = 0;
};

// ---------------------------------------------------------------------------
// FP32 row filter for runtime widths (the packet traversal's PointFilter with
// the width and the margins taken at run time).  The FP32 sum of d terms
// over-estimates |a|^2 (|a| for L1) by at most (d + 3) 2^-24 relative; its
// square root by half that plus s * rsqrtf(s)'s 3 ulp (6 2^-24); the
// triangle-inequality spread is sqrt(d) E (L2), d E (L1), E (L-inf).
// ---------------------------------------------------------------------------
template <int M>
struct PointFilterDyn {
  const float* sq;  // the query's FP32 copy, w32 floats (zero padded), shared memory
  uint32_t w32;
  float spread, grow, r_lo, r_hi;
  float abs_slack;

  // Every lane of the warp calls it; sq_w is the warp's w32-float area.
  __device__ __forceinline__ void init(const double* qg, uint32_t d, uint32_t w, float coord_max, float* sq_w,
                                       uint32_t lane) {
    float qmax = 0.f;
    for (uint32_t i = lane; i < w; i += 32) {
      const float v = i < d ? __double2float_rn(qg[i]) : 0.f;
      sq_w[i] = v;
      qmax = fmaxf(qmax, fabsf(v));
    }
#pragma unroll
    for (int s = 16; s; s >>= 1) qmax = fmaxf(qmax, __shfl_xor_sync(FULL_MASK, qmax, s));
    __syncwarp();
    sq = sq_w;
    w32 = w;
    const float e = __fmaf_ru(__fadd_ru(coord_max, qmax), TWO_M24, 2.9e-45f /* 2^-148 */);
    const float fd = static_cast<float>(d);
    spread = (M == M_L2) ? __fmul_ru(e, __fsqrt_ru(fd)) : (M == M_L1 ? __fmul_ru(e, fd) : e);
    // sum: (d + 3) 2^-24 relative, at least 2^-20
    grow = fmaxf(UB_GROW, __fadd_ru(1.f, __fmul_ru(fd + 4.f, TWO_M24)));
    // enclosure of |a| from s: half the sum's error plus s * rsqrtf(s)'s 3 ulp
    // (6 2^-24) for L2, the sum's error for L1 / L-inf; at least 2^-19
    const float m = (M == M_L2) ? __fmul_ru(__fadd_ru(__fmul_ru(fd, 0.5f), 8.f), TWO_M24)
                                : __fmul_ru(fd + 4.f, TWO_M24);
    const float mm = fmaxf(m, 1.9073486e-06f /* 2^-19 */);
    r_lo = __fsub_rd(1.f, mm);
    r_hi = __fadd_ru(1.f, mm);
    abs_slack = __fmul_ru(fd, 2.9e-45f);
  }
  __device__ __forceinline__ float threshold(float b) const {
    if (M == M_L2) {
      const float r = __fadd_ru(sqrt_up(b), spread);
      return __fadd_ru(__fmul_ru(__fmul_ru(r, r), grow), abs_slack);
    }
    return __fadd_ru(__fmul_ru(__fadd_ru(b, spread), grow), abs_slack);
  }
  __device__ __forceinline__ void enclose(float s, float* clo, float* chi) const {
    float lo, hi;
    if (M == M_L2) {
      const float r = s > 0.f ? s * rsqrtf(s) : 0.f;
      if (!(r <= 3.4e38f)) {
        *clo = 0.f;
        *chi = __int_as_float(0x7f800000);
        return;
      }
      lo = fmaxf(__fsub_rd(__fmul_rd(r, r_lo), spread), 0.f);
      hi = __fadd_ru(__fmul_ru(r, r_hi), spread);
      lo = __fmul_rd(lo, lo);
      hi = __fmul_ru(hi, hi);
    } else {
      lo = fmaxf(__fsub_rd(__fmul_rd(s, r_lo), spread), 0.f);
      hi = __fadd_ru(__fmul_ru(s, r_hi), spread);
      if (!(s <= 3.4e38f)) hi = __int_as_float(0x7f800000);
    }
    *clo = __fmul_rd(lo, LB_SHRINK);
    *chi = __fmul_ru(hi, UB_GROW);
  }
  // FP32 reduced distance of the padded row at p32 (16-byte aligned).
  __device__ __forceinline__ float sum(const float* p32) const {
    const float4* p4 = reinterpret_cast<const float4*>(p32);
    const float4* q4 = reinterpret_cast<const float4*>(sq);
    float s0 = 0.f, s1 = 0.f;
    for (uint32_t c = 0; c < w32 / 4; ++c) {
      const float4 p = p4[c], q = q4[c];
      const float t0 = __fsub_rn(p.x, q.x), t1 = __fsub_rn(p.y, q.y);
      const float t2 = __fsub_rn(p.z, q.z), t3 = __fsub_rn(p.w, q.w);
      if (M == M_L2) {
        s0 = __fmaf_rn(t0, t0, s0);
        s1 = __fmaf_rn(t1, t1, s1);
        s0 = __fmaf_rn(t2, t2, s0);
        s1 = __fmaf_rn(t3, t3, s1);
      } else if (M == M_L1) {
        s0 = __fadd_rn(s0, fabsf(t0));
        s1 = __fadd_rn(s1, fabsf(t1));
        s0 = __fadd_rn(s0, fabsf(t2));
        s1 = __fadd_rn(s1, fabsf(t3));
      } else {
        s0 = fmaxf(s0, fmaxf(fabsf(t0), fabsf(t2)));
        s1 = fmaxf(s1, fmaxf(fabsf(t1), fabsf(t3)));
      }
    }
    // two partial sums: no path through the sum holds more than d roundings,
    // which is all the (d + 3) 2^-24 bound needs
    return M == M_LINF ? fmaxf(s0, s1) : __fadd_rn(s0, s1);
  }
};

// The row filter of width D (static) or runtime width (D = 0).
template <int M, int D>
struct RowFilterOf {
  using type = PointFilter<M, D>;
};
template <int M>
struct RowFilterOf<M, 0> {
  using type = PointFilterDyn<M>;
};

// ---------------------------------------------------------------------------
// Lower bounds (and enclosures) of box distances with the dimensions split
// across the lanes.
//   Compile-time widths <= 16: lanes 0-15 take box A, lanes 16-31 box B, lane i
//   of a half dimension i (warp_box_lb2 below; my_qlo / my_qhi: the query's
//   enclosure in dimension lane % 16).
//   Runtime widths: the whole warp takes one box at a time, lane i the
//   dimensions i + 32 j (LaneQ: the query's enclosures there).
// Each term is rounded toward the safe side and folded with directed rounding
// (any order bounds the exact FP64 sum, whose own rounding LB_SHRINK /
// UB_GROW cover).
// ---------------------------------------------------------------------------
template <int M, int D>
__device__ __forceinline__ void warp_box_lb2(const float* bl, const float* br, float my_qlo, float my_qhi,
                                             uint32_t lane, float* lb_l, float* lb_r) {
  static_assert(D > 0 && D <= 16, "one 16-lane half per box");
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

struct LaneQ {
  float lo[WARP_MAX_D / 32], hi[WARP_MAX_D / 32];
};

__device__ __forceinline__ void lane_query_enclosure(const double* qg, uint32_t d, uint32_t lane, LaneQ* lq) {
#pragma unroll
  for (int j = 0; j < static_cast<int>(WARP_MAX_D / 32); ++j) {
    const uint32_t i = lane + 32u * j;
    float lo = 0.f, hi = 0.f;
    if (i < d) rn_enclose(__double2float_rn(qg[i]), &lo, &hi);
    lq->lo[j] = lo;
    lq->hi[j] = hi;
  }
}

// Lower and upper bounds of the exact FP64 box distance (kernel.rs:565-616)
// to the outward-rounded FP32 box b32 ([lo | hi], d each), all lanes.
template <int M>
__device__ __forceinline__ void warp_box_enc_dyn(const float* b32, uint32_t d, uint32_t lane, const LaneQ& lq,
                                                 float* lb_out, float* ub_out) {
  float lb = 0.f, ub = 0.f;
#pragma unroll
  for (int j = 0; j < static_cast<int>(WARP_MAX_D / 32); ++j) {
    const uint32_t i = lane + 32u * j;
    if (i < d) {
      const float lo32 = b32[i], hi32 = b32[d + i];
      const float lo_up = __fadd_ru(lo32, __fmaf_ru(fabsf(lo32), TWO_M23, TINY32));
      const float hi_dn = __fsub_rd(hi32, __fmaf_ru(fabsf(hi32), TWO_M23, TINY32));
      float o_lb = fmaxf(__fsub_rd(lo32, lq.hi[j]), __fsub_rd(lq.lo[j], hi32));
      o_lb = o_lb > 0.f ? o_lb : 0.f;
      const float o_ub = fmaxf(fmaxf(__fsub_ru(lo_up, lq.lo[j]), __fsub_ru(lq.hi[j], hi_dn)), 0.f);
      lb = fold_lb<M>(lb, red_lb<M>(o_lb));
      ub = fold_ub<M>(ub, red_ub<M>(o_ub));
    }
  }
#pragma unroll
  for (int s = 16; s; s >>= 1) {
    lb = fold_lb<M>(lb, __shfl_xor_sync(FULL_MASK, lb, s));
    ub = fold_ub<M>(ub, __shfl_xor_sync(FULL_MASK, ub, s));
  }
  *lb_out = __fmul_rd(lb, LB_SHRINK);
  *ub_out = __fmul_ru(ub, UB_GROW);
}

// Lower bounds only, two boxes (runtime widths).
template <int M>
__device__ __forceinline__ void warp_box_lb2_dyn(const float* bl, const float* br, uint32_t d, uint32_t lane,
                                                 const LaneQ& lq, float* lb_l, float* lb_r) {
  float a = 0.f, b = 0.f;
#pragma unroll
  for (int j = 0; j < static_cast<int>(WARP_MAX_D / 32); ++j) {
    const uint32_t i = lane + 32u * j;
    if (i < d) {
      float oa = fmaxf(__fsub_rd(bl[i], lq.hi[j]), __fsub_rd(lq.lo[j], bl[d + i]));
      float ob = fmaxf(__fsub_rd(br[i], lq.hi[j]), __fsub_rd(lq.lo[j], br[d + i]));
      oa = oa > 0.f ? oa : 0.f;
      ob = ob > 0.f ? ob : 0.f;
      a = fold_lb<M>(a, red_lb<M>(oa));
      b = fold_lb<M>(b, red_lb<M>(ob));
    }
  }
#pragma unroll
  for (int s = 16; s; s >>= 1) {
    a = fold_lb<M>(a, __shfl_xor_sync(FULL_MASK, a, s));
    b = fold_lb<M>(b, __shfl_xor_sync(FULL_MASK, b, s));
  }
  *lb_l = __fmul_rd(a, LB_SHRINK);
  *lb_r = __fmul_rd(b, LB_SHRINK);
}

// A warp's scratch for WarpList::offer_all: the merged list, one slot a rank.
struct WarpSlots {
  float lo[32], hi[32];
  uint32_t row[32], id[32];
  uint8_t chunk[32];
};

// ---------------------------------------------------------------------------
// The warp's sorted k best, KS slots per lane (k <= 32 KS): rank r lives in
// lane r % 32, slot r / 32.  An entry keeps an FP32 enclosure [lo, hi] of its
// exact FP64 distance (a one-point enclosure once that is known), its tree
// row and original index; entries are in exact (distance, index) order --
// BestK's (src/query.rs:461-481).  A candidate's rank comes from enclosure
// comparisons; only entries whose enclosure overlaps the candidate's compute
// exact values (one lane each, in parallel), and the candidate's own exact
// value is computed then too.  Empty slots: row ROW_NONE, after everything.
// Offers are warp-uniform (every lane passes the same candidate).
//
// `runner` is the FP32 lower bound of every dropped point (see the note on
// near ties at the top of this file); the reference-order kernel ignores it.
// ---------------------------------------------------------------------------
template <int M, int D, int KS>
struct WarpList {
  float lo[KS], hi[KS];
  uint32_t row[KS], id[KS];
  bool chunk[KS];  // the point lies in a full Packed d4 / d8 chunk (kernel.rs:517-562)
  uint32_t k, lane;
  uint64_t cut_bits;
  float cut_lo, cut_hi;
  float bound32;   // FP32 upper bound of min(k-th best, cutoff)
  float bound_lo;  // FP32 lower bound of min(k-th best, cutoff)
  float runner;
  const double* q;
  const double* data;
  uint32_t d;
  int strat;
  double pexp;

  __device__ __forceinline__ double exact_of(uint32_t r, bool in_chunk) const {
    if constexpr (D > 0) {
      QMem<D> qm;
      qm.g = q;
      return exact_dist<M, D>(qm, data + static_cast<uint64_t>(r) * D, D, S_PACKED, in_chunk, pexp);
    } else {
      QVec<0> qv;
      qv.g = q;
      return exact_dist<M, 0>(qv, data + static_cast<uint64_t>(r) * d, d, strat, in_chunk, pexp);
    }
  }
  __device__ __forceinline__ void init(uint32_t k_, double cutoff, uint32_t lane_, const double* qg,
                                       const double* data_, uint32_t d_, double pexp_) {
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
    q = qg;
    data = data_;
    d = d_;
    pexp = pexp_;
    strat = (M != M_LP && d_ <= 8) ? S_PACKED : ((M == M_L1 || M == M_L2) && d_ <= 16 ? S_FOLDED : S_STREAMED);
    runner = __int_as_float(0x7f800000);
    refresh();
  }
  __device__ __forceinline__ void note(float x) { runner = fminf(runner, x); }
  __device__ __forceinline__ void refresh() {
    const uint32_t r = k - 1;
    float kth = __shfl_sync(FULL_MASK, hi[0], static_cast<int>(r & 31));
    float kl = __shfl_sync(FULL_MASK, lo[0], static_cast<int>(r & 31));
#pragma unroll
    for (int s = 1; s < KS; ++s) {
      const float h = __shfl_sync(FULL_MASK, hi[s], static_cast<int>(r & 31));
      const float l = __shfl_sync(FULL_MASK, lo[s], static_cast<int>(r & 31));
      if (r / 32 == static_cast<uint32_t>(s)) {
        kth = h;
        kl = l;
      }
    }
    bound32 = fminf(kth, cut_hi);
    bound_lo = fminf(kl, cut_lo);
  }
  // Exact min(k-th best, cutoff) as bits (query.rs:452-459); the k-th entry's
  // enclosure tightens to its exact value.
  __device__ __forceinline__ uint64_t bound_exact() {
    const uint32_t r = k - 1;
    uint64_t kb = INF_BITS;
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      uint64_t xb = INF_BITS;
      const bool mine = lane == (r & 31) && r / 32 == static_cast<uint32_t>(s);
      if (mine && row[s] != ROW_NONE) {
        xb = dbits(exact_of(row[s], chunk[s]));
        lo[s] = mag_dn32(xb);
        hi[s] = mag_up32(xb);
      }
      xb = __shfl_sync(FULL_MASK, xb, static_cast<int>(r & 31));
      if (r / 32 == static_cast<uint32_t>(s)) kb = xb;
    }
    refresh();
    return kb < cut_bits ? kb : cut_bits;
  }
  // A dropped point (tree row r; warp-uniform arguments) whose exact distance
  // is at least lb: noted, by lane 0, as near_window (kd_query_common.cuh)
  // describes.
  __device__ __forceinline__ void note_point(float lb, uint32_t r, bool in_chunk) {
    if (lb > near_window(bound32)) return;
    if (lane == 0) note(mag_dn32(dbits(exact_of(r, in_chunk))));
  }
  // Offer the candidate at tree row cr (original index cid) whose exact
  // distance lies in [cl, ch]; warp-uniform arguments.
  __device__ __forceinline__ void offer(float cl, float ch, uint32_t cr, uint32_t cid, bool cchunk) {
    if (cl > bound32) {
      note_point(cl, cr, cchunk);
      return;
    }
    uint64_t cx_bits = 0;
    bool have_x = false;
    if (!(ch <= cut_lo)) {  // the cutoff test, unless clearly inside
      if (cl > cut_hi) return;
      cx_bits = dbits(exact_of(cr, cchunk));
      have_x = true;
      if (cx_bits > cut_bits) return;  // outside max_distance: not a candidate at all
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
      note_point(cl, cr, cchunk);
      refresh();  // enclosures may have tightened
      return;
    }
    // the k-th entry, if real, drops out: its owner lane keeps its row and
    // lower enclosure, noted against the bound after the insert
    float ev_lo = __int_as_float(0x7f800000);
    uint32_t ev_row = ROW_NONE;
    bool ev_chunk = false;
    {
      const uint32_t r = k - 1;
#pragma unroll
      for (int s = 0; s < KS; ++s)
        if (lane == (r & 31) && r / 32 == static_cast<uint32_t>(s) && row[s] != ROW_NONE) {
          ev_lo = lo[s];
          ev_row = row[s];
          ev_chunk = chunk[s];
        }
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
#pragma unroll
    for (int s = 1; s < KS; ++s) {  // lane 0 of slot s takes lane 31 of slot s - 1
      const float wl = __shfl_sync(FULL_MASK, lo[s - 1], 31), wh = __shfl_sync(FULL_MASK, hi[s - 1], 31);
      const uint32_t wr = __shfl_sync(FULL_MASK, row[s - 1], 31), wi = __shfl_sync(FULL_MASK, id[s - 1], 31);
      const bool wc = __shfl_sync(FULL_MASK, static_cast<int>(chunk[s - 1]), 31);
      if (lane == 0) {
        up_lo[s] = wl;
        up_hi[s] = wh;
        up_row[s] = wr;
        up_id[s] = wi;
        up_chunk[s] = wc;
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
    if (ev_row != ROW_NONE && !(ev_lo > near_window(bound32))) note(mag_dn32(dbits(exact_of(ev_row, ev_chunk))));
  }
  // Offer the candidates of one leaf chunk together (one slot a lane, k <=
  // 32): lane j's (cl, ch, cr, cid, cchunk) where `mine`, `mask` the ballot
  // of `mine`.  Each candidate is ranked against the entries and the other
  // candidates on enclosures alone, and the first k of the merged order come
  // back through `sl`: the list that offering them one at a time would leave,
  // since that list too is the k first of the entries and the candidates in
  // exact order.  When two enclosures overlap (an exact value would be
  // needed) or a candidate may lie outside max_distance, nothing changes and
  // it returns false: the caller then offers them one at a time.  Dropped
  // points (the evicted entries, the candidates ranked k or later) are noted
  // against the bound after the merge.
  __device__ __forceinline__ bool offer_all(bool mine, float cl, float ch, uint32_t cr, uint32_t cid, bool cchunk,
                                            uint32_t mask, WarpSlots* sl) {
    static_assert(KS == 1, "one slot a lane");
    if (!__all_sync(FULL_MASK, !mine || ch <= cut_lo)) return false;
    const bool entry = lane < k && row[0] != ROW_NONE;
    uint32_t e_rank = lane;  // this lane's entry: its rank plus the candidates before it
    uint32_t c_rank = 0;     // this lane's candidate: the entries and candidates before it
    bool amb = false;
    for (uint32_t m = mask; m; m &= m - 1) {  // uniform
      const int c = __ffs(m) - 1;
      const float xl = __shfl_sync(FULL_MASK, cl, c), xh = __shfl_sync(FULL_MASK, ch, c);
      const bool e_first = entry && hi[0] < xl;
      const bool x_first = entry && xh < lo[0];
      amb |= entry && !e_first && !x_first;
      e_rank += x_first ? 1u : 0u;
      if (mine && c != static_cast<int>(lane)) {
        const bool y_first = xh < cl;
        amb |= !y_first && !(ch < xl);
        c_rank += y_first ? 1u : 0u;
      }
      const uint32_t eb = __popc(__ballot_sync(FULL_MASK, e_first));
      if (c == static_cast<int>(lane)) c_rank += eb;
    }
    if (__any_sync(FULL_MASK, amb)) return false;
    const float inf = __int_as_float(0x7f800000);
    if (lane < k) {
      sl->lo[lane] = inf;
      sl->hi[lane] = inf;
      sl->row[lane] = ROW_NONE;
      sl->id[lane] = NO_ID;
      sl->chunk[lane] = 0;
    }
    __syncwarp();
    if (entry && e_rank < k) {
      sl->lo[e_rank] = lo[0];
      sl->hi[e_rank] = hi[0];
      sl->row[e_rank] = row[0];
      sl->id[e_rank] = id[0];
      sl->chunk[e_rank] = chunk[0] ? 1 : 0;
    }
    if (mine && c_rank < k) {
      sl->lo[c_rank] = cl;
      sl->hi[c_rank] = ch;
      sl->row[c_rank] = cr;
      sl->id[c_rank] = cid;
      sl->chunk[c_rank] = cchunk ? 1 : 0;
    }
    __syncwarp();
    const bool evicted = entry && e_rank >= k;
    const float ev_lo = lo[0];
    const uint32_t ev_row = row[0];
    const bool ev_chunk = chunk[0];
    if (lane < k) {
      lo[0] = sl->lo[lane];
      hi[0] = sl->hi[lane];
      row[0] = sl->row[lane];
      id[0] = sl->id[lane];
      chunk[0] = sl->chunk[lane] != 0;
    }
    __syncwarp();  // the slots are free again
    refresh();
    const float win = near_window(bound32);
    if (evicted && !(ev_lo > win)) note(mag_dn32(dbits(exact_of(ev_row, ev_chunk))));
    if (mine && c_rank >= k && !(cl > win)) note(mag_dn32(dbits(exact_of(cr, cchunk))));
    return true;
  }
  // write_results (query.rs:421-429, 483-493): lane j writes rank j (and
  // 32 + j, ...); the entries are in exact order already, their exact values
  // are computed once here.  Returns (to every lane) whether the query is a
  // near tie (see the top of this file); `track` = false skips that test.
  __device__ __forceinline__ bool write(double* od, int64_t* oi, uint64_t n_points, bool track) {
    uint64_t dmax = 0;
    bool any = false;
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const uint32_t r = lane + 32u * s;
      if (r < k) {
        const bool real = row[s] != ROW_NONE;
        double x = bitsd(INF_BITS);
        if (real) {
          x = exact_of(row[s], chunk[s]);
          dmax = dbits(x) > dmax ? dbits(x) : dmax;
          any = true;
        }
        od[r] = real ? restore<M>(x, pexp) : bitsd(INF_BITS);
        oi[r] = real ? static_cast<int64_t>(id[s]) : static_cast<int64_t>(n_points);
      }
    }
    if (!track) return false;
    float rn = runner;
#pragma unroll
    for (int s = 16; s; s >>= 1) {
      rn = fminf(rn, __shfl_xor_sync(FULL_MASK, rn, s));
      const uint64_t o = __shfl_xor_sync(FULL_MASK, dmax, s);
      dmax = o > dmax ? o : dmax;
    }
    if (!__any_sync(FULL_MASK, any)) return false;  // nothing within max_distance: nothing to leave out
    const float g = near_window(mag_up32(dmax));
    return rn <= g || cut_lo <= g;
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
  WarpSlots slots;  // WarpList::offer_all's merge
};
