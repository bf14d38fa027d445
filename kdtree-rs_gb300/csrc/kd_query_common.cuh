// kd_query_common.cuh -- the query kernels' shared vocabulary: launch arguments,
// the reference's metric algebra and FP64 distance orders (exact, never
// contracted), and the FP32 interval helpers the filters are built from.
// Included inside namespace kd { namespace { ... } } by each query translation
// unit, so every unit gets its own internal copies.
#pragma once

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

// A query read from memory at each use.  The k-best lists of the filtered
// traversals need the FP64 query only for the rare exact distances; holding
// it in registers across their FP32 row loops keeps 2 D registers live that
// the FP32 copies were derived from.
template <int D>
struct QMem {
  const double* g;
  __device__ __forceinline__ double operator[](uint64_t i) const { return g[i]; }
};

// ---------------------------------------------------------------------------
// Exact reduced point distance (src/kernel.rs:163-218, 343-354, 411-562).
// `in_chunk`: the point lies inside a full Packed chunk of its leaf (d4: pairs,
// d8: groups of 8); only then do d4 / d8 use their pairwise orders.
// ---------------------------------------------------------------------------
template <int M, int D, class Q>
__device__ __forceinline__ double exact_dist(const Q& q, const double* p, uint64_t d, int strat, bool in_chunk,
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
  if (D > 8) strat = D <= 16 ? S_FOLDED : S_STREAMED;  // L1 / L2 above 8 (kernel.rs:244-270)
  if (D > 0 && D <= 8) {
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
  if (D > 0) d = D;
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
// FP32 interval bounds with directed rounding.
//
// A double x is enclosed by FP32 values: q32 = RN(q) gives
// q in [q32 - e, q32 + e], e = 2^-24 |q32| + 2^-149 (likewise the RN copies of
// the points); a double converted through its bits (mag_dn32 / mag_up32) is
// bracketed directly.  Interval sums, differences and squares rounded toward
// the safe side give an FP32 lower bound lb and upper bound ub of the exact real
// distance.  The FP64 value the reference computes from the same inputs is
// within (d + 3) relative roundings of 2^-53 of that real value, so with the
// FP64 pruning bound b enclosed as [b_lo, b_hi] = [b (1 - 2^-20), b (1 + 2^-20)]
// (rounded outward):
//   lb > b_hi  implies  exact > b   (the reference rejects: skip it),
//   ub < b_lo  implies  exact <= b  (the reference admits: no FP64 needed),
// and only the remaining cases compute the exact FP64 value.  Non-finite FP32
// values (inputs beyond FP32 range) make lb 0 and ub inf, deciding nothing.
// ---------------------------------------------------------------------------
constexpr float TWO_M24 = 5.9604645e-08f;  // 2^-24
constexpr float TWO_M23 = 1.1920929e-07f;  // 2^-23
constexpr float TINY32 = 1.4e-45f;         // 2^-149
constexpr float LB_SHRINK = 0.99999905f;   // 1 - 2^-20 (exact in FP32)
constexpr float UB_GROW = 1.0000010f;      // 1 + 2^-20 (exact in FP32)

// |x| of a double given by its bits, rounded down / up to FP32.
__device__ __forceinline__ float mag_dn32(uint64_t b) {
  b &= 0x7fffffffffffffffull;
  const int e = static_cast<int>(b >> 52) - 896;  // FP32 biased exponent
  if ((b >> 52) == 0x7ff) return (b & 0xfffffffffffffull) ? 0.f : __int_as_float(0x7f800000);
  if (e >= 255) return 3.40282347e38f;
  if (e <= 0) return 0.f;
  return __uint_as_float((static_cast<uint32_t>(e) << 23) | static_cast<uint32_t>((b >> 29) & 0x7fffffu));
}
__device__ __forceinline__ float mag_up32(uint64_t b) {
  b &= 0x7fffffffffffffffull;
  if (b == 0) return 0.f;
  const int e = static_cast<int>(b >> 52) - 896;
  if (e >= 255) return __int_as_float(0x7f800000);
  if (e <= 0) return 1.17549435e-38f;  // FLT_MIN bounds everything below it
  uint32_t r = (static_cast<uint32_t>(e) << 23) | static_cast<uint32_t>((b >> 29) & 0x7fffffu);
  if (b & 0x1fffffffull) r += 1;  // carries into the exponent (or to +inf) correctly
  return __uint_as_float(r);
}
// Signed double (bits) rounded down / up to FP32.
__device__ __forceinline__ float rd32(uint64_t b) { return (b >> 63) ? -mag_up32(b) : mag_dn32(b); }
__device__ __forceinline__ float ru32(uint64_t b) { return (b >> 63) ? -mag_dn32(b) : mag_up32(b); }

// Enclosure [lo, hi] of a double whose FP32 round-to-nearest copy is x32.
__device__ __forceinline__ void rn_enclose(float x32, float* lo, float* hi) {
  const float e = __fmaf_ru(fabsf(x32), TWO_M24, TINY32);
  *lo = __fsub_rd(x32, e);
  *hi = __fadd_ru(x32, e);
}
// Lower / upper bound of |x - y| for x in [xl, xh], y in [yl, yh].
__device__ __forceinline__ float absdiff_lb(float xl, float xh, float yl, float yh) {
  const float a = __fsub_rd(xl, yh), b = __fsub_rd(yl, xh);
  const float m = a > b ? a : b;
  return m > 0.f ? m : 0.f;  // NaN lands on 0
}
__device__ __forceinline__ float absdiff_ub(float xl, float xh, float yl, float yh) {
  const float a = __fsub_ru(xh, yl), b = __fsub_ru(yh, xl);
  return fmaxf(fmaxf(a, b), 0.f);
}
template <int M>
__device__ __forceinline__ float red_lb(float t) {  // reduce(), rounded down
  return M == M_L2 ? __fmul_rd(t, t) : t;
}
template <int M>
__device__ __forceinline__ float red_ub(float t) {
  return M == M_L2 ? __fmul_ru(t, t) : t;
}
template <int M>
__device__ __forceinline__ float fold_lb(float acc, float t) {  // fold(), rounded down
  if (M == M_LINF) return acc > t ? acc : t;
  return __fadd_rd(acc, t);
}
template <int M>
__device__ __forceinline__ float fold_ub(float acc, float t) {
  if (M == M_LINF) return fmaxf(acc, t);
  return __fadd_ru(acc, t);
}

// dist <= bound for a non-negative bound given by its bits, with dist of any
// sign: a cell bound fl(fl(cell - old) + far_axis) can round slightly below
// zero, which f64 '<=' admits; NaN never is.
__device__ __forceinline__ bool leq_bound(double dist, uint64_t bound_bits) {
  const uint64_t b = dbits(dist);
  if (b >> 63) return (b & 0x7fffffffffffffffull) <= INF_BITS;
  return b <= bound_bits;
}

// The IEEE order of finite doubles as an unsigned key (-0 folded onto +0), so
// the near-child test q[dim] <= split (query.rs:263-268) is an integer compare.
__device__ __forceinline__ uint64_t ieee_key(uint64_t b) {
  uint64_t k = total_key_bits(b);
  return k == 0x7fffffffffffffffull ? 0x8000000000000000ull : k;
}

// x (1 + 2^-20) rounded up, never below the smallest normal FP32: the near-tie
// window above a distance's upper enclosure.  A query is a near tie when a
// point it dropped (within max_distance) may lie inside the window above its
// k-th distance.  The window only shrinks as the bound does, so a dropped
// point whose lower bound exceeds the window of the present bound never
// counts; one whose bound is inside is noted by its exact distance (a loose
// FP32 enclosure there would flag queries whose dropped points are not ties).
__device__ __forceinline__ float near_window(float x) { return fmaxf(__fmul_ru(x, UB_GROW), 1.17549435e-38f); }

// FP32 rows the filters read: the copy padded to w32 floats for width 3 (4
// floats: one 16-byte load a row) and the runtime widths (D = 0), the plain
// copy for the other compile-time widths.
template <int D>
__device__ __forceinline__ const float* filter_rows(const QArgs& a) {
  return (D == 0 || D == 3) ? a.data32w : a.data32;
}
template <int D>
__device__ __forceinline__ uint64_t filter_stride(const QArgs& a) {
  return D == 3 ? 4 : (D > 0 ? static_cast<uint64_t>(D) : a.w32);
}

// Append query qi (with the launch's tag) to the list of queries whose eps = 0
// fast-path result is a near tie and must be run again in the reference's
// order (kd_warp.cuh, kd_query_ref.cuh).
__device__ __forceinline__ void flag_rerun(const QArgs& a, uint64_t qi) {
  if (!a.rerun_count) return;
  const uint32_t pos = atomicAdd(a.rerun_count, 1u);
  a.rerun_list[pos] = (static_cast<uint64_t>(a.rerun_tag) << 32) | static_cast<uint32_t>(qi);
}
