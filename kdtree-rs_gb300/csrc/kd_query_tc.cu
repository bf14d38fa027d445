// kd_query_tc.cu -- exact k-NN at higher dimension through a tcgen05 tensor-core
// distance filter (L2, eps = 0, 16 <= d <= 128, k <= 32).
//
// At d = 64 a kd-tree descent visits about half of all points (the split planes
// stop pruning), so this path scores every (query, point) pair -- as a GEMM on
// the tensor cores -- and uses that score only as a filter:
//
//   rows are centred (p - c, q - c; c = root box centre) and rounded to BF16;
//   acc = q_b . p_b on tcgen05 (BF16 x BF16, FP32 accumulation in TMEM);
//   a pair is rejected when  w_p - 2 acc - 2 R_q v_p > T_q,
//     w_p = |p_b|^2 (1 - 2^-12) - v_p^2,  v_p = 2^-8 |p_b|,
//     R_q = sqrt(b) + 2^-8 |q_b| + 2^-126,  T_q = R_q^2 - |q_b|^2 (1 - 2^-12),
//   which implies |q - p| > sqrt(b) for the exact real distance: every BF16
//   coordinate is within 2^-8 of its (centred) value relative, so
//   |q - p| >= |q_b - p_b| - 2^-8 (|q_b| + |p_b|), and the 2^-12 slack covers the
//   FP32 norms, the tensor cores' FP32 accumulation (taken as <= 2^-15 of
//   sum |q_i p_i|) and the FP32 rounding of the test itself.  b is an FP32 upper
//   enclosure of the query's current pruning bound (its k-th best so far).
//
// Pairs that survive are refined with the FP32 copy of the coordinates into an
// enclosure of the exact FP64 distance and offered to the query's k-best set
// (LazySetDyn), which computes the reference's exact FP64 distance (Folded order
// for d <= 16, Streamed above, kernel.rs) only when two enclosures overlap and
// for the final k.  The result is the k smallest (exact FP64 distance, index)
// within max_distance -- the reference's answer for eps = 0 unless a near tie
// lets the reference's own descent leave one of them out; those queries are
// flagged (every dropped pair's lower bound is tracked, skipped tiles through
// their box bound) and run again in the reference's order (kd_query_ref.cuh).
//
// Pipeline (one persistent CTA per SM, a 128-query tile at a time):
//   warp 0  TMA: the query tile once, then 256-point tiles into a ring of
//           stages, nearest tiles first; a point tile whose FP32 box bound to
//           the query tile's box exceeds the largest current bound of the
//           query tile's rows is skipped (clustered data: the tiles of other
//           clusters), and an end marker closes the query tile
//   warp 1  tcgen05.mma: 128 x 256 x d into one of two TMEM accumulators
//   warps 2-5  epilogue: tcgen05.ld one accumulator row per thread, filter,
//              refine, offer; free the accumulator for the next tile; publish
//              the warp's largest bound for the producer's skip test.
// Every wait is bounded; a timeout sets an error bit and all roles leave.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "kd_internal.hpp"

namespace kd {

namespace {

#include "kd_query_common.cuh"
#include "kd_lazy_best.cuh"

constexpr int TC_M = 128;        // queries per tile (MMA M)
constexpr int TC_N = 256;        // points per tile (MMA N)
constexpr int TC_KC = 64;        // BF16 elements per 128-byte swizzled row chunk
constexpr int TC_THREADS = 192;  // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr uint32_t TC_SPIN = 1u << 22;
constexpr uint32_t TC_STATUS_TIMEOUT = 2u;
constexpr uint32_t TC_END = 0xffffffffu;  // stage / accumulator marker: the query tile is done

struct TcArgs {
  const double* queries;  // nq x d, FP64
  const double* data;     // tree-ordered points, FP64
  const float* data32;    // tree-ordered points, FP32
  const uint32_t* indices;
  const uint32_t* order;  // sorted row -> query index (rows are grouped by landing leaf)
  const uint32_t* tile_start;  // per query tile: the point tile holding its landing leaf
  const float* q32;       // nq x w32, FP32 copies of the queries (zero padded), in sorted row order
  const float* data32w;   // tree-ordered points, FP32, rows padded to w32 floats (zeros)
  uint32_t w32;           // d rounded up to a multiple of 4
  const float* qn2;       // |q_b|^2, FP32 sum
  const float* qnorm;     // |q_b| rounded up
  const float* pw;        // per point w (padded to whole tiles with +inf)
  const float* pv;        // per point v (padding 0)
  const float* qbox;      // per query tile: [lo | hi] FP32 enclosure of its queries (d each)
  const float* tbox;      // per point tile: [lo | hi] FP32 enclosure of its points (d each)
  double* out_d;
  int64_t* out_i;
  uint32_t* status;
  unsigned long long* survivors;
  uint32_t* rerun_count;  // near ties: query indices appended to rerun_list
  uint64_t* rerun_list;
  uint64_t nq, n_points, d, k;
  double cutoff;
  float coord_max;
  int strat;
  uint32_t n_qt, n_pt, kch, nst;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Bounded wait for the phase with the given parity; gives up on abort.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
  for (uint32_t i = 0; i < TC_SPIN; ++i) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (*abort_flag) return false;
  }
  return false;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// K-major operand in 128-byte swizzled rows: 8-row atoms 1024 B apart.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  return static_cast<uint64_t>((saddr & 0x3FFFF) >> 4) | (static_cast<uint64_t>(1024 >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Filter constants of one query from its current bound enclosure b (sqrt(b)
// bounded above from rsqrtf, within 3 units in the last place, grown by 2^-19).
__device__ __forceinline__ void tc_threshold(float b, float qn2, float qnorm, float* m2r, float* thr) {
  const float sb = !(b > 0.f) ? 0.f : (!(b <= 3.4e38f) ? b : __fmul_ru(b * rsqrtf(b), 1.0000020f /* 1 + 2^-19 */));
  const float r = __fadd_ru(sb, __fmaf_ru(qnorm, 0.00390625f /* 2^-8 */, 1.1754944e-38f /* 2^-126 */));
  *m2r = -2.f * r;
  *thr = __fsub_ru(__fmul_ru(r, r), __fmul_rd(qn2, 0.99975586f /* 1 - 2^-12 */));
}

// The i-th point tile a query tile visits: its own tile s first, then
// alternately the next and previous ones (s, s+1, s-1, s+2, ...) -- rows are in
// tree order, so nearby tiles hold nearby points and bounds tighten early.
__device__ __forceinline__ uint32_t zigzag(uint32_t s, uint32_t i, uint32_t n) {
  const uint32_t left = s, right = n - 1 - s, m = left < right ? left : right;
  if (i == 0) return s;
  if (i <= 2 * m) {
    const uint32_t j = (i + 1) / 2;
    return (i & 1) ? s + j : s - j;
  }
  const uint32_t off = i - 2 * m;
  return right > left ? s + m + off : s - m - off;
}

// Lower bound of the exact FP64 reduced distance between any query of a tile
// and any point of a tile, from their FP32 box enclosures ([lo | hi], d each):
// per-axis gaps rounded down, squared and summed rounded down, then the FP64
// rounding margin of box_lb.
__device__ __forceinline__ float tile_lb(const float* qb, const float* tb, uint64_t d) {
  float lb = 0.f;
  for (uint64_t i = 0; i < d; ++i) {
    float o = fmaxf(__fsub_rd(tb[i], qb[d + i]), __fsub_rd(qb[i], tb[d + i]));
    o = o > 0.f ? o : 0.f;
    lb = __fadd_rd(lb, __fmul_rd(o, o));
  }
  return __fmul_rd(lb, LB_SHRINK);
}

template <int K>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_query_tc(const __grid_constant__ CUtensorMap tmap_q, const __grid_constant__ CUtensorMap tmap_p, TcArgs a) {
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t kch = a.kch, nst = a.nst;
  const uint32_t q_bytes = kch * TC_M * 128, p_bytes = kch * TC_N * 128;
  unsigned char* s_q = smem;
  unsigned char* s_p = smem + q_bytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_p + nst * p_bytes);
  uint64_t* full = bars;             // [nst] TMA -> MMA
  uint64_t* empty = bars + nst;      // [nst] MMA -> TMA
  uint64_t* accf = bars + 2 * nst;   // [2] MMA -> epilogue
  uint64_t* acce = accf + 2;         // [2] epilogue -> MMA
  uint64_t* qfull = acce + 2;        // query tile loaded
  uint64_t* qempty = qfull + 1;      // query tile no longer read
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  __shared__ unsigned long long s_surv;
  __shared__ int s_zero;  // a flag that never rises: the drain waits ignore aborts
  __shared__ uint32_t s_tile[4];      // per stage: the point tile it holds, or TC_END
  __shared__ uint32_t s_acc_tile[2];  // per accumulator: the point tile it scored, or TC_END
  __shared__ float s_skip[4];         // per stage holding TC_END: the smallest box bound of the tiles skipped
  __shared__ float s_acc_skip[2];     // ... passed on with the accumulator's TC_END
  __shared__ float s_wb[4];           // per epilogue warp: the largest bound of its rows ...
  __shared__ uint32_t s_wq[4];        // ... for the CTA's query tile number s_wq
  volatile int* abort_flag = &s_abort;
  volatile uint32_t* v_tile = s_tile;
  volatile uint32_t* v_acc_tile = s_acc_tile;
  volatile float* v_skip = s_skip;
  volatile float* v_acc_skip = s_acc_skip;
  volatile float* v_wb = s_wb;
  volatile uint32_t* v_wq = s_wq;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < nst; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&accf[b]), 2);  // the MMA thread's arrive (tile id) + the MMA commit
      mbar_init(smem_u32(&acce[b]), 4 * 32);
    }
    for (int w = 0; w < 4; ++w) {
      s_wb[w] = __int_as_float(0x7f800000);
      s_wq[w] = TC_END;
    }
    mbar_init(smem_u32(qfull), 1);
    mbar_init(smem_u32(qempty), 1);
    s_abort = 0;
    s_zero = 0;
    s_surv = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
    asm volatile("fence.proxy.async.shared::cta;");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(2 * TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;

  if (warp == 0) {
    // ---------------- TMA producer (the whole warp decides, lane 0 issues) ----------------
    // A point tile is skipped when its box bound exceeds the largest current
    // bound of the query tile's rows (published by the epilogue warps for this
    // query tile; none published yet: nothing is skipped).  Bounds only shrink,
    // so every skipped pair is farther than its query's final k-th best.
    uint32_t ld = 0, qj = 0;
    uint32_t last_use[4] = {0, 0, 0, 0};
    int ok = 1;
    for (uint32_t qt = blockIdx.x; qt < a.n_qt && ok; qt += gridDim.x, ++qj) {
      if (lane == 0) {
        ok = mbar_wait(smem_u32(qempty), (qj & 1) ^ 1, abort_flag);
        if (ok) {
          mbar_expect_tx(smem_u32(qfull), q_bytes);
          for (uint32_t kc = 0; kc < kch; ++kc)
            tma_load_2d(smem_u32(s_q + kc * TC_M * 128), &tmap_q, kc * TC_KC, qt * TC_M, smem_u32(qfull));
        }
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      const float* qb = a.qbox + static_cast<uint64_t>(qt) * 2 * a.d;
      float skip_min = __int_as_float(0x7f800000);  // lane 0: the skipped tiles' smallest box bound
      for (uint32_t p0 = 0; p0 < a.n_pt && ok; p0 += 32) {
        const uint32_t pt = p0 + lane;
        uint32_t tile = 0;
        float lb = __int_as_float(0x7f800000);
        if (pt < a.n_pt) {
          tile = zigzag(a.tile_start[qt], pt, a.n_pt);
          lb = tile_lb(qb, a.tbox + static_cast<uint64_t>(tile) * 2 * a.d, a.d);
        }
        for (int j = 0; j < 32 && ok; ++j) {
          const uint32_t tj = __shfl_sync(0xffffffffu, tile, j);
          const float lbj = __shfl_sync(0xffffffffu, lb, j);
          if (p0 + j >= a.n_pt) break;
          if (lane == 0) {
            bool cur = true;
            for (int w = 0; w < 4; ++w) cur = cur && v_wq[w] == qj;
            __threadfence_block();
            float bound = __int_as_float(0x7f800000);
            if (cur) bound = fmaxf(fmaxf(v_wb[0], v_wb[1]), fmaxf(v_wb[2], v_wb[3]));
            if (lbj > bound) {
              skip_min = fminf(skip_min, lbj);
            } else {
              const uint32_t s = ld % nst, u = ld / nst;
              ok = mbar_wait(smem_u32(&empty[s]), (u & 1) ^ 1, abort_flag);
              if (ok) {
                v_tile[s] = tj;
                unsigned char* dst = s_p + s * p_bytes;
                mbar_expect_tx(smem_u32(&full[s]), p_bytes);
                for (uint32_t kc = 0; kc < kch; ++kc)
                  tma_load_2d(smem_u32(dst + kc * TC_N * 128), &tmap_p, kc * TC_KC, tj * TC_N, smem_u32(&full[s]));
                last_use[s] = u + 1;
              }
              ++ld;
            }
          }
          ok = __shfl_sync(0xffffffffu, ok, 0);
        }
      }
      if (!ok) break;
      if (lane == 0) {  // the query tile's end marker
        const uint32_t s = ld % nst, u = ld / nst;
        ok = mbar_wait(smem_u32(&empty[s]), (u & 1) ^ 1, abort_flag);
        if (ok) {
          v_tile[s] = TC_END;
          v_skip[s] = skip_min;
          mbar_arrive(smem_u32(&full[s]));
          last_use[s] = u + 1;
        }
        ++ld;
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
    }
    // Leaving early (its own wait ran out, or another role's did): let the
    // copies already issued land before the CTA leaves.
    if (lane == 0 && !ok) atomicExch(&s_abort, 1);
    if (lane == 0 && (!ok || *abort_flag)) {
      for (uint32_t s = 0; s < nst; ++s)
        if (last_use[s]) mbar_wait(smem_u32(&full[s]), (last_use[s] - 1) & 1, &s_zero);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((static_cast<uint32_t>(TC_N) >> 3) << 17) |
                             ((static_cast<uint32_t>(TC_M) >> 4) << 24);
      uint32_t ld = 0, t = 0, qj = 0;
      bool ok = true;
      for (uint32_t qt = blockIdx.x; qt < a.n_qt && ok; qt += gridDim.x, ++qj) {
        if (!mbar_wait(smem_u32(qfull), qj & 1, abort_flag)) {
          ok = false;
          break;
        }
        for (;;) {  // the producer's tiles for this query tile, up to its end marker
          const uint32_t b = t & 1, ub = t >> 1;
          const uint32_t s = ld % nst, us = ld / nst;
          if (!mbar_wait(smem_u32(&acce[b]), (ub & 1) ^ 1, abort_flag) ||
              !mbar_wait(smem_u32(&full[s]), us & 1, abort_flag)) {
            ok = false;
            break;
          }
          const uint32_t tile = v_tile[s];
          ++ld;
          ++t;
          if (tile == TC_END) {
            v_acc_skip[b] = v_skip[s];
            mbar_arrive(smem_u32(&empty[s]));  // the stage carried no data
            v_acc_tile[b] = TC_END;
            mbar_arrive(smem_u32(&accf[b]));
            mbar_arrive(smem_u32(&accf[b]));
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t d_tmem = tmem + b * TC_N;
          for (uint32_t kc = 0; kc < kch; ++kc) {
            const uint64_t ad = umma_desc(smem_u32(s_q + kc * TC_M * 128));
            const uint64_t bd = umma_desc(smem_u32(s_p + s * p_bytes + kc * TC_N * 128));
#pragma unroll
            for (uint32_t k = 0; k < TC_KC / 16; ++k)
              umma_bf16(d_tmem, ad + 2 * k, bd + 2 * k, idesc, (kc | k) ? 1u : 0u);  // +32 B per K step
          }
          v_acc_tile[b] = tile;
          mbar_arrive(smem_u32(&accf[b]));  // publishes the tile id; the commit below completes the phase
          umma_commit(smem_u32(&empty[s]));
          umma_commit(smem_u32(&accf[b]));
        }
        if (ok) umma_commit(smem_u32(qempty));
      }
      if (!ok) atomicExch(&s_abort, 1);
    }
  } else {
    // ---------------- epilogue: one query row per thread ----------------
    const uint32_t quarter = static_cast<uint32_t>(warp & 3);  // TMEM lanes this warp may read
    const uint32_t row = quarter * 32 + lane;
    uint32_t t = 0, qj = 0;
    unsigned long long surv = 0;
    bool ok = true;
    for (uint32_t qt = blockIdx.x; qt < a.n_qt && ok; qt += gridDim.x, ++qj) {
      const uint64_t srow = static_cast<uint64_t>(qt) * TC_M + row;  // sorted row
      const bool active = srow < a.nq;
      const uint64_t qrow = active ? srow : 0;
      const uint64_t qi = a.order[qrow];  // the query's own index
      LazySetDyn<K> set;
      set.init(a.k, a.cutoff, DynPoint{a.queries + qi * a.d, a.data, a.d, a.strat}, a.indices);
      const float* q32 = a.q32 + qrow * a.w32;
      float qmax = 0.f;
      for (uint64_t i = 0; i < a.d; ++i) qmax = fmaxf(qmax, fabsf(q32[i]));
      // enclosure of a survivor's exact distance from its FP32 coordinates
      const float e = __fmaf_ru(__fadd_ru(a.coord_max, qmax), TWO_M24, 2.9e-45f);
      const float spread = __fmul_ru(e, __fsqrt_ru(static_cast<float>(a.d)));
      const float qn2 = a.qn2[qrow], qnorm = a.qnorm[qrow];
      float m2r, thr, m2r2, thr2;  // (m2r2, thr2): the near-tie band just above the bound
      tc_threshold(set.b_hi, qn2, qnorm, &m2r, &thr);
      tc_threshold(__fmul_ru(set.b_hi, 1.0000020f /* 1 + 2^-19 */), qn2, qnorm, &m2r2, &thr2);
      if (lane == 0) {  // this query tile's bound: none yet
        v_wb[warp - 2] = __int_as_float(0x7f800000);
        __threadfence_block();
        v_wq[warp - 2] = qj;
      }
      for (;;) {
        const uint32_t b = t & 1, ub = t >> 1;
        // warp-uniform outcome: the lanes below shuffle and load TMEM together
        if (!__all_sync(0xffffffffu, mbar_wait(smem_u32(&accf[b]), ub & 1, abort_flag))) {
          ok = false;
          break;
        }
        const uint32_t tile = v_acc_tile[b];
        ++t;
        if (tile == TC_END) {
          set.note(v_acc_skip[b]);  // every pair of a skipped tile is at least that far
          mbar_arrive(smem_u32(&acce[b]));
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = tile * TC_N;
        for (uint32_t c = 0; c < TC_N; c += 32) {
          uint32_t r[32];
          tmem_ld32(tmem + ((quarter * 32) << 16) + b * TC_N + c, r);
          const float4* w4 = reinterpret_cast<const float4*>(a.pw + base + c);
          const float4* v4 = reinterpret_cast<const float4*>(a.pv + base + c);
          uint32_t mask = 0, band = 0;
#pragma unroll
          for (int j4 = 0; j4 < 8; ++j4) {
            const float4 w = __ldg(w4 + j4), v = __ldg(v4 + j4);
            const float ww[4] = {w.x, w.y, w.z, w.w}, vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int j = j4 * 4 + u;
              const float x0 = __fmaf_rn(-2.f, __uint_as_float(r[j]), ww[u]);
              const float x = __fmaf_rn(m2r, vv[u], x0);
              mask |= static_cast<uint32_t>(!(x > thr)) << j;
              band |= static_cast<uint32_t>(!(__fmaf_rn(m2r2, vv[u], x0) > thr2)) << j;
            }
          }
          if (!active) mask = band = 0;
          // survivors, and the pairs the filter rejected inside the near-tie
          // band (farther than the bound): those are noted by their FP32
          // enclosure, and by their exact value when it lies in the window
          uint32_t todo = mask | band;
          while (todo) {
            const uint32_t j = __ffs(todo) - 1;
            todo &= todo - 1;
            const bool survivor = (mask >> j) & 1u;
            const uint32_t p = base + c + j;
            if (p >= a.n_points) continue;
            surv += survivor;
            // FP32 sum of squares and its enclosure (triangle inequality, as the
            // packet filter; the sqrt margin 2^-16 covers d <= 128), in
            // dimension order from the zero-padded rows, four floats a load
            // and four loads in flight
            const float4* p4 = reinterpret_cast<const float4*>(a.data32w + static_cast<uint64_t>(p) * a.w32);
            const float4* q4 = reinterpret_cast<const float4*>(q32);
            float s2 = 0.f;
#pragma unroll 4
            for (uint32_t i = 0; i < a.w32 / 4; ++i) {
              const float4 pv4 = p4[i], qv4 = q4[i];
              float dd = __fsub_rn(pv4.x, qv4.x);
              s2 = __fmaf_rn(dd, dd, s2);
              dd = __fsub_rn(pv4.y, qv4.y);
              s2 = __fmaf_rn(dd, dd, s2);
              dd = __fsub_rn(pv4.z, qv4.z);
              s2 = __fmaf_rn(dd, dd, s2);
              dd = __fsub_rn(pv4.w, qv4.w);
              s2 = __fmaf_rn(dd, dd, s2);
            }
            const float rr = s2 > 0.f ? s2 * rsqrtf(s2) : 0.f;
            float clo = 0.f, chi = __int_as_float(0x7f800000);
            if (rr <= 3.4e38f) {
              const float lo = fmaxf(__fsub_rd(__fmul_rd(rr, 0.9999847f /* 1 - 2^-16 */), spread), 0.f);
              const float hi = __fadd_ru(__fmul_ru(rr, 1.0000153f /* 1 + 2^-16 */), spread);
              clo = __fmul_rd(__fmul_rd(lo, lo), LB_SHRINK);
              chi = __fmul_ru(__fmul_ru(hi, hi), UB_GROW);
            }
            if (!survivor || clo > set.b_hi) {
              set.note_point(clo, p);
              continue;
            }
            set.offer(clo, chi, p);
            tc_threshold(set.b_hi, qn2, qnorm, &m2r, &thr);
            tc_threshold(__fmul_ru(set.b_hi, 1.0000020f), qn2, qnorm, &m2r2, &thr2);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(smem_u32(&acce[b]));
        // publish the largest bound of this warp's rows
        float mb = active ? set.b_hi : 0.f;
#pragma unroll
        for (int off = 16; off; off >>= 1) mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, off));
        if (lane == 0) v_wb[warp - 2] = mb;
      }
      if (ok && active && set.write(a.out_d + qi * a.k, a.out_i + qi * a.k, a.k, a.n_points) && a.rerun_count)
        a.rerun_list[atomicAdd(a.rerun_count, 1u)] = qi;
    }
    if (!ok) atomicExch(&s_abort, 1);
    atomicAdd(&s_surv, surv);
  }

  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_abort) atomicOr(a.status, TC_STATUS_TIMEOUT);
    if (a.survivors) atomicAdd(a.survivors, s_surv);
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_N));
  }
}

// ---------------------------------------------------------------------------
// Inputs of the filter.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint16_t bf16_rn_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

// Centred BF16 rows (zero padded to dpad) and the per-row norm terms.
__global__ void k_tc_rows(const double* src, const uint32_t* order, uint64_t n, uint64_t d, uint32_t dpad,
                          const double* centre, uint16_t* dst, float* n2_out, float* norm_out, float* w_out,
                          float* v_out) {
  const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint64_t from = order ? order[i] : i;  // row i of the output holds source row `from`
  float n2 = 0.f;
  for (uint32_t j = 0; j < dpad; ++j) {
    uint16_t h = 0;
    if (j < d) {
      const double c = __dsub_rn(src[from * d + j], centre[j]);
      h = bf16_rn_bits(__double2float_rn(c));
      const float f = __bfloat162float(__ushort_as_bfloat16(h));
      n2 = __fmaf_rn(f, f, n2);  // BF16 squares are exact in FP32
    }
    dst[i * dpad + j] = h;
  }
  const float norm = __fsqrt_ru(__fmul_ru(n2, 1.0000610f /* 1 + 2^-14 */));
  if (n2_out) n2_out[i] = n2;
  if (norm_out) norm_out[i] = norm;
  if (w_out) {
    const float v = __fmul_ru(norm, 0.00390625f);
    v_out[i] = v;
    w_out[i] = __fsub_rd(__fmul_rd(n2, 0.99975586f), __fmul_ru(v, v));
  }
}

__global__ void k_tc_pad(float* w, float* v, uint64_t from, uint64_t to) {
  const uint64_t i = from + blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i < to) {
    w[i] = __int_as_float(0x7f800000);
    v[i] = 0.f;
  }
}

__global__ void k_f32_gather(const double* src, const uint32_t* order, uint64_t n, uint64_t d, uint64_t w,
                             float* dst) {
  const uint64_t f = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (f >= n * w) return;
  const uint64_t r = f / w, j = f - r * w;
  dst[f] = j < d ? __double2float_rn(src[static_cast<uint64_t>(order[r]) * d + j]) : 0.f;
}

// FP32 box enclosure ([lo | hi], d each) of each tile of `rows` consecutive
// rows of a row-major FP32 array: every coordinate's round-to-nearest copy x32
// stands for a value in [x32 - e, x32 + e] (rn_enclose).  One block per tile,
// thread j takes dimension j (blockDim >= d).
__global__ void k_tile_boxes(const float* x32, uint64_t n, uint64_t d, uint32_t rows, float* box) {
  const uint64_t t = blockIdx.x, j = threadIdx.x;
  if (j >= d) return;
  float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
  const uint64_t r0 = t * rows, r1 = min(n, r0 + rows);
  for (uint64_t r = r0; r < r1; ++r) {
    float l, h;
    rn_enclose(x32[r * d + j], &l, &h);
    lo = fminf(lo, l);
    hi = fmaxf(hi, h);
  }
  box[t * 2 * d + j] = lo;
  box[t * 2 * d + d + j] = hi;
}

// Point tile of each query tile's middle query's landing leaf.
__global__ void k_tile_start(const DNode* nodes, const uint32_t* leaf_of, const uint32_t* order, uint64_t nq,
                             uint32_t n_qt, uint32_t* tile_start) {
  const uint32_t qt = blockIdx.x * blockDim.x + threadIdx.x;
  if (qt >= n_qt) return;
  uint64_t r = static_cast<uint64_t>(qt) * TC_M + TC_M / 2;
  if (r >= nq) r = nq - 1;
  const uint64_t se = static_cast<uint64_t>(__double_as_longlong(nodes[leaf_of[order[r]]].split));
  tile_start[qt] = static_cast<uint32_t>(se) / TC_N;  // the leaf's first row
}

__global__ void k_centre(const double* root_box, uint64_t d, double* centre) {
  const uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (j < d) centre[j] = __dmul_rn(__dadd_rn(root_box[j], root_box[d + j]), 0.5);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return static_cast<EncodeTiledFn>(nullptr);
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// 2-D map over rows x dpad BF16, boxes of 64 elements x box_rows, 128B swizzle.
int make_rows_map(CUtensorMap* m, const void* base, uint64_t rows, uint32_t dpad, uint32_t box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(KD_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint64_t dims[2] = {dpad, rows};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(dpad) * 2};
  const cuuint32_t box[2] = {TC_KC, box_rows};
  const cuuint32_t elem[2] = {1, 1};
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(KD_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return KD_OK;
}

// Tree-side inputs, made once per tree.
// The caller's stream waits (on the device) for the kernels that made them,
// whichever stream those ran on; no host wait.
int ensure_tc_points(kd_tree* t, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(t->tc_mutex);
  if (t->tc_points) {
    KD_TRY_CUDA(cudaStreamWaitEvent(st, t->tc_ready, 0));
    return KD_OK;
  }
  const uint64_t n = t->n_points, d = t->ndim;
  const uint32_t dpad = static_cast<uint32_t>((d + TC_KC - 1) / TC_KC * TC_KC);
  const uint64_t n_pad = (n + TC_N - 1) / TC_N * TC_N;
  const uint64_t n_pt = n_pad / TC_N;
  uint16_t* pts = nullptr;
  float *w = nullptr, *v = nullptr, *tbox = nullptr;
  double* centre = nullptr;
  if (cudaMalloc(&pts, n * dpad * sizeof(uint16_t)) != cudaSuccess ||
      cudaMalloc(&w, n_pad * sizeof(float)) != cudaSuccess || cudaMalloc(&v, n_pad * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&centre, d * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&tbox, n_pt * 2 * d * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(pts);
    cudaFree(w);
    cudaFree(v);
    cudaFree(centre);
    cudaFree(tbox);
    return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
  }
  k_centre<<<static_cast<unsigned>((d + 127) / 128), 128, 0, st>>>(t->boxes, d, centre);
  k_tc_rows<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(t->data, nullptr, n, d, dpad, centre, pts,
                                                                     nullptr, nullptr, w, v);
  if (n_pad > n) k_tc_pad<<<1, 256, 0, st>>>(w, v, n, n_pad);
  k_tile_boxes<<<static_cast<unsigned>(n_pt), 128, 0, st>>>(t->data32, n, d, TC_N, tbox);
  cudaEvent_t ready = nullptr;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(ready, st);
  if (e != cudaSuccess) {
    cudaStreamSynchronize(st);  // nothing may still write them when they are freed
    if (ready) cudaEventDestroy(ready);
    cudaFree(pts);
    cudaFree(w);
    cudaFree(v);
    cudaFree(centre);
    cudaFree(tbox);
    return cuda_fail(e, "tensor-core inputs");
  }
  t->tc_ready = ready;
  t->tc_tbox = tbox;
  t->tc_points = pts;
  t->tc_w = w;
  t->tc_v = v;
  t->tc_centre = centre;
  t->tc_dpad = dpad;
  return KD_OK;
}

}  // namespace

bool tc_applicable(const kd_tree* t, const QueryParams& qp) {
  return qp.metric == M_L2 && qp.eps_factor == 1.0 && t->ndim >= 16 && t->ndim <= 128 && qp.k <= 32 &&
         t->n_points < 0xfffffff0ull;
}

int query_tc_on_device(kd_tree* t, const double* d_queries, uint64_t nq, const QueryParams& qp, double* d_out_d,
                       int64_t* d_out_i, cudaStream_t st, uint32_t* d_status, unsigned long long* d_survivors) {
  if (!tc_applicable(t, qp)) return KD_ERR_INVALID_ARGUMENT;
  int rc;
  if ((rc = ensure_tc_points(t, st))) return rc;
  const uint64_t d = t->ndim;
  const uint32_t dpad = t->tc_dpad;
  // query-side inputs, rows sorted by landing leaf
  const uint32_t n_qt = static_cast<uint32_t>((nq + TC_M - 1) / TC_M);
  void* mem = nullptr;
  const uint64_t qbytes = nq * dpad * sizeof(uint16_t), fbytes = nq * sizeof(float);
  const uint64_t q32_bytes = nq * t->w32 * sizeof(float);
  const uint64_t sort_words = 2 * nq + order_scratch_words(t) + n_qt;
  const uint64_t qbox_bytes = static_cast<uint64_t>(n_qt) * 2 * d * sizeof(float);
  // rounded to 256 bytes: the BF16 query rows after it are a TMA source (16-byte aligned base)
  const uint64_t rerun_bytes = (16 + nq * sizeof(uint64_t) + 255) / 256 * 256;
  const uint64_t total = rerun_bytes + qbytes + 2 * fbytes + q32_bytes + qbox_bytes + sort_words * sizeof(uint32_t) +
                         256;
  if (dev_alloc(&mem, total, st) != cudaSuccess) {
    cudaGetLastError();
    return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
  }
  uint32_t* rerun_count = static_cast<uint32_t*>(mem);
  uint64_t* rerun_list = reinterpret_cast<uint64_t*>(static_cast<unsigned char*>(mem) + 16);
  uint16_t* qb = reinterpret_cast<uint16_t*>(static_cast<unsigned char*>(mem) + rerun_bytes);
  // the FP32 rows follow the BF16 ones (a whole number of 128-byte rows), so
  // they start on a 16-byte boundary for their float4 reads
  float* q32 = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(qb) + qbytes);
  float* qn2 = q32 + nq * t->w32;
  float* qnorm = qn2 + nq;
  float* qbox = qnorm + nq;
  uint32_t* leaf_of = reinterpret_cast<uint32_t*>(qbox + static_cast<uint64_t>(n_qt) * 2 * d);
  uint32_t* order = leaf_of + nq;
  uint32_t* tile_start = order + nq;
  uint32_t* scratch = tile_start + n_qt;
  order_by_landing_leaf(t, d_queries, nq, leaf_of, order, scratch, st);
  k_tile_start<<<(n_qt + 127) / 128, 128, 0, st>>>(t->nodes, leaf_of, order, nq, n_qt, tile_start);
  k_tc_rows<<<static_cast<unsigned>((nq + 255) / 256), 256, 0, st>>>(d_queries, order, nq, d, dpad, t->tc_centre, qb,
                                                                      qn2, qnorm, nullptr, nullptr);
  k_f32_gather<<<static_cast<unsigned>((nq * t->w32 + 255) / 256), 256, 0, st>>>(d_queries, order, nq, d, t->w32,
                                                                                q32);
  k_tile_boxes<<<n_qt, 128, 0, st>>>(q32, nq, d, TC_M, qbox);
  CUtensorMap mq, mp;
  if ((rc = make_rows_map(&mq, qb, nq, dpad, TC_M)) || (rc = make_rows_map(&mp, t->tc_points, t->n_points, dpad, TC_N))) {
    cudaFreeAsync(mem, st);
    return rc;
  }
  TcArgs a{};
  a.queries = d_queries;
  a.data = t->data;
  a.data32 = t->data32;
  a.indices = t->indices;
  a.order = order;
  a.tile_start = tile_start;
  a.q32 = q32;
  a.data32w = t->data32w;
  a.w32 = t->w32;
  a.qn2 = qn2;
  a.qnorm = qnorm;
  a.pw = t->tc_w;
  a.pv = t->tc_v;
  a.qbox = qbox;
  a.tbox = t->tc_tbox;
  a.out_d = d_out_d;
  a.out_i = d_out_i;
  a.status = d_status;
  a.survivors = d_survivors;
  a.rerun_count = rerun_count;
  a.rerun_list = rerun_list;
  a.nq = nq;
  a.n_points = t->n_points;
  a.d = d;
  a.k = qp.k;
  a.cutoff = qp.cutoff;
  a.coord_max = t->coord_max32;
  a.strat = d <= 16 ? S_FOLDED : S_STREAMED;
  a.n_qt = n_qt;
  a.n_pt = static_cast<uint32_t>((t->n_points + TC_N - 1) / TC_N);
  a.kch = dpad / TC_KC;
  a.nst = a.kch == 1 ? 4 : 2;
  const size_t smem = 1024 + static_cast<size_t>(a.kch) * TC_M * 128 + static_cast<size_t>(a.nst) * a.kch * TC_N * 128 +
                      (2 * a.nst + 6) * sizeof(uint64_t);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(a.n_qt, static_cast<uint64_t>(sms)));
  cudaError_t e = cudaMemsetAsync(rerun_count, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_query_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e == cudaSuccess) {
    k_query_tc<32><<<grid, TC_THREADS, smem, st>>>(mq, mp, a);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    cudaFreeAsync(mem, st);
    return cuda_fail(e, "k_query_tc launch");
  }
  // the near ties, again in the reference's order
  QArgs ra = query_args(t, d_queries, nq, qp, d_out_d, d_out_i, d_status);
  ra.rerun_total = d_survivors ? d_survivors + 1 : nullptr;
  rc = launch_rerun(ra, M_L2, st, rerun_count, rerun_list);
  cudaFreeAsync(mem, st);
  return rc;
}

}  // namespace kd
