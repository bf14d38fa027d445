// kd_build.cu -- GPU median-split kd-tree build, level by level.
//
// Restates src/build.rs:19-314 of FujishigeTemma/kdtree-rs as per-level
// segmented kernels.  The reference recurses depth-first; because the split is
// always at len / 2 (build.rs:162-164) the tree's shape is a pure function of
// (n_points, leafsize), so every node of one depth can be processed at once:
//
//   level L segments = the nodes at depth L, each a contiguous row range.
//   per level:  bbox (min / max per dim, build.rs:175-181, kernel.rs:93-151)
//            -> split_dim = widest axis (layout.rs:168-179)
//            -> pivot = mid-th key under f64::total_cmp (build.rs:199-205),
//               by a segmented 8-bit radix select over total-order keys
//            -> lt = #{key < pivot} (build.rs:209)
//            -> the exact row permutation of partition_rows (build.rs:266-314)
//            -> node records and the next level's segments.
//
// The permutation: with R = ascending positions in [0, lt) holding key >= pivot
// and L = ascending positions in [lt, len) holding key < pivot (|R| = |L| = n),
// the reference swaps R[i] <-> L[n-1-i].  Listing the 2n misplaced positions in
// ascending order as P[0..2n) (R then L), that swap sends P[r] to P[2n-1-r]: a
// reversal of the misplaced list, computed from one segmented prefix sum.  The
// pivot-equal fix-up (build.rs:303-313) is a Lomuto compaction of the first
// m = mid - lt pivot-equal rows of [lt, len) into [lt, mid); with E[t] the t-th
// such row, the row at place lt+t moves to E[t], so a displaced row's final
// position is the end of the chain pos -> E[pos - lt] while pos - lt < m --
// evaluated sequentially in shared memory for small segments and by pointer
// jumping for large ones.  Only data with duplicated split coordinates takes it.
//
// Segments above SMALL_MAX rows (the top levels) are processed level by level
// by grids of CTAs over row chunks with global histograms, counts and scans;
// from the first level at or below it, one CTA builds each segment's whole
// subtree in shared memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "kd_internal.hpp"

namespace kd {

namespace {

// The build is a chain of dependent launches on one stream.  Each is launched
// with programmatic stream serialisation, so the next kernel's launch is
// processed while its predecessor runs; every kernel first waits for the
// grids it depends on (griddepcontrol.wait: all of their memory operations
// are then visible), so the ordering is that of plain stream launches.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... P, typename... A>
cudaError_t chain(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

constexpr uint32_t HOLE = 0xffffffffu;
constexpr uint32_t NONE = 0xffffffffu;
constexpr int SMALL_MAX = 8192;  // rows a single CTA partitions in shared memory
constexpr int LG_THREADS = 256;
constexpr int LG_ITEMS = 8;
constexpr int LG_CHUNK = LG_THREADS * LG_ITEMS;  // rows per CTA in the large path
constexpr int RADIX_PASSES = 8;
constexpr uint64_t KEY_MAX = ~0ull;

// IEEE comparison key: total order with -0 folded onto +0, so that integer
// '<' and '==' on it are f64 '<' and '==' for finite values
// (partition_rows compares with '<', '>=', '==', not total_cmp).
__device__ __forceinline__ uint64_t canon(uint64_t k) {
  return k == 0x7fffffffffffffffull ? 0x8000000000000000ull : k;
}

// count_nodes (src/build.rs:166-173), level by level over the at most two
// distinct sizes of one depth (same result as the reference's recursion).
__host__ __device__ uint64_t count_nodes_impl(uint64_t len, uint64_t leafsize) {
  uint64_t sz[4] = {len, 0, 0, 0}, cnt[4] = {1, 0, 0, 0};
  int n = 1;
  uint64_t total = 0;
  while (n > 0) {
    uint64_t nsz[8], ncnt[8];
    int nn = 0;
    for (int i = 0; i < n; ++i) {
      total += cnt[i];
      if (sz[i] <= leafsize) continue;
      uint64_t halves[2] = {sz[i] / 2, sz[i] - sz[i] / 2};
      for (int h = 0; h < 2; ++h) {
        int j = 0;
        while (j < nn && nsz[j] != halves[h]) ++j;
        if (j == nn) {
          nsz[nn] = halves[h];
          ncnt[nn] = 0;
          ++nn;
        }
        ncnt[j] += cnt[i];
      }
    }
    for (int i = 0; i < nn; ++i) {
      sz[i] = nsz[i];
      cnt[i] = ncnt[i];
    }
    n = nn;
  }
  return total;
}

// widest_axis (src/layout.rs:168-179) on a box held as total-order keys.
__device__ uint32_t widest_axis_keys(const uint64_t* box, uint64_t d) {
  uint32_t best = 0;
  double span = dsub(from_total_key(box[d]), from_total_key(box[0]));
  for (uint64_t j = 1; j < d; ++j) {
    double s = dsub(from_total_key(box[d + j]), from_total_key(box[j]));
    if (s > span) {
      span = s;
      best = static_cast<uint32_t>(j);
    }
  }
  return best;
}

struct Level {
  const double* din;
  double* dout;
  const uint32_t* iin;
  uint32_t* iout;
  uint64_t d;
  uint64_t leafsize;
  // current level's segments (slot-indexed; HOLE marks an absent node)
  const uint32_t* seg_node;
  const uint32_t* seg_start;
  const uint32_t* seg_len;
  // next level's segments: children of slot s go to slots 2s and 2s+1
  uint32_t* nseg_node;
  uint32_t* nseg_start;
  uint32_t* nseg_len;
  DNode* nodes;
  uint64_t* boxkeys;  // n_nodes * 2d total-order keys during the build
  uint32_t* node_len;
  uint64_t n_slots;
};

__device__ __forceinline__ void write_leaf(DNode* nodes, uint32_t node, uint32_t start, uint32_t len) {
  DNode nd;
  nd.split = bitsd(static_cast<uint64_t>(start) | (static_cast<uint64_t>(start + len) << 32));
  nd.right = 0;
  nd.meta = KD_NODE_LEAF;
  nodes[node] = nd;
}

// Record an inner node and open its two children in the next level (their box
// keys start at the identities of min / max for the bbox atomics).
__device__ void expand_inner(const Level& L, uint64_t slot, uint32_t node, uint32_t start, uint32_t len,
                             uint32_t dim, uint64_t pivot_key) {
  uint32_t mid = len / 2;
  uint32_t right = node + 1 + static_cast<uint32_t>(count_nodes_impl(mid, L.leafsize));
  DNode nd;
  nd.split = from_total_key(pivot_key);
  nd.right = right;
  nd.meta = dim;
  L.nodes[node] = nd;
  L.node_len[node] = len;
  L.nseg_node[2 * slot] = node + 1;
  L.nseg_start[2 * slot] = start;
  L.nseg_len[2 * slot] = mid;
  L.nseg_node[2 * slot + 1] = right;
  L.nseg_start[2 * slot + 1] = start + mid;
  L.nseg_len[2 * slot + 1] = len - mid;
}

__device__ void close_leaf(const Level& L, uint64_t slot, uint32_t node, uint32_t start, uint32_t len) {
  write_leaf(L.nodes, node, start, len);
  L.node_len[node] = len;
  L.nseg_node[2 * slot] = HOLE;
  L.nseg_node[2 * slot + 1] = HOLE;
  L.nseg_len[2 * slot] = 0;
  L.nseg_len[2 * slot + 1] = 0;
}

// ---------------------------------------------------------------------------
// Bounding boxes: per (segment, chunk) CTA, min / max per dim as total-order
// keys, merged into the node's box with 64-bit atomics.  The block size is a
// multiple of d (d <= 256) so each thread's dimension is fixed and it reduces in
// registers.  Level 0 also checks finiteness (all_finite, kernel.rs:67-74).
// ---------------------------------------------------------------------------
__global__ void k_init_boxkeys(uint64_t* boxkeys, uint64_t n_nodes, uint64_t d) {
  wait_prior_grid();
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  uint64_t total = n_nodes * 2 * d;
  if (i < total) boxkeys[i] = ((i / d) & 1) ? 0ull : KEY_MAX;
}

__global__ void k_bbox(Level L, uint32_t chunk_rows, uint32_t n_chunks, int check_finite, uint32_t* status) {
  wait_prior_grid();
  extern __shared__ uint64_t sbox[];  // [lo d | hi d]
  const uint64_t slot = blockIdx.x;
  const uint32_t node = L.seg_node[slot];
  if (node == HOLE) return;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  if (static_cast<uint64_t>(blockIdx.y) * chunk_rows >= len) return;
  const uint64_t d = L.d;
  for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) {
    sbox[j] = KEY_MAX;
    sbox[d + j] = 0;
  }
  __syncthreads();
  bool bad = false;
  uint64_t lo = KEY_MAX, hi = 0;
  for (uint32_t c = blockIdx.y; c < n_chunks; c += gridDim.y) {
    const uint64_t r0 = static_cast<uint64_t>(c) * chunk_rows;
    if (r0 >= len) break;
    const uint64_t r1 = min(static_cast<uint64_t>(len), r0 + chunk_rows);
    const double* base = L.din + (static_cast<uint64_t>(start) + r0) * d;
    const uint64_t n_el = (r1 - r0) * d;
    if (d <= 256) {
      // blockDim.x is a multiple of d: the thread's dimension is fixed.
      for (uint64_t f = threadIdx.x; f < n_el; f += blockDim.x) {
        double v = base[f];
        bad |= !isfinite(v);
        uint64_t k = total_key(v);
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
      }
    } else {
      for (uint64_t f = threadIdx.x; f < n_el; f += blockDim.x) {
        double v = base[f];
        bad |= !isfinite(v);
        uint64_t k = total_key(v);
        uint64_t j = f % d;
        atomicMin(reinterpret_cast<unsigned long long*>(&sbox[j]), k);
        atomicMax(reinterpret_cast<unsigned long long*>(&sbox[d + j]), k);
      }
    }
  }
  if (d <= 256) {
    const uint32_t j = threadIdx.x % d;
    atomicMin(reinterpret_cast<unsigned long long*>(&sbox[j]), lo);
    atomicMax(reinterpret_cast<unsigned long long*>(&sbox[d + j]), hi);
  }
  if (check_finite && bad) atomicOr(status, 1u);
  __syncthreads();
  uint64_t* gbox = L.boxkeys + static_cast<uint64_t>(node) * 2 * d;
  for (uint64_t j = threadIdx.x; j < d; j += blockDim.x) {
    atomicMin(reinterpret_cast<unsigned long long*>(&gbox[j]), sbox[j]);
    atomicMax(reinterpret_cast<unsigned long long*>(&gbox[d + j]), sbox[d + j]);
  }
}

// ---------------------------------------------------------------------------
// Block-wide helpers.
// ---------------------------------------------------------------------------
template <int THREADS>
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* total, uint32_t* sh_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < THREADS / 32 ? sh_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < THREADS / 32) sh_warp[lane] = w;
  }
  __syncthreads();
  uint32_t warp_off = warp ? sh_warp[warp - 1] : 0;
  *total = sh_warp[THREADS / 32 - 1];
  __syncthreads();
  return warp_off + x - v;
}

template <int THREADS>
__device__ uint32_t block_sum(uint32_t v, uint32_t* sh_warp) {
  uint32_t total;
  block_excl_scan<THREADS>(v, &total, sh_warp);
  return total;
}

// ---------------------------------------------------------------------------
// Small subtrees.  From the first depth whose segments have at most SMALL_MAX
// rows, one CTA builds the whole subtree below each segment -- every node's box
// (build.rs:175-181), split dimension, pivot, exact partition permutation and
// record, down to the leaves -- and then writes the subtree's rows once, in
// their final order.  The rows stay where the level above left them: the CTA
// permutes 16-bit local row numbers (perm: position -> local row) and keeps each
// local row's key on its segment's current split dimension (krow).  All the
// segments of a depth are split at once, each by a group of warps (the whole
// CTA for the subtree root, one warp each for segments of at most WARP_SEG
// rows) synchronised on its own named barrier.  Segment (depth j, index s) is
// reached from the subtree root by the bits of s, with the node counts of the
// at most two segment lengths of each depth.
// ---------------------------------------------------------------------------
constexpr int SUB_THREADS = 512;
constexpr int SUB_WARPS = SUB_THREADS / 32;
constexpr int WARP_SEG = 512;  // rows a warp of a group takes (16 keys a lane)
constexpr uint32_t FULL = 0xffffffffu;

struct SubArgs {
  const double* din;
  const uint32_t* iin;
  double* dout;
  uint32_t* iout;
  uint64_t d;
  uint32_t leafsize;
  const uint32_t* seg_node;
  const uint32_t* seg_start;
  const uint32_t* seg_len;
  DNode* nodes;
  uint64_t* boxkeys;
  uint32_t* node_len;
  int check_finite;
  uint32_t* status;
};

struct SubShared {
  uint64_t krow[SMALL_MAX];   // key of each local row on its segment's split dimension
  uint16_t perm[SMALL_MAX];   // position -> local row
  uint16_t plist[SMALL_MAX];  // misplaced positions (relative to their segment), by rank
  uint16_t moved[SMALL_MAX];  // the partition's moves, staged
};

struct SubSeg {
  uint32_t node, pos, len;  // pos: first position within the subtree
  bool ok;                  // false: an ancestor is a leaf (no such segment)
};

__device__ __forceinline__ uint64_t warp_min64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(FULL, v, o);
    v = w < v ? w : v;
  }
  return v;
}
__device__ __forceinline__ uint64_t warp_max64(uint64_t v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(FULL, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// Segment (depth j, index s) of the subtree rooted at (node0, length l0);
// ok = false when an ancestor of it is a leaf.
__device__ __forceinline__ SubSeg sub_segment(const uint32_t* lo_len, const uint32_t (*cn)[2], uint32_t node0,
                                              uint32_t l0, uint32_t leafsize, int j, uint32_t s) {
  uint32_t node = node0, pos = 0, len = l0;
  for (int i = 0; i < j; ++i) {
    if (len <= leafsize) return SubSeg{0, 0, 0, false};
    const uint32_t mid = len / 2;
    if (!((s >> (j - 1 - i)) & 1u)) {
      node += 1;
      len = mid;
    } else {
      node += 1 + cn[i + 1][mid - lo_len[i + 1]];
      pos += mid;
      len -= mid;
    }
  }
  return SubSeg{node, pos, len, true};
}

// The inner node's record (expand_inner without the next level's segments).
__device__ __forceinline__ void sub_record(const SubArgs& A, const uint32_t (*cn)[2], const uint32_t* lo_len,
                                           int j, const SubSeg& g, uint32_t dim, uint64_t pivot_key) {
  const uint32_t mid = g.len / 2;
  DNode nd;
  nd.split = from_total_key(pivot_key);
  nd.right = g.node + 1 + cn[j + 1][mid - lo_len[j + 1]];
  nd.meta = dim;
  A.nodes[g.node] = nd;
  A.node_len[g.node] = g.len;
}

// Group-wide collectives for G warps (G = 1, 2, 4, 8, 16) of group `gid`:
// every thread of the group gets the result.  `red` holds one word per warp.
struct SubReduce {
  uint64_t lo[SUB_WARPS], hi[SUB_WARPS];
  uint32_t sum[SUB_WARPS];
};
template <int G>
__device__ __forceinline__ void group_sync(uint32_t gid) {
  if constexpr (G == 1) {
    __syncwarp();
  } else if constexpr (G == SUB_WARPS) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(G * 32) : "memory");
  }
}
template <int G>
__device__ __forceinline__ uint32_t group_add(uint32_t v, SubReduce* red, uint32_t gid) {
  v = __reduce_add_sync(FULL, v);
  if constexpr (G == 1) {
    return v;
  } else {
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red->sum[w] = v;
    group_sync<G>(gid);
    uint32_t t = 0;
#pragma unroll
    for (int i = 0; i < G; ++i) t += red->sum[gid * G + i];
    group_sync<G>(gid);
    return t;
  }
}
template <int G>
__device__ __forceinline__ void group_minmax(uint64_t* lo, uint64_t* hi, SubReduce* red, uint32_t gid) {
  uint64_t a = warp_min64(*lo), b = warp_max64(*hi);
  if constexpr (G > 1) {
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      red->lo[w] = a;
      red->hi[w] = b;
    }
    group_sync<G>(gid);
    a = red->lo[gid * G];
    b = red->hi[gid * G];
#pragma unroll
    for (int i = 1; i < G; ++i) {
      a = red->lo[gid * G + i] < a ? red->lo[gid * G + i] : a;
      b = red->hi[gid * G + i] > b ? red->hi[gid * G + i] : b;
    }
    group_sync<G>(gid);
  }
  *lo = a;
  *hi = b;
}
template <int G>
__device__ __forceinline__ uint64_t group_max64(uint64_t v, SubReduce* red, uint32_t gid) {
  v = warp_max64(v);
  if constexpr (G > 1) {
    const uint32_t w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red->hi[w] = v;
    group_sync<G>(gid);
    v = red->hi[gid * G];
#pragma unroll
    for (int i = 1; i < G; ++i) v = red->hi[gid * G + i] > v ? red->hi[gid * G + i] : v;
    group_sync<G>(gid);
  }
  return v;
}
// Exclusive prefix of v over the group's threads in order; *total: the sum.
template <int G>
__device__ __forceinline__ uint32_t group_excl_scan(uint32_t v, uint32_t* total, SubReduce* red, uint32_t gid) {
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, x, o);
    if (lane >= static_cast<uint32_t>(o)) x += y;
  }
  const uint32_t wtot = __shfl_sync(FULL, x, 31);
  if constexpr (G == 1) {
    *total = wtot;
    return x - v;
  } else {
    if (lane == 0) red->sum[w] = wtot;
    group_sync<G>(gid);
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int i = 0; i < G; ++i) {
      const uint32_t c = red->sum[gid * G + i];
      before += (gid * G + i < w) ? c : 0;
      all += c;
    }
    group_sync<G>(gid);
    *total = all;
    return before + x - v;
  }
}

// One segment split by a group of G warps (g.len <= 512 G): each thread owns
// a contiguous run of at most 16 positions, so misplaced ranks ascend in thread
// order.  The pivot is found bit by bit (a group sum per bit) from the first
// bit where the segment's smallest and largest keys differ, until one
// candidate key is left (distinct keys: about log2(len) bits).
template <int G>
__device__ __forceinline__ void sub_split(const SubArgs& A, SubShared& S, const uint32_t (*cn)[2],
                                          const uint32_t* lo_len, int j, const SubSeg g, uint64_t row0,
                                          SubReduce* red, uint32_t gid) {
  constexpr int T = WARP_SEG / 32;  // positions a thread owns, at most
  const uint32_t tg = (threadIdx.x & 31) + 32u * ((threadIdx.x >> 5) % G);  // thread within the group
  const uint64_t d = A.d;
  const uint32_t per = (g.len + 32u * G - 1) / (32u * G);
  const uint32_t b0 = min(g.len, tg * per), nown = min(g.len, b0 + per) - b0;
  uint32_t best_dim = 0;
  double best_span = 0.0;
  uint64_t blo = 0, bhi = 0;
  for (uint64_t dj = 0; dj < d; ++dj) {
    uint64_t lo = KEY_MAX, hi = 0;
#pragma unroll
    for (int t = 0; t < T; ++t) {
      if (t >= static_cast<int>(per)) break;  // group-uniform
      if (t < static_cast<int>(nown)) {
        const uint64_t k = total_key(A.din[(row0 + S.perm[g.pos + b0 + t]) * d + dj]);
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
      }
    }
    group_minmax<G>(&lo, &hi, red, gid);
    if (tg == 0) {
      A.boxkeys[static_cast<uint64_t>(g.node) * 2 * d + dj] = lo;
      A.boxkeys[static_cast<uint64_t>(g.node) * 2 * d + d + dj] = hi;
    }
    const double span = dsub(from_total_key(hi), from_total_key(lo));  // widest_axis (layout.rs:168-179)
    if (dj == 0 || span > best_span) {
      best_span = span;
      best_dim = static_cast<uint32_t>(dj);
      blo = lo;
      bhi = hi;
    }
  }
  if (g.len <= A.leafsize) {
    if (tg == 0) {
      write_leaf(A.nodes, g.node, static_cast<uint32_t>(row0) + g.pos, g.len);
      A.node_len[g.node] = g.len;
    }
    return;
  }
  const uint32_t dim = best_dim, mid = g.len / 2;
  uint64_t key[T];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    key[t] = 0;
    if (t >= static_cast<int>(per)) continue;
    if (t < static_cast<int>(nown)) {
      const uint32_t lr = S.perm[g.pos + b0 + t];
      key[t] = total_key(A.din[(row0 + lr) * d + dim]);
      S.krow[lr] = key[t];
    }
  }
  // pivot = the mid-th smallest key under total order (select_nth_unstable_by)
  uint64_t pivot = blo;
  if (blo != bhi && G == 1 && g.len <= 32) {
    // one key a lane: its rank among the segment's keys, by shuffles
    const uint32_t lane = threadIdx.x & 31;
    const bool mine = lane < g.len;
    uint32_t cl = 0, ce = 0;
    for (uint32_t q = 0; q < g.len; ++q) {
      const uint64_t kq = __shfl_sync(FULL, key[0], static_cast<int>(q));
      cl += kq < key[0];
      ce += kq == key[0];
    }
    const uint32_t at = __ballot_sync(FULL, mine && cl <= mid && mid < cl + ce);  // those lanes agree
    pivot = __shfl_sync(FULL, key[0], __ffs(at) - 1);
  } else if (blo != bhi) {
    const int hb = 63 - __clzll(static_cast<long long>(blo ^ bhi));
    uint64_t prefix = hb == 63 ? 0 : (blo >> (hb + 1)) << (hb + 1);
    uint32_t rank = mid, n_cand = g.len;  // keys matching prefix on the bits above b
    int b = hb;
    for (; b >= 0; --b) {
      uint32_t c0 = 0;
#pragma unroll
      for (int t = 0; t < T; ++t) {
        if (t >= static_cast<int>(per)) break;
        c0 += t < static_cast<int>(nown) && ((key[t] ^ prefix) >> b) == 0;
      }
      c0 = group_add<G>(c0, red, gid);
      if (rank >= c0) {  // every thread of the group decides alike
        rank -= c0;
        prefix |= 1ull << b;
        n_cand -= c0;
      } else {
        n_cand = c0;
      }
      if (n_cand == 1) break;  // that key is the pivot
    }
    if (b > 0 && n_cand == 1) {  // the one key matching prefix on bits b and above
      uint64_t found = 0;
#pragma unroll
      for (int t = 0; t < T; ++t) {
        if (t >= static_cast<int>(per)) break;
        if (t < static_cast<int>(nown) && ((key[t] ^ prefix) >> b) == 0) found = key[t];
      }
      pivot = group_max64<G>(found, red, gid);
    } else {
      pivot = prefix;  // every bit decided
    }
  }
  const uint64_t pc = canon(pivot);
  // lt = #{key < pivot} under f64 '<' (build.rs:209)
  uint32_t my_lt = 0;
#pragma unroll
  for (int t = 0; t < T; ++t) {
    if (t >= static_cast<int>(per)) break;
    my_lt += t < static_cast<int>(nown) && canon(key[t]) < pc;
  }
  const uint32_t lt = group_add<G>(my_lt, red, gid);
  // misplaced positions: key >= pivot in [0, lt), key < pivot in [lt, len)
  uint32_t cnt = 0;
#pragma unroll
  for (int t = 0; t < T; ++t) {
    if (t >= static_cast<int>(per)) break;
    const bool below = canon(key[t]) < pc;
    cnt += t < static_cast<int>(nown) && ((b0 + t < lt) ? !below : below);
  }
  uint32_t n2;
  uint32_t r = group_excl_scan<G>(cnt, &n2, red, gid);
#pragma unroll
  for (int t = 0; t < T; ++t) {
    if (t >= static_cast<int>(per)) break;
    const bool below = canon(key[t]) < pc;
    if (t < static_cast<int>(nown) && ((b0 + t < lt) ? !below : below))
      S.plist[g.pos + r++] = static_cast<uint16_t>(b0 + t);
  }
  group_sync<G>(gid);
  // swap R[i] <-> L[n-1-i]: the row at plist[n2-1-j] lands on plist[j]
  // (through `moved`, so that no read sees a written place)
  for (uint32_t jj = tg; jj < n2; jj += 32u * G)
    S.moved[g.pos + S.plist[g.pos + jj]] = S.perm[g.pos + S.plist[g.pos + n2 - 1 - jj]];
  group_sync<G>(gid);
  for (uint32_t jj = tg; jj < n2; jj += 32u * G) {
    const uint32_t at = g.pos + S.plist[g.pos + jj];
    S.perm[at] = S.moved[at];
  }
  group_sync<G>(gid);
  if (mid > lt && tg == 0) {
    // pivot-equal fix-up (build.rs:303-313), sequentially
    uint32_t place = lt, scan = lt;
    while (place < mid && scan < g.len) {
      if (canon(S.krow[S.perm[g.pos + scan]]) == pc) {
        const uint16_t x = S.perm[g.pos + scan];
        S.perm[g.pos + scan] = S.perm[g.pos + place];
        S.perm[g.pos + place] = x;
        ++place;
      }
      ++scan;
    }
  }
  if (tg == 0) sub_record(A, cn, lo_len, j, g, dim, pivot);
  group_sync<G>(gid);
}

// Every segment of depth j, split by groups of G warps.
template <int G>
__device__ __forceinline__ void sub_depth(const SubArgs& A, SubShared& S, const uint32_t (*cn)[2],
                                          const uint32_t* lo_len, int j, uint32_t node0, uint32_t l0, uint64_t row0,
                                          SubReduce* red) {
  const uint32_t gid = (threadIdx.x >> 5) / G;
  for (uint32_t sidx = gid; sidx < (1u << j); sidx += SUB_WARPS / G) {
    const SubSeg g = sub_segment(lo_len, cn, node0, l0, A.leafsize, j, sidx);
    if (!g.ok) continue;  // uniform per group
    sub_split<G>(A, S, cn, lo_len, j, g, row0, red, gid);
  }
}

__global__ void __launch_bounds__(SUB_THREADS) k_small_subtree(SubArgs A) {
  wait_prior_grid();
  extern __shared__ __align__(16) unsigned char sub_smem[];
  SubShared& S = *reinterpret_cast<SubShared*>(sub_smem);
  __shared__ uint32_t lo_len[KD_MAX_DEPTH + 1];
  __shared__ uint32_t cn[KD_MAX_DEPTH + 1][2];
  __shared__ SubReduce red;
  __shared__ int s_depths;

  const uint32_t node0 = A.seg_node[blockIdx.x];
  if (node0 == HOLE) return;
  const uint32_t row0 = A.seg_start[blockIdx.x], l0 = A.seg_len[blockIdx.x];
  const uint64_t d = A.d;
  if (threadIdx.x == 0) {
    // segment lengths at depth i are floor / ceil of l0 / 2^i
    int i = 0;
    for (;; ++i) {
      const uint32_t lo = l0 >> i, hi = (l0 + (1u << i) - 1) >> i;
      lo_len[i] = lo;
      cn[i][0] = static_cast<uint32_t>(count_nodes_impl(lo, A.leafsize));
      cn[i][1] = static_cast<uint32_t>(count_nodes_impl(lo + 1, A.leafsize));
      if (hi <= A.leafsize || i == KD_MAX_DEPTH) break;
    }
    s_depths = i + 1;  // depths 0 .. i hold segments
  }
  for (uint32_t p = threadIdx.x; p < l0; p += SUB_THREADS) S.perm[p] = static_cast<uint16_t>(p);
  __syncthreads();
  bool bad = false;
  for (int j = 0; j < s_depths; ++j) {
    // warps a segment of this depth gets: the longest is split by groups of
    // at least ceil(len / 512) warps, so a thread owns at most 16 positions
    const uint32_t hi_len = (l0 + (1u << j) - 1) >> j;
    const uint32_t need = (hi_len + WARP_SEG - 1) / WARP_SEG;
    if (need > 8) sub_depth<16>(A, S, cn, lo_len, j, node0, l0, row0, &red);
    else if (need > 4) sub_depth<8>(A, S, cn, lo_len, j, node0, l0, row0, &red);
    else if (need > 2) sub_depth<4>(A, S, cn, lo_len, j, node0, l0, row0, &red);
    else if (need > 1) sub_depth<2>(A, S, cn, lo_len, j, node0, l0, row0, &red);
    else sub_depth<1>(A, S, cn, lo_len, j, node0, l0, row0, &red);
    __syncthreads();
  }
  // the subtree's rows, once, in their final order (and, at level 0, the
  // finiteness check: an exponent field of all ones is inf or NaN)
  const double* din = A.din;
  auto move = [&](uint64_t to, uint64_t from) {
    const double v = din[from];
    bad |= (static_cast<uint64_t>(__double_as_longlong(v)) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
    A.dout[to] = v;
  };
  if (static_cast<uint64_t>(l0) * d < (1ull << 32)) {
    const uint32_t dd = static_cast<uint32_t>(d);
    for (uint32_t f = threadIdx.x; f < l0 * dd; f += SUB_THREADS) {
      const uint32_t p = f / dd, jd = f - p * dd;
      move(static_cast<uint64_t>(row0) * d + f, (static_cast<uint64_t>(row0) + S.perm[p]) * d + jd);
    }
  } else {  // very wide rows: a warp a row
    for (uint32_t p = threadIdx.x >> 5; p < l0; p += SUB_WARPS)
      for (uint64_t jd = threadIdx.x & 31; jd < d; jd += 32)
        move((static_cast<uint64_t>(row0) + p) * d + jd, (static_cast<uint64_t>(row0) + S.perm[p]) * d + jd);
  }
  if (A.check_finite && bad) atomicOr(A.status, 1u);
  for (uint32_t p = threadIdx.x; p < l0; p += SUB_THREADS) A.iout[row0 + p] = A.iin[row0 + S.perm[p]];
}

// ---------------------------------------------------------------------------
// Large path: grids of (segment slot, row chunk) CTAs.
// ---------------------------------------------------------------------------
struct LargeScratch {
  uint64_t* keys;       // N: split-coordinate keys of the current level
  uint64_t* keys_out;   // N: keys moved with their rows (for the fix-up)
  uint32_t* rankbuf;    // N: rank among the misplaced rows, or NONE
  uint32_t* plist;      // N: misplaced positions by rank
  uint32_t* hist;       // slots * RADIX_PASSES * 256
  uint64_t* sel_prefix; // slots * (RADIX_PASSES + 1)
  uint32_t* sel_rank;   // slots * (RADIX_PASSES + 1)
  uint32_t* seg_dim;    // slots
  uint64_t* seg_pivot;  // slots
  uint32_t* seg_lt;     // slots
  uint32_t* chunk_cnt;  // slots * n_chunks
  uint32_t* seg_mis;    // slots
  uint32_t* seg_first;  // slots: first radix pass whose byte the segment's keys do not share (8: all equal)
};

__global__ void k_lg_prepare(Level L, LargeScratch S) {
  wait_prior_grid();
  uint64_t slot = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (slot >= L.n_slots) return;
  uint32_t node = L.seg_node[slot];
  if (node == HOLE || L.seg_len[slot] <= L.leafsize) {
    S.seg_dim[slot] = NONE;
    return;
  }
  const uint64_t* box = L.boxkeys + static_cast<uint64_t>(node) * 2 * L.d;
  const uint32_t dim = widest_axis_keys(box, L.d);
  S.seg_dim[slot] = dim;
  // every key lies between the box's smallest and largest on dim: the bytes
  // those share need no histogram pass
  const uint64_t blo = box[dim], bhi = box[L.d + dim];
  const int first = blo == bhi ? RADIX_PASSES : __clzll(static_cast<long long>(blo ^ bhi)) / 8;
  const uint64_t prefix = first == 0 ? 0 : (first == RADIX_PASSES ? blo : (blo >> (64 - 8 * first)) << (64 - 8 * first));
  S.seg_first[slot] = static_cast<uint32_t>(first);
  S.sel_prefix[slot * (RADIX_PASSES + 1) + first] = prefix;
  S.sel_rank[slot * (RADIX_PASSES + 1) + first] = L.seg_len[slot] / 2;
  S.seg_lt[slot] = 0;
}

// Pick the digit bucket of pass `pass` holding the wanted rank; returns (to
// every thread of the block) the state after that pass.  Every CTA of the
// segment computes the same answer.  The block's LG_THREADS = 256 threads load
// one bin each and scan them; `scratch` holds LG_THREADS / 32 + 3 words.
static_assert(LG_THREADS == 256, "one bin per thread");
__device__ void pick_digit_block(const uint32_t* hist, int pass, uint64_t prefix_in, uint32_t rank_in,
                                 uint64_t* prefix_out, uint32_t* rank_out, uint32_t* scratch) {
  const uint32_t b = threadIdx.x;
  const uint32_t c = hist[b];
  uint32_t total;
  const uint32_t excl = block_excl_scan<LG_THREADS>(c, &total, scratch);
  uint32_t* found = scratch + LG_THREADS / 32;  // [bin, rank in it, flag]
  if (b == 0) found[2] = 0;
  __syncthreads();
  if (excl <= rank_in && rank_in < excl + c) {  // exactly one bin
    found[0] = b;
    found[1] = rank_in - excl;
    found[2] = 1;
  }
  __syncthreads();
  const int shift = 56 - 8 * pass;
  if (found[2]) {
    *prefix_out = prefix_in | (static_cast<uint64_t>(found[0]) << shift);
    *rank_out = found[1];
  } else {
    *prefix_out = prefix_in;
    *rank_out = rank_in;
  }
  __syncthreads();
}

// Chunks of one segment: CTA (slot, y) handles chunks y, y + gridDim.y, ...
#define KD_FOR_CHUNKS(len)                                                        \
  for (uint32_t chunk = blockIdx.y, r0 = blockIdx.y * LG_CHUNK; r0 < (len);      \
       chunk += gridDim.y, r0 = chunk * LG_CHUNK)

__global__ void k_lg_keys(Level L, LargeScratch S) {
  wait_prior_grid();
  const uint64_t slot = blockIdx.x;
  const uint32_t dim = S.seg_dim[slot];
  if (dim == NONE) return;
  if (blockIdx.y == 0)  // the segment's histograms for this level's passes start empty
    for (uint32_t b = threadIdx.x; b < RADIX_PASSES * 256; b += LG_THREADS) S.hist[slot * RADIX_PASSES * 256 + b] = 0;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  KD_FOR_CHUNKS(len) {
    for (uint32_t i = r0 + threadIdx.x; i < min(len, r0 + LG_CHUNK); i += LG_THREADS) {
      uint64_t row = static_cast<uint64_t>(start) + i;
      S.keys[row] = total_key(L.din[row * L.d + dim]);
    }
  }
}

// Histogram pass `pass`; first replays the pick of pass-1 from its histogram.
__global__ void k_lg_hist(Level L, LargeScratch S, int pass) {
  wait_prior_grid();
  __shared__ uint32_t sh[256];
  __shared__ uint64_t s_prefix;
  __shared__ uint32_t pick_scratch[LG_THREADS / 32 + 3];
  const uint64_t slot = blockIdx.x;
  if (S.seg_dim[slot] == NONE) return;
  const int first = static_cast<int>(S.seg_first[slot]);
  if (pass < first) return;  // a byte every key of the segment shares
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  if (blockIdx.y * LG_CHUNK >= len) return;
  for (int b = threadIdx.x; b < 256; b += LG_THREADS) sh[b] = 0;
  if (pass > first) {  // replay the previous pass's pick (every CTA of the segment agrees)
    uint64_t np;
    uint32_t nr;
    pick_digit_block(S.hist + (slot * RADIX_PASSES + pass - 1) * 256, pass - 1,
                     S.sel_prefix[slot * (RADIX_PASSES + 1) + pass - 1],
                     S.sel_rank[slot * (RADIX_PASSES + 1) + pass - 1], &np, &nr, pick_scratch);
    if (threadIdx.x == 0) {
      s_prefix = np;
      if (blockIdx.y == 0) {  // publish the state for the next pass
        S.sel_prefix[slot * (RADIX_PASSES + 1) + pass] = np;
        S.sel_rank[slot * (RADIX_PASSES + 1) + pass] = nr;
      }
    }
  } else if (threadIdx.x == 0) {
    s_prefix = S.sel_prefix[slot * (RADIX_PASSES + 1) + pass];
  }
  __syncthreads();
  const uint64_t prefix = s_prefix;
  const int shift = 56 - 8 * pass;
  const uint32_t lane = threadIdx.x & 31;
  KD_FOR_CHUNKS(len) {
    const uint32_t end = min(len, r0 + LG_CHUNK);
    uint64_t kk[LG_ITEMS];  // the thread's keys, loaded together
#pragma unroll
    for (int t = 0; t < LG_ITEMS; ++t) {
      const uint32_t i = r0 + threadIdx.x + t * LG_THREADS;
      kk[t] = i < end ? S.keys[static_cast<uint64_t>(start) + i] : 0;
    }
#pragma unroll
    for (int t = 0; t < LG_ITEMS; ++t) {  // uniform: whole warps count together
      const uint32_t i = r0 + threadIdx.x + t * LG_THREADS;
      bool in = false;
      uint32_t digit = 256 + lane;  // distinct per lane when not counted
      if (i < end) {
        const uint64_t k = kk[t];
        in = pass == 0 || ((k ^ prefix) >> (shift + 8)) == 0;
        if (in) digit = static_cast<uint32_t>(k >> shift) & 255u;
      }
      // one shared atomic per distinct digit of the warp (uniform data puts
      // most keys of a pass in a few bins)
      const uint32_t same = __match_any_sync(0xffffffffu, digit);
      if (in && lane == static_cast<uint32_t>(__ffs(same) - 1)) atomicAdd(&sh[digit], __popc(same));
    }
  }
  __syncthreads();
  uint32_t* g = S.hist + (slot * RADIX_PASSES + pass) * 256;
  for (int b = threadIdx.x; b < 256; b += LG_THREADS)
    if (sh[b]) atomicAdd(&g[b], sh[b]);
}

// Final pick -> pivot; then lt = #{key < pivot}.
__global__ void k_lg_count_lt(Level L, LargeScratch S) {
  wait_prior_grid();
  __shared__ uint32_t sh_warp[LG_THREADS / 32];
  __shared__ uint64_t s_pivot;
  __shared__ uint32_t pick_scratch[LG_THREADS / 32 + 3];
  const uint64_t slot = blockIdx.x;
  if (S.seg_dim[slot] == NONE) return;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  if (blockIdx.y * LG_CHUNK >= len) return;
  {
    const int p = RADIX_PASSES - 1;
    uint64_t np = S.sel_prefix[slot * (RADIX_PASSES + 1) + RADIX_PASSES];  // every key equal
    uint32_t nr;
    if (S.seg_first[slot] < static_cast<uint32_t>(RADIX_PASSES))
      pick_digit_block(S.hist + (slot * RADIX_PASSES + p) * 256, p, S.sel_prefix[slot * (RADIX_PASSES + 1) + p],
                       S.sel_rank[slot * (RADIX_PASSES + 1) + p], &np, &nr, pick_scratch);
    if (threadIdx.x == 0) {
      s_pivot = np;
      if (blockIdx.y == 0) S.seg_pivot[slot] = np;
    }
  }
  __syncthreads();
  const uint64_t pc = canon(s_pivot);
  uint32_t c = 0;
  KD_FOR_CHUNKS(len) {
    const uint32_t end = min(len, r0 + LG_CHUNK);
    uint64_t kk[LG_ITEMS];
#pragma unroll
    for (int t = 0; t < LG_ITEMS; ++t) {
      const uint32_t i = r0 + threadIdx.x + t * LG_THREADS;
      kk[t] = i < end ? S.keys[static_cast<uint64_t>(start) + i] : KEY_MAX;
    }
#pragma unroll
    for (int t = 0; t < LG_ITEMS; ++t) c += r0 + threadIdx.x + t * LG_THREADS < end && canon(kk[t]) < pc;
  }
  uint32_t total = block_sum<LG_THREADS>(c, sh_warp);
  if (threadIdx.x == 0 && total) atomicAdd(&S.seg_lt[slot], total);
}

__device__ __forceinline__ bool misplaced(uint64_t key, uint64_t pc, uint32_t i, uint32_t lt) {
  bool below = canon(key) < pc;
  return (i < lt) ? !below : below;
}

__global__ void k_lg_flagcount(Level L, LargeScratch S, uint32_t n_chunks) {
  wait_prior_grid();
  __shared__ uint32_t sh_warp[LG_THREADS / 32];
  const uint64_t slot = blockIdx.x;
  if (S.seg_dim[slot] == NONE) return;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  const uint64_t pc = canon(S.seg_pivot[slot]);
  const uint32_t lt = S.seg_lt[slot];
  KD_FOR_CHUNKS(len) {
    uint32_t c = 0;
    const uint32_t end = min(len, r0 + LG_CHUNK);
    uint64_t kk[LG_ITEMS];
#pragma unroll
    for (int t = 0; t < LG_ITEMS; ++t) {
      const uint32_t i = r0 + threadIdx.x + t * LG_THREADS;
      kk[t] = i < end ? S.keys[static_cast<uint64_t>(start) + i] : 0;
    }
#pragma unroll
    for (int t = 0; t < LG_ITEMS; ++t) {
      const uint32_t i = r0 + threadIdx.x + t * LG_THREADS;
      c += i < end && misplaced(kk[t], pc, i, lt);
    }
    uint32_t total = block_sum<LG_THREADS>(c, sh_warp);
    if (threadIdx.x == 0) S.chunk_cnt[slot * n_chunks + chunk] = total;
  }
}

__global__ void k_lg_chunkscan(Level L, LargeScratch S, uint32_t n_chunks) {
  wait_prior_grid();
  __shared__ uint32_t sh_warp[1024 / 32];
  __shared__ uint32_t s_run;
  const uint64_t slot = blockIdx.x;
  if (S.seg_dim[slot] == NONE) return;
  uint32_t* c = S.chunk_cnt + slot * n_chunks;
  if (threadIdx.x == 0) s_run = 0;
  __syncthreads();
  for (uint32_t b = 0; b < n_chunks; b += 1024) {
    uint32_t i = b + threadIdx.x;
    uint32_t v = i < n_chunks ? c[i] : 0;
    uint32_t tot;
    uint32_t ex = block_excl_scan<1024>(v, &tot, sh_warp);
    uint32_t run = s_run;
    if (i < n_chunks) c[i] = run + ex;
    __syncthreads();
    if (threadIdx.x == 0) s_run = run + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) S.seg_mis[slot] = s_run;
}

__global__ void k_lg_lists(Level L, LargeScratch S, uint32_t n_chunks) {
  wait_prior_grid();
  __shared__ uint32_t sh_warp[LG_THREADS / 32];
  const uint64_t slot = blockIdx.x;
  if (S.seg_dim[slot] == NONE) return;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  const uint64_t pc = canon(S.seg_pivot[slot]);
  const uint32_t lt = S.seg_lt[slot];
  KD_FOR_CHUNKS(len) {
  // each thread owns LG_ITEMS consecutive rows
  const uint32_t i0 = r0 + threadIdx.x * LG_ITEMS;
  uint32_t flags = 0, c = 0;
#pragma unroll
  for (int t = 0; t < LG_ITEMS; ++t) {
    uint32_t i = i0 + t;
    if (i < len && misplaced(S.keys[static_cast<uint64_t>(start) + i], pc, i, lt)) {
      flags |= 1u << t;
      ++c;
    }
  }
  uint32_t tot;
  uint32_t r = block_excl_scan<LG_THREADS>(c, &tot, sh_warp) + S.chunk_cnt[slot * n_chunks + chunk];
#pragma unroll
  for (int t = 0; t < LG_ITEMS; ++t) {
    uint32_t i = i0 + t;
    if (i >= len) break;
    uint64_t row = static_cast<uint64_t>(start) + i;
    if (flags & (1u << t)) {
      S.rankbuf[row] = r;
      S.plist[static_cast<uint64_t>(start) + r] = i;
      ++r;
    } else {
      S.rankbuf[row] = NONE;
    }
  }
  }
}

// Move rows to their post-swap positions; leaf segments copy through.
__global__ void k_lg_move(Level L, LargeScratch S) {
  wait_prior_grid();
  const uint64_t slot = blockIdx.x;
  const uint32_t node = L.seg_node[slot];
  if (node == HOLE) return;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  const bool inner = S.seg_dim[slot] != NONE;
  const uint32_t n2 = inner ? S.seg_mis[slot] : 0;
  const uint64_t d = L.d;
  KD_FOR_CHUNKS(len)
  for (uint32_t i = r0 + threadIdx.x; i < min(len, r0 + LG_CHUNK); i += LG_THREADS) {
    const uint64_t row = static_cast<uint64_t>(start) + i;
    uint32_t p = i;
    if (inner) {
      uint32_t r = S.rankbuf[row];
      if (r != NONE) p = S.plist[static_cast<uint64_t>(start) + n2 - 1 - r];
    }
    const uint64_t dst = static_cast<uint64_t>(start) + p;
    for (uint64_t j = 0; j < d; ++j) L.dout[dst * d + j] = L.din[row * d + j];
    L.iout[dst] = L.iin[row];
    if (inner) S.keys_out[dst] = S.keys[row];
  }
}

// Pivot-equal fix-up for large segments (build.rs:303-313), one CTA per
// segment, in place on the moved rows; only segments with mid > lt do work.
constexpr int FIX_THREADS = 1024;
__global__ void __launch_bounds__(FIX_THREADS) k_lg_fixup(Level L, LargeScratch S) {
  wait_prior_grid();
  __shared__ uint32_t sh_warp[FIX_THREADS / 32];
  __shared__ uint32_t s_count, s_changed, s_stop;
  const uint64_t slot = blockIdx.x;
  if (S.seg_dim[slot] == NONE) return;
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  const uint32_t lt = S.seg_lt[slot], mid = len / 2;
  if (mid <= lt) return;
  const uint32_t m = mid - lt;
  const uint64_t pc = canon(S.seg_pivot[slot]);
  const uint64_t d = L.d;
  const uint64_t base = start;
  uint32_t* E = S.plist + base;     // E[t]: relative position of the t-th pivot-equal row
  uint32_t* J = S.rankbuf + base;   // J[t]: chain pointer of place lt + t
  uint32_t* dest = reinterpret_cast<uint32_t*>(S.keys + base);  // destinations of [lt, stop]
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  // 1. first m pivot-equal rows of [lt, len), in order
  for (uint32_t b = lt; b < len; b += FIX_THREADS) {
    uint32_t i = b + threadIdx.x;
    uint32_t eq = (i < len) && canon(S.keys_out[base + i]) == pc;
    uint32_t tot;
    uint32_t r = block_excl_scan<FIX_THREADS>(eq, &tot, sh_warp);
    uint32_t c0 = s_count;
    if (eq && c0 + r < m) {
      E[c0 + r] = i;
      dest[i - lt] = lt + c0 + r;
    } else if (i < len) {
      dest[i - lt] = NONE;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_count = c0 + tot;
    __syncthreads();
    if (s_count >= m) break;
  }
  // The pivot is the mid-th order statistic, so [lt, len) holds at least m
  // pivot-equal rows; if not, leave the rows unpermuted rather than read past E.
  if (s_count < m) return;
  if (threadIdx.x == 0) s_stop = E[m - 1];
  __syncthreads();
  const uint32_t stop = s_stop;
  // 2. chains: the row at place lt+t moves to E[t]; follow until past the places
  for (uint32_t t = threadIdx.x; t < m; t += FIX_THREADS) J[t] = E[t];
  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) s_changed = 0;
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < m; t += FIX_THREADS) {
      uint32_t j = J[t];
      if (j - lt < m) {
        uint32_t nj = J[j - lt];
        if (nj != j) {
          J[t] = nj;
          s_changed = 1;
        }
      }
    }
    __syncthreads();
    if (!s_changed) break;
    __syncthreads();
  }
  // 3. destinations of the displaced (not pivot-equal or beyond the m-th) rows
  for (uint32_t i = lt + threadIdx.x; i <= stop; i += FIX_THREADS) {
    if (dest[i - lt] == NONE) dest[i - lt] = (i - lt < m) ? J[i - lt] : i;
  }
  __syncthreads();
  // 4. permute [lt, stop] through the (now free) source buffer of this segment
  double* tmp = const_cast<double*>(L.din);
  uint32_t* itmp = const_cast<uint32_t*>(L.iin);
  for (uint64_t f = static_cast<uint64_t>(lt) * d + threadIdx.x; f < (static_cast<uint64_t>(stop) + 1) * d;
       f += FIX_THREADS)
    tmp[base * d + f] = L.dout[base * d + f];
  for (uint32_t i = lt + threadIdx.x; i <= stop; i += FIX_THREADS) itmp[base + i] = L.iout[base + i];
  __syncthreads();
  for (uint64_t f = static_cast<uint64_t>(lt) * d + threadIdx.x; f < (static_cast<uint64_t>(stop) + 1) * d;
       f += FIX_THREADS) {
    uint32_t i = static_cast<uint32_t>(f / d);
    uint64_t j = f - static_cast<uint64_t>(i) * d;
    L.dout[(base + dest[i - lt]) * d + j] = tmp[base * d + f];
  }
  for (uint32_t i = lt + threadIdx.x; i <= stop; i += FIX_THREADS) L.iout[base + dest[i - lt]] = itmp[base + i];
}

__global__ void k_lg_expand(Level L, LargeScratch S) {
  wait_prior_grid();
  uint64_t slot = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (slot >= L.n_slots) return;
  const uint32_t node = L.seg_node[slot];
  if (node == HOLE) {
    L.nseg_node[2 * slot] = HOLE;
    L.nseg_node[2 * slot + 1] = HOLE;
    L.nseg_len[2 * slot] = 0;
    L.nseg_len[2 * slot + 1] = 0;
    return;
  }
  const uint32_t start = L.seg_start[slot], len = L.seg_len[slot];
  if (S.seg_dim[slot] == NONE) {
    close_leaf(L, slot, node, start, len);
    return;
  }
  expand_inner(L, slot, node, start, len, S.seg_dim[slot], S.seg_pivot[slot]);
  const uint64_t d = L.d;
  uint64_t* cl = L.boxkeys + static_cast<uint64_t>(node + 1) * 2 * d;
  uint64_t* cr = L.boxkeys + static_cast<uint64_t>(L.nseg_node[2 * slot + 1]) * 2 * d;
  for (uint64_t j = 0; j < 2 * d; ++j) {
    cl[j] = (j < d) ? KEY_MAX : 0;
    cr[j] = (j < d) ? KEY_MAX : 0;
  }
}

// All-leaf level: record the leaves.
__global__ void k_leaf_records(Level L) {
  wait_prior_grid();
  uint64_t slot = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (slot >= L.n_slots) return;
  const uint32_t node = L.seg_node[slot];
  if (node == HOLE) return;
  write_leaf(L.nodes, node, L.seg_start[slot], L.seg_len[slot]);
  L.node_len[node] = L.seg_len[slot];
}

// order_by_box (src/build.rs:234-238, 248-252), after every box is known.
__global__ void k_order_by_box(DNode* nodes, const uint64_t* boxkeys, const uint32_t* node_len,
                               uint64_t n_nodes, uint64_t d) {
  wait_prior_grid();
  uint64_t id = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (id >= n_nodes) return;
  DNode nd = nodes[id];
  if (nd.meta & KD_NODE_LEAF) return;
  if (d <= 1 || node_len[id] < 64) return;
  const uint32_t dim = nd.meta & KD_NODE_DIM_MASK;
  const uint64_t* own = boxkeys + id * 2 * d;
  const uint64_t kids[2] = {id + 1, nd.right};
  for (int c = 0; c < 2; ++c) {
    const uint64_t* ch = boxkeys + kids[c] * 2 * d;
    for (uint64_t j = 0; j < d; ++j) {
      if (j == dim) continue;
      double ce = dsub(from_total_key(ch[d + j]), from_total_key(ch[j]));
      double pe = dsub(from_total_key(own[d + j]), from_total_key(own[j]));
      if (!(ce < dmul(0.6, pe))) return;
    }
  }
  nodes[id].meta = nd.meta | KD_NODE_BOX_ORDER;
}

__global__ void k_boxes_finalize(uint64_t* boxkeys, uint64_t total) {
  wait_prior_grid();
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i < total) boxkeys[i] = from_total_key_bits(boxkeys[i]);
}

__global__ void k_root_segment(uint32_t* node, uint32_t* start, uint32_t* len, uint32_t n) {
  wait_prior_grid();
  *node = 0;
  *start = 0;
  *len = n;
}

__global__ void k_invert_rows(const uint32_t* idx, uint32_t* rows_of, uint64_t n) {
  wait_prior_grid();
  const uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (r < n) rows_of[idx[r]] = static_cast<uint32_t>(r);
}

__global__ void k_iota(uint32_t* idx, uint64_t n) {
  wait_prior_grid();
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i < n) idx[i] = static_cast<uint32_t>(i);
}

// FP32 filter copies: data rounded to nearest; boxes rounded outward.
__global__ void k_make_f32(const double* data, float* data32, uint64_t n_el, const double* boxes, float* boxes32,
                           uint64_t n_nodes, uint64_t d) {
  wait_prior_grid();
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i < n_el) data32[i] = __double2float_rn(data[i]);
  uint64_t nb = n_nodes * 2 * d;
  if (i < nb) {
    bool hi = ((i / d) & 1) != 0;
    boxes32[i] = hi ? __double2float_ru(boxes[i]) : __double2float_rd(boxes[i]);
  }
}

// Rows of `d` floats copied to rows of `w` (>= d) floats, zero padded: the
// runtime-width warp kernels load every row as whole float4 vectors.
__global__ void k_pad_rows(const float* src, uint64_t n, uint64_t d, uint64_t w, float* dst) {
  wait_prior_grid();
  const uint64_t f = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (f >= n * w) return;
  const uint64_t r = f / w, j = f - r * w;
  dst[f] = j < d ? src[r * d + j] : 0.f;
}

// Arrays carved out of one device block, each starting on a 256-byte boundary:
// a first pass with base == nullptr sizes the block, a second one sets the
// pointers.
struct Carve {
  unsigned char* base = nullptr;
  uint64_t off = 0;
  template <typename T>
  T* take(uint64_t count) {
    T* q = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += (std::max<uint64_t>(count, 1) * sizeof(T) + 255) / 256 * 256;
    return q;
  }
};

// A block from the library's stream-ordered pool, returned to it on the
// build's stream unless handed to the tree.
struct PoolBlock {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~PoolBlock() {
    if (p) cudaFreeAsync(p, st);
  }
  int alloc(uint64_t bytes, cudaStream_t s) {
    st = s;
    if (dev_alloc(&p, bytes, s) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
    }
    return KD_OK;
  }
};

inline unsigned grid1(uint64_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

uint64_t count_nodes(uint64_t len, uint64_t leafsize) { return count_nodes_impl(len, leafsize); }

int build_on_device(const double* d_src, uint64_t n, uint64_t d, uint64_t leafsize, cudaStream_t st,
                    kd_tree* t) {
  const uint64_t n_nodes = count_nodes_impl(n, leafsize);
  // Level structure (data-independent): sizes per depth, at most two values.
  struct LevelShape {
    uint64_t slots, max_len;
    bool any_inner;
  };
  std::vector<LevelShape> shape;
  {
    std::vector<std::pair<uint64_t, uint64_t>> cur = {{n, 1}};
    uint64_t slots = 1;
    for (;;) {
      LevelShape s{slots, 0, false};
      std::vector<std::pair<uint64_t, uint64_t>> nxt;
      for (auto& sc : cur) {
        s.max_len = std::max(s.max_len, sc.first);
        if (sc.first > leafsize) {
          s.any_inner = true;
          for (uint64_t h : {sc.first / 2, sc.first - sc.first / 2}) {
            auto it = std::find_if(nxt.begin(), nxt.end(), [&](auto& x) { return x.first == h; });
            if (it == nxt.end())
              nxt.push_back({h, sc.second});
            else
              it->second += sc.second;
          }
        }
      }
      shape.push_back(s);
      if (!s.any_inner) break;
      cur = nxt;
      slots *= 2;
    }
  }
  const uint64_t max_slots = shape.back().slots;
  uint64_t large_slots = 0;  // widest level handled by the large path
  for (auto& s : shape)
    if (s.any_inner && s.max_len > static_cast<uint64_t>(SMALL_MAX)) large_slots = std::max(large_slots, s.slots);
  const uint32_t max_chunks = static_cast<uint32_t>((n + LG_CHUNK - 1) / LG_CHUNK);

  // The levels above SMALL_MAX rows permute rows level by level (large path);
  // from the first level at or below it, one CTA per segment builds the rest
  // of that segment's subtree and writes its rows in their final order.  When
  // that level holds leaves only and lies below a large level (leafsize >
  // SMALL_MAX / 2), it just records them.  Level 0 reads the input itself; the
  // levels alternate between the tree's own row array and a scratch one,
  // arranged so that the last writer writes the tree's.
  size_t lv_small = 0;
  while (lv_small + 1 < shape.size() && shape[lv_small].max_len > static_cast<uint64_t>(SMALL_MAX) &&
         shape[lv_small].any_inner)
    ++lv_small;
  const bool by_subtree = shape[lv_small].max_len <= static_cast<uint64_t>(SMALL_MAX) &&
                          (lv_small == 0 || shape[lv_small].any_inner);
  const size_t n_perm = lv_small + (by_subtree ? 1 : 0);  // writers: large levels (+ the subtree kernel)
  const bool need_pad = padded_rows(d) && (d + 3) / 4 * 4 != d;
  const uint64_t w32 = (d + 3) / 4 * 4;

  // The tree's arrays: one pool block, owned by the tree.
  struct TreeArrays {
    double* data;
    uint32_t* idx;
    uint32_t* rows_of;
    DNode* nodes;
    uint64_t* boxes;
    float *data32, *boxes32, *data32w;
  } T{};
  auto carve_tree = [&](Carve& c) {
    T.data = c.take<double>(n * d);
    T.idx = c.take<uint32_t>(n);
    T.rows_of = c.take<uint32_t>(n);
    T.nodes = c.take<DNode>(n_nodes);
    T.boxes = c.take<uint64_t>(n_nodes * 2 * d);
    T.data32 = c.take<float>(n * d);
    T.boxes32 = c.take<float>(n_nodes * 2 * d);
    T.data32w = need_pad ? c.take<float>(n * w32) : nullptr;
  };
  // Scratch: one pool block, returned on the build's stream at the end.
  struct Scratch {
    double* data;
    uint32_t* idx;
    uint32_t* node_len;
    uint32_t* status;
    uint32_t* seg[2][3];
    LargeScratch lg;
  } X{};
  auto carve_scratch = [&](Carve& c) {
    X.data = c.take<double>(n * d);
    X.idx = c.take<uint32_t>(n);
    X.node_len = c.take<uint32_t>(n_nodes);
    X.status = c.take<uint32_t>(1);
    for (auto& sg : X.seg)
      for (auto& a : sg) a = c.take<uint32_t>(max_slots);
    if (large_slots) {
      X.lg.keys = c.take<uint64_t>(n);
      X.lg.keys_out = c.take<uint64_t>(n);
      X.lg.rankbuf = c.take<uint32_t>(n);
      X.lg.plist = c.take<uint32_t>(n);
      X.lg.hist = c.take<uint32_t>(large_slots * RADIX_PASSES * 256);
      X.lg.sel_prefix = c.take<uint64_t>(large_slots * (RADIX_PASSES + 1));
      X.lg.sel_rank = c.take<uint32_t>(large_slots * (RADIX_PASSES + 1));
      X.lg.seg_dim = c.take<uint32_t>(large_slots);
      X.lg.seg_pivot = c.take<uint64_t>(large_slots);
      X.lg.seg_lt = c.take<uint32_t>(large_slots);
      X.lg.chunk_cnt = c.take<uint32_t>(large_slots * static_cast<uint64_t>(max_chunks));
      X.lg.seg_mis = c.take<uint32_t>(large_slots);
      X.lg.seg_first = c.take<uint32_t>(large_slots);
    }
  };
  PoolBlock tree_block, scratch_block;
  int rc;
  {
    Carve ct, cs;
    carve_tree(ct);
    carve_scratch(cs);
    if ((rc = tree_block.alloc(ct.off, st)) || (rc = scratch_block.alloc(cs.off, st))) return rc;
    ct = Carve{static_cast<unsigned char*>(tree_block.p), 0};
    cs = Carve{static_cast<unsigned char*>(scratch_block.p), 0};
    carve_tree(ct);
    carve_scratch(cs);
  }
  // writer lv (the large levels, then the subtree kernel) writes the tree's
  // arrays when (n_perm - 1 - lv) is even
  auto writes_tree = [&](size_t lv) { return ((n_perm - 1 - lv) & 1) == 0; };

  KD_TRY_CUDA(chain(k_init_boxkeys, grid1(2 * d, 256), 256, 0, st, T.boxes, 1, d));
  KD_TRY_CUDA(cudaMemsetAsync(X.status, 0, sizeof(uint32_t), st));
  const double* din;
  const uint32_t* iin;
  if (n_perm == 0) {  // the root is a leaf of more than SMALL_MAX rows
    KD_TRY_CUDA(cudaMemcpyAsync(T.data, d_src, n * d * sizeof(double), cudaMemcpyDeviceToDevice, st));
    KD_TRY_CUDA(chain(k_iota, grid1(n, 256), 256, 0, st, T.idx, n));
    din = T.data;
    iin = T.idx;
  } else {
    // the identity permutation sits in the index array level 0 does not write
    uint32_t* iota = writes_tree(0) ? X.idx : T.idx;
    KD_TRY_CUDA(chain(k_iota, grid1(n, 256), 256, 0, st, iota, n));
    din = d_src;
    iin = iota;
  }
  KD_TRY_CUDA(chain(k_root_segment, 1, 1, 0, st, X.seg[0][0], X.seg[0][1], X.seg[0][2], static_cast<uint32_t>(n)));
  KD_TRY_CUDA(cudaGetLastError());
  KD_TRY_CUDA(cudaFuncSetAttribute(k_small_subtree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(sizeof(SubShared))));

  int cur = 0;
  const unsigned bbox_threads = d <= 256 ? static_cast<unsigned>(d * (256 / d)) : 256u;

  for (size_t lv = 0; lv < shape.size(); ++lv) {
    const LevelShape& s = shape[lv];
    double* dout = nullptr;
    uint32_t* iout = nullptr;
    if (lv < n_perm) {
      dout = writes_tree(lv) ? T.data : X.data;
      iout = writes_tree(lv) ? T.idx : X.idx;
    }
    Level L{din, dout, iin, iout, d, leafsize,
            X.seg[cur][0], X.seg[cur][1], X.seg[cur][2],
            X.seg[cur ^ 1][0], X.seg[cur ^ 1][1], X.seg[cur ^ 1][2],
            T.nodes, T.boxes, X.node_len, s.slots};
    if (lv == lv_small && by_subtree) {
      // every box, split and record below, and the rows in their final order;
      // at level 0 it also checks that every coordinate is finite
      SubArgs A{din, iin, dout, iout, d, static_cast<uint32_t>(leafsize),
                X.seg[cur][0], X.seg[cur][1], X.seg[cur][2], T.nodes, T.boxes, X.node_len, lv == 0, X.status};
      KD_TRY_CUDA(chain(k_small_subtree, static_cast<unsigned>(s.slots), SUB_THREADS, sizeof(SubShared), st, A));
      KD_TRY_CUDA(cudaGetLastError());
      break;
    }
    // Boxes of the large levels (and of a leaves-only last level) come from the
    // bbox kernel.  Level 0 also checks that every coordinate is finite; the
    // status is read once the build has finished (non-finite keys still order
    // consistently).
    {
      const uint64_t chunk_rows = std::max<uint64_t>(1, (bbox_threads * 8) / d);
      const uint64_t nchunk = (s.max_len + chunk_rows - 1) / chunk_rows;
      dim3 g(static_cast<unsigned>(s.slots), static_cast<unsigned>(std::min<uint64_t>(nchunk, 65535)));
      KD_TRY_CUDA(chain(k_bbox, g, bbox_threads, 2 * d * sizeof(uint64_t), st, L, static_cast<uint32_t>(chunk_rows),
                                                                static_cast<uint32_t>(nchunk), lv == 0, X.status));
      KD_TRY_CUDA(cudaGetLastError());
    }
    if (!s.any_inner) {
      KD_TRY_CUDA(chain(k_leaf_records, grid1(s.slots, 256), 256, 0, st, L));
      KD_TRY_CUDA(cudaGetLastError());
      break;
    }
    {
      const LargeScratch& S = X.lg;
      const uint32_t nch = static_cast<uint32_t>((s.max_len + LG_CHUNK - 1) / LG_CHUNK);
      dim3 g(static_cast<unsigned>(s.slots), std::min<uint32_t>(nch, 65535u));
      KD_TRY_CUDA(chain(k_lg_prepare, grid1(s.slots, 256), 256, 0, st, L, S));
      KD_TRY_CUDA(chain(k_lg_keys, g, LG_THREADS, 0, st, L, S));
      for (int pass = 0; pass < RADIX_PASSES; ++pass) KD_TRY_CUDA(chain(k_lg_hist, g, LG_THREADS, 0, st, L, S, pass));
      KD_TRY_CUDA(chain(k_lg_count_lt, g, LG_THREADS, 0, st, L, S));
      KD_TRY_CUDA(chain(k_lg_flagcount, g, LG_THREADS, 0, st, L, S, nch));
      KD_TRY_CUDA(chain(k_lg_chunkscan, static_cast<unsigned>(s.slots), 1024, 0, st, L, S, nch));
      KD_TRY_CUDA(chain(k_lg_lists, g, LG_THREADS, 0, st, L, S, nch));
      KD_TRY_CUDA(chain(k_lg_move, g, LG_THREADS, 0, st, L, S));
      KD_TRY_CUDA(chain(k_lg_fixup, static_cast<unsigned>(s.slots), FIX_THREADS, 0, st, L, S));
      KD_TRY_CUDA(chain(k_lg_expand, grid1(s.slots, 256), 256, 0, st, L, S));
      KD_TRY_CUDA(cudaGetLastError());
    }
    din = dout;
    iin = iout;
    cur ^= 1;
  }

  KD_TRY_CUDA(chain(k_order_by_box, grid1(n_nodes, 256), 256, 0, st, T.nodes, T.boxes, X.node_len, n_nodes, d));
  KD_TRY_CUDA(chain(k_boxes_finalize, grid1(n_nodes * 2 * d, 256), 256, 0, st, T.boxes, n_nodes * 2 * d));
  KD_TRY_CUDA(cudaGetLastError());

  // The final row order sits in the tree's row array (din).
  KD_TRY_CUDA(chain(k_invert_rows, grid1(n, 256), 256, 0, st, T.idx, T.rows_of, n));
  KD_TRY_CUDA(chain(k_make_f32, grid1(std::max(n * d, n_nodes * 2 * d), 256), 256, 0, st, 
      T.data, T.data32, n * d, reinterpret_cast<const double*>(T.boxes), T.boxes32, n_nodes, d));
  KD_TRY_CUDA(cudaGetLastError());
  // FP32 rows padded to a multiple of 4 floats for width 3 and the
  // runtime-width warp kernels (widths other than 1, 2, 3, 4, 8, 16, up to
  // 128): the FP32 copy itself when d is a multiple of 4
  if (need_pad) {
    KD_TRY_CUDA(chain(k_pad_rows, grid1(n * w32, 256), 256, 0, st, T.data32, n, d, w32, T.data32w));
    KD_TRY_CUDA(cudaGetLastError());
  }
  // The one host synchronisation: the finiteness status and the root box.
  std::vector<double> root_box(2 * d);
  uint32_t h_status = 0;
  KD_TRY_CUDA(cudaMemcpyAsync(&h_status, X.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaMemcpyAsync(root_box.data(), T.boxes, 2 * d * sizeof(double), cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  if (h_status) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
  double cmax = 0.0;  // the root box holds every coordinate
  for (double v : root_box) cmax = std::max(cmax, std::fabs(v));
  float cmax32 = static_cast<float>(cmax);
  while (static_cast<double>(cmax32) < cmax) cmax32 = std::nextafter(cmax32, INFINITY);
  t->coord_max32 = cmax32;

  t->n_points = n;
  t->ndim = d;
  t->leafsize = leafsize;
  t->n_nodes = n_nodes;
  t->block = tree_block.p;
  tree_block.p = nullptr;
  t->data = T.data;
  t->indices = T.idx;
  t->rows_of = T.rows_of;
  t->nodes = T.nodes;
  t->boxes = reinterpret_cast<double*>(T.boxes);
  t->data32 = T.data32;
  t->boxes32 = T.boxes32;
  t->w32 = static_cast<uint32_t>(w32);
  t->data32w = need_pad ? T.data32w : T.data32;
  return KD_OK;
}

}  // namespace kd
