/*
 * kd_oracle.c -- CPU restatement of FujishigeTemma/kdtree-rs's kd-tree build and
 * exact k-NN query.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU engine is compared
 * against, and the timed CPU baseline ("kind": "port") in bench.py.  Nothing in
 * the product (the CUDA library and the `kdtree` Python package) links, loads or
 * calls it; the product fails loudly instead of falling back to it.
 *
 * Every function names the reference file:line it follows.  The arithmetic is
 * restated operation by operation so the FP64 results are bit-identical to the
 * reference's on the same platform:
 *   - no FMA contraction (build with -ffp-contract=off, as rustc never contracts),
 *   - the per-strategy summation orders of src/kernel.rs (Packed d4/d8 chunk
 *     versus tail, Folded lane accumulation + hsum, Streamed per-chunk hsum),
 *   - the DFS order, plane bounds and box gates of src/query.rs,
 *   - the row permutation of src/build.rs:266-314 (partition_rows).
 * Pinning: tests/test_oracle.py checks this oracle against the reference's own
 * test oracle (SciPy, tests/test_kdtree.py:55-89 of the reference) on the
 * reference's table cases and on random problems, and against committed golden
 * fixtures generated by SciPy (tests/golden/make_golden.py).
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC (see oracle/Makefile).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Status codes: the same numbering as include/kdtree_gb300.h (KD_*). */
enum {
  ORK_OK = 0,
  ORK_EMPTY_DATA = 1,
  ORK_INVALID_LEAFSIZE = 2,
  ORK_INVALID_K = 3,
  ORK_INVALID_METRIC = 4,
  ORK_INVALID_EPS = 5,
  ORK_INVALID_MAX_DISTANCE = 6,
  ORK_NONFINITE_DATA = 7,
  ORK_TOO_MANY_POINTS = 8,
  ORK_TOO_MANY_NODES = 9,
  ORK_INVALID_SHAPE = 10,
  ORK_OUT_OF_MEMORY = 101,
};

/* Metric kinds (src/metric.rs:37-42). */
enum { M_L1 = 0, M_L2 = 1, M_LINF = 2, M_LP = 3 };
/* Scan strategies (src/kernel.rs:244-270). */
enum { S_PACKED = 0, S_FOLDED = 1, S_STREAMED = 2 };

#define LANES 8 /* src/simd.rs:6 */
#define BOX_ORDER_MAX_SHRINK_RATIO 0.6 /* src/build.rs:13 */
#define BOX_ORDER_MIN_SUBTREE 64       /* src/build.rs:17 */

/* One node of the flat preorder array (src/tree.rs:11-27).  Leaf: [a, b) rows.
 * Inner: a = left id, b = right id. */
typedef struct {
  uint32_t is_leaf;
  uint32_t a;
  uint32_t b;
  uint32_t split_dim;
  uint32_t order_by_box;
  uint32_t pad_;
  double split_value;
} ork_node;

typedef struct {
  double* data;      /* n_points x ndim, tree order (src/tree.rs:30) */
  uint32_t* indices; /* tree position -> original row (src/tree.rs:31) */
  ork_node* nodes;   /* preorder, left child = id + 1 (src/tree.rs:1-4) */
  double* boxes;     /* per node [lo[ndim] | hi[ndim]] (src/layout.rs:197-225) */
  uint64_t n_points, ndim, leafsize, n_nodes;
} ork_tree;

/* ------------------------------------------------------------------ */
/* Shape of the tree (src/build.rs:161-173).                           */
/* ------------------------------------------------------------------ */

/* count_nodes (src/build.rs:166-173).  The reference recurses over every node;
 * the sizes at one depth take at most two adjacent values, so the same count is
 * accumulated level by level over (size, multiplicity) pairs. */
uint64_t ork_count_nodes(uint64_t len, uint64_t leafsize) {
  uint64_t sz[4], cnt[4];
  int n = 1;
  sz[0] = len;
  cnt[0] = 1;
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

/* ------------------------------------------------------------------ */
/* Total order on f64 (Rust's f64::total_cmp).                         */
/* ------------------------------------------------------------------ */
static inline uint64_t total_key(double v) {
  uint64_t b;
  memcpy(&b, &v, 8);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
static inline double from_total_key(uint64_t k) {
  uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  memcpy(&v, &b, 8);
  return v;
}

/* The mid-th smallest key.  Only the VALUE matters (src/build.rs:204-205 keeps
 * the rows untouched and reads the pivot out), so any exact selection gives the
 * reference's pivot.  Iterative three-way quickselect, median-of-three. */
static uint64_t select_nth(uint64_t* k, size_t len, size_t nth) {
  size_t lo = 0, hi = len; /* [lo, hi) contains nth */
  while (hi - lo > 1) {
    size_t m = lo + (hi - lo) / 2;
    uint64_t a = k[lo], b = k[m], c = k[hi - 1];
    uint64_t piv = (a < b) ? ((b < c) ? b : (a < c ? c : a)) : ((a < c) ? a : (b < c ? c : b));
    /* Dutch-flag partition: [lo, lt) < piv, [lt, gt) == piv, [gt, hi) > piv */
    size_t lt = lo, i = lo, gt = hi;
    while (i < gt) {
      uint64_t x = k[i];
      if (x < piv) {
        k[i] = k[lt];
        k[lt] = x;
        ++lt;
        ++i;
      } else if (x > piv) {
        --gt;
        k[i] = k[gt];
        k[gt] = x;
      } else {
        ++i;
      }
    }
    if (nth < lt)
      hi = lt;
    else if (nth >= gt)
      lo = gt;
    else
      return piv;
  }
  return k[lo];
}

/* ------------------------------------------------------------------ */
/* Build (src/build.rs:19-314).                                        */
/* ------------------------------------------------------------------ */

typedef struct {
  uint64_t leafsize, ndim;
  int parallel;
  double* data;
  uint32_t* indices;
  ork_node* nodes;
  double* boxes;
  uint64_t* keys;
  uint32_t* marks;
} build_ctx;

/* bbox_into (src/kernel.rs:79-151): per-dimension min / max of a block.  Min and
 * max are exact, so the reference's lane-wise order gives the same values (the
 * sign of a zero bound aside, which no query result depends on). */
static void bbox_into(const build_ctx* c, size_t first, size_t len, double* lo, double* hi) {
  const size_t d = c->ndim;
  for (size_t j = 0; j < d; ++j) {
    lo[j] = INFINITY;
    hi[j] = -INFINITY;
  }
  const double* r = c->data + first * d;
  for (size_t i = 0; i < len; ++i, r += d)
    for (size_t j = 0; j < d; ++j) {
      double v = r[j];
      if (v < lo[j]) lo[j] = v;
      if (v > hi[j]) hi[j] = v;
    }
}

/* widest_axis (src/layout.rs:168-179): strict '>', ties to the lowest dim. */
static size_t widest_axis(const double* lo, const double* hi, size_t d) {
  size_t best = 0;
  double span = hi[0] - lo[0];
  for (size_t j = 1; j < d; ++j) {
    double s = hi[j] - lo[j];
    if (s > span) {
      span = s;
      best = j;
    }
  }
  return best;
}

static inline void swap_rows(double* data, uint32_t* idx, size_t d, size_t a, size_t b) {
  if (a == b) return;
  double* ra = data + a * d;
  double* rb = data + b * d;
  for (size_t j = 0; j < d; ++j) {
    double t = ra[j];
    ra[j] = rb[j];
    rb[j] = t;
  }
  uint32_t t = idx[a];
  idx[a] = idx[b];
  idx[b] = t;
}

/* partition_rows (src/build.rs:266-314), the exact permutation:
 *   R = ascending positions in [0, lt) with key >= pivot,
 *   L = ascending positions in [lt, len) with key <  pivot,
 *   swap R[i] <-> L[n-1-i], then move pivot-equal rows into [lt, mid). */
static void partition_rows(double* data, uint32_t* idx, uint32_t* marks, size_t len, size_t d,
                           size_t dim, double pivot, size_t lt, size_t mid) {
  uint32_t* right_of_lt = marks;
  uint32_t* left_of_ge = marks + lt;
  size_t n_right = 0, n_left = 0;
  for (size_t row = 0; row < lt; ++row) {
    right_of_lt[n_right] = (uint32_t)row;
    n_right += (data[row * d + dim] >= pivot);
  }
  for (size_t row = lt; row < len; ++row) {
    left_of_ge[n_left] = (uint32_t)row;
    n_left += (data[row * d + dim] < pivot);
  }
  for (size_t pair = 0; pair < n_right; ++pair)
    swap_rows(data, idx, d, right_of_lt[pair], left_of_ge[n_left - 1 - pair]);
  size_t place = lt, scan = lt;
  while (place < mid) {
    if (data[scan * d + dim] == pivot) {
      swap_rows(data, idx, d, scan, place);
      ++place;
    }
    ++scan;
  }
}

/* shrank_off_axis (src/build.rs:248-252). */
static int shrank_off_axis(const double* p, const double* ch, size_t d, size_t split_dim) {
  for (size_t j = 0; j < d; ++j) {
    if (j == split_dim) continue;
    double ce = ch[d + j] - ch[j];
    double pe = p[d + j] - p[j];
    if (!(ce < BOX_ORDER_MAX_SHRINK_RATIO * pe)) return 0;
  }
  return 1;
}

static void build_subtree(const build_ctx* c, size_t first, size_t len, uint32_t id);

/* bound_and_build (src/build.rs:175-181). */
static void bound_and_build(const build_ctx* c, size_t first, size_t len, uint32_t id) {
  double* box = c->boxes + (size_t)id * 2 * c->ndim;
  bbox_into(c, first, len, box, box + c->ndim);
  build_subtree(c, first, len, id);
}

/* build_subtree (src/build.rs:184-246).  `first` is the global row offset. */
static void build_subtree(const build_ctx* c, size_t first, size_t len, uint32_t id) {
  const size_t d = c->ndim;
  ork_node* node = c->nodes + id;
  if (len <= c->leafsize) {
    node->is_leaf = 1;
    node->a = (uint32_t)first;
    node->b = (uint32_t)(first + len);
    node->split_dim = 0;
    node->order_by_box = 0;
    node->split_value = 0.0;
    return;
  }
  const double* own = c->boxes + (size_t)id * 2 * d;
  size_t split_dim = widest_axis(own, own + d, d);
  size_t mid = len / 2; /* split_point (src/build.rs:162-164) */
  double* rows = c->data + first * d;
  uint64_t* keys = c->keys + first;
  for (size_t i = 0; i < len; ++i) keys[i] = total_key(rows[i * d + split_dim]);
  double pivot = from_total_key(select_nth(keys, len, mid));
  size_t lt = 0; /* src/build.rs:209 -- '<', not total order */
  for (size_t i = 0; i < len; ++i) lt += (rows[i * d + split_dim] < pivot);
  partition_rows(rows, c->indices + first, c->marks + first, len, d, split_dim, pivot, lt, mid);

  uint64_t left_nodes = ork_count_nodes(mid, c->leafsize);
  uint32_t left_id = id + 1;
  uint32_t right_id = id + 1 + (uint32_t)left_nodes;
  if (c->parallel && len >= 8192) {
#pragma omp task default(shared) firstprivate(first, mid, left_id)
    bound_and_build(c, first, mid, left_id);
#pragma omp task default(shared) firstprivate(first, mid, len, right_id)
    bound_and_build(c, first + mid, len - mid, right_id);
#pragma omp taskwait
  } else {
    bound_and_build(c, first, mid, left_id);
    bound_and_build(c, first + mid, len - mid, right_id);
  }
  const double* lb = c->boxes + (size_t)left_id * 2 * d;
  const double* rb = c->boxes + (size_t)right_id * 2 * d;
  int obb = d > 1 && len >= BOX_ORDER_MIN_SUBTREE && shrank_off_axis(own, lb, d, split_dim) &&
            shrank_off_axis(own, rb, d, split_dim);
  node->is_leaf = 0;
  node->a = left_id;
  node->b = right_id;
  node->split_dim = (uint32_t)split_dim;
  node->order_by_box = (uint32_t)obb;
  node->split_value = pivot;
}

void ork_free(ork_tree* t) {
  if (!t) return;
  free(t->data);
  free(t->indices);
  free(t->nodes);
  free(t->boxes);
  free(t);
}

/* build (src/build.rs:19-82).  `data` holds n_values = n_points * ndim values. */
int ork_build(const double* data, uint64_t n_values, uint64_t ndim, uint64_t leafsize, int parallel,
              ork_tree** out) {
  *out = NULL;
  if (leafsize == 0) return ORK_INVALID_LEAFSIZE;
  if (ndim == 0 || n_values == 0) return ORK_EMPTY_DATA;
  if (n_values % ndim) return ORK_INVALID_SHAPE;
  uint64_t n = n_values / ndim;
  if (n > 0xffffffffull) return ORK_TOO_MANY_POINTS;
  uint64_t n_nodes = ork_count_nodes(n, leafsize);
  if (n_nodes > 0xffffffffull) return ORK_TOO_MANY_NODES;
  /* all_finite (src/kernel.rs:67-74) fused into the root box (src/build.rs:51-57) */
  for (uint64_t i = 0; i < n_values; ++i)
    if (!isfinite(data[i])) return ORK_NONFINITE_DATA;

  ork_tree* t = (ork_tree*)calloc(1, sizeof(ork_tree));
  if (!t) return ORK_OUT_OF_MEMORY;
  t->n_points = n;
  t->ndim = ndim;
  t->leafsize = leafsize;
  t->n_nodes = n_nodes;
  t->data = (double*)malloc(n_values * sizeof(double));
  t->indices = (uint32_t*)malloc(n * sizeof(uint32_t));
  t->nodes = (ork_node*)calloc(n_nodes, sizeof(ork_node));
  t->boxes = (double*)calloc(n_nodes * 2 * ndim, sizeof(double));
  uint64_t* keys = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint32_t* marks = (uint32_t*)malloc(n * sizeof(uint32_t));
  if (!t->data || !t->indices || !t->nodes || !t->boxes || !keys || !marks) {
    free(keys);
    free(marks);
    ork_free(t);
    return ORK_OUT_OF_MEMORY;
  }
  memcpy(t->data, data, n_values * sizeof(double));
  for (uint64_t i = 0; i < n; ++i) t->indices[i] = (uint32_t)i;

  build_ctx c = {leafsize, ndim, parallel, t->data, t->indices, t->nodes, t->boxes, keys, marks};
  bbox_into(&c, 0, n, t->boxes, t->boxes + ndim);
  if (parallel) {
#pragma omp parallel
#pragma omp single
    build_subtree(&c, 0, n, 0);
  } else {
    build_subtree(&c, 0, n, 0);
  }
  free(keys);
  free(marks);
  *out = t;
  return ORK_OK;
}

/* ------------------------------------------------------------------ */
/* Metric algebra (src/metric.rs:44-99).                               */
/* ------------------------------------------------------------------ */
typedef struct {
  int kind;
  double p;
} metric_t;

static inline double m_reduce(metric_t m, double x) { /* metric.rs:64-71 */
  switch (m.kind) {
    case M_L2: return x * x;
    case M_LP: return pow(x, m.p);
    default: return x;
  }
}
static inline double m_restore(metric_t m, double x) { /* metric.rs:74-80 */
  switch (m.kind) {
    case M_L2: return sqrt(x);
    case M_LP: return pow(x, 1.0 / m.p);
    default: return x;
  }
}
static inline double fmax_nn(double a, double b) { return b > a ? b : a; }

/* axis_offset (src/layout.rs:147-149). */
static inline double axis_offset(double q, double lo, double hi) {
  double a = lo - q, b = q - hi;
  double m = a > b ? a : b;
  return m > 0.0 ? m : 0.0;
}

/* hsum (src/simd.rs:26-30). */
static inline double hsum8(const double* v) {
  return ((v[0] + v[4]) + (v[2] + v[6])) + ((v[1] + v[5]) + (v[3] + v[7]));
}

static inline double axis_of(int kind, double delta) { /* axes_lanes, kernel.rs:22-29 */
  return kind == M_L2 ? delta * delta : fabs(delta);
}

/* fold_scalar (src/kernel.rs:40-65): sequential ((dist + a0) + a1) + ... */
static inline double fold_seq(int kind, double dist, const double* q, const double* p, size_t n) {
  if (kind == M_LINF) {
    for (size_t i = 0; i < n; ++i) {
      double delta = fabs(q[i] - p[i]);
      if (delta > dist) dist = delta;
    }
  } else if (kind == M_L2) {
    for (size_t i = 0; i < n; ++i) {
      double delta = q[i] - p[i];
      dist += delta * delta;
    }
  } else {
    for (size_t i = 0; i < n; ++i) dist += fabs(q[i] - p[i]);
  }
  return dist;
}

/* Full reduced distance of one leaf point under the reference's strategy.
 * `in_chunk` is true when a Packed d4/d8 point sits inside a full SIMD chunk of
 * its leaf (src/kernel.rs:441-457); elsewhere the order does not depend on the
 * position.  The Streamed early exit (kernel.rs:183-185, 213-215) only ever
 * returns values already above the bound, which are rejected either way, so the
 * full value is computed here and compared to the bound by the caller. */
static inline double point_dist(metric_t m, int strat, const double* q, const double* p, size_t d,
                                int in_chunk) {
  const int kind = m.kind;
  if (kind == M_LP) { /* point_dist_lp (kernel.rs:207-218) */
    double dist = 0.0;
    for (size_t i = 0; i < d; ++i) dist += pow(fabs(q[i] - p[i]), m.p);
    return dist;
  }
  if (kind == M_LINF) { /* max: order-free (kernel.rs:190-205, 470-562) */
    double dist = 0.0;
    for (size_t i = 0; i < d; ++i) {
      double delta = fabs(q[i] - p[i]);
      if (delta > dist) dist = delta;
    }
    return dist;
  }
  if (strat == S_PACKED) {
    if (d == 4 && in_chunk) { /* d4 (kernel.rs:517-533) */
      double a0 = axis_of(kind, p[0] - q[0]), a1 = axis_of(kind, p[1] - q[1]);
      double a2 = axis_of(kind, p[2] - q[2]), a3 = axis_of(kind, p[3] - q[3]);
      return (a0 + a2) + (a1 + a3);
    }
    if (d == 8 && in_chunk) { /* d8 (kernel.rs:540-562) */
      double a[8];
      for (int i = 0; i < 8; ++i) a[i] = axis_of(kind, p[i] - q[i]);
      return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    }
    /* d1..d3, d5..d7 and every tail point: sequential (kernel.rs:414-435, 472-513) */
    return fold_seq(kind, 0.0, q, p, d);
  }
  size_t nch = d / LANES;
  if (strat == S_FOLDED) { /* point_dist_folded (kernel.rs:343-354) */
    double acc[LANES] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t c = 0; c < nch; ++c)
      for (int j = 0; j < LANES; ++j) acc[j] += axis_of(kind, q[c * LANES + j] - p[c * LANES + j]);
    double dist = nch ? hsum8(acc) : 0.0;
    return fold_seq(kind, dist, q + nch * LANES, p + nch * LANES, d - nch * LANES);
  }
  /* Streamed L1/L2: point_dist_sum (kernel.rs:177-188) */
  double dist = 0.0;
  for (size_t c = 0; c < nch; ++c) {
    double v[LANES];
    for (int j = 0; j < LANES; ++j) v[j] = axis_of(kind, q[c * LANES + j] - p[c * LANES + j]);
    dist += hsum8(v);
  }
  return fold_seq(kind, dist, q + nch * LANES, p + nch * LANES, d - nch * LANES);
}

/* box_dist (src/kernel.rs:565-616). */
static inline double box_dist(metric_t m, const double* q, const double* box, size_t d) {
  const double* lo = box;
  const double* hi = box + d;
  if (m.kind == M_LINF) {
    double worst = 0.0;
    for (size_t i = 0; i < d; ++i) {
      double off = axis_offset(q[i], lo[i], hi[i]);
      if (off > worst) worst = off;
    }
    return worst;
  }
  if (m.kind == M_LP) {
    double dist = 0.0;
    for (size_t i = 0; i < d; ++i) {
      double off = axis_offset(q[i], lo[i], hi[i]);
      if (off > 0.0) dist += pow(off, m.p);
    }
    return dist;
  }
  size_t nch = d / LANES;
  double acc[LANES] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (size_t c = 0; c < nch; ++c)
    for (int j = 0; j < LANES; ++j) {
      size_t i = c * LANES + j;
      double off = fmax_nn(fmax_nn(lo[i] - q[i], q[i] - hi[i]), 0.0);
      acc[j] += axis_of(m.kind, off);
    }
  double dist = nch ? hsum8(acc) : 0.0;
  for (size_t i = nch * LANES; i < d; ++i) dist += m_reduce(m, axis_offset(q[i], lo[i], hi[i]));
  return dist;
}

/* ------------------------------------------------------------------ */
/* Query (src/query.rs).                                               */
/* ------------------------------------------------------------------ */

/* BestK / Best1 (src/query.rs:379-494), with Best1 as the k == 1 case of the
 * same sorted list: `consider` keeps the k smallest by (dist, idx). */
typedef struct {
  size_t k, len;
  double* dists;
  uint32_t* ids;
} best_t;

static inline double best_bound(const best_t* b, double cutoff) { /* query.rs:408-411, 452-459 */
  if (b->len < b->k) return cutoff;
  double w = b->dists[b->k - 1];
  return w < cutoff ? w : cutoff;
}

static inline void best_consider(best_t* b, double dist, uint32_t idx) { /* query.rs:413-419, 461-481 */
  if (b->len == b->k) {
    double wd = b->dists[b->k - 1];
    if (dist > wd || (dist == wd && b->ids[b->k - 1] <= idx)) return;
    b->len--;
  }
  size_t pos = b->len;
  while (pos > 0) {
    double pd = b->dists[pos - 1];
    if (pd < dist || (pd == dist && b->ids[pos - 1] < idx)) break;
    pos--;
  }
  memmove(b->dists + pos + 1, b->dists + pos, (b->len - pos) * sizeof(double));
  memmove(b->ids + pos + 1, b->ids + pos, (b->len - pos) * sizeof(uint32_t));
  b->dists[pos] = dist;
  b->ids[pos] = idx;
  b->len++;
}

typedef struct {
  const ork_tree* t;
  metric_t m;
  int strat;
  double cutoff, eps_factor;
  const double* q;
  double* axes; /* CellBound (query.rs:156-211) */
  best_t best;
  uint64_t n_visit, n_scan, n_box;
} descent_t;

static inline int admits_at(const descent_t* s, double dist, double bound) { /* query.rs:242-244 */
  return dist * s->eps_factor <= bound;
}

static inline double bdist(descent_t* s, uint32_t id) {
  s->n_box++;
  return box_dist(s->m, s->q, s->t->boxes + (size_t)id * 2 * s->t->ndim, s->t->ndim);
}

/* scan_leaf + Strategy::scan + LeafSink (query.rs:343-375, kernel.rs:366-562). */
static void scan_leaf(descent_t* s, size_t start, size_t end) {
  const size_t d = s->t->ndim;
  const size_t len = end - start;
  size_t chunk_pts = len; /* points inside full Packed chunks */
  if (s->strat == S_PACKED && s->m.kind != M_LINF) {
    if (d == 4) chunk_pts = len / 2 * 2;
    else if (d == 8) chunk_pts = len / 8 * 8;
  }
  double bound = best_bound(&s->best, s->cutoff);
  const double* rows = s->t->data + start * d;
  for (size_t j = 0; j < len; ++j) {
    double dist = point_dist(s->m, s->strat, s->q, rows + j * d, d, j < chunk_pts);
    if (dist <= bound) {
      best_consider(&s->best, dist, s->t->indices[start + j]);
      bound = best_bound(&s->best, s->cutoff);
    }
  }
  s->n_scan += len;
}

static void descend(descent_t* s, uint32_t node_id, double cell_dist);

/* enter_far (query.rs:329-341). */
static inline void enter_far(descent_t* s, uint32_t far, size_t dim, double far_axis, double far_dist) {
  double saved = s->axes[dim];
  s->axes[dim] = far_axis;
  descend(s, far, far_dist);
  s->axes[dim] = saved;
}

/* descend_by_box (query.rs:298-327). */
static void descend_by_box(descent_t* s, uint32_t near, uint32_t far, size_t dim, double cell_dist,
                           double far_axis, double far_dist) {
  double near_box = bdist(s, near);
  double far_box = bdist(s, far);
  if (near_box <= far_box) {
    if (admits_at(s, near_box, best_bound(&s->best, s->cutoff))) descend(s, near, cell_dist);
    if (admits_at(s, far_box, best_bound(&s->best, s->cutoff))) enter_far(s, far, dim, far_axis, far_dist);
  } else {
    if (admits_at(s, far_box, best_bound(&s->best, s->cutoff))) enter_far(s, far, dim, far_axis, far_dist);
    if (admits_at(s, near_box, best_bound(&s->best, s->cutoff))) descend(s, near, cell_dist);
  }
}

/* Descent::descend (query.rs:248-289). */
static void descend(descent_t* s, uint32_t node_id, double cell_dist) {
  s->n_visit++;
  const ork_node* n = s->t->nodes + node_id;
  if (n->is_leaf) {
    scan_leaf(s, n->a, n->b);
    return;
  }
  size_t dim = n->split_dim;
  double diff = s->q[dim] - n->split_value;
  uint32_t near, far;
  if (diff <= 0.0) {
    near = n->a;
    far = n->b;
  } else {
    near = n->b;
    far = n->a;
  }
  double far_axis = m_reduce(s->m, fabs(diff));
  double far_dist; /* replace_axis (metric.rs:93-98) */
  if (s->m.kind == M_LINF)
    far_dist = far_axis > cell_dist ? far_axis : cell_dist;
  else
    far_dist = cell_dist - s->axes[dim] + far_axis;
  if (n->order_by_box) {
    descend_by_box(s, near, far, dim, cell_dist, far_axis, far_dist);
    return;
  }
  descend(s, near, cell_dist);
  double bound = best_bound(&s->best, s->cutoff);
  if (admits_at(s, far_dist, bound)) {
    if (admits_at(s, bdist(s, far), bound)) enter_far(s, far, dim, far_axis, far_dist);
  }
}

/* Descent::run (query.rs:223-232) with CellBound::start/seed/finish
 * (query.rs:169-194) and write_results (query.rs:421-429, 483-493). */
static void run_one(descent_t* s, double* out_d, int64_t* out_i) {
  const ork_tree* t = s->t;
  const size_t d = t->ndim;
  s->best.len = 0;
  double seed = 0.0;
  if (bdist(s, 0) != 0.0) {
    const double* lo = t->boxes;
    const double* hi = t->boxes + d;
    for (size_t i = 0; i < d; ++i) {
      double axis = m_reduce(s->m, axis_offset(s->q[i], lo[i], hi[i]));
      s->axes[i] = axis;
      seed = (s->m.kind == M_LINF) ? (axis > seed ? axis : seed) : seed + axis;
    }
  }
  if (admits_at(s, seed, best_bound(&s->best, s->cutoff))) descend(s, 0, seed);
  for (size_t i = 0; i < d; ++i) s->axes[i] = 0.0;
  for (size_t j = 0; j < s->best.k; ++j) {
    if (j < s->best.len) {
      out_d[j] = m_restore(s->m, s->best.dists[j]);
      out_i[j] = (int64_t)s->best.ids[j];
    } else {
      out_d[j] = INFINITY;
      out_i[j] = (int64_t)t->n_points;
    }
  }
}

/* Tree::query (src/query.rs:29-78) plus run (query.rs:81-122).
 * `counts`, when non-NULL, receives {nodes visited, leaf rows scanned, boxes
 * evaluated} summed over all queries -- the per-query work figures the GPU
 * roofline divides by. */
int ork_query(const ork_tree* t, const double* queries, uint64_t n_values, uint64_t k, double p,
              int has_max_distance, double max_distance, double eps, int n_threads, double* out_d,
              int64_t* out_i, uint64_t* counts) {
  if (k == 0) return ORK_INVALID_K;
  if (n_values == 0 || n_values % t->ndim) return ORK_INVALID_SHAPE;
  for (uint64_t i = 0; i < n_values; ++i)
    if (!isfinite(queries[i])) return ORK_NONFINITE_DATA;
  if (!isfinite(eps) || eps < 0.0) return ORK_INVALID_EPS;
  if (!has_max_distance) max_distance = INFINITY;
  if (isnan(max_distance) || max_distance < 0.0) return ORK_INVALID_MAX_DISTANCE;
  metric_t m; /* Metric::new (metric.rs:45-59) */
  if (isinf(p) && p > 0) {
    m.kind = M_LINF;
  } else if (!isfinite(p) || p < 1.0) {
    return ORK_INVALID_METRIC;
  } else if (p == 1.0) {
    m.kind = M_L1;
  } else if (p == 2.0) {
    m.kind = M_L2;
  } else {
    m.kind = M_LP;
  }
  m.p = p;
  const size_t d = t->ndim;
  int strat; /* with_plan! (kernel.rs:244-270) */
  if (m.kind != M_LP && d <= 8)
    strat = S_PACKED;
  else if ((m.kind == M_L1 || m.kind == M_L2) && d <= 16)
    strat = S_FOLDED;
  else
    strat = S_STREAMED;
  const double cutoff = m_reduce(m, max_distance);
  const double eps_factor = m_reduce(m, 1.0 + eps);
  const uint64_t nq = n_values / d;
  uint64_t tv = 0, ts = 0, tb = 0;
  int status = ORK_OK;
  if (n_threads < 1) n_threads = 1;
#pragma omp parallel num_threads(n_threads) reduction(+ : tv, ts, tb)
  {
    descent_t s;
    s.t = t;
    s.m = m;
    s.strat = strat;
    s.cutoff = cutoff;
    s.eps_factor = eps_factor;
    s.axes = (double*)calloc(d, sizeof(double));
    s.best.k = k;
    s.best.len = 0;
    s.best.dists = (double*)malloc(k * sizeof(double));
    s.best.ids = (uint32_t*)malloc(k * sizeof(uint32_t));
    s.n_visit = s.n_scan = s.n_box = 0;
    if (!s.axes || !s.best.dists || !s.best.ids) {
#pragma omp atomic write
      status = ORK_OUT_OF_MEMORY;
    } else {
      /* rayon's with_min_len(16) (query.rs:26, 104-113) */
#pragma omp for schedule(dynamic, 16)
      for (uint64_t i = 0; i < nq; ++i) {
        s.q = queries + i * d;
        run_one(&s, out_d + i * k, out_i + i * k);
      }
    }
    tv += s.n_visit;
    ts += s.n_scan;
    tb += s.n_box;
    free(s.axes);
    free(s.best.dists);
    free(s.best.ids);
  }
  if (counts) {
    counts[0] = tv;
    counts[1] = ts;
    counts[2] = tb;
  }
  return status;
}

/* ------------------------------------------------------------------ */
/* Brute force: the exact top-k without the descent.                   */
/* ------------------------------------------------------------------ */

/* For each query, the k smallest (reduced distance, original index) over every
 * point within max_distance, each point's distance computed exactly as the
 * reference's leaf scan computes it at its tree position (point_dist with the
 * Packed d4/d8 chunk flag of its leaf, kernel.rs:441-457), kept by BestK's
 * order (query.rs:461-481).  This is what the reference's descent returns
 * when none of its FP64 gates -- the root seed (query.rs:169-194), the
 * split-plane bound (metric.rs:93-98) and the box distance (kernel.rs:565-616)
 * -- rounds above the distance of a point it would have kept.  The tests use it
 * to find inputs where one does (tests/golden/make_adversarial.py).  eps = 0
 * only; same arguments and outputs as ork_query. */
int ork_query_brute(const ork_tree* t, const double* queries, uint64_t n_values, uint64_t k, double p,
                    int has_max_distance, double max_distance, double* out_d, int64_t* out_i) {
  if (k == 0) return ORK_INVALID_K;
  if (n_values == 0 || n_values % t->ndim) return ORK_INVALID_SHAPE;
  if (!has_max_distance) max_distance = INFINITY;
  metric_t m;
  if (isinf(p) && p > 0) m.kind = M_LINF;
  else if (!isfinite(p) || p < 1.0) return ORK_INVALID_METRIC;
  else if (p == 1.0) m.kind = M_L1;
  else if (p == 2.0) m.kind = M_L2;
  else m.kind = M_LP;
  m.p = p;
  const size_t d = t->ndim;
  int strat;
  if (m.kind != M_LP && d <= 8) strat = S_PACKED;
  else if ((m.kind == M_L1 || m.kind == M_L2) && d <= 16) strat = S_FOLDED;
  else strat = S_STREAMED;
  const double cutoff = m_reduce(m, max_distance);
  /* the Packed chunk flag of every tree row, from its leaf */
  uint8_t* in_chunk = (uint8_t*)malloc(t->n_points ? t->n_points : 1);
  if (!in_chunk) return ORK_OUT_OF_MEMORY;
  for (uint64_t i = 0; i < t->n_nodes; ++i) {
    const ork_node* n = t->nodes + i;
    if (!n->is_leaf) continue;
    size_t len = n->b - n->a, chunk_pts = len;
    if (strat == S_PACKED && m.kind != M_LINF) {
      if (d == 4) chunk_pts = len / 2 * 2;
      else if (d == 8) chunk_pts = len / 8 * 8;
    }
    for (size_t j = 0; j < len; ++j) in_chunk[n->a + j] = j < chunk_pts;
  }
  const uint64_t nq = n_values / d;
  best_t b;
  b.k = k;
  b.dists = (double*)malloc(k * sizeof(double));
  b.ids = (uint32_t*)malloc(k * sizeof(uint32_t));
  if (!b.dists || !b.ids) {
    free(in_chunk);
    free(b.dists);
    free(b.ids);
    return ORK_OUT_OF_MEMORY;
  }
  for (uint64_t qi = 0; qi < nq; ++qi) {
    const double* q = queries + qi * d;
    b.len = 0;
    for (uint64_t r = 0; r < t->n_points; ++r) {
      double dist = point_dist(m, strat, q, t->data + r * d, d, in_chunk[r]);
      if (dist <= best_bound(&b, cutoff)) best_consider(&b, dist, t->indices[r]);
    }
    for (size_t j = 0; j < k; ++j) {
      if (j < b.len) {
        out_d[qi * k + j] = m_restore(m, b.dists[j]);
        out_i[qi * k + j] = (int64_t)b.ids[j];
      } else {
        out_d[qi * k + j] = INFINITY;
        out_i[qi * k + j] = (int64_t)t->n_points;
      }
    }
  }
  free(in_chunk);
  free(b.dists);
  free(b.ids);
  return ORK_OK;
}

/* ------------------------------------------------------------------ */
/* Accessors for the tests.                                            */
/* ------------------------------------------------------------------ */
void ork_info(const ork_tree* t, uint64_t* n_points, uint64_t* ndim, uint64_t* leafsize, uint64_t* n_nodes) {
  *n_points = t->n_points;
  *ndim = t->ndim;
  *leafsize = t->leafsize;
  *n_nodes = t->n_nodes;
}

/* Canonical export shared with the GPU library's kd_export: data in tree order,
 * indices, per-node {is_leaf, a, b, split_dim | order_by_box << 31}, split
 * values and boxes. */
void ork_export(const ork_tree* t, double* data, uint32_t* indices, uint32_t* node_words, double* split,
                double* boxes) {
  if (data) memcpy(data, t->data, t->n_points * t->ndim * sizeof(double));
  if (indices) memcpy(indices, t->indices, t->n_points * sizeof(uint32_t));
  for (uint64_t i = 0; i < t->n_nodes; ++i) {
    const ork_node* n = t->nodes + i;
    if (node_words) {
      node_words[4 * i + 0] = n->is_leaf;
      node_words[4 * i + 1] = n->a;
      node_words[4 * i + 2] = n->b;
      node_words[4 * i + 3] = n->split_dim | (n->order_by_box << 31);
    }
    if (split) split[i] = n->split_value;
  }
  if (boxes) memcpy(boxes, t->boxes, t->n_nodes * 2 * t->ndim * sizeof(double));
}

/* Tree::original_data (src/tree.rs:60-68). */
void ork_original_data(const ork_tree* t, double* out) {
  const size_t d = t->ndim;
  for (uint64_t pos = 0; pos < t->n_points; ++pos)
    memcpy(out + (size_t)t->indices[pos] * d, t->data + pos * d, d * sizeof(double));
}

int ork_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
