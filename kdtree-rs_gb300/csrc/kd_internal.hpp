// kd_internal.hpp -- host-side definitions shared by the C-ABI, the build and the
// query translation units of libkdtree_gb300.so.
#pragma once

#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "kd_common.cuh"

// The tree object behind the opaque `kd_tree*` of the C ABI.  Everything the
// query touches lives in device memory; the host keeps only the sizes.
struct kd_tree {
  uint64_t n_points = 0;
  uint64_t ndim = 0;
  uint64_t leafsize = 0;
  uint64_t n_nodes = 0;
  int device = 0;
  // One block from the library's device pool holds the arrays below up to
  // data32w; the tensor-core arrays are separate allocations.
  void* block = nullptr;
  double* data = nullptr;       // n_points * ndim, tree (leaf-contiguous) order
  uint32_t* indices = nullptr;  // tree position -> original row
  uint32_t* rows_of = nullptr;  // original row -> tree position
  kd::DNode* nodes = nullptr;   // n_nodes, preorder
  double* boxes = nullptr;      // n_nodes * 2 * ndim, [lo | hi] per node
  float* data32 = nullptr;      // n_points * ndim, round-to-nearest FP32 copy (filters)
  float* boxes32 = nullptr;     // n_nodes * 2 * ndim, [lo rounded down | hi rounded up]
  float coord_max32 = 0.f;      // FP32 upper bound of every |coordinate| (the root box)
  // FP32 rows padded to w32 = ndim rounded up to a multiple of 4 floats, for
  // width 3 and the runtime-width warp kernels (made by the build; data32
  // itself when ndim is a multiple of 4 or another compile-time width).
  float* data32w = nullptr;
  uint32_t w32 = 0;
  // Tensor-core filter inputs, made on first use (guarded by tc_mutex):
  // centred BF16 rows padded to tc_dpad, and the per-point filter terms.
  std::mutex tc_mutex;
  uint16_t* tc_points = nullptr;  // n_points x tc_dpad BF16 of (p - centre)
  float* tc_w = nullptr;          // per point: |p_b|^2 (1 - 2^-12) - v^2, rounded down
  float* tc_v = nullptr;          // per point: 2^-8 |p_b|, rounded up
  double* tc_centre = nullptr;    // ndim, the root box centre
  float* tc_tbox = nullptr;       // per 256-point tile: [lo | hi] FP32 enclosure (ndim each)
  uint32_t tc_dpad = 0;
  cudaEvent_t tc_ready = nullptr;  // recorded after the kernels that fill them; later users wait on it
  // Width 16: which exact path the automatic choice measured faster on this
  // tree, per batch-size class (index 0: batches below AUTO_LARGE_BATCH
  // queries, 1: at or above it); -1 not yet measured, 0 warp-per-query
  // traversal, 1 tensor-core filter.
  std::mutex choice_mutex;
  int auto_choice[2] = {-1, -1};
  // Widths 2 and 3, eps = 0, batches of TRAVERSAL_TIMED_MIN up to
  // TRAVERSAL_TIMED_MAX queries: which traversal the automatic choice
  // measured faster on this tree, per class (bit 1: k > 16, bit 0: at least
  // TRAVERSAL_TIMED_SPLIT queries); -1 not yet measured, 0 one warp a query,
  // 1 packet traversal.
  int auto_traversal[4] = {-1, -1, -1, -1};
};

namespace kd {

// Widths the warp kernels take: compile-time kernels for 1, 2, 3, 4, 8 and 16,
// the runtime-width kernel (padded FP32 rows) for the others up to 128.
constexpr uint64_t WARP_MAX_WIDTH = 128;
inline bool warp_static_width(uint64_t d) { return d == 1 || d == 2 || d == 3 || d == 4 || d == 8 || d == 16; }
inline bool warp_runtime_width(uint64_t d) { return d >= 1 && d <= WARP_MAX_WIDTH && !warp_static_width(d); }
// Widths whose filters read the FP32 rows padded to w32 floats: the runtime
// widths, and 3 (one 16-byte load a row instead of three 4-byte ones).
inline bool padded_rows(uint64_t d) { return d == 3 || warp_runtime_width(d); }

// Launch arguments of the query kernels (every query translation unit).
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
  float coord_max;        // >= every |coordinate| of the tree, FP32
  const double* queries;  // nq * d
  double* out_d;          // nq * k
  int64_t* out_i;         // nq * k
  double* axes_scratch;   // nq * d, dynamic-d CellBound (unused for static d)
  uint32_t* status;       // bit 0: non-finite query
  const uint32_t* order;  // optional: thread t runs query order[t] (spatially sorted)
  const uint32_t* leaf_of;  // optional: landing leaf node of each query (by query index)
  const float* data32w;   // FP32 rows padded to w32 floats (width 3 and the runtime widths)
  uint32_t w32;
  // Near ties (eps = 0 kernels outside the reference's visiting order): the
  // query gets (rerun_tag << 32 | query index) appended to rerun_list; NULL
  // rerun_count: no tracking.
  uint32_t* rerun_count;
  uint64_t* rerun_list;
  uint32_t rerun_tag;
  // optional (measurement): rerun_total[0] gets the flagged queries,
  // rerun_total[1] those the path test could not confirm (run again)
  unsigned long long* rerun_total;
  const uint32_t* rows_of;  // original index -> tree row (inverse of indices)
  bool reference_order;   // run the reference-order descent even where eps = 0
  uint64_t nq;
  uint64_t d;
  uint64_t k;
  uint64_t n_points;
  double p;               // LP exponent
  double cutoff;          // reduced max_distance, >= +0
  double eps_factor;
  int use_eps;            // eps_factor != 1
};

// Thread-local last-error text (read through kd_last_error).
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t err, const char* what);

// Stream-ordered device allocation from the library's own memory pool on the
// current device.  The pool keeps up to KD_POOL_KEEP_BYTES of freed blocks for
// later calls, so a steady query loop maps no new memory; freed with
// cudaFreeAsync.
constexpr uint64_t KD_POOL_KEEP_BYTES = 1ull << 30;
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t st);

#define KD_TRY_CUDA(call)                                   \
  do {                                                      \
    cudaError_t kd_err_ = (call);                           \
    if (kd_err_ != cudaSuccess) return ::kd::cuda_fail(kd_err_, #call); \
  } while (0)

uint64_t count_nodes(uint64_t len, uint64_t leafsize);

// Build the tree from device data (already validated for shape and size).
// Returns a KD_* status; on success fills t's device buffers.
int build_on_device(const double* d_src, uint64_t n_points, uint64_t ndim, uint64_t leafsize,
                    cudaStream_t stream, kd_tree* t);

// Parameters of one query call after validation (src/query.rs:38-62).
// Which query kernel runs (kd_query_device_path): the automatic choice, the
// reference-order descent, the packet traversal, or the tensor-core filter.
enum QueryPath : int { PATH_AUTO = 0, PATH_REFERENCE_ORDER = 1, PATH_PACKET = 2, PATH_TENSOR_CORE = 3, PATH_WARP = 4 };

struct QueryParams {
  int path = PATH_AUTO;
  bool no_sync = false;  // stream-ordered call (kd_query_async): no host waits, no timing on first use
  int metric;         // MetricKind
  double p;           // exponent (LP only)
  double cutoff;      // reduce(max_distance), -0 normalised to +0
  double eps_factor;  // reduce(1 + eps)
  uint64_t k;
};

// Scalar validation of Tree::query (query.rs:49-62, metric.rs:45-59): KD_OK
// and qp filled, or the status with its message in *msg.
int validate_scalars(uint64_t k, double p, int has_max, double max_distance, double eps, QueryParams* qp,
                     std::string* msg);

// Resolve the device address of kd_query_device_noalloc's fixed scratch array
// on device `dev` (current), which loads the module holding it.  Called at the
// end of every tree build, whose allocations this one-time set-up joins, so a
// later kd_query_device_noalloc call on that device allocates nothing even
// when CUDA loads modules lazily.  Best effort: a failure here is retried (and
// reported) by the first kd_query_device_noalloc call.
void noalloc_prepare(int dev);

// Sets bit 0 of *status when any of the n values is not finite.
__global__ void k_check_finite(const double* v, uint64_t n, uint32_t* status);

// The launch arguments of a query on tree t: no order, no scratch, no rerun list.
QArgs query_args(const kd_tree* t, const double* d_queries, uint64_t n_queries, const QueryParams& qp,
                 double* d_out_d, int64_t* d_out_i, uint32_t* d_status);

// Run the query on device buffers; `d_status` is a device word the kernels set
// when a query is non-finite.  Work is ordered on `stream`.
int query_on_device(const kd_tree* t, const double* d_queries, uint64_t n_queries,
                    const QueryParams& qp, double* d_out_d, int64_t* d_out_i,
                    cudaStream_t stream, uint32_t* d_status, unsigned long long* d_survivors = nullptr);

// Same as query_on_device with the scratch supplied by the caller; allocates
// nothing and does not sort the batch.  `d_scratch` serves (one at a time)
// as the dynamic-width CellBound scratch of the one-thread reference-order
// kernels (n_queries * ndim doubles) or as the near-tie rerun list of the
// eps = 0 fast paths (n_queries u64); `d_rerun_count` is one u32.
int query_on_device_scratch(const kd_tree* t, const double* d_queries, uint64_t n_queries,
                            const QueryParams& qp, double* d_out_d, int64_t* d_out_i,
                            cudaStream_t stream, uint32_t* d_status, void* d_scratch, uint32_t* d_rerun_count);

// Bytes query_on_device_scratch's d_scratch must hold for n_queries of width ndim.
uint64_t query_scratch_bytes(uint64_t n_queries, uint64_t ndim);

// Whether the query kernels that query_on_device would run for these
// parameters write each query's result row as whole contiguous segments (so
// results may go straight to page-locked host memory over the host link).
bool writes_whole_rows(const kd_tree* t, const QueryParams& qp);

// Sort a batch by landing leaf (the leaf each query's descent reaches first):
// leaf_of[i] = that leaf's node id, order = query indices grouped by leaf in
// preorder.  `scratch` holds order_scratch_words(t) u32.  Work on `stream`.
uint64_t order_scratch_words(const kd_tree* t);
void order_by_landing_leaf(const kd_tree* t, const double* d_queries, uint64_t nq, uint32_t* leaf_of,
                           uint32_t* order, uint32_t* scratch, cudaStream_t stream);

// The packet traversal (warp-shared descent, eps = 0, k <= 64, L1 / L2 /
// L-inf, widths 2, 3, 8, 16): whether it covers a query, and its launch.
bool packet_applicable(uint64_t d, int metric, uint64_t k, uint64_t n_points, bool use_eps);
int launch_packet_query(const QArgs& a, int metric, cudaStream_t stream);
// One warp per query, best-first (eps = 0, L1 / L2 / L-inf, widths up to
// 128, k <= 64): for queries that scan many leaf rows, and every width the
// packet traversal lacks.  Flags near ties when a.rerun_count is set.
bool warp_applicable(uint64_t d, int metric, uint64_t k, uint64_t n_points, bool use_eps);
int launch_warp_query(const QArgs& a, int metric, cudaStream_t stream);

// The reference's own descent with one warp per query (any eps, every
// metric, widths up to 128, k <= 64): a.nq queries (a.order when set), or the
// `count` queries of `list` (a near-tie rerun; low 32 bits of each entry: the
// query index).
bool ref_warp_applicable(uint64_t d, uint64_t k, uint64_t n_points);
int launch_ref_query(const QArgs& a, int metric, cudaStream_t stream);
int launch_rerun(const QArgs& a, int metric, cudaStream_t stream, const uint32_t* count, const uint64_t* list);

// Exact k-NN through the tensor-core filter (L2, eps = 0, 16 <= d <= 128,
// k <= 32).  Returns KD_OK, or KD_ERR_INVALID_ARGUMENT without doing anything
// when the case is outside that envelope.  `d_survivors`, if not NULL,
// accumulates the number of (query, point) pairs the filter could not reject.
int query_tc_on_device(kd_tree* t, const double* d_queries, uint64_t n_queries, const QueryParams& qp,
                       double* d_out_d, int64_t* d_out_i, cudaStream_t stream, uint32_t* d_status,
                       unsigned long long* d_survivors);
bool tc_applicable(const kd_tree* t, const QueryParams& qp);

}  // namespace kd
