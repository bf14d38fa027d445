/*
 * kdtree_gb300.h -- C ABI of the GB300 kd-tree engine (libkdtree_gb300.so).
 *
 * This is the drop-in boundary for FujishigeTemma/kdtree-rs's hot path: the
 * median-split build and the pruned exact k-NN query.  Each entry point names
 * the reference interface it replaces.  Plain pointers and sizes only; no CUDA
 * or torch types (a CUDA stream is passed as `void*`).
 *
 * Conventions
 *  - Every function returning `int` returns a KD_* status; KD_OK is 0.  The
 *    message of the last failure on the calling thread is read with
 *    kd_last_error() and matches the reference's `KDTreeError` Display text
 *    (src/error.rs:18-51) for the statuses that mirror it.
 *  - Arrays are row-major.  A point set is `n_values = n_points * ndim`
 *    doubles, as the reference's `&[f64]` slices are (src/tree.rs:39-46,
 *    src/query.rs:29-37).
 *  - A tree is immutable once built; concurrent queries on one tree from many
 *    host threads are safe (each call owns its scratch and stream work),
 *    except kd_query_device_noalloc, whose calls share one fixed scratch
 *    array (see there).
 *  - `parallel` is accepted for API parity and has no effect: the GPU path
 *    computes the same result either way, as the reference's serial and rayon
 *    paths do (src/build.rs:345-359).
 */
#ifndef KDTREE_GB300_H
#define KDTREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  1..10 map 1:1 to the reference's KDTreeError variants
 * (src/error.rs:3-16); 11 is the boundary's DimensionMismatch; 100+ are
 * device-side failures the reference has no counterpart for. */
enum kd_status {
  KD_OK = 0,
  KD_ERR_EMPTY_DATA = 1,            /* KDTreeError::EmptyData */
  KD_ERR_INVALID_LEAFSIZE = 2,      /* KDTreeError::InvalidLeafsize */
  KD_ERR_INVALID_K = 3,             /* KDTreeError::InvalidK */
  KD_ERR_INVALID_METRIC = 4,        /* KDTreeError::InvalidMetric(p) */
  KD_ERR_INVALID_EPS = 5,           /* KDTreeError::InvalidEps(eps) */
  KD_ERR_INVALID_MAX_DISTANCE = 6,  /* KDTreeError::InvalidMaxDistance(d) */
  KD_ERR_NONFINITE_DATA = 7,        /* KDTreeError::NonFiniteData */
  KD_ERR_TOO_MANY_POINTS = 8,       /* KDTreeError::TooManyPoints(n) */
  KD_ERR_TOO_MANY_NODES = 9,        /* KDTreeError::TooManyNodes(n) */
  KD_ERR_INVALID_SHAPE = 10,        /* KDTreeError::InvalidShape(msg) */
  KD_ERR_DIMENSION_MISMATCH = 11,   /* KDTreeError::DimensionMismatch */
  KD_ERR_CUDA = 100,                /* a CUDA runtime call failed */
  KD_ERR_OUT_OF_MEMORY = 101,       /* device or host allocation failed */
  KD_ERR_INVALID_ARGUMENT = 102,    /* NULL pointer or unusable argument */
  KD_ERR_NO_DEVICE = 103            /* no CUDA device is visible */
};

typedef struct kd_tree kd_tree;

/* Build a tree from host data.  Replaces `Tree::new(data, ndim, leafsize,
 * parallel)` (src/tree.rs:39-46 -> src/build.rs:19-82): the same validation
 * order, and a layout (row order, indices, nodes, boxes) bit-identical to the
 * reference's.  The data is copied; the caller keeps ownership of `data`. */
int kd_build(const double* data, uint64_t n_values, uint64_t ndim, uint64_t leafsize,
             int parallel, kd_tree** out);

/* Same as kd_build with `d_data` already in device memory (it is read, not
 * modified), the build work ordered on `stream` (NULL = the legacy default
 * stream).  Returns once the tree is complete. */
int kd_build_device(const double* d_data, uint64_t n_values, uint64_t ndim, uint64_t leafsize,
                    void* stream, kd_tree** out);

/* Release a tree and its device memory.  NULL is ignored. */
void kd_free(kd_tree* tree);

/* Exact k-NN query from host buffers.  Replaces `Tree::query(queries, k, p,
 * max_distance, eps, parallel)` (src/query.rs:29-78): same validation order
 * and messages, same (distance, index) results and tie order.  `out_distances`
 * and `out_indices` hold n_queries * k values; slots without a neighbour are
 * (+inf, n_points).  `has_max_distance` = 0 is the reference's `None`. */
int kd_query(const kd_tree* tree, const double* queries, uint64_t n_values, uint64_t k, double p,
             int has_max_distance, double max_distance, double eps, int parallel,
             double* out_distances, int64_t* out_indices);

/* Same as kd_query with queries and outputs in device memory, the work ordered
 * on `stream`.  Returns after the stream work of this call has finished (the
 * finiteness check of the queries is read back before returning). */
int kd_query_device(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k,
                    double p, int has_max_distance, double max_distance, double eps,
                    double* d_out_distances, int64_t* d_out_indices, void* stream);

/* kd_query_device without any host wait, for callers that pipeline uploads,
 * queries and downloads on their own streams (a framework binding, a serving
 * loop).  No reference counterpart beyond `Tree::query` (src/query.rs:29-78),
 * whose pyo3 wrapper releases the GIL around it (src/lib.rs:176-177): this is
 * that seam made stream-ordered.
 *
 * Every device step of the call is ordered on `stream` and the call returns
 * once they are enqueued.  `d_status` is a device u32 the call first clears
 * (stream-ordered) and the kernels then set: bit 0 a non-finite query (the
 * reference's NonFiniteData), bit 1 a tensor-core pipeline wait that ran out
 * (KD_ERR_CUDA); read it after the stream work, e.g. with the results.
 * The return value covers what the host can check: shape, k, NULL buffers,
 * and the scalar arguments (p, max_distance, eps, with the reference's
 * messages).  For a scalar error the finiteness check still runs into bit 0 of
 * *d_status, and the reference reports that error first.  Scratch comes from
 * the library's stream-ordered pool.  Two one-time set-ups stay asynchronous
 * too: a tree's first tensor-core query enqueues its BF16 copy (other streams
 * wait for it on the device), and at ndim = 16 a call that finds no timed
 * choice between the two exact paths takes the warp traversal instead of
 * timing both. */
int kd_query_async(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k, double p,
                   int has_max_distance, double max_distance, double eps, double* d_out_distances,
                   int64_t* d_out_indices, uint32_t* d_status, void* stream);

/* Query kernels kd_query_device_path can be asked for.  No reference
 * counterpart: the reference has one CPU descent; these are the engine's
 * implementations of it, for measurement and cross-checking.
 *   KD_PATH_AUTO            what kd_query / kd_query_device run: a rule per
 *                           width, k and batch size, timed on the tree where
 *                           the packet and warp traversals are close (widths 2
 *                           and 3, 32,768 to 524,287 queries: the first such
 *                           call of a class runs both and keeps the faster)
 *   KD_PATH_REFERENCE_ORDER the reference's depth-first order with its FP64
 *                           gate decisions (the only order for eps > 0 and
 *                           general p): one warp per query, leaf rows split
 *                           across the lanes (d <= 128, k <= 64), one thread
 *                           per query otherwise
 *   KD_PATH_PACKET          warp-shared traversal (d in {2, 3, 8, 16}, eps = 0, k <= 64)
 *   KD_PATH_TENSOR_CORE     tcgen05 BF16 distance filter + FP64 re-rank
 *                           (L2, eps = 0, 16 <= d <= 128, k <= 32)
 *   KD_PATH_WARP            one warp per query, best-first, rows and
 *                           dimensions split across the lanes (d <= 128,
 *                           eps = 0, k <= 64): for queries that scan many rows
 * The eps = 0 paths other than the reference order compute the exact top-k
 * and run again, in the reference's order, the queries where a near tie lets
 * the reference's own descent leave a point out, so every path returns the
 * reference's answer.  A path that does not apply to a call falls back to the
 * reference order. */
enum kd_query_path {
  KD_PATH_AUTO = 0,
  KD_PATH_REFERENCE_ORDER = 1,
  KD_PATH_PACKET = 2,
  KD_PATH_TENSOR_CORE = 3,
  KD_PATH_WARP = 4
};

/* kd_query_device with the kernel chosen by `path` (see kd_query_path).
 * `d_counters`, when not NULL, points to three device counters the call adds
 * to: [0] the (query, point) pairs the tensor-core filter could not reject,
 * [1] the queries an eps = 0 path flagged as near ties, [2] those of them
 * whose results a test of the reference's gates along the paths to the
 * result points could not confirm, run again in the reference's order. */
int kd_query_device_path(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k,
                         double p, int has_max_distance, double max_distance, double eps,
                         double* d_out_distances, int64_t* d_out_indices, void* stream, int path,
                         unsigned long long* d_counters);

/* Largest n_values (n_queries * ndim) one kd_query_device_noalloc call takes. */
#define KD_NOALLOC_MAX_VALUES 524256ull

/* kd_query_device for callers that cannot allocate device memory.  This entry
 * point has no counterpart in the reference; it exists for callers such as
 * frameworks that reserve almost all device memory for their own pool (where an
 * allocation from this library fails or fragments that pool) and latency-bound
 * request loops that keep allocation out of their serving path.
 *
 * Same arguments, validation, results and synchronous return as
 * kd_query_device, but no allocation of any kind: the per-call status word and
 * the per-query CellBound scratch live in one fixed 4 MiB device array that is
 * part of the library (every GPU that loads the library holds it until the
 * process exits).  Hence:
 *  - n_values must not exceed KD_NOALLOC_MAX_VALUES; larger calls fail with
 *    KD_ERR_INVALID_ARGUMENT and a message, before any device work;
 *  - every call on a device uses the same array, which keeps the last call's
 *    contents (each call clears what must start at zero): calls whose work
 *    overlaps on the GPU race, so issue them from one stream or serialise them;
 *  - the array's device address is looked up once per device, with that
 *    device current, at the end of the first kd_build / kd_build_device on it
 *    (which allocates anyway).  That lookup is also when the CUDA runtime
 *    places the array in device memory if it loads modules lazily (the
 *    default).  Should that set-up have failed, the first call on the device
 *    repeats it (and may then allocate the array); make that first call before
 *    any stream capture;
 *  - it never runs the tensor-core filter that kd_query_device takes for L2
 *    at 16 <= ndim <= 128: the CUDA-core traversals it runs instead give the
 *    same results. */
int kd_query_device_noalloc(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k,
                            double p, int has_max_distance, double max_distance, double eps,
                            double* d_out_distances, int64_t* d_out_indices, void* stream);

/* ---- Batched queries over many trees -------------------------------------
 * No reference counterpart: the reference answers one `Tree::query` call at a
 * time (src/query.rs:29-78); a batch is its caller's loop over many trees,
 * fused into one pass on the device.  Each job's results are exactly those of
 * kd_query_device on the same job. */

/* One job: a tree, its queries and its outputs, all in device memory with the
 * layout of kd_query_device (n_queries * ndim values in, n_queries * k out). */
typedef struct kd_batch_job {
  const kd_tree* tree;
  const double* d_queries;
  uint64_t n_queries;
  uint64_t k;
  double* d_out_distances;
  int64_t* d_out_indices;
} kd_batch_job;

typedef struct kd_batch kd_batch;

/* Plan a fixed set of jobs: trees, sizes, k and buffer addresses are recorded
 * (the buffers must stay valid while the plan is used; their contents may
 * change between runs).  p, max_distance and eps apply to every job and are
 * validated as kd_query validates them; each job as a kd_query_device call
 * (k > 0, n_queries > 0, buffers not NULL); every tree must live on the current
 * device.  Device scratch for the plan is allocated here. */
int kd_batch_create(const kd_batch_job* jobs, uint64_t n_jobs, double p, int has_max_distance,
                    double max_distance, double eps, kd_batch** out);

/* How kd_batch_run_mode executes a plan. */
enum kd_batch_mode {
  KD_BATCH_GRAPH = 0,   /* one CUDA graph: the sort and ONE persistent kernel launch
                           for every job the packet traversal serves (what
                           kd_batch_run does); the first run tunes the launch */
  KD_BATCH_FUSED = 1,   /* the same launches issued one by one (no graph) */
  KD_BATCH_PER_JOB = 2  /* one kd_query_device-style launch sequence per job */
};

/* Run every job of the plan on `stream` and return once the work has finished
 * (a non-finite query in any job: KD_ERR_NONFINITE_DATA after all jobs ran). */
int kd_batch_run(kd_batch* batch, void* stream);

/* What the first graph run's autotuner chose (before it: the defaults):
 * the persistent grid in CTAs, whether queries are sorted by landing leaf,
 * and the widths whose jobs with k <= 4 run as packet tasks (bit 0: width 2,
 * bit 1: 3, bit 2: 8) instead of one query a warp.  Any pointer may be NULL.
 * The environment variable KD_BATCH_PACKET=all (or none), read when a plan is
 * tuned, fixes the packet-task choice instead of timing it; results do not
 * depend on it. */
int kd_batch_choice(const kd_batch* batch, unsigned* blocks, int* sorted, unsigned* packet_widths);
int kd_batch_run_mode(kd_batch* batch, void* stream, int mode);

/* Release a plan (NULL is ignored). */
void kd_batch_free(kd_batch* batch);

/* ---- Serving: continuous batching over a fixed set of trees --------------
 * No reference counterpart: a request loop in front of `Tree::query`
 * (src/query.rs:29-78).  At creation the server times each tree once (up to
 * 32,768 of its own points as queries) for an estimate of its GPU time per
 * query.  A request runs as pieces of about 4 ms of that estimated time
 * (4,096 to 16,384 queries, fewer for large k).  A scheduler thread forms a
 * batch whenever one of two batch slots is free: every waiting single-piece
 * request that fits the slot, in arrival order, then pieces of larger
 * requests while the batch's estimated time stays within about 5 ms (one
 * piece at least when no small request waits, or when a piece has waited
 * 20 ms), so a small request waits for a few milliseconds of other work, not
 * a large request's whole scan.
 * A batch runs the kernels of kd_batch_run (plus per-request launches for
 * requests outside the fused kernel).  A request's results are exactly
 * kd_query's for the same tree and queries, whatever it is batched with. */
typedef struct kd_server kd_server;

/* Start a server over n_trees trees (all on the current device); p,
 * max_distance and eps apply to every request and are validated as kd_query
 * validates them.  max_batch_queries caps the queries of one batch (0: sized
 * from free device memory, at most 2^20); the two slots' staging (queries, 64
 * results per query on average) is allocated here. */
int kd_server_create(const kd_tree* const* trees, uint64_t n_trees, double p, int has_max_distance,
                     double max_distance, double eps, uint64_t max_batch_queries, kd_server** out);

/* Queue a request for tree index `tree`: n_queries rows in HOST memory, k
 * results each into host out_distances / out_indices (n_queries * k).  The
 * three buffers must stay valid until kd_server_wait returns for the ticket.
 * Validated as kd_query validates a call (k > 0, n_queries > 0); a k whose
 * results for even one query do not fit a batch fails with
 * KD_ERR_INVALID_ARGUMENT.  Returns at once; the latency kd_server_wait
 * reports runs to the completion of the request's last piece. */
int kd_server_submit(kd_server* server, uint64_t tree, const double* queries, uint64_t n_queries, uint64_t k,
                     double* out_distances, int64_t* out_indices, uint64_t* ticket);

/* Wait for a request; returns its status (KD_ERR_NONFINITE_DATA for a
 * non-finite query) and, when latency_s is not NULL, the seconds from its
 * submission to the completion of its batch.  Each ticket is waited for once. */
int kd_server_wait(kd_server* server, uint64_t ticket, double* latency_s);

/* Finish every queued request, stop the threads, release everything.  No
 * other thread may be inside kd_server_submit / kd_server_wait on this server
 * when it is called; tickets not yet waited for are dropped. */
void kd_server_free(kd_server* server);

/* Device time in milliseconds of the last query kernel this thread launched
 * (the traversal or the tensor-core filter; the sort and set-up kernels
 * around it excluded), from CUDA events recorded on its stream; -1 when there
 * is none.  No reference counterpart: a measurement aid. */
double kd_last_query_kernel_ms(void);

/* Getters: `Tree::ndim`, `Tree::n_points`, `Tree::leafsize`
 * (src/tree.rs:48-58).  kd_n_nodes has no Python getter in the reference. */
uint64_t kd_ndim(const kd_tree* tree);
uint64_t kd_n_points(const kd_tree* tree);
uint64_t kd_leafsize(const kd_tree* tree);
uint64_t kd_n_nodes(const kd_tree* tree);

/* Copy the points back in the caller's original row order into host memory
 * (n_points * ndim doubles).  Replaces `Tree::original_data`
 * (src/tree.rs:60-68). */
int kd_original_data(const kd_tree* tree, double* out);

/* Export the tree layout into host memory for inspection and parity tests
 * (any pointer may be NULL to skip that array).  Mirrors the reference's
 * `Tree` fields (src/tree.rs:29-36):
 *   data       n_points * ndim doubles, tree (leaf-contiguous) row order
 *   indices    n_points u32, tree position -> original row
 *   node_words n_nodes * 4 u32: {is_leaf, left|start, right|end,
 *              split_dim | order_by_box << 31}
 *   split      n_nodes doubles (split_value; 0 for leaves)
 *   boxes      n_nodes * 2 * ndim doubles, [lo | hi] per node. */
int kd_export(const kd_tree* tree, double* data, uint32_t* indices, uint32_t* node_words,
              double* split, double* boxes);

/* Copy the calling thread's last error message (NUL-terminated, truncated to
 * `len`) and return its full length.  The Rust reference surfaces the same
 * text through `KDTreeError`'s Display (src/error.rs:18-51). */
size_t kd_last_error(char* buf, size_t len);

/* Page-locked host memory for result arrays (no reference counterpart: the
 * reference's pyo3 layer returns fresh numpy arrays, src/lib.rs:86-98).
 * kd_query writes each result row straight from the kernel into page-locked
 * outputs (no download phase), while a freshly allocated pageable array first
 * takes a page fault per page.  Blocks are pooled: kd_host_free keeps up to
 * 4 GiB of freed blocks for later kd_host_alloc calls of about the same size;
 * NULL and pointers this pool did not hand out are ignored. */
int kd_host_alloc(uint64_t bytes, void** out);
void kd_host_free(void* p);

/* Number of nodes `count_nodes(n_points, leafsize)` (src/build.rs:166-173)
 * a tree of this size has; lets callers size kd_export buffers up front. */
uint64_t kd_count_nodes(uint64_t n_points, uint64_t leafsize);

#ifdef __cplusplus
}
#endif

#endif /* KDTREE_GB300_H */
