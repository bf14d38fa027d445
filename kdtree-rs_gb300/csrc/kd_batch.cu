// kd_batch.cu -- many (tree, query batch) jobs in one pass on the device.
//
// No reference counterpart: the reference answers one Tree::query call at a
// time (src/query.rs:29-78); a batch is its caller's loop over many trees,
// fused.  Running a plan:
//  1. one kernel walks every query of every packet job down its own tree to
//     its landing leaf and counts it into bin (job, leaf); one scan over all
//     bins and one scatter leave each job's queries grouped by landing leaf,
//     jobs one after another in the batch order;
//  2. ONE persistent kernel: each warp takes the next task -- 32 consecutive
//     positions of one job's sorted queries -- from a global counter and runs
//     the packet traversal (kd_query_packet.cuh) for that job's width and k.
//     Jobs are laid out most expensive class first, so the long tasks start
//     early and the short ones fill the tail;
//  3. jobs outside the packet traversal's envelope (general L^p, eps > 0,
//     k > 32, widths other than 2, 3 and 8, the reference-order switch) run as
//     ordinary per-job launches of the same kernels kd_query_device uses,
//     without the tensor-core filter (its set-up allocates and synchronises).
// A query's result depends on that query and its tree alone, so every job
// gets exactly what kd_query_device returns for it.
//
// The first graph run of a plan times a few launch shapes -- persistent grid
// size and whether to sort -- and keeps the fastest (the autotuner), then
// captures the whole sequence in a CUDA graph; later runs replay the graph.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "kd_internal.hpp"

namespace kd {
namespace {

#include "kd_query_common.cuh"
#include "kd_scan.cuh"
#include "kd_lazy_best.cuh"
#include "kd_query_packet.cuh"

constexpr uint32_t CLS_OTHER = 0xffffffffu;
constexpr int BATCH_K[5] = {1, 4, 8, 16, 32};

// Packet class of a job: width index * 5 + k index, or CLS_OTHER.
uint32_t packet_class(const kd_tree* t, const QueryParams& qp, bool reference_order) {
  if (qp.metric == M_LP || qp.eps_factor != 1.0 || qp.k > 32 || t->n_points >= ROW_NONE || reference_order)
    return CLS_OTHER;
  int di;
  switch (t->ndim) {
    case 2: di = 0; break;
    case 3: di = 1; break;
    case 8: di = 2; break;
    default: return CLS_OTHER;
  }
  int ki = 0;
  while (BATCH_K[ki] < static_cast<int>(qp.k)) ++ki;
  return static_cast<uint32_t>(di * 5 + ki);
}

struct BatchJob {
  QArgs a;             // the job's query arguments; a.order points into the batch order
  uint64_t bin_start;  // the job's first landing-leaf bin
  uint32_t cls;        // packet class or CLS_OTHER
  uint32_t pad;
};

struct BatchArgs {
  const BatchJob* jobs;
  const uint32_t* task_start;  // n_jobs + 1: first 32-query task of each job
  uint32_t n_jobs;
  uint32_t n_tasks;
  uint32_t* next_task;
};

// Largest j < n with start[j] <= x, for non-decreasing start[0..n] with
// start[0] = 0 <= x < start[n]: the job whose range [start[j], start[j+1])
// holds x (empty ranges are skipped).
__device__ __forceinline__ uint32_t find_range(const uint32_t* start, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void k_batch_landing(const BatchJob* jobs, const uint32_t* q_start, uint32_t n_jobs, uint32_t total,
                                uint64_t* bin_of, uint32_t* bins) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint32_t j = find_range(q_start, n_jobs, g);
  const BatchJob& J = jobs[j];
  const uint32_t i = g - q_start[j];
  uint32_t node = 0;
  if (J.cls != CLS_OTHER) {
    const double* q = J.a.queries + static_cast<uint64_t>(i) * J.a.d;
    for (;;) {
      const DNode nd = J.a.nodes[node];
      if (nd.meta & KD_NODE_LEAF) break;
      node = (q[nd.meta & KD_NODE_DIM_MASK] <= nd.split) ? node + 1 : nd.right;
    }
  }
  const uint64_t bin = J.bin_start + node;
  bin_of[g] = bin;
  atomicAdd(&bins[bin], 1u);
}

// bins holds the exclusive scan of the counts: global batch positions.
__global__ void k_batch_scatter(const uint32_t* q_start, uint32_t n_jobs, uint32_t total, const uint64_t* bin_of,
                                uint32_t* bins, uint32_t* order) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const uint32_t j = find_range(q_start, n_jobs, g);
  order[atomicAdd(&bins[bin_of[g]], 1u)] = g - q_start[j];
}

template <int M, int D, int K>
__device__ __noinline__ void batch_task(const QArgs* a, uint64_t tid, float* lo, float* hi, uint32_t* row) {
  packet_queries<M, D, K>(*a, tid, lo, hi, row);
}

template <int M, int D, int KMAX>
__device__ __forceinline__ void run_k(uint32_t ki, const QArgs* a, uint64_t tid, float* lo, float* hi,
                                      uint32_t* row) {
  switch (ki) {
    case 0: batch_task<M, D, 1>(a, tid, lo, hi, row); break;
    case 1: if constexpr (KMAX >= 4) batch_task<M, D, 4>(a, tid, lo, hi, row); break;
    case 2: if constexpr (KMAX >= 8) batch_task<M, D, 8>(a, tid, lo, hi, row); break;
    case 3: if constexpr (KMAX >= 16) batch_task<M, D, 16>(a, tid, lo, hi, row); break;
    default: if constexpr (KMAX >= 32) batch_task<M, D, 32>(a, tid, lo, hi, row); break;
  }
}

// The persistent kernel: warps take 32-query tasks until none is left.
template <int M, int KMAX>
__global__ void __launch_bounds__(QUERY_THREADS) k_query_batch(BatchArgs b) {
  __shared__ PacketSmem<KMAX> sm;
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(b.next_task, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= b.n_tasks) return;
    const uint32_t j = find_range(b.task_start, b.n_jobs, t);
    const BatchJob* J = b.jobs + j;
    const uint32_t cls = J->cls;
    const uint64_t tid = static_cast<uint64_t>(t - b.task_start[j]) * 32 + lane;
    switch (cls / 5) {
      case 0: run_k<M, 2, KMAX>(cls % 5, &J->a, tid, sm.lo, sm.hi, sm.row); break;
      case 1: run_k<M, 3, KMAX>(cls % 5, &J->a, tid, sm.lo, sm.hi, sm.row); break;
      default: run_k<M, 8, KMAX>(cls % 5, &J->a, tid, sm.lo, sm.hi, sm.row); break;
    }
  }
}

template <int M, int KMAX>
cudaError_t launch_batch(const BatchArgs& b, unsigned blocks, cudaStream_t st) {
  k_query_batch<M, KMAX><<<blocks, QUERY_THREADS, 0, st>>>(b);
  return cudaGetLastError();
}

template <int M>
cudaError_t launch_batch_k(const BatchArgs& b, int kmax, unsigned blocks, cudaStream_t st) {
  if (kmax <= 4) return launch_batch<M, 4>(b, blocks, st);
  if (kmax <= 16) return launch_batch<M, 16>(b, blocks, st);
  return launch_batch<M, 32>(b, blocks, st);
}

template <int M, int KMAX>
int max_blocks_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_query_batch<M, KMAX>, QUERY_THREADS, 0);
  return std::max(n, 1);
}

int resident_blocks_per_sm(int metric, int kmax) {
  auto pick = [&](auto m) {
    constexpr int MM = decltype(m)::value;
    if (kmax <= 4) return max_blocks_per_sm<MM, 4>();
    if (kmax <= 16) return max_blocks_per_sm<MM, 16>();
    return max_blocks_per_sm<MM, 32>();
  };
  switch (metric) {
    case M_L1: return pick(std::integral_constant<int, M_L1>{});
    case M_L2: return pick(std::integral_constant<int, M_L2>{});
    default: return pick(std::integral_constant<int, M_LINF>{});
  }
}

bool reference_order_forced() {
  static const bool force = [] {
    const char* m = std::getenv("KD_QUERY_MODE");
    return m && std::strcmp(m, "dfs") == 0;
  }();
  return force;
}

struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceScope() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace
}  // namespace kd

using namespace kd;

// The plan behind the opaque kd_batch* of the C ABI.
struct kd_batch {
  int device = 0;
  QueryParams qp{};
  std::vector<kd_batch_job> jobs;       // caller's jobs, in caller order
  std::vector<uint32_t> cls;            // packet class per caller job
  std::vector<uint32_t> packet_order;   // caller job ids of packet jobs, batch order
  std::vector<uint32_t> other;          // caller job ids run per job
  std::vector<uint64_t> other_axes;     // offset of each other job in axes scratch
  uint32_t total_q = 0;                 // queries of packet jobs
  uint32_t n_tasks = 0;
  uint64_t n_bins = 0;
  int kmax = 1;
  int sms = 1;
  // device memory (one allocation)
  void* mem = nullptr;
  BatchJob* jobs_sorted = nullptr;  // packet jobs, order = batch order
  BatchJob* jobs_plain = nullptr;   // packet jobs, no order
  uint32_t* q_start = nullptr;      // n_packet + 1
  uint32_t* task_start = nullptr;   // n_packet + 1
  uint64_t* bin_of = nullptr;       // total_q
  uint32_t* order = nullptr;        // total_q
  uint32_t* bins = nullptr;         // n_bins
  uint32_t* tile_sums = nullptr;
  uint32_t* counter = nullptr;
  uint32_t* status = nullptr;
  double* axes = nullptr;           // other jobs' CellBound scratch
  // tuned launch and the captured graph
  bool tuned = false;
  unsigned blocks = 0;
  bool sort = true;
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

// Enqueue one run of the plan on st: fused (sort + persistent kernel + other
// jobs) or per job.
int enqueue(kd_batch* b, cudaStream_t st, bool per_job, unsigned blocks, bool sort) {
  KD_TRY_CUDA(cudaMemsetAsync(b->status, 0, sizeof(uint32_t), st));
  if (per_job) {
    for (size_t j = 0; j < b->jobs.size(); ++j) {
      const kd_batch_job& J = b->jobs[j];
      QueryParams qp = b->qp;
      qp.k = J.k;
      if (b->cls[j] == CLS_OTHER) continue;
      int rc = query_on_device(J.tree, J.d_queries, J.n_queries, qp, J.d_out_distances, J.d_out_indices, st,
                               b->status);
      if (rc) return rc;
    }
  } else if (b->n_tasks) {
    const uint32_t n_packet = static_cast<uint32_t>(b->packet_order.size());
    if (sort) {
      KD_TRY_CUDA(cudaMemsetAsync(b->bins, 0, b->n_bins * sizeof(uint32_t), st));
      const unsigned qb = (b->total_q + 255) / 256;
      k_batch_landing<<<qb, 256, 0, st>>>(b->jobs_sorted, b->q_start, n_packet, b->total_q, b->bin_of, b->bins);
      const uint64_t n_tiles = (b->n_bins + SCAN_TILE - 1) / SCAN_TILE;
      k_scan_tiles<<<static_cast<unsigned>(n_tiles), SCAN_THREADS, 0, st>>>(b->bins, b->n_bins, b->tile_sums);
      k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(b->tile_sums, n_tiles);
      k_scan_add<<<static_cast<unsigned>((b->n_bins + 255) / 256), 256, 0, st>>>(b->bins, b->n_bins,
                                                                                 b->tile_sums);
      k_batch_scatter<<<qb, 256, 0, st>>>(b->q_start, n_packet, b->total_q, b->bin_of, b->bins, b->order);
      KD_TRY_CUDA(cudaGetLastError());
    }
    KD_TRY_CUDA(cudaMemsetAsync(b->counter, 0, sizeof(uint32_t), st));
    BatchArgs a{sort ? b->jobs_sorted : b->jobs_plain, b->task_start, n_packet, b->n_tasks, b->counter};
    cudaError_t e;
    switch (b->qp.metric) {
      case M_L1: e = launch_batch_k<M_L1>(a, b->kmax, blocks, st); break;
      case M_L2: e = launch_batch_k<M_L2>(a, b->kmax, blocks, st); break;
      default: e = launch_batch_k<M_LINF>(a, b->kmax, blocks, st); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "k_query_batch");
  }
  for (size_t o = 0; o < b->other.size(); ++o) {
    const kd_batch_job& J = b->jobs[b->other[o]];
    QueryParams qp = b->qp;
    qp.k = J.k;
    int rc;
    if (per_job)
      rc = query_on_device(J.tree, J.d_queries, J.n_queries, qp, J.d_out_distances, J.d_out_indices, st,
                           b->status);
    else
      rc = query_on_device_scratch(J.tree, J.d_queries, J.n_queries, qp, J.d_out_distances, J.d_out_indices, st,
                                   b->status, b->axes + b->other_axes[o]);
    if (rc) return rc;
  }
  return KD_OK;
}

int finish(kd_batch* b, cudaStream_t st) {
  uint32_t h = 0;
  KD_TRY_CUDA(cudaMemcpyAsync(&h, b->status, sizeof h, cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  if (h) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
  return KD_OK;
}

// The autotuner: every candidate launch shape runs the plan once to warm up
// and twice timed; the fastest is kept.  Results are identical for all.
int tune(kd_batch* b, cudaStream_t st) {
  const int per_sm = resident_blocks_per_sm(b->qp.metric, b->kmax);
  std::vector<unsigned> grids;
  for (int m : {1, 2, 4, 8})
    if (m <= per_sm) grids.push_back(static_cast<unsigned>(b->sms * m));
  grids.push_back(static_cast<unsigned>(b->sms * per_sm));
  std::sort(grids.begin(), grids.end());
  grids.erase(std::unique(grids.begin(), grids.end()), grids.end());
  cudaEvent_t e0, e1;
  KD_TRY_CUDA(cudaEventCreate(&e0));
  KD_TRY_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int rc = KD_OK;
  for (bool sort : {true, false}) {
    for (unsigned g : grids) {
      float t_min = 1e30f;
      for (int rep = 0; rep < 3 && rc == KD_OK; ++rep) {
        cudaEventRecord(e0, st);
        rc = enqueue(b, st, false, g, sort);
        cudaEventRecord(e1, st);
        if (rc == KD_OK) rc = finish(b, st);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) t_min = std::min(t_min, ms);
      }
      if (rc != KD_OK) break;
      if (t_min < best) {
        best = t_min;
        b->blocks = g;
        b->sort = sort;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == KD_OK) b->tuned = true;
  return rc;
}

int capture(kd_batch* b) {
  if (!b->capture_stream) KD_TRY_CUDA(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  KD_TRY_CUDA(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal));
  const int rc = enqueue(b, b->capture_stream, false, b->blocks, b->sort);
  cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->exec = nullptr;
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  return KD_OK;
}

void release(kd_batch* b) {
  if (!b) return;
  DeviceScope scope(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  if (b->mem) cudaFree(b->mem);
  delete b;
}

}  // namespace

extern "C" {

int kd_batch_create(const kd_batch_job* jobs, uint64_t n_jobs, double p, int has_max_distance, double max_distance,
                    double eps, kd_batch** out) {
  if (!out) return fail(KD_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!jobs || n_jobs == 0) return fail(KD_ERR_INVALID_ARGUMENT, "a batch needs at least one job");
  if (n_jobs >= 0xffffffffull) return fail(KD_ERR_INVALID_ARGUMENT, "too many jobs");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(KD_ERR_NO_DEVICE, "no CUDA device is visible; the GB300 engine has no CPU fallback");
  }
  QueryParams qp{};
  std::string msg;
  int rc = validate_scalars(1, p, has_max_distance, max_distance, eps, &qp, &msg);
  if (rc) return fail(rc, msg);
  kd_batch* b = new (std::nothrow) kd_batch();
  if (!b) return fail(KD_ERR_OUT_OF_MEMORY, "host allocation failed");
  b->device = dev;
  b->qp = qp;
  b->jobs.assign(jobs, jobs + n_jobs);
  const bool ref = reference_order_forced();
  uint64_t total_q = 0, axes_words = 0;
  for (uint64_t j = 0; j < n_jobs; ++j) {
    const kd_batch_job& J = jobs[j];
    if (!J.tree) rc = fail(KD_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": tree is NULL");
    else if (J.k == 0) rc = fail(KD_ERR_INVALID_K, "k must be greater than zero");
    else if (J.n_queries == 0)
      rc = fail(KD_ERR_INVALID_SHAPE, "queries must be a contiguous row-major matrix");
    else if (!J.d_queries || !J.d_out_distances || !J.d_out_indices)
      rc = fail(KD_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": NULL buffer");
    else if (J.tree->device != dev)
      rc = fail(KD_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": tree lives on another device");
    else if (J.n_queries > (~0ull / sizeof(double)) / J.k / J.tree->ndim)
      rc = fail(KD_ERR_OUT_OF_MEMORY, "output would not fit in memory");
    if (rc) {
      delete b;
      return rc;
    }
    QueryParams jq = qp;
    jq.k = J.k;
    const uint32_t c = packet_class(J.tree, jq, ref);
    b->cls.push_back(c);
    if (c == CLS_OTHER) {
      b->other.push_back(static_cast<uint32_t>(j));
      b->other_axes.push_back(axes_words);
      axes_words += J.n_queries * J.tree->ndim;
    } else {
      b->packet_order.push_back(static_cast<uint32_t>(j));
      total_q += J.n_queries;
      b->kmax = std::max(b->kmax, BATCH_K[c % 5]);
    }
  }
  if (total_q >= 0xffffffffull) {
    delete b;
    return fail(KD_ERR_INVALID_ARGUMENT, "a batch holds at most 2^32 - 1 queries");
  }
  // most expensive class first: larger k, then wider points
  std::stable_sort(b->packet_order.begin(), b->packet_order.end(), [&](uint32_t x, uint32_t y) {
    const uint32_t cx = b->cls[x], cy = b->cls[y];
    if (cx % 5 != cy % 5) return cx % 5 > cy % 5;
    return cx / 5 > cy / 5;
  });
  const uint32_t n_packet = static_cast<uint32_t>(b->packet_order.size());
  std::vector<uint32_t> q_start(n_packet + 1), task_start(n_packet + 1);
  std::vector<uint64_t> bin_start(n_packet + 1);
  for (uint32_t i = 0; i < n_packet; ++i) {
    const kd_batch_job& J = jobs[b->packet_order[i]];
    q_start[i + 1] = q_start[i] + static_cast<uint32_t>(J.n_queries);
    task_start[i + 1] = task_start[i] + static_cast<uint32_t>((J.n_queries + 31) / 32);
    bin_start[i + 1] = bin_start[i] + J.tree->n_nodes;
  }
  b->total_q = static_cast<uint32_t>(total_q);
  b->n_tasks = task_start[n_packet];
  b->n_bins = std::max<uint64_t>(bin_start[n_packet], 1);
  const uint64_t n_tiles = (b->n_bins + SCAN_TILE - 1) / SCAN_TILE;
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);

  // one device allocation, 256-byte aligned pieces
  auto up = [](uint64_t x) { return (x + 255) & ~255ull; };
  const uint64_t sz_jobs = up(std::max<uint32_t>(n_packet, 1) * sizeof(BatchJob));
  const uint64_t sz_qs = up((n_packet + 1) * sizeof(uint32_t));
  const uint64_t sz_binof = up(std::max<uint64_t>(total_q, 1) * sizeof(uint64_t));
  const uint64_t sz_order = up(std::max<uint64_t>(total_q, 1) * sizeof(uint32_t));
  const uint64_t sz_bins = up(b->n_bins * sizeof(uint32_t));
  const uint64_t sz_tiles = up(n_tiles * sizeof(uint32_t));
  const uint64_t sz_axes = up(std::max<uint64_t>(axes_words, 1) * sizeof(double));
  const uint64_t total = 2 * sz_jobs + 2 * sz_qs + sz_binof + sz_order + sz_bins + sz_tiles + 512 + sz_axes;
  cudaError_t e = cudaMalloc(&b->mem, total);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "cudaMalloc");
  }
  char* m = static_cast<char*>(b->mem);
  b->jobs_sorted = reinterpret_cast<BatchJob*>(m);
  m += sz_jobs;
  b->jobs_plain = reinterpret_cast<BatchJob*>(m);
  m += sz_jobs;
  b->q_start = reinterpret_cast<uint32_t*>(m);
  m += sz_qs;
  b->task_start = reinterpret_cast<uint32_t*>(m);
  m += sz_qs;
  b->bin_of = reinterpret_cast<uint64_t*>(m);
  m += sz_binof;
  b->order = reinterpret_cast<uint32_t*>(m);
  m += sz_order;
  b->bins = reinterpret_cast<uint32_t*>(m);
  m += sz_bins;
  b->tile_sums = reinterpret_cast<uint32_t*>(m);
  m += sz_tiles;
  b->counter = reinterpret_cast<uint32_t*>(m);
  b->status = reinterpret_cast<uint32_t*>(m + 256);
  m += 512;
  b->axes = reinterpret_cast<double*>(m);

  std::vector<BatchJob> hs(n_packet), hp(n_packet);
  for (uint32_t i = 0; i < n_packet; ++i) {
    const kd_batch_job& J = jobs[b->packet_order[i]];
    const kd_tree* t = J.tree;
    QArgs a{};
    a.data = t->data;
    a.data32 = t->data32;
    a.indices = t->indices;
    a.nodes = t->nodes;
    a.boxes = t->boxes;
    a.boxes32 = t->boxes32;
    a.coord_max = t->coord_max32;
    a.queries = J.d_queries;
    a.out_d = J.d_out_distances;
    a.out_i = J.d_out_indices;
    a.status = b->status;
    a.nq = J.n_queries;
    a.d = t->ndim;
    a.k = J.k;
    a.n_points = t->n_points;
    a.p = qp.p;
    a.cutoff = qp.cutoff;
    a.eps_factor = qp.eps_factor;
    a.use_eps = 0;
    hs[i].a = a;
    hs[i].a.order = b->order + q_start[i];
    hs[i].bin_start = bin_start[i];
    hs[i].cls = b->cls[b->packet_order[i]];
    hp[i] = hs[i];
    hp[i].a.order = nullptr;
  }
  e = cudaMemcpy(b->jobs_sorted, hs.data(), n_packet * sizeof(BatchJob), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->jobs_plain, hp.data(), n_packet * sizeof(BatchJob), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->q_start, q_start.data(), q_start.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->task_start, task_start.data(), task_start.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    release(b);
    return cuda_fail(e, "cudaMemcpy");
  }
  b->blocks = static_cast<unsigned>(b->sms * resident_blocks_per_sm(qp.metric, b->kmax));
  *out = b;
  return KD_OK;
}

int kd_batch_run_mode(kd_batch* b, void* stream, int mode) {
  if (!b) return fail(KD_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (mode < KD_BATCH_GRAPH || mode > KD_BATCH_PER_JOB) return fail(KD_ERR_INVALID_ARGUMENT, "unknown batch mode");
  DeviceScope scope(b->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc;
  if (mode == KD_BATCH_GRAPH) {
    if (!b->tuned && (rc = tune(b, st))) return rc;
    if (!b->exec && (rc = capture(b))) return rc;
    KD_TRY_CUDA(cudaGraphLaunch(b->exec, st));
  } else if ((rc = enqueue(b, st, mode == KD_BATCH_PER_JOB, b->blocks, b->sort))) {
    return rc;
  }
  return finish(b, st);
}

int kd_batch_run(kd_batch* b, void* stream) { return kd_batch_run_mode(b, stream, KD_BATCH_GRAPH); }

void kd_batch_free(kd_batch* b) { release(b); }

}  // extern "C"
