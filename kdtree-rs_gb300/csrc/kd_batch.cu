// kd_batch.cu -- many (tree, query batch) jobs in one pass on the device: the
// batch plan (kd_batch_*) and the serving loop built on it (kd_server_*).
//
// No reference counterpart: the reference answers one Tree::query call at a
// time (src/query.rs:29-78); a batch is its caller's loop over many trees,
// fused.  Running a batch:
//  1. one kernel walks every query of every packet job down its own tree to
//     its landing leaf and counts it into bin (job, leaf); one scan over all
//     bins and one scatter leave each job's queries grouped by landing leaf,
//     jobs one after another in the batch order (jobs below 1,024 queries
//     keep their own order: one bin);
//  2. ONE persistent kernel: each warp takes the next task -- 4 consecutive
//     positions of one job's queries -- from a global counter and runs them
//     one by one with the warp-per-query traversal (kd_query_warp.cuh) for the
//     job's width.  Jobs are laid out widest (most expensive) first, so the
//     long tasks start early and the short ones fill the tail;
//  3. jobs outside the fused kernel's envelope (general L^p, eps > 0, k > 64,
//     widths other than 2, 3, 8 and 16, the reference-order switch) run as
//     ordinary per-job launches of the kernels kd_query_device uses, on side
//     streams beside the fused kernel -- the packet traversal for k <= 64,
//     the reference-order descent otherwise; never the tensor-core filter,
//     whose brute-force scan only pays on trees that do not prune.
// A query's result depends on that query and its tree alone, so every job
// gets exactly what kd_query_device returns for it.
//
// A plan (kd_batch_create) fixes its jobs.  Its first graph run times a few
// launch shapes -- persistent grid size, sorting on or off -- and keeps the
// fastest (the autotuner), then captures the whole sequence in a CUDA graph;
// later runs replay the graph.  The server (kd_server_create) forms a new batch
// from the waiting requests whenever one of its two batch slots is free
// (continuous batching), with the same kernels.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "kd_internal.hpp"

namespace kd {
namespace {

#include "kd_query_common.cuh"
#include "kd_scan.cuh"
#include "kd_lazy_best.cuh"
#include "kd_query_packet.cuh"
#include "kd_warp.cuh"
#include "kd_query_warp.cuh"
#include "kd_query_ref.cuh"

constexpr uint32_t CLS_OTHER = 0xffffffffu;
constexpr uint64_t SORT_MIN_QUERIES = 1024;
constexpr uint32_t TASK_QUERIES = 4;  // queries per warp-traversal task: one after another on one warp
constexpr uint32_t PACKET_TASK = 32;  // queries per packet task: one per lane
// Packet classes (the packet traversal, k-best lists in registers):
// CLS_PACKET + 2 * width index + (k > 1 ? 1 : 0), for k <= 4.
constexpr uint32_t CLS_PACKET = 8;

// Class of a job in the fused kernel (width index, + 4 for k > 32: two list
// slots per lane), or CLS_OTHER.
uint32_t fused_class(const kd_tree* t, const QueryParams& qp, uint64_t k, bool reference_order) {
  if (qp.metric == M_LP || qp.eps_factor != 1.0 || k > 64 || t->n_points >= ROW_NONE || reference_order)
    return CLS_OTHER;
  const uint32_t wide = k > 32 ? 4 : 0;
  switch (t->ndim) {
    case 2: return 0 + wide;
    case 3: return 1 + wide;
    case 8: return 2 + wide;
    case 16: return 3 + wide;
    default: return CLS_OTHER;
  }
}

bool reference_order_forced() {
  static const bool force = [] {
    const char* m = std::getenv("KD_QUERY_MODE");
    return m && std::strcmp(m, "dfs") == 0;
  }();
  return force;
}

struct BatchJob {
  QArgs a;             // the job's query arguments; a.order points into the batch order or is NULL
  uint64_t bin_start;  // the job's first landing-leaf bin
  uint32_t cls;        // fused class (warp traversal 0-7, packet traversal CLS_PACKET + ...)
  uint32_t sorted;     // 1: bins per node (sorted by landing leaf); 0: one bin
};

// Queries per task of a job of class cls.
__host__ __device__ __forceinline__ uint32_t task_queries(uint32_t cls) {
  return cls >= CLS_PACKET ? PACKET_TASK : TASK_QUERIES;
}

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
  uint32_t node = 0;
  if (J.sorted) {
    const double* q = J.a.queries + static_cast<uint64_t>(g - q_start[j]) * J.a.d;
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

template <int M, int D, int KS>
__device__ __forceinline__ void batch_query(const QArgs* a, uint64_t w, WarpStack* stack) {
  warp_query<M, D, KS>(*a, w, stack, nullptr);
}

// The persistent kernel: warps take tasks until none is left -- TASK_QUERIES
// consecutive positions of one job, each run with the warp-per-query traversal
// (kd_query_warp.cuh) for the job's width, or, for the packet classes, 32
// consecutive positions of the job's landing-leaf order run together by the
// packet traversal (kd_query_packet.cuh; k <= 4, lists in registers).  W16: the
// batch holds 16-wide jobs; without them the kernel is held to 72 registers,
// 7 blocks an SM instead of 5 (measured faster on the mixed 2/3/8-wide batch
// than the 87 registers the compiler picks unbounded).
template <int M, bool W16>
__global__ void __launch_bounds__(QUERY_THREADS, W16 ? 5 : 7) k_query_batch(BatchArgs b) {
  __shared__ WarpStack s_stack[QUERY_THREADS / 32];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(b.next_task, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= b.n_tasks) return;
    const uint32_t j = find_range(b.task_start, b.n_jobs, t);
    const BatchJob* J = b.jobs + j;
    if (J->cls >= CLS_PACKET) {
      // the warp's own stack words (its WarpStack is free during a packet task)
      uint32_t* stack = s_stack[wid].node;
      const uint64_t tid = static_cast<uint64_t>(t - b.task_start[j]) * PACKET_TASK + lane;
      switch (J->cls - CLS_PACKET) {
        case 0: packet_queries<M, 2, 1>(J->a, tid, nullptr, nullptr, nullptr, stack); break;
        case 1: packet_queries<M, 2, 4>(J->a, tid, nullptr, nullptr, nullptr, stack); break;
        case 2: packet_queries<M, 3, 1>(J->a, tid, nullptr, nullptr, nullptr, stack); break;
        case 3: packet_queries<M, 3, 4>(J->a, tid, nullptr, nullptr, nullptr, stack); break;
        case 4: packet_queries<M, 8, 1>(J->a, tid, nullptr, nullptr, nullptr, stack); break;
        default: packet_queries<M, 8, 4>(J->a, tid, nullptr, nullptr, nullptr, stack); break;
      }
      continue;
    }
    const uint64_t first = static_cast<uint64_t>(t - b.task_start[j]) * TASK_QUERIES;
    const uint64_t last = min(first + TASK_QUERIES, J->a.nq);
    for (uint64_t w = first; w < last; ++w) {
      switch (J->cls) {
        case 0: batch_query<M, 2, 1>(&J->a, w, &s_stack[wid]); break;
        case 1: batch_query<M, 3, 1>(&J->a, w, &s_stack[wid]); break;
        case 2: batch_query<M, 8, 1>(&J->a, w, &s_stack[wid]); break;
        case 4: batch_query<M, 2, 2>(&J->a, w, &s_stack[wid]); break;
        case 5: batch_query<M, 3, 2>(&J->a, w, &s_stack[wid]); break;
        case 6: batch_query<M, 8, 2>(&J->a, w, &s_stack[wid]); break;
        default:  // classes 3 and 7, present only when W16
          if constexpr (W16) {
            if (J->cls == 3) batch_query<M, 16, 1>(&J->a, w, &s_stack[wid]);
            else batch_query<M, 16, 2>(&J->a, w, &s_stack[wid]);
          }
          break;
      }
    }
  }
}

// Near-tie reruns of the fused kernel's queries (kd_warp.cuh): each entry of
// `list` is (packet job << 32 | query index); warps run them in the
// reference's order with that job's arguments.
template <int M>
__global__ void __launch_bounds__(QUERY_THREADS) k_batch_rerun(const BatchJob* jobs, const uint32_t* count,
                                                               const uint64_t* list) {
  __shared__ RefFrame s_fr[QUERY_THREADS / 32][REF_FRAMES];
  __shared__ double s_axes[QUERY_THREADS / 32][16];
  const uint32_t wid = threadIdx.x >> 5;
  const uint64_t n = *count;
  const uint64_t warps = static_cast<uint64_t>(gridDim.x) * (QUERY_THREADS / 32);
  for (uint64_t w = blockIdx.x * static_cast<uint64_t>(QUERY_THREADS / 32) + wid; w < n; w += warps) {
    const uint64_t e = list[w];
    const BatchJob* J = jobs + (e >> 32);
    const uint64_t qi = static_cast<uint32_t>(e);
    // the warp class of the job (a packet class: its width, one list slot a lane)
    const uint32_t wc = J->cls >= CLS_PACKET ? (J->cls - CLS_PACKET) / 2 : J->cls;
    bool stands;
    switch (wc & 3) {  // widths 2, 3, 8, 16 (the class's low bits)
      case 0: stands = ref_results_stand<M, 2>(J->a, qi); break;
      case 1: stands = ref_results_stand<M, 3>(J->a, qi); break;
      case 2: stands = ref_results_stand<M, 8>(J->a, qi); break;
      default: stands = ref_results_stand<M, 16>(J->a, qi); break;
    }
    if (stands) continue;
    switch (wc) {
      case 0: ref_query<M, 2, 1>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      case 1: ref_query<M, 3, 1>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      case 2: ref_query<M, 8, 1>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      case 3: ref_query<M, 16, 1>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      case 4: ref_query<M, 2, 2>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      case 5: ref_query<M, 3, 2>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      case 6: ref_query<M, 8, 2>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
      default: ref_query<M, 16, 2>(J->a, qi, s_fr[wid], s_axes[wid], nullptr); break;
    }
  }
}

template <int M, bool W16>
int max_blocks_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_query_batch<M, W16>, QUERY_THREADS, 0);
  return std::max(n, 1);
}

int resident_blocks_per_sm(int metric, bool w16) {
  switch (metric) {
    case M_L1: return w16 ? max_blocks_per_sm<M_L1, true>() : max_blocks_per_sm<M_L1, false>();
    case M_L2: return w16 ? max_blocks_per_sm<M_L2, true>() : max_blocks_per_sm<M_L2, false>();
    default: return w16 ? max_blocks_per_sm<M_LINF, true>() : max_blocks_per_sm<M_LINF, false>();
  }
}

template <int M>
void launch_batch(bool w16, unsigned blocks, cudaStream_t st, const BatchArgs& a, const uint32_t* rerun_count,
                  const uint64_t* rerun_list, unsigned rerun_blocks) {
  if (w16) k_query_batch<M, true><<<blocks, QUERY_THREADS, 0, st>>>(a);
  else k_query_batch<M, false><<<blocks, QUERY_THREADS, 0, st>>>(a);
  k_batch_rerun<M><<<rerun_blocks, QUERY_THREADS, 0, st>>>(a.jobs, rerun_count, rerun_list);
}

// ---------------------------------------------------------------------------
// Host side: a batch's layout and its device buffers.
// ---------------------------------------------------------------------------

// One job as the batch code sees it: device buffers and a device status word.
struct JobSpec {
  const kd_tree* tree;
  const double* queries;
  uint64_t nq, k;
  double* out_d;
  int64_t* out_i;
  uint32_t* status;
};

struct Layout {
  std::vector<uint32_t> packet;  // spec ids of the packet jobs, in batch order
  std::vector<uint32_t> other;   // spec ids run per job
  std::vector<uint32_t> q_start, task_start;
  std::vector<BatchJob> table;
  uint64_t n_bins = 1;
  uint32_t total_q = 0, n_tasks = 0;
  bool wide16 = false;  // some fused job is 16 wide
};

void fill_args(QArgs* a, const JobSpec& J, const QueryParams& qp) {
  const kd_tree* t = J.tree;
  *a = QArgs{};
  a->data = t->data;
  a->data32 = t->data32;
  a->data32w = t->data32w;
  a->w32 = t->w32;
  a->indices = t->indices;
  a->rows_of = t->rows_of;
  a->nodes = t->nodes;
  a->boxes = t->boxes;
  a->boxes32 = t->boxes32;
  a->coord_max = t->coord_max32;
  a->queries = J.queries;
  a->out_d = J.out_d;
  a->out_i = J.out_i;
  a->status = J.status;
  a->nq = J.nq;
  a->d = t->ndim;
  a->k = J.k;
  a->n_points = t->n_points;
  a->p = qp.p;
  a->cutoff = qp.cutoff;
  a->eps_factor = qp.eps_factor;
  a->use_eps = qp.eps_factor != 1.0;
}

// Lay the jobs out.  `order` is the device batch order (total packet queries
// u32); sort = false gives every job one bin and no order.  The fused jobs
// flag their near ties into (rerun_count, rerun_list), tagged with their
// position in the table.
// packet_widths: bit w (width index: 2, 3, 8) set -- that width's jobs with
// k <= 4 run as packet tasks.
void make_layout(const std::vector<JobSpec>& specs, const QueryParams& qp, bool sort, uint32_t* order,
                 uint32_t* rerun_count, uint64_t* rerun_list, Layout* L, uint32_t packet_widths = 0) {
  *L = Layout{};
  const bool ref = reference_order_forced();
  std::vector<uint32_t> cls(specs.size());
  for (size_t j = 0; j < specs.size(); ++j) {
    cls[j] = fused_class(specs[j].tree, qp, specs[j].k, ref);
    (cls[j] == CLS_OTHER ? L->other : L->packet).push_back(static_cast<uint32_t>(j));
  }
  // most expensive first: wider points, then larger k
  std::stable_sort(L->packet.begin(), L->packet.end(), [&](uint32_t x, uint32_t y) {
    if (cls[x] % 4 != cls[y] % 4) return cls[x] % 4 > cls[y] % 4;
    return specs[x].k > specs[y].k;
  });
  const size_t n = L->packet.size();
  L->q_start.assign(n + 1, 0);
  L->task_start.assign(n + 1, 0);
  L->table.resize(n);
  uint64_t bins = 0;
  for (size_t i = 0; i < n; ++i) {
    const JobSpec& J = specs[L->packet[i]];
    BatchJob& B = L->table[i];
    fill_args(&B.a, J, qp);
    B.a.rerun_count = rerun_count;
    B.a.rerun_list = rerun_list;
    B.a.rerun_tag = static_cast<uint32_t>(i);
    B.cls = cls[L->packet[i]];
    L->wide16 |= B.cls % 4 == 3;
    if (B.cls < 3 && J.k <= 4 && ((packet_widths >> B.cls) & 1u)) B.cls = CLS_PACKET + 2 * B.cls + (J.k > 1 ? 1 : 0);
    B.sorted = sort && J.nq >= SORT_MIN_QUERIES;
    B.a.order = B.sorted ? order + L->q_start[i] : nullptr;
    B.bin_start = bins;
    bins += B.sorted ? J.tree->n_nodes : 1;
    L->q_start[i + 1] = L->q_start[i] + static_cast<uint32_t>(J.nq);
    const uint32_t tq = task_queries(B.cls);
    L->task_start[i + 1] = L->task_start[i] + static_cast<uint32_t>((J.nq + tq - 1) / tq);
  }
  L->n_bins = std::max<uint64_t>(bins, 1);
  L->total_q = L->q_start[n];
  L->n_tasks = L->task_start[n];
}

// Device buffers of one batch, carved from one allocation.
struct Buffers {
  void* mem = nullptr;
  BatchJob* jobs[2] = {nullptr, nullptr};
  uint32_t* q_start = nullptr;
  uint32_t* task_start = nullptr;
  uint64_t* bin_of = nullptr;
  uint32_t* order = nullptr;
  uint32_t* bins = nullptr;
  uint32_t* tile_sums = nullptr;
  uint32_t* counter = nullptr;
  uint32_t* rerun_count = nullptr;  // near ties of the fused kernel
  uint64_t* rerun_list = nullptr;   // cap_q entries
  uint64_t cap_jobs = 0, cap_q = 0, cap_bins = 0;
  ~Buffers() {
    if (mem) cudaFree(mem);
  }
};

// Sizes of the carve-up; `extra` bytes at the end are the caller's.
uint64_t round256(uint64_t x) { return (x + 255) & ~255ull; }

int alloc_buffers(Buffers* B, uint64_t cap_jobs, uint64_t cap_q, uint64_t cap_bins, uint64_t extra, char** extra_p) {
  cap_jobs = std::max<uint64_t>(cap_jobs, 1);
  cap_q = std::max<uint64_t>(cap_q, 1);
  cap_bins = std::max<uint64_t>(cap_bins, 1);
  const uint64_t n_tiles = (cap_bins + SCAN_TILE - 1) / SCAN_TILE;
  const uint64_t sz_jobs = round256(cap_jobs * sizeof(BatchJob));
  const uint64_t sz_st = round256((cap_jobs + 1) * sizeof(uint32_t));
  const uint64_t total = 2 * sz_jobs + 2 * sz_st + round256(cap_q * 8) + round256(cap_q * 4) +
                         round256(cap_bins * 4) + round256(n_tiles * 4) + 256 + round256(cap_q * 8) +
                         round256(extra);
  cudaError_t e = cudaMalloc(&B->mem, total);
  if (e != cudaSuccess) {
    B->mem = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  char* m = static_cast<char*>(B->mem);
  auto take = [&](uint64_t bytes) {
    char* p = m;
    m += bytes;
    return p;
  };
  B->jobs[0] = reinterpret_cast<BatchJob*>(take(sz_jobs));
  B->jobs[1] = reinterpret_cast<BatchJob*>(take(sz_jobs));
  B->q_start = reinterpret_cast<uint32_t*>(take(sz_st));
  B->task_start = reinterpret_cast<uint32_t*>(take(sz_st));
  B->bin_of = reinterpret_cast<uint64_t*>(take(round256(cap_q * 8)));
  B->order = reinterpret_cast<uint32_t*>(take(round256(cap_q * 4)));
  B->bins = reinterpret_cast<uint32_t*>(take(round256(cap_bins * 4)));
  B->tile_sums = reinterpret_cast<uint32_t*>(take(round256(n_tiles * 4)));
  B->counter = reinterpret_cast<uint32_t*>(take(256));
  B->rerun_count = B->counter + 32;  // same 256-byte block, its own 128 bytes
  B->rerun_list = reinterpret_cast<uint64_t*>(take(round256(cap_q * 8)));
  if (extra_p) *extra_p = take(round256(extra));
  B->cap_jobs = cap_jobs;
  B->cap_q = cap_q;
  B->cap_bins = cap_bins;
  return KD_OK;
}

// Enqueue the sort and the persistent kernel of a layout whose table, q_start
// and task_start are already in B (table in B->jobs[table]).
int enqueue_packet(const Layout& L, const Buffers& B, int table, int metric, unsigned blocks, cudaStream_t st) {
  if (!L.n_tasks) return KD_OK;
  const uint32_t n = static_cast<uint32_t>(L.packet.size());
  KD_TRY_CUDA(cudaMemsetAsync(B.bins, 0, L.n_bins * sizeof(uint32_t), st));
  const unsigned qb = (L.total_q + 255) / 256;
  k_batch_landing<<<qb, 256, 0, st>>>(B.jobs[table], B.q_start, n, L.total_q, B.bin_of, B.bins);
  const uint64_t n_tiles = (L.n_bins + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_tiles<<<static_cast<unsigned>(n_tiles), SCAN_THREADS, 0, st>>>(B.bins, L.n_bins, B.tile_sums);
  k_scan_sums<<<1, SCAN_THREADS, 0, st>>>(B.tile_sums, n_tiles);
  k_scan_add<<<static_cast<unsigned>((L.n_bins + 255) / 256), 256, 0, st>>>(B.bins, L.n_bins, B.tile_sums);
  k_batch_scatter<<<qb, 256, 0, st>>>(B.q_start, n, L.total_q, B.bin_of, B.bins, B.order);
  KD_TRY_CUDA(cudaGetLastError());
  KD_TRY_CUDA(cudaMemsetAsync(B.counter, 0, 256, st));  // task counter and rerun count
  BatchArgs a{B.jobs[table], B.task_start, n, L.n_tasks, B.counter};
  // the reruns: a few warps an SM at most (their count is only known on the device)
  const unsigned rerun_blocks = std::max(1u, std::min(blocks, (L.total_q + 3) / 4));
  switch (metric) {
    case M_L1: launch_batch<M_L1>(L.wide16, blocks, st, a, B.rerun_count, B.rerun_list, rerun_blocks); break;
    case M_L2: launch_batch<M_L2>(L.wide16, blocks, st, a, B.rerun_count, B.rerun_list, rerun_blocks); break;
    default: launch_batch<M_LINF>(L.wide16, blocks, st, a, B.rerun_count, B.rerun_list, rerun_blocks); break;
  }
  KD_TRY_CUDA(cudaGetLastError());
  return KD_OK;
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

// Streams for a batch's per-job launches: they fork from the batch stream and
// join back into it, so those jobs' kernels overlap one another (and the fused
// kernel) instead of queueing one after the other.
struct SideStreams {
  static constexpr int N = 4;
  cudaStream_t s[N] = {};
  cudaEvent_t fork = nullptr, join[N] = {};
  int create() {
    for (int i = 0; i < N; ++i) {
      KD_TRY_CUDA(cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking));
      KD_TRY_CUDA(cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming));
    }
    KD_TRY_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    return KD_OK;
  }
  ~SideStreams() {
    for (int i = 0; i < N; ++i) {
      if (s[i]) cudaStreamDestroy(s[i]);
      if (join[i]) cudaEventDestroy(join[i]);
    }
    if (fork) cudaEventDestroy(fork);
  }
};

// st waits for the side streams that n_other per-job launches used.
void join_others(SideStreams& ss, size_t n_other, cudaStream_t st) {
  const int used = static_cast<int>(std::min<size_t>(SideStreams::N, n_other));
  for (int i = 0; i < used; ++i) {
    cudaEventRecord(ss.join[i], ss.s[i]);
    cudaStreamWaitEvent(st, ss.join[i], 0);
  }
}

// Per-job launches of `other` on the side streams, forked from st (join them
// with join_others once st's own work is enqueued).  scratch != NULL: the
// allocation-free kernels with that scratch (byte offsets scratch_off, see
// query_on_device_scratch) and one rerun counter per job (counters), as a
// graph capture needs.
int enqueue_others(const std::vector<JobSpec>& specs, const std::vector<uint32_t>& other, const QueryParams& base,
                   SideStreams& ss, cudaStream_t st, unsigned char* scratch, const std::vector<uint64_t>& scratch_off,
                   uint32_t* counters) {
  if (other.empty()) return KD_OK;
  const int used = static_cast<int>(std::min<size_t>(SideStreams::N, other.size()));
  KD_TRY_CUDA(cudaEventRecord(ss.fork, st));
  for (int i = 0; i < used; ++i) KD_TRY_CUDA(cudaStreamWaitEvent(ss.s[i], ss.fork, 0));
  int rc = KD_OK;
  for (size_t o = 0; o < other.size() && rc == KD_OK; ++o) {
    const JobSpec& J = specs[other[o]];
    QueryParams qp = base;
    qp.k = J.k;
    qp.path = PATH_PACKET;  // never the tensor-core filter inside a batch
    cudaStream_t side = ss.s[o % SideStreams::N];
    rc = scratch ? query_on_device_scratch(J.tree, J.queries, J.nq, qp, J.out_d, J.out_i, side, J.status,
                                           scratch + scratch_off[o], counters + o)
                 : query_on_device(J.tree, J.queries, J.nq, qp, J.out_d, J.out_i, side, J.status);
  }
  if (rc) join_others(ss, other.size(), st);  // nothing is left behind on a failure
  return rc;
}

int job_error(const kd_tree* tree, uint64_t nq, uint64_t k, const void* q, const void* od, const void* oi,
              int dev, const std::string& who) {
  if (!tree) return fail(KD_ERR_INVALID_ARGUMENT, who + ": tree is NULL");
  if (k == 0) return fail(KD_ERR_INVALID_K, "k must be greater than zero");
  if (nq == 0) return fail(KD_ERR_INVALID_SHAPE, "queries must be a contiguous row-major matrix");
  if (!q || !od || !oi) return fail(KD_ERR_INVALID_ARGUMENT, who + ": NULL buffer");
  if (tree->device != dev) return fail(KD_ERR_INVALID_ARGUMENT, who + ": tree lives on another device");
  if (nq > (~0ull / sizeof(double)) / k / tree->ndim) return fail(KD_ERR_OUT_OF_MEMORY, "output would not fit in memory");
  return KD_OK;
}

// Rows of a tree spread over it (every (n / m)-th), as queries for the
// server's calibration.
__global__ void k_sample_rows(const double* data, uint64_t n, uint64_t d, uint64_t m, double* out) {
  const uint64_t f = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (f >= m * d) return;
  const uint64_t r = f / d, j = f - r * d;
  out[f] = data[(r * (n / m)) * d + j];
}

}  // namespace
}  // namespace kd

using namespace kd;

// ===========================================================================
// The batch plan behind the opaque kd_batch* of the C ABI.
// ===========================================================================
struct kd_batch {
  int device = 0;
  int sms = 1;
  QueryParams qp{};
  std::vector<JobSpec> specs;  // caller order
  Layout layout[2];            // [0] sorted, [1] unsorted (same jobs and positions)
  Buffers buf;
  uint32_t* status = nullptr;
  unsigned char* scratch = nullptr;    // other jobs' scratch (query_on_device_scratch)
  std::vector<uint64_t> scratch_off;   // per other job (layout order), bytes
  uint32_t* counters = nullptr;        // per other job: its near-tie rerun count
  bool tuned = false;
  unsigned blocks = 0;
  int table = 0;
  uint32_t packet_widths = 0;  // widths (bit: index of 2, 3, 8) whose k <= 4 jobs run as packet tasks
  SideStreams side;
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

int enqueue_plan(kd_batch* b, cudaStream_t st, bool per_job, unsigned blocks, int table) {
  KD_TRY_CUDA(cudaMemsetAsync(b->status, 0, sizeof(uint32_t), st));
  const Layout& L = b->layout[table];
  if (per_job) {  // one launch sequence per job, one after another (the baseline)
    for (const JobSpec& J : b->specs) {
      QueryParams qp = b->qp;
      qp.k = J.k;
      qp.path = PATH_PACKET;
      int rc = query_on_device(J.tree, J.queries, J.nq, qp, J.out_d, J.out_i, st, b->status);
      if (rc) return rc;
    }
    return KD_OK;
  }
  int rc = enqueue_others(b->specs, L.other, b->qp, b->side, st, b->scratch, b->scratch_off, b->counters);
  if (rc) return rc;
  rc = enqueue_packet(L, b->buf, table, b->qp.metric, blocks, st);
  join_others(b->side, L.other.size(), st);
  return rc;
}

int finish_plan(kd_batch* b, cudaStream_t st) {
  uint32_t h = 0;
  KD_TRY_CUDA(cudaMemcpyAsync(&h, b->status, sizeof h, cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  if (h) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
  return KD_OK;
}

// Lay the fused jobs out again with packet_widths and upload the tables (the
// jobs and task ranges change; the query ranges and the other jobs do not).
int apply_layouts(kd_batch* b, uint32_t packet_widths) {
  for (int t = 0; t < 2; ++t)
    make_layout(b->specs, b->qp, t == 0, b->buf.order, b->buf.rerun_count, b->buf.rerun_list, &b->layout[t],
                packet_widths);
  const size_t np = b->layout[0].packet.size();
  if (np) {
    KD_TRY_CUDA(cudaMemcpy(b->buf.jobs[0], b->layout[0].table.data(), np * sizeof(BatchJob), cudaMemcpyHostToDevice));
    KD_TRY_CUDA(cudaMemcpy(b->buf.jobs[1], b->layout[1].table.data(), np * sizeof(BatchJob), cudaMemcpyHostToDevice));
    KD_TRY_CUDA(cudaMemcpy(b->buf.task_start, b->layout[0].task_start.data(), (np + 1) * 4, cudaMemcpyHostToDevice));
  }
  b->packet_widths = packet_widths;
  return KD_OK;
}

// The autotuner: every candidate launch shape runs the plan once to warm up
// and twice timed; the fastest is kept.  Then, width by width (2, 3, 8), the
// jobs with k <= 4 run as packet tasks instead of warp tasks, kept where that is
// faster.  Results are identical for all.
int tune(kd_batch* b, cudaStream_t st) {
  const int per_sm = resident_blocks_per_sm(b->qp.metric, b->layout[0].wide16);
  std::vector<unsigned> grids;
  for (int m : {1, 2, 4, 8})
    if (m <= per_sm) grids.push_back(static_cast<unsigned>(b->sms * m));
  grids.push_back(static_cast<unsigned>(b->sms * per_sm));
  std::sort(grids.begin(), grids.end());
  grids.erase(std::unique(grids.begin(), grids.end()), grids.end());
  cudaEvent_t e0, e1;
  KD_TRY_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail(cudaErrorMemoryAllocation, "cudaEventCreate");
  }
  float best = 1e30f;
  int rc = KD_OK;
  for (int table = 0; table < 2 && rc == KD_OK; ++table) {
    for (unsigned g : grids) {
      float t_min = 1e30f;
      for (int rep = 0; rep < 3 && rc == KD_OK; ++rep) {
        cudaEventRecord(e0, st);
        rc = enqueue_plan(b, st, false, g, table);
        cudaEventRecord(e1, st);
        if (rc == KD_OK) rc = finish_plan(b, st);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) t_min = std::min(t_min, ms);
      }
      if (rc != KD_OK) break;
      if (t_min < best) {
        best = t_min;
        b->blocks = g;
        b->table = table;
      }
    }
  }
  auto time_plan = [&](float* t_min) {
    *t_min = 1e30f;
    for (int rep = 0; rep < 3 && rc == KD_OK; ++rep) {
      cudaEventRecord(e0, st);
      rc = enqueue_plan(b, st, false, b->blocks, b->table);
      cudaEventRecord(e1, st);
      if (rc == KD_OK) rc = finish_plan(b, st);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) *t_min = std::min(*t_min, ms);
    }
  };
  // KD_BATCH_PACKET=all (or none) fixes that choice instead of timing it:
  // every width that has jobs with k <= 4 runs them as packet tasks (or none
  // does).  Results are the same either way; tests use it to cover both.
  const char* fix = std::getenv("KD_BATCH_PACKET");
  const int fixed = !fix ? -1 : (std::strcmp(fix, "all") == 0 ? 1 : (std::strcmp(fix, "none") == 0 ? 0 : -1));
  for (uint32_t w = 0; w < 3 && rc == KD_OK && fixed != 0; ++w) {
    bool present = false;
    for (const BatchJob& J : b->layout[0].table) present |= J.cls == w && J.a.k <= 4;
    if (!present) continue;
    const uint32_t keep = b->packet_widths;
    if ((rc = apply_layouts(b, keep | (1u << w)))) break;
    if (fixed == 1) continue;
    float t = 1e30f;
    time_plan(&t);
    if (rc != KD_OK) break;
    if (t < best) best = t;
    else rc = apply_layouts(b, keep);
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
  const int rc = enqueue_plan(b, b->capture_stream, false, b->blocks, b->table);
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

void release_plan(kd_batch* b) {
  if (!b) return;
  DeviceScope scope(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  delete b;  // frees buf
}

}  // namespace

// ===========================================================================
// The server behind the opaque kd_server* of the C ABI.
// ===========================================================================
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  uint32_t tree = 0;
  const double* q = nullptr;
  uint64_t nq = 0, k = 0;
  double* od = nullptr;
  int64_t* oi = nullptr;
  Clock::time_point t_submit;
  double latency = 0.0;
  uint64_t pieces_left = 0;  // pieces not completed yet
  int status = KD_OK;
  bool done = false;
};

// A request runs as pieces of at most the server's slice size (queries
// [q0, q0 + nq) of it), each one job of a batch: a large request's remaining
// pieces queue behind requests that arrive after it, so those need not wait
// for its whole scan.
struct Piece {
  Request* r;
  uint64_t q0, nq;
  double est_ns;  // estimated GPU time (the tree's calibrated cost per query)
};

// One batch in flight: device staging, batch buffers, pinned host tables.
struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  Buffers buf;
  double* in = nullptr;        // staged queries
  double* out_d = nullptr;     // staged distances
  int64_t* out_i = nullptr;    // staged indices
  uint32_t* status = nullptr;  // one word per job
  void* host = nullptr;        // pinned: tables, q_start, task_start, status words
  SideStreams side;
  std::vector<Piece> pieces;
  int error = KD_OK;
  std::string error_msg;
  bool busy = false;
};

}  // namespace

struct kd_server {
  int device = 0;
  int sms = 1;
  QueryParams qp{};
  std::vector<const kd_tree*> trees;
  uint64_t cap_q = 0, cap_in = 0, cap_out = 0, cap_jobs = 0, cap_bins = 0;
  Slot slots[2];
  std::mutex mu;
  std::condition_variable cv;  // queue, slots, completions
  uint64_t slice = 0;              // largest piece, in queries
  std::vector<double> ns_per_query;  // per tree: calibrated GPU time of one query (k = 16)
  std::deque<Piece> small_q;  // requests of one piece, arrival order
  std::deque<Piece> large_q;  // pieces of larger requests, arrival order
  std::deque<Slot*> inflight;
  std::unordered_map<uint64_t, Request*> reqs;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread scheduler, completer;
};

namespace {

constexpr uint64_t SERVER_JOBS = 4096;
// Work a batch takes on, and the size of a large request's pieces, in
// estimated GPU time (a tree's cost per query differs a hundredfold between a
// 3-wide tree of 1e5 points and a 16-wide one of 4e6): a batch holds every
// waiting small request and large pieces up to about SERVER_BATCH_NS, so a
// small request waits for at most about that much GPU work ahead of it.  The
// largest piece is SERVER_SLICE queries whatever its cost; a large piece that
// waited SERVER_AGE_NS goes into the next batch regardless.
constexpr uint64_t SERVER_SLICE = 16384;
constexpr double SERVER_BATCH_NS = 5.0e6;
constexpr double SERVER_PIECE_NS = 4.0e6;
constexpr uint64_t SERVER_MIN_PIECE = 4096;  // below this a batch cannot fill the GPU
constexpr double SERVER_AGE_NS = 20.0e6;

// Estimated GPU time of nq queries of k results on tree t (cost grows with k).
double piece_cost(const kd_server* s, uint32_t tree, uint64_t nq, uint64_t k) {
  return static_cast<double>(nq) * s->ns_per_query[tree] * (0.5 + static_cast<double>(k) / 32.0);
}

// Each tree's cost per query at a batch size that fills the GPU: one timed
// call of up to 32768 of its own points (rows spread over the tree) as
// queries, k = 16, after an untimed one.
int calibrate(kd_server* s) {
  s->ns_per_query.assign(s->trees.size(), 0.0);
  cudaStream_t st;
  KD_TRY_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = KD_OK;
  for (size_t i = 0; i < s->trees.size() && !rc; ++i) {
    const kd_tree* t = s->trees[i];
    const uint64_t m = std::min<uint64_t>(32768, t->n_points), k = std::min<uint64_t>(16, t->n_points);
    void* mem = nullptr;
    const uint64_t bytes = round256(m * t->ndim * 8) + 2 * round256(m * k * 8) + 256;
    if (dev_alloc(&mem, bytes, st) != cudaSuccess) {
      cudaGetLastError();
      rc = fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
      break;
    }
    double* q = static_cast<double*>(mem);
    double* od = reinterpret_cast<double*>(static_cast<char*>(mem) + round256(m * t->ndim * 8));
    int64_t* oi = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(od) + round256(m * k * 8));
    uint32_t* status = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(oi) + round256(m * k * 8));
    kd::k_sample_rows<<<static_cast<unsigned>((m * t->ndim + 255) / 256), 256, 0, st>>>(t->data, t->n_points,
                                                                                        t->ndim, m, q);
    QueryParams qp = s->qp;
    qp.k = k;
    cudaMemsetAsync(status, 0, 4, st);
    rc = query_on_device(t, q, m, qp, od, oi, st, status, nullptr);
    cudaEventRecord(e0, st);
    if (!rc) rc = query_on_device(t, q, m, qp, od, oi, st, status, nullptr);
    cudaEventRecord(e1, st);
    cudaFreeAsync(mem, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = cuda_fail(cudaGetLastError(), "calibration");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    s->ns_per_query[i] = std::max(1.0, static_cast<double>(ms) * 1e6 / static_cast<double>(m));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  return rc;
}

uint64_t host_bytes(const kd_server* s) {
  return round256(s->cap_jobs * sizeof(BatchJob)) + 2 * round256((s->cap_jobs + 1) * 4) +
         round256(s->cap_jobs * 4);
}

// Stage one batch of requests on slot `sl` (called without the lock).
int stage_batch(kd_server* s, Slot* sl) {
  DeviceScope scope(s->device);
  cudaStream_t st = sl->st;
  const size_t n = sl->pieces.size();
  std::vector<JobSpec> specs(n);
  uint64_t in_off = 0, out_off = 0;
  for (size_t j = 0; j < n; ++j) {
    const Piece& pc = sl->pieces[j];
    const Request* r = pc.r;
    const kd_tree* t = s->trees[r->tree];
    specs[j] = JobSpec{t, sl->in + in_off, pc.nq, r->k, sl->out_d + out_off, sl->out_i + out_off, sl->status + j};
    KD_TRY_CUDA(cudaMemcpyAsync(sl->in + in_off, r->q + pc.q0 * t->ndim, pc.nq * t->ndim * sizeof(double),
                                cudaMemcpyHostToDevice, st));
    in_off += pc.nq * t->ndim;
    out_off += pc.nq * r->k;
  }
  KD_TRY_CUDA(cudaMemsetAsync(sl->status, 0, n * sizeof(uint32_t), st));
  Layout L;
  make_layout(specs, s->qp, true, sl->buf.order, sl->buf.rerun_count, sl->buf.rerun_list, &L);
  char* h = static_cast<char*>(sl->host);
  BatchJob* h_jobs = reinterpret_cast<BatchJob*>(h);
  uint32_t* h_qs = reinterpret_cast<uint32_t*>(h + round256(s->cap_jobs * sizeof(BatchJob)));
  uint32_t* h_ts = h_qs + round256((s->cap_jobs + 1) * 4) / 4;
  const size_t np = L.packet.size();
  if (np) {
    std::memcpy(h_jobs, L.table.data(), np * sizeof(BatchJob));
    std::memcpy(h_qs, L.q_start.data(), (np + 1) * 4);
    std::memcpy(h_ts, L.task_start.data(), (np + 1) * 4);
    KD_TRY_CUDA(cudaMemcpyAsync(sl->buf.jobs[0], h_jobs, np * sizeof(BatchJob), cudaMemcpyHostToDevice, st));
    KD_TRY_CUDA(cudaMemcpyAsync(sl->buf.q_start, h_qs, (np + 1) * 4, cudaMemcpyHostToDevice, st));
    KD_TRY_CUDA(cudaMemcpyAsync(sl->buf.task_start, h_ts, (np + 1) * 4, cudaMemcpyHostToDevice, st));
  }
  // the per-job launches fork first, so they run beside the fused kernel
  int rc = enqueue_others(specs, L.other, s->qp, sl->side, st, nullptr, {}, nullptr);
  if (rc) return rc;
  if (np) {
    const unsigned blocks = static_cast<unsigned>(s->sms * resident_blocks_per_sm(s->qp.metric, L.wide16));
    rc = enqueue_packet(L, sl->buf, 0, s->qp.metric, blocks, st);
  }
  join_others(sl->side, L.other.size(), st);
  if (rc) return rc;
  KD_TRY_CUDA(cudaEventRecord(sl->done, st));
  return KD_OK;
}

// Results of a computed batch into the requests' host buffers (issued by the
// completion thread, so a pageable destination never blocks the scheduler).
int deliver_batch(Slot* sl, uint32_t* h_status) {
  cudaStream_t st = sl->st;
  uint64_t out_off = 0;
  for (const Piece& pc : sl->pieces) {
    const Request* r = pc.r;
    const uint64_t n = pc.nq * r->k;
    KD_TRY_CUDA(cudaMemcpyAsync(r->od + pc.q0 * r->k, sl->out_d + out_off, n * sizeof(double), cudaMemcpyDeviceToHost,
                                st));
    KD_TRY_CUDA(cudaMemcpyAsync(r->oi + pc.q0 * r->k, sl->out_i + out_off, n * sizeof(int64_t),
                                cudaMemcpyDeviceToHost, st));
    out_off += n;
  }
  KD_TRY_CUDA(cudaMemcpyAsync(h_status, sl->status, sl->pieces.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  return KD_OK;
}

void scheduler_loop(kd_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    Slot* free_slot = nullptr;
    auto empty = [&] { return s->small_q.empty() && s->large_q.empty(); };
    s->cv.wait(lk, [&] {
      free_slot = !s->slots[0].busy ? &s->slots[0] : (!s->slots[1].busy ? &s->slots[1] : nullptr);
      return (s->stop && empty()) || (free_slot && !empty());
    });
    if (empty()) return;  // stopping, nothing left
    // continuous batching: every waiting single-piece request that fits, in
    // arrival order, then pieces of larger requests while the batch's estimated
    // GPU time stays within SERVER_BATCH_NS (at least one piece when no small
    // request waits, or when the oldest piece waited SERVER_AGE_NS)
    Slot* sl = free_slot;
    sl->busy = true;
    sl->pieces.clear();
    uint64_t q = 0, in = 0, out = 0, bins = 0;
    double cost = 0.0;
    int n_large = 0;
    const Clock::time_point now = Clock::now();
    auto take = [&](std::deque<Piece>& from, bool budget) {
      while (!from.empty() && sl->pieces.size() < s->cap_jobs) {
        const Piece pc = from.front();
        const kd_tree* t = s->trees[pc.r->tree];
        const uint64_t nb = pc.nq >= SORT_MIN_QUERIES ? t->n_nodes : 1;
        if (!sl->pieces.empty() && (q + pc.nq > s->cap_q || in + pc.nq * t->ndim > s->cap_in ||
                                    out + pc.nq * pc.r->k > s->cap_out || bins + nb > s->cap_bins))
          return;
        if (budget) {
          const bool first = n_large == 0;
          const bool aged = std::chrono::duration<double, std::nano>(now - pc.r->t_submit).count() > SERVER_AGE_NS;
          const bool fits = cost + pc.est_ns <= SERVER_BATCH_NS;
          if (!(fits || (first && (sl->pieces.empty() || aged)))) return;
          ++n_large;
        }
        q += pc.nq;
        in += pc.nq * t->ndim;
        out += pc.nq * pc.r->k;
        bins += nb;
        cost += pc.est_ns;
        sl->pieces.push_back(pc);
        from.pop_front();
      }
    };
    take(s->small_q, false);
    take(s->large_q, true);
    lk.unlock();
    const int rc = stage_batch(s, sl);
    lk.lock();
    sl->error = rc;
    if (rc) sl->error_msg = "batch failed: status " + std::to_string(rc);
    s->inflight.push_back(sl);
    s->cv.notify_all();
  }
}

void completer_loop(kd_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv.wait(lk, [&] {
      return !s->inflight.empty() ||
             (s->stop && s->small_q.empty() && s->large_q.empty() && !s->slots[0].busy && !s->slots[1].busy);
    });
    if (s->inflight.empty()) return;
    Slot* sl = s->inflight.front();
    lk.unlock();
    int err = sl->error;
    uint32_t* h_status = reinterpret_cast<uint32_t*>(static_cast<char*>(sl->host) +
                                                     round256(s->cap_jobs * sizeof(BatchJob)) +
                                                     2 * round256((s->cap_jobs + 1) * 4));
    {
      DeviceScope scope(s->device);
      if (!err) {
        cudaError_t e = cudaEventSynchronize(sl->done);
        err = e != cudaSuccess ? cuda_fail(e, "cudaEventSynchronize") : deliver_batch(sl, h_status);
      }
      if (err) cudaStreamSynchronize(sl->st);  // let whatever was staged drain
    }
    const Clock::time_point now = Clock::now();
    lk.lock();
    for (size_t j = 0; j < sl->pieces.size(); ++j) {
      Request* r = sl->pieces[j].r;
      const int st = err ? err : (h_status[j] ? KD_ERR_NONFINITE_DATA : KD_OK);
      if (st && (!r->status || st != KD_ERR_NONFINITE_DATA)) r->status = st;  // device failures outrank
      if (--r->pieces_left == 0) {
        r->latency = std::chrono::duration<double>(now - r->t_submit).count();
        r->done = true;
      }
    }
    sl->pieces.clear();
    sl->busy = false;
    s->inflight.pop_front();
    s->cv.notify_all();
  }
}

void release_server(kd_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->scheduler.joinable()) s->scheduler.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
  }
  s->cv.notify_all();
  if (s->completer.joinable()) s->completer.join();
  DeviceScope scope(s->device);
  for (Slot& sl : s->slots) {
    if (sl.st) cudaStreamSynchronize(sl.st);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.st) cudaStreamDestroy(sl.st);
    if (sl.host) cudaFreeHost(sl.host);
  }
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Batch plans
// ---------------------------------------------------------------------------
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
  for (uint64_t j = 0; j < n_jobs; ++j) {
    const kd_batch_job& J = jobs[j];
    if ((rc = job_error(J.tree, J.n_queries, J.k, J.d_queries, J.d_out_distances, J.d_out_indices, dev,
                        "job " + std::to_string(j))))
      return rc;
  }
  kd_batch* b = new (std::nothrow) kd_batch();
  if (!b) return fail(KD_ERR_OUT_OF_MEMORY, "host allocation failed");
  b->device = dev;
  b->qp = qp;
  cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  uint64_t total_q = 0, scratch_bytes = 0, bins = 0;
  for (uint64_t j = 0; j < n_jobs; ++j) {
    const kd_batch_job& J = jobs[j];
    b->specs.push_back(JobSpec{J.tree, J.d_queries, J.n_queries, J.k, J.d_out_distances, J.d_out_indices, nullptr});
    total_q += J.n_queries;
    bins += J.tree->n_nodes;
    scratch_bytes += round256(query_scratch_bytes(J.n_queries, J.tree->ndim));
  }
  if (total_q >= 0xffffffffull) {
    delete b;
    return fail(KD_ERR_INVALID_ARGUMENT, "a batch holds at most 2^32 - 1 queries");
  }
  char* extra = nullptr;
  const uint64_t counter_bytes = round256(n_jobs * sizeof(uint32_t));
  if ((rc = alloc_buffers(&b->buf, n_jobs, total_q, bins, 256 + counter_bytes + scratch_bytes, &extra))) {
    delete b;
    return rc;
  }
  b->status = reinterpret_cast<uint32_t*>(extra);
  b->counters = reinterpret_cast<uint32_t*>(extra + 256);
  b->scratch = reinterpret_cast<unsigned char*>(extra + 256 + counter_bytes);
  for (JobSpec& J : b->specs) J.status = b->status;
  make_layout(b->specs, qp, true, b->buf.order, b->buf.rerun_count, b->buf.rerun_list, &b->layout[0]);
  make_layout(b->specs, qp, false, b->buf.order, b->buf.rerun_count, b->buf.rerun_list, &b->layout[1]);
  uint64_t off = 0;
  for (uint32_t j : b->layout[0].other) {
    b->scratch_off.push_back(off);
    off += round256(query_scratch_bytes(b->specs[j].nq, b->specs[j].tree->ndim));
  }
  const Layout& L = b->layout[0];
  const size_t np = L.packet.size();
  cudaError_t e = cudaSuccess;
  if (np) {
    e = cudaMemcpy(b->buf.jobs[0], b->layout[0].table.data(), np * sizeof(BatchJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->buf.jobs[1], b->layout[1].table.data(), np * sizeof(BatchJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->buf.q_start, L.q_start.data(), (np + 1) * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->buf.task_start, L.task_start.data(), (np + 1) * 4, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    release_plan(b);
    return cuda_fail(e, "cudaMemcpy");
  }
  if ((rc = b->side.create())) {
    release_plan(b);
    return rc;
  }
  b->blocks = static_cast<unsigned>(b->sms * resident_blocks_per_sm(qp.metric, b->layout[0].wide16));
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
  } else if ((rc = enqueue_plan(b, st, mode == KD_BATCH_PER_JOB, b->blocks, b->table))) {
    return rc;
  }
  return finish_plan(b, st);
}

int kd_batch_run(kd_batch* b, void* stream) { return kd_batch_run_mode(b, stream, KD_BATCH_GRAPH); }

int kd_batch_choice(const kd_batch* b, unsigned* blocks, int* sorted, unsigned* packet_widths) {
  if (!b) return fail(KD_ERR_INVALID_ARGUMENT, "batch is NULL");
  if (blocks) *blocks = b->blocks;
  if (sorted) *sorted = b->table == 0;
  if (packet_widths) *packet_widths = b->packet_widths;
  return KD_OK;
}

void kd_batch_free(kd_batch* b) { release_plan(b); }

// ---------------------------------------------------------------------------
// Server
// ---------------------------------------------------------------------------
int kd_server_create(const kd_tree* const* trees, uint64_t n_trees, double p, int has_max_distance,
                     double max_distance, double eps, uint64_t max_batch_queries, kd_server** out) {
  if (!out) return fail(KD_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!trees || n_trees == 0) return fail(KD_ERR_INVALID_ARGUMENT, "a server needs at least one tree");
  if (n_trees >= 0xffffffffull) return fail(KD_ERR_INVALID_ARGUMENT, "too many trees");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(KD_ERR_NO_DEVICE, "no CUDA device is visible; the GB300 engine has no CPU fallback");
  }
  QueryParams qp{};
  std::string msg;
  int rc = validate_scalars(1, p, has_max_distance, max_distance, eps, &qp, &msg);
  if (rc) return fail(rc, msg);
  uint64_t dmax = 1, nodes = 0, nodes_max = 0;
  for (uint64_t i = 0; i < n_trees; ++i) {
    if (!trees[i]) return fail(KD_ERR_INVALID_ARGUMENT, "tree " + std::to_string(i) + " is NULL");
    if (trees[i]->device != dev)
      return fail(KD_ERR_INVALID_ARGUMENT, "tree " + std::to_string(i) + " lives on another device");
    dmax = std::max(dmax, trees[i]->ndim);
    nodes += trees[i]->n_nodes;
    nodes_max = std::max(nodes_max, trees[i]->n_nodes);
  }
  kd_server* s = new (std::nothrow) kd_server();
  if (!s) return fail(KD_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->device = dev;
  s->qp = qp;
  s->trees.assign(trees, trees + n_trees);
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
  // Batch capacity: the requested number of queries, or what a quarter of the
  // free device memory holds (two slots) at the widest tree and 64 results per
  // query, at most 2^20 queries.
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const uint64_t per_q = dmax * 8 + 64 * 16 + 16;
  uint64_t cap = max_batch_queries ? max_batch_queries : std::min<uint64_t>(1ull << 20, free_b / 8 / per_q);
  cap = std::max<uint64_t>(cap, 1024);
  s->cap_q = cap;
  s->cap_in = cap * dmax;
  s->cap_out = cap * 64;
  s->cap_jobs = SERVER_JOBS;
  s->cap_bins = std::max(2 * nodes, nodes_max + SERVER_JOBS);
  s->slice = std::min<uint64_t>(SERVER_SLICE, cap);
  for (Slot& sl : s->slots) {
    char* extra = nullptr;
    const uint64_t extra_b = round256(s->cap_in * 8) + round256(s->cap_out * 8) * 2 + round256(SERVER_JOBS * 4);
    if ((rc = alloc_buffers(&sl.buf, SERVER_JOBS, cap, s->cap_bins, extra_b, &extra))) {
      release_server(s);
      return rc;
    }
    sl.in = reinterpret_cast<double*>(extra);
    extra += round256(s->cap_in * 8);
    sl.out_d = reinterpret_cast<double*>(extra);
    extra += round256(s->cap_out * 8);
    sl.out_i = reinterpret_cast<int64_t*>(extra);
    extra += round256(s->cap_out * 8);
    sl.status = reinterpret_cast<uint32_t*>(extra);
    if ((rc = sl.side.create())) {
      release_server(s);
      return rc;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc(&sl.host, host_bytes(s) + round256(SERVER_JOBS * 4), cudaHostAllocDefault);
    if (e != cudaSuccess) {
      sl.host = nullptr;
      release_server(s);
      return cuda_fail(e, "server set-up");
    }
  }
  if ((rc = calibrate(s))) {
    release_server(s);
    return rc;
  }
  try {
    s->scheduler = std::thread(scheduler_loop, s);
    s->completer = std::thread(completer_loop, s);
  } catch (...) {
    release_server(s);
    return fail(KD_ERR_OUT_OF_MEMORY, "could not start the server threads");
  }
  *out = s;
  return KD_OK;
}

int kd_server_submit(kd_server* s, uint64_t tree, const double* queries, uint64_t n_queries, uint64_t k,
                     double* out_distances, int64_t* out_indices, uint64_t* ticket) {
  if (!s || !ticket) return fail(KD_ERR_INVALID_ARGUMENT, "server or ticket is NULL");
  if (tree >= s->trees.size()) return fail(KD_ERR_INVALID_ARGUMENT, "no tree " + std::to_string(tree));
  const kd_tree* t = s->trees[tree];
  int rc = job_error(t, n_queries, k, queries, out_distances, out_indices, s->device, "request");
  if (rc) return rc;
  // a piece must fit one batch: about SERVER_PIECE_NS of estimated GPU time
  // (256 to SERVER_SLICE queries), fewer for wide rows or large k
  const double per_q = piece_cost(s, static_cast<uint32_t>(tree), 1, k);
  const uint64_t by_cost = std::max<uint64_t>(SERVER_MIN_PIECE, static_cast<uint64_t>(SERVER_PIECE_NS / per_q));
  const uint64_t piece = std::min({s->slice, by_cost, s->cap_in / t->ndim, s->cap_out / k});
  if (piece == 0)
    return fail(KD_ERR_INVALID_ARGUMENT, "k = " + std::to_string(k) + " exceeds the server's batch capacity (" +
                                             std::to_string(s->cap_out) + " results)");
  Request* r = new (std::nothrow) Request();
  if (!r) return fail(KD_ERR_OUT_OF_MEMORY, "host allocation failed");
  r->tree = static_cast<uint32_t>(tree);
  r->q = queries;
  r->nq = n_queries;
  r->k = k;
  r->od = out_distances;
  r->oi = out_indices;
  r->t_submit = Clock::now();
  r->pieces_left = (n_queries + piece - 1) / piece;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      delete r;
      return fail(KD_ERR_INVALID_ARGUMENT, "server is stopping");
    }
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    if (r->pieces_left == 1) {
      s->small_q.push_back(Piece{r, 0, n_queries, per_q * static_cast<double>(n_queries)});
    } else {
      for (uint64_t q0 = 0; q0 < n_queries; q0 += piece) {
        const uint64_t nq = std::min(piece, n_queries - q0);
        s->large_q.push_back(Piece{r, q0, nq, per_q * static_cast<double>(nq)});
      }
    }
  }
  s->cv.notify_all();
  *ticket = r->ticket;
  return KD_OK;
}

int kd_server_wait(kd_server* s, uint64_t ticket, double* latency_s) {
  if (!s) return fail(KD_ERR_INVALID_ARGUMENT, "server is NULL");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(KD_ERR_INVALID_ARGUMENT, "unknown ticket " + std::to_string(ticket));
  Request* r = it->second;
  s->cv.wait(lk, [&] { return r->done; });
  const int st = r->status;
  if (latency_s) *latency_s = r->latency;
  s->reqs.erase(it);
  delete r;
  lk.unlock();
  if (st == KD_ERR_NONFINITE_DATA) return fail(st, "all coordinates must be finite");
  if (st) return fail(st, "the batch holding this request failed on the device");
  return KD_OK;
}

void kd_server_free(kd_server* s) { release_server(s); }

}  // extern "C"
