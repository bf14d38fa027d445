// kd_api.cu -- the C ABI of libkdtree_gb300.so (include/kdtree_gb300.h).
//
// Host-side validation and error reporting restate the reference's boundary:
// src/build.rs:25-43 (build), src/query.rs:38-62 (query), src/metric.rs:45-59
// (metric), with the messages of src/error.rs:18-51.  The compute runs on the
// GPU; there is no CPU fallback -- without a device every call fails with
// KD_ERR_NO_DEVICE.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "kd_internal.hpp"

namespace kd {

namespace {
thread_local std::string g_last_error;

// Rust's `{}` Display for f64: the shortest digits that round-trip, written
// positionally (no exponent), "inf", "-inf", "NaN", "-0" for negative zero.
std::string rust_f64(double v) {
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
  std::string sign = std::signbit(v) ? "-" : "";
  double a = std::fabs(v);
  if (a == 0.0) return sign + "0";
  char buf[64];
  int prec = 0;
  for (prec = 0; prec < 17; ++prec) {
    std::snprintf(buf, sizeof buf, "%.*e", prec, a);
    if (std::strtod(buf, nullptr) == a) break;
  }
  std::string s(buf);
  size_t epos = s.find('e');
  int exp10 = std::atoi(s.c_str() + epos + 1);
  std::string digits;
  for (size_t i = 0; i < epos; ++i)
    if (s[i] != '.') digits.push_back(s[i]);
  while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
  std::string out;
  if (exp10 >= 0) {
    if (static_cast<int>(digits.size()) <= exp10 + 1) {
      out = digits + std::string(exp10 + 1 - digits.size(), '0');
    } else {
      out = digits.substr(0, exp10 + 1) + "." + digits.substr(exp10 + 1);
    }
  } else {
    out = "0." + std::string(-exp10 - 1, '0') + digits;
  }
  return sign + out;
}

int ensure_device(int* dev) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(KD_ERR_NO_DEVICE, "no CUDA device is visible; the GB300 engine has no CPU fallback");
  }
  KD_TRY_CUDA(cudaGetDevice(dev));
  return KD_OK;
}

cudaStream_t thread_stream() {
  thread_local cudaStream_t s = nullptr;
  thread_local int s_dev = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (!s || s_dev != dev) {
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    s_dev = dev;
  }
  return s;
}

struct DevicePin {
  int prev = -1;
  explicit DevicePin(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DevicePin() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

int validate_build(uint64_t n_values, uint64_t ndim, uint64_t leafsize, uint64_t* n_points) {
  if (leafsize == 0) return fail(KD_ERR_INVALID_LEAFSIZE, "leafsize must be greater than zero");
  if (ndim == 0 || n_values == 0) return fail(KD_ERR_EMPTY_DATA, "data must contain at least one point");
  if (n_values % ndim) return fail(KD_ERR_INVALID_SHAPE, "data length must be a multiple of ndim");
  uint64_t n = n_values / ndim;
  if (n > 0xffffffffull)
    return fail(KD_ERR_TOO_MANY_POINTS, "n_points must fit in a 32-bit index, got " + std::to_string(n));
  uint64_t nodes = count_nodes(n, leafsize);
  if (nodes > 0xffffffffull)
    return fail(KD_ERR_TOO_MANY_NODES, "tree would need " + std::to_string(nodes) +
                                           " nodes, which exceeds the 32-bit node index; increase leafsize");
  *n_points = n;
  return KD_OK;
}

__global__ void k_original(const double* data, const uint32_t* idx, double* out, uint64_t n, uint64_t d) {
  uint64_t f = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (f >= n * d) return;
  uint64_t pos = f / d, j = f - pos * d;
  out[static_cast<uint64_t>(idx[pos]) * d + j] = data[f];
}

__global__ void k_export_nodes(const DNode* nodes, uint64_t n_nodes, uint32_t* words, double* split) {
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i >= n_nodes) return;
  DNode nd = nodes[i];
  if (nd.meta & KD_NODE_LEAF) {
    uint64_t se = static_cast<uint64_t>(__double_as_longlong(nd.split));
    if (words) {
      words[4 * i] = 1;
      words[4 * i + 1] = static_cast<uint32_t>(se);
      words[4 * i + 2] = static_cast<uint32_t>(se >> 32);
      words[4 * i + 3] = 0;
    }
    if (split) split[i] = 0.0;
  } else {
    if (words) {
      words[4 * i] = 0;
      words[4 * i + 1] = static_cast<uint32_t>(i + 1);
      words[4 * i + 2] = nd.right;
      words[4 * i + 3] = (nd.meta & KD_NODE_DIM_MASK) | ((nd.meta & KD_NODE_BOX_ORDER) ? 0x80000000u : 0u);
    }
    if (split) split[i] = nd.split;
  }
}

void free_tree(kd_tree* t) {
  if (!t) return;
  DevicePin pin(t->device);
  if (t->block) {
    // calls on other streams may still read the tree: let them finish, then
    // return the block to the pool
    cudaDeviceSynchronize();
    cudaFreeAsync(t->block, thread_stream());
  }
  cudaFree(t->tc_points);
  cudaFree(t->tc_w);
  cudaFree(t->tc_v);
  cudaFree(t->tc_centre);
  cudaFree(t->tc_tbox);
  if (t->tc_ready) cudaEventDestroy(t->tc_ready);
  delete t;
}

struct DevMem {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~DevMem() {
    if (p) cudaFreeAsync(p, st);
  }
  int alloc(size_t bytes, cudaStream_t s) {
    st = s;
    cudaError_t e = dev_alloc(&p, bytes, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(KD_ERR_OUT_OF_MEMORY, "device allocation failed");
    }
    return KD_OK;
  }
};

// Error carried by a query's device status word: bit 0 a non-finite query
// coordinate, bit 1 a tensor-core pipeline wait that ran out.
int status_word(uint32_t h) {
  if (h & 2u) return fail(KD_ERR_CUDA, "the tensor-core pipeline timed out waiting on a barrier");
  if (h) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
  return KD_OK;
}

// Device-accessible address of page-locked (pinned) host memory, or nullptr
// for pageable memory.
void* mapped_host(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int query_common(const kd_tree* t, const double* queries, bool on_device, uint64_t n_values, uint64_t k,
                 double p, int has_max, double max_distance, double eps, double* out_d, int64_t* out_i,
                 cudaStream_t st, int path = PATH_AUTO, unsigned long long* d_survivors = nullptr) {
  if (!t) return fail(KD_ERR_INVALID_ARGUMENT, "tree is NULL");
  if (k == 0) return fail(KD_ERR_INVALID_K, "k must be greater than zero");
  if (n_values == 0 || n_values % t->ndim)
    return fail(KD_ERR_INVALID_SHAPE, "queries must be a contiguous row-major matrix");
  if (!queries || !out_d || !out_i) return fail(KD_ERR_INVALID_ARGUMENT, "NULL buffer");
  QueryParams qp{};
  std::string msg;
  int scalar = validate_scalars(k, p, has_max, max_distance, eps, &qp, &msg);
  const uint64_t nq = n_values / t->ndim;
  DevicePin pin(t->device);
  DevMem status;
  int rc;
  if ((rc = status.alloc(sizeof(uint32_t), st))) return rc;
  KD_TRY_CUDA(cudaMemsetAsync(status.p, 0, sizeof(uint32_t), st));
  if (scalar != KD_OK) {
    // Error path: a non-finite query outranks the scalar errors (query.rs:46-48).
    bool nonfinite = false;
    if (!on_device) {
      for (uint64_t i = 0; i < n_values && !nonfinite; ++i) nonfinite = !std::isfinite(queries[i]);
    } else {
      k_check_finite<<<static_cast<unsigned>((n_values + 255) / 256), 256, 0, st>>>(
          queries, n_values, static_cast<uint32_t*>(status.p));
      uint32_t h = 0;
      KD_TRY_CUDA(cudaMemcpyAsync(&h, status.p, sizeof h, cudaMemcpyDeviceToHost, st));
      KD_TRY_CUDA(cudaStreamSynchronize(st));
      nonfinite = h != 0;
    }
    if (nonfinite) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
    return fail(scalar, msg);
  }
  if (k > (~0ull / sizeof(double)) / nq) return fail(KD_ERR_OUT_OF_MEMORY, "output would not fit in memory");
  qp.path = path;
  if (on_device) {
    if ((rc = query_on_device(t, queries, nq, qp, out_d, out_i, st, static_cast<uint32_t*>(status.p), d_survivors)))
      return rc;
    uint32_t h = 0;
    KD_TRY_CUDA(cudaMemcpyAsync(&h, status.p, sizeof h, cudaMemcpyDeviceToHost, st));
    KD_TRY_CUDA(cudaStreamSynchronize(st));
    return status_word(h);
  }
  // Host buffers: the queries are uploaded.  Page-locked outputs that the
  // chosen kernel writes as whole rows receive the results directly over the
  // host link while the kernel runs (the transfer overlaps the compute);
  // otherwise the results are staged in device memory and downloaded.
  DevMem mq, md, mi;
  if ((rc = mq.alloc(n_values * sizeof(double), st))) return rc;
  double* dq = static_cast<double*>(mq.p);
  uint32_t* ds = static_cast<uint32_t*>(status.p);
  double* dd = static_cast<double*>(mapped_host(out_d));
  int64_t* di = static_cast<int64_t*>(mapped_host(out_i));
  const bool direct = dd && di && writes_whole_rows(t, qp);
  if (!direct) {
    if ((rc = md.alloc(nq * k * sizeof(double), st)) || (rc = mi.alloc(nq * k * sizeof(int64_t), st))) return rc;
    dd = static_cast<double*>(md.p);
    di = static_cast<int64_t*>(mi.p);
  }
  KD_TRY_CUDA(cudaMemcpyAsync(dq, queries, n_values * sizeof(double), cudaMemcpyHostToDevice, st));
  if ((rc = query_on_device(t, dq, nq, qp, dd, di, st, ds, d_survivors))) return rc;
  if (!direct) {
    KD_TRY_CUDA(cudaMemcpyAsync(out_d, dd, nq * k * sizeof(double), cudaMemcpyDeviceToHost, st));
    KD_TRY_CUDA(cudaMemcpyAsync(out_i, di, nq * k * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  }
  uint32_t h = 0;
  KD_TRY_CUDA(cudaMemcpyAsync(&h, status.p, sizeof h, cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  return status_word(h);
}

}  // namespace

// Scalar validation of Tree::query after the shape and finiteness checks
// (query.rs:49-62, metric.rs:45-59).  Returns KD_OK and fills qp, or the status
// with its message staged in *msg (the caller decides which error wins).
int validate_scalars(uint64_t k, double p, int has_max, double max_distance, double eps, QueryParams* qp,
                     std::string* msg) {
  if (!std::isfinite(eps) || eps < 0.0) {
    *msg = "eps must be finite and non-negative, got " + rust_f64(eps);
    return KD_ERR_INVALID_EPS;
  }
  double md = has_max ? max_distance : INFINITY;
  if (std::isnan(md) || md < 0.0) {
    *msg = "max_distance must be finite and non-negative, or infinity, got " + rust_f64(md);
    return KD_ERR_INVALID_MAX_DISTANCE;
  }
  int metric;
  if (std::isinf(p) && p > 0) {
    metric = M_LINF;
  } else if (!std::isfinite(p) || p < 1.0) {
    *msg = "p must be finite and >= 1, or infinity, got " + rust_f64(p);
    return KD_ERR_INVALID_METRIC;
  } else if (p == 1.0) {
    metric = M_L1;
  } else if (p == 2.0) {
    metric = M_L2;
  } else {
    metric = M_LP;
  }
  auto reduce = [&](double x) {
    if (metric == M_L2) return x * x;
    if (metric == M_LP) return std::pow(x, p);
    return x;
  };
  qp->metric = metric;
  qp->p = p;
  qp->cutoff = reduce(md);
  if (qp->cutoff == 0.0) qp->cutoff = 0.0;  // -0 -> +0: compares equal, sorts as bits
  qp->eps_factor = reduce(1.0 + eps);
  qp->k = k;
  return KD_OK;
}

__global__ void k_check_finite(const double* v, uint64_t n, uint32_t* status) {
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i < n && !isfinite(v[i])) atomicOr(status, 1u);
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int cuda_fail(cudaError_t err, const char* what) {
  std::string m = std::string("CUDA error: ") + cudaGetErrorString(err) + " (" + what + ")";
  cudaGetLastError();
  return fail(err == cudaErrorMemoryAllocation ? KD_ERR_OUT_OF_MEMORY : KD_ERR_CUDA, m);
}

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t st) {
  constexpr int MAX_DEV = 64;
  static std::mutex mu;
  static cudaMemPool_t pools[MAX_DEV] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEV) return cudaMallocAsync(p, bytes, st);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t fresh;
      if ((e = cudaMemPoolCreate(&fresh, &props)) != cudaSuccess) return e;
      uint64_t keep = KD_POOL_KEEP_BYTES;
      cudaMemPoolSetAttribute(fresh, cudaMemPoolAttrReleaseThreshold, &keep);
      pools[dev] = fresh;
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes ? bytes : 1, pool, st);
}

}  // namespace kd

using namespace kd;

extern "C" {

int kd_build(const double* data, uint64_t n_values, uint64_t ndim, uint64_t leafsize, int parallel,
             kd_tree** out) {
  (void)parallel;
  if (!out) return fail(KD_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  uint64_t n = 0;
  int rc = validate_build(n_values, ndim, leafsize, &n);
  if (rc) return rc;
  if (!data) return fail(KD_ERR_INVALID_ARGUMENT, "data is NULL");
  int dev = 0;
  if ((rc = ensure_device(&dev))) return rc;
  cudaStream_t st = thread_stream();
  void* src = nullptr;
  KD_TRY_CUDA(dev_alloc(&src, n_values * sizeof(double), st));
  cudaError_t ce = cudaMemcpyAsync(src, data, n_values * sizeof(double), cudaMemcpyHostToDevice, st);
  if (ce != cudaSuccess) {
    cudaFreeAsync(src, st);
    return cuda_fail(ce, "cudaMemcpyAsync");
  }
  kd_tree* t = new (std::nothrow) kd_tree();
  if (!t) {
    cudaFreeAsync(src, st);
    return fail(KD_ERR_OUT_OF_MEMORY, "host allocation failed");
  }
  t->device = dev;
  rc = build_on_device(static_cast<const double*>(src), n, ndim, leafsize, st, t);
  cudaFreeAsync(src, st);
  cudaStreamSynchronize(st);
  if (rc) {
    free_tree(t);
    return rc;
  }
  noalloc_prepare(dev);
  *out = t;
  return KD_OK;
}

int kd_build_device(const double* d_data, uint64_t n_values, uint64_t ndim, uint64_t leafsize, void* stream,
                    kd_tree** out) {
  if (!out) return fail(KD_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  uint64_t n = 0;
  int rc = validate_build(n_values, ndim, leafsize, &n);
  if (rc) return rc;
  if (!d_data) return fail(KD_ERR_INVALID_ARGUMENT, "data is NULL");
  int dev = 0;
  if ((rc = ensure_device(&dev))) return rc;
  kd_tree* t = new (std::nothrow) kd_tree();
  if (!t) return fail(KD_ERR_OUT_OF_MEMORY, "host allocation failed");
  t->device = dev;
  rc = build_on_device(d_data, n, ndim, leafsize, static_cast<cudaStream_t>(stream), t);
  if (rc) {
    free_tree(t);
    return rc;
  }
  noalloc_prepare(dev);
  *out = t;
  return KD_OK;
}

void kd_free(kd_tree* tree) { free_tree(tree); }

int kd_query(const kd_tree* tree, const double* queries, uint64_t n_values, uint64_t k, double p,
             int has_max_distance, double max_distance, double eps, int parallel, double* out_distances,
             int64_t* out_indices) {
  (void)parallel;
  if (!tree) return fail(KD_ERR_INVALID_ARGUMENT, "tree is NULL");
  DevicePin pin(tree->device);
  return query_common(tree, queries, false, n_values, k, p, has_max_distance, max_distance, eps, out_distances,
                      out_indices, thread_stream());
}

int kd_query_device(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k, double p,
                    int has_max_distance, double max_distance, double eps, double* d_out_distances,
                    int64_t* d_out_indices, void* stream) {
  return query_common(tree, d_queries, true, n_values, k, p, has_max_distance, max_distance, eps,
                      d_out_distances, d_out_indices, static_cast<cudaStream_t>(stream));
}

int kd_query_async(const kd_tree* t, const double* d_queries, uint64_t n_values, uint64_t k, double p,
                   int has_max_distance, double max_distance, double eps, double* d_out_distances,
                   int64_t* d_out_indices, uint32_t* d_status, void* stream) {
  if (!t) return fail(KD_ERR_INVALID_ARGUMENT, "tree is NULL");
  if (k == 0) return fail(KD_ERR_INVALID_K, "k must be greater than zero");
  if (n_values == 0 || n_values % t->ndim)
    return fail(KD_ERR_INVALID_SHAPE, "queries must be a contiguous row-major matrix");
  if (!d_queries || !d_out_distances || !d_out_indices || !d_status)
    return fail(KD_ERR_INVALID_ARGUMENT, "NULL buffer");
  QueryParams qp{};
  std::string msg;
  const int scalar = validate_scalars(k, p, has_max_distance, max_distance, eps, &qp, &msg);
  const uint64_t nq = n_values / t->ndim;
  DevicePin pin(t->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  KD_TRY_CUDA(cudaMemsetAsync(d_status, 0, sizeof(uint32_t), st));
  if (scalar != KD_OK) {
    // The reference reports a non-finite query before these (query.rs:46-48):
    // its check still runs, into bit 0 of *d_status.
    k_check_finite<<<static_cast<unsigned>((n_values + 255) / 256), 256, 0, st>>>(d_queries, n_values, d_status);
    KD_TRY_CUDA(cudaGetLastError());
    return fail(scalar, msg);
  }
  if (k > (~0ull / sizeof(double)) / nq) return fail(KD_ERR_OUT_OF_MEMORY, "output would not fit in memory");
  qp.no_sync = true;
  return query_on_device(t, d_queries, nq, qp, d_out_distances, d_out_indices, st, d_status, nullptr);
}

int kd_query_device_path(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k, double p,
                         int has_max_distance, double max_distance, double eps, double* d_out_distances,
                         int64_t* d_out_indices, void* stream, int path, unsigned long long* d_survivors) {
  if (path < KD_PATH_AUTO || path > KD_PATH_WARP) return fail(KD_ERR_INVALID_ARGUMENT, "unknown query path");
  return query_common(tree, d_queries, true, n_values, k, p, has_max_distance, max_distance, eps, d_out_distances,
                      d_out_indices, static_cast<cudaStream_t>(stream), path, d_survivors);
}

uint64_t kd_ndim(const kd_tree* t) { return t ? t->ndim : 0; }
uint64_t kd_n_points(const kd_tree* t) { return t ? t->n_points : 0; }
uint64_t kd_leafsize(const kd_tree* t) { return t ? t->leafsize : 0; }
uint64_t kd_n_nodes(const kd_tree* t) { return t ? t->n_nodes : 0; }
uint64_t kd_count_nodes(uint64_t n_points, uint64_t leafsize) {
  return leafsize ? count_nodes(n_points, leafsize) : 0;
}

int kd_original_data(const kd_tree* t, double* out) {
  if (!t || !out) return fail(KD_ERR_INVALID_ARGUMENT, "NULL argument");
  DevicePin pin(t->device);
  cudaStream_t st = thread_stream();
  const uint64_t n = t->n_points * t->ndim;
  DevMem tmp;
  int rc;
  if ((rc = tmp.alloc(n * sizeof(double), st))) return rc;
  k_original<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(t->data, t->indices,
                                                                      static_cast<double*>(tmp.p), t->n_points,
                                                                      t->ndim);
  KD_TRY_CUDA(cudaGetLastError());
  KD_TRY_CUDA(cudaMemcpyAsync(out, tmp.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  return KD_OK;
}

int kd_export(const kd_tree* t, double* data, uint32_t* indices, uint32_t* node_words, double* split,
              double* boxes) {
  if (!t) return fail(KD_ERR_INVALID_ARGUMENT, "tree is NULL");
  DevicePin pin(t->device);
  cudaStream_t st = thread_stream();
  if (data)
    KD_TRY_CUDA(cudaMemcpyAsync(data, t->data, t->n_points * t->ndim * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (indices)
    KD_TRY_CUDA(cudaMemcpyAsync(indices, t->indices, t->n_points * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  if (boxes)
    KD_TRY_CUDA(cudaMemcpyAsync(boxes, t->boxes, t->n_nodes * 2 * t->ndim * sizeof(double), cudaMemcpyDeviceToHost,
                                st));
  if (node_words || split) {
    DevMem w, s;
    int rc;
    if ((rc = w.alloc(t->n_nodes * 4 * sizeof(uint32_t), st)) || (rc = s.alloc(t->n_nodes * sizeof(double), st)))
      return rc;
    k_export_nodes<<<static_cast<unsigned>((t->n_nodes + 255) / 256), 256, 0, st>>>(
        t->nodes, t->n_nodes, static_cast<uint32_t*>(w.p), static_cast<double*>(s.p));
    KD_TRY_CUDA(cudaGetLastError());
    if (node_words)
      KD_TRY_CUDA(cudaMemcpyAsync(node_words, w.p, t->n_nodes * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (split) KD_TRY_CUDA(cudaMemcpyAsync(split, s.p, t->n_nodes * sizeof(double), cudaMemcpyDeviceToHost, st));
    KD_TRY_CUDA(cudaStreamSynchronize(st));
  }
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  return KD_OK;
}

// Page-locked host blocks for result arrays.  Kept for reuse up to
// HOST_POOL_KEEP_BYTES (the largest cached blocks are unpinned first to make
// room for a freed one): allocating (pinning) a block costs about 4 ms per
// 128 MB, which a query loop would otherwise pay on every call.
namespace {
constexpr uint64_t HOST_POOL_KEEP_BYTES = 4ull << 30;
std::mutex g_host_mu;
std::multimap<uint64_t, void*> g_host_free;       // size -> block
std::unordered_map<void*, uint64_t> g_host_size;  // every live or pooled block
uint64_t g_host_free_bytes = 0;
}  // namespace

int kd_host_alloc(uint64_t bytes, void** out) {
  if (!out) return fail(KD_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  const uint64_t want = std::max<uint64_t>(bytes, 1);
  {
    std::lock_guard<std::mutex> lock(g_host_mu);
    auto it = g_host_free.lower_bound(want);
    if (it != g_host_free.end() && it->first <= 2 * want) {  // reuse a block of about this size:
      it = std::prev(g_host_free.upper_bound(it->first));     // the one freed last (warmest)
      *out = it->second;
      g_host_free_bytes -= it->first;
      g_host_free.erase(it);
      return KD_OK;
    }
  }
  const uint64_t size = (want + (2ull << 20) - 1) / (2ull << 20) * (2ull << 20);
  void* p = nullptr;
  cudaError_t e = cudaHostAlloc(&p, size, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    std::lock_guard<std::mutex> lock(g_host_mu);  // give the cached blocks back and try once more
    for (auto& kv : g_host_free) {
      g_host_size.erase(kv.second);
      cudaFreeHost(kv.second);
    }
    g_host_free.clear();
    g_host_free_bytes = 0;
    cudaGetLastError();
    e = cudaHostAlloc(&p, size, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc");
  }
  std::lock_guard<std::mutex> lock(g_host_mu);
  g_host_size[p] = size;
  *out = p;
  return KD_OK;
}

void kd_host_free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lock(g_host_mu);
  auto it = g_host_size.find(p);
  if (it == g_host_size.end()) return;  // not ours
  const uint64_t size = it->second;
  if (size > HOST_POOL_KEEP_BYTES) {
    g_host_size.erase(it);
    cudaFreeHost(p);
    return;
  }
  // the block just freed is the likeliest to be asked for again: make room
  // for it by unpinning the largest cached blocks
  while (g_host_free_bytes + size > HOST_POOL_KEEP_BYTES) {
    auto big = std::prev(g_host_free.end());
    g_host_free_bytes -= big->first;
    g_host_size.erase(big->second);
    cudaFreeHost(big->second);
    g_host_free.erase(big);
  }
  g_host_free.emplace(size, p);
  g_host_free_bytes += size;
}

size_t kd_last_error(char* buf, size_t len) {
  const std::string& m = g_last_error;
  if (buf && len) {
    size_t n = m.size() < len - 1 ? m.size() : len - 1;
    std::memcpy(buf, m.data(), n);
    buf[n] = '\0';
  }
  return m.size();
}

}  // extern "C"
