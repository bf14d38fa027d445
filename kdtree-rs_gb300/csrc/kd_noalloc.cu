// kd_noalloc.cu -- kd_query_device_noalloc: the exact k-NN query for callers
// that must not allocate device memory.
//
// Some callers cannot let a library allocate: frameworks that reserve nearly all
// of HBM up front for their own memory pool (an extra cudaMalloc from here fails
// or fragments what they manage), and latency-critical request loops that keep
// allocation -- its failure modes and the synchronisation cudaMalloc / cudaFree
// imply -- out of the serving path.  kd_query_device allocates a status word, and
// for widths without a register path also a per-query scratch array, on every
// call.  This entry point runs the same query kernel with both placed in one
// fixed, file-scope device array instead, so it calls no allocator at all.
//
// The array (KD_NOALLOC_SCRATCH_BYTES = 4 MiB) is part of the loaded module:
// every GPU that loads the library holds it until the process exits.  Its
// layout: bytes [0, 4) the status word, [128, 132) the count of near-tie
// reruns, then KD_NOALLOC_MAX_VALUES doubles used either as the one-thread
// kernels' CellBound scratch (n_queries * ndim doubles) or as the near-tie
// rerun list (n_queries entries) -- never both in one call -- which is why a
// call takes at most KD_NOALLOC_MAX_VALUES = n_queries * ndim query values.
#include <cmath>
#include <mutex>
#include <string>

#include "kd_internal.hpp"

namespace kd {
namespace {

constexpr uint64_t NOALLOC_SCRATCH_BYTES = 4ull << 20;
constexpr uint64_t NOALLOC_STATUS_BYTES = 256;
constexpr uint64_t NOALLOC_MAX_VALUES = (NOALLOC_SCRATCH_BYTES - NOALLOC_STATUS_BYTES) / sizeof(double);
static_assert(NOALLOC_MAX_VALUES == KD_NOALLOC_MAX_VALUES, "header and implementation disagree");

// Shared by every call on a device; it keeps whatever the last call left in it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on device `dev` (current).  In host code
// the symbol is only a host-side stand-in, so the address is looked up once
// per device (with that device current) and remembered.  The lookup is also
// what makes the CUDA runtime load this file's module -- and so place the
// array in device memory -- when modules load lazily (the default), which is
// why noalloc_prepare runs it during the allocating set-up of a tree.
int scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= MAX_DEVICES) return fail(KD_ERR_INVALID_ARGUMENT, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return KD_OK;
}

}  // namespace

void noalloc_prepare(int dev) {
  void* p = nullptr;
  if (scratch_address(dev, &p) != KD_OK) set_error("");  // retried by the first kd_query_device_noalloc call
}

namespace {

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

extern "C" int kd_query_device_noalloc(const kd_tree* tree, const double* d_queries, uint64_t n_values, uint64_t k,
                                       double p, int has_max_distance, double max_distance, double eps,
                                       double* d_out_distances, int64_t* d_out_indices, void* stream) {
  if (!tree) return fail(KD_ERR_INVALID_ARGUMENT, "tree is NULL");
  if (k == 0) return fail(KD_ERR_INVALID_K, "k must be greater than zero");
  if (n_values == 0 || n_values % tree->ndim)
    return fail(KD_ERR_INVALID_SHAPE, "queries must be a contiguous row-major matrix");
  if (!d_queries || !d_out_distances || !d_out_indices) return fail(KD_ERR_INVALID_ARGUMENT, "NULL buffer");
  if (n_values > NOALLOC_MAX_VALUES)
    return fail(KD_ERR_INVALID_ARGUMENT,
                "kd_query_device_noalloc takes at most " + std::to_string(NOALLOC_MAX_VALUES) +
                    " query values (n_queries * ndim) per call, got " + std::to_string(n_values) +
                    "; split the batch or use kd_query_device");
  QueryParams qp{};
  std::string msg;
  const int scalar = validate_scalars(k, p, has_max_distance, max_distance, eps, &qp, &msg);

  DeviceScope scope(tree->device);
  void* base = nullptr;
  int rc = scratch_address(tree->device, &base);
  if (rc) return rc;
  uint32_t* d_status = static_cast<uint32_t*>(base);
  uint32_t* d_rerun_count = d_status + 32;
  void* d_scratch = static_cast<unsigned char*>(base) + NOALLOC_STATUS_BYTES;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // The status word still holds the previous call's value: clear it first.
  KD_TRY_CUDA(cudaMemsetAsync(d_status, 0, sizeof(uint32_t), st));
  uint32_t h_status = 0;
  if (scalar != KD_OK) {
    // A non-finite query outranks the scalar errors (query.rs:46-48).
    k_check_finite<<<static_cast<unsigned>((n_values + 255) / 256), 256, 0, st>>>(d_queries, n_values, d_status);
    KD_TRY_CUDA(cudaGetLastError());
    KD_TRY_CUDA(cudaMemcpyAsync(&h_status, d_status, sizeof h_status, cudaMemcpyDeviceToHost, st));
    KD_TRY_CUDA(cudaStreamSynchronize(st));
    if (h_status) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
    return fail(scalar, msg);
  }
  const uint64_t nq = n_values / tree->ndim;
  if ((rc = query_on_device_scratch(tree, d_queries, nq, qp, d_out_distances, d_out_indices, st, d_status, d_scratch,
                                    d_rerun_count)))
    return rc;
  KD_TRY_CUDA(cudaMemcpyAsync(&h_status, d_status, sizeof h_status, cudaMemcpyDeviceToHost, st));
  KD_TRY_CUDA(cudaStreamSynchronize(st));
  if (h_status) return fail(KD_ERR_NONFINITE_DATA, "all coordinates must be finite");
  return KD_OK;
}
