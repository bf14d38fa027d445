// kd_query_ref.cu -- launches of the reference-order warp-per-query kernel
// (kd_query_ref.cuh): queries with eps > 0 or general p, the reference-order
// path asked for explicitly, and the reruns of near-tie queries flagged by the
// eps = 0 fast paths.  Compile-time kernels for widths 1, 2, 3, 4, 8 and 16,
// one runtime-width kernel for the rest up to 128 (and for every width under
// general p); k <= 64.
#include <algorithm>
#include <type_traits>

#include "kd_internal.hpp"

namespace kd {
namespace {

#include "kd_query_common.cuh"
#include "kd_lazy_best.cuh"
#include "kd_query_packet.cuh"
#include "kd_warp.cuh"
#include "kd_query_ref.cuh"

template <int M, int D, int KS>
int launch_one(const QArgs& a, cudaStream_t st, const uint32_t* count, const uint64_t* list, unsigned blocks) {
  const uint64_t d = D > 0 ? D : a.d;
  const size_t smem = (QUERY_THREADS / 32) * ref_warp_smem(d, (D == 0 && M != M_LP) ? a.w32 : 0);
  if (smem > 48 * 1024)
    KD_TRY_CUDA(cudaFuncSetAttribute(k_query_ref<M, D, KS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
  k_query_ref<M, D, KS><<<blocks, QUERY_THREADS, smem, st>>>(a, count, list);
  KD_TRY_CUDA(cudaGetLastError());
  return KD_OK;
}

template <int M, int KS>
int launch_ks(const QArgs& a, cudaStream_t st, const uint32_t* count, const uint64_t* list, unsigned blocks) {
  if constexpr (M == M_LP) {
    return launch_one<M, 0, KS>(a, st, count, list, blocks);
  } else {
    switch (a.d) {
      case 1: return launch_one<M, 1, KS>(a, st, count, list, blocks);
      case 2: return launch_one<M, 2, KS>(a, st, count, list, blocks);
      case 3: return launch_one<M, 3, KS>(a, st, count, list, blocks);
      case 4: return launch_one<M, 4, KS>(a, st, count, list, blocks);
      case 8: return launch_one<M, 8, KS>(a, st, count, list, blocks);
      case 16: return launch_one<M, 16, KS>(a, st, count, list, blocks);
      default: return launch_one<M, 0, KS>(a, st, count, list, blocks);
    }
  }
}

template <int M>
int launch_m(const QArgs& a, cudaStream_t st, const uint32_t* count, const uint64_t* list, unsigned blocks) {
  return a.k <= 32 ? launch_ks<M, 1>(a, st, count, list, blocks) : launch_ks<M, 2>(a, st, count, list, blocks);
}

int launch_any(const QArgs& a, int metric, cudaStream_t st, const uint32_t* count, const uint64_t* list,
               unsigned blocks) {
  switch (metric) {
    case M_L1: return launch_m<M_L1>(a, st, count, list, blocks);
    case M_L2: return launch_m<M_L2>(a, st, count, list, blocks);
    case M_LINF: return launch_m<M_LINF>(a, st, count, list, blocks);
    default: return launch_m<M_LP>(a, st, count, list, blocks);
  }
}

}  // namespace

bool ref_warp_applicable(uint64_t d, uint64_t k, uint64_t n_points) {
  return k >= 1 && k <= 64 && d >= 1 && d <= WARP_MAX_WIDTH && n_points < 0xffffffffull;
}

int launch_ref_query(const QArgs& a, int metric, cudaStream_t st) {
  if (!ref_warp_applicable(a.d, a.k, a.n_points))
    return fail(KD_ERR_INVALID_ARGUMENT, "the reference-order warp kernel does not cover this query");
  QArgs b = a;
  b.rerun_count = nullptr;  // it is the reference's order: nothing to rerun
  const unsigned blocks = static_cast<unsigned>((a.nq + QUERY_THREADS / 32 - 1) / (QUERY_THREADS / 32));
  return launch_any(b, metric, st, nullptr, nullptr, blocks);
}

__global__ void k_add_count(unsigned long long* total, const uint32_t* count) { *total += *count; }

int launch_rerun(const QArgs& a, int metric, cudaStream_t st, const uint32_t* count, const uint64_t* list) {
  if (!ref_warp_applicable(a.d, a.k, a.n_points))
    return fail(KD_ERR_INVALID_ARGUMENT, "the reference-order warp kernel does not cover this query");
  if (a.rerun_total) {
    k_add_count<<<1, 1, 0, st>>>(a.rerun_total, count);
    KD_TRY_CUDA(cudaGetLastError());
  }
  QArgs b = a;
  b.rerun_count = nullptr;
  b.order = nullptr;
  // at most one warp per possible entry, at most eight blocks an SM: the
  // count is only known on the device (usually 0, a few for tie-heavy data)
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t need = (a.nq + QUERY_THREADS / 32 - 1) / (QUERY_THREADS / 32);
  const unsigned blocks = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(need, 8ull * sms)));
  return launch_any(b, metric, st, count, list, blocks);
}

}  // namespace kd
