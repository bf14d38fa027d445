// kd_query_warp.cu -- launches of the best-first warp-per-query kernel
// (kd_query_warp.cuh) for every width up to 128 (compile-time kernels for 1,
// 2, 3, 4, 8 and 16, one runtime-width kernel for the rest), the L1 / L2 /
// L-inf metrics and k <= 64 (one or two list slots per lane); a translation
// unit of its own so it compiles in parallel with the other query kernels.
#include <type_traits>

#include "kd_internal.hpp"

namespace kd {
namespace {

#include "kd_query_common.cuh"
#include "kd_lazy_best.cuh"
#include "kd_query_packet.cuh"
#include "kd_warp.cuh"
#include "kd_query_warp.cuh"

template <int M, int KS>
int launch_ks(const QArgs& a, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((a.nq + QUERY_THREADS / 32 - 1) / (QUERY_THREADS / 32));
  switch (a.d) {
    case 1: k_query_warp<M, 1, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
    case 2: k_query_warp<M, 2, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
    case 3: k_query_warp<M, 3, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
    case 4: k_query_warp<M, 4, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
    case 8: k_query_warp<M, 8, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
    case 16: k_query_warp<M, 16, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
    default: k_query_warp<M, 0, KS><<<blocks, QUERY_THREADS, 0, st>>>(a); break;
  }
  KD_TRY_CUDA(cudaGetLastError());
  return KD_OK;
}

template <int M>
int launch_m(const QArgs& a, cudaStream_t st) {
  return a.k <= 32 ? launch_ks<M, 1>(a, st) : launch_ks<M, 2>(a, st);
}

}  // namespace

bool warp_applicable(uint64_t d, int metric, uint64_t k, uint64_t n_points, bool use_eps) {
  return metric != M_LP && !use_eps && k >= 1 && k <= 64 && n_points < 0xffffffffull && d >= 1 &&
         d <= WARP_MAX_WIDTH;
}

int launch_warp_query(const QArgs& a, int metric, cudaStream_t st) {
  if (!warp_applicable(a.d, metric, a.k, a.n_points, a.use_eps))
    return fail(KD_ERR_INVALID_ARGUMENT, "the warp-per-query kernel does not cover this query");
  switch (metric) {
    case M_L1: return launch_m<M_L1>(a, st);
    case M_L2: return launch_m<M_L2>(a, st);
    default: return launch_m<M_LINF>(a, st);
  }
}

}  // namespace kd
