// kd_query_packet.cu -- launches of the packet traversal (kd_query_packet.cuh)
// for the compile-time widths 2, 3, 8 and 16 and the L1 / L2 / L-inf metrics;
// a translation unit of its own so it compiles in parallel with the other
// query kernels.
#include <type_traits>

#include "kd_internal.hpp"

namespace kd {
namespace {

#include "kd_query_common.cuh"
#include "kd_lazy_best.cuh"
#include "kd_query_packet.cuh"

template <int M, int D>
int launch_k(const QArgs& a, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((a.nq + QUERY_THREADS - 1) / QUERY_THREADS);
  if (a.k == 1) k_query_packet<M, D, 1><<<blocks, QUERY_THREADS, 0, st>>>(a);
  else if (a.k <= 4) k_query_packet<M, D, 4><<<blocks, QUERY_THREADS, 0, st>>>(a);
  else if (a.k <= 8) k_query_packet<M, D, 8><<<blocks, QUERY_THREADS, 0, st>>>(a);
  else if (a.k <= 16) k_query_packet<M, D, 16><<<blocks, QUERY_THREADS, 0, st>>>(a);
  else k_query_packet<M, D, 32><<<blocks, QUERY_THREADS, 0, st>>>(a);
  KD_TRY_CUDA(cudaGetLastError());
  return KD_OK;
}

template <int M>
int launch_d(const QArgs& a, cudaStream_t st) {
  switch (a.d) {
    case 2: return launch_k<M, 2>(a, st);
    case 3: return launch_k<M, 3>(a, st);
    case 8: return launch_k<M, 8>(a, st);
    default: return launch_k<M, 16>(a, st);
  }
}

}  // namespace

bool packet_applicable(uint64_t d, int metric, uint64_t k, uint64_t n_points, bool use_eps) {
  return metric != M_LP && !use_eps && k >= 1 && k <= 32 && n_points < 0xffffffffull &&
         (d == 2 || d == 3 || d == 8 || d == 16);
}

int launch_packet_query(const QArgs& a, int metric, cudaStream_t st) {
  if (!packet_applicable(a.d, metric, a.k, a.n_points, a.use_eps))
    return fail(KD_ERR_INVALID_ARGUMENT, "the packet traversal does not cover this query");
  switch (metric) {
    case M_L1: return launch_d<M_L1>(a, st);
    case M_L2: return launch_d<M_L2>(a, st);
    default: return launch_d<M_LINF>(a, st);
  }
}

}  // namespace kd
